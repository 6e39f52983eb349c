"""ctypes binding of libfimgpu.so (the C-ABI declared in include/fim_gpu.h).

The library is the only compute path: if it is missing the import fails
loudly; there is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

FIM_OK, FIM_EINVAL, FIM_ENOMEM, FIM_ECUDA, FIM_ENUMERIC, FIM_ETIMEDOUT, FIM_ENOTSUP = range(7)
FIM_PREC_F64, FIM_PREC_F32 = 0, 1
STATUS_NAMES = {0: "FIM_OK", 1: "FIM_EINVAL", 2: "FIM_ENOMEM", 3: "FIM_ECUDA", 4: "FIM_ENUMERIC",
                5: "FIM_ETIMEDOUT", 6: "FIM_ENOTSUP"}

FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "u_tdcy", "v_tdcy",
          "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy", "massfx", "ws3d", "sdot", "relvor", "psrf", "ptdcy",
          "u_edg", "v_edg", "dp_edg", "lp_edg", "mont_edg", "uvsq_edg", "geop_edg", "trc_edg", "cumufx", "dpinit"]
FIELD_ID = {n: i for i, n in enumerate(FIELDS)}

c_int_p = ctypes.POINTER(ctypes.c_int32)
c_dbl_p = ctypes.POINTER(ctypes.c_double)


class GridDesc(ctypes.Structure):
    _fields_ = [("glvl", ctypes.c_int), ("nip", ctypes.c_int),
                ("nprox", ctypes.c_void_p), ("prox", ctypes.c_void_p), ("proxs", ctypes.c_void_p),
                ("lat", ctypes.c_void_p), ("lon", ctypes.c_void_p), ("area", ctypes.c_void_p),
                ("cs", ctypes.c_void_p), ("sn", ctypes.c_void_p), ("sidevec_c", ctypes.c_void_p),
                ("sidevec_e", ctypes.c_void_p), ("sideln", ctypes.c_void_p), ("rprox_ln", ctypes.c_void_p),
                ("corner_xy", ctypes.c_void_p), ("hfcoef", ctypes.c_void_p)]


class Config(ctypes.Structure):
    _fields_ = [("nvl", ctypes.c_int), ("ntra", ctypes.c_int), ("precision", ctypes.c_int),
                ("members", ctypes.c_int), ("host_pointers", ctypes.c_int), ("dt", ctypes.c_double),
                ("kbl", ctypes.c_int), ("flux_conserv_schm", ctypes.c_int), ("hi_order_flux_comp", ctypes.c_int),
                ("intfc_smooth", ctypes.c_double), ("slak", ctypes.c_double), ("miglim", ctypes.c_int),
                ("remap_optn", ctypes.c_int), ("ptop", ctypes.c_double), ("thktop", ctypes.c_double),
                ("veldff_bkgnd", ctypes.c_double), ("veldff_boost", ctypes.c_double),
                ("biharm_frst", ctypes.c_int), ("biharm_last", ctypes.c_int), ("rleigh", ctypes.c_double),
                ("rlthresh", ctypes.c_double), ("rltaper", ctypes.c_double), ("pure_sig", ctypes.c_int),
                ("thetac", ctypes.c_void_p), ("dpsig", ctypes.c_void_p), ("ntrb", ctypes.c_int),
                ("dtratio", ctypes.c_int), ("member_group", ctypes.c_int), ("hi_order_uv_comp", ctypes.c_int),
                ("stream_priority", ctypes.c_int), ("tracer_chunk", ctypes.c_int)]


class Budget(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ["qmass", "qmsqv", "qmsqw", "qmso3", "qmste", "qmstr", "qmstrn", "qmstrc"]]


# exported symbols and their argument kinds: p = pointer, i = int, vp = void*
_VP = ctypes.c_void_p
_I = ctypes.c_int
_SIGS = {
    "fim_grid_nip": ([_I], _I),
    "fim_grid_build": ([_I, _VP], _I),
    "fim_ctx_create": ([_VP, _VP, _VP], _I),
    "fim_ctx_destroy": ([_VP], _I),
    "fim_ctx_last_error": ([_VP], ctypes.c_char_p),
    "fim_ctx_stream": ([_VP], _VP),
    "fim_get_ab": ([_VP, _VP, _VP, _VP, _VP, _VP, _VP], _I),
    "fim_set_ab": ([_VP, _I, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double], _I),
    "fim_abstart": ([_VP, _I, _I, _VP, _VP, _VP, _VP, _VP, _VP], _I),
    "fim_state_alloc": ([_VP, _VP], _I),
    "fim_state_free": ([_VP, _VP], _I),
    "fim_state_field": ([_VP, _VP, _I, _I, _VP, _VP], _I),
    "fim_state_upload": ([_VP, _VP, _I, _I, _VP], _I),
    "fim_state_download": ([_VP, _VP, _I, _I, _VP], _I),
    "fim_state_upload_f64": ([_VP, _VP, _I, _I, _VP], _I),
    "fim_state_upload_slot": ([_VP, _VP, _I, _I, _I, _VP], _I),
    "fim_state_download_slot": ([_VP, _VP, _I, _I, _I, _VP], _I),
    "fim_state_init": ([_VP, _VP], _I),
    "fim_step": ([_VP, _VP, _I, _I], _I),
    "fim_step_active": ([_VP, _VP, _I], _I),
    "fim_state_set_host": ([_VP, _VP, _I, _I, _VP], _I),
    "fim_step_io": ([_VP, _VP, _I, _VP, _VP], _I),
    "fim_set_persistent": ([_VP, _I, ctypes.c_double], _I),
    "fim_set_barrier_test": ([_VP, _I], _I),
    "fim_state_init_member": ([_VP, _VP, _I], _I),
    "fim_member_set_active": ([_VP, _VP, _I, _I], _I),
    "fim_member_its": ([_VP, _I], _I),
    "fim_member_set_tracers": ([_VP, _I, _I], _I),
    "fim_state_synthetic": ([_VP, _VP, _I, ctypes.c_ulonglong, _I, ctypes.c_double, ctypes.c_double], _I),
    "fim_member_get_step": ([_VP, _I] + [_VP] * 7, _I),
    "fim_member_set_step": ([_VP, _I, _I, _I, _I, _I, ctypes.c_double, ctypes.c_double, ctypes.c_double], _I),
    "fim_state_budget": ([_VP, _VP, _I, _VP, _VP], _I),
    "fim_check": ([_VP, _VP, _VP], _I),
    "fim_launch_count": ([_VP], ctypes.c_int64),
    "fim_ctx_device_bytes": ([_VP], ctypes.c_int64),
    "fim_tracer_shape": ([_VP, _VP, _VP, _VP], _I),
    "fim_grid_patches": ([_VP, _I, _VP, _VP, _VP, _VP], _I),
    "fim_profile_enable": ([_VP, _I], _I),
    "fim_profile_report": ([_VP, ctypes.c_char_p, _I], _I),
    "fim_cnuity_noalloc": ([_VP, _I] + [_VP] * 13, _I),
}
_ROUTINES = {
    "fim_edgvar1": [_VP, _I] + [_VP] * 16,
    "fim_edgvar2": [_VP, _I] + [_VP] * 16,
    "fim_edgvar3": [_VP, _I] + [_VP] * 16,
    "fim_cnuity": [_VP, _I] + [_VP] * 13,
    "fim_trcadv": [_VP, _I] + [_VP] * 7,
    "fim_mass_adv": [_VP, _I] + [_VP] * 12,
    "fim_momtum": [_VP, _I] + [_VP] * 13,
    "fim_hybgen": [_VP, _I] + [_VP] * 8,
    "fim_hystat": [_VP, _I] + [_VP] * 8,
    "fim_globsum": [_VP, _I] + [_VP] * 9,
    "fim_transp0": [_VP, _I] + [_VP] * 3,
    "fim_transp1": [_VP, _I] + [_VP] * 2,
    "fim_transp2": [_VP, _I] + [_VP] * 4,
    "fim_cpl_dyn_to_phy": [_VP, _I, _I] + [_VP] * 15,
    "fim_cpl_phy_to_dyn": [_VP, _I, _I, _I, _I, ctypes.c_double] + [_VP] * 17,
}
for _name, _args in _ROUTINES.items():
    for _sfx in ("_r8", "_r4"):
        _SIGS[_name + _sfx] = (_args, _I)

EXPORTED = sorted(_SIGS)

_lib = None


def load(build=True):
    """Load (and if needed build) libfimgpu.so; raises if it cannot."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if build:
        path = _build.build_library()
    if not os.path.exists(path):
        raise RuntimeError("libfimgpu.so is missing (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


class FimError(RuntimeError):
    def __init__(self, code, what, detail=""):
        self.code = code
        super().__init__("%s failed with %s%s" % (what, STATUS_NAMES.get(code, str(code)),
                                                  (": " + detail) if detail else ""))


def check(code, what, ctx=None):
    if code != FIM_OK:
        detail = ""
        if ctx:
            msg = load().fim_ctx_last_error(ctx)
            detail = msg.decode() if msg else ""
        raise FimError(code, what, detail)
