"""Host-side mirror of the reference dycore interface over the C-ABI.

`Dycore` owns one fim_ctx (grid tables uploaded once) and exposes the
reference subroutines under their own names and argument order:
abstart, edgvar1, edgvar3, cnuity, trcadv, momtum, hybgen, hystat, globsum
(FIMsrc/fim/horizontal/dyn_run.F90:119-425).  Arrays are torch CUDA tensors
(device-resident mode) or numpy arrays (host_pointers mode), flat in the
reference layout.  `DycoreState` is the library-owned device state that the
fused step advances; with use_graph=True each step replays one CUDA graph.
"""
import ctypes

import numpy as np

from . import _lib
from .config import FimConfig
from .grid import Grid

FIELDS = _lib.FIELDS


def _ptr(a):
    """Raw pointer of a torch tensor or numpy array (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


class Dycore:
    def __init__(self, grid: Grid, cfg: FimConfig):
        self.lib = _lib.load()
        self.grid = grid
        self.cfg = cfg
        self._desc = grid.desc()
        self._ccfg = cfg.to_c()
        ctx = ctypes.c_void_p()
        _lib.check(self.lib.fim_ctx_create(ctypes.byref(self._desc), ctypes.byref(self._ccfg), ctypes.byref(ctx)),
                   "fim_ctx_create")
        self.ctx = ctx
        self.N, self.L, self.T = grid.nip, cfg.nvl, cfg.ntra
        self.TB = cfg.ntrb
        self._sfx = "_r8" if cfg.precision == "f64" else "_r4"

    def close(self):
        if self.ctx:
            self.lib.fim_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- sizes of the reference arrays ----
    def sizes(self):
        N, L, T = self.N, self.L, self.T
        return dict(cell=N * L, intf=N * (L + 1), edge=6 * N * L, ab=3 * N * L, tr=T * N * L,
                    trab=3 * T * N * L, tredg=6 * T * N * L, mf=18 * N * L, col=N)

    @property
    def stream(self):
        return self.lib.fim_ctx_stream(self.ctx)

    def launches(self):
        return self.lib.fim_launch_count(self.ctx)

    def set_persistent(self, on, timeout_s=1.0):
        """cnuity1..4 as one cooperative persistent launch (fim_set_persistent)."""
        _lib.check(self.lib.fim_set_persistent(self.ctx, 1 if on else 0, float(timeout_s)), "fim_set_persistent",
                   self.ctx)

    def set_barrier_test(self, phantom_arrivals):
        """1: the persistent launch's barriers wait for a block that never
        arrives, so their time limit runs out (fim_set_barrier_test)."""
        _lib.check(self.lib.fim_set_barrier_test(self.ctx, int(phantom_arrivals)), "fim_set_barrier_test", self.ctx)

    def device_bytes(self):
        """Device memory the context and its states currently own."""
        return self.lib.fim_ctx_device_bytes(self.ctx)

    def profile(self, on):
        _lib.check(self.lib.fim_profile_enable(self.ctx, 1 if on else 0), "fim_profile_enable", self.ctx)

    def profile_report(self):
        """{kernel: (launches, total ms)} since the last report."""
        buf = ctypes.create_string_buffer(1 << 16)
        _lib.check(self.lib.fim_profile_report(self.ctx, buf, len(buf)), "fim_profile_report", self.ctx)
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms = line.split()
            out[name] = (int(n), float(ms))
        return out

    def _need_tracer_edges(self, a, what):
        """The per-routine entry points take the reference's trc_edg(nvl, 6,
        nip, ntra): refuse a smaller array (e.g. a fused-step state's trc_edg,
        which holds theta's edge values only) rather than let a kernel write
        past its end."""
        n = a.numel() if hasattr(a, "numel") else getattr(a, "size", None)
        need = 6 * self.cfg.nvl * self.grid.nip * self.T
        if n is not None and n < need:
            raise ValueError("%s: %d values, the routine needs nvl x 6 x nip x ntra = %d" % (what, n, need))

    def _call(self, name, *args):
        """Run one entry point.  Device arrays written by torch on its own
        stream are complete before the library's stream starts, and the
        library's results are complete when the call returns."""
        fn = getattr(self.lib, name + self._sfx)
        device = not self.cfg.host_pointers
        if device:
            import torch
            torch.cuda.current_stream().synchronize()
        _lib.check(fn(self.ctx, *args), name, self.ctx)
        if device:
            self.sync_stream()

    def sync_stream(self):
        import torch
        torch.cuda.ExternalStream(self.stream).synchronize()

    def sync(self):
        import torch
        torch.cuda.synchronize()

    # ---- AB3 bookkeeping (module_variables nf, of, vof, adbash1..3) ----
    def abstart(self, its, its_start=1):
        nf, of, vof = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        a1, a2, a3 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _lib.check(self.lib.fim_abstart(self.ctx, its, its_start, ctypes.byref(nf), ctypes.byref(of),
                                        ctypes.byref(vof), ctypes.byref(a1), ctypes.byref(a2), ctypes.byref(a3)),
                   "fim_abstart", self.ctx)
        return nf.value, of.value, vof.value, a1.value, a2.value, a3.value

    def set_ab(self, nf, of, vof, ab1, ab2, ab3):
        _lib.check(self.lib.fim_set_ab(self.ctx, nf, of, vof, ab1, ab2, ab3), "fim_set_ab", self.ctx)

    def get_ab(self):
        v = [ctypes.c_int() for _ in range(3)] + [ctypes.c_double() for _ in range(3)]
        _lib.check(self.lib.fim_get_ab(self.ctx, *[ctypes.byref(x) for x in v]), "fim_get_ab", self.ctx)
        return tuple(x.value for x in v)

    # ---- the reference routines ----
    def edgvar1(self, its, u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg, v_edg, dp_edg, lp_edg,
                geop_edg, mont_edg, uvsq_edg, trc_edg):
        self._call("fim_edgvar1", its, *map(_ptr, (u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg,
                                                     v_edg, dp_edg, lp_edg, geop_edg, mont_edg, uvsq_edg, trc_edg)))

    def edgvar2(self, its, u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg, v_edg, dp_edg, lp_edg,
                geop_edg, mont_edg, uvsq_edg, trc_edg):
        self._need_tracer_edges(trc_edg, "trc_edg")
        self._call("fim_edgvar2", its, *map(_ptr, (u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg,
                                                     v_edg, dp_edg, lp_edg, geop_edg, mont_edg, uvsq_edg, trc_edg)))

    def edgvar3(self, its, u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg, v_edg, dp_edg, lp_edg,
                geop_edg, mont_edg, uvsq_edg, trc_edg):
        self._need_tracer_edges(trc_edg, "trc_edg")
        self._call("fim_edgvar3", its, *map(_ptr, (u_vel, v_vel, delp, pres, exner, geop, montg, tracr, u_edg,
                                                     v_edg, dp_edg, lp_edg, geop_edg, mont_edg, uvsq_edg, trc_edg)))

    def cnuity(self, its, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, dplo_tndcy,
               massfx, omega):
        self._call("fim_cnuity", its, *map(_ptr, (u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner,
                                                    dp_tndcy, dplo_tndcy, massfx, omega)))

    def cnuity_noalloc(self, its, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy,
                       dplo_tndcy, massfx, omega):
        """cnuity with its scratch in the library's static array (device
        pointers only; no device allocation by the call)."""
        import torch
        torch.cuda.current_stream().synchronize()
        _lib.check(self.lib.fim_cnuity_noalloc(self.ctx, its, *map(_ptr, (u_velo, v_velo, u_edg, v_edg, dp_edg,
                                                                            lp_edg, delp, pres, exner, dp_tndcy,
                                                                            dplo_tndcy, massfx, omega))),
                   "fim_cnuity_noalloc", self.ctx)
        self.sync_stream()

    def mass_adv(self, its, u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, massfx,
                 omega):
        self._call("fim_mass_adv", its, *map(_ptr, (u_velo, v_velo, u_edg, v_edg, dp_edg, lp_edg, delp, pres,
                                                      exner, dp_tndcy, massfx, omega)))

    def trcadv(self, its, trcr_edg, tracr, trcdp, trc_tdcy, trclo_tdcy, massfx, delp):
        self._need_tracer_edges(trcr_edg, "trcr_edg")
        self._call("fim_trcadv", its, *map(_ptr, (trcr_edg, tracr, trcdp, trc_tdcy, trclo_tdcy, massfx, delp)))

    def momtum(self, its, u_velo, v_velo, exner, relvor, u_edg, v_edg, trcr_edg, geop_edg, mont_edg, uvsq_edg,
               u_tndcy, v_tndcy, dp3d):
        self._call("fim_momtum", its, *map(_ptr, (u_velo, v_velo, exner, relvor, u_edg, v_edg, trcr_edg, geop_edg,
                                                    mont_edg, uvsq_edg, u_tndcy, v_tndcy, dp3d)))

    def hybgen(self, its, targt, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d):
        self._call("fim_hybgen", its, *map(_ptr, (targt, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d)))

    def hystat(self, its, ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy):
        self._call("fim_hystat", its, *map(_ptr, (ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy)))

    # physics coupling (cpl_run.F90): GFS arrays are float64 (nip, nvl), cell fastest
    GFS_NAMES = ("ps", "dp", "p", "u", "v", "dpdt", "q", "oz", "cld", "t")

    def cpl_dyn_to_phy(self, its, pr3d, us3d, vs3d, ws3d, tr3d, gfs, callphy=True):
        """cpl_dyn_to_phy: fills gfs[name] for the GFS_NAMES (ps: nip values)."""
        self._call("fim_cpl_dyn_to_phy", its, int(callphy), *map(_ptr, (pr3d, us3d, vs3d, ws3d, tr3d)),
                   *[_ptr(gfs[n]) for n in self.GFS_NAMES])

    def cpl_phy_to_dyn(self, its, gfs, geshem, rainc, evap, dp3d, us3d, vs3d, tr3d, rn2d, rc2d, qf2d, dtp,
                       addtend=False, smoothtend=False, callphy=True):
        """cpl_phy_to_dyn: the dynamics state and the rain / evaporation columns."""
        self._call("fim_cpl_phy_to_dyn", its, int(callphy), int(addtend), int(smoothtend), ctypes.c_double(dtp),
                   *[_ptr(gfs[n]) for n in ("p", "u", "v", "q", "cld", "oz", "t")],
                   *map(_ptr, (geshem, rainc, evap, dp3d, us3d, vs3d, tr3d, rn2d, rc2d, qf2d)))

    def transp0(self, its, cumufx, dp3d, dpinit):
        self._call("fim_transp0", its, *map(_ptr, (cumufx, dp3d, dpinit)))

    def transp1(self, its, cumufx, massfx):
        self._call("fim_transp1", its, *map(_ptr, (cumufx, massfx)))

    def transp2(self, its, tracr, cumufx, dpinit, dpfinl):
        self._call("fim_transp2", its, *map(_ptr, (tracr, cumufx, dpinit, dpfinl)))

    def globsum(self, its, dp3d, tr, pr3d, ex3d, rn2d=None, rc2d=None, qf2d=None):
        qtrcr = np.zeros(self.T + self.TB, np.float64)
        b = _lib.Budget()
        self._call("fim_globsum", its, *map(_ptr, (dp3d, tr, rn2d, rc2d, pr3d, ex3d, qf2d)), qtrcr.ctypes.data,
                   ctypes.byref(b))
        return qtrcr, {n: getattr(b, n) for n, _ in _lib.Budget._fields_}

    def tracer_shape(self):
        """(levels per thread, threads per block, probe ms) of the fused tracer kernels."""
        v, t, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _lib.check(self.lib.fim_tracer_shape(self.ctx, ctypes.byref(v), ctypes.byref(t), ctypes.byref(ms)),
                   "fim_tracer_shape", self.ctx)
        return v.value, t.value, ms.value

    def state(self):
        return DycoreState(self)


class DycoreState:
    """Library-owned device state of all members (module_variables arrays)."""

    def __init__(self, dyc: Dycore):
        self.dyc = dyc
        self.lib = dyc.lib
        st = ctypes.c_void_p()
        _lib.check(self.lib.fim_state_alloc(dyc.ctx, ctypes.byref(st)), "fim_state_alloc", dyc.ctx)
        self.st = st
        self.its = 0

    def free(self):
        if self.st:
            self.lib.fim_state_free(self.dyc.ctx, self.st)
            self.st = None

    def field_ptr(self, name, member=0):
        p = ctypes.c_void_p()
        n = ctypes.c_int64()
        _lib.check(self.lib.fim_state_field(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, ctypes.byref(p),
                                            ctypes.byref(n)), "fim_state_field", self.dyc.ctx)
        return p.value, n.value

    def tensor(self, name, member=0):
        """Zero-copy torch view of one member's field."""
        import torch
        ptr, n = self.field_ptr(name, member)
        dt = torch.float64 if self.dyc.cfg.precision == "f64" else torch.float32
        return _torch_from_ptr(ptr, n, dt)

    def upload(self, name, host, member=0):
        ptr, n = self.field_ptr(name, member)
        host = np.ascontiguousarray(host, dtype=self.dyc.cfg.dtype) if isinstance(host, np.ndarray) else host
        if isinstance(host, np.ndarray) and host.size != n:
            raise ValueError("%s: %d elements, expected %d" % (name, host.size, n))
        _lib.check(self.lib.fim_state_upload(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, _ptr(host)),
                   "fim_state_upload", self.dyc.ctx)
        if isinstance(host, np.ndarray):
            self.dyc.sync()

    def download(self, name, member=0, out=None):
        ptr, n = self.field_ptr(name, member)
        if out is None:
            out = np.empty(n, self.dyc.cfg.dtype)
        _lib.check(self.lib.fim_state_download(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, _ptr(out)),
                   "fim_state_download", self.dyc.ctx)
        self.dyc.sync()
        return out

    def upload_slot(self, name, slot, host, member=0):
        """Upload AB3 slot `slot` (1..3) of a tendency field from the whole-field host array."""
        ptr, n = self.field_ptr(name, member)
        host = np.ascontiguousarray(host, dtype=self.dyc.cfg.dtype) if isinstance(host, np.ndarray) else host
        if isinstance(host, np.ndarray) and host.size != n:
            raise ValueError("%s: %d elements, expected %d" % (name, host.size, n))
        _lib.check(self.lib.fim_state_upload_slot(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, slot,
                                                  _ptr(host)), "fim_state_upload_slot", self.dyc.ctx)
        if isinstance(host, np.ndarray):
            self.dyc.sync()

    def download_slot(self, name, slot, member=0, out=None):
        """Download AB3 slot `slot` (1..3) of a tendency field into the whole-field host array."""
        ptr, n = self.field_ptr(name, member)
        if out is None:
            out = np.zeros(n, self.dyc.cfg.dtype)
        _lib.check(self.lib.fim_state_download_slot(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, slot,
                                                    _ptr(out)), "fim_state_download_slot", self.dyc.ctx)
        self.dyc.sync()
        return out

    def next_slots(self, member=0):
        """(nf, of, vof) of the member's next step, Fortran numbering: the slot
        it writes and the two it reads."""
        _, nf, of, vof, _ = self.get_step(member)
        return nf % 3 + 1, of % 3 + 1, vof % 3 + 1

    # fields dyn_init's adjustment reads; FP64 arrays of these go to an
    # FP32-mixed state through fim_state_upload_f64
    INIT_INPUTS = ("us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "tr3d")

    def upload_f64(self, name, host, member=0):
        """FP64 initial field: the FP32 copy is set and the FP64 values feed
        the next initial adjustment (fim_state_upload_f64)."""
        ptr, n = self.field_ptr(name, member)
        host = np.ascontiguousarray(host, dtype=np.float64)
        if host.size != n:
            raise ValueError("%s: %d elements, expected %d" % (name, host.size, n))
        _lib.check(self.lib.fim_state_upload_f64(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, _ptr(host)),
                   "fim_state_upload_f64", self.dyc.ctx)
        self.dyc.sync()

    def load(self, fields, member=0):
        """Upload a member's fields; FP64 arrays of the initial fields keep
        their precision for the initial adjustment of an FP32-mixed state."""
        f32 = self.dyc.cfg.precision != "f64"
        for k, v in fields.items():
            if f32 and k in self.INIT_INPUTS and isinstance(v, np.ndarray) and v.dtype == np.float64:
                self.upload_f64(k, v, member)
            else:
                self.upload(k, v, member)

    def init(self):
        _lib.check(self.lib.fim_state_init(self.dyc.ctx, self.st), "fim_state_init", self.dyc.ctx)
        self.its = 0

    def step(self, its=None, use_graph=False):
        its = self.its + 1 if its is None else its
        _lib.check(self.lib.fim_step(self.dyc.ctx, self.st, its, 1 if use_graph else 0), "fim_step", self.dyc.ctx)
        self.its = its

    def set_host(self, name, host, member=0):
        """Register the host copy of a member's field for step_io (a pinned
        torch tensor or numpy array of the field's size; None unregisters)."""
        ptr, n = self.field_ptr(name, member)
        if host is not None:
            size = host.numel() if hasattr(host, "numel") else host.size
            if size != n:
                raise ValueError("%s: %d elements, expected %d" % (name, size, n))
        _lib.check(self.lib.fim_state_set_host(self.dyc.ctx, self.st, _lib.FIELD_ID[name], member, _ptr(host)),
                   "fim_state_set_host", self.dyc.ctx)

    def step_io(self, its=None):
        """One step with the registered fields moved in and out around it
        (fim_step_io); returns the (host-to-device, device-to-host) bytes."""
        its = self.its + 1 if its is None else its
        up, down = ctypes.c_int64(0), ctypes.c_int64(0)
        _lib.check(self.lib.fim_step_io(self.dyc.ctx, self.st, its, ctypes.byref(up), ctypes.byref(down)),
                   "fim_step_io", self.dyc.ctx)
        self.its = its
        return up.value, down.value

    def init_member(self, member):
        """Initialise (dyn_init) and activate one member slot after its upload."""
        _lib.check(self.lib.fim_state_init_member(self.dyc.ctx, self.st, member), "fim_state_init_member",
                   self.dyc.ctx)

    def set_active(self, member, active):
        _lib.check(self.lib.fim_member_set_active(self.dyc.ctx, self.st, member, 1 if active else 0),
                   "fim_member_set_active", self.dyc.ctx)

    def synthetic(self, member, seed, ntra, sigma_ps=200.0, noise=0.0):
        """The seeded balanced state made on the device in member slot
        `member` (fim_state_synthetic; asynchronous on the library stream)."""
        _lib.check(self.lib.fim_state_synthetic(self.dyc.ctx, self.st, member, int(seed) & (2 ** 64 - 1), ntra,
                                                float(sigma_ps), float(noise)), "fim_state_synthetic", self.dyc.ctx)

    def set_tracers(self, member, ntr):
        """Member `member` carries ntr tracers (theta included): later steps
        leave its tracer slots ntr.. untouched and do no work for them."""
        _lib.check(self.lib.fim_member_set_tracers(self.dyc.ctx, member, ntr), "fim_member_set_tracers",
                   self.dyc.ctx)

    def member_its(self, member):
        return self.lib.fim_member_its(self.dyc.ctx, member)

    def get_step(self, member=0):
        """(itsm1, nf, of, vof, (adbash1, adbash2, adbash3)) of one member."""
        v = [ctypes.c_int() for _ in range(4)] + [ctypes.c_double() for _ in range(3)]
        _lib.check(self.lib.fim_member_get_step(self.dyc.ctx, member, *[ctypes.byref(x) for x in v]),
                   "fim_member_get_step", self.dyc.ctx)
        return v[0].value, v[1].value, v[2].value, v[3].value, (v[4].value, v[5].value, v[6].value)

    def set_step(self, member, itsm1, nf, of, vof, adbash):
        _lib.check(self.lib.fim_member_set_step(self.dyc.ctx, member, itsm1, nf, of, vof, *adbash),
                   "fim_member_set_step", self.dyc.ctx)
        self.its = itsm1

    def save_restart(self, path, member=0, extras=None):
        """Write one member's state as the dynamics section of a FIM restart
        file (restart_io); returns itsm1."""
        from .restart_io import STATE_FIELDS, write_restart
        itsm1, nf, of, vof, ab = self.get_step(member)
        fields = {n: self.download(n, member) for n in STATE_FIELDS if self.field_ptr(n, member)[1] > 0}
        write_restart(path, self.dyc.grid, self.dyc.cfg, itsm1, nf, of, vof, ab, fields, extras=extras)
        return itsm1

    def load_restart(self, path, member=0):
        """Restore one member from a restart file; its next step is itsm1+1.
        Returns the file's contents (restart_io.read_restart)."""
        from .restart_io import read_restart
        cfg = self.dyc.cfg
        r = read_restart(path, self.dyc.grid.nip, cfg.nvl, cfg.ntra, cfg.ntrb)
        for n, a in r["fields"].items():
            if self.field_ptr(n, member)[1] > 0:  # the class-B integrals exist only with class-B tracers
                self.upload(n, a, member)
        self.set_step(member, r["itsm1"], r["nf"], r["of"], r["vof"], r["adbash"])
        return r

    def step_active(self, use_graph=True):
        """Advance every active member by one step (each at its own its)."""
        _lib.check(self.lib.fim_step_active(self.dyc.ctx, self.st, 1 if use_graph else 0), "fim_step_active",
                   self.dyc.ctx)

    def budget(self, member=0):
        qtrcr = np.zeros(self.dyc.T + self.dyc.TB, np.float64)
        b = _lib.Budget()
        _lib.check(self.lib.fim_state_budget(self.dyc.ctx, self.st, member, qtrcr.ctypes.data, ctypes.byref(b)),
                   "fim_state_budget", self.dyc.ctx)
        return qtrcr, {n: getattr(b, n) for n, _ in _lib.Budget._fields_}

    def check(self):
        flags = ctypes.c_int()
        rc = self.lib.fim_check(self.dyc.ctx, self.st, ctypes.byref(flags))
        return rc, flags.value


def _torch_from_ptr(ptr, n, dtype):
    """Wrap device memory owned by the library as a torch tensor (no copy)."""
    import torch

    class _Holder:
        pass

    h = _Holder()
    esz = 8 if dtype == torch.float64 else 4
    typestr = "<f8" if esz == 8 else "<f4"
    h.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 2,
                                  "strides": None}
    return torch.as_tensor(h, device="cuda")
