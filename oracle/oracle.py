"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the cpu_baseline / reference arm
of bench.py as the checker.  Parity status: the routines are unpinned, the
integer grid tables pinned (see fim_oracle.h).
Arrays are float64 numpy, flat, in the reference layout.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libfimoracle.so")

_VP = ctypes.c_void_p


class OrcCtx(ctypes.Structure):
    _fields_ = [("nip", ctypes.c_int), ("nvl", ctypes.c_int), ("ntra", ctypes.c_int),
                ("prox", _VP), ("proxs", _VP), ("nprox", _VP),
                ("cs", _VP), ("sn", _VP), ("sidevec_c", _VP), ("sidevec_e", _VP), ("sideln", _VP),
                ("area", _VP), ("rarea", _VP), ("corio", _VP), ("grndspd", _VP), ("hfcoef", _VP),
                ("dt", ctypes.c_double), ("kbl", ctypes.c_int), ("hi_order", ctypes.c_int),
                ("miglim", ctypes.c_int), ("remap_optn", ctypes.c_int), ("flux_schm", ctypes.c_int),
                ("intfc_smooth", ctypes.c_double), ("slak", ctypes.c_double), ("ptop", ctypes.c_double),
                ("thktop", ctypes.c_double), ("rleigh", ctypes.c_double), ("rlthresh", ctypes.c_double),
                ("rltaper", ctypes.c_double),
                ("thetac", _VP), ("dpsig", _VP), ("dfflen", _VP), ("biharw", _VP), ("smoo_coeff", _VP),
                ("dfflen_max", ctypes.c_double),
                ("nf", ctypes.c_int), ("of", ctypes.c_int), ("vof", ctypes.c_int),
                ("ab1", ctypes.c_double), ("ab2", ctypes.c_double), ("ab3", ctypes.c_double),
                ("diag_flags", ctypes.c_long), ("ntrb", ctypes.c_int), ("corner_xy", _VP)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "fim_oracle.c")):
            build()
        lib = ctypes.CDLL(LIB)
        D, I, P = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        sigs = {
            "orc_derived": [I, I, I, D, D, D, D, I, I] + [P] * 9 + [P],
            "orc_abstart": [P, I],
            "orc_edgvar1": [P] + [P] * 16,
            "orc_edgvar3": [P] * 5,
            "orc_edgvar2": [P] * 6,
            "orc_cnuity": [P] * 14,
            "orc_trcadv": [P] * 8,
            "orc_mass_adv": [P] * 13,
            "orc_momtum": [P] * 13,
            "orc_hybgen": [P, I] + [P] * 8,
            "orc_hystat": [P, I] + [P] * 8,
            "orc_globsum": [P] * 10,
            "orc_prdp_from_ex": [P] * 4,
            "orc_set_threads": [I],
            "orc_transp0": [P] * 4,
            "orc_transp1": [P] * 3,
            "orc_transp2": [P, I, P, P, P, P],
            "orc_cpl_dyn_to_phy": [P] * 17,
            "orc_cpl_phy_to_dyn": [P, I, I, D] + [P] * 18,
        }
        for name, args in sigs.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = None
        _lib = lib
    return _lib


def set_threads(n):
    load().orc_set_threads(int(n))


def _p(a):
    return None if a is None else a.ctypes.data


class Oracle:
    """FP64 CPU restatement of the reference routines on one grid."""

    def __init__(self, grid, cfg):
        self.lib = load()
        self.grid, self.cfg = grid, cfg
        N, L = grid.nip, cfg.nvl
        nprox, prox, proxs = grid.zero_based()
        self._keep = dict(nprox=nprox, prox=prox, proxs=proxs)
        self.rarea = np.zeros(N)
        self.corio = np.zeros(N)
        self.grndspd = np.zeros(N)
        self.dfflen = np.zeros(L)
        self.biharw = np.zeros(L)
        self.smoo = np.zeros(L + 1)
        dmax = ctypes.c_double()
        self.lib.orc_derived(N, L, cfg.kbl, ctypes.c_double(cfg.dt), ctypes.c_double(cfg.intfc_smooth),
                             ctypes.c_double(cfg.veldff_bkgnd), ctypes.c_double(cfg.veldff_boost), cfg.biharm_frst,
                             cfg.biharm_last, _p(grid.lat), _p(grid.area), _p(grid.sideln), _p(self.rarea),
                             _p(self.corio), _p(self.grndspd), _p(self.dfflen), _p(self.biharw), _p(self.smoo),
                             ctypes.byref(dmax))
        c = OrcCtx()
        c.nip, c.nvl, c.ntra = N, L, cfg.ntra
        c.prox, c.proxs, c.nprox = _p(prox), _p(proxs), _p(nprox)
        for n in ("cs", "sn", "sidevec_c", "sidevec_e", "sideln", "area", "hfcoef", "corner_xy"):
            setattr(c, n, _p(getattr(grid, n)))
        c.rarea, c.corio, c.grndspd = _p(self.rarea), _p(self.corio), _p(self.grndspd)
        c.dt, c.kbl, c.hi_order = cfg.dt, cfg.kbl, cfg.hi_order_flux_comp
        c.miglim, c.remap_optn = cfg.miglim, cfg.remap_optn
        c.flux_schm = cfg.flux_conserv_schm
        c.intfc_smooth, c.slak, c.ptop, c.thktop = cfg.intfc_smooth, cfg.slak, cfg.ptop, cfg.thktop
        c.rleigh, c.rlthresh, c.rltaper = cfg.rleigh, cfg.rlthresh, cfg.rltaper
        c.thetac, c.dpsig = _p(cfg.thetac), _p(cfg.dpsig)
        c.dfflen, c.biharw, c.smoo_coeff = _p(self.dfflen), _p(self.biharw), _p(self.smoo)
        c.dfflen_max = dmax.value
        c.nf, c.of, c.vof = -1, 1, 0
        c.ntrb = cfg.ntrb
        self.c = c
        self.N, self.L, self.T = N, L, cfg.ntra
        self.TB = cfg.ntrb

    @property
    def diag_flags(self):
        return self.c.diag_flags

    def abstart(self, its):
        self.lib.orc_abstart(ctypes.byref(self.c), its)

    def edgvar1(self, u, v, delp, pres, exner, geop, montg, tracr, u_edg, v_edg, dp_edg, lp_edg, geop_edg,
                mont_edg, uvsq_edg, trc_edg):
        self.lib.orc_edgvar1(ctypes.byref(self.c), *map(_p, (u, v, delp, pres, exner, geop, montg, tracr, u_edg,
                                                              v_edg, dp_edg, lp_edg, geop_edg, mont_edg, uvsq_edg,
                                                              trc_edg)))

    def edgvar3(self, delp, tracr, dp_edg, trc_edg):
        self.lib.orc_edgvar3(ctypes.byref(self.c), _p(delp), _p(tracr), _p(dp_edg), _p(trc_edg))

    def cnuity(self, u, v, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, dplo_tndcy, massfx, omega):
        self.lib.orc_cnuity(ctypes.byref(self.c), *map(_p, (u, v, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner,
                                                             dp_tndcy, dplo_tndcy, massfx, omega)))

    def mass_adv(self, u, v, u_edg, v_edg, dp_edg, lp_edg, delp, pres, exner, dp_tndcy, massfx, omega):
        self.lib.orc_mass_adv(ctypes.byref(self.c), *map(_p, (u, v, u_edg, v_edg, dp_edg, lp_edg, delp, pres,
                                                               exner, dp_tndcy, massfx, omega)))

    def trcadv(self, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp):
        self.lib.orc_trcadv(ctypes.byref(self.c), *map(_p, (trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx,
                                                             delp)))

    def momtum(self, u, v, exner, relvor, u_edg, v_edg, trc_edg, mont_edg, uvsq_edg, u_tndcy, v_tndcy, dp3d):
        self.lib.orc_momtum(ctypes.byref(self.c), *map(_p, (u, v, exner, relvor, u_edg, v_edg, trc_edg, mont_edg,
                                                             uvsq_edg, u_tndcy, v_tndcy, dp3d)))

    def hybgen(self, its, us3d, vs3d, tr3d, sdot, ex3d, dp3d, pr3d, targt=None):
        self.lib.orc_hybgen(ctypes.byref(self.c), its, _p(targt), *map(_p, (us3d, vs3d, tr3d, sdot, ex3d, dp3d,
                                                                             pr3d)))

    def edgvar2(self, u, v, u_edg, v_edg, uvsq_edg):
        self.lib.orc_edgvar2(ctypes.byref(self.c), *map(_p, (u, v, u_edg, v_edg, uvsq_edg)))

    def hystat(self, its, ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy):
        self.lib.orc_hystat(ctypes.byref(self.c), its, *map(_p, (ph3d, ex3d, mp3d, dp3d, tr3d, trdp, psrf, ptdcy)))

    def globsum(self, dp3d, tr, pr3d, ex3d, rn2d=None, rc2d=None, qf2d=None):
        qtrcr = np.zeros(self.T + self.TB)
        sums = np.zeros(8)
        self.lib.orc_globsum(ctypes.byref(self.c), _p(dp3d), _p(tr), _p(rn2d), _p(rc2d), _p(pr3d), _p(ex3d),
                             _p(qf2d), _p(qtrcr), _p(sums))
        names = ["qmass", "qmsqv", "qmsqw", "qmso3", "qmste", "qmstr", "qmstrn", "qmstrc"]
        return qtrcr, dict(zip(names, sums))

    def transp0(self, cumufx, dp3d, dpinit):
        self.lib.orc_transp0(ctypes.byref(self.c), _p(cumufx), _p(dp3d), _p(dpinit))

    def transp1(self, cumufx, massfx):
        self.lib.orc_transp1(ctypes.byref(self.c), _p(cumufx), _p(massfx))

    def transp2(self, tracr, cumufx, dpinit, dpfinl):
        self.lib.orc_transp2(ctypes.byref(self.c), self.TB, _p(tracr), _p(cumufx), _p(dpinit), _p(dpfinl))

    # ---- physics coupling (cpl_run.F90), GFS arrays (nip, nvl), cell fastest ----
    GFS_NAMES = ["ps", "dp", "p", "u", "v", "dpdt", "q", "oz", "cld", "t"]

    def cpl_dyn_to_phy(self, pr3d, us3d, vs3d, ws3d, tr3d):
        """cpl_dyn_to_phy (callphy): returns (gfs dict, old6)."""
        NL = self.N * self.L
        gfs = {n: np.zeros(self.N if n == "ps" else NL) for n in self.GFS_NAMES}
        old6 = np.zeros(6 * NL)
        self.lib.orc_cpl_dyn_to_phy(ctypes.byref(self.c), *map(_p, (pr3d, us3d, vs3d, ws3d, tr3d)),
                                    *[_p(gfs[n]) for n in self.GFS_NAMES], _p(old6))
        return gfs, old6

    def cpl_phy_to_dyn(self, gfs, old6, dp3d, us3d, vs3d, tr3d, geshem, rainc, evap, rn2d, rc2d, qf2d,
                       dtp, addtend=False, smoothtend=False):
        """cpl_phy_to_dyn (callphy): updates us3d, vs3d, tr3d[0:4], rn2d, rc2d, qf2d in place."""
        self.lib.orc_cpl_phy_to_dyn(ctypes.byref(self.c), int(addtend), int(smoothtend), float(dtp),
                                    *[_p(gfs[n]) for n in ("p", "u", "v", "q", "cld", "oz", "t")], _p(old6),
                                    *map(_p, (dp3d, us3d, vs3d, tr3d, geshem, rainc, evap, rn2d, rc2d, qf2d)))

    def prdp_from_ex(self, ex3d, pr3d, dp3d):
        self.lib.orc_prdp_from_ex(ctypes.byref(self.c), _p(ex3d), _p(pr3d), _p(dp3d))

    # ---- whole-state helpers mirroring fim_state_init / fim_step ----
    def new_state(self, fields):
        N, L, T = self.N, self.L, self.T
        z = lambda n: np.zeros(n)  # noqa: E731
        s = dict(trdp=z((T + self.TB) * N * L), cumufx=z(6 * N * L), dpinit=z(N * L), u_tdcy=z(3 * N * L), v_tdcy=z(3 * N * L), dp_tdcy=z(3 * N * L),
                 dpl_tdcy=z(3 * N * L), trc_tdcy=z(3 * T * N * L), trl_tdcy=z(3 * T * N * L),
                 massfx=z(18 * N * L), ws3d=z(N * L), sdot=z(N * (L + 1)), relvor=z(N * L), psrf=z(N),
                 ptdcy=z(2 * N), u_edg=z(6 * N * L), v_edg=z(6 * N * L), dp_edg=z(6 * N * L),
                 lp_edg=z(6 * N * L), mont_edg=z(6 * N * L), uvsq_edg=z(6 * N * L), geop_edg=z(6 * N * L),
                 trc_edg=z(6 * T * N * L))
        for k, v in fields.items():
            s[k] = np.array(v, dtype=np.float64, copy=True)
        return s

    def init_state(self, s):
        """dyn_init.F90:870-906,1037,1092-1094."""
        self.hybgen(0, s["us3d"], s["vs3d"], s["tr3d"], s["sdot"], s["ex3d"], s["dp3d"], s["pr3d"])
        self.prdp_from_ex(s["ex3d"], s["pr3d"], s["dp3d"])
        s["psrf"][:] = 0.0
        s["ptdcy"][:] = 0.0
        self.hystat(0, s["ph3d"], s["ex3d"], s["mp3d"], s["dp3d"], s["tr3d"], s["trdp"], s["psrf"], s["ptdcy"])
        if self.TB > 0:
            self.transp0(s["cumufx"], s["dp3d"], s["dpinit"])  # dyn_init.F90:1096-1097
        self.c.nf, self.c.of, self.c.vof = -1, 1, 0
        return s

    def step(self, s, its):
        """One dyn_run iteration (dyn_run.F90:119-425): hybgen and hystat of
        step its-1 (from the second step on), then the horizontal dynamics of
        step its; returns the budgets of the resulting state (globsum)."""
        self.abstart(its)
        if its > 1:
            self.hybgen(its - 1, s["us3d"], s["vs3d"], s["tr3d"], s["sdot"], s["ex3d"], s["dp3d"], s["pr3d"])
            self.hystat(its - 1, s["ph3d"], s["ex3d"], s["mp3d"], s["dp3d"], s["tr3d"], s["trdp"], s["psrf"],
                        s["ptdcy"])
        self.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"],
                     s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"],
                     s["trc_edg"])
        if getattr(self.cfg, "hi_order_uv_comp", 0):
            self.edgvar2(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["uvsq_edg"])
        if self.cfg.hi_order_flux_comp:
            self.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        if self.cfg.flux_conserv_schm == 1:
            self.cnuity(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["dp3d"],
                        s["pr3d"], s["ex3d"], s["dp_tdcy"], s["dpl_tdcy"], s["massfx"], s["ws3d"])
        else:
            self.mass_adv(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["dp3d"],
                          s["pr3d"], s["ex3d"], s["dp_tdcy"], s["massfx"], s["ws3d"])
        if self.TB > 0:  # class-B transport (dyn_run.F90:388-403)
            self.transp1(s["cumufx"], s["massfx"])
            if its % self.cfg.dtratio == 0:
                self.transp2(s["tr3d"], s["cumufx"], s["dpinit"], s["dp3d"])
                self.transp0(s["cumufx"], s["dp3d"], s["dpinit"])
        self.trcadv(s["trc_edg"], s["tr3d"], s["trdp"], s["trc_tdcy"], s["trl_tdcy"], s["massfx"], s["dp3d"])
        self.momtum(s["us3d"], s["vs3d"], s["ex3d"], s["relvor"], s["u_edg"], s["v_edg"], s["trc_edg"],
                    s["mont_edg"], s["uvsq_edg"], s["u_tdcy"], s["v_tdcy"], s["dp3d"])
        return self.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"])
