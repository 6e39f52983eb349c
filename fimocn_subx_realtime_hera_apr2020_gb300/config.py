"""Dycore configuration (the namelist knobs on the path) and the workloads.

Defaults are the reference's (FIMsrc/cntl/fimnamelist.F90:95-119) with
flux_conserv_schm = 1 (the FCT cnuity) because that is the scheme this build
provides.  Vertical tables (hybgen targets and minimum thicknesses) come from
data/vertical_tables.json, extracted from the reference's run configuration.
"""
import ctypes
import json
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib

_HERE = os.path.dirname(os.path.abspath(__file__))


def vertical_tables(nvl):
    with open(os.path.join(_HERE, "data", "vertical_tables.json")) as fh:
        d = json.load(fh)
    if str(nvl) not in d:
        raise ValueError("no vertical tables for nvl=%d (have %s)" % (nvl, sorted(d)))
    return np.array(d[str(nvl)]["thetac"], np.float64), np.array(d[str(nvl)]["dpsig"], np.float64)


def default_dt(glvl):
    """Time step of FIMsrc/cntl/module_control.F90:220 for bisected grids."""
    return 1.2 * 4800.0 / 2 ** (glvl - 1)


@dataclass
class FimConfig:
    nvl: int
    ntra: int
    dt: float
    precision: str = "f64"          # "f64" or "f32" (FP32-mixed)
    members: int = 1
    host_pointers: bool = False
    kbl: int = 2
    flux_conserv_schm: int = 1
    hi_order_flux_comp: int = 1
    intfc_smooth: float = 30.0
    slak: float = 0.5
    miglim: int = 1
    remap_optn: int = 2
    ptop: float = 30.0
    thktop: float = 30.0
    veldff_bkgnd: float = 0.3
    veldff_boost: float = 3.0
    biharm_frst: int = 0
    biharm_last: int = 0
    rleigh: float = 2.0
    rlthresh: float = 90.0
    rltaper: float = 0.4
    pure_sig: int = 0
    ntrb: int = 0                   # class-B tracers (transported every dtratio steps by fct3d)
    dtratio: int = 6
    member_group: int = 0           # members advanced together through the dynamics (0: all)
    hi_order_uv_comp: int = 0       # hiOrderUVComp: edgvar2 after edgvar1 in the step
    stream_priority: int = 0        # CUDA priority of the context's streams (lower runs first)
    tracer_chunk: int = 0           # tracers per launch of the fused tracer kernels (0: auto)
    thetac: np.ndarray = field(default=None, repr=False)
    dpsig: np.ndarray = field(default=None, repr=False)

    def __post_init__(self):
        if self.thetac is None or self.dpsig is None:
            th, dp = vertical_tables(self.nvl)
            if self.thetac is None:
                self.thetac = th
            if self.dpsig is None:
                self.dpsig = dp
        self.thetac = np.ascontiguousarray(self.thetac, np.float64)
        self.dpsig = np.ascontiguousarray(self.dpsig, np.float64)

    @property
    def dtype(self):
        return np.float64 if self.precision == "f64" else np.float32

    def to_c(self):
        c = _lib.Config()
        for name, _ in _lib.Config._fields_:
            if name in ("thetac", "dpsig", "precision", "host_pointers"):
                continue
            setattr(c, name, getattr(self, name))
        c.precision = _lib.FIM_PREC_F64 if self.precision == "f64" else _lib.FIM_PREC_F32
        c.host_pointers = 1 if self.host_pointers else 0
        c.thetac = self.thetac.ctypes.data
        c.dpsig = self.dpsig.ctypes.data
        return c


# Workloads of the benchmark configurations (synthetic balanced states).
WORKLOADS = {
    "glvl4_nvl38_t4": dict(glvl=4, nvl=38, ntra=5, dt=400.0, sigma_ps=200.0, noise=0.0, seed=1000),
    "glvl6_nvl64_t10": dict(glvl=6, nvl=64, ntra=11, dt=180.0, sigma_ps=200.0, noise=1.0, seed=2000),
    # FIM's own glvl-8 step (module_control.F90:220, 45 s); 72 s makes the
    # reference algorithm itself diverge within ~10 steps (AB3 gravity-wave limit)
    "glvl8_nvl64_t20": dict(glvl=8, nvl=64, ntra=21, dt=45.0, sigma_ps=200.0, noise=0.0, seed=3000),
    # 32 members do not fit in HBM with a full set of step work fields each:
    # the dynamics run in groups of 8 members
    "glvl7_nvl64_t10_x32": dict(glvl=7, nvl=64, ntra=11, dt=default_dt(7), sigma_ps=100.0, noise=0.5,
                                seed=4000, members=32, member_group=8),
}
