"""Shared helpers of the test suite: cases, oracle states, error norms."""
import numpy as np

import fimocn_subx_realtime_hera_apr2020_gb300 as F
from oracle import Oracle


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    n = np.linalg.norm(b)
    d = np.linalg.norm(a - b)
    return d / n if n > 0 else d


def make_case(glvl=3, nvl=38, ntra=5, dt=None, seed=1000, sigma_ps=200.0, noise=1.0, precision="f64", **kw):
    grid = F.Grid.cached(glvl)
    cfg = F.FimConfig(nvl=nvl, ntra=ntra, dt=dt if dt else F.default_dt(glvl), precision=precision, **kw)
    fields = F.synthetic_state(grid, cfg, seed=seed, sigma_ps=sigma_ps, noise=noise)
    return grid, cfg, fields


def oracle_for(grid, cfg):
    ocfg = F.FimConfig(**{k: getattr(cfg, k) for k in cfg.__dataclass_fields__})
    ocfg.precision = "f64"
    ocfg.members = 1
    ocfg.host_pointers = False
    return Oracle(grid, ocfg)


PROGNOSTIC = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp"]
