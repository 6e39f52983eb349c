"""Physics coupling on the GPU (fim_cpl_dyn_to_phy / fim_cpl_phy_to_dyn)
against the CPU oracle, both precisions, device and host pointers."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300._lib import FIM_EINVAL, FimError  # noqa: E402
from helpers import make_case, oracle_for, rel_l2  # noqa: E402
from test_cpl import physics_perturbation  # noqa: E402

pytestmark = pytest.mark.gpu

# FP64: the oracle's operations; FP32: inputs in FP32, the layer pressure from
# the cancellation-free form, so well inside the FP32-mixed bar
TOL = {"f64": 1e-12, "f32": 1e-5}
DYN = ("pr3d", "us3d", "vs3d", "ws3d", "tr3d", "dp3d")


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def _case(precision, seed, **kw):
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, seed=seed, precision=precision, **kw)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    s["ws3d"][:] = np.random.default_rng(seed + 1).normal(0.0, 2.0, s["ws3d"].size)
    if precision == "f32":
        # the FP32 context holds FP32 fields: give the oracle the same values
        for k in DYN:
            s[k] = s[k].astype(np.float32).astype(np.float64)
    return grid, cfg, o, s


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("addtend,smoothtend", [(False, False), (True, False), (True, True)])
def test_cpl_matches_oracle(precision, addtend, smoothtend):
    grid, cfg, o, s = _case(precision, 1310)
    rt = torch.float32 if precision == "f32" else torch.float64
    N, L, NL = grid.nip, cfg.nvl, grid.nip * cfg.nvl
    dyc = F.Dycore(grid, cfg)
    d = {k: dev(s[k], rt) for k in DYN}
    gfs = {n: torch.zeros(N if n == "ps" else NL, dtype=torch.float64, device="cuda") for n in F.Dycore.GFS_NAMES}
    dyc.cpl_dyn_to_phy(1, d["pr3d"], d["us3d"], d["vs3d"], d["ws3d"], d["tr3d"], gfs)
    og, old6 = o.cpl_dyn_to_phy(s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"])
    for n in F.Dycore.GFS_NAMES:
        assert rel_l2(host(gfs[n]), og[n]) <= TOL[precision], n
    # the same physics stand-in on both sides
    pg, col = physics_perturbation(o, og, 1312)
    for n in pg:
        gfs[n].copy_(torch.from_numpy(pg[n]))
    dtp = 2.0 * cfg.dt
    u, v, tr = s["us3d"].copy(), s["vs3d"].copy(), s["tr3d"].copy()
    rn, rc, qf = np.full(N, 0.5), np.full(N, 0.25), np.zeros(N)
    o.cpl_phy_to_dyn(pg, old6, s["dp3d"], u, v, tr, col["geshem"], col["rainc"], col["evap"], rn, rc, qf, dtp,
                     addtend, smoothtend)
    dcol = {k: dev(col[k]) for k in col}
    drn, drc, dqf = dev(np.full(N, 0.5), rt), dev(np.full(N, 0.25), rt), dev(np.zeros(N), rt)
    dyc.cpl_phy_to_dyn(1, gfs, dcol["geshem"], dcol["rainc"], dcol["evap"], d["dp3d"], d["us3d"], d["vs3d"],
                       d["tr3d"], drn, drc, dqf, dtp, addtend, smoothtend)
    assert rel_l2(host(d["us3d"]), u) <= TOL[precision]
    assert rel_l2(host(d["vs3d"]), v) <= TOL[precision]
    gt = host(d["tr3d"])
    for t in range(4):
        assert rel_l2(gt[t * NL:(t + 1) * NL], tr[t * NL:(t + 1) * NL]) <= TOL[precision], t
    assert np.array_equal(gt[4 * NL:], s["tr3d"][4 * NL:])
    for a, b in ((drn, rn), (drc, rc), (dqf, qf)):
        assert rel_l2(host(a), b) <= TOL[precision]


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_cpl_round_trip(precision):
    """No physics change: winds come back exactly, theta to rounding."""
    grid, cfg, o, s = _case(precision, 1320)
    rt = torch.float32 if precision == "f32" else torch.float64
    N, NL = grid.nip, grid.nip * cfg.nvl
    dyc = F.Dycore(grid, cfg)
    d = {k: dev(s[k], rt) for k in DYN}
    gfs = {n: torch.zeros(N if n == "ps" else NL, dtype=torch.float64, device="cuda") for n in F.Dycore.GFS_NAMES}
    dyc.cpl_dyn_to_phy(1, d["pr3d"], d["us3d"], d["vs3d"], d["ws3d"], d["tr3d"], gfs)
    u, v, tr = torch.zeros_like(d["us3d"]), torch.zeros_like(d["vs3d"]), d["tr3d"].clone()
    z = dev(np.zeros(N))
    dyc.cpl_phy_to_dyn(1, gfs, z, z, z, d["dp3d"], u, v, tr, dev(np.zeros(N), rt), dev(np.zeros(N), rt),
                       dev(np.zeros(N), rt), cfg.dt)
    assert np.array_equal(host(u), host(d["us3d"])) and np.array_equal(host(v), host(d["vs3d"]))
    th = host(tr)[:NL]
    np.testing.assert_allclose(th, s["tr3d"][:NL], rtol=1e-13 if precision == "f64" else 1e-6)


def test_cpl_host_pointers_and_callphy():
    grid, cfg, o, s = _case("f64", 1330, host_pointers=True)
    N, NL = grid.nip, grid.nip * cfg.nvl
    dyc = F.Dycore(grid, cfg)
    gfs = {n: np.zeros(N if n == "ps" else NL) for n in F.Dycore.GFS_NAMES}
    dyc.cpl_dyn_to_phy(1, s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"], gfs, callphy=False)
    assert not any(np.any(v) for v in gfs.values())  # callphy = 0: nothing happens
    # addtend needs the copies a preceding cpl_dyn_to_phy keeps
    z = np.zeros(N)
    with pytest.raises(FimError) as err:
        dyc.cpl_phy_to_dyn(1, gfs, z, z, z, s["dp3d"], s["us3d"].copy(), s["vs3d"].copy(), s["tr3d"].copy(),
                           z.copy(), z.copy(), z.copy(), cfg.dt, addtend=True)
    assert err.value.code == FIM_EINVAL
    dyc.cpl_dyn_to_phy(1, s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"], gfs)
    og, old6 = o.cpl_dyn_to_phy(s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"])
    for n in F.Dycore.GFS_NAMES:
        assert rel_l2(gfs[n], og[n]) <= 1e-12, n
