"""Physics coupling (cpl_run.F90), the dynamics side of phy_run: the C oracle
against a vectorised NumPy restatement of cpl_dyn_to_phy / cpl_phy_to_dyn
(cpl_run.F90:151-263, 266-536) and dffusn8_lyr (dffusn.F90:110-129), and the
dyn -> phy -> dyn round trip with the physics leaving its state unchanged."""
import numpy as np
import pytest

from helpers import make_case, oracle_for

RD, CP, P1000, QVMIN, QWMIN = 287.0586, 1004.6855, 100000.0, 1.e-10, 1.e-10


@pytest.fixture(scope="module")
def cpl_case():
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, seed=1300)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    rng = np.random.default_rng(1301)
    s["ws3d"][:] = rng.normal(0.0, 2.0, s["ws3d"].size)
    return grid, cfg, o, s


def np_dyn_to_phy(N, L, s):
    pr = s["pr3d"].reshape(N, L + 1)
    tr = s["tr3d"].reshape(-1, N, L)
    pk, pk1 = pr[:, :L], pr[:, 1:]
    a = RD / CP + 1.0
    q2 = np.maximum(QVMIN, tr[1])
    p = ((pk ** a - pk1 ** a) / ((pk - pk1) * a)) ** (CP / RD)
    t = tr[0] / (1.0 + 0.6078 * np.maximum(QVMIN, q2)) * (p / P1000) ** (RD / CP)
    g = dict(ps=0.001 * pr[:, 0], dp=0.001 * pk - 0.001 * pk1, p=p, u=s["us3d"].reshape(N, L),
             v=s["vs3d"].reshape(N, L), dpdt=0.001 * s["ws3d"].reshape(N, L), q=q2, oz=tr[3], cld=tr[2], t=t)
    # GFS layout (nip, nvl), cell fastest
    return {k: (v if k == "ps" else v.T).ravel() for k, v in g.items()}


def np_dffusn8_lyr(o, fld, delp, dfflen):
    N, L = o.N, o.L
    prox = np.asarray(o.grid.prox).reshape(N, 6) - 1
    npx = np.asarray(o.grid.nprox)
    sl = np.asarray(o.grid.sideln).reshape(N, 6)
    rarea = 1.0 / np.asarray(o.grid.area)
    d = np.maximum(delp.reshape(N, L), 1.e-11)
    f = fld.reshape(N, L)
    flx = np.zeros((N, L))
    for e in range(6):
        live = (e < npx)[:, None]
        x = prox[:, e]
        h = d * d[x] / (d + d[x])
        flx = flx + np.where(live, (f - f[x]) * sl[:, e:e + 1] * 2.0 * h, 0.0)
    return (f + flx * (-dfflen * rarea[:, None] / d)).ravel()


def np_phy_to_dyn(o, gfs, old6, dp3d, dtp, addtend, smoothtend):
    N, L, dt = o.N, o.L, o.c.dt
    G = lambda a: a.reshape(L, N).T  # noqa: E731  (nip, nvl) -> (N, L)
    old = [G(old6[j * N * L:(j + 1) * N * L]) for j in range(6)]  # u, v, t, q, oz, cld
    now = dict(u=G(gfs["u"]), v=G(gfs["v"]), t=G(gfs["t"]), q=G(gfs["q"]), cld=G(gfs["cld"]), oz=G(gfs["oz"]))
    p = G(gfs["p"])
    kap = RD / CP
    if addtend:
        td = {k: (now[k] - old[j]) / dtp for k, j in (("u", 0), ("v", 1), ("t", 2), ("q", 3), ("cld", 5), ("oz", 4))}
        if smoothtend:
            td = {k: np_dffusn8_lyr(o, v.ravel(), dp3d, dt * 20.0).reshape(N, L) for k, v in td.items()}
        u, v = old[0] + td["u"] * dt, old[1] + td["v"] * dt
        q = old[3] + td["q"] * dt
        th = (old[2] + td["t"] * dt) * (P1000 / p) ** kap * (1.0 + 0.6078 * np.maximum(QVMIN, q))
        t2, t3, t4 = np.maximum(QVMIN, q), np.maximum(QWMIN, old[5] + td["cld"] * dt), \
            np.maximum(QVMIN, old[4] + td["oz"] * dt)
    else:
        u, v = now["u"], now["v"]
        th = now["t"] * (P1000 / p) ** kap * (1.0 + 0.6078 * np.maximum(QVMIN, now["q"]))
        t2, t3, t4 = np.maximum(QVMIN, now["q"]), np.maximum(QWMIN, now["cld"]), np.maximum(QVMIN, now["oz"])
    return u.ravel(), v.ravel(), [th.ravel(), t2.ravel(), t3.ravel(), t4.ravel()]


def physics_perturbation(o, gfs, seed):
    """Stand-in for phy_run: small seeded changes of the GFS state."""
    rng = np.random.default_rng(seed)
    g = {k: v.copy() for k, v in gfs.items()}
    g["u"] += rng.normal(0.0, 0.2, g["u"].size)
    g["v"] += rng.normal(0.0, 0.2, g["v"].size)
    g["t"] += rng.normal(0.0, 0.3, g["t"].size)
    g["q"] *= 1.0 + rng.normal(0.0, 0.01, g["q"].size)
    g["cld"] += rng.uniform(-2e-3, 1e-3, g["cld"].size)  # some below the floor
    g["oz"] *= 1.0 + rng.normal(0.0, 0.01, g["oz"].size)
    col = dict(geshem=rng.uniform(-1e-4, 1e-3, o.N), rainc=rng.uniform(-1e-4, 5e-4, o.N),
               evap=rng.normal(0.0, 1e-5, o.N))
    return g, col


def test_cpl_dyn_to_phy_oracle(cpl_case):
    grid, cfg, o, s = cpl_case
    gfs, old6 = o.cpl_dyn_to_phy(s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"])
    ref = np_dyn_to_phy(o.N, o.L, s)
    for k in o.GFS_NAMES:
        np.testing.assert_allclose(gfs[k], ref[k], rtol=1e-12, atol=1e-300, err_msg=k)
    NL = o.N * o.L
    for j, k in enumerate(["u", "v", "t", "q", "oz", "cld"]):
        assert np.array_equal(old6[j * NL:(j + 1) * NL], gfs[k]), k
    # layer pressure lies inside its layer
    pr = s["pr3d"].reshape(o.N, o.L + 1)
    p = gfs["p"].reshape(o.L, o.N).T
    assert np.all(p < pr[:, :-1]) and np.all(p > pr[:, 1:])


@pytest.mark.parametrize("addtend,smoothtend", [(False, False), (True, False), (True, True)])
def test_cpl_phy_to_dyn_oracle(cpl_case, addtend, smoothtend):
    grid, cfg, o, s = cpl_case
    gfs, old6 = o.cpl_dyn_to_phy(s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"])
    g, col = physics_perturbation(o, gfs, 1302)
    u, v, tr = s["us3d"].copy(), s["vs3d"].copy(), s["tr3d"].copy()
    rn, rc, qf = np.full(o.N, 0.5), np.full(o.N, 0.25), np.zeros(o.N)
    dtp = 2.0 * o.c.dt
    o.cpl_phy_to_dyn(g, old6, s["dp3d"], u, v, tr, col["geshem"], col["rainc"], col["evap"], rn, rc, qf, dtp,
                     addtend, smoothtend)
    ru, rv, rt = np_phy_to_dyn(o, g, old6, s["dp3d"], dtp, addtend, smoothtend)
    np.testing.assert_allclose(u, ru, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(v, rv, rtol=1e-12, atol=1e-12)
    NL = o.N * o.L
    for t in range(4):
        np.testing.assert_allclose(tr[t * NL:(t + 1) * NL], rt[t], rtol=1e-12, atol=1e-20, err_msg=str(t))
    assert np.array_equal(tr[4 * NL:], s["tr3d"][4 * NL:])  # tracers 5.. untouched
    np.testing.assert_allclose(rn, 0.5 + np.maximum(0.0, col["geshem"]) * 1000.0, rtol=1e-15)
    np.testing.assert_allclose(rc, 0.25 + np.maximum(0.0, col["rainc"]) * 1000.0, rtol=1e-15)
    assert np.array_equal(qf, -col["evap"])


def test_cpl_round_trip(cpl_case):
    """No physics change: u and v come back exactly, theta to rounding, the
    moisture tracers with their floors."""
    grid, cfg, o, s = cpl_case
    gfs, old6 = o.cpl_dyn_to_phy(s["pr3d"], s["us3d"], s["vs3d"], s["ws3d"], s["tr3d"])
    u, v, tr = np.zeros_like(s["us3d"]), np.zeros_like(s["vs3d"]), s["tr3d"].copy()
    z = np.zeros(o.N)
    o.cpl_phy_to_dyn(gfs, old6, s["dp3d"], u, v, tr, z, z, z, z.copy(), z.copy(), z.copy(), o.c.dt)
    assert np.array_equal(u, s["us3d"]) and np.array_equal(v, s["vs3d"])
    NL = o.N * o.L
    np.testing.assert_allclose(tr[:NL], s["tr3d"][:NL], rtol=1e-13)
    assert np.array_equal(tr[NL:2 * NL], np.maximum(QVMIN, s["tr3d"][NL:2 * NL]))
    assert np.array_equal(tr[2 * NL:3 * NL], np.maximum(QWMIN, s["tr3d"][2 * NL:3 * NL]))
