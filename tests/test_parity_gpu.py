"""GPU parity: every routine and the fused step against the CPU oracle.

FP64 path: relative L2 per field <= 1e-12 after one step (the parity bar).
FP32-mixed path: relative L2 per prognostic field <= 1e-5 after one step.
All calls go through the C-ABI (libfimgpu.so) via the package's host mirror.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from helpers import PROGNOSTIC, make_case, oracle_for, rel_l2  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300._lib import FimError  # noqa: E402

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


@pytest.fixture(scope="module")
def case4():
    """Level-4 grid, nvl 38, 4 tracers + theta, noisy wind (the CPU-sized workload)."""
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1000, noise=1.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    return grid, cfg, fields, o, s


def test_routines_fp64(case4):
    """Each routine fed the oracle's inputs reproduces the oracle's outputs."""
    grid, cfg, fields, o0, s0 = case4
    o = oracle_for(grid, cfg)
    s = {k: v.copy() for k, v in s0.items()}
    dyc = F.Dycore(grid, cfg)
    errs = {}
    for its in range(1, 5):
        o.abstart(its)
        dyc.set_ab(o.c.nf + 1, o.c.of + 1, o.c.vof + 1, o.c.ab1, o.c.ab2, o.c.ab3)
        # edgvar1
        names = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "u_edg", "v_edg", "dp_edg",
                 "lp_edg", "geop_edg", "mont_edg", "uvsq_edg", "trc_edg"]
        g = {n: dev(s[n]) for n in names}
        o.edgvar1(*[s[n] for n in names])
        dyc.edgvar1(its, *[g[n] for n in names])
        for n in ["u_edg", "v_edg", "lp_edg", "mont_edg", "uvsq_edg", "trc_edg"]:
            errs[("edgvar1", n)] = max(errs.get(("edgvar1", n), 0), rel_l2(host(g[n]), s[n]))
        # edgvar3
        g = {n: dev(s[n]) for n in names}
        o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        dyc.edgvar3(its, *[g[n] for n in names])
        for n in ["dp_edg", "trc_edg"]:
            errs[("edgvar3", n)] = max(errs.get(("edgvar3", n), 0), rel_l2(host(g[n]), s[n]))
        # cnuity
        names = ["us3d", "vs3d", "u_edg", "v_edg", "dp_edg", "lp_edg", "dp3d", "pr3d", "ex3d", "dp_tdcy",
                 "dpl_tdcy", "massfx", "ws3d"]
        g = {n: dev(s[n]) for n in names}
        o.cnuity(*[s[n] for n in names])
        dyc.cnuity(its, *[g[n] for n in names])
        for n in ["dp3d", "pr3d", "ex3d", "dp_tdcy", "dpl_tdcy", "massfx", "ws3d"]:
            errs[("cnuity", n)] = max(errs.get(("cnuity", n), 0), rel_l2(host(g[n]), s[n]))
        # trcadv
        names = ["trc_edg", "tr3d", "trdp", "trc_tdcy", "trl_tdcy", "massfx", "dp3d"]
        g = {n: dev(s[n]) for n in names}
        o.trcadv(*[s[n] for n in names])
        dyc.trcadv(its, *[g[n] for n in names])
        for n in ["tr3d", "trdp", "trc_tdcy", "trl_tdcy"]:
            errs[("trcadv", n)] = max(errs.get(("trcadv", n), 0), rel_l2(host(g[n]), s[n]))
        # momtum
        onames = ["us3d", "vs3d", "ex3d", "relvor", "u_edg", "v_edg", "trc_edg", "mont_edg", "uvsq_edg",
                  "u_tdcy", "v_tdcy", "dp3d"]
        g = {n: dev(s[n]) for n in onames + ["geop_edg"]}
        o.momtum(*[s[n] for n in onames])
        dyc.momtum(its, g["us3d"], g["vs3d"], g["ex3d"], g["relvor"], g["u_edg"], g["v_edg"], g["trc_edg"],
                   g["geop_edg"], g["mont_edg"], g["uvsq_edg"], g["u_tdcy"], g["v_tdcy"], g["dp3d"])
        for n in ["us3d", "vs3d", "relvor", "u_tdcy", "v_tdcy"]:
            errs[("momtum", n)] = max(errs.get(("momtum", n), 0), rel_l2(host(g[n]), s[n]))
        # hybgen
        names = ["us3d", "vs3d", "tr3d", "sdot", "ex3d", "dp3d", "pr3d"]
        g = {n: dev(s[n]) for n in names}
        o.hybgen(its, *[s[n] for n in names])
        dyc.hybgen(its, None, *[g[n] for n in names])
        for n in ["us3d", "vs3d", "tr3d", "ex3d", "dp3d", "pr3d"]:
            errs[("hybgen", n)] = max(errs.get(("hybgen", n), 0), rel_l2(host(g[n]), s[n]))
        # hystat
        names = ["ph3d", "ex3d", "mp3d", "dp3d", "tr3d", "trdp", "psrf", "ptdcy"]
        g = {n: dev(s[n]) for n in names}
        o.hystat(its, *[s[n] for n in names])
        dyc.hystat(its, *[g[n] for n in names])
        for n in ["ph3d", "mp3d", "tr3d", "trdp", "psrf"]:
            errs[("hystat", n)] = max(errs.get(("hystat", n), 0), rel_l2(host(g[n]), s[n]))
        # globsum
        qo, bo = o.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"])
        qg, bg = dyc.globsum(its, dev(s["dp3d"]), dev(s["tr3d"]), dev(s["pr3d"]), dev(s["ex3d"]))
        errs[("globsum", "qtrcr")] = max(errs.get(("globsum", "qtrcr"), 0), rel_l2(qg, qo))
        errs[("globsum", "qmass")] = max(errs.get(("globsum", "qmass"), 0), abs(bg["qmass"] / bo["qmass"] - 1))
    bad = {k: v for k, v in errs.items() if not v <= TOL64}
    assert not bad, bad


def collapse_layers(s, N, L, every=7, k0=12, nl=3):
    """Layers k0 .. k0+nl-1 of every `every`-th column made massless (their
    interfaces moved onto interface k0), with pr3d, ex3d and dp3d consistent."""
    pr = s["pr3d"].reshape(N, L + 1)
    ex = s["ex3d"].reshape(N, L + 1)
    cols = np.arange(0, N, every)
    for j in range(1, nl + 1):
        pr[cols, k0 + j] = pr[cols, k0]
        ex[cols, k0 + j] = ex[cols, k0]
    s["dp3d"].reshape(N, L)[:] = pr[:, :L] - pr[:, 1:]


@pytest.mark.parametrize("precision,tol", [("f64", TOL64), ("f32", TOL32)])
def test_hybgen_massless_layers(precision, tol):
    """remap_1d on columns with massless layers and thktop = 0: pcwise's
    massless-layer fills and the tracer fill from above (hybgen.F90:672-680)
    both act, over two successive regrid/remap passes (the second pass starts
    from the massless layers the first one leaves)."""
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1001, noise=1.0, thktop=0.0,
                                  precision=precision)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    collapse_layers(s, grid.nip, cfg.nvl)
    dyc = F.Dycore(grid, cfg)
    dt = torch.float64 if precision == "f64" else torch.float32
    names = ["us3d", "vs3d", "tr3d", "sdot", "ex3d", "dp3d", "pr3d"]
    errs = {}
    for its in (1, 2):
        g = {n: dev(s[n], dt) for n in names}
        o.hybgen(its, *[s[n] for n in names])
        dyc.hybgen(its, None, *[g[n] for n in names])
        for n in ["us3d", "vs3d", "tr3d", "ex3d", "dp3d", "pr3d"]:
            errs[(its, n)] = rel_l2(host(g[n]), s[n])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, bad


def _gpu_state(grid, cfg, fields, members=1, member_fields=None):
    dyc = F.Dycore(grid, cfg)
    st = dyc.state()
    for m in range(members):
        st.load(member_fields[m] if member_fields else fields, member=m)
    st.init()
    return dyc, st


def test_state_init_fp64(case4):
    grid, cfg, fields, o, s = case4
    dyc, st = _gpu_state(grid, cfg, fields)
    for n in PROGNOSTIC:
        assert rel_l2(st.download(n), s[n]) <= TOL64, n


def test_fused_step_fp64(case4):
    grid, cfg, fields, o0, s0 = case4
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc, st = _gpu_state(grid, cfg, fields)
    for its in range(1, 4):
        qo, bo = o.step(s, its)
        st.step(its)
        # steps 2 and 3 add hybgen/hystat of the previous step, AB2 and AB3
        errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC + ["ws3d", "relvor", "sdot"]}
        bad = {k: v for k, v in errs.items() if not v <= TOL64}
        assert not bad, (its, bad)
        qg, bg = st.budget()
        assert abs(bg["qmass"] / bo["qmass"] - 1) < 1e-12
        assert rel_l2(qg, qo) < 1e-11
    rc, flags = st.check()
    assert rc == 0 and flags == 0


@pytest.mark.parametrize("precision,steps,tol", [("f64", 3, TOL64), ("f32", 1, TOL32)])
def test_fused_step_odd_nvl(precision, steps, tol):
    """nvl 37: one level a thread in every kernel, and level tiles of the
    tracer kernels that the column height does not fill."""
    th, dp = F.vertical_tables(38)
    grid, cfg, fields = make_case(glvl=3, nvl=37, ntra=5, dt=400.0, seed=37, noise=1.0, precision=precision,
                                  thetac=th[:37], dpsig=dp[:37])
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc, st = _gpu_state(grid, cfg, fields)
    for its in range(1, steps + 1):
        o.step(s, its)
        st.step(its)
        errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC}
        bad = {k: v for k, v in errs.items() if not v <= tol}
        assert not bad, (its, bad)
    rc, flags = st.check()
    assert rc == 0 and flags == 0


def test_graph_replay_matches_direct(case4):
    grid, cfg, fields, _, _ = case4
    d1, s1 = _gpu_state(grid, cfg, fields)
    d2, s2 = _gpu_state(grid, cfg, fields)
    for its in range(1, 5):
        s1.step(its, use_graph=False)
        s2.step(its, use_graph=True)
    for n in PROGNOSTIC:
        assert np.array_equal(s1.download(n), s2.download(n)), n


def test_members_independent():
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=11, noise=1.0)
    f2 = F.synthetic_state(grid, cfg, seed=12, sigma_ps=100.0, noise=0.5)
    cfg3 = F.FimConfig(nvl=38, ntra=5, dt=400.0, members=2)
    d, st = _gpu_state(grid, cfg3, None, members=2, member_fields=[fields, f2])
    da, sa = _gpu_state(grid, F.FimConfig(nvl=38, ntra=5, dt=400.0), fields)
    db, sb = _gpu_state(grid, F.FimConfig(nvl=38, ntra=5, dt=400.0), f2)
    for its in (1, 2, 3):
        st.step(its)
        sa.step(its)
        sb.step(its)
    for n in PROGNOSTIC:
        assert np.array_equal(st.download(n, 0), sa.download(n)), n
        assert np.array_equal(st.download(n, 1), sb.download(n)), n


@pytest.mark.parametrize("group", [2, 3])
def test_member_groups_match_one_batch(group):
    """member_group < members runs the dynamics group by group with the edge
    work fields held for one group: bit-identical to one batch of all."""
    grid = F.Grid.cached(3)
    mk = lambda **kw: F.FimConfig(nvl=38, ntra=5, dt=400.0, precision="f32", members=4, **kw)  # noqa: E731
    fields = [F.synthetic_state(grid, mk(), seed=60 + m, sigma_ps=150.0, noise=0.5, dtype=np.float32)
              for m in range(4)]
    d1, s1 = _gpu_state(grid, mk(), None, members=4, member_fields=fields)
    d2, s2 = _gpu_state(grid, mk(member_group=group), None, members=4, member_fields=fields)
    for its in (1, 2, 3):
        s1.step(its, use_graph=True)
        s2.step(its, use_graph=True)
    for m in range(4):
        for n in PROGNOSTIC + ["massfx", "trc_tdcy", "u_tdcy"]:
            assert np.array_equal(s2.download(n, m), s1.download(n, m)), (m, n)
    with pytest.raises(F._lib.FimError):
        s2.download("u_edg", 3)


def test_fp32_mixed_one_step(case4):
    grid, cfg, fields, o0, s0 = case4
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    cfg32 = F.FimConfig(nvl=cfg.nvl, ntra=cfg.ntra, dt=cfg.dt, precision="f32")
    dyc, st = _gpu_state(grid, cfg32, fields)
    for n in PROGNOSTIC:
        assert rel_l2(st.download(n), s[n]) <= TOL32, ("init", n)
    o.step(s, 1)
    st.step(1)
    errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC}
    bad = {k: v for k, v in errs.items() if not v <= TOL32}
    assert not bad, bad


@pytest.mark.parametrize("precision,tol", [("f64", TOL64), ("f32", TOL32)])
def test_one_step_glvl5_nvl64(precision, tol):
    """One step at the benchmark's column height: glvl 5 (10,242 cells),
    nvl 64, 10 tracers + theta, noisy wind; every prognostic field against
    the FP64 oracle.  nvl 64 selects the remap's two-columns-per-warp FP32
    layout and its 2-levels-per-lane FP64 layout at full column height."""
    grid, cfg, fields = make_case(glvl=5, nvl=64, ntra=11, dt=240.0, seed=2005, noise=1.0, precision=precision)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc, st = _gpu_state(grid, cfg, fields)
    o.step(s, 1)
    st.step(1, use_graph=True)
    errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC}
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, bad
    # the step after: hybgen and hystat of step 1 open it
    o.step(s, 2)
    st.step(2, use_graph=True)
    if precision == "f64":
        errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC}
        bad = {k: v for k, v in errs.items() if not v <= tol}
        assert not bad, bad
    rc, flags = st.check()
    assert rc == 0 and flags == 0


def test_fp32_mixed_mass_conservation(case4):
    """FP32-mixed global mass (globsum qmass) over 40 steps stays within 2e-7 of
    its value after the first step, as the FP64 oracle's does to rounding: the
    remap recomputes the pressures of unmoved interfaces exactly as they were
    formed, so the layer thicknesses keep summing to the column mass."""
    grid, cfg, fields, o0, s0 = case4
    cfg32 = F.FimConfig(nvl=cfg.nvl, ntra=cfg.ntra, dt=cfg.dt, precision="f32")
    dyc, st = _gpu_state(grid, cfg32, fields)
    st.step(1)
    q1 = st.budget()[1]["qmass"]
    for its in range(2, 41):
        st.step(its)
    q = st.budget()[1]["qmass"]
    assert abs(q / q1 - 1) < 2e-7, q / q1 - 1
    # hybgen's column-integral checks (FP32 tolerance) never fired
    rc, flags = st.check()
    assert rc == 0 and flags == 0, flags


def test_host_pointer_mode(case4):
    """host_pointers=1 stages numpy arrays through the device; same results."""
    grid, cfg, fields, o0, s0 = case4
    cfgh = F.FimConfig(nvl=cfg.nvl, ntra=cfg.ntra, dt=cfg.dt, host_pointers=True)
    dh = F.Dycore(grid, cfgh)
    dd = F.Dycore(grid, cfg)
    s = {k: v.copy() for k, v in s0.items()}
    for d in (dh, dd):
        d.abstart(1)
    names = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "u_edg", "v_edg", "dp_edg",
             "lp_edg", "geop_edg", "mont_edg", "uvsq_edg", "trc_edg"]
    hs = {n: s[n].copy() for n in names}
    gs = {n: dev(s[n]) for n in names}
    dh.edgvar1(1, *[hs[n] for n in names])
    dd.edgvar1(1, *[gs[n] for n in names])
    for n in ["u_edg", "v_edg", "lp_edg", "trc_edg"]:
        assert np.array_equal(hs[n], host(gs[n])), n


def test_fused_step_matches_routine_sequence(case4):
    """fim_step (fused tracer kernels, graph) == the per-routine entry points
    called in dyn_run order on the same state, bit for bit."""
    grid, cfg, fields, o0, s0 = case4
    dyc, st = _gpu_state(grid, cfg, fields)
    d2 = F.Dycore(grid, cfg)
    names = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "u_tdcy", "v_tdcy",
             "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy", "massfx", "ws3d", "sdot", "relvor", "psrf", "ptdcy",
             "u_edg", "v_edg", "dp_edg", "lp_edg", "mont_edg", "uvsq_edg", "geop_edg", "trc_edg"]
    g = {n: dev(st.download(n)) for n in names}
    # the routines take the reference's trc_edg of every tracer; the fused
    # step's state keeps theta's only (its first nvl x 6 x nip values)
    te = np.zeros(6 * grid.nip * cfg.nvl * cfg.ntra)
    te[:g["trc_edg"].numel()] = st.download("trc_edg")
    g["trc_edg"] = dev(te)
    d2.set_ab(3, 2, 1, 0.0, 0.0, 0.0)  # the post-init slots (Fortran 0,2,1 before the first abstart)
    for its in range(1, 5):
        st.step(its, use_graph=True)
        d2.abstart(its)
        if its > 1:
            # dyn_run opens step its with hybgen and hystat of step its-1
            d2.hybgen(its - 1, None, g["us3d"], g["vs3d"], g["tr3d"], g["sdot"], g["ex3d"], g["dp3d"], g["pr3d"])
            d2.hystat(its - 1, g["ph3d"], g["ex3d"], g["mp3d"], g["dp3d"], g["tr3d"], g["trdp"], g["psrf"],
                      g["ptdcy"])
        d2.edgvar1(its, g["us3d"], g["vs3d"], g["dp3d"], g["pr3d"], g["ex3d"], g["ph3d"], g["mp3d"], g["tr3d"],
                   g["u_edg"], g["v_edg"], g["dp_edg"], g["lp_edg"], g["geop_edg"], g["mont_edg"], g["uvsq_edg"],
                   g["trc_edg"])
        d2.edgvar3(its, g["us3d"], g["vs3d"], g["dp3d"], g["pr3d"], g["ex3d"], g["ph3d"], g["mp3d"], g["tr3d"],
                   g["u_edg"], g["v_edg"], g["dp_edg"], g["lp_edg"], g["geop_edg"], g["mont_edg"], g["uvsq_edg"],
                   g["trc_edg"])
        d2.cnuity(its, g["us3d"], g["vs3d"], g["u_edg"], g["v_edg"], g["dp_edg"], g["lp_edg"], g["dp3d"],
                  g["pr3d"], g["ex3d"], g["dp_tdcy"], g["dpl_tdcy"], g["massfx"], g["ws3d"])
        d2.trcadv(its, g["trc_edg"], g["tr3d"], g["trdp"], g["trc_tdcy"], g["trl_tdcy"], g["massfx"], g["dp3d"])
        d2.momtum(its, g["us3d"], g["vs3d"], g["ex3d"], g["relvor"], g["u_edg"], g["v_edg"], g["trc_edg"],
                  g["geop_edg"], g["mont_edg"], g["uvsq_edg"], g["u_tdcy"], g["v_tdcy"], g["dp3d"])
        for n in PROGNOSTIC + ["ws3d", "relvor", "sdot", "trc_tdcy", "trl_tdcy", "massfx"]:
            assert np.array_equal(st.download(n), host(g[n])), (its, n)


EDG1_NAMES = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "u_edg", "v_edg", "dp_edg",
              "lp_edg", "geop_edg", "mont_edg", "uvsq_edg", "trc_edg"]


@pytest.mark.parametrize("precision,tol", [("f64", TOL64), ("f32", TOL32)])
def test_edgvar2_routine(precision, tol):
    """fim_edgvar2 (hiOrderUVComp) on the oracle's edgvar1 output."""
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1401, noise=1.0, precision=precision)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    o.abstart(1)
    o.edgvar1(*[s[n] for n in EDG1_NAMES])
    rt = torch.float32 if precision == "f32" else torch.float64
    g = {n: dev(s[n], rt) for n in EDG1_NAMES}
    dyc = F.Dycore(grid, cfg)
    dyc.edgvar2(1, *[g[n] for n in EDG1_NAMES])
    ue0 = s["u_edg"].copy()
    o.edgvar2(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["uvsq_edg"])
    assert rel_l2(s["u_edg"], ue0) > 1e-6  # the correction acts on this state
    for n in ("u_edg", "v_edg", "uvsq_edg"):
        assert rel_l2(host(g[n]), s[n]) <= tol, n


def test_fused_step_with_edgvar2_fp64():
    """fim_step with hi_order_uv_comp runs edgvar2 between edgvar1 and
    edgvar3, as dyn_run.F90:353-360 does."""
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1402, noise=1.0, hi_order_uv_comp=1)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc, st = _gpu_state(grid, cfg, fields)
    for its in range(1, 3):
        o.step(s, its)
        st.step(its, use_graph=True)
        errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC + ["ws3d", "relvor"]}
        bad = {k: v for k, v in errs.items() if not v <= TOL64}
        assert not bad, (its, bad)


AB3_FIELDS = ["u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy"]
STEP_OUTPUTS = ["ws3d", "sdot", "relvor"]


def test_ab3_slot_transfer(case4):
    """fim_state_upload_slot / fim_state_download_slot move exactly one AB3
    slot of a tendency field (one block per slot, or one per tracer)."""
    grid, cfg, fields, o, s = case4
    dyc, st = _gpu_state(grid, cfg, fields)
    NL = grid.nip * cfg.nvl
    rng = np.random.default_rng(11)
    for name, nb in (("u_tdcy", 1), ("dpl_tdcy", 1), ("trc_tdcy", cfg.ntra), ("trl_tdcy", cfg.ntra)):
        n = st.field_ptr(name)[1]
        assert n == nb * 3 * NL
        full = rng.standard_normal(n)
        st.upload(name, full)
        blocks = full.reshape(nb, 3, NL)
        for slot in (1, 2, 3):
            got = st.download_slot(name, slot).reshape(nb, 3, NL)
            assert np.array_equal(got[:, slot - 1], blocks[:, slot - 1])
            assert not np.any(got[:, [q for q in range(3) if q != slot - 1]])
        new = full.copy().reshape(nb, 3, NL)
        new[:, 1] += 1.0
        new[:, 0] -= 5.0
        st.upload_slot(name, 2, new.reshape(-1))
        back = st.download(name).reshape(nb, 3, NL)
        assert np.array_equal(back[:, 1], new[:, 1])
        assert np.array_equal(back[:, 0], blocks[:, 0]) and np.array_equal(back[:, 2], blocks[:, 2])
    with pytest.raises(FimError):
        st.upload_slot("us3d", 1, st.download("us3d"))
    with pytest.raises(FimError):
        st.download_slot("u_tdcy", 4)


def test_step_reads_only_uploaded_data(case4):
    """The end-to-end transfer set is complete: a step reads no AB3 slot other
    than the two the host uploads (of, vof of the next step) and none of the
    fields it only writes, so poisoning those with NaN between steps leaves
    every result bit-identical."""
    grid, cfg, fields, o0, s0 = case4
    _, ref = _gpu_state(grid, cfg, fields)
    _, st = _gpu_state(grid, cfg, fields)
    for its in range(1, 6):
        nf, of, vof = st.next_slots()
        assert len({nf, of, vof}) == 3
        for f in STEP_OUTPUTS:
            st.upload(f, np.full(st.field_ptr(f)[1], np.nan))
        for f in AB3_FIELDS:
            h = st.download(f)
            h.reshape(-1, 3, grid.nip * cfg.nvl)[:, nf - 1] = np.nan
            st.upload_slot(f, nf, h)
        ref.step(its, use_graph=True)
        st.step(its, use_graph=True)
        names = PROGNOSTIC + AB3_FIELDS + ["ws3d", "relvor", "psrf"] + (["sdot"] if its > 1 else [])
        for n in names:
            assert np.array_equal(st.download(n), ref.download(n)), (its, n)


def test_mass_adv_fp64():
    """flux_conserv_schm=2 (mass_adv + flux limiter): routine and fused step vs the oracle."""
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=21, noise=1.0, flux_conserv_schm=2)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    s0 = {k: v.copy() for k, v in s.items()}
    dyc = F.Dycore(grid, cfg)
    for its in (1, 2, 3):
        o.abstart(its)
        dyc.set_ab(o.c.nf + 1, o.c.of + 1, o.c.vof + 1, o.c.ab1, o.c.ab2, o.c.ab3)
        o.edgvar1(*[s[n] for n in ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "u_edg",
                                   "v_edg", "dp_edg", "lp_edg", "geop_edg", "mont_edg", "uvsq_edg", "trc_edg"]])
        o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        names = ["us3d", "vs3d", "u_edg", "v_edg", "dp_edg", "lp_edg", "dp3d", "pr3d", "ex3d", "dp_tdcy",
                 "massfx", "ws3d"]
        g = {n: dev(s[n]) for n in names}
        o.mass_adv(*[s[n] for n in names])
        dyc.mass_adv(its, *[g[n] for n in names])
        for n in ["dp_edg", "dp3d", "pr3d", "ex3d", "dp_tdcy", "massfx", "ws3d"]:
            assert rel_l2(host(g[n]), s[n]) <= TOL64, (its, n)
    o2 = oracle_for(grid, cfg)
    s2 = o2.init_state(o2.new_state(fields))
    d2, st = _gpu_state(grid, cfg, fields)
    qo, bo = o2.step(s2, 1)
    st.step(1, use_graph=True)
    for n in PROGNOSTIC:
        assert rel_l2(st.download(n), s2[n]) <= TOL64, n
    qg, bg = st.budget()
    assert abs(bg["qmass"] / bo["qmass"] - 1) < 1e-12
