"""Class-B tracer transport (transp0/1/2 + fct3d) on the GPU against the CPU
oracle: each routine fed the oracle's inputs, and the fused step with class-B
tracers transported every dtratio steps.

FP64: relative L2 <= 1e-12 per field; FP32-mixed: <= 1e-5 after one step.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from helpers import PROGNOSTIC, oracle_for, rel_l2  # noqa: E402

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)


def host(t):
    torch.cuda.synchronize()
    return t.double().cpu().numpy()


def _case(precision="f64", ntrb=2, dtratio=2, seed=41):
    grid = F.Grid.cached(3)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=F.default_dt(3), precision=precision, ntrb=ntrb, dtratio=dtratio)
    fields = F.synthetic_state(grid, cfg, seed=seed, sigma_ps=200.0, noise=1.0)
    return grid, cfg, fields


def test_transp_routines_fp64():
    grid, cfg, fields = _case()
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    for its in (1, 2):
        o.step(s, its)  # a state with live mass fluxes and a thickness history
    dyc = F.Dycore(grid, cfg)
    o.abstart(3)
    dyc.set_ab(o.c.nf + 1, o.c.of + 1, o.c.vof + 1, o.c.ab1, o.c.ab2, o.c.ab3)
    cum = dev(s["cumufx"])
    o.transp1(s["cumufx"], s["massfx"])
    dyc.transp1(3, cum, dev(s["massfx"]))
    assert rel_l2(host(cum), s["cumufx"]) <= TOL64
    tr = dev(s["tr3d"])
    dpf = s["dp3d"] * (1 + 1e-3 * np.sin(np.arange(s["dp3d"].size)))  # a thickness change to close
    o.transp2(s["tr3d"], s["cumufx"], s["dpinit"], dpf)
    dyc.transp2(3, tr, dev(s["cumufx"]), dev(s["dpinit"]), dev(dpf))
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    got, ref = host(tr).reshape(T + 2, N, L), s["tr3d"].reshape(T + 2, N, L)
    assert np.array_equal(got[:T], ref[:T])  # class-A tracers untouched
    for t in (T, T + 1):
        assert rel_l2(got[t], ref[t]) <= TOL64, t
    cum, dpi = dev(s["cumufx"]), dev(np.zeros_like(s["dpinit"]))
    o.transp0(s["cumufx"], s["dp3d"], s["dpinit"])
    dyc.transp0(3, cum, dev(s["dp3d"]), dpi)
    assert not host(cum).any() and np.array_equal(host(dpi), s["dpinit"])


@pytest.mark.parametrize("use_graph", [False, True])
def test_fused_step_classb_fp64(use_graph):
    grid, cfg, fields = _case()
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc = F.Dycore(grid, cfg)
    st = dyc.state()
    st.load(fields)
    st.init()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    for its in range(1, 5):
        qo, _ = o.step(s, its)
        st.step(its, use_graph=use_graph)
        for n in PROGNOSTIC + ["cumufx", "dpinit"]:
            assert rel_l2(st.download(n), s[n]) <= TOL64, (its, n)
        got = st.download("tr3d").reshape(T + 2, N, L)
        for t in (T, T + 1):
            assert rel_l2(got[t], s["tr3d"].reshape(T + 2, N, L)[t]) <= TOL64, (its, t)
        qg, _ = st.budget()
        assert qg.size == T + 2 and rel_l2(qg, qo) <= TOL64, its


def test_fused_step_classb_fp32():
    grid, cfg, fields = _case(precision="f32", dtratio=1)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    dyc = F.Dycore(grid, cfg)
    st = dyc.state()
    st.load({k: v.astype(np.float32) for k, v in fields.items()})
    st.init()
    o.step(s, 1)
    st.step(1, use_graph=True)
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    got = st.download("tr3d").reshape(T + 2, N, L)
    for t in (T, T + 1):
        assert rel_l2(got[t], s["tr3d"].reshape(T + 2, N, L)[t]) <= TOL32, t
