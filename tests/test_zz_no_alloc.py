"""fim_cnuity_noalloc (scratch in the library's static array) against
fim_cnuity_r8/_r4 on the same inputs, two calls in a row, through the C-ABI.

Collected last so it runs after the other GPU tests have used the library in
the same process; it also passes alone in a fresh process.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32": 1e-5}
NAMES = ["us3d", "vs3d", "u_edg", "v_edg", "dp_edg", "lp_edg", "dp3d", "pr3d", "ex3d", "dp_tdcy", "dpl_tdcy",
         "massfx", "ws3d"]
OUTS = ["dp3d", "pr3d", "ex3d", "dp_tdcy", "dpl_tdcy", "massfx", "ws3d"]


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / n if n > 0 else np.linalg.norm(a - b)


def _inputs(grid, cfg):
    """A stepped device state, so the edge fields and mass fluxes are live."""
    dyc = F.Dycore(grid, cfg)
    st = dyc.state()
    st.load(F.synthetic_state(grid, cfg, seed=77, sigma_ps=200.0, noise=1.0, dtype=cfg.dtype))
    st.init()
    st.step(1, use_graph=False)
    out = {n: st.download(n).copy() for n in NAMES}
    st.free()
    dyc.close()
    return out


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_noalloc_matches_cnuity(precision):
    grid = F.Grid.cached(4)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0, precision=precision)
    tdt = torch.float64 if precision == "f64" else torch.float32
    h = _inputs(grid, cfg)
    ref = F.Dycore(grid, cfg)
    new = F.Dycore(grid, cfg)
    a = {n: torch.from_numpy(h[n]).to("cuda", tdt) for n in NAMES}
    b = {n: torch.from_numpy(h[n]).to("cuda", tdt) for n in NAMES}
    for its in (1, 2):
        ref.abstart(its)
        new.abstart(its)
        ref.cnuity(its, *[a[n] for n in NAMES])
        new.cnuity_noalloc(its, *[b[n] for n in NAMES])
        for n in OUTS:
            x = b[n].double().cpu().numpy()
            y = a[n].double().cpu().numpy()
            assert np.all(np.isfinite(x)), (its, n)
            assert rel_l2(x, y) <= TOL[precision], (its, n, rel_l2(x, y))
    ref.close()
    new.close()


def test_noalloc_rejects_large_grid():
    # glvl 6 / nvl 64 needs 110 MiB of scratch even in FP32; the size check
    # comes before any pointer is looked at, so no field buffers are needed
    grid = F.Grid.cached(6)
    cfg = F.FimConfig(nvl=64, ntra=5, dt=180.0, precision="f32")
    dyc = F.Dycore(grid, cfg)
    rc = dyc.lib.fim_cnuity_noalloc(dyc.ctx, 1, *([None] * 13))
    assert rc == _lib.FIM_EINVAL
    assert b"static array holds" in dyc.lib.fim_ctx_last_error(dyc.ctx)
    dyc.close()
