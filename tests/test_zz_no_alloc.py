"""fim_cnuity_noalloc against fim_cnuity_r8/_r4, through the C-ABI.

fim_cnuity_noalloc serves callers that may not allocate device memory once
their run has started: a host model whose device memory its own pool carves
up at start-up, a memory-capped process, or a time loop that cannot take
cudaMalloc's device-wide synchronisation.  It takes its FCT scratch from a
static array in the library instead of the context's lazily allocated
buffers.  Both entry points launch the same kernels on the same inputs, so
their results must be identical bit for bit, on two calls in a row.

The allocation-free call runs first, on a fresh context: the context's own
scratch must stay unallocated and the device's free memory must not change
across the calls.  Collected last so it runs after the other GPU tests have
used the library in the same process; it also passes alone in a fresh
process.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300 import _lib  # noqa: E402

pytestmark = pytest.mark.gpu

NAMES = ["us3d", "vs3d", "u_edg", "v_edg", "dp_edg", "lp_edg", "dp3d", "pr3d", "ex3d", "dp_tdcy", "dpl_tdcy",
         "massfx", "ws3d"]
OUTS = ["dp3d", "pr3d", "ex3d", "dp_tdcy", "dpl_tdcy", "massfx", "ws3d"]
STATIC_BYTES = 64 << 20


def _scratch_bytes(nip, nvl, esz):
    """Bytes of the 11 FCT scratch values per cell-level, six fields rounded
    to 256 bytes each (the entry point's own layout)."""
    r = lambda b: (b + 255) // 256 * 256  # noqa: E731
    cells = nip * nvl
    return r(cells * 6 * esz) + 5 * r(cells * esz)


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


def _run(dyc, h, tdt, noalloc):
    """Two calls in a row; outputs after each, and the free device memory
    before the first call and after each call."""
    a = {n: torch.from_numpy(h[n]).to("cuda", tdt) for n in NAMES}
    torch.cuda.synchronize()
    free = [torch.cuda.mem_get_info()[0]]
    outs = []
    for its in (1, 2):
        dyc.abstart(its)
        (dyc.cnuity_noalloc if noalloc else dyc.cnuity)(its, *[a[n] for n in NAMES])
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        outs.append({n: a[n].cpu().numpy().copy() for n in OUTS})
    return outs, free


@pytest.mark.parametrize("precision,glvl,nvl", [("f64", 4, 38), ("f32", 4, 38), ("f64", 5, 64)])
def test_noalloc_matches_cnuity(precision, glvl, nvl):
    grid = F.Grid.cached(glvl)
    cfg = F.FimConfig(nvl=nvl, ntra=5, dt=F.default_dt(glvl), precision=precision)
    esz = 8 if precision == "f64" else 4
    assert _scratch_bytes(grid.nip, nvl, esz) <= STATIC_BYTES
    tdt = torch.float64 if precision == "f64" else torch.float32
    h = _inputs(grid, cfg)
    new = F.Dycore(grid, cfg)
    own = new.device_bytes()
    got, free = _run(new, h, tdt, noalloc=True)
    assert new.device_bytes() == own, "the context allocated scratch"
    assert free[1] == free[0] and free[2] == free[0], free
    ref = F.Dycore(grid, cfg)
    want, _ = _run(ref, h, tdt, noalloc=False)
    assert ref.device_bytes() > own  # fim_cnuity allocates its scratch on its first call
    for its in (0, 1):
        for n in OUTS:
            assert np.all(np.isfinite(got[its][n])), (its, n)
            assert np.array_equal(got[its][n], want[its][n]), (its + 1, n)
    ref.close()
    new.close()


def test_noalloc_size_limit():
    """At glvl 5 in FP64, nvl 74 is the deepest column whose scratch fits the
    array and nvl 75 the first that does not.  The size check comes before
    any pointer is looked at, so null field pointers tell the two apart: the
    fitting size fails on the pointers, the other on the size."""
    grid = F.Grid.cached(5)
    assert _scratch_bytes(grid.nip, 74, 8) <= STATIC_BYTES < _scratch_bytes(grid.nip, 75, 8)
    for nvl, msg in ((74, b"null field pointer"), (75, b"static array holds")):
        cfg = F.FimConfig(nvl=nvl, ntra=5, dt=F.default_dt(5), precision="f64",
                          thetac=np.linspace(300.0, 600.0, nvl), dpsig=np.full(nvl, 5.0))
        dyc = F.Dycore(grid, cfg)
        rc = dyc.lib.fim_cnuity_noalloc(dyc.ctx, 1, *([None] * 13))
        assert rc == _lib.FIM_EINVAL
        assert msg in dyc.lib.fim_ctx_last_error(dyc.ctx), (nvl, dyc.lib.fim_ctx_last_error(dyc.ctx))
        dyc.close()


def test_noalloc_rejects_large_grid():
    # glvl 6 / nvl 64 needs 110 MiB of scratch even in FP32
    grid = F.Grid.cached(6)
    cfg = F.FimConfig(nvl=64, ntra=5, dt=180.0, precision="f32")
    dyc = F.Dycore(grid, cfg)
    rc = dyc.lib.fim_cnuity_noalloc(dyc.ctx, 1, *([None] * 13))
    assert rc == _lib.FIM_EINVAL
    assert b"static array holds" in dyc.lib.fim_ctx_last_error(dyc.ctx)
    dyc.close()
