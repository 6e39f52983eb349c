"""The tracer kernels on breadth-first patches (a grid numbered otherwise).

A grid in the reference's IJ numbering gets patches of 8 x 8 cells of a
rhombus; any other numbering gets patches grown breadth-first.  Every value
of the step is formed per cell in slot order, so renumbering the cells
renumbers the results and changes nothing else: the step on a grid whose
cells are renumbered by a seeded permutation must return the renumbered
results of the step on the original grid bit for bit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from helpers import PROGNOSTIC, make_case  # noqa: E402

pytestmark = pytest.mark.gpu

# values per cell of each table of the grid descriptor
PER_CELL = dict(nprox=1, prox=6, proxs=6, lat=1, lon=1, area=1, cs=24, sn=24, sidevec_c=12, sidevec_e=12,
                sideln=6, rprox_ln=6, corner_xy=12, hfcoef=36)


def renumbered(glvl, seed):
    """A fresh grid whose cell j is cell inv[j] of the original numbering."""
    g = F.Grid(glvl)
    n = g.nip
    perm = np.random.default_rng(seed).permutation(n)  # new number of old cell i
    inv = np.argsort(perm)
    for name, k in PER_CELL.items():
        a = getattr(g, name)
        a[:] = a.reshape(n, k)[inv].reshape(-1)
    g.prox[:] = perm[g.prox - 1] + 1
    return g, inv


def cells_first(a, n):
    """(cells, values per cell) view of a level-fastest field."""
    return a.reshape(n, -1)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_renumbered_grid_gives_renumbered_results(precision):
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=2024, noise=1.0, precision=precision)
    n = grid.nip
    gp, inv = renumbered(3, seed=7)
    pf = {}
    for name, a in fields.items():
        if name == "tr3d":
            T = a.size // (n * cfg.nvl)
            pf[name] = a.reshape(T, n, cfg.nvl)[:, inv].reshape(-1).copy()
        else:
            pf[name] = cells_first(a, n)[inv].reshape(-1).copy()
    d0 = F.Dycore(grid, cfg)
    s0 = d0.state()
    s0.load(fields)
    s0.init()
    d1 = F.Dycore(gp, cfg)
    s1 = d1.state()
    s1.load(pf)
    s1.init()
    for its in (1, 2, 3):
        s0.step(its)
        s1.step(its)
    for name in PROGNOSTIC + ["ws3d", "relvor", "sdot"]:
        a0, a1 = s0.download(name), s1.download(name)
        if name in ("tr3d", "trdp"):
            T = a0.size // (n * cfg.nvl)
            want = a0.reshape(T, n, cfg.nvl)[:, inv]
            got = a1.reshape(T, n, cfg.nvl)
        else:
            want = cells_first(a0, n)[inv]
            got = cells_first(a1, n)
        assert np.array_equal(got, want), name
    assert s0.check()[0] == 0 and s1.check()[0] == 0


def test_coarse_grid_small_patches():
    """glvl 2 (162 cells): patches of 4 x 4 cells whose frames exceed three
    rows a thread, so the tracer kernels stage through their general loop;
    three FP64 steps against the oracle."""
    from helpers import oracle_for, rel_l2
    grid, cfg, fields = make_case(glvl=2, nvl=38, ntra=5, dt=1200.0, seed=202, noise=1.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    d = F.Dycore(grid, cfg)
    st = d.state()
    st.load(fields)
    st.init()
    for its in (1, 2, 3):
        o.step(s, its)
        st.step(its)
        errs = {n: rel_l2(st.download(n), s[n]) for n in PROGNOSTIC}
        bad = {k: v for k, v in errs.items() if not v <= 1e-12}
        assert not bad, (its, bad)
    assert st.check()[0] == 0


@pytest.mark.parametrize("precision,shapes", [
    ("f32", [(4, 4), (4, 2), (2, 4), (2, 2), (1, 4), (1, 2)]),
    ("f64", [(2, 4), (2, 2), (1, 4), (1, 2)]),
])
def test_every_tracer_shape_same_results(precision, shapes, monkeypatch):
    """Every shape the tracer kernels' autotuner can pick (levels a thread x
    threads a cell, so the level tile and the block) forms each cell-level's
    values in the same order: three steps agree bit for bit."""
    grid, cfg, fields = make_case(glvl=3, nvl=64, ntra=5, dt=400.0, seed=64, noise=1.0, precision=precision)
    results = []
    for vk, gc in shapes:
        monkeypatch.setenv("FIM_TRC_VK", str(vk))
        monkeypatch.setenv("FIM_TRC_GC", str(gc))
        d = F.Dycore(grid, cfg)
        st = d.state()
        st.load(fields)
        st.init()
        for its in (1, 2, 3):
            st.step(its)
        assert d.tracer_shape()[0] == vk, (vk, gc)
        results.append({n: st.download(n) for n in PROGNOSTIC})
        assert st.check()[0] == 0
    for (vk, gc), r in zip(shapes[1:], results[1:]):
        for n in PROGNOSTIC:
            assert np.array_equal(r[n], results[0][n]), (vk, gc, n)
