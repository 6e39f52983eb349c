"""Cell patches of the fused tracer kernels, built and checked on the host.

fim_grid_patches builds the patch tables exactly as fim_ctx_create does and
checks that every cell lies in one patch and that every frame neighbour and
every edge's other side resolve to the grid's prox/proxs.  No GPU is used.
"""
import ctypes

import numpy as np
import pytest

import fimocn_subx_realtime_hera_apr2020_gb300 as F
import fimocn_subx_realtime_hera_apr2020_gb300._lib as L


def patches(grid, side=8):
    lib = L.load()
    out = [ctypes.c_int(0) for _ in range(4)]
    d = grid.desc()
    rc = lib.fim_grid_patches(ctypes.byref(d), side, *[ctypes.byref(o) for o in out])
    return rc, [o.value for o in out]


@pytest.mark.parametrize("glvl", [1, 2, 3, 4, 5, 6])
def test_rhombus_patches(glvl):
    g = F.Grid.cached(glvl)
    rc, (n, cells, frame, ring_edges) = patches(g)
    assert rc == L.FIM_OK
    sl = 2 ** glvl
    side = min(8, sl)
    # 10 rhombi of (sl / side)^2 patches, and the two poles
    assert n == 10 * (sl // side) ** 2 + 2
    assert cells == side * side
    # a patch and its two neighbour rings: (side + 4)^2 less the two corners
    # the hexagonal rings skip (the frame indices fit a byte)
    assert frame <= (side + 4) ** 2 and frame <= 255
    assert ring_edges <= 8 * side


def test_smaller_sides():
    g = F.Grid.cached(4)
    for side in (1, 3, 4, 7):
        rc, (n, cells, frame, _) = patches(g, side)
        assert rc == L.FIM_OK, side
        assert cells <= side * side
        assert n >= g.nip // (side * side)


def test_other_numbering_grows_patches():
    """A grid numbered otherwise (here: cells renumbered by a seeded
    permutation) gets breadth-first patches that still pass every check."""
    g = F.Grid(3)
    n = g.nip
    rng = np.random.default_rng(7)
    perm = rng.permutation(n)          # new index of old cell i
    inv = np.argsort(perm)             # old index of new cell j
    prox = g.prox.reshape(n, 6)
    proxs = g.proxs.reshape(n, 6)
    nprox = g.nprox.copy()
    g.nprox[:] = nprox[inv]
    g.prox[:] = (perm[prox[inv] - 1] + 1).reshape(-1)
    g.proxs[:] = proxs[inv].reshape(-1)
    rc, (npatch, cells, frame, _) = patches(g)
    assert rc == L.FIM_OK
    assert cells <= 64 and frame <= 255
    assert npatch * 64 >= n


def test_rejects_bad_input():
    g = F.Grid(3)
    assert patches(g, 0)[0] == L.FIM_EINVAL
    assert patches(g, 9)[0] == L.FIM_EINVAL
    g.prox[5] = g.nip + 1  # a neighbour out of range
    assert patches(g)[0] == L.FIM_EINVAL
