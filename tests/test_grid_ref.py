"""Integer grid tables against a restatement of the reference's grid generator.

oracle/grid_ref.py restates the reference's point numbering (icos.F90 with
bisect_triangle.F90) and its pattern-based neighbour lists (GridGen.F90,
getlvl.F90:145-157, dyn_init.F90:545-549).  The product's builder
(csrc/fim_grid.cpp) finds neighbours by walking the triangulation instead;
nprox, prox and proxs must nevertheless equal the reference's entry for
entry, slot order included, since every edge sum of the dycore runs in slot
order.
"""
import math

import numpy as np
import pytest

import fimocn_subx_realtime_hera_apr2020_gb300 as F
import grid_ref


def _xyz(lat, lon):
    return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)


@pytest.mark.parametrize("glvl", [1, 2, 3])
def test_restated_tables_are_the_grid(glvl):
    """The restatement itself: every listed neighbour is one of the nearest
    points, listed counter-clockwise seen from outside, and edges pair up."""
    lat, lon = grid_ref.icos_points(glvl)
    d2r = grid_ref._PI32 / 180.0  # the generator's own degree factor
    x = _xyz(lat * d2r, lon * d2r)
    nprox, prox, proxs = grid_ref.neighbour_tables(glvl)
    nip = 10 * 4 ** glvl + 2
    assert len(lat) == nip and (nprox == 5).sum() == 12
    for i in range(nip):
        n = nprox[i]
        d = np.linalg.norm(x - x[i], axis=1)
        assert set((np.argsort(d)[1:1 + n] + 1).tolist()) == set(prox[i, :n].tolist()), i
        for e in range(n):
            a, b, c = x[i], x[prox[i, e] - 1], x[prox[i, (e + 1) % n] - 1]
            assert np.dot(a, np.cross(b - a, c - a)) > 0
            assert prox[prox[i, e] - 1, proxs[i, e] - 1] == i + 1


@pytest.mark.parametrize("glvl", [1, 2, 3, 4, 5, 6])
def test_builder_tables_bit_exact(glvl):
    nprox, prox, proxs = grid_ref.neighbour_tables(glvl)
    g = F.Grid.cached(glvl)
    assert np.array_equal(g.nprox, nprox)
    assert np.array_equal(g.prox.reshape(-1, 6), prox)
    assert np.array_equal(g.proxs.reshape(-1, 6), proxs)


@pytest.mark.parametrize("glvl", [2, 4])
def test_builder_points_follow_reference_numbering(glvl, monkeypatch):
    """Cell i of the builder is point i of the reference generator.  The
    generator converts degrees with 4*atan(1.0) in single precision
    (middle.F90, rotate.F90), which moves its points by up to ~1e-6 of the
    radius; with that factor in double precision the points agree to
    round-off."""
    g = F.Grid.cached(glvl)
    xo = _xyz(g.lat, g.lon)
    lat, lon = grid_ref.icos_points(glvl)
    d2r = grid_ref._PI32 / 180.0
    assert np.abs(_xyz(lat * d2r, lon * d2r) - xo).max() < 2e-6
    monkeypatch.setattr(grid_ref, "_PI32", math.pi)
    lat, lon = grid_ref.icos_points(glvl)
    assert np.abs(_xyz(np.radians(lat), np.radians(lon)) - xo).max() < 1e-14
