"""CPU oracle: invariants of the reference algorithm and a regression fixture.

The reference has no golden vectors for this path (parity unpinned); the
oracle is checked against the reference's own in-code invariants: global
mass conservation of the FCT continuity equation, FCT positivity, the hybgen
column-integral checks (hybgen.F90:694,873,1262), and non-negative tracers.
"""
import os

import numpy as np
import pytest

import fimocn_subx_realtime_hera_apr2020_gb300 as F
from helpers import make_case, oracle_for, rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def run3():
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=7, noise=1.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    hist = []
    for its in range(1, 6):
        q, b = o.step(s, its)
        hist.append((q.copy(), b))
    return grid, cfg, o, s, hist


def test_mass_conserved(run3):
    *_, hist = run3
    m = np.array([b["qmass"] for _, b in hist])
    assert np.max(np.abs(m / m[0] - 1)) < 1e-12


def test_tracer_mass_conserved_forward_step():
    """With forward-Euler weights (its=1) FCT transport and the hybgen remap
    conserve tracer mass to round-off.  Later AB2/AB3 steps advance trcdp and
    delp with separate multistep updates before dividing (trcadv3), so the
    reference algorithm itself drifts slightly there."""
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=7, noise=1.0)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    q0, _ = o.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"])
    q1, _ = o.step(s, 1)
    assert np.max(np.abs(q1[1:] / q0[1:] - 1)) < 1e-12


def test_positivity_and_checks(run3):
    grid, cfg, o, s, _ = run3
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    tr = s["tr3d"].reshape(T, N, L)
    assert tr[1:].min() >= 0.0
    assert s["dp3d"].min() > 0.0
    assert o.diag_flags == 0
    for v in s.values():
        assert np.all(np.isfinite(v))


def test_abstart_weights():
    grid, cfg, fields = make_case(glvl=1, nvl=38, ntra=5, dt=100.0)
    o = oracle_for(grid, cfg)
    o.c.nf, o.c.of, o.c.vof = -1, 1, 0
    seen = []
    for its in range(1, 5):
        o.abstart(its)
        seen.append((o.c.nf, o.c.of, o.c.vof, o.c.ab1, o.c.ab2, o.c.ab3))
    assert seen[0] == (0, 2, 1, 100.0, 0.0, 0.0)
    assert seen[1][:3] == (1, 0, 2) and seen[1][3:] == (150.0, -50.0, 0.0)
    assert seen[2][3:] == pytest.approx((100 * 23 / 12, -100 * 16 / 12, 100 * 5 / 12))
    assert seen[3][:3] == (0, 2, 1)


def test_pcwise_constant_field_preserved():
    """A horizontally and vertically uniform tracer stays uniform through a step."""
    grid, cfg, fields = make_case(glvl=2, nvl=38, ntra=5, dt=400.0, seed=3)
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    tr = fields["tr3d"].reshape(T, N, L)
    tr[4] = 3.0e-3
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    o.step(s, 1)
    t4 = s["tr3d"].reshape(T, N, L)[4]
    assert np.max(np.abs(t4 / 3.0e-3 - 1)) < 1e-12


def test_regression_fixture():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import compute
    ref = np.load(os.path.join(HERE, "golden", "oracle_glvl2.npz"))
    now = compute()
    for k in ref.files:
        assert rel_l2(now[k], ref[k]) < 1e-13, k


def test_mass_adv_conserves_mass():
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=9, noise=1.0, flux_conserv_schm=2)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    _, b0 = o.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"])
    for its in range(1, 6):
        _, b = o.step(s, its)
        assert abs(b["qmass"] / b0["qmass"] - 1) < 1e-12
    assert s["dp3d"].min() >= 0.0 and o.diag_flags == 0


# ---- class-B transport (transp3d.F90, fct3d.F90) ---------------------------

def _classb_case(ntrb=2, dtratio=2, seed=5):
    grid = F.Grid.cached(3)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=F.default_dt(3), ntrb=ntrb, dtratio=dtratio)
    fields = F.synthetic_state(grid, cfg, seed=seed, sigma_ps=200.0, noise=1.0)
    return grid, cfg, fields


def test_classb_uniform_and_bounds():
    """A uniform class-B tracer stays uniform; FCT keeps the others within
    their initial range (fct3d's local bounds)."""
    grid, cfg, fields = _classb_case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    tr = fields["tr3d"].reshape(T + 2, N, L)
    tr[T] = 3.0e-3
    lo, hi = tr[T + 1].min(), tr[T + 1].max()
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    for its in range(1, 7):
        o.step(s, its)
        b = s["tr3d"].reshape(T + 2, N, L)
        assert np.abs(b[T] / 3.0e-3 - 1).max() < 1e-13, its
        assert b[T + 1].min() >= lo * (1 - 1e-12) and b[T + 1].max() <= hi * (1 + 1e-12), its
    assert not np.array_equal(s["tr3d"].reshape(T + 2, N, L)[T + 1], tr[T + 1])


def test_classb_conservation_of_fluxes():
    """transp2 with antisymmetric horizontal fluxes and a consistent final
    thickness conserves tracer mass to rounding; so does a vertical exchange
    of a tracer that is uniform in each column (no bound is active)."""
    grid, cfg, fields = _classb_case(ntrb=1)
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    nprox, prox, _ = grid.zero_based()
    rng = np.random.Generator(np.random.PCG64(9))
    dp = s["dp3d"].reshape(N, L)
    phi = rng.standard_normal((N, L)) * 1e9
    cum = np.zeros((N, 6, L))
    for i in range(N):
        for e in range(nprox[i]):
            cum[i, e] = phi[i] - phi[prox[i * 6 + e]]
    div = np.stack([cum[i, :nprox[i]].sum(0) for i in range(N)]) / grid.area[:, None]
    mass = lambda tr, d: (grid.area[:, None] * d * tr.reshape(T + 1, N, L)[T]).sum()  # noqa: E731
    tr = s["tr3d"].copy()
    dpf = dp - div
    assert dpf.min() > 0
    m0 = mass(tr, dp)
    o.transp2(tr, cum.reshape(-1), dp.reshape(-1).copy(), dpf.reshape(-1))
    assert abs(mass(tr, dpf) / m0 - 1) < 1e-13
    tr = s["tr3d"].copy()
    col = tr.reshape(T + 1, N, L)
    col[T] = rng.random(N)[:, None] * 1e-2
    dpv = dp.copy()
    d = 0.3 * np.minimum(dpv[:, 5], dpv[:, 6])
    dpv[:, 5] -= d
    dpv[:, 6] += d
    m0 = mass(tr, dp)
    o.transp2(tr, np.zeros(6 * N * L), dp.reshape(-1).copy(), dpv.reshape(-1))
    assert abs(mass(tr, dpv) / m0 - 1) < 1e-13
