"""Second restatements, in vectorised NumPy, of two oracle routines whose
arithmetic is short (hystat.F90:53-109, globsum.F90:58-108): they check the C
code against an independent transcription of the reference loops.  This is a
check of the oracle's own code, not a pin to the reference."""
import numpy as np

from helpers import make_case, oracle_for

GRVITY, RD, CP, QVMIN, QWMIN = 9.80665, 287.0586, 1004.6855, 1.e-10, 1.e-10


def _case():
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, seed=1500)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    return grid, cfg, o, s


def test_hystat_matches_numpy():
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    rng = np.random.default_rng(1501)
    s["tr3d"][N * L:3 * N * L] = rng.uniform(-1e-9, 1e-3, 2 * N * L)  # some below the floors
    s["psrf"][:] = rng.uniform(9e4, 1e5, N)
    ph0 = s["ph3d"].reshape(N, L + 1)[:, 0].copy()
    ex = s["ex3d"].reshape(N, L + 1)
    dp = s["dp3d"].reshape(N, L)
    tr = s["tr3d"].reshape(T, N, L).copy()
    work = s["psrf"].copy()
    # reference loops, vectorised over cells
    ps = dp[:, L - 1].copy()
    for k in range(L - 2, -1, -1):
        ps = ps + dp[:, k]
    th = tr[0]
    mp = np.zeros((N, L))
    ph = np.zeros((N, L + 1))
    ph[:, 0] = ph0
    mp[:, 0] = ex[:, 0] * th[:, 0] + ph[:, 0]
    ph[:, 1] = mp[:, 0] - th[:, 0] * ex[:, 1]
    for k in range(1, L):
        mp[:, k] = mp[:, k - 1] + ex[:, k] * (th[:, k] - th[:, k - 1])
        ph[:, k + 1] = mp[:, k] - th[:, k] * ex[:, k + 1]
    tr[1] = np.maximum(QVMIN, tr[1])
    tr[2] = np.maximum(QWMIN, tr[2])
    trdp = tr * dp[None]
    its = 3
    o.hystat(its, s["ph3d"], s["ex3d"], s["mp3d"], s["dp3d"], s["tr3d"], s["trdp"], s["psrf"], s["ptdcy"])
    assert np.array_equal(s["psrf"], ps)
    assert np.array_equal(s["ptdcy"].reshape(2, N)[its % 2], ps - work)
    assert np.array_equal(s["mp3d"].reshape(N, L), mp)
    assert np.array_equal(s["ph3d"].reshape(N, L + 1), ph)
    assert np.array_equal(s["tr3d"].reshape(T, N, L), tr)
    assert np.array_equal(s["trdp"][:T * N * L].reshape(T, N, L), trdp)


def test_globsum_matches_numpy():
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    rng = np.random.default_rng(1502)
    rn, rc, qf = rng.uniform(0, 5, N), rng.uniform(0, 2, N), rng.normal(0, 1e-4, N)
    qtrcr, b = o.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"], rn, rc, qf)
    a = np.asarray(grid.area)
    dp = s["dp3d"].reshape(N, L)
    tr = s["tr3d"].reshape(T, N, L)
    ad = a[:, None] * dp
    ref_q = [(ad * tr[t]).sum() for t in range(T)]
    np.testing.assert_allclose(qtrcr, ref_q, rtol=1e-13)
    np.testing.assert_allclose(b["qmass"], ad.sum() / GRVITY, rtol=1e-13)
    np.testing.assert_allclose(b["qmsqv"], (ad * tr[1]).sum() / GRVITY, rtol=1e-13)
    np.testing.assert_allclose(b["qmsqw"], (ad * tr[2]).sum() / GRVITY, rtol=1e-13)
    np.testing.assert_allclose(b["qmso3"], (ad * tr[3]).sum() / GRVITY, rtol=1e-13)
    np.testing.assert_allclose(b["qmstr"], (a * rn).sum(), rtol=1e-13)
    np.testing.assert_allclose(b["qmstrc"], (a * rc).sum(), rtol=1e-13)
    np.testing.assert_allclose(b["qmstrn"], (a * (rn - rc)).sum(), rtol=1e-13)
    pr0 = s["pr3d"].reshape(N, L + 1)[:, 0]
    ex0 = s["ex3d"].reshape(N, L + 1)[:, 0]
    den = pr0 / ((RD / CP) * ex0 * tr[0][:, 0])
    np.testing.assert_allclose(b["qmste"], (a * den * qf * cfg.dt / (1.25 * 2.5e6)).sum(), rtol=1e-12)


def test_edgvar3_matches_numpy():
    """edgvar3.F90:64-133: edgvalEval's least-squares edge values of dp and
    tracers 2..ntra, then the two-sided average stored in both slots."""
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    proxs = np.asarray(grid.proxs).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    hf = np.asarray(grid.hfcoef).reshape(N, 6, 6)
    rng = np.random.default_rng(1503)
    s["tr3d"][N * L:] += rng.uniform(0, 1e-3, (T - 1) * N * L)

    def own(f):  # f (N, L) -> own-side edge values (N, 6, L)
        out = np.zeros((N, 6, L))
        for i in range(N):
            n = npx[i]
            d = f[prox[i, :n]] - f[i][None]
            for e in range(n):
                acc = f[i].copy()
                for j in range(n):
                    acc = acc + d[j] * hf[i, e, j]
                out[i, e] = acc
        return out

    def average(x):
        y = x.copy()
        for i in range(N):
            for e in range(npx[i]):
                nb, os_ = prox[i, e], proxs[i, e]
                if i < nb:
                    w = 0.5 * (x[i, e] + x[nb, os_])
                    y[i, e] = w
                    y[nb, os_] = w
        return y

    dp_ref = average(own(s["dp3d"].reshape(N, L)))
    tr = s["tr3d"].reshape(T, N, L)
    tr_ref = [average(own(tr[t])) for t in range(1, T)]
    o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
    assert np.array_equal(s["dp_edg"].reshape(N, 6, L), dp_ref)
    te = s["trc_edg"].reshape(T, N, 6, L)
    for t in range(1, T):
        assert np.array_equal(te[t], tr_ref[t - 1]), t
