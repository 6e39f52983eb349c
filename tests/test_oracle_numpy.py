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


def test_cnuity_matches_numpy():
    """cnuity_compute.F90 cnuity1..5: donor-cell and high-order mass fluxes,
    Zalesak limiter over the 1-ring, AB3 thickness update, top-down pressure,
    Exner function and omega."""
    grid, cfg, o, s = _case()
    N, L = grid.nip, cfg.nvl
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    proxs = np.asarray(grid.proxs).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    sve = np.asarray(grid.sidevec_e).reshape(N, 6, 2)
    svc = np.asarray(grid.sidevec_c).reshape(N, 6, 2)
    area = np.asarray(grid.area)
    rarea = 1.0 / area
    for its in (1, 2, 3):  # Euler, AB2, AB3 weights
        o.abstart(its)
        o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"],
                  s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"],
                  s["trc_edg"])
        o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        nf, of, vof = o.c.nf, o.c.of, o.c.vof
        ab1, ab2, ab3, dt = o.c.ab1, o.c.ab2, o.c.ab3, o.c.dt
        ue, ve = s["u_edg"].reshape(N, 6, L), s["v_edg"].reshape(N, 6, L)
        dpe, lpe = s["dp_edg"].reshape(N, 6, L), s["lp_edg"].reshape(N, 6, L)
        delp = s["dp3d"].reshape(N, L).copy()
        pres = s["pr3d"].reshape(N, L + 1).copy()
        dpt = s["dp_tdcy"].reshape(3, N, L).copy()
        dplt = s["dpl_tdcy"].reshape(3, N, L).copy()
        u, v = s["us3d"].reshape(N, L), s["vs3d"].reshape(N, L)
        live = np.arange(6)[None, :] < npx[:, None]
        vn = sve[:, :, 1:2] * ue - sve[:, :, 0:1] * ve
        psl = np.where(live, proxs, 0)            # a pentagon's slot 5 has no mirror: masked below
        vx = vn[prox, psl]                        # the neighbour's normal velocity on the shared edge
        mass = 0.5 * ((vn + np.abs(vn)) * delp[:, None, :] - (vx + np.abs(vx)) * delp[prox])
        mass = np.where(live[:, :, None], mass, 0.0)
        anti = np.where(live[:, :, None], vn * dpe - mass, 0.0)
        acc = np.zeros((N, L))
        for e in range(6):
            acc = acc + mass[:, e]
        dplt[nf] = -acc * rarea[:, None]
        dlo = delp + ab1 * dplt[nf] + ab2 * dplt[of] + ab3 * dplt[vof]
        pp, pm = np.zeros((N, L)), np.zeros((N, L))
        for e in range(6):
            a = anti[:, e]
            pp = np.where(live[:, e:e + 1] & (a <= 0), pp - a, pp)
            pm = np.where(live[:, e:e + 1] & (a > 0), pm + a, pm)
        dmx, dmn = np.maximum(dlo, delp), np.minimum(dlo, delp)
        for e in range(6):
            dmx, dmn = np.maximum(dmx, dlo[prox[:, e]]), np.minimum(dmn, dlo[prox[:, e]])
        for e in range(6):
            dmx, dmn = np.maximum(dmx, delp[prox[:, e]]), np.minimum(dmn, delp[prox[:, e]])
        dmx, dmn = np.maximum(0.0, dmx), np.maximum(0.0, dmn)
        qp = (dmx - dlo - (ab2 * np.minimum(0.0, dpt[of]) + ab3 * np.maximum(0.0, dpt[vof]))) / ab1 * area[:, None]
        qm = (dlo - dmn + (ab2 * np.maximum(0.0, dpt[of]) + ab3 * np.minimum(0.0, dpt[vof]))) / ab1 * area[:, None]
        rp = np.maximum(0.0, np.minimum(1.0, qp / np.maximum(pp, 1e-11)))
        rm = np.maximum(0.0, np.minimum(1.0, qm / np.maximum(pm, 1e-11)))
        clip = np.where(anti >= 0, np.minimum(rm[:, None, :], rp[prox]), np.minimum(rp[:, None, :], rm[prox]))
        anti = anti * clip
        mass = mass + anti
        at = np.zeros((N, L))
        for e in range(6):
            at = at + np.where(live[:, e:e + 1], anti[:, e], 0.0)
        dpt[nf] = dplt[nf] + (-at * rarea[:, None])
        delp = delp + ab1 * dpt[nf] + ab2 * dpt[of] + ab3 * dpt[vof]
        omega = np.zeros((N, L))
        col = np.zeros(N)
        for k in range(L - 1, -1, -1):
            pres[:, k] = pres[:, k + 1] + delp[:, k]
            lyr = (ab1 * dpt[nf][:, k] + ab2 * dpt[of][:, k] + ab3 * dpt[vof][:, k]) / dt
            om = col + 0.5 * lyr
            col = col + lyr
            dx, dy = np.zeros(N), np.zeros(N)
            for e in range(6):
                dx = np.where(live[:, e], dx + lpe[:, e, k] * svc[:, e, 1], dx)
                dy = np.where(live[:, e], dy - lpe[:, e, k] * svc[:, e, 0], dy)
            omega[:, k] = om + (u[:, k] * dx + v[:, k] * dy) * rarea
        exner = CP * (pres / 100000.0) ** (RD / CP)
        o.cnuity(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["dp3d"], s["pr3d"],
                 s["ex3d"], s["dp_tdcy"], s["dpl_tdcy"], s["massfx"], s["ws3d"])
        mf = s["massfx"].reshape(3, N, 6, L)[nf]
        np.testing.assert_allclose(mf[live], mass[live], rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(s["dp3d"].reshape(N, L), delp, rtol=1e-13)
        np.testing.assert_allclose(s["dp_tdcy"].reshape(3, N, L)[nf], dpt[nf], rtol=1e-11, atol=1e-11)
        np.testing.assert_allclose(s["pr3d"].reshape(N, L + 1), pres, rtol=1e-13)
        np.testing.assert_allclose(s["ex3d"].reshape(N, L + 1)[:, :L], exner[:, :L], rtol=1e-13)
        np.testing.assert_allclose(s["ws3d"].reshape(N, L), omega, rtol=1e-9, atol=1e-9)


def np_trcadv(grid, L, T, nf, of, vof, ab1, ab2, ab3, trc_edg, tracr, trcdp, trc_tdcy, trl_tdcy, massfx, delp):
    """trcadv_compute.F90 trcadv1..3 for every tracer, vectorised over cells."""
    N = grid.nip
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    proxs = np.asarray(grid.proxs).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    area = np.asarray(grid.area)
    rarea = 1.0 / area
    live = np.arange(6)[None, :] < npx[:, None]
    psl = np.where(live, proxs, 0)
    mf = massfx.reshape(3, N, 6, L)[nf]
    mfx = mf[prox, psl]
    te = trc_edg.reshape(T, N, 6, L)
    tr = tracr.reshape(T, N, L)
    td = trcdp.reshape(T, N, L)
    tc = trc_tdcy.reshape(T, 3, N, L)
    tl = trl_tdcy.reshape(T, 3, N, L)
    dp = delp.reshape(N, L)
    ring = [prox[:, e] for e in range(6)]
    for t in range(T):
        trt = tr[t]
        lo = np.where(live[:, :, None], 0.5 * ((mf + np.abs(mf)) * trt[:, None, :] - (mfx + np.abs(mfx)) * trt[prox]), 0.0)
        anti = np.where(live[:, :, None], mf * te[t] - lo, 0.0)
        acc = np.zeros((N, L))
        for e in range(6):
            acc = acc + np.where(live[:, e:e + 1], lo[:, e], 0.0)
        tl[t, nf] = -acc * rarea[:, None]
        tdlo = td[t] + ab1 * tl[t, nf] + ab2 * tl[t, of] + ab3 * tl[t, vof]
        mx, mn = trt.copy(), trt.copy()
        for x in ring:
            mx, mn = np.maximum(mx, trt[x]), np.minimum(mn, trt[x])
        mx, mn = np.maximum(0.0, mx), np.maximum(0.0, mn)
        trlo = np.maximum(mn, np.minimum(mx, tdlo / np.maximum(1e-11, dp)))
        sp, sm = np.zeros((N, L)), np.zeros((N, L))
        for e in range(6):
            a = np.where(live[:, e:e + 1], anti[:, e], 0.0)
            sp = sp - np.minimum(0.0, a)
            sm = sm + np.maximum(0.0, a)
        mx, mn = np.maximum(mx, trlo), np.minimum(mn, trlo)
        for x in ring:
            mx, mn = np.maximum(mx, trlo[x]), np.minimum(mn, trlo[x])
        mx, mn = np.maximum(0.0, mx), np.maximum(0.0, mn)
        qp = ((mx - trlo) * dp - (ab2 * np.minimum(0.0, tc[t, of]) + ab3 * np.maximum(0.0, tc[t, vof]))) / ab1 \
            * area[:, None]
        qm = ((trlo - mn) * dp + (ab2 * np.maximum(0.0, tc[t, of]) + ab3 * np.minimum(0.0, tc[t, vof]))) / ab1 \
            * area[:, None]
        rp = np.maximum(0.0, np.minimum(1.0, qp / np.maximum(sp, 1e-11)))
        rm = np.maximum(0.0, np.minimum(1.0, qm / np.maximum(sm, 1e-11)))
        clip = np.where(anti >= 0, np.minimum(rm[:, None, :], rp[prox]), np.minimum(rp[:, None, :], rm[prox]))
        at = np.zeros((N, L))
        for e in range(6):
            at = at + np.where(live[:, e:e + 1], anti[:, e] * clip[:, e], 0.0)
        tc[t, nf] = tl[t, nf] + (-at * rarea[:, None])
        td[t] = td[t] + ab1 * tc[t, nf] + ab2 * tc[t, of] + ab3 * tc[t, vof]
        tr[t] = np.maximum(mn, np.minimum(mx, td[t] / np.maximum(1e-11, dp)))


def test_trcadv_matches_numpy():
    """trcadv (FCT tracer transport) over three steps (Euler, AB2, AB3)."""
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    rng = np.random.default_rng(1504)
    s["tr3d"][N * L:] = rng.uniform(0.0, 1e-2, (T - 1) * N * L)
    s["trdp"][:T * N * L] = (s["tr3d"].reshape(T, N, L) * s["dp3d"].reshape(1, N, L)).ravel()
    for its in (1, 2, 3):
        o.abstart(its)
        o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"],
                  s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"],
                  s["trc_edg"])
        o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        o.cnuity(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["dp3d"], s["pr3d"],
                 s["ex3d"], s["dp_tdcy"], s["dpl_tdcy"], s["massfx"], s["ws3d"])
        ref = {k: s[k].copy() for k in ("tr3d", "trdp", "trc_tdcy", "trl_tdcy")}
        np_trcadv(grid, L, T, o.c.nf, o.c.of, o.c.vof, o.c.ab1, o.c.ab2, o.c.ab3, s["trc_edg"], ref["tr3d"],
                  ref["trdp"][:T * N * L], ref["trc_tdcy"], ref["trl_tdcy"], s["massfx"], s["dp3d"])
        o.trcadv(s["trc_edg"], s["tr3d"], s["trdp"], s["trc_tdcy"], s["trl_tdcy"], s["massfx"], s["dp3d"])
        for k in ("tr3d", "trdp", "trc_tdcy", "trl_tdcy"):
            np.testing.assert_allclose(s[k], ref[k], rtol=1e-11, atol=1e-15, err_msg="%d %s" % (its, k))


def test_edgvar1_matches_numpy():
    """edgvar1.F90:156-511 (eqwgt, janjic=0): rotated four-cell wind with the
    magnitude correction, mid-layer pressure, Montgomery potential, kinetic
    energy and theta on the cell's own edges."""
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    cs = np.asarray(grid.cs).reshape(N, 6, 4)
    sn = np.asarray(grid.sn).reshape(N, 6, 4)
    u, v = s["us3d"].reshape(N, L), s["vs3d"].reshape(N, L)
    pr, mo = s["pr3d"].reshape(N, L + 1), s["mp3d"].reshape(N, L)
    th = s["tr3d"].reshape(T, N, L)[0]
    plev = pr[:, :L] + pr[:, 1:]
    ue = np.zeros((N, 6, L)); ve = np.zeros((N, 6, L)); lp = np.zeros((N, 6, L))
    me = np.zeros((N, 6, L)); uv = np.zeros((N, 6, L)); te = np.zeros((N, 6, L))
    d6 = 1.0 / 6.0
    idx = np.arange(N)
    for e in range(6):
        live = e < npx
        i2 = prox[:, e]
        i3t = prox[idx, (e - 1 + npx) % npx]
        i3l = prox[idx, (e + 1) % npx]
        c, sg = cs[:, e, :], sn[:, e, :]
        rot = lambda q, x: (c[:, q:q + 1] * u[x] + sg[:, q:q + 1] * v[x],  # noqa: E731
                            -sg[:, q:q + 1] * u[x] + c[:, q:q + 1] * v[x])
        u3t, v3t = rot(2, i3t)
        u1, v1 = rot(0, idx)
        u2, v2 = rot(1, i2)
        u3l, v3l = rot(3, i3l)
        a = (2.0 * (u1 + u2) + u3t + u3l) * d6
        b = (2.0 * (v1 + v2) + v3t + v3l) * d6
        m2 = (2.0 * (np.sqrt(u1 * u1 + v1 * v1) + np.sqrt(u2 * u2 + v2 * v2)) + np.sqrt(u3t * u3t + v3t * v3t)
              + np.sqrt(u3l * u3l + v3l * v3l)) * d6
        m1 = np.sqrt(a * a + b * b)
        a = a * m2 / np.maximum(0.001, m1)
        b = b * m2 / np.maximum(0.001, m1)
        w = live[:, None]
        ue[:, e] = np.where(w, a, 0.0)
        ve[:, e] = np.where(w, b, 0.0)
        lp[:, e] = np.where(w, (plev[idx] + plev[i2] + 0.5 * (plev[i3t] + plev[i3l])) * d6, 0.0)
        me[:, e] = np.where(w, (2.0 * (mo[idx] + mo[i2]) + mo[i3t] + mo[i3l]) * d6, 0.0)
        uv[:, e] = np.where(w, 0.5 * (a * a + b * b), 0.0)
        te[:, e] = np.where(w, (2.0 * (th[idx] + th[i2]) + th[i3t] + th[i3l]) * d6, 0.0)
    for k in ("u_edg", "v_edg", "lp_edg", "mont_edg", "uvsq_edg"):
        s[k][:] = 0.0
    s["trc_edg"][:] = 0.0
    o.abstart(1)
    o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"], s["u_edg"],
              s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"], s["trc_edg"])
    for k, ref in (("u_edg", ue), ("v_edg", ve), ("lp_edg", lp), ("mont_edg", me), ("uvsq_edg", uv)):
        np.testing.assert_allclose(s[k].reshape(N, 6, L), ref, rtol=1e-13, atol=1e-9, err_msg=k)
    np.testing.assert_allclose(s["trc_edg"].reshape(T, N, 6, L)[0], te, rtol=1e-13, err_msg="trc_edg")


def test_momtum_matches_numpy():
    """momtum.F90:86-152 with dissip (momtum_compute.F90:102-229) and momtum1
    (231-450): ground-speed-shifted harmonic dissipation, Montgomery PGF and
    vorticity line integrals, Coriolis, AB3 update and the Rayleigh damping of
    the top quarter of the layers (forced here by a 120 m/s top jet)."""
    grid, cfg, o, s = _case()
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    cs = np.asarray(grid.cs).reshape(N, 6, 4)
    sn = np.asarray(grid.sn).reshape(N, 6, 4)
    svc = np.asarray(grid.sidevec_c).reshape(N, 6, 2)
    sve = np.asarray(grid.sidevec_e).reshape(N, 6, 2)
    sl = np.asarray(grid.sideln).reshape(N, 6)
    rarea, corio, grnd, dfflen = o.rarea, o.corio, o.grndspd, o.dfflen
    u3 = s["us3d"].reshape(N, L)
    u3[:, L - 3:] = 120.0  # above rlthresh: the damping acts
    for its in (1, 2, 3):
        o.abstart(its)
        o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"],
                  s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"],
                  s["trc_edg"])
        nf, of, vof, ab1, ab2, ab3, dt = o.c.nf, o.c.of, o.c.vof, o.c.ab1, o.c.ab2, o.c.ab3, o.c.dt
        u, v = s["us3d"].reshape(N, L).copy(), s["vs3d"].reshape(N, L).copy()
        dp = np.maximum(s["dp3d"].reshape(N, L), 1e-11)
        ex = s["ex3d"].reshape(N, L + 1)
        ue, ve = s["u_edg"].reshape(N, 6, L), s["v_edg"].reshape(N, 6, L)
        me, uv = s["mont_edg"].reshape(N, 6, L), s["uvsq_edg"].reshape(N, 6, L)
        te = s["trc_edg"].reshape(T, N, 6, L)[0]
        ut, vt = s["u_tdcy"].reshape(3, N, L).copy(), s["v_tdcy"].reshape(3, N, L).copy()
        # dissip on the ground-speed-shifted wind
        wu, wv = u + grnd[:, None], v.copy()
        su, sv = np.zeros((N, L)), np.zeros((N, L))
        factor = rarea[:, None] / dp
        for e in range(6):
            live = (e < npx)[:, None]
            x = prox[:, e]
            c0, s0, c1, s1 = cs[:, e, 0:1], sn[:, e, 0:1], cs[:, e, 1:2], sn[:, e, 1:2]
            uxy1, vxy1 = c0 * wu + s0 * wv, -s0 * wu + c0 * wv
            uxy2, vxy2 = c1 * wu[x] + s1 * wv[x], -s1 * wu[x] + c1 * wv[x]
            hf = dp * dp[x] / (dp + dp[x])
            ufx = (uxy2 - uxy1) * dfflen[None, :] * sl[:, e:e + 1] * 2.0 * hf
            vfx = (vxy2 - vxy1) * dfflen[None, :] * sl[:, e:e + 1] * 2.0 * hf
            su = np.where(live, su + (c0 * ufx - s0 * vfx) * factor, su)
            sv = np.where(live, sv + (s0 * ufx + c0 * vfx) * factor, sv)
        u, v = u + su, v + sv
        # momtum1
        exm = 0.5 * (ex[:, :L] + ex[:, 1:])
        pgx, pgy, rv = np.zeros((N, L)), np.zeros((N, L)), np.zeros((N, L))
        for e in range(6):
            live = (e < npx)[:, None]
            mu = me[:, e] + uv[:, e]
            pgx = np.where(live, pgx - mu * svc[:, e, 1:2] + exm * te[:, e] * svc[:, e, 1:2], pgx)
            pgy = np.where(live, pgy + mu * svc[:, e, 0:1] - exm * te[:, e] * svc[:, e, 0:1], pgy)
            rv = np.where(live, rv + (sve[:, e, 0:1] * ue[:, e] + sve[:, e, 1:2] * ve[:, e]), rv)
        pgx, pgy, rv = pgx * rarea[:, None], pgy * rarea[:, None], rv * rarea[:, None]
        ut[nf] = pgx + (corio[:, None] + rv) * v
        vt[nf] = pgy - (corio[:, None] + rv) * u
        u = u + ab1 * ut[nf] + ab2 * ut[of] + ab3 * ut[vof]
        v = v + ab1 * vt[nf] + ab2 * vt[of] + ab3 * vt[vof]
        q = np.maximum(np.maximum(u[:, L - 1] ** 2 + v[:, L - 1] ** 2, u[:, L - 2] ** 2 + v[:, L - 2] ** 2),
                       u[:, L - 3] ** 2 + v[:, L - 3] ** 2) / (cfg.rlthresh * cfg.rlthresh)
        damp = q > 1.0
        qq = np.sqrt(np.where(damp, (q - 1.0) * q, 0.0))
        ndamp = int(0.25 * L)
        for k in range(L - 1 - ndamp, L):
            f = 1.0 - (dt / 86400.0) * cfg.rleigh * qq * 2.0 ** (cfg.rltaper * (k + 1 - L))
            u[:, k] = np.where(damp, u[:, k] * f, u[:, k])
            v[:, k] = np.where(damp, v[:, k] * f, v[:, k])
        assert damp.any()
        o.momtum(s["us3d"], s["vs3d"], s["ex3d"], s["relvor"], s["u_edg"], s["v_edg"], s["trc_edg"],
                 s["mont_edg"], s["uvsq_edg"], s["u_tdcy"], s["v_tdcy"], s["dp3d"])
        np.testing.assert_allclose(s["relvor"].reshape(N, L), rv, rtol=1e-11, atol=1e-17, err_msg=str(its))
        np.testing.assert_allclose(s["u_tdcy"].reshape(3, N, L)[nf], ut[nf], rtol=1e-10, atol=1e-13)
        np.testing.assert_allclose(s["us3d"].reshape(N, L), u, rtol=1e-12, atol=1e-10, err_msg=str(its))
        np.testing.assert_allclose(s["vs3d"].reshape(N, L), v, rtol=1e-12, atol=1e-10, err_msg=str(its))


def test_mass_adv_matches_numpy():
    """mass_adv (flux_conserv_schm = 2): flux_limiter.F90 edge normal velocity
    and the M1 limiter, massflux_newdepth and update_pres, three AB steps."""
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, seed=1505, flux_conserv_schm=2)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    N, L = grid.nip, cfg.nvl
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    sve = np.asarray(grid.sidevec_e).reshape(N, 6, 2)
    svc = np.asarray(grid.sidevec_c).reshape(N, 6, 2)
    rarea = o.rarea
    idx = np.arange(N)
    for its in (1, 2, 3):
        o.abstart(its)
        o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"],
                  s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"],
                  s["trc_edg"])
        o.edgvar3(s["dp3d"], s["tr3d"], s["dp_edg"], s["trc_edg"])
        nf, of, vof, ab1, ab2, ab3, dt = o.c.nf, o.c.of, o.c.vof, o.c.ab1, o.c.ab2, o.c.ab3, o.c.dt
        ue, ve = s["u_edg"].reshape(N, 6, L), s["v_edg"].reshape(N, 6, L)
        dpe = s["dp_edg"].reshape(N, 6, L).copy()
        lpe = s["lp_edg"].reshape(N, 6, L)
        g = s["dp3d"].reshape(N, L).copy()
        pres = s["pr3d"].reshape(N, L + 1).copy()
        dpt = s["dp_tdcy"].reshape(3, N, L).copy()
        u, v = s["us3d"].reshape(N, L), s["vs3d"].reshape(N, L)
        vn = sve[:, :, 1:2] * ue - sve[:, :, 0:1] * ve
        cn = np.abs(vn) * dt * rarea[:, None, None]
        qs = np.zeros((N, 6, L))
        for e in range(6):
            x = prox[:, e]
            m1 = prox[idx, (e - 1 + npx) % npx]
            p1 = prox[idx, (e + 1) % npx]
            qmn = np.minimum(np.minimum(np.minimum(g, g[x]), g[m1]), g[p1])
            qmx = np.maximum(np.maximum(np.maximum(g, g[x]), g[m1]), g[p1])
            qs[:, e] = np.maximum(qmn, np.minimum(qmx, dpe[:, e]))
        qminin = np.full((N, L), np.finfo(np.float64).max)
        qmaxin, cqmin, cqmax, cin, cout = (np.zeros((N, L)) for _ in range(5))
        for e in range(6):
            live = (e < npx)[:, None]
            out = live & (vn[:, e] > 0)
            inn = live & ~(vn[:, e] > 0)
            x = prox[:, e]
            cout = np.where(out, cout + cn[:, e], cout)
            qmn = np.minimum(qs[:, e], g[x])
            qmx = np.maximum(qs[:, e], g[x])
            cin = np.where(inn, cin + cn[:, e], cin)
            qminin = np.where(inn, np.minimum(qminin, qmn), qminin)
            qmaxin = np.where(inn, np.maximum(qmaxin, qmx), qmaxin)
            cqmin = np.where(inn, cqmin + cn[:, e] * qmn, cqmin)
            cqmax = np.where(inn, cqmax + cn[:, e] * qmx, cqmax)
        qmin_next, qmax_next = np.minimum(g, qminin), np.maximum(g, qmaxin)
        tail = ab2 * dpt[of] + ab3 * dpt[vof]
        with np.errstate(divide="ignore", invalid="ignore"):
            qmo = (g + ab1 / dt * cqmax - qmax_next * (1.0 + cin - cout) + tail) / cout / ab1 * dt
            qxo = (g + ab1 / dt * cqmin - qmin_next * (1.0 + cin - cout) + tail) / cout / ab1 * dt
        qmo = np.where(cout != 0.0, qmo, -100000.0)
        qxo = np.where(cout != 0.0, qxo, 100000.0)
        mf = np.zeros((N, 6, L))
        for e in range(6):
            src = np.where(vn[:, e] > 0, idx[:, None], prox[:, e][:, None])
            kk = np.arange(L)[None, :]
            dpe[:, e] = np.maximum(qmo[src, kk], np.minimum(qxo[src, kk], qs[:, e]))
            mf[:, e] = np.where((e < npx)[:, None], vn[:, e] * dpe[:, e], 0.0)
        tsum = np.zeros((N, L))
        for e in range(6):
            tsum = tsum + mf[:, e]
        dpt[nf] = -tsum * rarea[:, None]
        g = np.maximum(g + ab1 * dpt[nf] + ab2 * dpt[of] + ab3 * dpt[vof], 0.0)
        omega = np.zeros((N, L))
        col = np.zeros(N)
        for k in range(L - 1, -1, -1):
            pres[:, k] = pres[:, k + 1] + g[:, k]
            lyr = (ab1 * dpt[nf][:, k] + ab2 * dpt[of][:, k] + ab3 * dpt[vof][:, k]) / dt
            om = col + 0.5 * lyr
            col = col + lyr
            dx, dy = np.zeros(N), np.zeros(N)
            for e in range(6):
                live = e < npx
                dx = np.where(live, dx + lpe[:, e, k] * svc[:, e, 1], dx)
                dy = np.where(live, dy - lpe[:, e, k] * svc[:, e, 0], dy)
            omega[:, k] = om + (u[:, k] * dx + v[:, k] * dy) * rarea
        o.mass_adv(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["dp_edg"], s["lp_edg"], s["dp3d"], s["pr3d"],
                   s["ex3d"], s["dp_tdcy"], s["massfx"], s["ws3d"])
        live = np.arange(6)[None, :] < npx[:, None]
        np.testing.assert_allclose(s["dp_edg"].reshape(N, 6, L)[live], dpe[live], rtol=1e-13, err_msg=str(its))
        np.testing.assert_allclose(s["massfx"].reshape(3, N, 6, L)[nf][live], mf[live], rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(s["dp3d"].reshape(N, L), g, rtol=1e-13)
        np.testing.assert_allclose(s["pr3d"].reshape(N, L + 1), pres, rtol=1e-13)
        np.testing.assert_allclose(s["ws3d"].reshape(N, L), omega, rtol=1e-9, atol=1e-9)
