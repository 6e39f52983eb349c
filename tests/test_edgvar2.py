"""edgvar2 (edgvar2.F90:24-319, hiOrderUVComp): the C oracle against a
vectorised NumPy restatement of uv_speed_edge / gradient / uv_speed and the
per-edge magnitude correction, on a state after edgvar1."""
import numpy as np

from helpers import make_case, oracle_for


def np_edgvar2(grid, L, u, v, u_edg, v_edg):
    N = grid.nip
    prox = np.asarray(grid.prox).reshape(N, 6) - 1
    proxs = np.asarray(grid.proxs).reshape(N, 6) - 1
    npx = np.asarray(grid.nprox)
    svc = np.asarray(grid.sidevec_c).reshape(N, 6, 2)
    cxy = np.asarray(grid.corner_xy).reshape(N, 2, 6)
    rarea = 1.0 / np.asarray(grid.area)
    ue, ve = u_edg.reshape(N, 6, L).copy(), v_edg.reshape(N, 6, L).copy()
    live = (np.arange(6)[None, :] < npx[:, None])[:, :, None]
    spe = np.where(live, np.sqrt(ue * ue + ve * ve), 0.0)
    g1 = (spe * svc[:, :, 1:2]).sum(axis=1) * rarea[:, None]
    g2 = -(spe * svc[:, :, 0:1]).sum(axis=1) * rarea[:, None]
    gc = 0.5 * (g1[:, None, :] * cxy[:, 0, :, None] + g2[:, None, :] * cxy[:, 1, :, None])
    spd = np.sqrt(u.reshape(N, L) ** 2 + v.reshape(N, L) ** 2)
    uvsq = np.zeros((N, 6, L))
    for i in range(N):
        n = npx[i]
        for e in range(n):
            nba, nbaedg = prox[i, e], proxs[i, e]
            em1, ep1 = (e - 1 + n) % n, (e + 1) % n
            nbm1, nbp1 = prox[i, em1], prox[i, ep1]
            corners = [(i, e), (nba, (nbaedg + 1) % npx[nba]), (nbm1, proxs[i, em1]),
                       (i, (e + 1) % n), (nba, nbaedg), (nbp1, (proxs[i, ep1] + 1) % npx[nbp1])]
            uvm2 = sum(spd[c] + gc[c, q] for c, q in corners) / 6.0
            uvm1 = np.sqrt(ue[i, e] ** 2 + ve[i, e] ** 2)
            r = np.where(uvm1 < 1e-5, 1.0, uvm2 / np.where(uvm1 < 1e-5, 1.0, uvm1))
            ue[i, e] *= r
            ve[i, e] *= r
            uvsq[i, e] = 0.5 * (ue[i, e] ** 2 + ve[i, e] ** 2)
    return ue.ravel(), ve.ravel(), uvsq.ravel()


def test_edgvar2_oracle_matches_numpy():
    grid, cfg, fields = make_case(glvl=2, nvl=38, ntra=5, seed=1400)
    o = oracle_for(grid, cfg)
    s = o.init_state(o.new_state(fields))
    o.abstart(1)
    o.edgvar1(s["us3d"], s["vs3d"], s["dp3d"], s["pr3d"], s["ex3d"], s["ph3d"], s["mp3d"], s["tr3d"], s["u_edg"],
              s["v_edg"], s["dp_edg"], s["lp_edg"], s["geop_edg"], s["mont_edg"], s["uvsq_edg"], s["trc_edg"])
    ue0, ve0 = s["u_edg"].copy(), s["v_edg"].copy()
    ru, rv, rq = np_edgvar2(grid, cfg.nvl, s["us3d"], s["vs3d"], ue0, ve0)
    o.edgvar2(s["us3d"], s["vs3d"], s["u_edg"], s["v_edg"], s["uvsq_edg"])
    np.testing.assert_allclose(s["u_edg"], ru, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(s["v_edg"], rv, rtol=1e-12, atol=1e-12)
    mask = rq != 0.0  # pentagon slot 5 is not written by either
    np.testing.assert_allclose(s["uvsq_edg"][mask], rq[mask], rtol=1e-12, atol=1e-12)
    # the correction moves the edge wind: not the identity on this state
    assert np.abs(s["u_edg"] - ue0).max() > 1e-6
