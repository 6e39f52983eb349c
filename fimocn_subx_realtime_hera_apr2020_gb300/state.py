"""Seeded synthetic initial state (host, numpy; or on the device).

Stands in for the reference's GFS-derived initial condition (ss2icos,
dyn_init.F90:826), which is not in the tree: a hydrostatically balanced
column per cell with surface pressure 1000 hPa + N(0, sigma_ps), layer
thicknesses proportional to dpsig, potential temperature rising linearly
from 300 K to 600 K, zonal wind 35 m/s cos(lat) (+ optional N(0, noise) on
u and v), tracers 2..ntra and the ntrb class-B tracers drawn U[0, 1e-2],
flat topography.  Arrays are
flat in the reference layout (level index fastest).  The start-up hybgen and
hystat of dyn_init run afterwards on the device (fim_state_init).
"""
import numpy as np

CP = 1004.6855
RD = 287.0586
P1000 = 100000.0


def synthetic_state(grid, cfg, seed, sigma_ps=200.0, noise=0.0, dtype=np.float64):
    N, L, T = grid.nip, cfg.nvl, cfg.ntra + getattr(cfg, "ntrb", 0)
    rng = np.random.Generator(np.random.PCG64(seed))
    ps = P1000 + rng.standard_normal(N) * sigma_ps
    dps = cfg.dpsig / cfg.dpsig.sum()
    dp = (ps[:, None] - cfg.ptop) * dps[None, :]                      # (N, L)
    pr = np.empty((N, L + 1))
    pr[:, L] = cfg.ptop
    pr[:, :L] = cfg.ptop + np.cumsum(dp[:, ::-1], axis=1)[:, ::-1]   # top-down sums
    ex = CP * (pr / P1000) ** (RD / CP)
    theta = 300.0 + 300.0 * np.arange(L) / (L - 1)
    u = np.broadcast_to(35.0 * np.cos(grid.lat)[:, None], (N, L)).copy()
    v = np.zeros((N, L))
    if noise > 0.0:
        u += rng.standard_normal((N, L)) * noise
        v += rng.standard_normal((N, L)) * noise
    big = N * L * T > 100_000_000
    tr = np.empty((T, N, L), dtype=np.float32 if big else np.float64)
    tr[0] = theta[None, :]
    if T > 1:
        if big:
            for t in range(1, T):
                tr[t] = rng.random((N, L), dtype=np.float32) * np.float32(1e-2)
        else:
            tr[1:] = rng.random((T - 1, N, L)) * 1e-2
    out = dict(us3d=u, vs3d=v, dp3d=pr[:, :L] - pr[:, 1:], pr3d=pr, ex3d=ex,
               ph3d=np.zeros((N, L + 1)), mp3d=np.zeros((N, L)), tr3d=tr)
    return {k: np.ascontiguousarray(a, dtype=dtype).reshape(-1) for k, a in out.items()}


def synthetic_state_device(st, member, grid, cfg, seed, sigma_ps=200.0, noise=0.0):
    """The balanced state of synthetic_state, made on the device straight
    into member slot `member` of a State by the library's own kernels
    (fim_state_synthetic): the same recipe, drawn from a counter-based
    generator (so other random numbers than the host PCG64 stream; the same
    seed and grid give the same state in any slot or context).  Tracers of
    the slot past cfg.ntra + cfg.ntrb are zeroed.  Asynchronous on the
    library's stream."""
    if grid.nip != st.dyc.grid.nip or cfg.nvl != st.dyc.cfg.nvl:
        raise ValueError("the state's grid and levels differ from the context's")
    st.synthetic(member, seed, cfg.ntra + getattr(cfg, "ntrb", 0), sigma_ps=sigma_ps, noise=noise)
