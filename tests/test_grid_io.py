"""glvl.dat (the reference's on-disk grid) round trip."""
import numpy as np

import fimocn_subx_realtime_hera_apr2020_gb300 as F
from fimocn_subx_realtime_hera_apr2020_gb300.grid_io import read_glvl_dat, write_glvl_dat


def test_round_trip(tmp_path):
    g = F.Grid.cached(3)
    p = tmp_path / "glvl.dat"
    write_glvl_dat(g, p)
    t = read_glvl_dat(p, glvl=3)
    assert t.nip == g.nip and t.curve == 0
    for n in ("nprox", "prox", "proxs"):
        assert np.array_equal(getattr(t, n), getattr(g, n)), n
    for n in ("lat", "lon", "area", "cs", "sn", "sidevec_c", "sidevec_e", "sideln", "rprox_ln", "corner_xy",
              "hfcoef"):
        assert np.array_equal(getattr(t, n), getattr(g, n).astype(np.float32).astype(np.float64)), n
    assert np.array_equal(t.perm, np.arange(1, g.nip + 1))
    # record framing: 2 headers + 3 + 12 + 1 + 48 + 24 + 12 + 1 + 12 + 36 records
    raw = p.read_bytes()
    nrec, off = 0, 0
    while off < len(raw):
        (n,) = np.frombuffer(raw[off:off + 4], "<i4")
        off += 8 + int(n)
        nrec += 1
    assert nrec == 2 + 3 + 12 + 1 + 48 + 24 + 12 + 1 + 12 + 36


def test_file_grid_feeds_oracle(tmp_path):
    """A grid read back from glvl.dat drives the dycore like the in-memory one."""
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    from oracle import Oracle
    g = F.Grid.cached(2)
    write_glvl_dat(g, tmp_path / "glvl.dat")
    t = read_glvl_dat(tmp_path / "glvl.dat")
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0)
    fields = F.synthetic_state(t, cfg, seed=5)
    o = Oracle(t, cfg)
    s = o.init_state(o.new_state(fields))
    _, b0 = o.globsum(s["dp3d"], s["tr3d"], s["pr3d"], s["ex3d"])
    _, b1 = o.step(s, 1)
    assert abs(b1["qmass"] / b0["qmass"] - 1) < 1e-12
    assert np.all(np.isfinite(s["us3d"]))
