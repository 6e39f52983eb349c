"""Restart files in the reference's layout (restart_dyn.F90): record
structure, write/read round trip, and a full reference-style file with
sections after the dynamics one."""
import struct

import numpy as np

import fimocn_subx_realtime_hera_apr2020_gb300 as F
from fimocn_subx_realtime_hera_apr2020_gb300.restart_io import STATE_FIELDS, read_restart, write_restart


def _fields(grid, cfg, seed=3):
    rng = np.random.Generator(np.random.PCG64(seed))
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    sizes = dict(u_tdcy=3 * N * L, v_tdcy=3 * N * L, dp_tdcy=3 * N * L, dpl_tdcy=3 * N * L, tr3d=T * N * L,
                 trdp=T * N * L, trc_tdcy=3 * T * N * L, trl_tdcy=3 * T * N * L, us3d=N * L, vs3d=N * L,
                 ws3d=N * L, mp3d=N * L, dp3d=N * L, relvor=N * L, pr3d=N * (L + 1), ex3d=N * (L + 1),
                 ph3d=N * (L + 1), sdot=N * (L + 1), massfx=18 * N * L, psrf=N, ptdcy=2 * N, dpinit=N * L,
                 cumufx=6 * N * L)
    assert set(sizes) == set(STATE_FIELDS)
    return {k: rng.standard_normal(n).astype(np.float32) for k, n in sizes.items()}


def _records(path):
    out = []
    with open(path, "rb") as fh:
        while True:
            h = fh.read(4)
            if not h:
                return out
            (n,) = struct.unpack("<i", h)
            fh.seek(n, 1)
            assert struct.unpack("<i", fh.read(4))[0] == n
            out.append(n)


def test_round_trip_and_layout(tmp_path):
    grid = F.Grid.cached(2)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0, precision="f32")
    f = _fields(grid, cfg)
    p = tmp_path / "restart_00000012"
    write_restart(str(p), grid, cfg, 12, 2, 1, 3, (7.5, -5.0, 2.5), f, extras={"qmstr": 1.5, "qdtr_set": True})
    N, L, T = grid.nip, cfg.nvl, cfg.ntra
    recs = _records(p)
    # itsm1, six scalar/table records, 12 AB3 slots, 8 per tracer, 9 cell, 4 interface, 3+1 edge records
    assert len(recs) == 1 + 6 + 12 + 8 * T + 9 + 4 + 4
    assert recs[0] == 4
    assert recs[1] == 4 * 4 + 4 * 3 + 4 * 2 * L + 4 * 2 * (L + 1)
    assert recs[2] == 4 * (N * 3 + N + 6 * N + 24 * N * 2 + N + 2 * N)
    assert recs[7] == 4 * N * L and recs[-1] == 4 * 6 * N * L
    r = read_restart(str(p), N, L, T)
    assert (r["itsm1"], r["nf"], r["of"], r["vof"]) == (12, 2, 1, 3)
    assert r["adbash"] == (7.5, -5.0, 2.5)
    assert r["extras"]["qmstr"] == 1.5 and r["extras"]["qdtr_set"]
    for k in STATE_FIELDS:
        assert np.array_equal(r["fields"][k], f[k]), k
    assert np.array_equal(r["extras"]["proxs"], grid.proxs)
    assert np.allclose(r["extras"]["dpsig"], cfg.dpsig, rtol=1e-6)


def test_reads_dynamics_section_of_full_file(tmp_path):
    """A reference restart file continues with the coupler/physics/ocean
    sections; the reader stops after the dynamics records."""
    grid = F.Grid.cached(2)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0, precision="f32")
    f = _fields(grid, cfg, seed=4)
    p = tmp_path / "restart_full"
    write_restart(str(p), grid, cfg, 3, 1, 3, 2, (1.0, 2.0, 3.0), f)
    with open(p, "ab") as fh:
        for n in (16, 4 * grid.nip):
            fh.write(struct.pack("<i", n) + bytes(n) + struct.pack("<i", n))
    r = read_restart(str(p), grid.nip, cfg.nvl, cfg.ntra)
    assert r["itsm1"] == 3 and np.array_equal(r["fields"]["massfx"], f["massfx"])
