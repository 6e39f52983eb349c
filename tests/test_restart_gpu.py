"""A forecast saved to a restart file after step 2 and resumed in a fresh
context reproduces the uninterrupted forecast bit for bit (FP32-mixed state,
whose fields are exactly the file's 32-bit records)."""
import numpy as np
import pytest

pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402

pytestmark = pytest.mark.gpu

FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "ws3d", "relvor", "sdot",
          "massfx", "trc_tdcy", "u_tdcy"]


def _start(grid, cfg, fields):
    d = F.Dycore(grid, cfg)
    st = d.state()
    st.load(fields)
    st.init()
    return d, st


@pytest.mark.parametrize("use_graph", [False, True])
def test_restart_resumes_bit_identical(tmp_path, use_graph):
    grid = F.Grid.cached(3)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=F.default_dt(3), precision="f32")
    fields = F.synthetic_state(grid, cfg, seed=31, sigma_ps=200.0, noise=1.0, dtype=np.float32)
    d1, s1 = _start(grid, cfg, fields)
    for its in range(1, 5):
        s1.step(its, use_graph=use_graph)
    ref = {n: s1.download(n) for n in FIELDS}
    d2, s2 = _start(grid, cfg, fields)
    for its in (1, 2):
        s2.step(its, use_graph=use_graph)
    path = str(tmp_path / "restart_00000002")
    assert s2.save_restart(path) == 2
    d3 = F.Dycore(grid, cfg)
    s3 = d3.state()
    r = s3.load_restart(path)
    assert r["itsm1"] == 2 and s3.get_step(0)[0] == 2
    for its in (3, 4):
        s3.step(its, use_graph=use_graph)
    for n in FIELDS:
        assert np.array_equal(s3.download(n), ref[n]), n
    for d, s in ((d1, s1), (d2, s2), (d3, s3)):
        s.free()
        d.close()
