"""The persistent cnuity1..4 launch and its time-limited grid barriers.

fim_set_persistent runs cnuity1 to cnuity4 of every member as one cooperative
launch with grid barriers between the stages.  Its results must equal the
kernel-per-stage path's bit for bit.  Each barrier gives up after its time
limit: a barrier made to wait for a block that never arrives
(fim_set_barrier_test) must end the launch, fim_check must report
FIM_ETIMEDOUT, and the context must keep working afterwards.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300 import _lib  # noqa: E402
from helpers import PROGNOSTIC, make_case  # noqa: E402

pytestmark = pytest.mark.gpu


def _state(grid, cfg, fields, persistent):
    d = F.Dycore(grid, cfg)
    if persistent:
        d.set_persistent(True)
    st = d.state()
    for m in range(cfg.members):
        st.load(fields[m], member=m)
    st.init()
    return d, st


@pytest.mark.parametrize("precision,members", [("f64", 1), ("f32", 1), ("f32", 3)])
def test_persistent_matches_kernels(precision, members):
    grid, cfg, f0 = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1701, noise=1.0, precision=precision,
                              members=members)
    fields = [f0] + [F.synthetic_state(grid, cfg, seed=1702 + m, sigma_ps=150.0, noise=0.5)
                     for m in range(1, members)]
    _, ref = _state(grid, cfg, fields, False)
    _, st = _state(grid, cfg, fields, True)
    for its in (1, 2, 3):
        ref.step(its, use_graph=True)
        st.step(its, use_graph=its != 2)
    for m in range(members):
        for n in PROGNOSTIC + ["massfx", "dp_tdcy", "ws3d"]:
            assert np.array_equal(st.download(n, m), ref.download(n, m)), (m, n)
    rc, flags = st.check()
    assert rc == 0 and flags == 0


def test_persistent_barrier_time_limit():
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1703, noise=1.0, precision="f32")
    dyc, st = _state(grid, cfg, [fields], True)
    dyc.set_persistent(True, timeout_s=0.05)
    dyc.set_barrier_test(1)
    st.step(1, use_graph=False)
    rc, flags = st.check()
    assert rc == _lib.FIM_ETIMEDOUT and flags & 8, (rc, flags)
    # the context keeps working: a fresh state steps cleanly afterwards
    dyc.set_barrier_test(0)
    st2 = dyc.state()
    st2.load(fields)
    st2.init()
    st2.step(1, use_graph=True)
    rc, flags = st2.check()
    assert rc == 0 and flags == 0
    _, ref = _state(grid, cfg, [fields], False)
    ref.step(1, use_graph=True)
    for n in PROGNOSTIC:
        assert np.array_equal(st2.download(n), ref.download(n)), n
