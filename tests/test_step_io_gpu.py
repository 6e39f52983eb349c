"""fim_step_io: the step with the state kept in host buffers.

The fields a step reads go up stage by stage and the fields it writes come
down as soon as they are final, on copy streams beside the kernels.  Before
every step the device copy of every registered field is overwritten with
NaN, so any field (or AB3 slot) that the step read without having uploaded
it, or any upload that landed after a kernel wrote the field, would show up
in the results.  Five steps must equal a resident run bit for bit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from helpers import make_case  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300._lib import FimError  # noqa: E402

pytestmark = pytest.mark.gpu

FIELDS = ["us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d", "trdp", "u_tdcy", "v_tdcy", "dp_tdcy",
          "dpl_tdcy", "trc_tdcy", "trl_tdcy", "ws3d", "sdot", "relvor", "psrf", "ptdcy"]
AB3 = {"u_tdcy", "v_tdcy", "dp_tdcy", "dpl_tdcy", "trc_tdcy", "trl_tdcy"}
OUT = {"ws3d", "sdot", "relvor"}
# rewritten whole by the step's opening hybgen and hystat from the second
# step on, so they go up only at the first step (the poison then shows they
# are not read)
RECOMPUTED = {"mp3d", "trdp", "dp3d"}


def _state(grid, cfg, fields):
    d = F.Dycore(grid, cfg)
    st = d.state()
    st.load(fields)
    st.init()
    return d, st


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_step_io_matches_resident(precision):
    grid, cfg, fields = make_case(glvl=4, nvl=38, ntra=5, dt=400.0, seed=1601, noise=1.0, precision=precision)
    _, ref = _state(grid, cfg, fields)
    _, st = _state(grid, cfg, fields)
    tdt = torch.float64 if precision == "f64" else torch.float32
    NL = grid.nip * cfg.nvl
    host = {}
    for f in FIELDS:
        n = st.field_ptr(f)[1]
        host[f] = torch.empty(n, dtype=tdt, pin_memory=True)
        st.download(f, out=host[f].numpy())
        st.set_host(f, host[f])
    esz = 8 if precision == "f64" else 4
    def want_up(its):
        return sum(host[f].numel() for f in FIELDS
                   if f not in OUT and f not in AB3 and not (its > 1 and f in RECOMPUTED)) * esz + \
            sum(2 * host[f].numel() // 3 for f in AB3) * esz
    want_down = sum(host[f].numel() for f in FIELDS if f not in AB3) * esz + \
        sum(host[f].numel() // 3 for f in AB3) * esz
    for its in range(1, 6):
        for f in FIELDS:
            st.upload(f, np.full(host[f].numel(), np.nan))
        up, down = st.step_io(its)
        ref.step(its, use_graph=True)
        assert (up, down) == (want_up(its), want_down)
        for f in FIELDS:
            got = host[f].numpy()
            want = ref.download(f)
            if f in AB3:
                # the slot the step wrote; the others are the host's own copies
                nf = st.get_step()[1] - 1  # slot the step just done wrote, 0-based
                nb = want.size // (3 * NL)
                got = got.reshape(nb, 3, NL)[:, nf]
                want = want.reshape(nb, 3, NL)[:, nf]
            if f == "sdot" and its == 1:
                continue  # hybgen does not run at the first step: the poison stays
            assert np.array_equal(got, want), (its, f)
    rc, flags = st.check()
    assert rc == 0 and flags == 0


def test_step_io_rejects_member_groups():
    grid = F.Grid.cached(3)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=400.0, precision="f32", members=2, member_group=1)
    d = F.Dycore(grid, cfg)
    st = d.state()
    with pytest.raises(FimError):
        st.step_io(1)
    with pytest.raises(FimError):
        st.set_host("u_edg", None)


def test_step_io_timeline():
    """With the profiler on, fim_step_io reports its timeline: each stage's
    uploads end before its kernels are done, the downloads of a stage end
    after its kernels, and the step ends last; a second step with the same
    marks doubles their counts."""
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=7, dt=400.0, seed=1602, noise=1.0, precision="f32")
    d, st = _state(grid, cfg, fields)
    for f in FIELDS:
        n = st.field_ptr(f)[1]
        h = torch.empty(n, dtype=torch.float32, pin_memory=True)
        st.download(f, out=h.numpy())
        st.set_host(f, h)
    d.profile(True)
    st.step_io(1)
    st.step_io(2)
    rep = d.profile_report()
    d.profile(False)
    io = {k[3:]: (n, ms / n) for k, (n, ms) in rep.items() if k.startswith("io:")}
    assert io["start"] == (2, 0.0)
    end = io["end"][1]
    stages = {k.split(".", 1)[1] for k in io if k.startswith("computed.")}
    assert {"A.0", "C.0", "U.0", "E.0"} <= stages and any(s.startswith("T.") for s in stages)
    for s in stages:
        assert io["computed." + s][0] == 2
        assert io["computed." + s][1] <= io["down_begin." + s][1] <= io["down_end." + s][1] <= end, s
        if "up_end." + s in io:
            assert io["up_end." + s][1] <= io["computed." + s][1] + 1e-6, s
    # kernel timings are reported beside the marks
    assert any(not k.startswith("io:") for k in rep)


def test_step_io_tendencies_on_device():
    """A driver that registers only the state fields and leaves the AB3
    tendency history on the device: the same steps as a resident run, bit
    for bit, with only those fields moved."""
    grid, cfg, fields = make_case(glvl=3, nvl=38, ntra=5, dt=400.0, seed=1603, noise=1.0, precision="f32")
    _, ref = _state(grid, cfg, fields)
    _, st = _state(grid, cfg, fields)
    host = {}
    for f in FIELDS:
        if f in AB3:
            continue
        host[f] = torch.empty(st.field_ptr(f)[1], dtype=torch.float32, pin_memory=True)
        st.download(f, out=host[f].numpy())
        st.set_host(f, host[f])
    for its in range(1, 5):
        up, down = st.step_io(its)
        ref.step(its, use_graph=True)
        assert down == sum(h.numel() for h in host.values()) * 4
        for f in FIELDS:
            got = host[f].numpy() if f in host else st.download(f)
            if f == "sdot" and its == 1:
                continue  # hybgen does not run at the first step
            assert np.array_equal(got, ref.download(f)), (its, f)
