"""Continuous-batching server: results are the same alone and in the mix."""
import copy

import numpy as np
import pytest

pytest.importorskip("torch")

import fimocn_subx_realtime_hera_apr2020_gb300 as F  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300.config import default_dt  # noqa: E402
from fimocn_subx_realtime_hera_apr2020_gb300.serve import Request, Server, latency_stats  # noqa: E402

pytestmark = pytest.mark.gpu


def _mix():
    return [Request(arrival=0.0, rid=0, glvl=2, nvl=38, ntra=5, steps=7, seed=11),
            Request(arrival=0.1, rid=1, glvl=2, nvl=38, ntra=5, steps=4, seed=12),
            Request(arrival=0.2, rid=2, glvl=3, nvl=38, ntra=6, steps=5, seed=13),
            Request(arrival=0.3, rid=3, glvl=2, nvl=38, ntra=5, steps=6, seed=14),
            Request(arrival=0.4, rid=4, glvl=2, nvl=38, ntra=5, steps=3, seed=15)]


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_same_alone_and_in_mix(precision):
    # two slots per grid pool, 8 tracer slots: later requests wait, join running
    # batches mid-forecast and reuse freed slots
    srv = Server(precision=precision, slots=2, max_tracers=8)
    mixed = {r.rid: r for r in srv.run(copy.deepcopy(_mix()), realtime=False)}
    srv.close()
    assert sorted(mixed) == [0, 1, 2, 3, 4]
    for req in _mix():
        # alone: a context sized for this request only (no padded tracer slots)
        alone = Server(precision=precision, slots=1, max_tracers=req.ntra)
        (r,) = alone.run([copy.deepcopy(req)], realtime=False)
        alone.close()
        for k, v in r.result.items():
            assert np.array_equal(np.asarray(v), np.asarray(mixed[req.rid].result[k])), (req.rid, k)
    st = latency_stats(list(mixed.values()))
    assert st["p99_s"] >= st["p50_s"] > 0


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_own_state_matches_plain_context(precision):
    """A request that brings its own host state, served beside seeded
    requests on a pool with padded tracer slots (joining mid-forecast), ends
    where a context of its own size stepping the same state ends, bit for
    bit."""
    grid = F.Grid.cached(2)
    cfg = F.FimConfig(nvl=38, ntra=5, dt=default_dt(2), precision=precision)
    fields = F.synthetic_state(grid, cfg, seed=77, sigma_ps=200.0, noise=0.5, dtype=cfg.dtype)
    own = Request(arrival=0.15, rid=9, glvl=2, nvl=38, ntra=5, steps=6, fields=fields)
    srv = Server(precision=precision, slots=2, max_tracers=8)
    done = {r.rid: r for r in srv.run(copy.deepcopy(_mix()[:2]) + [own], realtime=False)}
    srv.close()
    d = F.Dycore(grid, cfg)
    st = d.state()
    st.load(fields)
    st.init()
    for its in range(1, 7):
        st.step(its)
    for name in ("us3d", "tr3d"):
        assert np.array_equal(np.asarray(done[9].result[name]), st.download(name)), name
    st.free()
    d.close()


def test_device_state_is_seeded_and_balanced():
    """The seeded state made on the device in a member slot: hydrostatic
    columns from the drawn surface pressure, the slot's extra tracers zero,
    the same seed the same state and another seed another."""
    import torch
    grid = F.Grid.cached(3)
    N, L = grid.nip, 38
    d = F.Dycore(grid, F.FimConfig(nvl=L, ntra=6, dt=400.0, members=2))
    st = d.state()
    own = F.FimConfig(nvl=L, ntra=4, dt=400.0)

    def make(seed):
        F.synthetic_state_device(st, 1, grid, own, seed, sigma_ps=200.0, noise=0.5)
        torch.cuda.synchronize()
        return {n: st.download(n, 1) for n in ("us3d", "vs3d", "dp3d", "pr3d", "ex3d", "ph3d", "mp3d", "tr3d")}

    a = make(3)
    pr = a["pr3d"].reshape(N, L + 1)
    assert np.all(pr[:, L] == own.ptop)
    assert np.array_equal(a["dp3d"].reshape(N, L), pr[:, :L] - pr[:, 1:])
    assert np.all(a["dp3d"] > 0)
    dps = own.dpsig / own.dpsig.sum()
    assert np.allclose(a["dp3d"].reshape(N, L), (pr[:, :1] - own.ptop) * dps[None, :], rtol=1e-12)
    ps = pr[:, 0]
    assert abs(ps.mean() - 1e5) < 50.0 and 150.0 < ps.std() < 250.0
    assert np.allclose(a["ex3d"], F.state.CP * (a["pr3d"] / F.state.P1000) ** (F.state.RD / F.state.CP),
                       rtol=1e-14)
    du = a["us3d"].reshape(N, L) - 35.0 * np.cos(grid.lat)[:, None]
    assert 0.4 < du.std() < 0.6 and 0.4 < a["vs3d"].std() < 0.6
    assert not a["ph3d"].any() and not a["mp3d"].any()
    tr = a["tr3d"].reshape(6, N, L)
    assert np.array_equal(tr[0], np.broadcast_to(300.0 + 300.0 * np.arange(L) / (L - 1), (N, L)))
    assert tr[1:4].min() >= 0.0 and tr[1:4].max() < 1e-2 and tr[1:4].std() > 1e-3
    assert not tr[4:].any()
    b = make(3)
    assert all(np.array_equal(a[n], b[n]) for n in a)
    c = make(4)
    assert not np.array_equal(a["us3d"], c["us3d"]) and not np.array_equal(a["tr3d"], c["tr3d"])
    st.free()
    d.close()


def test_stream_priority():
    """fim_config.stream_priority sets the context stream's CUDA priority,
    clamped to the device's range (0 the lowest; -100 gives the highest)."""
    import torch
    grid = F.Grid.cached(2)
    got = {}
    for want in (0, -1, -100, 5):
        d = F.Dycore(grid, F.FimConfig(nvl=38, ntra=5, dt=400.0, stream_priority=want))
        got[want] = torch.cuda.ExternalStream(d.stream).priority
        d.close()
    assert got[0] == 0 and got[-1] == -1 and got[-100] < -1 and got[5] == 0


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_member_with_fewer_tracers(precision):
    """fim_member_set_tracers: a member carrying 5 of a context's 8 tracers
    evolves as in a context of 5 tracers, bit for bit (fields, tracers and
    budgets), leaves its other tracer slots as they are, and changes nothing
    for the member beside it."""
    from helpers import PROGNOSTIC
    grid = F.Grid.cached(3)
    L, NL = 38, grid.nip * 38
    cfg = lambda n, **kw: F.FimConfig(nvl=L, ntra=n, dt=400.0, precision=precision, **kw)  # noqa: E731
    f8 = F.synthetic_state(grid, cfg(8), seed=31, noise=1.0)
    f5 = F.synthetic_state(grid, cfg(5), seed=32, noise=1.0)
    pad = dict(f5)
    pad["tr3d"] = np.concatenate([f5["tr3d"], np.full(3 * NL, 7.0)])
    d = F.Dycore(grid, cfg(8, members=2))
    st = d.state()
    st.load(f8, member=0)
    st.load(pad, member=1)
    st.set_tracers(1, 5)
    st.init()
    alone = {}
    for n, f in ((8, f8), (5, f5)):
        da = F.Dycore(grid, cfg(n))
        sa = da.state()
        sa.load(f)
        sa.init()
        alone[n] = (da, sa)
    for its in (1, 2, 3):
        st.step(its, use_graph=True)
        for n in alone:
            alone[n][1].step(its)
    s8, s5 = alone[8][1], alone[5][1]
    for name in PROGNOSTIC:
        assert np.array_equal(st.download(name, 0), s8.download(name)), name
        got, want = st.download(name, 1), s5.download(name)
        if name in ("tr3d", "trdp"):
            got = got[:5 * NL]
        assert np.array_equal(got, want), name
    assert np.all(st.download("tr3d", 1)[5 * NL:] == 7.0)
    q1, b1 = st.budget(1)
    q5, b5 = s5.budget()
    assert np.array_equal(q1[:5], q5) and not q1[5:].any() and b1["qmass"] == b5["qmass"]
    assert np.array_equal(st.budget(0)[0], s8.budget()[0])
    assert st.check()[0] == 0


def test_set_tracers_rejects():
    grid = F.Grid.cached(2)
    d = F.Dycore(grid, F.FimConfig(nvl=38, ntra=6, dt=400.0, members=2))
    st = d.state()
    from fimocn_subx_realtime_hera_apr2020_gb300._lib import FimError
    for m, n in ((0, 0), (0, 7), (2, 3)):
        with pytest.raises(FimError):
            st.set_tracers(m, n)
    st.set_tracers(1, 6)
    d2 = F.Dycore(grid, F.FimConfig(nvl=38, ntra=6, dt=400.0, ntrb=2))
    with pytest.raises(FimError):
        d2.state().set_tracers(0, 3)


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_state_bytes_matches_the_library(precision):
    """serve.state_bytes (what admission by free HBM counts a slot at)
    covers one more member slot of a pool context, within 12%."""
    from fimocn_subx_realtime_hera_apr2020_gb300.serve import POOL_TRACER_CHUNK, state_bytes
    grid = F.Grid.cached(4)
    got = []
    for slots in (1, 3):
        d = F.Dycore(grid, F.FimConfig(nvl=64, ntra=9, dt=300.0, precision=precision, members=slots,
                                       tracer_chunk=POOL_TRACER_CHUNK))
        st = d.state()
        got.append(d.device_bytes())
        st.free()
        d.close()
    per_slot = (got[1] - got[0]) / 2
    est = state_bytes(4, 64, 9, precision)
    assert per_slot <= est <= 1.12 * per_slot, (per_slot, est)


def _draw(seed, stream, idx):
    """numpy restatement of the generator of fim_state_synthetic (SplitMix64's
    output function on a Weyl sequence keyed by seed and stream)."""
    g = np.uint64(0x9E3779B97F4A7C15)

    def mix(z):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))

    with np.errstate(over="ignore"):
        key = mix(np.uint64(seed) * g + np.uint64(stream))
        return mix(key + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * g)


def _unit(x, plus_one=False):
    return ((x >> np.uint64(11)) + np.uint64(1 if plus_one else 0)).astype(np.float64) * 2.0 ** -53


def test_synthetic_state_generator():
    """fim_state_synthetic against its numpy restatement: the drawn tracers
    bit for bit, the surface pressure and winds (Box-Muller through log and
    cos) to 1e-12."""
    grid = F.Grid.cached(3)
    N, L, T, seed = grid.nip, 38, 5, 4242
    d = F.Dycore(grid, F.FimConfig(nvl=L, ntra=T, dt=400.0))
    st = d.state()
    st.synthetic(0, seed, T, sigma_ps=200.0, noise=0.5)
    c = np.arange(N * L)
    tr = st.download("tr3d").reshape(T, N * L)
    for t in range(1, T):
        assert np.array_equal(tr[t], _unit(_draw(seed, 16 + t, c)) * 1e-2), t

    def normal(stream, idx):
        u1 = _unit(_draw(seed, stream, 2 * idx), plus_one=True)
        u2 = _unit(_draw(seed, stream, 2 * idx + 1))
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)

    ps = st.download("pr3d").reshape(N, L + 1)[:, 0]
    assert np.allclose(ps, 1e5 + normal(1, np.arange(N)) * 200.0, rtol=1e-12, atol=0)
    u = st.download("us3d")
    want_u = np.repeat(35.0 * np.cos(grid.lat), L) + normal(2, c) * 0.5
    assert np.allclose(u, want_u, rtol=0, atol=1e-11)
    assert np.allclose(st.download("vs3d"), normal(3, c) * 0.5, rtol=0, atol=1e-12)
    st.free()
    d.close()
