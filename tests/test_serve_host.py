"""Host logic of the serving benchmark, on the CPU: the seeded Poisson
request stream of the served mix (glvl 5-7, nvl 38/64, 4-20 tracers), the latency statistics and the per-slot
HBM estimate that admission uses."""
import numpy as np

from fimocn_subx_realtime_hera_apr2020_gb300.serve import Request, latency_stats, poisson_requests, state_bytes


def test_poisson_stream_is_seeded_and_in_range():
    a = poisson_requests(200, 20.0, seed=5000)
    b = poisson_requests(200, 20.0, seed=5000)
    assert [(r.arrival, r.glvl, r.nvl, r.ntra, r.steps) for r in a] == \
           [(r.arrival, r.glvl, r.nvl, r.ntra, r.steps) for r in b]
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) > 0)
    # mean inter-arrival 1/rate within sampling error
    assert abs(np.diff(np.concatenate([[0.0], t])).mean() - 1 / 20.0) < 0.02
    assert {r.glvl for r in a} <= {5, 6, 7} and {r.nvl for r in a} <= {38, 64}
    assert all(5 <= r.ntra <= 21 and 24 <= r.steps <= 240 for r in a)  # theta + 4..20 tracers
    assert len({r.seed for r in a}) == 200
    assert poisson_requests(5, 20.0, seed=5001)[0].arrival != a[0].arrival


def test_request_work_and_grouping():
    r = Request(arrival=0.0, rid=0, glvl=5, nvl=38, ntra=5, steps=24)
    assert r.work == (10 * 4 ** 5 + 2) * 38 * 24
    assert r.key == (5, 38)
    assert Request(arrival=1.0, rid=1, glvl=5, nvl=38, ntra=9, steps=50).key == r.key


def test_latency_stats():
    done = []
    for i, lat in enumerate([1.0, 2.0, 3.0, 4.0, 10.0]):
        r = Request(arrival=float(i), rid=i, glvl=5, nvl=38, ntra=5, steps=24)
        r.t_queue, r.t_done = float(i), float(i) + lat
        done.append(r)
    st = latency_stats(done)
    assert st["requests"] == 5
    assert st["p50_s"] == 3.0
    assert abs(st["p99_s"] - np.percentile([1, 2, 3, 4, 10], 99)) < 1e-12
    assert abs(st["mean_s"] - 4.0) < 1e-12
    span = 14.0 - 0.0
    assert abs(st["cell_level_steps_per_s"] - 5 * done[0].work / span) < 1e-6


def test_state_bytes_scales():
    b32 = state_bytes(6, 64, 11, "f32")
    # FP64 words are twice as wide; the FP32-mixed state keeps three more
    # values a cell-level (float-float Montgomery potential, theta copy)
    assert 1.9 < state_bytes(6, 64, 11, "f64") / b32 < 2.0
    assert state_bytes(7, 64, 11, "f32") > 3.9 * b32
    assert state_bytes(6, 64, 21, "f32") > b32


class _FakePool:
    """Stands in for serve.Pool: a step of a pool on grid level glvl stays in
    flight for glvl - 4 polls of its stream."""
    made = []

    def __init__(self, key, precision, slots, collect, ntra, priority=0):
        self.key, self.priority = key, priority
        self.slots = [None] * slots
        self.its = [0] * slots
        self.inflight = 0
        self.steps_launched = 0
        _FakePool.made.append(self)

    def free_slot(self):
        return next((i for i, r in enumerate(self.slots) if r is None), -1)

    def admit(self, req, now):
        assert self.inflight == 0, "admitted while a step was in flight"
        m = self.free_slot()
        self.slots[m], self.its[m] = req, 0
        req.t_admit = now

    def active(self):
        return any(r is not None for r in self.slots)

    def idle(self):
        if self.inflight:
            self.inflight -= 1
        return self.inflight == 0

    def step(self):
        assert self.inflight == 0, "stepped while a step was in flight"
        for m, r in enumerate(self.slots):
            if r is not None:
                self.its[m] += 1
        self.inflight = self.key[0] - 4
        self.steps_launched += 1

    def finished(self):
        return [m for m, r in enumerate(self.slots) if r is not None and self.its[m] >= r.steps]

    def retire(self, m, now):
        assert self.inflight == 0, "retired while a step was in flight"
        r = self.slots[m]
        assert self.its[m] == r.steps
        r.t_done, r.result = now, {"steps": self.its[m]}
        self.slots[m] = None
        return r

    def close(self):
        pass


def _run_fake(monkeypatch, priorities):
    import torch
    import fimocn_subx_realtime_hera_apr2020_gb300.serve as S
    _FakePool.made = []
    monkeypatch.setattr(S, "Pool", _FakePool)
    monkeypatch.setattr(S.Server, "_free_hbm", lambda self: 1e15)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    reqs = [Request(arrival=0.0, rid=i, glvl=g, nvl=38, ntra=5, steps=n)
            for i, (g, n) in enumerate([(7, 12), (5, 12), (7, 6), (5, 20), (5, 3), (6, 9), (5, 7)])]
    srv = S.Server(slots=2, priorities=priorities)
    done = srv.run(reqs, realtime=False)
    srv.close()
    return done


def test_serving_loop_pools_at_their_own_pace(monkeypatch):
    """The request loop on fake pools: every request runs its steps, a pool is
    admitted to, stepped and retired only between its steps, a small grid's
    pool takes several steps while a larger grid's step is in flight, and
    smaller grids get higher stream priorities."""
    done = _run_fake(monkeypatch, priorities=True)
    assert sorted(r.rid for r in done) == list(range(7))
    assert all(r.result["steps"] == r.steps for r in done)
    pools = {p.key[0]: p for p in _FakePool.made}
    assert {g: p.priority for g, p in pools.items()} == {5: -3, 6: -2, 7: -1}
    # 42 steps of glvl-5 requests on 2 slots against 18 of glvl 7
    assert pools[5].steps_launched > pools[7].steps_launched
    # the glvl-5 requests do not wait for the glvl-7 ones: the last glvl-5
    # request is done before the last glvl-7 one
    by = {g: max(r.t_done for r in done if r.glvl == g) for g in (5, 7)}
    assert by[5] < by[7]
    _run_fake(monkeypatch, priorities=False)
    assert {p.priority for p in _FakePool.made} == {0}
