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
    assert state_bytes(6, 64, 11, "f64") == 2 * b32 or abs(state_bytes(6, 64, 11, "f64") - 2 * b32) <= 1
    assert state_bytes(7, 64, 11, "f32") > 3.9 * b32
    assert state_bytes(6, 64, 21, "f32") > b32
