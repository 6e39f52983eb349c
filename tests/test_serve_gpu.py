"""Continuous-batching server: results are the same alone and in the mix."""
import copy

import numpy as np
import pytest

pytest.importorskip("torch")

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
