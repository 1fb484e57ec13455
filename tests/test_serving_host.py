"""Host-side pieces of the serving loop (no GPU): request ordering, the HBM footprint used
for admission, and the latency / throughput summary."""
import heapq
import types

import numpy as np

from fermicg_gb300.serving import Request, Result, footprint_bytes, latency_summary


def _req(arrival, rid, n=1000, R=2, tdm=5000, ints=300):
    ops = types.SimpleNamespace(data=np.zeros(tdm))
    terms = types.SimpleNamespace(ints=np.zeros(ints))
    return Request(arrival, rid, ops, terms, np.zeros((n, 4, 2), np.int16), np.zeros((n, 4), np.int16),
                   np.zeros((n, R)))


def test_requests_queue_by_arrival_only():
    q = []
    for r in (_req(0.3, 0), _req(0.1, 1), _req(0.2, 2)):
        heapq.heappush(q, r)
    assert [heapq.heappop(q).rid for _ in range(3)] == [1, 2, 0]
    assert sorted([_req(0.5, 7), _req(0.5, 3)])[0].arrival == 0.5  # equal arrivals do not compare payloads


def test_footprint_grows_with_the_space_and_the_roots():
    base = footprint_bytes(_req(0.0, 0))
    assert base > 0
    assert footprint_bytes(_req(0.0, 0, n=2000)) > base
    assert footprint_bytes(_req(0.0, 0, R=4)) > base
    assert footprint_bytes(_req(0.0, 0, tdm=50000)) > base
    # the Davidson subspace alone: 2 x (12 R + R) vectors of n doubles
    small = footprint_bytes(_req(0.0, 0, n=1, R=1, tdm=0, ints=0))
    big = footprint_bytes(_req(0.0, 0, n=1001, R=1, tdm=0, ints=0))
    assert big - small >= 1000 * 8 * 2 * 13


def test_latency_summary():
    res = [Result(i, "s", np.zeros(1), np.zeros(1), 10, arrival=0.1 * i, start=0.1 * i, end=0.1 * i + 0.5)
           for i in range(10)]
    s = latency_summary(res)
    assert s["n"] == 10
    assert abs(s["p50_s"] - 0.5) < 1e-12 and abs(s["p99_s"] - 0.5) < 1e-12 and abs(s["mean_s"] - 0.5) < 1e-12
    assert abs(s["solves_per_s"] - 10 / 1.4) < 1e-9  # from the first arrival to the last result
