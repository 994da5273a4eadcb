"""The serving loop's host logic on CPU: admission under the HBM budget,
continuous batching over slots, latency bookkeeping, and that a request's
result is the same alone and in a mix.  The oracle stands in for the GPU
executor; the GPU path is in test_gpu_serve.py."""
from __future__ import annotations

import threading

import numpy as np

import cortrace as ct
import pyoracle
import serve


def _small(reqs):
    for r in reqs:
        r.rig = (4.0, 20.0, 4.0)          # 5 rigidities: the oracle finishes in milliseconds
        r.external = ct.EXTERNAL_T96
    return reqs


class _Oracle:
    def __init__(self, server_ref):
        self.server_ref = server_ref
        self.peak = 0
        self.lock = threading.Lock()

    def __call__(self, ctx, jobs, params, models, feats):
        with self.lock:
            self.peak = max(self.peak, self.server_ref[0].in_flight)
        res = pyoracle.scan_batch(jobs, params, models=models, threads=2)
        return res.sites, np.zeros(len(jobs), bool)


def _run(reqs, budget=40e9, slots=2):
    ref = [None]
    ex = _Oracle(ref)
    srv = serve.Server(slots=slots, hbm_budget=budget, executor=ex)
    ref[0] = srv
    out = serve.run_stream(srv, reqs)
    return out, ex.peak, srv


def test_stream_is_seeded_and_shaped():
    a = serve.poisson_stream(3, 5.0, 12)
    b = serve.poisson_stream(3, 5.0, 12)
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert all(len(r.directions) in (1, 9) for r in a)
    assert all(1 <= len(r.sites) <= 64 for r in a)


def test_results_same_alone_and_in_mix():
    mix = _small(serve.poisson_stream(5, 200.0, 6, max_box_sites=4))
    out, _, _ = _run(mix)
    assert out["completed"] == 6 and out["rejected"] == 0
    for k in (0, 3):
        alone = _small([serve.poisson_stream(5, 200.0, 6, max_box_sites=4)[k]])
        alone[0].arrival = 0.0
        _run(alone)
        assert np.array_equal(alone[0].result.view(np.uint8), mix[k].result.view(np.uint8))
    for r in mix:
        assert r.done_at >= r.arrival
    assert out["latency_p50_s"] <= out["latency_p99_s"]


def test_admission_keeps_in_flight_memory_under_budget():
    reqs = _small(serve.poisson_stream(9, 1000.0, 8, max_box_sites=4))
    budget = 2 * max(r.device_bytes() for r in reqs)
    out, peak, srv = _run(reqs, budget=budget, slots=3)
    assert out["completed"] == 8
    assert 0 < peak <= budget
    assert srv.in_flight == 0


def test_request_over_budget_is_rejected():
    reqs = _small(serve.poisson_stream(11, 100.0, 3, max_box_sites=4))
    budget = min(r.device_bytes() for r in reqs) - 1
    out, _, srv = _run(reqs, budget=budget)
    assert out["rejected"] == 3 and out["completed"] == 0
