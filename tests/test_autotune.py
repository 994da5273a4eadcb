"""The autotuner's host logic on CPU: batches stream through the slots once
each, every candidate's settings reach every context, the fastest candidate
with the first candidate's results is chosen, and one whose results differ is
never chosen however fast.  Fake contexts stand in for the GPU (their time
depends on the settings they were given); the GPU run is autotune.py's main."""
from __future__ import annotations

import threading
import time

import numpy as np

import autotune
import cortrace as ct


class _FakeCtx:
    """Sites from the jobs' own fields (deterministic), a time per batch set
    by the settings, and perturbed results under the `bad` settings."""

    def __init__(self, speed, bad):
        self.speed, self.bad = speed, bad
        self.regroup, self.order = (16, 48, 256), True      # a context's own defaults
        self.calls = []
        self.lock = threading.Lock()

    def set_regroup(self, park_below, max_generations, min_park):
        self.regroup = (park_below, max_generations, min_park)

    def set_queue_order(self, rigidity_major):
        self.order = bool(rigidity_major)

    def trace_batch(self, jobs, p, models=None, want_status=False):
        key = self.regroup + (self.order,)
        time.sleep(self.speed(key))
        sites = np.zeros(len(jobs), ct.SITE_DTYPE)
        sites["r_cutoff"] = jobs["the0"] * 0.1 + jobs["fi0"] * 0.01
        if key == self.bad:
            sites["r_cutoff"][0] += 0.01
        with self.lock:
            self.calls.append(len(jobs))

        class R:
            pass
        r = R()
        r.sites = sites
        return r


def test_run_streams_every_batch_once_in_order():
    batches = autotune.sample_batches(5, 300)
    ctxs = [_FakeCtx(lambda k: 0.01, None) for _ in range(3)]
    _, out = autotune.run(ctxs, batches, None, None)
    assert sum(len(c.calls) for c in ctxs) == len(batches)
    for b, o in zip(batches, out):
        assert np.array_equal(o.sites["r_cutoff"], b["the0"] * 0.1 + b["fi0"] * 0.01)


def test_tune_picks_the_fastest_with_the_same_results():
    batches = autotune.sample_batches(4, 300)
    fastest = (8, 1, 256, True)
    bad = (16, 1, 256, True)                       # faster still, but its results differ

    def speed(key):
        return {fastest: 0.01, bad: 0.001}.get(key, 0.03)
    ctxs = [_FakeCtx(speed, bad) for _ in range(4)]
    best, results = autotune.tune(ctxs, batches, None, None, autotune.candidates())
    assert best == {"inflight": 4, "park_below": 8, "max_generations": 1, "min_park": 256, "rigidity_major": 1}
    assert len(results) == len(autotune.candidates())
    assert [r["same_results"] for r in results].count(False) == 2      # the bad settings at both inflight counts
    assert all(not r["same_results"] for r in results if (r["park_below"], r["max_generations"]) == (16, 1)
               and r["rigidity_major"] == 1)
    # the last candidate's settings reached every context
    last = autotune.candidates()[-1]
    for c in ctxs:
        assert c.regroup == (last["park_below"], last["max_generations"], last["min_park"])
        assert c.order == bool(last["rigidity_major"])


def test_committed_tuning_loads():
    t = autotune.load_tuning()
    assert t is not None and set(t) == set(autotune.KNOBS)
    assert t["inflight"] >= 1 and 0 <= t["park_below"] <= 32 and t["max_generations"] >= 1


def test_tune_stream_picks_the_fastest_with_the_same_results():
    """The stream autotuner's choice: the fastest candidate whose sites equal
    the first candidate's; a faster one with different results is never
    chosen."""
    sites = np.zeros(6, ct.SITE_DTYPE)
    sites["r_cutoff"] = np.arange(6) * 0.5
    cands = autotune.stream_candidates()
    times = {(16, 0, 1): 30.0, (16, 1, 1): 31.0, (16, 2, 1): 20.0, (4, 2, 1): 25.0, (64, 2, 1): 10.0,
             (16, 2, 0): 22.0}
    key = lambda c: (c["segments"], c["queue_order"], c["sort_lanes"])
    assert set(times) == {key(c) for c in cands}

    def run_launch(c):
        out = sites.copy()
        if key(c) == (64, 2, 1):
            out["r_cutoff"][2] += 0.01                   # fastest, but wrong
        return times[key(c)], out
    best, results = autotune.tune_stream(run_launch, cands)
    assert best == {"segments": 16, "queue_order": 2, "sort_lanes": 1}
    assert len(results) == len(cands) and sum(not r["same_results"] for r in results) == 1
