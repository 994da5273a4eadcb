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


def _run_logged(reqs, log_path, durable=False):
    ref = [None]
    log = serve.RequestLog(str(log_path), durable=durable)
    srv = serve.Server(slots=2, executor=_Oracle(ref), log=log)
    ref[0] = srv
    out = serve.run_stream(srv, reqs)
    log.close()
    return out


def test_request_log_resumes_a_stopped_server(tmp_path):
    """A log cut as if the server had stopped: requests 0-5 queued, the even
    ones finished, a torn "done" line at the end, requests 6-7 never seen.
    Resuming restores the finished results, runs the rest, and every result
    equals the uninterrupted run's bit for bit."""
    import json
    reqs = _small(serve.poisson_stream(13, 500.0, 8, max_box_sites=4))
    full = tmp_path / "full.jsonl"
    out = _run_logged(reqs, full)
    assert out["completed"] == 8
    done, pending = serve.RequestLog.replay(str(full))
    assert sorted(done) == list(range(8)) and pending == []
    for r in reqs:
        assert np.array_equal(done[r.rid][0].view(np.uint8), r.result.view(np.uint8))

    keep, torn = [], None
    for line in full.read_text().splitlines():
        rec = json.loads(line)
        rid = rec["request"]["rid"] if rec["event"] == "submit" else rec["rid"]
        if rid >= 6:
            continue
        if rec["event"] == "done" and rid % 2:
            torn = torn or line[:len(line) // 2]
            continue
        keep.append(line)
    stopped = tmp_path / "stopped.jsonl"
    stopped.write_text("\n".join(keep) + "\n" + torn)

    fresh = _small(serve.poisson_stream(13, 500.0, 8, max_box_sites=4))
    restored, todo = serve.resume(str(stopped), fresh)
    assert sorted(r.rid for r in restored) == [0, 2, 4]
    assert [r.rid for r in todo][:3] == [1, 3, 5] and all(r.arrival == 0.0 for r in todo[:3])
    assert sorted(r.rid for r in todo[3:]) == [6, 7] and min(r.arrival for r in todo[3:]) == 0.0
    out2 = _run_logged(todo, stopped, durable=True)
    assert out2["completed"] == 5
    by_rid = {r.rid: r for r in restored + todo}
    for r in reqs:
        assert np.array_equal(by_rid[r.rid].result.view(np.uint8), r.result.view(np.uint8)), r.rid
    done2, pending2 = serve.RequestLog.replay(str(stopped))
    assert sorted(done2) == list(range(8)) and pending2 == []


def test_rejected_requests_are_not_owed_after_a_stop(tmp_path):
    reqs = _small(serve.poisson_stream(11, 100.0, 3, max_box_sites=4))
    log = tmp_path / "log.jsonl"
    ref = [None]
    srv = serve.Server(slots=1, hbm_budget=min(r.device_bytes() for r in reqs) - 1, executor=_Oracle(ref),
                       log=serve.RequestLog(str(log)))
    ref[0] = srv
    out = serve.run_stream(srv, reqs)
    srv.log.close()
    assert out["rejected"] == 3
    done, pending = serve.RequestLog.replay(str(log))
    assert done == {} and pending == []


def test_windows_only_for_the_trained_field_model():
    """A window network trained with T96 is used for T96 requests only; TS05
    requests in the same stream get the full scan (their executor call has no
    features)."""
    import window
    assert window.trained_external('{"model": "igrf14+t96"}') == ct.EXTERNAL_T96
    assert window.trained_external('{"model": "igrf14+ts05"}') == ct.EXTERNAL_TS05
    assert window.trained_external("not json") is None

    class _Model:
        external = ct.EXTERNAL_T96
    seen = []

    def executor(ctx, jobs, params, models, feats):
        seen.append((models.external_model, feats is not None))
        res = pyoracle.scan_batch(jobs, params, models=models, threads=2)
        return res.sites, np.zeros(len(jobs), bool)
    reqs = _small(serve.poisson_stream(17, 500.0, 6, max_box_sites=4))
    for k, r in enumerate(reqs):
        r.external = ct.EXTERNAL_T96 if k % 2 else ct.EXTERNAL_TS05
        if r.external == ct.EXTERNAL_TS05:
            r.parmod = list(r.parmod[:4]) + [1.0] * 6
    srv = serve.Server(slots=1, executor=executor, window_model=_Model())
    out = serve.run_stream(srv, reqs)
    assert out["completed"] == 6
    assert all(used == (ext == ct.EXTERNAL_T96) for ext, used in seen)
    assert {ext for ext, _ in seen} == {ct.EXTERNAL_T96, ct.EXTERNAL_TS05}


def test_one_window_network_per_field_model():
    """With a T96 and a TS05 network, both kinds of request are windowed."""
    class _M:
        def __init__(self, ext):
            self.external = ext
    seen = []

    def executor(ctx, jobs, params, models, feats):
        seen.append((models.external_model, feats is not None))
        res = pyoracle.scan_batch(jobs, params, models=models, threads=2)
        return res.sites, np.zeros(len(jobs), bool)
    reqs = _small(serve.poisson_stream(19, 500.0, 4, max_box_sites=4))
    for k, r in enumerate(reqs):
        r.external = ct.EXTERNAL_T96 if k % 2 else ct.EXTERNAL_TS05
    srv = serve.Server(slots=1, executor=executor, window_model=[_M(ct.EXTERNAL_T96), _M(ct.EXTERNAL_TS05)])
    assert serve.run_stream(srv, reqs)["completed"] == 4
    assert {ext for ext, _ in seen} == {ct.EXTERNAL_T96, ct.EXTERNAL_TS05} and all(used for _, used in seen)


def test_admission_waits_for_free_device_memory():
    """The device reports too little free memory for the first polls: no
    request is admitted (the executor is not called) until it reports
    enough; then every request completes."""
    reqs = _small(serve.poisson_stream(23, 1000.0, 4, max_box_sites=4))
    polls = {"n": 0}

    def free():
        polls["n"] += 1
        return 0 if polls["n"] < 40 else 10 ** 12

    calls = []

    def executor(ctx, jobs, params, models, feats):
        calls.append(polls["n"])
        res = pyoracle.scan_batch(jobs, params, models=models, threads=2)
        return res.sites, np.zeros(len(jobs), bool)
    srv = serve.Server(slots=2, executor=executor, free_memory=free, reserve_bytes=1e9)
    out = serve.run_stream(srv, reqs)
    assert out["completed"] == 4
    assert srv.admission.waits > 0
    assert calls and min(calls) >= 40


def test_admission_rule():
    adm = serve.Admission(1000, free_memory=lambda: 700, reserve_bytes=200)
    assert adm.fits(0, 500) and not adm.fits(0, 501)          # free less the reserve
    assert not adm.fits(600, 500) and adm.fits(500, 500)      # the budget over the requests in flight
    assert serve.Admission(1000).fits(999, 1) and not serve.Admission(1000).fits(999, 2)


def test_window_state_widens_then_takes_the_whole_grid():
    """The per-request window state of the stream server follows
    window.trace_windows: an edge hit widens that side, and after the
    widenings the whole grid is scanned."""
    import window
    jobs = ct.make_job(10.0, 20.0, rig=0.01, rk=20.0, dele=0.01)
    st = serve._WindowState(jobs, [100], [120], widen=1)
    j1 = st.next_jobs()
    assert int(j1["i_first"][0]) == 100 and int(j1["i_count"][0]) == 21
    n = 21
    res = ct.ScanResult(np.zeros(1, ct.SITE_DTYPE), np.full(n, ct.TRAJ_ALLOWED, np.uint8), None,
                        np.array([0, n], np.uint64), {})
    assert st.absorb(res)                                   # first allowed: widen downwards
    j2 = st.next_jobs()
    assert int(j2["i_first"][0]) == 79
    assert st.absorb(ct.ScanResult(np.zeros(1, ct.SITE_DTYPE), np.full(42, ct.TRAJ_ALLOWED, np.uint8), None,
                                   np.array([0, 42], np.uint64), {}))
    j3 = st.next_jobs()                                     # after `widen` widenings: the whole grid
    assert int(j3["i_first"][0]) == 0 and int(j3["i_count"][0]) == window.GRID_N
