"""The persistent scan stream (cor_stream_*) against cor_trace_batch.

A stream keeps one launch of the scan kernel resident and feeds it batches as
they are submitted; every batch's flags, cutoffs, records and counters must be
those of the same batch traced alone by cor_trace_batch, bit for bit, whatever
else is in flight beside it, across kernel restarts, and through the
device-buffer submit path.  Failures are made on the host: a full ring, bad
arguments, and a kernel left without work past its idle limit (its bounded
wait ends and the stream reports COR_ERR_WATCHDOG)."""
from __future__ import annotations

import time

import numpy as np
import pytest

from conftest import golden
import cortrace as ct

pytestmark = pytest.mark.gpu

WAIT_MS = 300000


def _jobs(latlon, **kw):
    return np.concatenate([ct.make_job(float(a), float(o), **kw) for a, o in latlon])


def _same(got: ct.ScanResult, want: ct.ScanResult, records: bool = True):
    assert np.array_equal(got.sites.view(np.uint8), want.sites.view(np.uint8)), "site results differ"
    assert np.array_equal(got.status, want.status), "flags differ"
    if records:
        assert np.array_equal(got.records.view(np.uint8), want.records.view(np.uint8)), "records differ"
    for k in ("accepted_steps", "trials", "trajectories", "watchdog"):
        assert got.counters[k] == want.counters[k], k


def _batches():
    """Batches of different shapes: a uniform grid (rigidity-major order), a
    batch of windows of the grid (scan-by-scan order), one rigidity, and
    oblique arrivals."""
    uni = _jobs([(a, o) for a in (-60.0, -10.0, 35.0, 80.0) for o in (0.0, 150.0, 290.0)])
    win = _jobs([(50.0, 15.0), (-20.0, 100.0), (5.0, 250.0)])
    win["i_first"] = [10, 120, 250]
    win["i_count"] = [60, 40, 150]
    one = ct.make_job(45.0, 30.0, rig=9.0, rk=9.0, dele=0.05)
    obl = np.concatenate([ct.make_job(30.0, 60.0, rig=0.5, rk=15.0, dele=0.25, the1=38.0, fi1=70.0),
                          ct.make_job(-30.0, 200.0, rig=0.5, rk=15.0, dele=0.25, the1=-25.0, fi1=185.0)])
    return [uni, win, one, obl]


def test_stream_equals_trace_batch_igrf(ctx):
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    batches = _batches()
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), slots=4, want_records=1, idle_limit_s=30.0) as s:
        tickets = [s.submit(b, p, want_records=True) for b in batches]
        got = [s.wait(t, WAIT_MS) for t in tickets]
    for b, g in zip(batches, got):
        assert g is not None
        _same(g[0], ctx.trace_batch(b, p, want_records=True))
        assert g[0].counters["kernel_launches"] == 1


def _near(got: ct.ScanResult, want: ct.ScanResult, dele: float):
    """Two scans of the same batch by kernels whose FMA contractions may
    differ (the external-field units are compiled with contraction), held to
    the bar the scans are held to against the reference: every flag that
    differs lies inside the penumbra widened by one step, and P(S), P(C),
    P(M) agree within one step on all sites but at most one."""
    off = 0
    for j in range(len(want.sites)):
        a, b = got.sites[j], want.sites[j]
        off += any(abs(a[k] - b[k]) > dele * 1.0000001 for k in ("r_lower", "r_upper", "r_cutoff"))
        sa = got.status[got.offsets[j]:got.offsets[j + 1]] == ct.TRAJ_ALLOWED
        sb = want.status[want.offsets[j]:want.offsets[j + 1]] == ct.TRAJ_ALLOWED
        lo = min(a["r_lower"], b["r_lower"]) - dele
        hi = max(a["r_upper"], b["r_upper"]) + dele
        for i in np.nonzero(sa != sb)[0]:
            r = 0.1 + i * dele
            assert lo - 1e-9 <= r <= hi + 1e-9, (j, r)
    assert off <= 1, f"{off} sites off by more than one step"


def test_stream_t96_alone_and_in_the_mix(ctx):
    """IGRF-14 + T96 requests of different sizes and conditions: each gives
    the same result bit for bit when it is alone in the stream and when it is
    in flight with the others; against cor_trace_batch (a different kernel of
    the same unit, compiled with FMA contraction) within one rigidity step."""
    g = golden("scan_t96.json")
    t7 = g["time"]
    reqs = []
    for k, pm in enumerate(([2.0, -20.0, 0.0, -1.0], [6.5, -150.0, 8.0, -12.0], [1.2, -5.0, -3.0, 4.0])):
        sites = g["sites"][k * 5:k * 5 + 3 + 2 * k]
        reqs.append((np.concatenate([ct.make_job(s["lat"], s["lon"], rig=0.1, rk=20.0, dele=0.1) for s in sites]),
                     ct.internal_setup("igrf14", t7, parmod=pm)))
    models = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96)
    with ct.Stream(ctx, models, slots=8, idle_limit_s=30.0) as s:
        tickets = [s.submit(j, p) for j, p in reqs]
        mixed = [s.wait(t, WAIT_MS) for t in tickets]
        alone = []
        for j, p in reqs:
            alone.append(s.wait(s.submit(j, p), WAIT_MS))
            s.drain()                                 # nothing else in flight
    for (j, p), m, a in zip(reqs, mixed, alone):
        assert m is not None and a is not None
        _same(m[0], a[0], records=False)
        _near(m[0], ctx.trace_batch(j, p, models=models), 0.1)


def test_stream_restarts_keep_results(ctx):
    """A launch serves at most 2 segments and 1 submitted parameter block, so
    the stream restarts its kernel between most submits; results are
    unchanged and the parameter block of a repeated condition is reused."""
    pa = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    pb = ct.internal_setup("igrf14", [1990, 5, 5, 125, 0, 0, 0])
    jobs = _jobs([(a, 40.0) for a in (-50.0, 0.0, 50.0)], rig=1.0, rk=12.0, dele=0.25)
    order = [pa, pa, pb, pa, pb, pb]
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), slots=8, max_params=1, pool_params=1,
                   segments_per_launch=2, idle_limit_s=30.0) as s:
        tickets = [s.submit(jobs, p) for p in order]
        got = [s.wait(t, WAIT_MS) for t in tickets]
    want = {id(pa): ctx.trace_batch(jobs, pa), id(pb): ctx.trace_batch(jobs, pb)}
    for p, r in zip(order, got):
        _same(r[0], want[id(p)], records=False)


def test_stream_device_submit(ctx):
    torch = pytest.importorskip("torch")
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    jobs = _jobs([(a, o) for a in (-45.0, 15.0, 75.0) for o in (20.0, 200.0)])
    n, off = ct.batch_offsets(jobs)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), idle_limit_s=30.0) as s:
        base = s.upload_params(p)
        dj = jobs.copy()
        dj["param_index"] = base
        bj, bt, bo = dev(dj), dev(ct.prepare_trig(jobs)), dev(off)
        sites = torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        status = torch.zeros(n, dtype=torch.uint8, device="cuda")
        t = s.submit_device(bj.data_ptr(), bt.data_ptr(), bo.data_ptr(), off, len(jobs), sites.data_ptr(),
                            status.data_ptr())
        cnt, t_ns = s.wait(t, WAIT_MS)
    want = ctx.trace_batch(jobs, p)
    assert np.array_equal(sites.cpu().numpy().view(ct.SITE_DTYPE).view(np.uint8), want.sites.view(np.uint8))
    assert np.array_equal(status.cpu().numpy(), want.status)
    assert cnt["trajectories"] == n and cnt["accepted_steps"] == want.counters["accepted_steps"]
    assert t_ns > 0


def test_stream_host_side_errors(ctx):
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    jobs = ct.make_job(10.0, 10.0, rig=8.0, rk=9.0, dele=0.5)
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), slots=2, max_jobs=4, idle_limit_s=30.0) as s:
        a, b = s.submit(jobs, p), s.submit(jobs, p)
        with pytest.raises(ct.CorError) as e:
            s.submit(jobs, p)                         # both slots hold uncollected segments
        assert e.value.code == -8
        assert s.wait(a, WAIT_MS) is not None and s.wait(b, WAIT_MS) is not None
        with pytest.raises(ct.CorError) as e:
            s.wait(a, 0)                              # already collected
        assert e.value.code == -1
        bad = jobs.copy()
        bad["param_index"] = 1
        with pytest.raises(ct.CorError) as e:
            s.submit(bad, p)                          # parameter block out of range
        assert e.value.code == -1
        with pytest.raises(ct.CorError) as e:
            s.submit(np.concatenate([jobs] * 5), p)   # more scans than max_jobs
        assert e.value.code == -1
        empty = s.submit(np.zeros(0, ct.JOB_DTYPE), p)
        r, _ = s.wait(empty, WAIT_MS)
        assert len(r.sites) == 0 and r.counters["trajectories"] == 0
        # the stream still serves after the refusals
        r, _ = s.wait(s.submit(jobs, p), WAIT_MS)
    # (the plain scan only after the stream has ended: its kernel holds the SMs)
    _same(r, ctx.trace_batch(jobs, p), records=False)


def test_stream_idle_limit_ends_the_kernel(ctx):
    """The kernel's wait for work is bounded: left idle past idle_limit_s its
    blocks return, the stream reports COR_ERR_WATCHDOG, and the context stays
    usable."""
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    jobs = ct.make_job(10.0, 10.0, rig=8.0, rk=9.0, dele=0.5)
    s = ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), idle_limit_s=0.3)
    try:
        assert s.wait(s.submit(jobs, p), WAIT_MS) is not None
        time.sleep(2.0)
        with pytest.raises(ct.CorError) as e:
            s.wait(s.submit(jobs, p), WAIT_MS)
        assert e.value.code == -4
    finally:
        with pytest.raises(ct.CorError):
            s.close()
    r = ctx.trace_batch(jobs, p)
    assert r.counters["trajectories"] == 3


def test_stream_launch_on_drain(ctx):
    """Segments staged first and run by one launch that never waits on the
    host (the form a profiler can replay); cor_stream_drain times it."""
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    batches = _batches()[:3]
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), slots=4, launch_on_drain=1, idle_limit_s=30.0) as s:
        tickets = [s.submit(b, p) for b in batches]
        ms = s.drain()
        got = [s.wait(t, 0) for t in tickets]
        assert s.drain() == 0.0                       # nothing ran since
    assert ms > 0
    for b, g in zip(batches, got):
        _same(g[0], ctx.trace_batch(b, p), records=False)


def test_stream_labels_equal_batch_labels(ctx):
    """train_window.label_stream (the training labels, streamed in segments
    with one parameter block per sample) equals train_window.label through
    cor_trace_batch, sample for sample (IGRF-14 only: bit for bit)."""
    import train_window as tw
    s = tw.build_samples(np.random.default_rng(5), 7, "t96")
    models = ct.model_set(ct.INTERNAL_SH)
    ru, rl, traced = tw.label(ctx, s, models, chunk=3)
    ru2, rl2, rc2, traced2, _ = tw.label_stream(ctx, s, models, chunk=3)
    assert np.array_equal(ru, ru2) and np.array_equal(rl, rl2) and traced == traced2
    assert np.all(np.isfinite(rc2))


def test_window_scan_reacts_to_scan_events(ctx):
    """window.trace_windows_stream on a stream with per-scan events (each
    scan's result read the moment it is reduced, retraces submitted at once)
    gives the sites and widenings of window.trace_windows over
    cor_trace_batch, including windows placed wrong on purpose (edge hits)."""
    import window
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    jobs = _jobs([(a, o) for a in (-70.0, -30.0, 0.0, 30.0, 70.0) for o in (0.0, 180.0)], rig=0.01, rk=20.0,
                 dele=0.01)
    full = ctx.trace_batch(jobs, p)
    n = full.offsets[1] - full.offsets[0]
    i_lo, i_hi = np.zeros(len(jobs), np.int64), np.zeros(len(jobs), np.int64)
    for j in range(len(jobs)):
        st = full.status[full.offsets[j]:full.offsets[j + 1]]
        a = np.nonzero(st == ct.TRAJ_ALLOWED)[0]
        f = np.nonzero(st != ct.TRAJ_ALLOWED)[0]
        i_lo[j] = max(0, (a.min() if len(a) else 0) - 5)
        i_hi[j] = min(n - 1, (f.max() if len(f) else n - 1) + 5)
    i_lo[0], i_hi[0] = i_hi[0] + 10, min(n - 1, i_hi[0] + 40)     # above the penumbra: first rigidity allowed
    i_lo[1], i_hi[1] = max(0, i_lo[1] - 60), max(0, i_lo[1] - 20)  # below it: last rigidity forbidden
    want_sites, want_redone, _, _ = window.trace_windows(ctx, jobs, p, ct.model_set(ct.INTERNAL_SH), i_lo, i_hi)
    with ct.Stream(ctx, ct.model_set(ct.INTERNAL_SH), slots=4, scan_events=1, idle_limit_s=30.0) as s:
        (sites, redone, traced, _), = window.trace_windows_stream(s, [(jobs, p, i_lo, i_hi)])
    assert np.array_equal(sites.view(np.uint8), want_sites.view(np.uint8))
    assert np.array_equal(redone, want_redone) and redone[0] and redone[1]


@pytest.mark.parametrize("order", [0, 1, 2])
def test_stream_queue_orders_give_the_same_results(ctx, order):
    """Scan by scan, rigidity-major, and warp-wide chunks in ascending
    rigidity (uniform grids and windows alike) move time only: every result
    equals cor_trace_batch's bit for bit (IGRF-14)."""
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    batches = _batches()
    c2 = ct.Context(0)
    try:
        c2.set_queue_order(order)
        with ct.Stream(c2, ct.model_set(ct.INTERNAL_SH), slots=4, idle_limit_s=30.0) as s:
            got = [s.wait(s.submit(b, p), WAIT_MS) for b in batches]
    finally:
        c2.close()
    for b, g in zip(batches, got):
        _same(g[0], ctx.trace_batch(b, p), records=False)


@pytest.mark.parametrize("external", [ct.EXTERNAL_NONE, ct.EXTERNAL_T96])
def test_lane_regrouping_moves_time_only(ctx, external):
    """Regrouping a block's trajectories by field band before every field
    evaluation (sort_lanes, the default) moves trajectories between threads
    but not their arithmetic: flags, cutoffs, final records and counters equal
    the unsorted run's bit for bit, through the stream and through
    cor_trace_batch (IGRF-14 alone, and with T96, whose key also evaluates
    the Region-2 band)."""
    if external == ct.EXTERNAL_T96:
        g = golden("scan_t96.json")
        p = ct.internal_setup("igrf14", g["time"], parmod=[6.5, -150.0, 8.0, -12.0])
        batches = [_jobs([(s["lat"], s["lon"]) for s in g["sites"][:12]], rig=0.1, rk=20.0, dele=0.1)]
    else:
        p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
        batches = _batches()
    models = ct.model_set(ct.INTERNAL_SH, external)
    out = {}
    for sort in (0, 1):
        with ct.Stream(ctx, models, slots=4, want_records=1, sort_lanes=sort, idle_limit_s=120.0) as s:
            tickets = [s.submit(b, p, want_records=True) for b in batches]
            out[sort] = [s.wait(t, WAIT_MS) for t in tickets]
    for a, b in zip(out[0], out[1]):
        assert a is not None and b is not None
        _same(b[0], a[0])
    # the batch kernel (cor_trace_batch, its generations and parking) likewise
    batch = {}
    for sort in (0, 1):
        c = ct.Context(0)
        try:
            c.set_lane_sort(bool(sort))
            batch[sort] = [c.trace_batch(b, p, models=models, want_records=True) for b in batches]
        finally:
            c.close()
    for a, b in zip(batch[0], batch[1]):
        _same(b, a)
