"""Serving loop for cutoff-map requests (no counterpart in the reference).

A request is one site or a latitude/longitude grid box, one geomagnetic
condition, vertical incidence or 9 directions (vertical plus 30 deg zenith at
8 azimuths), scanned on the 0.01 GV grid.  Requests arrive as a seeded
Poisson stream.  Two servers share one interface:
* StreamServer (the default): persistent scan streams (cor_stream_*), one per
  field model; every admitted request goes into its model's stream at once as
  a segment, so requests that arrive while others run share the lanes of the
  one resident kernel at trajectory granularity (continuous batching);
* Server: several slots, each a context with its own CUDA stream; whenever a
  slot is free it takes every admitted request that is waiting, up to a
  per-batch trajectory cap, and traces them in one call while the other
  slots' batches run.
A request is admitted when its device memory (jobs, start vectors, offsets,
classes, results, parameter block) fits in what the HBM budget has left after
the requests in flight, and in the device's free memory less a reserve.  With a window model, each site-direction
of a request with the field model the network was trained with is first
scanned over its predicted window and falls back to the full scan on an edge
hit; requests with another field model get the full scan.  Each request's latency runs from its arrival to the end of
the batch that completed it; results are per site-direction P(S), P(C), P(M),
identical whether a request ran alone or in a mix (trajectories are
independent and deterministic).

With a request log (RequestLog) every queued, rejected and completed request
is on disk, and a stopped server resumes from it without losing work (only
the batches in flight at the stop run again).

    python cor-model_gb300/serve.py --rate 2 --requests 40 [--window FILE ...] [--log FILE [--resume]]
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import autotune  # noqa: E402
import cortrace as ct  # noqa: E402
import window  # noqa: E402

DIRECTIONS_9 = [(0.0, 0.0)] + [(30.0, 45.0 * k) for k in range(8)]
R0 = 1.0031391260673028


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float                 # seconds after the stream's start
    sites: list                    # [(lat, lon)]
    directions: list               # [(zenith, azimuth)]
    time7: list
    parmod: list
    external: int = ct.EXTERNAL_TS05
    rig: tuple = (0.01, 20.0, 0.01)
    # filled by the server
    done_at: float = -1.0
    result: np.ndarray | None = None   # SITE_DTYPE per site-direction
    fallback: int = 0

    @property
    def n_scans(self) -> int:
        return len(self.sites) * len(self.directions)

    @property
    def n_rig(self) -> int:
        r, rk, d = self.rig
        return int(round((rk - r) / d)) + 1

    def device_bytes(self) -> int:
        n = self.n_scans
        traj = n * self.n_rig
        return n * (ct.JOB_DTYPE.itemsize + ct.TRIG_DTYPE.itemsize + ct.SITE_DTYPE.itemsize + 8) + traj + \
            ct.PARAMS_DTYPE.itemsize + 4096


def poisson_stream(seed: int, rate: float, n: int, external=ct.EXTERNAL_TS05, max_box_sites: int = 64) -> list:
    """n requests with exponential inter-arrival times of mean 1/rate: half
    single sites, half grid boxes of 2-10 deg spacing (at most max_box_sites
    sites); vertical incidence or the 9 directions; storm-range conditions."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for k in range(n):
        t += rng.exponential(1.0 / rate)
        if rng.uniform() < 0.5:
            sites = [(float(np.degrees(np.arcsin(rng.uniform(-1, 1)))), float(rng.uniform(0, 360)))]
        else:
            sp = float(rng.integers(2, 11))
            side = int(max(1, np.floor(np.sqrt(max_box_sites))))
            nlat, nlon = int(rng.integers(1, side + 1)), int(rng.integers(1, side + 1))
            lat0 = float(rng.uniform(-88, 88 - sp * (nlat - 1))) if sp * (nlat - 1) < 176 else -88.0
            lon0 = float(rng.uniform(0, 360))
            sites = [(min(88.0, lat0 + sp * i), (lon0 + sp * j) % 360.0) for i in range(nlat) for j in range(nlon)]
        dirs = [(0.0, 0.0)] if rng.uniform() < 0.5 else DIRECTIONS_9
        cond = window.sample_conditions(rng, 1, "ts05" if external == ct.EXTERNAL_TS05 else "t96")[0]
        out.append(Request(k, t, sites, dirs, cond["time7"], cond["parmod"], external))
    return out


def request_jobs(req: Request, param_index: int) -> np.ndarray:
    r, rk, d = req.rig
    jobs = []
    for lat, lon in req.sites:
        for zen, az in req.directions:
            the1, fi1 = window.arrival_direction(lat, lon, zen, az)
            jobs.append(ct.make_job(lat, lon, rig=r, rk=rk, dele=d, r0=R0, the1=the1, fi1=fi1,
                                    param_index=param_index))
    return np.concatenate(jobs)


_REQ_FIELDS = ("rid", "arrival", "sites", "directions", "time7", "parmod", "external", "rig")
_SITE_FLOATS = ("r_lower", "r_upper", "r_cutoff")
_SITE_INTS = ("n_forbidden", "n_traj")


def request_to_json(r: Request) -> dict:
    return {k: getattr(r, k) for k in _REQ_FIELDS}


def request_from_json(d: dict) -> Request:
    return Request(d["rid"], d["arrival"], [tuple(s) for s in d["sites"]], [tuple(s) for s in d["directions"]],
                   list(d["time7"]), list(d["parmod"]), d["external"], tuple(d["rig"]))


def result_to_json(sites: np.ndarray) -> dict:
    """Per site-direction results, floats as exact hex."""
    out = {k: [float(v).hex() for v in sites[k]] for k in _SITE_FLOATS}
    return out | {k: [int(v) for v in sites[k]] for k in _SITE_INTS}


def result_from_json(d: dict) -> np.ndarray:
    n = len(d["r_lower"])
    sites = np.zeros(n, ct.SITE_DTYPE)
    for k in _SITE_FLOATS:
        sites[k] = [float.fromhex(v) for v in d[k]]
    for k in _SITE_INTS:
        sites[k] = d[k]
    return sites


class RequestLog:
    """Append-only JSON-lines log of a server's requests, so that a server
    that stopped (crash, restart, preemption) can be resumed without losing
    work, re-running at most the batches that were in flight when it stopped
    (their results are deterministic, so a re-run gives the same bytes).  One
    "submit" line when a request is queued, one
    "rejected" line when it is over the budget, one "done" line with its
    result when the batch that held it completes.  Each line is written
    whole, flushed and (durable=True) fsync'ed before the server moves on, so
    the log never says more than happened; a torn last line, the mark of a
    write cut off by the stop, is ignored by replay()."""

    def __init__(self, path: str, durable: bool = True):
        self.path = path
        self.durable = durable
        self.lock = threading.Lock()
        torn = False
        if os.path.exists(path) and os.path.getsize(path) > 0:
            with open(path, "rb") as f:
                f.seek(-1, os.SEEK_END)
                torn = f.read(1) != b"\n"
        self.f = open(path, "a", encoding="utf-8")
        if torn:
            self.f.write("\n")        # end the torn line so the next record starts clean

    def _write(self, recs: list[dict]):
        with self.lock:
            self.f.write("".join(json.dumps(r, separators=(",", ":")) + "\n" for r in recs))
            self.f.flush()
            if self.durable:
                os.fsync(self.f.fileno())

    def submitted(self, req: Request):
        self._write([{"event": "submit", "request": request_to_json(req)}])

    def rejected(self, req: Request):
        self._write([{"event": "rejected", "rid": req.rid}])

    def completed(self, reqs: list[Request]):
        self._write([{"event": "done", "rid": r.rid, "fallback": r.fallback, "result": result_to_json(r.result)}
                     for r in reqs])

    def close(self):
        with self.lock:
            self.f.close()

    @staticmethod
    def replay(path: str) -> tuple[dict, list[Request]]:
        """-> ({rid: (result, fallback)} of the completed requests, the
        requests submitted but neither completed nor rejected, in arrival
        order).  Lines that do not parse (a torn write) are skipped."""
        submitted, done, rejected = {}, {}, set()
        if not os.path.exists(path):
            return done, []
        with open(path, encoding="utf-8") as f:
            for line in f:
                try:
                    rec = json.loads(line)
                    ev = rec["event"]
                    if ev == "submit":
                        req = request_from_json(rec["request"])
                        submitted[req.rid] = req
                    elif ev == "done":
                        done[rec["rid"]] = (result_from_json(rec["result"]), rec["fallback"])
                    elif ev == "rejected":
                        rejected.add(rec["rid"])
                except (ValueError, KeyError, TypeError):
                    continue
        pending = [r for rid, r in submitted.items() if rid not in done and rid not in rejected]
        return done, sorted(pending, key=lambda r: r.arrival)


def request_features(req: Request, params: np.ndarray) -> np.ndarray:
    tilt = window.dipole_tilt(params)
    ep = window.decimal_epoch(req.time7)
    return np.array([window.features(lat, lon, zen, az, ep, req.parmod, tilt)
                     for lat, lon in req.sites for zen, az in req.directions])


class Server:
    """Continuous batching over `slots` contexts under an HBM budget."""

    def __init__(self, device: int = 0, slots: int = 3, hbm_budget: float = 40e9, max_batch_traj: int = 2_000_000,
                 window_model=None, executor=None, log: RequestLog | None = None, free_memory=None,
                 reserve_bytes: float = 2e9):
        self.budget = int(hbm_budget)
        self.admission = Admission(self.budget, free_memory, reserve_bytes)
        self.log = log
        self.in_flight = 0
        self.max_batch_traj = max_batch_traj
        # one window network per external field model (WindowModel.external):
        # a single network or several
        models = window_model if isinstance(window_model, (list, tuple)) else [window_model]
        self.window_models = {getattr(m, "external", None): m for m in models if m is not None}
        self.lock = threading.Condition()
        self.waiting: list[Request] = []
        self.closed = False
        self.t0 = None
        self.batches = 0
        self.rejected: list[Request] = []
        if executor is None:
            self.ctxs = [ct.Context(device) for _ in range(slots)]
            tune = autotune.load_tuning()
            if tune:
                for c in self.ctxs:
                    c.set_regroup(tune["park_below"], tune["max_generations"], tune["min_park"])
                    c.set_queue_order(bool(tune["rigidity_major"]))
            self.executor = self._gpu_execute
        else:
            self.ctxs = [None] * slots
            self.executor = executor
        self.threads = [threading.Thread(target=self._slot_loop, args=(c,), daemon=True) for c in self.ctxs]

    # -- the GPU path: one call per batch, windows first when a model is loaded
    def _gpu_execute(self, ctx, jobs, params, models, feats):
        wm = self.window_models.get(models.external_model)
        if wm is None or feats is None:
            res = ctx.trace_batch(jobs, params, models=models, want_status=False)
            return res.sites, np.zeros(len(jobs), bool)
        i_lo, i_hi = wm.windows(feats)
        sites, fb, _, _ = window.trace_windows(ctx, jobs, params, models, i_lo, i_hi)
        return sites, fb

    def start(self):
        self.t0 = time.perf_counter()
        for t in self.threads:
            t.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        if req.device_bytes() > self.budget:
            req.done_at = self.now()
            if self.log:
                self.log.rejected(req)
            with self.lock:
                self.rejected.append(req)
            return
        if self.log:
            self.log.submitted(req)       # logged before any slot can take it
        with self.lock:
            self.waiting.append(req)
            self.lock.notify_all()

    def close(self):
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        for t in self.threads:
            t.join()
        for c in self.ctxs:
            if c is not None:
                c.close()

    def _take(self) -> list[Request] | None:
        with self.lock:
            while True:
                batch, traj, mem = [], 0, 0
                for r in list(self.waiting):
                    b = r.device_bytes()
                    n = r.n_scans * r.n_rig
                    if not self.admission.fits(self.in_flight + mem, b):
                        break                      # admission: wait for memory to free up
                    if batch and traj + n > self.max_batch_traj:
                        break
                    batch.append(r)
                    traj += n
                    mem += b
                if batch:
                    for r in batch:
                        self.waiting.remove(r)
                    self.in_flight += mem
                    return batch
                if self.closed and not self.waiting:
                    return None
                self.lock.wait(0.05)

    def _slot_loop(self, ctx):
        while True:
            batch = self._take()
            if batch is None:
                return
            by_ext = {}
            for r in batch:
                by_ext.setdefault(r.external, []).append(r)
            for ext, reqs in by_ext.items():
                params = np.concatenate([ct.internal_setup("igrf14", r.time7, parmod=r.parmod) for r in reqs])
                jobs = np.concatenate([request_jobs(r, k) for k, r in enumerate(reqs)])
                feats = None
                # windows only for requests of the field model the network was trained with
                if ext in self.window_models:
                    feats = np.concatenate([request_features(r, params[k:k + 1]) for k, r in enumerate(reqs)])
                sites, fb = self.executor(ctx, jobs, params, ct.model_set(ct.INTERNAL_SH, ext), feats)
                o = 0
                t = self.now()
                for r in reqs:
                    r.result = sites[o:o + r.n_scans].copy()
                    r.fallback = int(fb[o:o + r.n_scans].sum())
                    r.done_at = t
                    o += r.n_scans
                if self.log:
                    self.log.completed(reqs)
            with self.lock:
                self.in_flight -= sum(r.device_bytes() for r in batch)
                self.batches += 1
                self.lock.notify_all()


def device_free_bytes(device: int = 0):
    """The device's free memory now (cudaMemGetInfo through torch)."""
    import torch
    return lambda: torch.cuda.mem_get_info(device)[0]


class Admission:
    """Admits a request of b bytes when the bytes of the requests in flight
    plus b stay within the HBM budget AND b fits in the device's free memory
    less a reserve (free_memory: a callable giving the free bytes now, or
    None to skip that check)."""

    def __init__(self, budget: int, free_memory=None, reserve_bytes: float = 2e9):
        self.budget = int(budget)
        self.free_memory = free_memory
        self.reserve = int(reserve_bytes)
        self.waits = 0           # times a request was held back

    def fits(self, in_flight: int, b: int) -> bool:
        ok = in_flight + b <= self.budget and (self.free_memory is None or b <= self.free_memory() - self.reserve)
        self.waits += not ok
        return ok


class _WindowState:
    """One request's learned-window scan (the rule of window.trace_windows):
    windows first, edge hits widened and traced again, then the whole grid."""

    def __init__(self, jobs, i_lo, i_hi, widen: int = 3):
        self.jobs = jobs
        self.n_grid = np.round((jobs["rk"] - jobs["rig"]) / jobs["del"]).astype(np.int64) + 1
        self.lo = np.asarray(i_lo, np.int64).copy()
        self.hi = np.asarray(i_hi, np.int64).copy()
        self.sites = np.zeros(len(jobs), ct.SITE_DTYPE)
        self.redone = np.zeros(len(jobs), bool)
        self.todo = np.arange(len(jobs))
        self.attempt = 0
        self.widen = widen

    def next_jobs(self):
        if self.attempt == self.widen + 1:
            self.lo[self.todo] = 0
            self.hi[self.todo] = self.n_grid[self.todo] - 1
        return window.window_jobs(self.jobs[self.todo], self.lo[self.todo], self.hi[self.todo])

    def absorb(self, res) -> bool:
        """Takes a pass's result; returns whether another pass is needed."""
        again = []
        for m, j in enumerate(self.todo):
            st = res.status[res.offsets[m]:res.offsets[m + 1]]
            allowed = st == ct.TRAJ_ALLOWED
            low = self.lo[j] > 0 and allowed[0]
            high = self.hi[j] < self.n_grid[j] - 1 and not allowed[-1]
            if not (low or high):
                self.sites[j] = res.sites[m]
                continue
            width = self.hi[j] - self.lo[j] + 1
            if low:
                self.lo[j] = max(0, self.lo[j] - width)
            if high:
                self.hi[j] = min(self.n_grid[j] - 1, self.hi[j] + width)
            again.append(j)
        self.redone[again] = True
        self.todo = np.array(again, np.int64)
        self.attempt += 1
        return len(again) > 0


class StreamServer:
    """Serving on persistent scan streams (cor_stream_*): one stream per field
    model, the SMs split between them with `reserve_sms` left for the window
    network.  Every admitted request goes in at once as a segment of its
    model's stream (window passes as further segments), so requests that
    arrive while others are on the GPU share the device's lanes with them at
    trajectory granularity: a lane that finishes a trajectory of one request
    takes the next trajectory of whichever request is next in the queue.
    Admission: the HBM budget over the requests in flight and the device's
    free memory (Admission).  Same interface as Server."""

    def __init__(self, device: int = 0, hbm_budget: float = 40e9, window_model=None, log: RequestLog | None = None,
                 externals=(ct.EXTERNAL_TS05,), free_memory="device", reserve_bytes: float = 2e9,
                 stream_slots: int = 32, max_segment_traj: int = 1_200_000, reserve_sms: int = 2,
                 idle_drain_s: float = 1.0):
        import torch
        self.budget = int(hbm_budget)
        if free_memory == "device":
            free_memory = device_free_bytes(device)
        self.admission = Admission(self.budget, free_memory, reserve_bytes)
        self.log = log
        models = window_model if isinstance(window_model, (list, tuple)) else [window_model]
        self.window_models = {getattr(m, "external", None): m for m in models if m is not None}
        self.lock = threading.Condition()
        self.waiting: list[Request] = []
        self.rejected: list[Request] = []
        self.closed = False
        self.in_flight = 0
        self.batches = 0
        self.t0 = None
        self.idle_drain_s = idle_drain_s
        self.ctx = ct.Context(device)
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        share = max(1, (sms - reserve_sms) // max(1, len(externals)))
        self.streams = {ext: ct.Stream(self.ctx, ct.model_set(ct.INTERNAL_SH, ext), slots=stream_slots,
                                       max_jobs=max_segment_traj // 100, max_trajectories=max_segment_traj,
                                       max_params=1, pool_params=4096, reserve_sms=sms - share, idle_limit_s=600.0)
                        for ext in externals}
        self.max_segment_traj = max_segment_traj
        self.thread = threading.Thread(target=self._loop, daemon=True)
        self.error = None

    def start(self):
        self.t0 = time.perf_counter()
        self.thread.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, req: Request):
        if req.device_bytes() > self.budget or req.external not in self.streams:
            req.done_at = self.now()
            if self.log:
                self.log.rejected(req)
            with self.lock:
                self.rejected.append(req)
            return
        if self.log:
            self.log.submitted(req)
        with self.lock:
            self.waiting.append(req)
            self.lock.notify_all()

    def close(self):
        with self.lock:
            self.closed = True
            self.lock.notify_all()
        self.thread.join()
        for st in self.streams.values():
            st.close()
        self.ctx.close()
        if self.error:
            raise self.error

    # -- the dispatcher: admit, submit segments, collect finished ones
    def _start(self, r: Request, pending: list):
        params = ct.internal_setup("igrf14", r.time7, parmod=r.parmod)
        jobs = request_jobs(r, 0)
        wm = self.window_models.get(r.external)
        state = None
        if wm is not None:
            i_lo, i_hi = wm.windows(request_features(r, params))   # on the SMs the streams leave free
            state = _WindowState(jobs, i_lo, i_hi)
            pending.append((r, params, state, state.next_jobs()))
        else:
            # whole scans, split so that no segment exceeds the stream's size
            per = max(1, self.max_segment_traj // r.n_rig)
            r._parts = [None] * ((len(jobs) + per - 1) // per)
            for k in range(0, len(jobs), per):
                pending.append((r, params, ("part", k // per), jobs[k:k + per]))
        r._state = state

    def _loop(self):
        from collections import deque
        pending = deque()        # (request, params, state or ("part", k), jobs) waiting for a ring slot
        inflight = {ext: deque() for ext in self.streams}   # (ticket, request, params, state)
        last_busy = time.perf_counter()
        try:
            while True:
                admitted = []
                with self.lock:
                    for r in list(self.waiting):
                        b = r.device_bytes()
                        if not self.admission.fits(self.in_flight, b):
                            break
                        self.waiting.remove(r)
                        self.in_flight += b
                        admitted.append(r)
                    done_all = self.closed and not self.waiting and not admitted and not pending and \
                        not any(inflight.values())
                if done_all:
                    return
                for r in admitted:
                    r._open = 0
                    self._start(r, pending)
                progressed = bool(admitted)
                for _ in range(len(pending)):
                    r, params, state, jobs = pending[0]
                    st = self.streams[r.external]
                    if len(inflight[r.external]) >= st.config.slots:
                        pending.rotate(-1)
                        continue
                    try:
                        t = st.submit(jobs, params)
                    except ct.CorError as e:
                        if e.code != ct.ERR_BUSY:
                            raise
                        pending.rotate(-1)       # the ring slot it needs is still held: later
                        continue
                    pending.popleft()
                    inflight[r.external].append((t, r, params, state))
                    r._open += 1
                    progressed = True
                for ext, q in inflight.items():
                    st = self.streams[ext]
                    for _ in range(len(q)):
                        t, r, params, state = q[0]
                        got = st.wait(t, 0)
                        if got is None:
                            q.rotate(-1)
                            continue
                        q.popleft()
                        progressed = True
                        r._open -= 1
                        res = got[0]
                        if isinstance(state, _WindowState):
                            if state.absorb(res):
                                pending.append((r, params, state, state.next_jobs()))
                                continue
                            r.result, r.fallback = state.sites, int(state.redone.sum())
                        else:
                            r._parts[state[1]] = res.sites
                            if r._open or any(p is None for p in r._parts):
                                continue
                            r.result, r.fallback = np.concatenate(r._parts), 0
                        if r._open:
                            continue
                        r.done_at = self.now()
                        if self.log:
                            self.log.completed([r])
                        with self.lock:
                            self.in_flight -= r.device_bytes()
                            self.batches += 1
                            self.lock.notify_all()
                if progressed:
                    last_busy = time.perf_counter()
                elif not pending and not any(inflight.values()):
                    if time.perf_counter() - last_busy > self.idle_drain_s:
                        for st in self.streams.values():
                            st.drain()                    # nothing in flight: let the kernels end
                        last_busy = time.perf_counter()
                    with self.lock:
                        self.lock.wait(0.005)
                else:
                    time.sleep(0.0005)
        except Exception as e:  # noqa: BLE001
            self.error = e


def run_stream(server: Server, reqs: list[Request]) -> dict:
    """Feeds the requests at their arrival times and waits for all of them."""
    server.start()
    for r in reqs:
        delay = r.arrival - server.now()
        if delay > 0:
            time.sleep(delay)
        server.submit(r)
    server.close()
    wall = max([r.done_at for r in reqs] + [server.now()])
    lat = np.array([r.done_at - r.arrival for r in reqs if r.result is not None])
    scans = sum(r.n_scans for r in reqs if r.result is not None)
    return {"requests": len(reqs), "completed": int(len(lat)), "rejected": len(server.rejected),
            "batches": server.batches, "site_cutoffs": scans, "wall_s": wall,
            "site_cutoffs_per_s": scans / wall if wall > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "fallbacks": int(sum(r.fallback for r in reqs))}


def resume(log_path: str, reqs: list[Request]) -> tuple[list[Request], list[Request]]:
    """Splits a stream against the log of an earlier run of it -> (restored,
    to_run).  Requests whose results the log holds get them back and are not
    run again.  The rest are to run: first those the log shows queued but
    unfinished (arrival 0: they are overdue), then those it never saw, their
    arrivals shifted so that the first of them arrives at 0."""
    done, pending = RequestLog.replay(log_path)
    restored = []
    for r in reqs:
        if r.rid in done:
            r.result, r.fallback = done[r.rid]
            r.done_at = r.arrival
            restored.append(r)
    seen = set(done) | {r.rid for r in pending}
    for r in pending:
        r.arrival = 0.0
    fresh = [r for r in reqs if r.rid not in seen]
    t0 = min((r.arrival for r in fresh), default=0.0)
    for r in fresh:
        r.arrival -= t0
    return restored, pending + fresh


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rate", type=float, default=1.0, help="requests per second")
    ap.add_argument("--sweep", default=None,
                    help="comma-separated rates: run the same seeded stream at each (one JSON line per rate)")
    ap.add_argument("--requests", type=int, default=20)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--server", default="stream", choices=["stream", "slots"],
                    help="stream: every request a segment of a persistent scan stream; slots: per-call batches "
                         "over --slots contexts")
    ap.add_argument("--slots", type=int, default=3)
    ap.add_argument("--budget-gb", type=float, default=40.0)
    ap.add_argument("--external", default="ts05", choices=["t96", "ts05"])
    ap.add_argument("--window", action="append", default=[],
                    help="trained window model (train_window.py output); repeat for one per field model")
    ap.add_argument("--max-box-sites", type=int, default=16)
    ap.add_argument("--log", default=None, help="request log (JSON lines) to append to")
    ap.add_argument("--resume", action="store_true",
                    help="with --log: take the results the log holds and run only what it shows unfinished")
    args = ap.parse_args()
    if args.sweep:
        rates = [float(v) for v in args.sweep.split(",")]
        for rate in rates:
            args.rate = rate
            serve_once(args)
        return
    serve_once(args)


def serve_once(args):
    ext = ct.EXTERNAL_TS05 if args.external == "ts05" else ct.EXTERNAL_T96
    reqs = poisson_stream(args.seed, args.rate, args.requests, ext, args.max_box_sites)
    restored = []
    if args.resume:
        if not args.log:
            raise SystemExit("--resume needs --log")
        restored, reqs = resume(args.log, reqs)
    wms = [window.WindowModel(f) for f in args.window]
    log = RequestLog(args.log) if args.log else None
    if args.server == "stream":
        srv = StreamServer(0, args.budget_gb * 1e9, window_model=wms, log=log, externals=(ext,))
    else:
        srv = Server(0, args.slots, args.budget_gb * 1e9, window_model=wms, log=log,
                     free_memory=device_free_bytes(0))
    out = run_stream(srv, reqs)
    out.update({"rate": args.rate, "seed": args.seed, "server": args.server, "external": args.external,
                "window": [os.path.basename(f) for f in args.window], "restored_from_log": len(restored),
                "admission_waits": srv.admission.waits})
    if args.server == "slots":
        out["slots"] = args.slots
    print(json.dumps(out), flush=True)
    if log:
        log.close()
    for wm in wms:
        wm.close()


if __name__ == "__main__":
    main()
