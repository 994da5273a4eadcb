"""Benchmark of the rigidity scan on GB300: site cutoffs/s on the 5-degree
global grid with IGRF-14 + T96 (Pdyn 2 nPa, Dst -20 nT, By 0, Bz -1 nT,
2020-06-21 12:00 UT), vertical incidence from 20 km, 20 -> 0.01 GV in 0.01 GV
steps (2,664 sites x 2,000 rigidities = 5.33 M trajectories), FP64.

One step = one batch of sites (the grid split into --batches interleaved
slices of equal size, taken in turn).  Every step's batch is one segment of a
scan stream (cor_stream_*): one resident launch of the scan kernel serves all
timed steps, its lanes refilling from the next segment as trajectories end.
`value` is the device-resident rate (inputs in device memory before the timed
region; the launch timed with CUDA events on its own stream); `e2e` is the
same work through cor_stream_submit / cor_stream_wait with host buffers, the
host<->device copies inside the timed region.  `learned_window` scans only the
windows the trained network predicts, through the same stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank takes its own batches (weak scaling, no data-path
collective); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cor-model_gb300"))

import cortrace as ct  # noqa: E402
import window  # noqa: E402

WORKLOAD = "igrf14+t96 5x5deg global grid, vertical, 20 km, 20->0.01 GV by 0.01 (2664 sites x 2000)"
TIME7 = [2020, 6, 21, 173, 12, 0, 0]
PARMOD = [2.0, -20.0, 0.0, -1.0]
N_RIG = 2000
METRIC = "site cutoffs/s on 1 GB300: plain scan vs learned window at |\u0394Rc|\u22640.01 GV"
UNIT = "site cutoffs/s"
WINDOW_FILE = os.path.join(ROOT, "cor-model_gb300", "window_t96.npz")
# DRAM bytes (read + write) per trajectory of the stream kernel, from the ncu
# capture of its bulk profiling case with lane regrouping
# (profiles/stream_kernel_igrf_t96_profile_case.md: 1.55 MB + 0.11 MB over the
# 256,000 trajectories of the launch)
DRAM_BYTES_PER_TRAJ = (1.551104e6 + 0.112640e6) / 256000
TUNING_FILE = os.path.join(ROOT, "cor-model_gb300", "tuning.json")


def tuning() -> dict:
    """The autotuner's choice (cor-model_gb300/autotune.py), else the defaults."""
    if os.path.exists(TUNING_FILE):
        with open(TUNING_FILE) as f:
            t = json.load(f)
        out = {k: t[k] for k in ("inflight", "park_below", "max_generations", "min_park")}
        if "stream" in t:
            out["stream_queue_order"] = t["stream"]["queue_order"]
            out["stream_sort_lanes"] = t["stream"].get("sort_lanes", 1)
        return out | {"rigidity_major": t.get("rigidity_major", 1), "source": "autotune"}
    return {"inflight": 3, "park_below": 16, "max_generations": 48, "min_park": 256, "rigidity_major": 1,
            "source": "defaults"}


def grid_sites() -> list[tuple[float, float]]:
    return [(float(lat), float(lon)) for lat in range(-90, 91, 5) for lon in range(0, 360, 5)]


def batch_sites(b: int, n_batches: int) -> list[tuple[float, float]]:
    return grid_sites()[b::n_batches]


def make_jobs(sites) -> np.ndarray:
    return np.concatenate([ct.make_job(lat, lon, rig=0.01, rk=20.0, dele=0.01) for lat, lon in sites])


def rank_batches(rank: int, world: int, n_batches: int) -> list[int]:
    """Batches a rank processes (weak scaling: every rank gets whole batches)."""
    return [b for b in range(n_batches) if b % world == rank] or [rank % n_batches]


def models():
    return ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96)


def params():
    return ct.internal_setup("igrf14", TIME7, parmod=PARMOD)


# ---- algorithmic work model ------------------------------------------------
def work_model() -> dict:
    """FP64 operations per accepted step and per rejected trial of this
    workload, from the op-counting build of the oracle (a seeded sample of the
    same workload), falling back to the hand count below if it is absent."""
    path = os.path.join(ROOT, "oracle", "work_model_igrf_t96.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    # hand count of the reference formulation (+ - * / sqrt = 1, each
    # transcendental = 20): RK velocity half 210 + trial overhead 30 + turn
    # test 4 + atan2; position half 138; geometry 26 + 2 atan2; step update
    # 19; field composition 51 + internal_geo (K = 14: 2574) + T96 (branch
    # mix, about 4300).
    return {"flops_per_step": 2574 + 51 + 4300 + 138 + 26 + 40 + 19 + 244 + 20,
            "flops_per_rejected_trial": 244 + 20, "source": "hand count"}


FN_INDEX = {"exp": 1, "log": 2, "sin": 3, "cos": 4, "atan": 5, "asin": 6, "atan2": 7, "pow": 8}


def step_flops(wm: dict, fn_flops) -> dict:
    """FP64 work per accepted step three ways: + - * / sqrt count 1 each and a
    transcendental counts (a) its cost measured on this GPU in FMA-pipe flops
    (cor_probe_fp64_functions), (b) the work model's fixed weight, (c) 0."""
    cls = wm.get("per_step_by_class")
    if not cls:
        return {"measured": wm["flops_per_step"], "fixed": wm["flops_per_step"], "excluded": wm["flops_per_step"]}
    base = sum(cls[k] for k in ("add", "mul", "div", "sqrt"))
    trans = {k: v for k, v in cls.items() if k not in ("add", "mul", "div", "sqrt") and v}
    measured = base + sum(v * fn_flops[FN_INDEX[k]] for k, v in trans.items())
    fixed = base + sum(trans.values()) * wm.get("transcendental_weight", 20)
    return {"measured": measured, "fixed": fixed, "excluded": base,
            "weights_measured": {k: round(float(fn_flops[FN_INDEX[k]]), 1) for k in trans}}


# ---- measurement helpers -----------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_info() -> dict:
    """The host's CPU model and its logical and physical core counts (lscpu)."""
    info = {"model": platform.processor() or platform.machine(), "logical_cpus": os.cpu_count() or 1,
            "physical_cores": None}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
    except (OSError, subprocess.SubprocessError):
        out = ""
    f = {}
    for ln in out.splitlines():
        k, _, v = ln.partition(":")
        f.setdefault(k.strip(), v.strip())
    if f.get("Model name"):
        info["model"] = f["Model name"]
    try:
        info["physical_cores"] = int(f["Core(s) per socket"]) * int(f.get("Socket(s)", "1"))
    except (KeyError, ValueError):
        info["physical_cores"] = info["logical_cpus"]
    return info


def reference_params():
    """The bench condition's parameter block for the CPU arms, taken from the
    reference's own set-up output (tests/golden/setup_params.json, made by the
    reference's internal_recalc) so that no product code runs on them."""
    with open(os.path.join(ROOT, "tests", "golden", "setup_params.json")) as f:
        cases = json.load(f)["cases"]
    case = next(c for c in cases if c["version"] == "igrf14" and c["time"] == TIME7)
    p = np.zeros(1, ct.PARAMS_DTYPE)
    for k in ("g", "h", "rec", "a1", "a2", "a3"):
        p[k][0] = [float.fromhex(v) for v in case[k]]
    p["parmod"][0, :4] = PARMOD
    return p


def cpu_sample_sites(n_batches: int, k: int, n: int) -> list[tuple[float, float]]:
    """n sites of step k's batch, spread over its latitudes."""
    sites = batch_sites(k % n_batches, n_batches)
    stride = max(1, len(sites) // n)
    return sites[::stride][:n]


def cpu_scan(sample, threads: int) -> tuple[float, int]:
    """The oracle port on `threads` host threads over the sample (chunks of
    rigidities handed out dynamically); returns (seconds, accepted steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    jobs = make_jobs(sample)
    t = time.perf_counter()
    res = pyoracle.scan_batch(jobs, reference_params(), models=models(), threads=threads)
    return time.perf_counter() - t, res.counters["accepted_steps"]


CPU_SAMPLE_SITES = 32


def cpu_baseline(n_batches: int) -> dict:
    """The oracle (CPU restatement) on a bounded sample of the same workload,
    all host threads, rigidities handed out in small chunks as the reference's
    OpenMP loop does."""
    info = cpu_info()
    threads = info["logical_cpus"]
    sample = cpu_sample_sites(n_batches, 0, CPU_SAMPLE_SITES)
    dt, steps = cpu_scan(sample, threads)
    return {"value": len(sample) / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(sample)} sites x {N_RIG} rigidities of the first step's batch "
                      f"({len(sample) * N_RIG} trajectories, {dt:.1f} s wall, 4-rigidity chunks over all threads)",
            "steps_per_s": steps / dt, "cpu": info}


# ---- the GPU arm -------------------------------------------------------------
SORT_LANES = None  # --sort-lanes; None: the tuning file's choice (default 1)


def sort_lanes() -> int:
    return int(SORT_LANES if SORT_LANES is not None else tuning().get("stream_sort_lanes", 1))


def stream_settings(n_jobs: int, n_traj: int) -> dict:
    return {"slots": 8, "max_jobs": max(1, n_jobs), "max_trajectories": max(1, n_traj), "max_params": 1,
            "fixed_params": 4, "pool_params": 64, "idle_limit_s": 120.0, "sort_lanes": sort_lanes()}


def run_device_segments(s, segs) -> list:
    """Publishes device-resident segments as the ring allows and collects them
    in order; returns (counters, completion ns) per segment."""
    from collections import deque
    out = [None] * len(segs)
    inflight = deque()
    nxt = 0
    while nxt < len(segs) or inflight:
        while nxt < len(segs) and len(inflight) < s.config.slots:
            bf = segs[nxt]
            t = s.submit_device(bf["jobs"].data_ptr(), bf["trig"].data_ptr(), bf["off"].data_ptr(), bf["off_host"],
                                bf["n_jobs"], bf["sites"].data_ptr(), bf["status"].data_ptr())
            inflight.append((t, nxt))
            nxt += 1
        t, i = inflight.popleft()
        out[i] = s.wait(t, -1)
    return out


def run_host_segments(s, jobs_list, p) -> list:
    """cor_stream_submit of host batches, results copied back to the host."""
    from collections import deque
    out = [None] * len(jobs_list)
    inflight = deque()
    nxt = 0
    while nxt < len(jobs_list) or inflight:
        while nxt < len(jobs_list) and len(inflight) < s.config.slots:
            inflight.append((s.submit(jobs_list[nxt], p), nxt))
            nxt += 1
        t, i = inflight.popleft()
        out[i] = s.wait(t, -1)[0]
    return out


def site_features(latlon) -> np.ndarray:
    """The window network's inputs for vertical incidence at this workload's
    condition (IGRF-14 + T96 at 2020-06-21 12 UT)."""
    p = params()
    tilt, ep = window.dipole_tilt(p), window.decimal_epoch(TIME7)
    return np.array([window.features(lat, lon, 0.0, 0.0, ep, PARMOD, tilt) for lat, lon in latlon])


def measure_window(args, ctx, bufs, plain, p, plain_e2e: float) -> dict:
    """The learned window on the timed steps' sites: windows predicted by the
    network (tensor cores) and traced through a scan stream with host buffers
    (like e2e), widened on an edge hit (full scan after 3 widenings), R_C
    compared with the plain scan of the same sites.  All timed sites' first
    windows go in as one segment, handed out in ascending rigidity over every
    trajectory, so the longest trajectories of all windows start first."""
    wm = window.WindowModel(args.window)
    timed = list(range(args.warmup, args.warmup + args.steps))
    jobs = np.concatenate([bufs[i]["host_jobs"] for i in timed])
    feats = np.concatenate([site_features(bufs[i]["latlon"]) for i in timed])
    s = ct.Stream(ctx, models(), scan_events=1, **stream_settings(len(jobs), len(jobs) * N_RIG))
    wm.windows(feats[:8])                            # load the network's kernels before timing
    t0 = time.perf_counter()
    i_lo, i_hi = wm.windows(feats, k=args.window_k)  # no stream kernel runs now: the network has the SMs
    (sites, fb, traced, _), = window.trace_windows_stream(s, [(jobs, p, i_lo, i_hi)])
    launch_ms = s.drain()
    wall = time.perf_counter() - t0
    s.close()
    wm.close()
    full = np.concatenate([plain[k].sites for k in range(len(timed))])
    d = np.abs(sites["r_cutoff"] - full["r_cutoff"])
    n_sites = len(full)
    full_traj = sum(bufs[i]["n"] for i in timed)
    v = n_sites / wall
    return {"value": v, "unit": UNIT, "speedup_vs_plain_e2e": v / plain_e2e if plain_e2e else None,
            "sites": n_sites, "agree_frac_dRc_le_0.01GV": int(np.sum(d <= 0.01 + 1e-9)) / n_sites,
            "max_abs_dRc_GV": float(d.max()), "widened_frac": int(fb.sum()) / n_sites,
            "trajectories_frac_of_full_scan": traced / full_traj, "stream_launch_ms": launch_ms,
            "model": json.loads(wm.info) if wm.info.startswith("{") else wm.info, "k_sigma": args.window_k,
            "how": f"predicted window +-{args.window_k:g} sigma on the 0.01 GV grid, widened on the hit side on an edge hit (full scan "
                   "after 3 widenings); the timed steps' windows as one segment of a scan stream (ascending "
                   "rigidity), each scan's result taken as soon as it is reduced so that a retrace starts at once; "
                   "host buffers, network inference on the tensor cores inside the timed region"}


def reduce_over_ranks(dist, seconds: float, counts: list, device: str) -> list:
    """Whole-job figures of a multi-rank run: the slowest rank's time (MAX)
    and the sums of the per-rank counts.  Returns [seconds, *counts]."""
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    out = [float(t.item())]
    if counts:
        c = torch.tensor([float(v) for v in counts], dtype=torch.float64, device=device)
        dist.all_reduce(c)
        out += [int(v) for v in c.tolist()]
    return out


def device_segments(torch, dev: int, jobs_list, base: int) -> list:
    """Each step's inputs and outputs in device memory (jobs refer to the
    stream's fixed parameter block `base`)."""
    out = []
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(f"cuda:{dev}")
    for jobs, latlon in jobs_list:
        n, off = ct.batch_offsets(jobs)
        dj = jobs.copy()
        dj["param_index"] = base
        out.append({"n_jobs": len(jobs), "n": n, "jobs": t(dj), "trig": t(ct.prepare_trig(jobs)), "off": t(off),
                    "off_host": off,
                    "sites": torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8,
                                         device=f"cuda:{dev}"),
                    "status": torch.zeros(n, dtype=torch.uint8, device=f"cuda:{dev}"),
                    "host_jobs": jobs, "latlon": latlon})
    return out


def run_ours(args, rank: int, world: int, dist) -> dict | None:
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p = params()
    tune = tuning()
    mine = rank_batches(rank, world, args.batches)
    n_steps = args.warmup + args.steps
    steps = [(make_jobs(batch_sites(mine[k % len(mine)], args.batches)), batch_sites(mine[k % len(mine)],
                                                                                   args.batches))
             for k in range(n_steps)]
    ctx = ct.Context(dev)
    ctx.set_queue_order(int(tune.get("stream_queue_order", tune["rigidity_major"])))
    peak = C.c_double(0.0)
    ctx.lib.cor_probe_fp64_peak(ctx.h, C.byref(peak))
    fn_flops = np.zeros(11)
    ctx._check(ctx.lib.cor_probe_fp64_functions(ctx.h, fn_flops.ctypes.data), "cor_probe_fp64_functions")
    max_jobs = max(len(j) for j, _ in steps)
    s = ct.Stream(ctx, models(), **stream_settings(max_jobs, max_jobs * N_RIG))
    base = s.upload_params(p)
    bufs = device_segments(torch, dev, steps, base)
    torch.cuda.synchronize()

    run_device_segments(s, bufs[:args.warmup])      # warm-up launch
    s.drain()
    if dist:
        dist.barrier(device_ids=[dev])
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        t0 = time.perf_counter()
        res = run_device_segments(s, bufs[args.warmup:])
        launch_ms = s.drain()                           # CUDA events around the launch, on its stream
        host_s = time.perf_counter() - t0
    dev_s = launch_ms / 1e3
    timed = bufs[args.warmup:]
    steps_acc = sum(int(c["accepted_steps"]) for c, _ in res)
    trials_acc = sum(int(c["trials"]) for c, _ in res)
    traj_done = sum(int(c["trajectories"]) for c, _ in res)
    sites_done = sum(b["n_jobs"] for b in timed)
    done_ns = [t_ns for _, t_ns in res]
    if dist:
        dev_s, sites_done, traj_done, steps_acc, trials_acc = reduce_over_ranks(
            dist, dev_s, [sites_done, traj_done, steps_acc, trials_acc], f"cuda:{dev}")

    # e2e through the public C ABI with host buffers: cor_stream_submit copies
    # each step's inputs in and cor_stream_wait its results out, inside the
    # timed region
    t0 = time.perf_counter()
    plain = run_host_segments(s, [b["host_jobs"] for b in timed], p)
    e2e_launch_ms = s.drain()
    e2e_s = time.perf_counter() - t0
    h2d = sum(b["host_jobs"].nbytes + b["n_jobs"] * ct.TRIG_DTYPE.itemsize + (b["n_jobs"] + 1) * 8 + 96 + 8
              for b in timed) + 3840
    d2h = sum(r.sites.nbytes + r.status.nbytes + 64 for r in plain)
    if dist:
        e2e_s = reduce_over_ranks(dist, e2e_s, [], f"cuda:{dev}")[0]
    for r, b in zip(plain, timed):
        # the device-resident run and the host-buffer run are the same scans
        assert np.array_equal(r.sites.view(np.uint8), b["sites"].cpu().numpy()), "e2e and device results differ"
    learned = None
    if args.window and os.path.exists(args.window) and world == 1:
        learned = measure_window(args, ctx, bufs, plain, p, sites_done / e2e_s)
    s.close()
    ctx.close()
    if rank != 0:
        return None
    wm = work_model()
    per_step = step_flops(wm, fn_flops)
    achieved = steps_acc * per_step["measured"] / dev_s / 1e12
    pk = peak.value / 1e12
    out = {
        "metric": METRIC, "value": sites_done / dev_s, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic grid of sites (the configuration's own sites; no dataset)",
        "config": {"workload": WORKLOAD, "sites_per_step": sites_done // max(1, args.steps * world),
                   "trajectories_per_step": traj_done // max(1, args.steps * world),
                   "batches": args.batches, "tuning": tune | {"stream_sort_lanes": sort_lanes()},
                   "execution": "one persistent scan-stream launch per timed run: every step's batch is a segment "
                                "published to the resident kernel, whose lanes refill from the next segment as "
                                "trajectories end",
                   "l2": "no L2 flush: the kernel is FP64-bound and its state lives in registers; inputs and "
                         "outputs are MB-sized", "parallelism": f"sites split over {world} GPU(s)"},
        "trajectories_per_s": traj_done / dev_s, "steps_per_s": steps_acc / dev_s,
        "timing": {"launch_ms_cuda_events": launch_ms, "host_wall_s": host_s,
                   "segment_done_s": [round((t - done_ns[0]) / 1e9, 3) for t in done_ns]},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": pk, "unit": "TFLOP/s",
                     "frac": achieved / pk if pk else None,
                     "frac_transcendentals_at_fixed_weight": steps_acc * per_step["fixed"] / dev_s / 1e12 / pk,
                     "frac_transcendentals_excluded": steps_acc * per_step["excluded"] / dev_s / 1e12 / pk,
                     "flops_per_step_measured_weights": per_step["measured"],
                     "transcendental_weights_measured": per_step.get("weights_measured"),
                     "division_sqrt_cost_measured": [round(float(fn_flops[9]), 1), round(float(fn_flops[10]), 1)],
                     "traffic": DRAM_BYTES_PER_TRAJ * traj_done / max(1, args.steps * world),
                     "traffic_unit": "bytes per step (one batch), scaled by trajectories from the ncu capture of "
                                     "the stream kernel's bulk profiling case (128 sites, 256,000 trajectories)",
                     "work_model": wm.get("source") + "; + - * / sqrt = 1 op, each transcendental at its cost "
                                   "measured on this GPU (cor_probe_fp64_functions, FMA-pipe flops per call)",
                     "flops_per_step_fixed_weight": wm["flops_per_step"],
                     "peak_source": "DFMA microbenchmark in libcortrace (cor_probe_fp64_peak), FMA = 2 flops"},
        "e2e": {"value": sites_done / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps,
                "stream_launch_ms": e2e_launch_ms},
        "gpu_launches": 1,
        "clocks": clocks.summary(),
    }
    if learned is not None:
        out["learned_window"] = learned
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.batches)
    return out


# ---- small cases of the same kernels, for profiler captures -------------------
PROFILE_SITES = 32
PROFILE_STEP_LIMIT = 2500


def run_profile_case(args) -> dict:
    """PROFILE_SITES sites spread over all latitudes x the 2,000 rigidities, with
    the step limit lowered to PROFILE_STEP_LIMIT so that a launch lasts about a
    second: the bulk of the scan's work without the 25,000-step tail.  With
    --profile-stream the same scans go through a scan stream staged before its
    launch (launch_on_drain), so the launch never waits on the host and a
    profiler can replay it; otherwise through cor_trace_batch_device.
    Not a bench line; it exists to be captured under ncu."""
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p = params()
    n_sites, step_limit = args.profile_sites, args.profile_step_limit
    sites = grid_sites()[::len(grid_sites()) // n_sites][:n_sites]
    jobs = make_jobs(sites)
    ctx = ct.Context(dev)
    tune = tuning()
    ctx.set_queue_order(int(tune.get("stream_queue_order", tune["rigidity_major"])))
    ctx.set_lane_sort(bool(sort_lanes()))
    ms = []
    if args.profile_stream:
        parts = [jobs[k::4] for k in range(4)]
        s = ct.Stream(ctx, models(), step_limit=step_limit, launch_on_drain=1,
                      **stream_settings(len(parts[0]), len(parts[0]) * N_RIG))
        base = s.upload_params(p)
        bufs = device_segments(torch, dev, [(j, None) for j in parts], base)
        for _ in range(args.warmup + args.steps):
            ts = [s.submit_device(b["jobs"].data_ptr(), b["trig"].data_ptr(), b["off"].data_ptr(), b["off_host"],
                                  b["n_jobs"], b["sites"].data_ptr(), b["status"].data_ptr()) for b in bufs]
            ms.append(s.drain())
            c = [s.wait(t, 0)[0] for t in ts]
        s.close()
        c = {k: sum(x[k] for x in c) for k in c[0]}
    else:
        n, off = ct.batch_offsets(jobs)
        t = lambda a: torch.from_numpy(a.view(np.uint8).copy()).to(f"cuda:{dev}")
        ctx._check(ctx.lib.cor_upload_params(ctx.h, p.ctypes.data, len(p)), "cor_upload_params")
        dj, dt, do = t(jobs), t(ct.prepare_trig(jobs)), t(off)
        sites_d = torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}")
        status = torch.zeros(n, dtype=torch.uint8, device=f"cuda:{dev}")
        cnt = torch.zeros(5, dtype=torch.int64, device=f"cuda:{dev}")
        st = torch.cuda.current_stream()
        for _ in range(args.warmup + args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            rc = ctx.lib.cor_trace_batch_device(ctx.h, dj.data_ptr(), dt.data_ptr(), len(jobs), do.data_ptr(), n,
                                                models(), step_limit, 0.01, ct.DEF_HM0_P,
                                                sites_d.data_ptr(), status.data_ptr(), None, cnt.data_ptr(),
                                                ct.FLAG_UNIFORM_GRID, C.c_void_p(st.cuda_stream))
            ctx._check(rc, "cor_trace_batch_device")
            e1.record(st)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        v = cnt.cpu().numpy()
        c = dict(zip(("accepted_steps", "trials", "trajectories", "watchdog", "kernel_launches"), v.tolist()))
    ctx.close()
    return {"profile_case": f"{len(sites)} sites x {N_RIG} rigidities, step limit {step_limit}",
            "path": "stream" if args.profile_stream else "batch", "sort_lanes": sort_lanes(),
            "trajectories": int(c["trajectories"]), "accepted_steps": int(c["accepted_steps"]),
            "trials": int(c["trials"]), "call_ms": ms}


def run_chaos_case(args) -> dict:
    """The CHAOS-7.16 crustal field (degree 185, the warp-cooperative sum) with
    IGRF-14 through cor_field_batch on seeded points 1-3 R_E, timed end to end
    (host buffers), against the oracle's restatement of the reference's
    chaos_geo on a few of the same points on one host core.  Not a bench
    line; it measures the high-degree field on its own."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    rng = np.random.default_rng(185)
    n = args.chaos_points
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    pts = u * (ct.DEF_RE * rng.uniform(1.0, 3.0, n))[:, None]
    p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
    m = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_NONE, ct.CRUSTAL_CHAOS)
    ctx = ct.Context(0)
    ctx.field_batch(pts[:1024], p, models=m)                # uploads the table, loads the kernel
    best = 1e30
    for _ in range(3):
        t = time.perf_counter()
        got = ctx.field_batch(pts, p, models=m)
        best = min(best, time.perf_counter() - t)
    ctx.close()
    k = 64
    t = time.perf_counter()
    want = pyoracle.calculate_field(pts[:k], p, models=m)
    cpu = (time.perf_counter() - t) / k
    rel = np.linalg.norm(got[:k] - want, axis=1) / np.linalg.norm(want, axis=1)
    return {"chaos_case": f"IGRF-14 + CHAOS-7.16 (n <= 185) at {n} seeded points, 1-3 R_E",
            "gpu_us_per_point": best / n * 1e6, "gpu_points_per_s": n / best,
            "cpu_oracle_us_per_point_one_core": cpu * 1e6, "max_rel_diff_vs_oracle": float(rel.max())}


def run_reference(args, rank: int) -> dict | None:
    """CPU reference arm: the oracle port on all host threads, one bounded
    sample per step (CPU_SAMPLE_SITES sites of that step's batch)."""
    if rank != 0:
        return None
    info = cpu_info()
    threads = info["logical_cpus"]
    done = 0
    dt_tot = 0.0
    steps = 0
    n_sample = 0
    for i in range(args.warmup + args.steps):
        sample = cpu_sample_sites(args.batches, i, CPU_SAMPLE_SITES)
        n_sample = len(sample)
        dt, _ = cpu_scan(sample, threads)
        if i >= args.warmup:
            done += len(sample)
            dt_tot += dt
            steps += 1
    v = done / dt_tot
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt_tot * 1e3 / max(1, steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic grid of sites",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sites_per_step": n_sample,
                       "devices": "host cores of rank 0 only; no GPU work"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "cpu": info,
                             "sample": f"{n_sample} sites x {N_RIG} rigidities of each step's batch, "
                                       f"4-rigidity chunks handed out over all threads"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batches", type=int, default=32,
                    help="the grid is split into this many interleaved batches; one step scans one batch")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--window-k", type=float, default=3.0,
                    help="half-width of the learned window in held-out sigmas of the network's band")
    ap.add_argument("--window", default=WINDOW_FILE, help="trained window model for the learned-window line "
                    "(train_window.py output); skipped when the file is absent")
    ap.add_argument("--profile-case", action="store_true",
                    help="run only the small profiling case of the scan kernel (prints its own JSON, not a bench line)")
    ap.add_argument("--chaos-case", action="store_true",
                    help="time the CHAOS-7.16 crustal field alone (prints its own JSON, not a bench line)")
    ap.add_argument("--chaos-points", type=int, default=1 << 20)
    ap.add_argument("--profile-sites", type=int, default=PROFILE_SITES)
    ap.add_argument("--profile-step-limit", type=int, default=PROFILE_STEP_LIMIT)
    ap.add_argument("--profile-stream", action="store_true",
                    help="with --profile-case: through a scan stream launched with everything staged")
    ap.add_argument("--sort-lanes", type=int, choices=(0, 1), default=None,
                    help="regroup each block's trajectories by field band before every field evaluation "
                         "(default: the tuning file's choice, else 1)")
    args = ap.parse_args()
    global SORT_LANES
    SORT_LANES = args.sort_lanes
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        backend = "gloo" if args.impl == "reference" else "nccl"
        tdist.init_process_group(backend)
        dist = tdist
    if args.chaos_case:
        out = run_chaos_case(args) if rank == 0 else None
    elif args.profile_case:
        out = run_profile_case(args) if rank == 0 else None
    elif args.impl == "reference":
        out = run_reference(args, rank)
    else:
        out = run_ours(args, rank, world, dist)
    if out is not None:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
