"""Benchmark of the rigidity scan on GB300: site cutoffs/s on the 5-degree
global grid with IGRF-14 + T96 (Pdyn 2 nPa, Dst -20 nT, By 0, Bz -1 nT,
2020-06-21 12:00 UT), vertical incidence from 20 km, 20 -> 0.01 GV in 0.01 GV
steps (2,664 sites x 2,000 rigidities = 5.33 M trajectories), FP64.

One step = one batch of sites (the grid split into --batches interleaved
slices of equal size, taken in turn).  `value` is the device-resident rate
(inputs uploaded before the timed region, CUDA events on the launch stream);
`e2e` is the same work through the C ABI call cor_trace_batch with host
buffers, the host<->device copies inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank takes its own batches (weak scaling, no data-path
collective); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
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
# DRAM bytes (read + write) per trajectory of the scan kernel, from the ncu
# capture of the profiling case (profiles/trace_kernel_igrf_t96_profile_case.md:
# 1.61 MB + 0.19 MB over the 64,000 trajectories of its generation-0 launch)
DRAM_BYTES_PER_TRAJ = (1.613312e6 + 0.185856e6) / 64000
TUNING_FILE = os.path.join(ROOT, "cor-model_gb300", "tuning.json")


def tuning() -> dict:
    """The autotuner's choice (cor-model_gb300/autotune.py), else the defaults."""
    if os.path.exists(TUNING_FILE):
        with open(TUNING_FILE) as f:
            t = json.load(f)
        out = {k: t[k] for k in ("inflight", "park_below", "max_generations", "min_park")}
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


def cpu_baseline(n_batches: int, seconds_hint: float = 20.0) -> dict:
    """The oracle (CPU restatement) on a bounded sample of the same workload,
    all host threads, one site per thread."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    threads = os.cpu_count() or 1
    sites = batch_sites(0, n_batches)
    # spread the sample over latitudes
    step = max(1, len(sites) // threads)
    sample = sites[::step][:threads]
    jobs = make_jobs(sample)
    t = time.perf_counter()
    res = pyoracle.scan_batch(jobs, params(), models=models(), threads=threads)
    dt = time.perf_counter() - t
    return {"value": len(sample) / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(sample)} sites x {N_RIG} rigidities of the same grid and conditions "
                      f"({res.counters['trajectories']} trajectories, {dt:.1f} s wall)",
            "steps_per_s": res.counters["accepted_steps"] / dt}


# ---- the GPU arm -------------------------------------------------------------
class Lane:
    """One in-flight slot: a context with its own stream, work queue and park
    buffers.  Batches on different slots overlap on the GPU, so one batch's
    tail of long trajectories runs beside the next batch's bulk."""

    def __init__(self, dev: int, p, tune: dict | None = None):
        import torch
        self.torch = torch
        self.ctx = ct.Context(dev)
        self.flags = ct.FLAG_UNIFORM_GRID
        if tune:
            self.ctx.set_regroup(tune["park_below"], tune["max_generations"], tune["min_park"])
            self.ctx.set_queue_order(bool(tune["rigidity_major"]))
            self.flags = ct.FLAG_UNIFORM_GRID if tune["rigidity_major"] else 0
        self.stream = torch.cuda.Stream(device=dev)
        rc = self.ctx.lib.cor_upload_params(self.ctx.h, p.ctypes.data, len(p))
        if rc != 0:
            raise ct.CorError(rc, self.ctx.error())
        self.cnt = torch.zeros(5, dtype=torch.int64, device=f"cuda:{dev}")

    def run(self, bf, step_limit: int = 25000) -> None:
        """Scan one batch (device buffers) on this slot's stream; returns when done."""
        lib = self.ctx.lib
        e0 = self.torch.cuda.Event(enable_timing=True)
        e1 = self.torch.cuda.Event(enable_timing=True)
        e0.record(self.stream)
        rc = lib.cor_trace_batch_device(
            self.ctx.h, bf["jobs"].data_ptr(), bf["trig"].data_ptr(), bf["n_jobs"], bf["off"].data_ptr(), bf["n"],
            models(), step_limit, 0.01, ct.DEF_HM0_P, bf["sites"].data_ptr(), bf["status"].data_ptr(), None,
            self.cnt.data_ptr(), self.flags, C.c_void_p(self.stream.cuda_stream))
        if rc != 0:
            raise ct.CorError(rc, self.ctx.error())
        e1.record(self.stream)
        self.stream.synchronize()
        bf["counters"] = self.cnt.cpu().numpy().copy()
        bf["kernel_ms"] = e0.elapsed_time(e1)
        bf["generations"] = self.ctx.generation_log()


def run_batches(slots, bufs, order) -> None:
    """Runs the batches in `order` over the slots, each slot taking the next
    batch as soon as it is free (one host thread per slot)."""
    import queue
    q = queue.Queue()
    for i in order:
        q.put(i)
    errors = []

    def worker(slot):
        while True:
            try:
                i = q.get_nowait()
            except queue.Empty:
                return
            try:
                slot.run(bufs[i])
            except Exception as e:  # noqa: BLE001
                errors.append(e)
                return

    ts = [threading.Thread(target=worker, args=(s,)) for s in slots]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    if errors:
        raise errors[0]


def site_features(latlon) -> np.ndarray:
    """The window network's inputs for vertical incidence at this workload's
    condition (IGRF-14 + T96 at 2020-06-21 12 UT)."""
    p = params()
    tilt, ep = window.dipole_tilt(p), window.decimal_epoch(TIME7)
    return np.array([window.features(lat, lon, 0.0, 0.0, ep, PARMOD, tilt) for lat, lon in latlon])


def measure_window(args, slots, bufs, p, plain_e2e: float) -> dict:
    """The learned window on the timed batches: predicted windows traced
    through cor_trace_batch (host buffers, like e2e), full-scan fallback on
    an edge hit, R_C compared with the plain scan of the same sites."""
    import queue
    wm = window.WindowModel(args.window)
    timed = list(range(args.warmup, args.warmup + args.steps))
    feats = {i: site_features(bufs[i]["latlon"]) for i in timed}
    wm.windows(feats[timed[0]])                     # load the network's kernels before timing
    q = queue.Queue()
    for i in timed:
        q.put(i)
    out = {}

    def worker(slot):
        while True:
            try:
                i = q.get_nowait()
            except queue.Empty:
                return
            i_lo, i_hi = wm.windows(feats[i])
            out[i] = window.trace_windows(slot.ctx, bufs[i]["host_jobs"], p, models(), i_lo, i_hi)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=worker, args=(s,)) for s in slots]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    wall = time.perf_counter() - t0
    n_sites = agree = fallback = traced = 0
    full_traj = 0
    worst = 0.0
    for i in timed:
        full = bufs[i]["sites"].cpu().numpy().view(ct.SITE_DTYPE)
        sites, fb, tr, _ = out[i]
        d = np.abs(sites["r_cutoff"] - full["r_cutoff"])
        agree += int(np.sum(d <= 0.01 + 1e-9))
        worst = max(worst, float(d.max()))
        n_sites += len(full)
        fallback += int(fb.sum())
        traced += tr
        full_traj += bufs[i]["n"]
    wm.close()
    v = n_sites / wall
    return {"value": v, "unit": UNIT, "speedup_vs_plain_e2e": v / plain_e2e if plain_e2e else None,
            "sites": n_sites, "agree_frac_dRc_le_0.01GV": agree / n_sites, "max_abs_dRc_GV": worst,
            "widened_frac": fallback / n_sites, "trajectories_frac_of_full_scan": traced / full_traj,
            "model": json.loads(wm.info) if wm.info.startswith("{") else wm.info,
            "how": "predicted window +-3 sigma on the 0.01 GV grid, widened on the hit side on an edge hit (full scan "
                   "after 3 widenings); host buffers through cor_trace_batch, network inference on the tensor cores "
                   "inside the timed region"}


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


def run_ours(args, rank: int, world: int, dist) -> dict | None:
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p = params()
    tune = tuning()
    if args.inflight is None:
        args.inflight = tune["inflight"]
    slots = [Lane(dev, p, tune) for _ in range(args.inflight)]
    mine = rank_batches(rank, world, args.batches)
    n_steps = args.warmup + args.steps
    bufs = []
    for k in range(n_steps):
        b = mine[k % len(mine)]
        jobs = make_jobs(batch_sites(b, args.batches))
        n, off = ct.batch_offsets(jobs)
        trig = ct.prepare_trig(jobs)
        t = lambda a: torch.from_numpy(a.view(np.uint8).copy()).to(f"cuda:{dev}")
        bufs.append({
            "n_jobs": len(jobs), "n": n, "jobs": t(jobs), "trig": t(trig), "off": t(off),
            "sites": torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}"),
            "status": torch.zeros(n, dtype=torch.uint8, device=f"cuda:{dev}"),
            "host_jobs": jobs, "latlon": batch_sites(b, args.batches),
        })
    peak = C.c_double(0.0)
    slots[0].ctx.lib.cor_probe_fp64_peak(slots[0].ctx.h, C.byref(peak))

    run_batches(slots, bufs, range(args.warmup))
    torch.cuda.synchronize()
    if dist:
        dist.barrier(device_ids=[dev])
    torch.cuda.synchronize()
    with ClockSampler(dev) as clocks:
        t0 = time.perf_counter()
        run_batches(slots, bufs, range(args.warmup, n_steps))
        torch.cuda.synchronize()
        dev_s = time.perf_counter() - t0
    timed = bufs[args.warmup:]
    steps_acc = sum(int(b["counters"][0]) for b in timed)
    trials_acc = sum(int(b["counters"][1]) for b in timed)
    traj_done = sum(int(b["counters"][2]) for b in timed)
    sites_done = sum(b["n_jobs"] for b in timed)
    launch_ms = [b["kernel_ms"] for b in timed]
    if dist:
        dev_s, sites_done, traj_done, steps_acc, trials_acc = reduce_over_ranks(
            dist, dev_s, [sites_done, traj_done, steps_acc, trials_acc], f"cuda:{dev}")

    # e2e through the public C ABI with host buffers (same overlap, one host
    # thread per slot, cor_trace_batch copies in and out inside the call)
    h2d = d2h = 0
    import queue
    qe = queue.Queue()
    for i in range(args.warmup, n_steps):
        qe.put(i)
    sizes = []

    def e2e_worker(slot):
        while True:
            try:
                i = qe.get_nowait()
            except queue.Empty:
                return
            jobs = bufs[i]["host_jobs"]
            r = slot.ctx.trace_batch(jobs, p, models=models())
            sizes.append((jobs.nbytes + len(jobs) * ct.TRIG_DTYPE.itemsize + (len(jobs) + 1) * 8 + p.nbytes,
                          r.sites.nbytes + r.status.nbytes + 40))

    t0 = time.perf_counter()
    ths = [threading.Thread(target=e2e_worker, args=(s,)) for s in slots]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    e2e_s = time.perf_counter() - t0
    h2d = sum(a for a, _ in sizes)
    d2h = sum(b for _, b in sizes)
    if dist:
        e2e_s = reduce_over_ranks(dist, e2e_s, [], f"cuda:{dev}")[0]
    learned = None
    if args.window and os.path.exists(args.window) and world == 1:
        learned = measure_window(args, slots, bufs, p, sites_done / e2e_s)
    for s in slots:
        s.ctx.close()
    if rank != 0:
        return None
    wm = work_model()
    rejected = trials_acc - steps_acc
    flops = steps_acc * wm["flops_per_step"] + rejected * wm["flops_per_rejected_trial"]
    achieved = flops / dev_s / 1e12
    out = {
        "metric": METRIC, "value": sites_done / dev_s, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic grid of sites (the configuration's own sites; no dataset)",
        "config": {"workload": WORKLOAD, "sites_per_step": sites_done // max(1, args.steps * world),
                   "trajectories_per_step": traj_done // max(1, args.steps * world),
                   "batches": args.batches, "inflight": args.inflight, "tuning": tune,
                   "l2": "no L2 flush: the kernel is FP64-bound and its state lives in registers; inputs and "
                         "outputs are MB-sized", "parallelism": f"sites split over {world} GPU(s)"},
        "trajectories_per_s": traj_done / dev_s, "steps_per_s": steps_acc / dev_s,
        "batch_kernel_ms": launch_ms,
        "batch_generations": [[(n, round(ms, 1)) for n, ms in b.get("generations", [])] for b in timed[:1]],
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak.value / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / (peak.value / 1e12) if peak.value else None,
                     "traffic": DRAM_BYTES_PER_TRAJ * traj_done / max(1, args.steps * world),
                     "traffic_unit": "bytes per step (one batch), scaled by trajectories from the ncu capture of "
                                     "the profiling case",
                     "work_model": wm.get("source"),
                     "flops_per_step": wm["flops_per_step"],
                     "peak_source": "DFMA microbenchmark in libcortrace (cor_probe_fp64_peak), FMA = 2 flops"},
        "e2e": {"value": sites_done / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps},
        "gpu_launches": sum(int(b["counters"][4]) for b in timed),
        "clocks": clocks.summary(),
    }
    if learned is not None:
        out["learned_window"] = learned
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.batches)
    return out


# ---- small case of the same kernel, for profiler captures ---------------------
PROFILE_SITES = 32
PROFILE_STEP_LIMIT = 2500


def run_profile_case(args) -> dict:
    """PROFILE_SITES sites spread over all latitudes x the 2,000 rigidities, with
    the step limit lowered to PROFILE_STEP_LIMIT so that a launch lasts about a
    second: the bulk of the scan kernel's work without the 25,000-step tail.
    Not a bench line; it exists to be captured under ncu."""
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    p = params()
    slot = Lane(dev, p)
    sites = grid_sites()[::len(grid_sites()) // PROFILE_SITES][:PROFILE_SITES]
    jobs = make_jobs(sites)
    n, off = ct.batch_offsets(jobs)
    t = lambda a: torch.from_numpy(a.view(np.uint8).copy()).to(f"cuda:{dev}")
    bf = {"n_jobs": len(jobs), "n": n, "jobs": t(jobs), "trig": t(ct.prepare_trig(jobs)), "off": t(off),
          "sites": torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device=f"cuda:{dev}"),
          "status": torch.zeros(n, dtype=torch.uint8, device=f"cuda:{dev}")}
    ms = []
    for _ in range(args.warmup + args.steps):
        slot.run(bf, step_limit=PROFILE_STEP_LIMIT)
        ms.append(bf["kernel_ms"])
    c = bf["counters"]
    slot.ctx.close()
    return {"profile_case": f"{len(sites)} sites x {N_RIG} rigidities, step limit {PROFILE_STEP_LIMIT}",
            "trajectories": int(c[2]), "accepted_steps": int(c[0]), "trials": int(c[1]),
            "kernel_launches": int(c[4]), "call_ms": ms}


def run_reference(args, rank: int) -> dict | None:
    """CPU reference arm: the oracle port on the host cores, bounded samples."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    threads = os.cpu_count() or 1
    sites = batch_sites(0, args.batches)
    stride = max(1, len(sites) // (threads * max(1, args.steps + args.warmup)))
    p = params()
    done = 0
    dt_tot = 0.0
    steps = 0
    for i in range(args.warmup + args.steps):
        sample = sites[(i * threads) % len(sites)::stride][:threads]
        jobs = make_jobs(sample)
        t = time.perf_counter()
        pyoracle.scan_batch(jobs, p, models=models(), threads=threads)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            done += len(sample)
            dt_tot += dt
            steps += 1
    v = done / dt_tot
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt_tot * 1e3 / max(1, steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic grid of sites",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "sites_per_step": threads,
                       "devices": "host cores of rank 0 only; no GPU work"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{threads} sites x {N_RIG} rigidities per step, one site per thread"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batches", type=int, default=16)
    ap.add_argument("--inflight", type=int, default=None,
                    help="batches in flight at once (one stream each; default: the autotuner's choice, else 3)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--window", default=WINDOW_FILE, help="trained window model for the learned-window line "
                    "(train_window.py output); skipped when the file is absent")
    ap.add_argument("--profile-case", action="store_true",
                    help="run only the small profiling case of the scan kernel (prints its own JSON, not a bench line)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as tdist
        backend = "gloo" if args.impl == "reference" else "nccl"
        tdist.init_process_group(backend)
        dist = tdist
    if args.profile_case:
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
