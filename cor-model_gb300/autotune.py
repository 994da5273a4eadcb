"""Autotuner of the scan's launch settings (no counterpart in the reference).

    python cor-model_gb300/autotune.py [--sites N] [--out FILE]

Times a sample of the IGRF-14 + T96 5-degree-grid workload (every k-th site,
the full 2,000-rigidity scans) under candidate settings and writes the
fastest to FILE (JSON), which bench.py and serve.py read:
  * regrouping (cor_ctx_set_regroup): park_below, the live lanes per warp
    under which a block parks its trajectories for the next kernel
    generation, and max_generations (1 = never regroup);
  * inflight: how many batches run at once, each on its own context and
    stream, so that one batch's tail of long trajectories overlaps the next
    batch's bulk;
  * the work-queue order (cor_ctx_set_queue_order): lowest rigidities of all
    scans first, or consecutive rigidities of one scan to neighbouring lanes.
Results do not depend on any setting (checked: every candidate's P(S), P(C),
P(M) must equal the first's); only the time does.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import cortrace as ct  # noqa: E402

TIME7 = [2020, 6, 21, 173, 12, 0, 0]
PARMOD = [2.0, -20.0, 0.0, -1.0]
DEFAULT_OUT = os.path.join(HERE, "tuning.json")


def load_tuning(path: str = DEFAULT_OUT) -> dict | None:
    """The autotuner's choice, or None when it has not been run."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        t = json.load(f)
    return {k: t.get(k, 1) if k == "rigidity_major" else t[k]
            for k in ("inflight", "park_below", "max_generations", "min_park", "rigidity_major")}


def sample_jobs(n_sites: int, parts: int):
    grid = [(float(la), float(lo)) for la in range(-90, 91, 5) for lo in range(0, 360, 5)]
    step = max(1, len(grid) // n_sites)
    sites = grid[::step][:n_sites]
    jobs = [np.concatenate([ct.make_job(la, lo, rig=0.01, rk=20.0, dele=0.01) for la, lo in sites[k::parts]])
            for k in range(parts)]
    return jobs


def run(ctxs, parts, p, models):
    out = [None] * len(parts)

    def work(k):
        out[k] = ctxs[k % len(ctxs)].trace_batch(parts[k], p, models=models, want_status=False)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(k,)) for k in range(len(parts))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    return time.perf_counter() - t0, out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sites", type=int, default=48)
    ap.add_argument("--out", default=DEFAULT_OUT)
    args = ap.parse_args()
    p = ct.internal_setup("igrf14", TIME7, parmod=PARMOD)
    models = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96)
    candidates = []
    for inflight in (1, 2, 3, 4):
        for park_below, gens in ((16, 48), (8, 48), (24, 48), (16, 1)):
            if inflight > 1 and (park_below, gens) not in ((16, 48), (8, 48), (24, 48)):
                continue
            candidates.append({"inflight": inflight, "park_below": park_below, "max_generations": gens,
                               "min_park": 256, "rigidity_major": 1})
    for inflight in (1, 3):
        candidates.append({"inflight": inflight, "park_below": 16, "max_generations": 48, "min_park": 256,
                           "rigidity_major": 0})
    ctxs = [ct.Context(0) for _ in range(4)]
    ref = None
    results = []
    for c in candidates:
        for x in ctxs:
            x.set_regroup(c["park_below"], c["max_generations"], c["min_park"])
            x.set_queue_order(bool(c["rigidity_major"]))
        parts = sample_jobs(args.sites, c["inflight"])
        run(ctxs[:c["inflight"]], [pp[:2] for pp in parts], p, models)      # warm the kernels
        dt, out = run(ctxs[:c["inflight"]], parts, p, models)
        # results must not depend on the setting
        sites = np.sort(np.concatenate([o.sites for o in out]),
                        order=["r_lower", "r_upper", "r_cutoff", "n_forbidden", "n_traj"])
        if ref is None:
            ref = sites
        same = bool(np.array_equal(sites, ref))
        results.append({**c, "seconds": dt, "site_cutoffs_per_s": args.sites / dt, "same_results": same})
        print(json.dumps(results[-1]), flush=True)
    for x in ctxs:
        x.close()
    ok = [r for r in results if r["same_results"]]
    best = min(ok, key=lambda r: r["seconds"])
    out = {"inflight": best["inflight"], "park_below": best["park_below"],
           "max_generations": best["max_generations"], "min_park": best["min_park"],
           "rigidity_major": best["rigidity_major"],
           "sample": f"{args.sites} sites of the 5-deg grid x 2000 rigidities, IGRF-14 + T96",
           "measurements": results}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("inflight", "park_below", "max_generations", "min_park", "rigidity_major")}))


if __name__ == "__main__":
    main()
