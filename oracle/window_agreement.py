"""TEST INFRASTRUCTURE: the committed learned window at storm-range conditions,
on CPU.

Seeded site-directions and conditions as the network was trained on
(train_window.build_samples: uniform sites, vertical or 30 deg zenith, Pdyn,
Dst, By, Bz over storm ranges, IGRF-14 + T96).  The committed weights
(cor-model_gb300/window_t96.npz) run through the numpy restatement of the
tensor-core forward pass (oracle/mlp_oracle.py); the oracle traces the
windows (with the edge-hit widening of window.trace_windows) and the full
0.01 GV scans.  Prints the share of site-directions whose R_C is within one
grid step (0.01 GV) of the full scan's, the largest difference, and the share
of the trajectories traced.  A few minutes per 100 samples on 8 threads.

    python oracle/window_agreement.py [--samples N] [--seed S]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [HERE, os.path.join(ROOT, "cor-model_gb300")]

import cortrace as ct  # noqa: E402
import mlp_oracle  # noqa: E402
import pyoracle  # noqa: E402
import train_window as tw  # noqa: E402
import window  # noqa: E402


class OracleCtx:
    def trace_batch(self, jobs, params, models=None, **kw):
        return pyoracle.scan_batch(jobs, params, models=models, threads=os.cpu_count() or 1)


def main(n: int, seed: int) -> dict:
    s = tw.build_samples(np.random.default_rng(seed), n, "t96")
    models = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96)
    d = np.load(os.path.join(ROOT, "cor-model_gb300", "window_t96.npz"))
    x = (s["features"] - d["feat_mean"]) / d["feat_std"]
    y = mlp_oracle.forward(d["params"], x)[0] * d["y_std"] + d["y_mean"]
    b = window.band_of(y[:, 1], d["band_edges"])
    i_lo, i_hi = window.window_indices(y[:, 0], y[:, 1], d["band_sigma"][b, 0], d["band_sigma"][b, 1])
    jobs = np.concatenate([ct.make_job(s["lat"][k], s["lon"][k], rig=window.GRID_RIG, rk=20.0,
                                       dele=window.GRID_DEL, r0=tw.R0, the1=s["dirs"][k][0], fi1=s["dirs"][k][1],
                                       param_index=k) for k in range(n)])
    t = time.perf_counter()
    full = OracleCtx().trace_batch(jobs, s["params"], models=models)
    t_full = time.perf_counter() - t
    t = time.perf_counter()
    got, redone, traced, steps = window.trace_windows(OracleCtx(), jobs, s["params"], models, i_lo, i_hi)
    t_win = time.perf_counter() - t
    d_rc = np.abs(got["r_cutoff"] - full.sites["r_cutoff"])
    return {"samples": n, "seed": seed, "within_0.01GV": float(np.mean(d_rc <= 0.01 + 1e-9)),
            "max_abs_dRc_GV": float(d_rc.max()), "widened": int(redone.sum()),
            "trajectories_frac": traced / int(full.counters["trajectories"]),
            "steps_frac": steps / int(full.counters["accepted_steps"]),
            "seconds_full": round(t_full, 1), "seconds_windows": round(t_win, 1)}


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=48)
    ap.add_argument("--seed", type=int, default=2024)
    a = ap.parse_args()
    print(json.dumps(main(a.samples, a.seed)))
