"""TEST INFRASTRUCTURE: how much of one accepted step could run at once.

Builds the depth-tracking oracle (the oracle's C sources compiled as C++ with
depth.hpp), runs it on the seeded sample of single-rigidity scans that
make_work_model.py uses, and reports per accepted step:
  * issue     -- FP64 instructions (add/mul 1, division 9, square root 10, a
                 C-library function 20), rejected RK trials included;
  * critical  -- the longest chain of dependent operations, in units of one
                 dependent FP64 add/mul latency (division 562/64, square root
                 678/64, a C-library function 20), branches included;
  * issue / critical -- the operations one step offers at once on average: how
                 far splitting a lone trajectory's step over the lanes of its
                 warp could shorten it.
Both over all trajectories and over the long ones (>= 5,000 accepted steps),
which set a batch's tail.

usage: python oracle/opcount/critical_path.py [igrf|igrf_t96|igrf_ts05 ...]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
ROOT = os.path.dirname(ORACLE)
sys.path[:0] = [HERE, os.path.join(ROOT, "cor-model_gb300")]
import cortrace as ct  # noqa: E402
from make_work_model import WORKLOADS, sample_jobs  # noqa: E402

EXE = os.path.join(HERE, "count_depth")
LOADS = dict(WORKLOADS)
LOADS["igrf_ts05"] = ([2020, 6, 21, 173, 12, 0, 0], [2.0, -20.0, 0.0, -1.0, 1, 1, 1, 1, 1, 1], (1, 2, 0),
                      (0.01, 20.0, 0.01))
LONG = 5000


def build() -> str:
    srcs = [os.path.join(ORACLE, f) for f in sorted(os.listdir(ORACLE)) if f.endswith(".c")]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include", os.path.join(HERE, "depth.hpp"),
           "-x", "c++", *srcs, "-x", "none", os.path.join(HERE, "depth_main.cpp"), "-o", EXE, "-lpthread"]
    subprocess.run(cmd, check=True)
    return EXE


def run(name: str, n_rig: int = 4) -> dict:
    time7, parmod, (mi, me, mc), grid = LOADS[name]
    jobs = sample_jobs(grid, n_rig=n_rig)
    p = ct.internal_setup("igrf14", time7, parmod=parmod)
    with tempfile.TemporaryDirectory() as td:
        fj, fp = os.path.join(td, "jobs.bin"), os.path.join(td, "params.bin")
        jobs.tofile(fj)
        p.tofile(fp)
        out = subprocess.run([EXE, fj, fp, str(mi), str(me), str(mc)], capture_output=True, text=True, check=True)
    rows = [json.loads(ln) for ln in out.stdout.splitlines() if ln.startswith("{")]
    steps = np.array([r["steps"] for r in rows], float)
    issue = np.array([r["issue"] for r in rows])
    crit = np.array([r["critical"] for r in rows])

    def agg(m):
        s = steps[m].sum()
        return {"trajectories": int(m.sum()), "accepted_steps": int(s), "issue_per_step": issue[m].sum() / s,
                "critical_per_step": crit[m].sum() / s, "issue_over_critical": issue[m].sum() / crit[m].sum()}
    return {"workload": name, "all": agg(steps > 0), f"steps>={LONG}": agg(steps >= LONG)}


if __name__ == "__main__":
    build()
    for name in sys.argv[1:] or ["igrf", "igrf_t96", "igrf_ts05"]:
        print(json.dumps(run(name)), flush=True)
