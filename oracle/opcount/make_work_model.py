"""TEST INFRASTRUCTURE: the algorithmic FP64 work of the rigidity scan.

Builds the op-counting oracle (the oracle's C sources compiled as C++ with
flop.hpp, which counts + - * / sqrt as one operation each and each libm
transcendental separately), runs it on a seeded sample of single-rigidity
scans of a workload, and writes the average work per accepted step (its
rejected RK trials included) to oracle/work_model_<name>.json.  A
transcendental is weighted TRANS_WEIGHT operations.

usage: python oracle/opcount/make_work_model.py [igrf_t96|igrf]
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
sys.path.insert(0, os.path.join(ROOT, "cor-model_gb300"))
import cortrace as ct  # noqa: E402

TRANS_WEIGHT = 20
EXE = os.path.join(HERE, "count_ops")

WORKLOADS = {
    # name: (time, parmod, models, rig grid (rig, rk, del))
    "igrf_t96": ([2020, 6, 21, 173, 12, 0, 0], [2.0, -20.0, 0.0, -1.0], (1, 1, 0), (0.01, 20.0, 0.01)),
    "igrf": ([2020, 1, 1, 1, 0, 0, 0], None, (1, 0, 0), (0.05, 20.0, 0.05)),
}


def build() -> str:
    srcs = [os.path.join(ORACLE, f) for f in sorted(os.listdir(ORACLE)) if f.endswith(".c")]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include", os.path.join(HERE, "flop.hpp"),
           "-x", "c++", *srcs, "-x", "none", os.path.join(HERE, "count_main.cpp"), "-o", EXE, "-lpthread"]
    subprocess.run(cmd, check=True)
    return EXE


def sample_jobs(grid, seed=2024, n_lon=3, n_rig=10) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rig0, rk, d = grid
    n = int(round((rk - rig0) / d)) + 1
    jobs = []
    for lat in range(-90, 91, 5):
        for lon in rng.choice(np.arange(0, 360, 5), n_lon, replace=False):
            for i in rng.choice(n, n_rig, replace=False):
                r = rig0 + int(i) * d
                jobs.append(ct.make_job(float(lat), float(lon), rig=r, rk=r, dele=d))
    return np.concatenate(jobs)


def main(name: str) -> dict:
    time7, parmod, (mi, me, mc), grid = WORKLOADS[name]
    build()
    jobs = sample_jobs(grid)
    p = ct.internal_setup("igrf14", time7, parmod=parmod)
    with tempfile.TemporaryDirectory() as td:
        fj, fp = os.path.join(td, "jobs.bin"), os.path.join(td, "params.bin")
        jobs.tofile(fj)
        p.tofile(fp)
        out = subprocess.run([EXE, fj, fp, str(mi), str(me), str(mc)], capture_output=True, text=True, check=True)
    c = json.loads(out.stdout)
    flops = c["ops"] + TRANS_WEIGHT * c["transcendentals"]
    model = {
        "workload": name, "sample_scans": c["scans"], "accepted_steps": c["accepted_steps"],
        "trials": c["trials"], "ops": c["ops"], "transcendentals": c["transcendentals"],
        "transcendental_weight": TRANS_WEIGHT,
        "flops_per_step": flops / c["accepted_steps"],
        "flops_per_rejected_trial": 0.0,
        "trials_per_step": c["trials"] / c["accepted_steps"],
        "per_step_by_class": {k: v / c["accepted_steps"] for k, v in c["by_class"].items()},
        "source": "op-counting build of the oracle on a seeded sample (rejected trials included per step)",
    }
    with open(os.path.join(ORACLE, f"work_model_{name}.json"), "w") as f:
        json.dump(model, f, indent=1)
    return model


if __name__ == "__main__":
    print(json.dumps(main(sys.argv[1] if len(sys.argv) > 1 else "igrf_t96"), indent=1))
