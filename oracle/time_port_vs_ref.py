"""TEST INFRASTRUCTURE: single-thread CPU time of the reference's own `cor`
(compiled from its sources into oracle/_ref/ by oracle/build.py) against the
oracle port, on the same sites of the benchmark workload (IGRF-14 + T96,
2020-06-21 12:00 UT, Pdyn 2 nPa, Dst -20 nT, By 0, Bz -1 nT; vertical incidence
from 20 km; 0.01 -> 20 GV by 0.01).  It shows how far the port, which stands in
for the reference on hosts where the reference cannot be built, is from the
reference's own speed, and that both print the same cutoffs.

    python oracle/time_port_vs_ref.py [LAT,LON ...]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [HERE, os.path.join(ROOT, "cor-model_gb300")]

import cortrace as ct  # noqa: E402
import pyoracle  # noqa: E402

TIME7 = [2020, 6, 21, 173, 12, 0, 0]
PARMOD = [2.0, -20.0, 0.0, -1.0]
R0 = 1.0031391260673028


def infile_text(lat: float, lon: float) -> str:
    """A `cor -m cutoff` INFILE (src/io.c:4-20 layout) with the T96 line."""
    return (f"0.01 1 20.0\n{R0!r} {lat!r} {lon!r}\n{lat!r} {lon!r}\n{' '.join(map(str, TIME7))}\n"
            f"100 0 0 0.01\n{PARMOD[1]!r} {PARMOD[0]!r} {PARMOD[2]!r} {PARMOD[3]!r}\n")


def main(sites):
    cor = os.path.join(HERE, "_ref", "cor")
    if not os.path.exists(cor):
        sys.exit("oracle/_ref/cor is not built (oracle/build.py build_ref)")
    p = ct.internal_setup("igrf14", TIME7, parmod=PARMOD)
    models = ct.model_set(ct.INTERNAL_SH, ct.EXTERNAL_T96)
    t_ref = t_port = 0.0
    steps = 0
    for lat, lon in sites:
        with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False) as f:
            f.write(infile_text(lat, lon))
            path = f.name
        try:
            t = time.perf_counter()
            out = subprocess.run([cor, "-m", "cutoff", "-i", "igrf14", "-e", "t96", path], capture_output=True,
                                 text=True, check=True, env=dict(os.environ, OMP_NUM_THREADS="1")).stdout
            dr = time.perf_counter() - t
        finally:
            os.unlink(path)
        lines = out.splitlines()
        k = next(i for i, ln in enumerate(lines) if ln.startswith("  CUTOFF"))
        ref_cut = [float(v) for v in lines[k + 1].split()[:3]]
        jobs = ct.make_job(lat, lon, rig=0.01, rk=20.0, dele=0.01, r0=R0)
        t = time.perf_counter()
        res = pyoracle.scan_batch(jobs, p, models=models, threads=1)
        dp = time.perf_counter() - t
        port_cut = [round(float(res.sites[0][f]), 5) for f in ("r_lower", "r_upper", "r_cutoff")]
        steps += int(res.counters["accepted_steps"])
        print(f"site {lat:g},{lon:g}: reference {dr:.2f} s, port {dp:.2f} s; cutoffs reference {ref_cut} "
              f"port {port_cut}{'' if ref_cut == port_cut else '  DIFFER'}", flush=True)
        t_ref += dr
        t_port += dp
    print(f"{len(sites)} sites, {steps} accepted steps: reference {t_ref:.2f} s, port {t_port:.2f} s, "
          f"port time / reference time {t_port / t_ref:.3f}")


if __name__ == "__main__":
    arg = [tuple(float(v) for v in a.split(",")) for a in sys.argv[1:]]
    main(arg or [(60.0, 0.0), (30.0, 90.0), (0.0, 180.0), (-45.0, 270.0)])
