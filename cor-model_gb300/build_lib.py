"""In-tree build of libcortrace.so (CUDA kernels + C ABI + host set-up) and
of the drop-in `cor` command-line program, for sm_103a only.

Host C is compiled with -ffp-contract=off and the CUDA sources with
--fmad=false, matching the reference's -ffp-contract=off (CMakeLists.txt:17),
so IGRF-only scans are bit-identical to the reference's.  The model sets with
an external or crustal field (FMA_SOURCES) go through CUDA's own exp, log,
sin, cos and pow, which already differ from the C library's by ulps; their
units are compiled with FMA contraction (--fmad=true), which takes about a
fifth of their FP64 instructions, and are held to the reference's own
one-ulp spread instead of bit equality.
Translation units compile in parallel; a full build takes well under a
minute.  No make or cmake is needed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcortrace.so")
BIN_DIR = os.path.join(PKG, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "-Xptxas", "-warn-spills", f"-I{ROOT}/include"]
CC_FLAGS = ["-O2", "-std=gnu17", "-fPIC", "-ffp-contract=off", "-fno-math-errno", "-fno-trapping-math",
            f"-I{ROOT}/include", "-Wall"]

# Sources of the shared library.
CU_SOURCES = ["cortrace.cu", "inst_igrf.cu", "inst_igrf_t96.cu", "inst_t96.cu", "inst_igrf_ts05.cu",
              "inst_ts05.cu", "inst_crustal.cu", "mlp.cu"]
# Units compiled with FMA contraction (see the module docstring).
FMA_SOURCES = {"inst_igrf_t96.cu", "inst_t96.cu", "inst_igrf_ts05.cu", "inst_ts05.cu", "inst_crustal.cu"}
LIB_C_SOURCES = ["setup.c", "coef_tables.c"]
# Sources of the drop-in CLI (linked against the library).
CLI_C_SOURCES = ["cli_main.c", "cli_io.c", "cli_models.c", "cli_scan.c", "cli_field.c"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> str:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def _deps(paths: list[str]) -> list[str]:
    out = []
    for d in (CSRC, HOST, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out + paths


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu = [os.path.join(CSRC, f) for f in CU_SOURCES]
    cc = [os.path.join(HOST, f) for f in LIB_C_SOURCES]
    cli = [os.path.join(HOST, f) for f in CLI_C_SOURCES if os.path.exists(os.path.join(HOST, f))]
    jobs = []
    objs = []
    for s in cu:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, _deps([s])):
            flags = NVCC_FLAGS
            if os.path.basename(s) in FMA_SOURCES:
                flags = [f if f != "--fmad=false" else "--fmad=true" for f in NVCC_FLAGS]
            jobs.append([nvcc(), *ARCH, *flags, "-c", s, "-o", o])
    for s in cc:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _stale(o, _deps([s])):
            jobs.append(["gcc", *CC_FLAGS, "-c", s, "-o", o])
    cli_objs = []
    for s in cli:
        o = os.path.join(BUILD, os.path.basename(s) + ".o")
        cli_objs.append(o)
        if force or _stale(o, _deps([s])):
            jobs.append(["gcc", *CC_FLAGS, "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for lg in logs:
            if lg.strip():
                sys.stderr.write(lg)
    if force or _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lm"])
    if cli_objs:
        os.makedirs(BIN_DIR, exist_ok=True)
        exe = os.path.join(BIN_DIR, "cor")
        if force or _stale(exe, cli_objs + [LIB]):
            _run(["gcc", "-o", exe, *cli_objs, f"-L{PKG}", "-lcortrace", f"-Wl,-rpath,{PKG}", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
