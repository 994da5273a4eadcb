"""TEST INFRASTRUCTURE, not part of the product: Python access to the CPU
restatement in oracle/liboracle.so (the checker) and, where it has been built
in this tree, to the reference itself in oracle/_ref/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "cor-model_gb300"))
sys.path.insert(0, HERE)

import cortrace as ct  # noqa: E402  (dtype and struct layouts of include/cor_trace.h)
import build as obuild  # noqa: E402

_lib = None
_load_lock = __import__("threading").Lock()


def load() -> C.CDLL:
    global _lib
    with _load_lock:          # one build at a time when several threads load it first
        return _load()


def _load() -> C.CDLL:
    global _lib
    if _lib is None:
        path = obuild.build_port()
        lib = C.CDLL(path)
        vp, dbl, i32 = C.c_void_p, C.c_double, C.c_int32
        lib.orc_internal_geo.argtypes = [dbl, dbl, dbl, vp, vp, vp, vp, vp, vp]
        lib.orc_t96_gsm.argtypes = [vp, dbl, dbl, dbl, vp, vp, vp]
        lib.orc_ts05_gsm.argtypes = [vp, dbl, dbl, dbl, vp, vp, vp]
        lib.orc_chaos_geo.argtypes = [dbl, dbl, dbl, vp, vp, C.c_int, vp, vp, vp]
        lib.orc_calculate_field.argtypes = [vp, ct.ModelSet, vp, vp]
        lib.orc_rk_step.argtypes = [dbl, dbl, vp, vp, vp]
        lib.orc_set_crustal_table.argtypes = [vp, vp, C.c_int]
        lib.orc_scan_job.argtypes = [vp, vp, ct.ModelSet, C.c_uint64, dbl, dbl, vp, vp, vp, vp]
        lib.orc_scan_batch.argtypes = [C.POINTER(ct.BatchReq), vp, C.c_int, vp, vp, vp, vp]
        lib.orc_trace_steps.argtypes = [vp, vp, ct.ModelSet, C.c_uint64, dbl, dbl, vp, C.c_uint32, vp]
        lib.orc_internal_geo_flops.argtypes = [dbl]
        lib.orc_internal_geo_flops.restype = C.c_int64
        _lib = lib
    return _lib


_nudge = None


def load_nudge() -> C.CDLL:
    """The oracle built with every libm transcendental moved by one ulp."""
    global _nudge
    if _nudge is None:
        lib = C.CDLL(obuild.build_nudge())
        vp, dbl = C.c_void_p, C.c_double
        lib.orc_ts05_gsm.argtypes = [vp, dbl, dbl, dbl, vp, vp, vp]
        lib.orc_t96_gsm.argtypes = [vp, dbl, dbl, dbl, vp, vp, vp]
        lib.orc_scan_batch.argtypes = [C.POINTER(ct.BatchReq), vp, C.c_int, vp, vp, vp, vp]
        lib.orc_nudge_seed.argtypes = [C.c_uint64]
        lib.orc_chaos_geo.argtypes = [dbl, dbl, dbl, vp, vp, C.c_int, vp, vp, vp]
        lib.orc_set_crustal_table.argtypes = [vp, vp, C.c_int]
        lib.orc_calculate_field.argtypes = [vp, ct.ModelSet, vp, vp]
        _nudge = lib
    return _nudge


def scan_batch_nudged(jobs, params, models, seed: int, threads=8, step_limit=25000):
    """orc_scan_batch of the one-ulp-perturbed oracle (each thread reseeds
    from `seed` and the job order, so the result is reproducible only per
    job; the statistics, not the bits, are what matter)."""
    lib = load_nudge()
    jobs = np.ascontiguousarray(jobs, ct.JOB_DTYPE)
    params = np.ascontiguousarray(params, ct.PARAMS_DTYPE)
    n, off = batch_offsets(jobs)
    sites = np.zeros(len(jobs), ct.SITE_DTYPE)
    status = np.zeros(n, np.uint8)
    req = ct.BatchReq(_p(jobs), len(jobs), len(params), _p(params), models, step_limit, 0.01, ct.DEF_HM0_P)
    cnt = ct.Counters()
    _crustal(lib, models)
    lib.orc_nudge_seed(seed)
    rc = lib.orc_scan_batch(C.byref(req), _p(off), threads, _p(sites), _p(status), None, C.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"nudged scan failed: {rc}")
    return ct.ScanResult(sites, status, None, off, cnt.as_dict())


def calculate_field_nudged(gsm_m: np.ndarray, params: np.ndarray, models) -> np.ndarray:
    """calculate_field of the one-ulp-perturbed oracle (seed it first)."""
    return calculate_field(gsm_m, params, models, lib=load_nudge())


def _p(a):
    return None if a is None else a.ctypes.data


_crust_keep = {}


def _crustal(lib, models) -> None:
    """Give `lib` the dense CHAOS-7.16 table when `models` has the crustal model."""
    if models is None or models.crustal_model == ct.CRUSTAL_NONE or id(lib) in _crust_keep:
        return
    G, H, nmax = ct.chaos_dense()
    _crust_keep[id(lib)] = (G, H)
    lib.orc_set_crustal_table(G.ctypes.data, H.ctypes.data, nmax)


def internal_geo(xyz: np.ndarray, params: np.ndarray) -> np.ndarray:
    lib = load()
    xyz = np.asarray(xyz, np.float64).reshape(-1, 3)
    p = np.ascontiguousarray(params, ct.PARAMS_DTYPE).reshape(-1)[0]
    g, h, rec = (np.ascontiguousarray(p[k]) for k in ("g", "h", "rec"))
    out = np.zeros_like(xyz)
    b = np.zeros(3)
    for i, (x, y, z) in enumerate(xyz):
        lib.orc_internal_geo(x, y, z, _p(g), _p(h), _p(rec), _p(b[0:]), b[1:].ctypes.data, b[2:].ctypes.data)
        out[i] = b
    return out


def calculate_field(gsm_m: np.ndarray, params: np.ndarray, models=None, lib=None) -> np.ndarray:
    lib = lib or load()
    pos = np.asarray(gsm_m, np.float64).reshape(-1, 3)
    p = np.ascontiguousarray(params, ct.PARAMS_DTYPE).reshape(-1)[:1]
    out = np.zeros_like(pos)
    m = models or ct.model_set()
    _crustal(lib, m)
    for i in range(len(pos)):
        x = np.ascontiguousarray(pos[i])
        o = np.zeros(3)
        lib.orc_calculate_field(_p(x), m, _p(p), _p(o))
        out[i] = o
    return out


def batch_offsets(jobs: np.ndarray) -> tuple[int, np.ndarray]:
    """Trajectories per scan, as src/trajectory.c:7,12 counts them
    ((int)round((rk-rig)/del) + 1, C's round: half away from zero), or a
    window's i_count; the exclusive prefix.  Computed here so that the oracle
    needs nothing from the product library."""
    x = (jobs["rk"] - jobs["rig"]) / jobs["del"]
    n_grid = (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64) + 1
    n = np.where(jobs["i_count"] > 0, jobs["i_count"], n_grid - jobs["i_first"]).astype(np.uint64)
    off = np.zeros(len(jobs) + 1, np.uint64)
    off[1:] = np.cumsum(n)
    return int(off[-1]), off


def scan_batch(jobs: np.ndarray, params: np.ndarray, models=None, step_limit=25000, tu_angle=0.01,
               particle_mass=ct.DEF_HM0_P, threads=1, want_records=False):
    """orc_scan_batch over `threads` host threads -> ScanResult like the product's."""
    lib = load()
    jobs = np.ascontiguousarray(jobs, ct.JOB_DTYPE)
    params = np.ascontiguousarray(params, ct.PARAMS_DTYPE)
    n, off = batch_offsets(jobs)
    sites = np.zeros(len(jobs), ct.SITE_DTYPE)
    status = np.zeros(n, np.uint8)
    records = np.zeros(n, ct.RECORD_DTYPE) if want_records else None
    req = ct.BatchReq(_p(jobs), len(jobs), len(params), _p(params), models or ct.model_set(), step_limit,
                      tu_angle, particle_mass)
    cnt = ct.Counters()
    _crustal(lib, req.models)
    rc = lib.orc_scan_batch(C.byref(req), _p(off), threads, _p(sites), _p(status), _p(records), C.byref(cnt))
    if rc != 0:
        raise RuntimeError(f"oracle scan failed: {rc}")
    return ct.ScanResult(sites, status, records, off, cnt.as_dict())


STEP_DTYPE = ct.STEP_DTYPE


def trace_steps(job: np.ndarray, params: np.ndarray, models=None, step_limit=25000, tu_angle=0.01,
                particle_mass=ct.DEF_HM0_P, cap=25000) -> np.ndarray:
    """Every accepted step of the job's first traced rigidity (cor_step_record)."""
    lib = load()
    job = np.ascontiguousarray(job, ct.JOB_DTYPE)
    params = np.ascontiguousarray(params, ct.PARAMS_DTYPE)
    out = np.zeros(cap, STEP_DTYPE)
    m = models or ct.model_set()
    _crustal(lib, m)
    n = lib.orc_trace_steps(_p(job), _p(params), m, step_limit, tu_angle, particle_mass, _p(out), cap, None)
    if n < 0:
        raise RuntimeError(f"oracle trajectory failed: {n}")
    return out[:n]


def internal_geo_flops(R: float) -> int:
    return int(load().orc_internal_geo_flops(R))


# ---- the reference itself (only where oracle/_ref was built here) --------
REF_DIR = os.path.join(HERE, "_ref")


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "cor")) and os.path.exists(os.path.join(REF_DIR, "libcorref.so"))


def run_ref_cor(infile_text: str, args: list[str], parallel: bool = True) -> str:
    """Run the reference `cor` binary on one INFILE; returns its text output."""
    import tempfile
    with tempfile.NamedTemporaryFile("w", suffix=".in", delete=False) as f:
        f.write(infile_text)
        path = f.name
    try:
        cmd = [os.path.join(REF_DIR, "cor"), *(["-p"] if parallel else []), *args, path]
        res = subprocess.run(cmd, capture_output=True, text=True, check=True)
        return res.stdout
    finally:
        os.unlink(path)
