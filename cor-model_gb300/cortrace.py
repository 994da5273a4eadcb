"""Python binding of libcortrace.so through its C ABI (include/cor_trace.h).

The structured numpy dtypes below have the exact C layouts of the header's
structs, so arrays of jobs, parameter blocks, records and site results pass
to the library as plain pointers.  Loading fails loudly when the library has
not been built: there is no fallback implementation behind this module.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcortrace.so")

COR_OK = 0
ERRORS = {-1: "invalid", -2: "nomem", -3: "cuda", -4: "watchdog", -5: "nodev", -6: "unsupported", -7: "range",
          -8: "busy"}
COR_PENDING = 1
ERR_BUSY = -8

INTERNAL_NONE, INTERNAL_SH = 0, 1
EXTERNAL_NONE, EXTERNAL_T96, EXTERNAL_TS05 = 0, 1, 2
CRUSTAL_NONE, CRUSTAL_CHAOS = 0, 1

FLAG_UNIFORM_GRID = 1

TRAJ_NONE, TRAJ_ALLOWED, TRAJ_REENTRY, TRAJ_SUPERLUM, TRAJ_STEP_LIMIT, TRAJ_WATCHDOG = range(6)

# Physical constants of the reference (src/common.h:4-11).
DEF_PI = 3.141592654
DEF_RE = 6.3712e+06
DEF_C = 2.99725e+08
DEF_HM0_P = 1.6725e-27
DEF_HM0_E = 9.1093826e-31

SH = 105

JOB_DTYPE = np.dtype([
    ("r0", "f8"), ("the0", "f8"), ("fi0", "f8"), ("the1", "f8"), ("fi1", "f8"),
    ("rig", "f8"), ("del", "f8"), ("rk", "f8"), ("zn", "f8"),
    ("nk1", "i4"), ("param_index", "i4"), ("i_first", "i4"), ("i_count", "i4")], align=True)
PARAMS_DTYPE = np.dtype([
    ("parmod", "f8", (10,)), ("g", "f8", (SH,)), ("h", "f8", (SH,)), ("rec", "f8", (SH,)),
    ("a1", "f8", (3,)), ("a2", "f8", (3,)), ("a3", "f8", (3,))], align=True)
RECORD_DTYPE = np.dtype([
    ("pos", "f8", (3,)), ("vel", "f8", (3,)), ("v", "f8"), ("time", "f8"), ("length", "f8"),
    ("steps", "u4"), ("trials", "u4"), ("status", "i4"), ("reserved", "i4")], align=True)
SITE_DTYPE = np.dtype([
    ("r_lower", "f8"), ("r_upper", "f8"), ("r_cutoff", "f8"),
    ("n_forbidden", "i4"), ("n_traj", "i4")], align=True)
SCAN_EVENT_DTYPE = np.dtype([("site", SITE_DTYPE), ("first_class", "u1"), ("last_class", "u1"),
                             ("reserved", "u2"), ("reserved2", "u4"), ("seq1", "u8")], align=True)
TRIG_DTYPE = np.dtype([(k, "f8") for k in ("st0", "ct0", "sp0", "cp0", "st1", "ct1", "sp1", "cp1")], align=True)

STEP_DTYPE = np.dtype([("gsm", "f8", 3), ("pos", "f8", 3), ("v", "f8"), ("time", "f8"), ("length", "f8"),
                       ("step", "u4"), ("reserved", "u4")], align=True)
assert JOB_DTYPE.itemsize == 88 and PARAMS_DTYPE.itemsize == 2672 and STEP_DTYPE.itemsize == 80
assert RECORD_DTYPE.itemsize == 88 and SITE_DTYPE.itemsize == 32 and SCAN_EVENT_DTYPE.itemsize == 48


class ModelSet(C.Structure):
    _fields_ = [("internal_model", C.c_int32), ("external_model", C.c_int32),
                ("crustal_model", C.c_int32), ("reserved", C.c_int32)]


class Counters(C.Structure):
    _fields_ = [("accepted_steps", C.c_uint64), ("trials", C.c_uint64), ("trajectories", C.c_uint64),
                ("watchdog", C.c_uint64), ("kernel_launches", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class BatchReq(C.Structure):
    _fields_ = [("jobs", C.c_void_p), ("n_jobs", C.c_int32), ("n_params", C.c_int32), ("params", C.c_void_p),
                ("models", ModelSet), ("step_limit", C.c_uint64), ("tu_angle", C.c_double),
                ("particle_mass", C.c_double)]


class StreamConfig(C.Structure):
    """cor_stream_config (include/cor_trace.h)."""
    _fields_ = [("slots", C.c_int32), ("max_jobs", C.c_int32), ("max_trajectories", C.c_int64),
                ("max_params", C.c_int32), ("want_records", C.c_int32), ("reserve_sms", C.c_int32),
                ("fixed_params", C.c_int32), ("pool_params", C.c_int32), ("segments_per_launch", C.c_int32),
                ("idle_limit_s", C.c_double), ("launch_on_drain", C.c_int32), ("scan_events", C.c_int32),
                ("sort_lanes", C.c_int32)]


class BatchResult(C.Structure):
    _fields_ = [("sites", C.c_void_p), ("status", C.c_void_p), ("records", C.c_void_p), ("counters", Counters)]


# Every symbol the header declares (checked by the CPU test suite).
EXPORTS = [
    "cor_ctx_create", "cor_ctx_destroy", "cor_last_error_string", "cor_abi_version", "cor_batch_count",
    "cor_prepare_trig", "cor_trace_batch", "cor_trace_batch_device", "cor_upload_params", "cor_field_batch",
    "cor_internal_setup", "cor_gsm_setup", "cor_probe_fp64_peak", "cor_probe_fp64_functions",
    "cor_upload_crustal",
    "cor_trace_batch_device_noalloc", "cor_ctx_set_regroup", "cor_trace_steps", "cor_ctx_set_queue_order",
    "cor_ctx_set_lane_sort",
    "cor_ctx_generation_log", "cor_stream_config_default", "cor_stream_create", "cor_stream_submit",
    "cor_stream_upload_params", "cor_stream_submit_device", "cor_stream_wait", "cor_stream_drain",
    "cor_stream_poll_scans",
    "cor_stream_close",
]
NOALLOC_MAX_TRAJ = 1048576  # COR_NOALLOC_MAX_TRAJ
ABI_VERSION = 3  # COR_TRACE_ABI_VERSION: the structure layouts above

_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libcortrace.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libcortrace.so is not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    vp, i32, i64, u64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_uint64, C.c_double
    lib.cor_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    lib.cor_ctx_destroy.argtypes = [vp]
    lib.cor_last_error_string.argtypes = [vp]
    lib.cor_last_error_string.restype = C.c_char_p
    lib.cor_abi_version.restype = C.c_int
    if lib.cor_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path} has ABI version {lib.cor_abi_version()}, this binding needs {ABI_VERSION}: "
                           "rebuild it with __graft_entry__.build()")
    lib.cor_batch_count.argtypes = [vp, i32, C.POINTER(u64), vp]
    lib.cor_prepare_trig.argtypes = [vp, i32, vp]
    lib.cor_trace_batch.argtypes = [vp, C.POINTER(BatchReq), C.POINTER(BatchResult)]
    lib.cor_trace_batch_device.argtypes = [vp, vp, vp, i32, vp, u64, ModelSet, u64, dbl, dbl,
                                           vp, vp, vp, vp, C.c_uint32, vp]
    lib.cor_upload_params.argtypes = [vp, vp, i32]
    lib.cor_upload_crustal.argtypes = [vp, vp, vp, i32]
    lib.cor_ctx_set_regroup.argtypes = [vp, i32, i32, i64]
    lib.cor_ctx_set_queue_order.argtypes = [vp, i32]
    lib.cor_ctx_set_lane_sort.argtypes = [vp, i32]
    lib.cor_ctx_generation_log.argtypes = [vp, i32, vp, vp]
    lib.cor_ctx_generation_log.restype = i32
    lib.cor_trace_steps.argtypes = [vp, C.POINTER(BatchReq), C.POINTER(BatchResult), vp, C.c_uint32]
    lib.cor_trace_batch_device_noalloc.argtypes = [vp, vp, vp, i32, vp, u64, ModelSet, u64, dbl, dbl,
                                                   vp, vp, vp, C.c_uint32, vp]
    lib.cor_probe_fp64_peak.argtypes = [vp, C.POINTER(C.c_double)]
    lib.cor_probe_fp64_functions.argtypes = [vp, vp]
    lib.cor_field_batch.argtypes = [vp, ModelSet, vp, i32, vp, vp, i64, vp]
    lib.cor_internal_setup.argtypes = [C.c_char_p, vp, vp]
    lib.cor_gsm_setup.argtypes = [vp, vp]
    lib.cor_stream_config_default.argtypes = [C.POINTER(StreamConfig)]
    lib.cor_stream_config_default.restype = None
    lib.cor_stream_create.argtypes = [vp, ModelSet, u64, dbl, dbl, C.POINTER(StreamConfig), C.POINTER(vp)]
    lib.cor_stream_submit.argtypes = [vp, vp, i32, vp, i32, C.POINTER(i64)]
    lib.cor_stream_upload_params.argtypes = [vp, vp, i32, C.POINTER(i32)]
    lib.cor_stream_submit_device.argtypes = [vp, vp, vp, vp, vp, i32, vp, vp, vp, C.POINTER(i64)]
    lib.cor_stream_wait.argtypes = [vp, i64, i32, C.POINTER(BatchResult), C.POINTER(u64)]
    lib.cor_stream_drain.argtypes = [vp, C.POINTER(C.c_double)]
    lib.cor_stream_poll_scans.argtypes = [vp, i64, i32, i32, vp, vp]
    lib.cor_stream_close.argtypes = [vp]
    _lib = lib
    return lib


def _ptr(a: np.ndarray | None) -> int | None:
    """Address of a C-contiguous array for the C ABI, which reads whole rows
    from it: a strided view would hand C the wrong elements (or memory past
    the array), so it is refused."""
    if a is None:
        return None
    if not a.flags.c_contiguous:
        raise ValueError("the C ABI needs a contiguous array (np.ascontiguousarray)")
    return a.ctypes.data


class CorError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cor error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


def internal_setup(version: str, time7, parmod=None) -> np.ndarray:
    """internal_recalc for model `version` at time {iy, mes, ide, id, ih, min, is}."""
    lib = load()
    p = np.zeros(1, PARAMS_DTYPE)
    t = np.ascontiguousarray(time7, dtype=np.int32)
    rc = lib.cor_internal_setup(version.encode(), _ptr(t), _ptr(p))
    if rc != COR_OK:
        raise CorError(rc, f"internal set-up of {version} at {list(time7)}")
    if parmod is not None:
        p["parmod"][0, :len(parmod)] = parmod
    return p


def batch_offsets(jobs: np.ndarray) -> tuple[int, np.ndarray]:
    lib = load()
    jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
    off = np.zeros(len(jobs) + 1, np.uint64)
    n = C.c_uint64(0)
    rc = lib.cor_batch_count(_ptr(jobs), len(jobs), C.byref(n), _ptr(off))
    if rc != COR_OK:
        raise CorError(rc, "invalid job: rigidity grid or window, nk1 <= 0, zero charge or non-finite start")
    return int(n.value), off


def prepare_trig(jobs: np.ndarray) -> np.ndarray:
    lib = load()
    jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
    out = np.zeros(len(jobs), TRIG_DTYPE)
    rc = lib.cor_prepare_trig(_ptr(jobs), len(jobs), _ptr(out))
    if rc != COR_OK:
        raise CorError(rc, "trig")
    return out


@dataclass
class ScanResult:
    sites: np.ndarray
    status: np.ndarray | None
    records: np.ndarray | None
    offsets: np.ndarray
    counters: dict


def model_set(internal=INTERNAL_SH, external=EXTERNAL_NONE, crustal=CRUSTAL_NONE) -> ModelSet:
    return ModelSet(internal, external, crustal, 0)


class Context:
    """One libcortrace context bound to a CUDA device."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.cor_ctx_create(device, C.byref(h))
        if rc != COR_OK:
            raise CorError(rc, f"cannot create a context on device {device}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.cor_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self) -> str:
        s = self.lib.cor_last_error_string(self.h)
        return s.decode() if s else ""

    def _check(self, rc: int, what: str):
        if rc != COR_OK:
            raise CorError(rc, f"{what}: {self.error()}")

    def trace_batch(self, jobs: np.ndarray, params: np.ndarray, models: ModelSet | None = None,
                    step_limit: int = 25000, tu_angle: float = 0.01, particle_mass: float = DEF_HM0_P,
                    want_status: bool = True, want_records: bool = False) -> ScanResult:
        """cor_trace_batch: host buffers in, host buffers out."""
        jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
        params = np.ascontiguousarray(params, PARAMS_DTYPE)
        n, off = batch_offsets(jobs)
        sites = np.zeros(len(jobs), SITE_DTYPE)
        status = np.zeros(n, np.uint8) if want_status else None
        records = np.zeros(n, RECORD_DTYPE) if want_records else None
        req = BatchReq(_ptr(jobs), len(jobs), len(params), _ptr(params), models or model_set(),
                       step_limit, tu_angle, particle_mass)
        res = BatchResult(_ptr(sites), _ptr(status), _ptr(records), Counters())
        self._check(self.lib.cor_trace_batch(self.h, C.byref(req), C.byref(res)), "trace_batch")
        return ScanResult(sites, status, records, off, res.counters.as_dict())

    def trace_steps(self, jobs: np.ndarray, params: np.ndarray, models: ModelSet | None = None,
                    step_limit: int = 25000, tu_angle: float = 0.01, particle_mass: float = DEF_HM0_P,
                    capacity: int = 25000) -> tuple[ScanResult, list[np.ndarray]]:
        """cor_trace_steps: the scan's result and, per trajectory, its
        accepted steps (STEP_DTYPE records, at most `capacity`)."""
        jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
        params = np.ascontiguousarray(params, PARAMS_DTYPE)
        n, off = batch_offsets(jobs)
        sites = np.zeros(len(jobs), SITE_DTYPE)
        status = np.zeros(n, np.uint8)
        records = np.zeros(n, RECORD_DTYPE)
        steps = np.zeros(n * capacity, STEP_DTYPE)
        req = BatchReq(_ptr(jobs), len(jobs), len(params), _ptr(params), models or model_set(),
                       step_limit, tu_angle, particle_mass)
        res = BatchResult(_ptr(sites), _ptr(status), _ptr(records), Counters())
        self._check(self.lib.cor_trace_steps(self.h, C.byref(req), C.byref(res), _ptr(steps), capacity), "trace_steps")
        per = []
        for t in range(n):
            s = steps[t * capacity:(t + 1) * capacity]
            k = int(np.argmax(s["step"] != np.arange(1, capacity + 1))) if np.any(
                s["step"] != np.arange(1, capacity + 1)) else capacity
            per.append(s[:k].copy())
        return ScanResult(sites, status, records, off, res.counters.as_dict()), per

    def set_regroup(self, park_below: int = 16, max_generations: int = 48, min_park: int = 256) -> None:
        """cor_ctx_set_regroup: the scan kernel's regrouping knobs."""
        self._check(self.lib.cor_ctx_set_regroup(self.h, park_below, max_generations, min_park), "cor_ctx_set_regroup")

    def generation_log(self) -> list[tuple[int, float]]:
        """(live trajectories, wall ms) per kernel generation of the last scan."""
        live = np.zeros(1024, np.uint64)
        ms = np.zeros(1024)
        n = self.lib.cor_ctx_generation_log(self.h, 1024, live.ctypes.data, ms.ctypes.data)
        return [(int(live[k]), float(ms[k])) for k in range(max(0, n))]

    def set_queue_order(self, rigidity_major=True) -> None:
        """cor_ctx_set_queue_order: lowest rigidities first (True or 1), scan
        by scan (False or 0), or warp-wide chunks of one scan in ascending
        rigidity (2, streams)."""
        mode = int(rigidity_major) if not isinstance(rigidity_major, bool) else (1 if rigidity_major else 0)
        self._check(self.lib.cor_ctx_set_queue_order(self.h, mode), "cor_ctx_set_queue_order")

    def set_lane_sort(self, on: bool = True) -> None:
        """cor_ctx_set_lane_sort: regroup each block's trajectories by field
        band before every field evaluation (the default) or never."""
        self._check(self.lib.cor_ctx_set_lane_sort(self.h, 1 if on else 0), "cor_ctx_set_lane_sort")

    def upload_crustal(self, g: np.ndarray, h: np.ndarray, nmax: int) -> None:
        """cor_upload_crustal: packed lower-triangle G, H (index n(n+1)/2 + m)."""
        g = np.ascontiguousarray(g, np.float64)
        h = np.ascontiguousarray(h, np.float64)
        if len(g) < nmax * (nmax + 1) // 2 or len(h) < nmax * (nmax + 1) // 2:
            raise ValueError("crustal table shorter than nmax(nmax+1)/2")
        self._check(self.lib.cor_upload_crustal(self.h, g.ctypes.data, h.ctypes.data, nmax), "cor_upload_crustal")

    def field_batch(self, gsm_pos_m: np.ndarray, params: np.ndarray, models: ModelSet | None = None,
                    param_index: np.ndarray | None = None) -> np.ndarray:
        """cor_field_batch: calculate_field at GSM positions [m] -> GEO field [nT]."""
        pos = np.ascontiguousarray(gsm_pos_m, np.float64).reshape(-1, 3)
        params = np.ascontiguousarray(params, PARAMS_DTYPE)
        idx = None if param_index is None else np.ascontiguousarray(param_index, np.int32)
        out = np.zeros_like(pos)
        rc = self.lib.cor_field_batch(self.h, models or model_set(), _ptr(params), len(params), _ptr(idx),
                                      _ptr(pos), len(pos), _ptr(out))
        self._check(rc, "field_batch")
        return out


class Stream:
    """A persistent scan stream (cor_stream_*): one resident launch of the scan
    kernel that traces every submitted batch of scans as it arrives.  Results
    are those of Context.trace_batch, bit for bit."""

    def __init__(self, ctx: Context, models: ModelSet | None = None, step_limit: int = 25000,
                 tu_angle: float = 0.01, particle_mass: float = DEF_HM0_P, **cfg):
        self.ctx = ctx
        self.lib = ctx.lib
        c = StreamConfig()
        self.lib.cor_stream_config_default(C.byref(c))
        for k, v in cfg.items():
            if not hasattr(c, k):
                raise TypeError(f"unknown stream setting {k}")
            setattr(c, k, v)
        self.config = c
        h = C.c_void_p()
        ctx._check(self.lib.cor_stream_create(ctx.h, models or model_set(), step_limit, tu_angle, particle_mass,
                                              C.byref(c), C.byref(h)), "cor_stream_create")
        self.h = h
        self._pending: dict[int, tuple] = {}

    def submit(self, jobs: np.ndarray, params: np.ndarray, want_status: bool = True,
               want_records: bool = False) -> int:
        """cor_stream_submit: publishes a batch; returns its ticket."""
        if want_records and not self.config.want_records:
            raise ValueError("records need a stream created with want_records=1")
        jobs = np.ascontiguousarray(jobs, JOB_DTYPE)
        params = np.ascontiguousarray(params, PARAMS_DTYPE)
        n, off = batch_offsets(jobs) if len(jobs) else (0, np.zeros(1, np.uint64))
        t = C.c_int64(-1)
        self.ctx._check(self.lib.cor_stream_submit(self.h, _ptr(jobs), len(jobs), _ptr(params), len(params),
                                                   C.byref(t)), "cor_stream_submit")
        self._pending[t.value] = (len(jobs), n, off, want_status, want_records)
        return t.value

    def upload_params(self, params: np.ndarray) -> int:
        """cor_stream_upload_params: fixed pool index of params[0]."""
        params = np.ascontiguousarray(params, PARAMS_DTYPE)
        first = C.c_int32(-1)
        self.ctx._check(self.lib.cor_stream_upload_params(self.h, _ptr(params), len(params), C.byref(first)),
                        "cor_stream_upload_params")
        return first.value

    def submit_device(self, jobs_dev: int, trig_dev: int, offsets_dev: int, offsets_host: np.ndarray, n_jobs: int,
                      sites_dev: int, status_dev: int, records_dev: int | None = None) -> int:
        """cor_stream_submit_device: buffers already in device memory (pointers)."""
        offsets_host = np.ascontiguousarray(offsets_host, np.uint64)
        t = C.c_int64(-1)
        self.ctx._check(self.lib.cor_stream_submit_device(self.h, jobs_dev, trig_dev, offsets_dev,
                                                          _ptr(offsets_host), n_jobs, sites_dev, status_dev,
                                                          records_dev, C.byref(t)), "cor_stream_submit_device")
        self._pending[t.value] = None
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """cor_stream_wait: None while pending; else (ScanResult or None for a
        device segment, completion time [ns of the device clock])."""
        meta = self._pending.get(ticket, ())
        t_ns = C.c_uint64(0)
        if meta:
            n_jobs, n, off, want_status, want_records = meta
            sites = np.zeros(n_jobs, SITE_DTYPE)
            status = np.zeros(n, np.uint8) if want_status else None
            records = np.zeros(n, RECORD_DTYPE) if want_records else None
            res = BatchResult(_ptr(sites), _ptr(status), _ptr(records), Counters())
        else:
            res = BatchResult(None, None, None, Counters())
        rc = self.lib.cor_stream_wait(self.h, ticket, timeout_ms, C.byref(res), C.byref(t_ns))
        if rc == COR_PENDING:
            return None
        self.ctx._check(rc, "cor_stream_wait")
        self._pending.pop(ticket, None)
        if meta:
            return ScanResult(sites, status, records, off, res.counters.as_dict()), int(t_ns.value)
        return res.counters.as_dict(), int(t_ns.value)

    def poll_scans(self, ticket: int, first: int = 0, count: int | None = None):
        """cor_stream_poll_scans: (done flags, SCAN_EVENT_DTYPE records) of
        scans first .. first+count-1 of an outstanding segment."""
        if count is None:
            count = self._pending[ticket][0] - first
        done = np.zeros(count, np.uint8)
        ev = np.zeros(count, SCAN_EVENT_DTYPE)
        rc = self.lib.cor_stream_poll_scans(self.h, ticket, first, count, _ptr(done), _ptr(ev))
        if rc < 0:
            self.ctx._check(rc, "cor_stream_poll_scans")
        return done.astype(bool), ev

    def drain(self) -> float:
        """cor_stream_drain: ends the current launch once everything published
        has finished; returns its duration in ms (CUDA events on the kernel's
        stream)."""
        ms = C.c_double(0.0)
        self.ctx._check(self.lib.cor_stream_drain(self.h, C.byref(ms)), "cor_stream_drain")
        return ms.value

    def close(self):
        if getattr(self, "h", None):
            rc = self.lib.cor_stream_close(self.h)
            self.h = None
            self.ctx._check(rc, "cor_stream_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def make_job(lat, lon, rig=0.05, rk=20.0, dele=0.05, r0=1.0031391260673028, the1=None, fi1=None,
             zn=1.0, nk1=100, param_index=0, i_first=0, i_last=None) -> np.ndarray:
    """One scan (INFILE) as a JOB_DTYPE record; vertical incidence by default.
    i_first / i_last (inclusive) trace only a window of the scan's grid."""
    j = np.zeros(1, JOB_DTYPE)
    j["r0"], j["the0"], j["fi0"] = r0, lat, lon
    j["the1"] = lat if the1 is None else the1
    j["fi1"] = lon if fi1 is None else fi1
    j["rig"], j["del"], j["rk"], j["zn"] = rig, dele, rk, zn
    j["nk1"], j["param_index"] = nk1, param_index
    j["i_first"] = i_first
    j["i_count"] = 0 if i_last is None else i_last - i_first + 1
    return j


class _ChaosTable(C.Structure):
    _fields_ = [("version", C.c_char_p), ("name", C.c_char_p), ("nmax", C.c_int),
                ("g", C.POINTER(C.c_double)), ("h", C.POINTER(C.c_double))]


def chaos_table() -> tuple[np.ndarray, np.ndarray, int]:
    """The CHAOS-7.16 lithospheric table compiled into the library, as the
    packed lower triangles (index n*(n+1)/2 + m) of G and H."""
    lib = load()
    t = _ChaosTable.in_dll(lib, "cor_chaos716")
    n = t.nmax * (t.nmax + 1) // 2
    g = np.ctypeslib.as_array(t.g, shape=(n,)).copy()
    h = np.ctypeslib.as_array(t.h, shape=(n,)).copy()
    return g, h, int(t.nmax)


def chaos_dense() -> tuple[np.ndarray, np.ndarray, int]:
    """CHAOS G and H as dense nmax x nmax tables (zero above the diagonal)."""
    g, h, nmax = chaos_table()
    G = np.zeros((nmax, nmax))
    H = np.zeros((nmax, nmax))
    rows, cols = np.tril_indices(nmax)
    G[rows, cols] = g
    H[rows, cols] = h
    return G, H, nmax
