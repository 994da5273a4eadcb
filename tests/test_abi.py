"""CPU tests of the C ABI: the library loads, exports every function that
include/cor_trace.h declares, and its host-only entry points behave."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT
import cortrace as ct


def header_functions() -> list[str]:
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(cor_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_function():
    lib = ct.load()
    declared = header_functions()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(lib, name), name
    assert set(ct.EXPORTS) <= set(declared)


def test_abi_version():
    assert ct.load().cor_abi_version() == ct.ABI_VERSION == 3


def test_batch_count_matches_reference_grid():
    # src/trajectory.c:7,12: i = 0 .. round((rk - rig)/del)
    jobs = np.concatenate([ct.make_job(0, 0, rig=0.05, rk=20.0, dele=0.05),
                           ct.make_job(0, 0, rig=0.01, rk=20.0, dele=0.01),
                           ct.make_job(0, 0, rig=5.0, rk=5.0, dele=0.1)])
    n, off = ct.batch_offsets(jobs)
    assert off.tolist() == [0, 400, 2400, 2401] and n == 2401


def test_batch_count_rejects_bad_grid():
    with pytest.raises(ct.CorError):
        ct.batch_offsets(ct.make_job(0, 0, dele=0.0))
    with pytest.raises(ct.CorError):
        ct.batch_offsets(ct.make_job(0, 0, rig=20.0, rk=0.05, dele=0.05))


def test_batch_count_rejects_jobs_the_step_loop_cannot_run():
    """nk1 <= 0 (the turn-angle halving doubles nk0 while nk0 <= 50000), a
    zero charge and non-finite start values are rejected before any device
    work; negative charges are valid."""
    for bad in (dict(nk1=0), dict(nk1=-100), dict(zn=0.0), dict(zn=float("nan")), dict(r0=float("inf"))):
        with pytest.raises(ct.CorError):
            ct.batch_offsets(ct.make_job(50.0, 15.0, **bad))
    j = ct.make_job(50.0, 15.0)
    j["the1"] = float("nan")
    with pytest.raises(ct.CorError):
        ct.batch_offsets(j)
    n, _ = ct.batch_offsets(ct.make_job(50.0, 15.0, zn=-1.0, nk1=1))
    assert n == 400


def test_prepare_trig_uses_host_libm():
    j = ct.make_job(50.0, 15.0)
    t = ct.prepare_trig(j)[0]
    th = (90.0 - 50.0) * (ct.DEF_PI / 180.0)
    assert t["st0"] == np.sin(th) and t["cp0"] == np.cos(15.0 * (ct.DEF_PI / 180.0))


def test_context_without_gpu_reports_nodev():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = ct.load()
    h = C.c_void_p()
    assert lib.cor_ctx_create(0, C.byref(h)) == -5


def test_batch_count_windows():
    # a window of the 0.01 GV grid: indices 100..199 (rigidities 1.01..2.00 GV)
    full = ct.make_job(0, 0, rig=0.01, rk=20.0, dele=0.01)
    win = ct.make_job(0, 0, rig=0.01, rk=20.0, dele=0.01, i_first=100, i_last=199)
    tail = ct.make_job(0, 0, rig=0.01, rk=20.0, dele=0.01, i_first=1990)
    n, off = ct.batch_offsets(np.concatenate([full, win, tail]))
    assert off.tolist() == [0, 2000, 2100, 2110] and n == 2110
    for bad in (dict(i_first=2000), dict(i_first=1990, i_last=2000), dict(i_first=-1)):
        with pytest.raises(ct.CorError):
            ct.batch_offsets(ct.make_job(0, 0, rig=0.01, rk=20.0, dele=0.01, **bad))


def test_regroup_and_steps_reject_null_context():
    lib = ct.load()
    assert lib.cor_ctx_set_regroup(None, 16, 48, 256) == -1
    assert lib.cor_trace_steps(None, None, None, None, 0) == -1


def test_binding_takes_strided_job_views_by_value():
    """The host helpers read whole job rows from the address they get: a
    strided or reversed view is copied to a contiguous array first, so every
    row is the one the caller meant, and a raw strided pointer is refused."""
    jobs = np.concatenate([ct.make_job(float(lat), float(lon), rig=1.0, rk=3.0 + lat / 90.0, dele=0.5)
                           for lat in (-60, -20, 0, 30, 70) for lon in (10, 200)])
    for view in (jobs[1::3], jobs[::-1], jobs[::2]):
        assert not view.flags.c_contiguous
        copy = view.copy()
        assert np.array_equal(ct.prepare_trig(view).view(np.uint8), ct.prepare_trig(copy).view(np.uint8))
        n_view, off_view = ct.batch_offsets(view)
        n_copy, off_copy = ct.batch_offsets(copy)
        assert n_view == n_copy and np.array_equal(off_view, off_copy)
    with pytest.raises(ValueError):
        ct._ptr(jobs[::2])
