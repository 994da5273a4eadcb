"""cor_trace_batch_device_noalloc against cor_trace_batch_device.

The file is named to be collected last: the no-allocation entry point must
give the existing device path's results both in a fresh process and after
every other test has used the library.  Two calls in a row (different
batches) check that the shared scratch array's leftover contents never leak
into a result."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cortrace as ct

pytestmark = pytest.mark.gpu

SEEN = ("accepted_steps", "trials", "trajectories", "watchdog")


def _batch(lats, lons, rig=0.05, rk=20.0, dele=0.05):
    return np.concatenate([ct.make_job(float(a), float(o), rig=rig, rk=rk, dele=dele)
                           for a in lats for o in lons])


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


def _run(torch, ctx, jobs, models, noalloc: bool):
    n, off = ct.batch_offsets(jobs)
    dj, dt, do = _dev(torch, jobs), _dev(torch, ct.prepare_trig(jobs)), _dev(torch, off)
    sites = torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    recs = torch.zeros(n * ct.RECORD_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    cnt = torch.zeros(5, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    lib = ctx.lib
    if noalloc:
        rc = lib.cor_trace_batch_device_noalloc(ctx.h, dj.data_ptr(), dt.data_ptr(), len(jobs), do.data_ptr(), n,
                                                models, 25000, 0.01, ct.DEF_HM0_P, sites.data_ptr(),
                                                recs.data_ptr(), cnt.data_ptr(), ct.FLAG_UNIFORM_GRID,
                                                C.c_void_p(stream))
    else:
        status = torch.zeros(n, dtype=torch.uint8, device="cuda")
        rc = lib.cor_trace_batch_device(ctx.h, dj.data_ptr(), dt.data_ptr(), len(jobs), do.data_ptr(), n, models,
                                        25000, 0.01, ct.DEF_HM0_P, sites.data_ptr(), status.data_ptr(),
                                        recs.data_ptr(), cnt.data_ptr(), ct.FLAG_UNIFORM_GRID, C.c_void_p(stream))
    assert rc == 0, ctx.error()
    torch.cuda.synchronize()
    c = cnt.cpu().numpy()
    return (sites.cpu().numpy().copy(), recs.cpu().numpy().copy(),
            dict(zip(("accepted_steps", "trials", "trajectories", "watchdog", "kernel_launches"), c.tolist())))


def test_noalloc_matches_device_path():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    ctx = ct.Context(0)
    try:
        models = ct.model_set(ct.INTERNAL_SH)
        p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
        ctx._check(ctx.lib.cor_upload_params(ctx.h, p.ctypes.data, len(p)), "cor_upload_params")
        first = _batch(range(-80, 81, 20), (0.0, 120.0, 240.0))          # 27 scans x 400 rigidities
        second = _batch((-35.0, 5.0, 45.0), (60.0, 300.0), rig=0.5, dele=0.25)   # 6 scans x 79
        for jobs in (first, second):
            want = _run(torch, ctx, jobs, models, noalloc=False)
            free_before = torch.cuda.mem_get_info()[0]
            got = _run(torch, ctx, jobs, models, noalloc=True)
            assert np.array_equal(got[0], want[0]), "site results differ"
            assert np.array_equal(got[1], want[1]), "trajectory records differ"
            for k in SEEN:
                assert got[2][k] == want[2][k], k
            assert got[2]["kernel_launches"] >= 2
            # the call itself reserved no device memory (the tensors above are
            # torch's, made before the measurement starts)
            assert torch.cuda.mem_get_info()[0] >= free_before - (2 << 20)
        # beyond the stated maximum: refused before any GPU work
        big = ct.NOALLOC_MAX_TRAJ + 1
        rc = ctx.lib.cor_trace_batch_device_noalloc(ctx.h, None, None, 0, None, big, models, 25000, 0.01,
                                                    ct.DEF_HM0_P, None, None, None, 0, None)
        assert rc == -7, ctx.error()  # COR_ERR_RANGE
        assert "maximum" in ctx.error()
    finally:
        ctx.close()
