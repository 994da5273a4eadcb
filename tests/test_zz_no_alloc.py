"""cor_trace_batch_device_noalloc against cor_trace_batch_device.

The file is named to be collected last: the no-allocation entry point must
give the existing device path's results both in a fresh process and after
every other test has used the library.  Two calls in a row (different
batches) check that the shared scratch array's leftover contents never leak
into a result.  Every buffer the calls use is made before free device memory
is measured, and one warm-up call first loads the entry point's kernels, so
the measured calls must leave free memory exactly as it was."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cortrace as ct

pytestmark = pytest.mark.gpu

SEEN = ("accepted_steps", "trials", "trajectories", "watchdog")
GUARD = 64  # trajectory records past the batch's end that must stay untouched


def _batch(lats, lons, rig=0.05, rk=20.0, dele=0.05):
    return np.concatenate([ct.make_job(float(a), float(o), rig=rig, rk=rk, dele=dele)
                           for a in lats for o in lons])


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


class _Buffers:
    """Device inputs and outputs of one batch, made before any measured call;
    the records buffer has GUARD extra records filled with 0xA5."""

    def __init__(self, torch, jobs):
        self.jobs = jobs
        self.n, off = ct.batch_offsets(jobs)
        self.dj, self.dt, self.do = _dev(torch, jobs), _dev(torch, ct.prepare_trig(jobs)), _dev(torch, off)
        self.sites = torch.zeros(len(jobs) * ct.SITE_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        self.recs = torch.full(((self.n + GUARD) * ct.RECORD_DTYPE.itemsize,), 0xA5, dtype=torch.uint8,
                               device="cuda")
        self.status = torch.zeros(self.n, dtype=torch.uint8, device="cuda")
        self.cnt = torch.zeros(5, dtype=torch.int64, device="cuda")

    def call(self, torch, ctx, models, noalloc: bool, flags=ct.FLAG_UNIFORM_GRID):
        stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        lib = ctx.lib
        if noalloc:
            rc = lib.cor_trace_batch_device_noalloc(ctx.h, self.dj.data_ptr(), self.dt.data_ptr(), len(self.jobs),
                                                    self.do.data_ptr(), self.n, models, 25000, 0.01, ct.DEF_HM0_P,
                                                    self.sites.data_ptr(), self.recs.data_ptr(),
                                                    self.cnt.data_ptr(), flags, stream)
        else:
            rc = lib.cor_trace_batch_device(ctx.h, self.dj.data_ptr(), self.dt.data_ptr(), len(self.jobs),
                                            self.do.data_ptr(), self.n, models, 25000, 0.01, ct.DEF_HM0_P,
                                            self.sites.data_ptr(), self.status.data_ptr(), self.recs.data_ptr(),
                                            self.cnt.data_ptr(), flags, stream)
        assert rc == 0, ctx.error()

    def results(self):
        c = self.cnt.cpu().numpy()
        rec = self.recs.cpu().numpy()
        used = self.n * ct.RECORD_DTYPE.itemsize
        return (self.sites.cpu().numpy().copy(), rec[:used].copy(), rec[used:].copy(),
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
        warm = _Buffers(torch, _batch((10.0,), (10.0,), rig=5.0, rk=6.0, dele=0.5))
        bufs = [(_Buffers(torch, jobs), _Buffers(torch, jobs)) for jobs in (first, second)]
        wants = []
        for dev_path, _ in bufs:
            dev_path.call(torch, ctx, models, noalloc=False)
            torch.cuda.synchronize()
            wants.append(dev_path.results())
        warm.call(torch, ctx, models, noalloc=True)       # loads the entry point's kernels
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for (_, nb), want in zip(bufs, wants):
            nb.call(torch, ctx, models, noalloc=True)
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] >= free_before, "the call reserved device memory"
            sites, recs, guard, cnt = nb.results()
            assert np.array_equal(sites, want[0]), "site results differ"
            assert np.array_equal(recs, want[1]), "trajectory records differ"
            assert np.all(guard == 0xA5), "a record was written past the batch's end"
            for k in SEEN:
                assert cnt[k] == want[3][k], k
            # uniform-grid check, one scan generation, the reduction, the counter kernel
            assert cnt["kernel_launches"] == 4
        # beyond the stated maximum: refused before any GPU work
        big = ct.NOALLOC_MAX_TRAJ + 1
        rc = ctx.lib.cor_trace_batch_device_noalloc(ctx.h, None, None, 0, None, big, models, 25000, 0.01,
                                                    ct.DEF_HM0_P, None, None, None, 0, None)
        assert rc == -7, ctx.error()  # COR_ERR_RANGE
        assert "maximum" in ctx.error()
    finally:
        ctx.close()


def test_noalloc_wrong_uniform_flag_stays_in_bounds():
    """A batch whose scans have different rigidity counts, passed with the
    uniform-grid flag: the device check keeps the scan-by-scan order, so the
    results equal the unflagged call's and nothing is written past the
    records buffer."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    ctx = ct.Context(0)
    try:
        models = ct.model_set(ct.INTERNAL_SH)
        p = ct.internal_setup("igrf14", [2020, 1, 1, 1, 0, 0, 0])
        ctx._check(ctx.lib.cor_upload_params(ctx.h, p.ctypes.data, len(p)), "cor_upload_params")
        # scans of 40, 79, 41 and 4 rigidities: 164 trajectories, 41 per scan on
        # average, so the trajectory count alone would pass for a uniform grid
        jobs = np.concatenate([ct.make_job(20.0, 30.0, rig=1.0, rk=20.5, dele=0.5),
                               ct.make_job(-40.0, 200.0, rig=0.5, rk=20.0, dele=0.25),
                               ct.make_job(60.0, 90.0, rig=0.5, rk=20.5, dele=0.5),
                               ct.make_job(0.0, 0.0, rig=5.0, rk=6.5, dele=0.5)])
        n, off = ct.batch_offsets(jobs)
        assert n % len(jobs) == 0 and len(set(np.diff(off).tolist())) > 1
        a, b = _Buffers(torch, jobs), _Buffers(torch, jobs)
        a.call(torch, ctx, models, noalloc=True, flags=0)
        torch.cuda.synchronize()
        b.call(torch, ctx, models, noalloc=True, flags=ct.FLAG_UNIFORM_GRID)
        torch.cuda.synchronize()
        ra, rb = a.results(), b.results()
        assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])
        assert np.all(rb[2] == 0xA5)
    finally:
        ctx.close()
