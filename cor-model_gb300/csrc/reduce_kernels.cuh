// reduce_kernels.cuh -- the kernels of a batch scan beside the scan kernel:
// the per-scan reduction (one warp per scan) and the uniform-grid check of
// the rigidity-major queue order.  Included by the C ABI unit only.
#pragma once

#include "reduce.cuh"

namespace cor {

// One warp per scan of a batch.  Offsets are clamped to n_traj, so offsets
// that disagree with the batch's trajectory count never read past status.
__global__ void reduce_kernel(const cor_scan_job* __restrict__ jobs, const uint64_t* __restrict__ off,
                              int n_jobs, uint64_t n_traj, const uint8_t* __restrict__ status,
                              cor_site_result* __restrict__ out) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= n_jobs) return;
    uint64_t b = off[w], e = off[w + 1];
    if (e > n_traj) e = n_traj;
    if (b > e) b = e;
    const cor_site_result r = reduce_scan_warp(jobs[w], status, b, e);
    if ((threadIdx.x & 31) == 0) out[w] = r;
}

// Checks, before a rigidity-major launch, that every scan of the batch has
// n_traj / n_jobs trajectories: offsets[j] == j * n_traj / n_jobs for
// j = 0 .. n_jobs.  One block; writes 1 or 0 to *ok.  The scan kernel uses
// the rigidity-major mapping only when *ok is 1, so a caller's wrong
// uniform-grid flag costs the queue order, never a write out of bounds.
__global__ void grid_check_kernel(const uint64_t* __restrict__ off, int n_jobs, uint64_t n_traj,
                                  unsigned int* ok) {
    int good = n_jobs > 0 && n_traj % (uint64_t)n_jobs == 0;
    const uint64_t per = n_jobs > 0 ? n_traj / (uint64_t)n_jobs : 0;
    for (int j = threadIdx.x; good && j <= n_jobs; j += blockDim.x)
        if (off[j] != (uint64_t)j * per) good = 0;
    good = __syncthreads_and(good);
    if (threadIdx.x == 0) *ok = good ? 1u : 0u;
}

}  // namespace cor
