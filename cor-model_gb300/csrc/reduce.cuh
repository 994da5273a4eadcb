// reduce.cuh -- per-scan reduction of the trajectory classes to P(S), P(C), P(M)
// by one warp (used by the batch reduction kernel and the scan stream).
#pragma once

#include "../../include/cor_trace.h"

namespace cor {

// Per-scan reduction, src/trajectory.c:156-160, by one whole warp: the
// classes status[b .. e-1] of scan `job` (grid indices i_first ..).  The
// reference's fmin/fmax over thread_rig = rig + i*del are taken through the
// extreme indices (thread_rig increases with i), so the result does not
// depend on the order in which trajectories finished.  For a window of the
// grid (i_first > 0 or i_count > 0) the indices are the grid's and the
// untraced indices below the window count as forbidden.  The classes are
// read through L2 (ld.global.cg): other SMs wrote them during the same
// kernel in the persistent stream.
__device__ __forceinline__ cor_site_result reduce_scan_warp(const cor_scan_job& job, const uint8_t* status,
                                                            uint64_t b, uint64_t e) {
    const int lane = threadIdx.x & 31;
    int imin_allowed = 0x7fffffff, imax1 = -1, imax2 = -1, nza = 0;
    const int i0 = job.i_first;  // grid index of the first traced trajectory
    for (uint64_t t = b + lane; t < e; t += 32) {
        const int i = i0 + (int)(t - b);
        const int st = __ldcg(status + t);
        if (st == COR_TRAJ_ALLOWED) {
            imin_allowed = min(imin_allowed, i);
        } else if (st == COR_TRAJ_REENTRY || st == COR_TRAJ_SUPERLUM) {
            imax1 = max(imax1, i);
            nza++;
        } else {
            imax2 = max(imax2, i);
            nza++;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        imin_allowed = min(imin_allowed, __shfl_xor_sync(0xffffffffu, imin_allowed, o));
        imax1 = max(imax1, __shfl_xor_sync(0xffffffffu, imax1, o));
        imax2 = max(imax2, __shfl_xor_sync(0xffffffffu, imax2, o));
        nza += __shfl_xor_sync(0xffffffffu, nza, o);
    }
    double rmi = job.rk, rmx1 = 0., rmx2 = 0.;
    if (imin_allowed != 0x7fffffff) rmi = fmin(rmi, job.rig + imin_allowed * job.del);
    if (imax1 >= 0) rmx1 = fmax(rmx1, job.rig + imax1 * job.del);
    if (imax2 >= 0) rmx2 = fmax(rmx2, job.rig + imax2 * job.del);
    double rmx = fmax(rmx1, rmx2);
    // the untraced indices below a window count as forbidden
    nza += job.i_first;
    const double zan = nza - (rmi - job.rig) / job.del;
    const double rms = rmi + zan * job.del;
    rmx = rmx + job.del;
    cor_site_result r;
    r.r_lower = rmi;
    r.r_upper = rmx;
    r.r_cutoff = rms;
    r.n_forbidden = nza;
    r.n_traj = (int32_t)(e - b);
    return r;
}

}  // namespace cor
