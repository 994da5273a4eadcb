// trace.cuh -- the persistent rigidity-scan kernel (trajectory_simulation_cutoff,
// src/trajectory.c:6-161) and the per-scan reduction (:156-160).
//
// One trajectory per thread.  Threads pull trajectory indices from a device
// work queue (one 64-bit counter, warp-aggregated atomics) and refill
// themselves as soon as their trajectory terminates, so a warp keeps all 32
// lanes busy while trajectory lengths range from tens to 25k steps.  Each
// pass of the main loop advances every lane by exactly one accepted step (or
// one termination + refill), and then evaluates the field for all lanes at
// once, so the expensive field evaluation runs converged.
#pragma once

#include "field.cuh"

namespace cor {

// Host-prepared per-scan trigonometry: sin/cos of the start colatitude and
// longitude and of the velocity direction (src/trajectory.c:18-28), taken
// from the host C library so the device start vectors equal the reference's.
struct JobTrig {
    double st0, ct0, sp0, cp0;
    double st1, ct1, sp1, cp1;
};

struct TraceArgs {
    const cor_scan_job* jobs;
    const JobTrig* trig;
    const uint64_t* offsets;  // n_jobs + 1 exclusive prefix
    int32_t n_jobs;
    uint64_t n_traj;
    const DevParams* params;
    uint64_t step_limit;
    double tu_angle;
    double gc_reject;   // turn test: reject iff gc <= gc_reject (exact host-derived threshold)
    int turn_exact;     // 1: use gc_reject; 0: evaluate atan2 as the reference does
    int rig_major;      // 1: queue index runs over rigidity first (all jobs share n_rig)
    uint32_t n_rig;
    double mass;
    uint8_t* status;
    cor_traj_record* records;
    unsigned long long* queue;     // scratch: next trajectory index
    cor_counters* counters;
    CrustalTables crust;
};

__device__ __forceinline__ int find_job(const uint64_t* __restrict__ off, int n_jobs, uint64_t t) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(reinterpret_cast<const unsigned long long*>(off) + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Per-lane trajectory state.
struct Lane {
    Vec3 pos, vel, field, gsm;
    double b, v, time, alength, rig;
    const cor_scan_job* job;
    const DevParams* par;
    uint64_t traj;
    uint32_t step, trials;
    int nk0;
};

// Claims the next trajectory index for every lane in `want` with one
// atomic per warp.  Returns this lane's index (>= n_traj when the queue is
// drained).
__device__ __forceinline__ uint64_t queue_pop(unsigned long long* q, bool want) {
    const unsigned mask = __ballot_sync(__activemask(), want);
    if (!want) return ~0ull;
    const int leader = __ffs(mask) - 1;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(q, (unsigned long long)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// Start of one trajectory, src/trajectory.c:13-44 (the field is evaluated
// by the caller in the converged section).
__device__ __forceinline__ void lane_init(Lane& L, const TraceArgs& a, uint64_t t) {
    // Queue position -> (scan j, rigidity index i).  In rigidity-major order
    // the lowest rigidities of every scan, whose trajectories are the
    // longest, are handed out first (longest-processing-time-first), which
    // keeps the end of the run from being a tail of lone long trajectories.
    int j;
    uint64_t i;
    if (a.rig_major) {
        i = t / (uint64_t)a.n_jobs;
        j = (int)(t - i * (uint64_t)a.n_jobs);
    } else {
        j = find_job(a.offsets, a.n_jobs, t);
        i = t - a.offsets[j];
    }
    const cor_scan_job* job = a.jobs + j;
    const JobTrig tg = a.trig[j];
    L.job = job;
    L.par = a.params + job->param_index;
    L.traj = a.offsets[j] + i;
    const double rig = job->rig + (int)i * job->del;
    L.rig = rig;
    L.nk0 = job->nk1;
    L.time = 0.;
    L.alength = 0.;
    const double zn = job->zn;
    const double aa = rig * 1.0e+09 * zn * kQ / (a.mass * kC * kC);
    const double vr0 = kC * sqrt(1. - 1. / (1. + aa * aa));
    {
        const double r = job->r0 * kRe;  // sph_to_car, src/utils.c:28-41
        const double sq = r * tg.st0;
        L.pos.x = sq * tg.cp0;
        L.pos.y = sq * tg.sp0;
        L.pos.z = r * tg.ct0;
    }
    {
        const double sq = vr0 * tg.st1;
        L.vel.x = sq * tg.cp1;
        L.vel.y = sq * tg.sp1;
        L.vel.z = vr0 * tg.ct1;
    }
    L.v = vr0;
    L.step = 0;
    L.trials = 0;
    L.gsm = geo_to_gsm(L.pos, &L.par->p);
}

// Advances one lane to its next accepted step (returns 0) or to its
// termination (returns the COR_TRAJ_* class).  src/trajectory.c:45-152,
// with the field evaluation left to the caller.  Bounded: at most 10
// turn-angle halvings (nk0 <= 50000) plus at most 30 boundary halvings
// (nk0 < 2^30) per step.
__device__ __forceinline__ int lane_advance(Lane& L, const TraceArgs& a) {
    const double zn = L.job->zn;
    const int nk1 = L.job->nk1;
    for (;;) {
        L.step++;
        const double vc = div_c(L.v, kC, 1. / kC);
        if (vc > 1.) return COR_TRAJ_SUPERLUM;  // :48-54
        const double hm = a.mass / sqrt(1. - vc * vc);
        const double t = (2. * kPi * hm) / (fabs(zn) * kQ * L.b);
        const double h = t / L.nk0;
        const double d = (1.E-09 * zn * kQ) / hm;
        const double vprev = L.v;
        const Vec3 nv = rk_velocity(h, d, L.field, L.vel);
        L.trials++;
        L.v = sqrt(nv.x * nv.x + nv.y * nv.y + nv.z * nv.z);
        const double gc = (nv.x * L.vel.x + nv.y * L.vel.y + nv.z * L.vel.z) / (L.v * vprev);
        // Turn-angle test, :69-79: reject iff gc < 1 and
        // atan2(sqrt((1-gc)(1+gc)), gc) >= tu_angle.  That predicate of the
        // rounded gc is a step function; the host finds its last true value
        // with the C library and checks the step, so one comparison gives
        // the reference's decision exactly.
        bool reject;
        if (a.turn_exact) {
            reject = gc <= a.gc_reject;
        } else {
            reject = false;
            if (gc < 1.) {
                const double gs = sqrt((1. - gc) * (1. + gc));
                reject = atan2(gs, gc) >= a.tu_angle;
            }
        }
        if (reject && L.nk0 <= 50000) {
            L.nk0 *= 2;
            L.step--;
            continue;
        }
        const Vec3 np = rk_position(h, L.vel, L.pos);
        const double rr = sqrt(np.x * np.x + np.y * np.y + np.z * np.z);  // car_to_sph radius
        const Vec3 gsm = geo_to_gsm(np, &L.par->p);
        const double pax = div_c(DIVRE(gsm.x) + 25.3, 36.08, 1. / 36.08);
        const double paz = div_c(gsm.y * gsm.y + gsm.z * gsm.z, kRe * kRe, 1. / (kRe * kRe));
        const double r = DIVRE(rr);
        const double paus = pax * pax + div_c(paz, 459.6736, 1. / 459.6736);
        if (r >= 25. || paus > 1.) {  // :89-131
            if ((r >= 25. && fabs(r - 25.) < 0.002) || (r <= 25. && paus > 1. && fabs(paus - 1.) < 0.002)) {
                L.pos = np;
                L.vel = nv;
                return COR_TRAJ_ALLOWED;
            }
            if (L.nk0 >= kNk0Cap) return COR_TRAJ_WATCHDOG;
            L.nk0 *= 2;
            L.step--;
            continue;
        }
        const Vec3 prev = L.pos;
        L.pos = np;
        L.vel = nv;
        if (r < 1.) return COR_TRAJ_REENTRY;                          // :133-138
        if ((uint64_t)L.step > a.step_limit) return COR_TRAJ_STEP_LIMIT;  // :140-145 (phi > 31.4 cannot hold)
        L.gsm = gsm;
        L.time = L.time + h;                                          // :150-152 (t/nk0 == h)
        L.alength += sqrt((np.x - prev.x) * (np.x - prev.x) + (np.y - prev.y) * (np.y - prev.y) +
                          (np.z - prev.z) * (np.z - prev.z));
        L.nk0 = nk1;
        return 0;
    }
}

__device__ __forceinline__ void lane_finish(Lane& L, const TraceArgs& a, int st) {
    if (a.status) a.status[L.traj] = (uint8_t)st;
    if (a.records) {
        cor_traj_record r;
        r.pos[0] = L.pos.x; r.pos[1] = L.pos.y; r.pos[2] = L.pos.z;
        r.vel[0] = L.vel.x; r.vel[1] = L.vel.y; r.vel[2] = L.vel.z;
        r.v = L.v;
        r.time = L.time;
        r.length = L.alength;
        r.steps = (st == COR_TRAJ_ALLOWED) ? L.step - 1 : L.step;
        r.trials = L.trials;
        r.status = st;
        r.reserved = 0;
        a.records[L.traj] = r;
    }
}

__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

template <class MS>
__global__ void __launch_bounds__(128) trace_kernel(const TraceArgs a) {
    Lane L;
    bool has = false, done = false;
    unsigned long long n_steps = 0, n_trials = 0, n_traj = 0, n_wd = 0;
    for (;;) {
        bool need_field = false;
        if (has) {
            const int st = lane_advance(L, a);
            if (st == 0) {
                need_field = true;
            } else {
                lane_finish(L, a, st);
                n_steps += (st == COR_TRAJ_ALLOWED) ? L.step - 1 : L.step;
                n_trials += L.trials;
                n_traj += 1;
                n_wd += (st == COR_TRAJ_WATCHDOG);
                has = false;
            }
        }
        const bool want = !has && !done;
        const uint64_t t = queue_pop(a.queue, want);
        if (want) {
            if (t < a.n_traj) {
                lane_init(L, a, t);
                has = true;
                need_field = true;
            } else {
                done = true;
            }
        }
        if (__all_sync(0xffffffffu, done)) break;
        if (need_field) {
            L.field = calculate_field<MS>(L.gsm, L.par, a.crust);
            L.b = 1.E-09 * sqrt(L.field.x * L.field.x + L.field.y * L.field.y + L.field.z * L.field.z);
        }
    }
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->accepted_steps), n_steps);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->trials), n_trials);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->trajectories), n_traj);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->watchdog), n_wd);
}

// Per-scan reduction, src/trajectory.c:156-160, one warp per scan.  The
// reference's fmin/fmax over thread_rig = rig + i*del are taken through the
// extreme indices (thread_rig increases with i), so the result does not
// depend on the order in which trajectories finished.
__global__ void reduce_kernel(const cor_scan_job* __restrict__ jobs, const uint64_t* __restrict__ off,
                              int n_jobs, const uint8_t* __restrict__ status, cor_site_result* __restrict__ out) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n_jobs) return;
    const uint64_t b = off[w], e = off[w + 1];
    int imin_allowed = 0x7fffffff, imax1 = -1, imax2 = -1, nza = 0;
    for (uint64_t t = b + lane; t < e; t += 32) {
        const int i = (int)(t - b);
        const int st = status[t];
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
    if (lane == 0) {
        const cor_scan_job job = jobs[w];
        double rmi = job.rk, rmx1 = 0., rmx2 = 0.;
        if (imin_allowed != 0x7fffffff) rmi = fmin(rmi, job.rig + imin_allowed * job.del);
        if (imax1 >= 0) rmx1 = fmax(rmx1, job.rig + imax1 * job.del);
        if (imax2 >= 0) rmx2 = fmax(rmx2, job.rig + imax2 * job.del);
        double rmx = fmax(rmx1, rmx2);
        const double zan = nza - (rmi - job.rig) / job.del;
        const double rms = rmi + zan * job.del;
        rmx = rmx + job.del;
        cor_site_result r;
        r.r_lower = rmi;
        r.r_upper = rmx;
        r.r_cutoff = rms;
        r.n_forbidden = nza;
        r.n_traj = (int32_t)(e - b);
        out[w] = r;
    }
}

template <class MS>
__global__ void field_kernel(const DevParams* __restrict__ params, int n_params,
                             const int32_t* __restrict__ pidx, const double* __restrict__ pos, int64_t n,
                             double* __restrict__ out, CrustalTables crust) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = pidx ? pidx[i] : 0;
    if (k < 0 || k >= n_params) k = 0;
    const Vec3 x = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const Vec3 b = calculate_field<MS>(x, params + k, crust);
    out[3 * i] = b.x;
    out[3 * i + 1] = b.y;
    out[3 * i + 2] = b.z;
}

}  // namespace cor
