// trace.cuh -- the persistent rigidity-scan kernel (trajectory_simulation_cutoff,
// src/trajectory.c:6-153); the per-scan reduction (:156-160) is reduce.cuh.
//
// One trajectory per thread.  Threads pull trajectory indices from a device
// work queue (one 64-bit counter, warp-aggregated atomics) and refill
// themselves as soon as their trajectory terminates, so a warp keeps all 32
// lanes busy while trajectory lengths range from tens to 25k steps.  Each
// pass of the main loop advances every lane by exactly one accepted step (or
// one termination + refill) and then evaluates the field for all lanes at
// once, so the expensive field evaluation runs converged; the pass's exit and
// park decisions are block-wide, which also keeps the block's warps in step
// through the field models' code.  The same loop records every accepted step
// when a trajectory dump is requested (cor_trace_steps).
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

// A trajectory in flight, parked between two generations of the kernel
// (bitwise copy of the lane state, so a parked and restored trajectory
// continues exactly as if it had not moved).
struct ParkedLane {
    double pos[3], vel[3], field[3], gsm[3];
    double b, v, time, alength, rig;
    unsigned long long traj;
    int32_t job;
    uint32_t step, trials;
    int32_t nk0;
    int32_t need_field;   // parked right after a step or its start: the field at pos is still to be evaluated
};

// Per-generation scratch counters (zeroed before each generation).
struct GenCounters {
    unsigned long long restore_cursor;  // next parked trajectory to restore
    unsigned int park_count;            // trajectories parked by this generation
    unsigned int parked_warps;          // warps that have parked and exited
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
    // device word written by grid_check_kernel before the launch: non-zero iff
    // offsets[j] == j * n_rig for every j (the rigidity-major mapping is then a
    // bijection onto 0 .. n_traj-1); rig_major is ignored when it is zero.
    // Null: rig_major is taken as given (the host checked the grid itself).
    const unsigned int* grid_ok;
    uint32_t n_rig;
    double mass;
    uint8_t* status;
    cor_traj_record* records;
    unsigned long long* queue;     // scratch: next trajectory index
    cor_counters* counters;
    CrustalTables crust;
    // compaction between generations
    const ParkedLane* restore;     // trajectories parked by the previous generation
    uint32_t n_restore;
    ParkedLane* park;              // where this generation parks (capacity = launched threads)
    GenCounters* gen;
    int allow_park;                // 0 in the last generation
    int park_below;                // a block parks when fewer lanes than this per working warp are live
    uint32_t launched_warps;
    // trajectory dump: every accepted step of trajectory t goes to
    // step_records[t * step_cap + step - 1] (null: not recorded)
    cor_step_record* step_records;
    uint32_t step_cap;
    // threads of each block that take trajectories (a multiple of 32, at
    // most kTraceThreads): a generation with few trajectories spreads them
    // over more SMs, a warp or two each, instead of packing them into a few
    // blocks whose warps would share one SM's FP64 pipe
    uint32_t active_threads;
    // 1: before each field evaluation the block regroups the trajectories
    // that need one by field_band (regroup_lanes); 0: never
    int sort_lanes;
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
    int32_t job_index;
};

__device__ __forceinline__ void lane_park(const Lane& L, bool need_field, ParkedLane& o) {
    o.pos[0] = L.pos.x; o.pos[1] = L.pos.y; o.pos[2] = L.pos.z;
    o.vel[0] = L.vel.x; o.vel[1] = L.vel.y; o.vel[2] = L.vel.z;
    o.field[0] = L.field.x; o.field[1] = L.field.y; o.field[2] = L.field.z;
    o.gsm[0] = L.gsm.x; o.gsm[1] = L.gsm.y; o.gsm[2] = L.gsm.z;
    o.b = L.b; o.v = L.v; o.time = L.time; o.alength = L.alength; o.rig = L.rig;
    o.traj = L.traj;
    o.job = L.job_index;
    o.step = L.step; o.trials = L.trials; o.nk0 = L.nk0;
    o.need_field = need_field ? 1 : 0;
}

// Returns whether the restored trajectory still needs its field evaluated.
__device__ __forceinline__ bool lane_restore(Lane& L, const ParkedLane& o, const cor_scan_job* jobs,
                                             const DevParams* params) {
    L.pos = {o.pos[0], o.pos[1], o.pos[2]};
    L.vel = {o.vel[0], o.vel[1], o.vel[2]};
    L.field = {o.field[0], o.field[1], o.field[2]};
    L.gsm = {o.gsm[0], o.gsm[1], o.gsm[2]};
    L.b = o.b; L.v = o.v; L.time = o.time; L.alength = o.alength; L.rig = o.rig;
    L.traj = o.traj;
    L.job_index = o.job;
    L.job = jobs + o.job;
    L.par = params + L.job->param_index;
    L.step = o.step; L.trials = o.trials; L.nk0 = o.nk0;
    return o.need_field != 0;
}

// Claims the next index of a queue for every lane in `want` with one atomic
// per warp; called by all 32 lanes of a warp together.  Returns this lane's
// index (the caller compares it with the queue length).
__device__ __forceinline__ uint64_t queue_pop(unsigned long long* q, bool want) {
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if (lane == leader) base = atomicAdd(q, (unsigned long long)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return want ? base + __popc(mask & ((1u << lane) - 1u)) : ~0ull;
}

// Start of one trajectory, src/trajectory.c:13-44: scan `job` (index j of
// its batch), grid position i of the traced range, batch-local trajectory
// index `traj` (the field is evaluated by the caller in the converged section).
__device__ __forceinline__ void lane_start(Lane& L, const cor_scan_job* job, const JobTrig& tg, const DevParams* par,
                                           int j, uint64_t i, uint64_t traj, double mass) {
    L.job = job;
    L.job_index = j;
    L.par = par;
    L.traj = traj;
    const double rig = job->rig + (int)(i + (uint64_t)job->i_first) * job->del;  // :14, absolute grid index
    L.rig = rig;
    L.nk0 = job->nk1;
    L.time = 0.;
    L.alength = 0.;
    const double zn = job->zn;
    const double aa = rig * 1.0e+09 * zn * kQ / (mass * kC * kC);
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

// Queue position t -> (scan j, rigidity index i), then lane_start.  In
// rigidity-major order (rig_major: every scan has n_traj / n_jobs
// trajectories, checked on the device by grid_check_kernel) the lowest
// rigidities of every scan, whose trajectories are the longest, are handed
// out first (longest-processing-time-first), which keeps the end of the run
// from being a tail of lone long trajectories.
__device__ __forceinline__ void lane_init(Lane& L, const TraceArgs& a, uint64_t t, bool rig_major) {
    int j;
    uint64_t i;
    if (rig_major) {
        i = t / (uint64_t)a.n_jobs;
        j = (int)(t - i * (uint64_t)a.n_jobs);
    } else {
        j = find_job(a.offsets, a.n_jobs, t);
        i = t - a.offsets[j];
    }
    lane_start(L, a.jobs + j, a.trig[j], a.params + a.jobs[j].param_index, j, i, a.offsets[j] + i, a.mass);
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

__device__ __forceinline__ void lane_record(const Lane& L, int st, uint8_t* status, cor_traj_record* records) {
    if (status) status[L.traj] = (uint8_t)st;
    if (records) {
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
        records[L.traj] = r;
    }
}

// A trajectory's class and final record into the batch's buffers; an index
// at or beyond n_traj (possible only with offsets that disagree with
// n_traj) writes nothing.
__device__ __forceinline__ void lane_finish(Lane& L, const TraceArgs& a, int st) {
    if (L.traj < a.n_traj) lane_record(L, st, a.status, a.records);
}

__device__ __forceinline__ void warp_add_u64(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

// Threads of a scan block: one block of 8 warps per SM (the kernels of the
// external-field sets need ~255 registers a thread, so 8 warps is also the
// register file's limit).
constexpr int kTraceThreads = 256;
constexpr int kTraceWarps = kTraceThreads / 32;

// A trajectory in flight as it moves between threads of a block: the lane
// state, its scan (the stream kernel keeps a per-thread copy of the scan's
// job, so there the two fields the steps read, zn and nk1, move instead of
// the pointer), and, in the stream kernel, its segment.
struct LaneMove {
    Vec3 pos, vel, field, gsm;
    double b, v, time, alength, rig, zn;
    const DevParams* par;
    const cor_scan_job* job;
    unsigned long long traj, seq;
    uint32_t step, trials;
    int32_t nk0, job_index, nk1;
    uint32_t slot;
};
static_assert(sizeof(LaneMove) == 200, "LaneMove layout");

// Dynamic shared memory of the trace and stream kernels (regroup_lanes).
struct RegroupScratch {
    LaneMove mv[kTraceThreads];
    unsigned key[kTraceThreads];
    unsigned short at[kTraceThreads];   // the threads that take part, in thread order
    unsigned warp_live[kTraceWarps];
};
constexpr size_t kRegroupSmem = sizeof(RegroupScratch);

// Block-wide: the threads that take part (part: they hold a trajectory whose
// field is evaluated next) trade trajectories so that, taken in thread order,
// their keys ascend (ties keep thread order).  The set of threads that take
// part does not change: a thread without a trajectory, or with one that
// waits for nothing this pass, keeps its place.  Every lane runs the same
// arithmetic wherever it sits, so a trajectory's results do not depend on
// the thread it ends on.  JobCopy: L.job points at the thread's own copy of
// the scan's job (my_job), which then takes the arriving trajectory's zn and
// nk1.  All threads of the block call this.
template <bool JobCopy>
__device__ __forceinline__ void regroup_lanes(RegroupScratch& sc, const bool part, const unsigned key, Lane& L,
                                              cor_scan_job* my_job, unsigned& slot, unsigned long long& seq,
                                              const int tid) {
    const int lane = tid & 31, warp = tid >> 5;
    sc.key[tid] = part ? key : 0xffffffffu;
    const unsigned live = __ballot_sync(0xffffffffu, part);
    if (lane == 0) sc.warp_live[warp] = __popc(live);
    __syncthreads();
    int pos = __popc(live & ((1u << lane) - 1u));
    for (int w = 0; w < warp; w++) pos += (int)sc.warp_live[w];
    if (part) sc.at[pos] = (unsigned short)tid;
    int rank = 0;
    if (part) {
        // keys of the threads that do not take part are above every real key
        for (int j = 0; j < kTraceThreads; j++) {
            const unsigned kj = sc.key[j];
            rank += (kj < key || (kj == key && j < tid)) ? 1 : 0;
        }
    }
    __syncthreads();
    if (part) {
        LaneMove& m = sc.mv[sc.at[rank]];
        m.pos = L.pos;
        m.vel = L.vel;
        m.field = L.field;
        m.gsm = L.gsm;
        m.b = L.b;
        m.v = L.v;
        m.time = L.time;
        m.alength = L.alength;
        m.rig = L.rig;
        m.par = L.par;
        m.job = L.job;
        if constexpr (JobCopy) {
            m.zn = L.job->zn;
            m.nk1 = L.job->nk1;
        }
        m.traj = L.traj;
        m.seq = seq;
        m.step = L.step;
        m.trials = L.trials;
        m.nk0 = L.nk0;
        m.job_index = L.job_index;
        m.slot = slot;
    }
    __syncthreads();
    if (part) {
        const LaneMove& m = sc.mv[tid];
        L.pos = m.pos;
        L.vel = m.vel;
        L.field = m.field;
        L.gsm = m.gsm;
        L.b = m.b;
        L.v = m.v;
        L.time = m.time;
        L.alength = m.alength;
        L.rig = m.rig;
        L.par = m.par;
        L.traj = m.traj;
        L.step = m.step;
        L.trials = m.trials;
        L.nk0 = m.nk0;
        L.job_index = m.job_index;
        if constexpr (JobCopy) {
            my_job->zn = m.zn;
            my_job->nk1 = m.nk1;
            L.job = my_job;
        } else {
            L.job = m.job;
        }
        seq = m.seq;
        slot = m.slot;
    }
}

// One generation of the scan.  Every thread of a block stays in the loop
// until the block leaves it as a whole: the exit and park decisions are
// block-wide (__syncthreads_count / _or), which also lines the block's warps
// up before each field evaluation, so they run through the field models'
// instructions together and share the instruction-cache fills.
// A lane with no trajectory takes the next parked one, else the next queue
// index.  Once the queue is drained, a block whose live lanes fall below
// park_below per working warp -- or any block, once half of the generation's
// warps have parked -- writes its live trajectories to the park list and leaves;
// the host then launches the next generation sized to the parked count,
// which restores them densely (the regroup step).
template <class MS>
__global__ void __launch_bounds__(kTraceThreads, 1) trace_kernel(const TraceArgs a) {
    extern __shared__ __align__(16) unsigned char s_dyn[];
    RegroupScratch& sc = *reinterpret_cast<RegroupScratch*>(s_dyn);
    Lane L;
    bool has = false, done = threadIdx.x >= a.active_threads;
    unsigned long long n_steps = 0, n_trials = 0, n_traj = 0, n_wd = 0;
    const int lane = threadIdx.x & 31;
    const bool rig_major = a.rig_major && (!a.grid_ok || *(volatile const unsigned int*)a.grid_ok != 0u);
    for (;;) {
        bool need_field = false;
        if (has) {
            const int st = lane_advance(L, a);
            if (st == 0) {
                need_field = true;
                if (a.step_records && L.step <= a.step_cap) {
                    cor_step_record r;
                    r.gsm[0] = L.gsm.x; r.gsm[1] = L.gsm.y; r.gsm[2] = L.gsm.z;
                    r.pos[0] = L.pos.x; r.pos[1] = L.pos.y; r.pos[2] = L.pos.z;
                    r.v = L.v;
                    r.time = L.time;
                    r.length = L.alength;
                    r.step = L.step;
                    r.reserved = 0;
                    a.step_records[L.traj * a.step_cap + (L.step - 1)] = r;
                }
            } else {
                lane_finish(L, a, st);
                n_steps += (st == COR_TRAJ_ALLOWED) ? L.step - 1 : L.step;
                n_trials += L.trials;
                n_traj += 1;
                n_wd += (st == COR_TRAJ_WATCHDOG);
                has = false;
            }
        }
        __syncwarp();
        bool want = !has && !done;
        if (a.n_restore) {
            const uint64_t r = queue_pop(&a.gen->restore_cursor, want);
            if (want && r < a.n_restore) {
                need_field = lane_restore(L, a.restore[r], a.jobs, a.params);
                has = true;
                want = false;
            }
        }
        const uint64_t t = queue_pop(a.queue, want);
        if (want) {
            if (t < a.n_traj) {
                lane_init(L, a, t, rig_major);
                has = true;
                need_field = true;
            } else {
                done = true;
            }
        }
        // block-wide decisions: every thread of the block takes the same
        // branch (threads beyond active_threads are done from the start)
        const int n_done = __syncthreads_count(done);
        if (n_done == kTraceThreads) break;
        if (a.allow_park && n_done > kTraceThreads - (int)a.active_threads) {
            const int n_live = __syncthreads_count(has);
            unsigned pw = 0;
            if (threadIdx.x == 0) pw = *((volatile unsigned int*)&a.gen->parked_warps);
            const int half = __syncthreads_or(threadIdx.x == 0 && 2u * pw >= a.launched_warps);
            if (n_live < a.park_below * (int)(a.active_threads / 32) || half) {
                // need_field lanes were just initialised or advanced: the
                // generation that restores them evaluates their field (the
                // loop keeps a single calculate_field call site, so the field
                // models are inlined once).
                const unsigned live = __ballot_sync(0xffffffffu, has);
                const int leader = __ffs(live) - 1;
                unsigned base = 0;
                if (live && lane == leader) base = atomicAdd(&a.gen->park_count, (unsigned)__popc(live));
                base = __shfl_sync(0xffffffffu, base, live ? leader : 0);
                if (has) lane_park(L, need_field, a.park[base + __popc(live & ((1u << lane) - 1u))]);
                if (lane == 0) atomicAdd(&a.gen->parked_warps, 1u);
                break;
            }
        }
        if (a.sort_lanes) {
            // the lanes whose field is evaluated now, grouped by band
            const unsigned key = need_field ? field_band<MS>(L.gsm, L.par) : 0u;
            unsigned no_slot = 0;
            unsigned long long no_seq = 0;
            regroup_lanes<false>(sc, need_field, key, L, nullptr, no_slot, no_seq, (int)threadIdx.x);
        }
        if constexpr (MS::crustal != 0) {
            // the crustal sum is evaluated by the whole (converged) warp
            const Vec3 f = calculate_field<MS>(need_field, L.gsm, L.par, a.crust);
            if (need_field) {
                L.field = f;
                L.b = 1.E-09 * sqrt(L.field.x * L.field.x + L.field.y * L.field.y + L.field.z * L.field.z);
            }
        } else if (need_field) {
            L.field = calculate_field<MS>(true, L.gsm, L.par, a.crust);
            L.b = 1.E-09 * sqrt(L.field.x * L.field.x + L.field.y * L.field.y + L.field.z * L.field.z);
        }
    }
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->accepted_steps), n_steps);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->trials), n_trials);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->trajectories), n_traj);
    warp_add_u64(reinterpret_cast<unsigned long long*>(&a.counters->watchdog), n_wd);
}

template <class MS>
__global__ void field_kernel(const DevParams* __restrict__ params, int n_params,
                             const int32_t* __restrict__ pidx, const double* __restrict__ pos, int64_t n,
                             double* __restrict__ out, CrustalTables crust) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool want = i < n;
    if (MS::crustal == 0 && !want) return;   // with the crustal model every lane takes part
    int k = 0;
    Vec3 x = {0., 0., 0.};
    if (want) {
        k = pidx ? pidx[i] : 0;
        if (k < 0 || k >= n_params) k = 0;
        x = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    }
    const Vec3 b = calculate_field<MS>(want, x, params + k, crust);
    if (!want) return;
    out[3 * i] = b.x;
    out[3 * i + 1] = b.y;
    out[3 * i + 2] = b.z;
}

}  // namespace cor
