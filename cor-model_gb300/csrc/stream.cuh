// stream.cuh -- the persistent scan stream: one long-running launch of the
// rigidity-scan kernel that serves batches ("segments") as the host publishes
// them, so that lanes whose trajectories end refill from the next batch
// instead of idling while their block's last long trajectories finish.
//
// Device-side layout:
//   * one global work-queue counter over a queue index space that the host
//     extends segment by segment (segment k covers [base_k, base_k + n_k));
//   * seg_end[k - first_seq] = base_k + n_k, written before segment k is
//     published and never rewritten during the launch;
//   * a ring of segment descriptors (segment k in slot k % n_slots) with the
//     segment's jobs, trig, offsets, outputs and per-scan finish counters;
//   * an append-only pool of parameter blocks (never rewritten during the
//     launch, each block 256-byte aligned so no cache line spans two blocks).
// Host-side, in mapped pinned memory: the control block (published end, stop
// index) the kernel reads with ld.acquire.sys, and one completion record per
// slot that the kernel writes with st.release.sys when a segment's last scan
// is reduced.
//
// A trajectory is integrated exactly as in trace_kernel (lane_start,
// lane_advance, the converged field evaluation); the per-scan reduction
// (src/trajectory.c:156-160) is done in the kernel by the warp whose lane
// finished a scan's last trajectory (reduce_scan_warp), so no second kernel
// is needed while the stream holds the SMs.
#pragma once

#include "reduce.cuh"
#include "trace.cuh"

namespace cor {

// One published segment.  Written by the host into its ring slot before the
// segment is published; read-only while the segment is live.
struct StreamSeg {
    const cor_scan_job* jobs;      // param_index = index into the stream's parameter pool
    const JobTrig* trig;
    const uint64_t* offsets;       // n_jobs + 1 exclusive prefix, offsets[n_jobs] == n_traj
    uint8_t* status;               // n_traj classes
    cor_traj_record* records;      // n_traj final records, or null
    cor_site_result* sites;        // n_jobs
    unsigned int* job_done;        // n_jobs finished counts: zero when published; reset by the reducing warp
    unsigned long long* acc;       // [5] steps, trials, trajectories, watchdog, scans reduced: zero when
                                   // published; reset when the segment completes
    unsigned long long base;       // queue index of the segment's first trajectory
    unsigned long long n_traj;
    unsigned long long seq;
    int32_t n_jobs;
    uint32_t n_rig;                // > 0: every scan has n_rig trajectories (checked by the host): rigidity-major
                                   // order, or with chunk > 0 chunks of `chunk` consecutive rigidities of one
                                   // scan, the chunks in ascending rigidity
    uint32_t chunk;
    const uint32_t* order;         // queue position -> trajectory (offsets space), or null; overrides n_rig
    cor_scan_event* events;        // device address of mapped host records, one per scan, or null
};

// Host-written control block (mapped pinned memory).
struct StreamCtl {
    unsigned long long published;  // end of the published queue range (release store by the host)
    unsigned long long stop_at;    // ~0 while running; else no index at or beyond it will be published
};

// Kernel-written completion record of a slot (mapped pinned memory).
struct StreamDone {
    unsigned long long seq1;       // seq + 1 of the segment that completed in this slot (written last)
    unsigned long long t_ns;       // %globaltimer when it completed
    unsigned long long steps, trials, traj, watchdog;
    unsigned long long pad[2];
};

struct StreamArgs {
    TraceArgs a;                   // step control, parameter pool (a.params), crustal tables, mass
    const StreamCtl* ctl;          // device address of the mapped control block
    StreamDone* done;              // device address of the mapped completion records (n_slots)
    unsigned int* error;           // device address of a mapped word: kStream* bits
    const StreamSeg* segs;         // n_slots descriptors
    uint32_t n_slots;
    const unsigned long long* seg_end;  // seg_end[k - first_seq]
    unsigned long long first_seq;  // first segment this launch serves
    unsigned long long first_index;  // its base
    unsigned long long* queue;     // device counter, first_index at launch
    unsigned long long idle_limit_ns;  // a block with no live lane gives up after waiting this long
    long long seg_cap;             // entries of seg_end
    int32_t n_params;              // blocks in the parameter pool (a job's param_index is checked against it)
};

// Bits of the mapped error word.
constexpr unsigned kStreamIdle = 1u;      // a block gave up waiting for work
constexpr unsigned kStreamBadParam = 2u;  // a job's param_index was outside the pool (trajectory not traced)
constexpr unsigned kStreamBadChain = 4u;  // the segment table ran out or was not increasing

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed_sys(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_sys(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Loads through L2 (ld.global.cg) of data the host rewrites during the
// launch (ring slots): never through the non-coherent path.
template <class T>
__device__ __forceinline__ T* ldcg_ptr(T* const* p) {
    return reinterpret_cast<T*>(__ldcg(reinterpret_cast<const unsigned long long*>(p)));
}

template <class T>
__device__ __forceinline__ void ldcg_copy(T* dst, const T* src) {
    static_assert(sizeof(T) % 8 == 0, "8-byte multiple");
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
#pragma unroll
    for (unsigned k = 0; k < sizeof(T) / 8; k++) d[k] = __ldcg(s + k);
}

__device__ __forceinline__ int find_job_cg(const uint64_t* off, int n_jobs, uint64_t t) {
    int lo = 0, hi = n_jobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldcg(reinterpret_cast<const unsigned long long*>(off) + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The segment's completion: counters into the slot's completion record,
// the slot's accumulators reset for its next segment, then seq + 1 with a
// release store (the host reads it with an acquire load).  One thread.
__device__ __forceinline__ void complete_segment(const StreamArgs& sa, unsigned slot, unsigned long long seq,
                                                 unsigned long long* acc) {
    StreamDone* d = sa.done + slot;
    d->steps = atomicExch(&acc[0], 0ull);
    d->trials = atomicExch(&acc[1], 0ull);
    d->traj = atomicExch(&acc[2], 0ull);
    d->watchdog = atomicExch(&acc[3], 0ull);
    atomicExch(&acc[4], 0ull);
    d->t_ns = global_ns();
    __threadfence_system();
    st_release_sys(&d->seq1, seq + 1);
}

// Bookkeeping of a trajectory that ended with class st (COR_TRAJ_NONE: not
// traced): its class and record, the segment's counters, then its scan's
// finish count.  Returns whether it was the scan's last trajectory.
__device__ __forceinline__ bool stream_finish(const StreamArgs& sa, unsigned slot, const Lane& L, int st) {
    const StreamSeg* sg = sa.segs + slot;
    const unsigned long long n_traj = __ldcg(&sg->n_traj);
    if (L.traj < n_traj) lane_record(L, st, ldcg_ptr(&sg->status), ldcg_ptr(&sg->records));
    unsigned long long* acc = ldcg_ptr(&sg->acc);
    atomicAdd(&acc[0], (unsigned long long)((st == COR_TRAJ_ALLOWED) ? L.step - 1 : L.step));
    atomicAdd(&acc[1], (unsigned long long)L.trials);
    atomicAdd(&acc[2], 1ull);
    if (st == COR_TRAJ_WATCHDOG) atomicAdd(&acc[3], 1ull);
    // the class and counters above before this scan's finish count
    __threadfence();
    const uint64_t* off = ldcg_ptr(&sg->offsets);
    const int j = L.job_index;
    const unsigned n_j = (unsigned)(__ldcg(reinterpret_cast<const unsigned long long*>(off) + j + 1) -
                                    __ldcg(reinterpret_cast<const unsigned long long*>(off) + j));
    const unsigned before = atomicAdd(ldcg_ptr(&sg->job_done) + j, 1u);
    return before + 1 == n_j;
}

template <class MS>
__global__ void __launch_bounds__(kTraceThreads, 1) stream_kernel(const StreamArgs sa) {
    // per thread: a copy of its scan's job (lane_advance reads zn and nk1
    // every step) and where its last queue index fell in the segment chain
    __shared__ cor_scan_job s_job[kTraceThreads];
    __shared__ long long s_k[kTraceThreads];
    __shared__ unsigned long long s_lo[kTraceThreads], s_hi[kTraceThreads];
    extern __shared__ __align__(16) unsigned char s_dyn[];
    RegroupScratch& sc = *reinterpret_cast<RegroupScratch*>(s_dyn);
    const TraceArgs& a = sa.a;
    const int tid = threadIdx.x, lane = tid & 31;
    s_k[tid] = -1;
    s_lo[tid] = sa.first_index;
    s_hi[tid] = sa.first_index;
    Lane L;
    bool has = false, done = false, pending = false, bad = false;
    unsigned long long pend = 0;
    unsigned slot = 0;
    unsigned long long seq = 0;
    unsigned long long pub = 0, stop = ~0ull;     // this warp's view of the control block
    unsigned long long idle_since = 0;            // thread 0: when the block last had no live lane
    for (;;) {
        bool need_field = false, need_reduce = false;
        int red_j = 0;
        if (has) {
            const int st = lane_advance(L, a);
            if (st == 0) {
                need_field = true;
            } else {
                if (stream_finish(sa, slot, L, st)) {
                    need_reduce = true;
                    red_j = L.job_index;
                }
                has = false;
            }
        } else if (bad) {
            // a job whose parameter block is outside the pool: not traced
            if (stream_finish(sa, slot, L, COR_TRAJ_NONE)) {
                need_reduce = true;
                red_j = L.job_index;
            }
            bad = false;
        }
        __syncwarp();
        // reductions of the scans whose last trajectory a lane of this warp just finished
        unsigned rmask = __ballot_sync(0xffffffffu, need_reduce);
        while (rmask) {
            const int src = __ffs(rmask) - 1;
            rmask &= rmask - 1;
            const int j = __shfl_sync(0xffffffffu, red_j, src);
            const unsigned sl = __shfl_sync(0xffffffffu, slot, src);
            const unsigned long long sq = __shfl_sync(0xffffffffu, seq, src);
            const StreamSeg* sg = sa.segs + sl;
            __threadfence();  // see every class the other lanes published before their finish counts
            const uint64_t* off = ldcg_ptr(&sg->offsets);
            cor_scan_job job;
            ldcg_copy(&job, ldcg_ptr(&sg->jobs) + j);
            const uint64_t b = __ldcg(reinterpret_cast<const unsigned long long*>(off) + j);
            const uint64_t e = __ldcg(reinterpret_cast<const unsigned long long*>(off) + j + 1);
            const cor_site_result r = reduce_scan_warp(job, ldcg_ptr(&sg->status), b, e);
            if (lane == 0) {
                ldcg_ptr(&sg->sites)[j] = r;
                cor_scan_event* ev = ldcg_ptr(&sg->events);
                if (ev) {
                    // this scan's result straight to the host, before its segment completes
                    ev[j].site = r;
                    ev[j].first_class = __ldcg(ldcg_ptr(&sg->status) + b);
                    ev[j].last_class = __ldcg(ldcg_ptr(&sg->status) + (e - 1));
                    ev[j].reserved = 0;
                    __threadfence_system();
                    st_release_sys(reinterpret_cast<unsigned long long*>(&ev[j].seq1), sq + 1);
                }
                atomicExch(ldcg_ptr(&sg->job_done) + j, 0u);
                __threadfence();
                unsigned long long* acc = ldcg_ptr(&sg->acc);
                const unsigned long long reduced = atomicAdd(&acc[4], 1ull) + 1;
                if (reduced == (unsigned long long)__ldcg(&sg->n_jobs)) complete_segment(sa, sl, sq, acc);
            }
            __syncwarp();
        }
        // claim the next queue index for every idle lane; a claimed index waits
        // (pending) until the host has published it
        const bool want = !has && !done && !pending && !bad;
        const uint64_t t = queue_pop(sa.queue, want);
        if (want) {
            pending = true;
            pend = t;
        }
        if (__any_sync(0xffffffffu, pending && pend >= pub)) {
            unsigned long long p = 0, sp = 0;
            if (lane == 0) {
                p = ld_acquire_sys(&sa.ctl->published);
                sp = ld_relaxed_sys(&sa.ctl->stop_at);
            }
            pub = __shfl_sync(0xffffffffu, p, 0);
            stop = __shfl_sync(0xffffffffu, sp, 0);
        }
        if (pending && pend < pub) {
            // walk this lane's segment chain forward to the segment holding pend
            long long k = s_k[tid];
            unsigned long long lo = s_lo[tid], hi = s_hi[tid];
            bool chain_ok = true;
            while (pend >= hi) {
                k++;
                if (k >= sa.seg_cap) {
                    chain_ok = false;
                    break;
                }
                lo = hi;
                hi = __ldcg(sa.seg_end + k);
                if (hi < lo) {
                    chain_ok = false;
                    break;
                }
            }
            pending = false;
            if (!chain_ok) {
                // cannot happen with a table the host wrote in order; the
                // stream fails instead of reading outside its buffers
                atomicOr(sa.error, kStreamBadChain);
                done = true;
            } else {
                s_k[tid] = k;
                s_lo[tid] = lo;
                s_hi[tid] = hi;
                seq = sa.first_seq + (unsigned long long)k;
                slot = (unsigned)(seq % sa.n_slots);
                const StreamSeg* sg = sa.segs + slot;
                const int n_jobs = __ldcg(&sg->n_jobs);
                const unsigned n_rig = __ldcg(&sg->n_rig);
                const uint64_t* off = ldcg_ptr(&sg->offsets);
                const uint32_t* order = ldcg_ptr(&sg->order);
                uint64_t tl = pend - lo;
                int j;
                uint64_t i;
                if (order) {
                    tl = __ldcg(order + tl);
                    j = find_job_cg(off, n_jobs, tl);
                    i = tl - __ldcg(reinterpret_cast<const unsigned long long*>(off) + j);
                } else if (n_rig && __ldcg(&sg->chunk)) {
                    // warp-wide chunks: the lanes that take consecutive queue
                    // positions trace neighbouring rigidities of one scan
                    const uint64_t W = __ldcg(&sg->chunk), J = (uint64_t)n_jobs, R = n_rig;
                    const uint64_t full = R / W, tf = full * W * J;
                    if (tl < tf) {
                        const uint64_t c = tl / (W * J), rem = tl - c * W * J;
                        j = (int)(rem / W);
                        i = c * W + rem % W;
                    } else {
                        const uint64_t wl = R - full * W, rem = tl - tf;
                        j = (int)(rem / wl);
                        i = full * W + rem % wl;
                    }
                } else if (n_rig) {
                    i = tl / (uint64_t)n_jobs;
                    j = (int)(tl - i * (uint64_t)n_jobs);
                } else {
                    j = find_job_cg(off, n_jobs, tl);
                    i = tl - __ldcg(reinterpret_cast<const unsigned long long*>(off) + j);
                }
                ldcg_copy(&s_job[tid], ldcg_ptr(&sg->jobs) + j);
                const uint64_t oj = __ldcg(reinterpret_cast<const unsigned long long*>(off) + j);
                const int pidx = s_job[tid].param_index;
                if (pidx < 0 || pidx >= sa.n_params) {
                    // finished untraced at the top of the next pass
                    atomicOr(sa.error, kStreamBadParam);
                    L.job_index = j;
                    L.traj = oj + i;
                    L.step = 0;
                    L.trials = 0;
                    bad = true;
                } else {
                    JobTrig tg;
                    ldcg_copy(&tg, ldcg_ptr(&sg->trig) + j);
                    lane_start(L, &s_job[tid], tg, a.params + pidx, j, i, oj + i, a.mass);
                    has = true;
                    need_field = true;
                }
            }
        } else if (pending && pend >= stop) {
            done = true;
            pending = false;
        }
        // block-wide decisions: every thread of the block takes the same branch
        const int n_done = __syncthreads_count(done);
        if (n_done == kTraceThreads) break;
        const int n_live = __syncthreads_count(has);
        if (n_live == 0) {
            // nothing to integrate: wait for the host to publish (or stop), bounded
            bool give_up = false;
            if (tid == 0) {
                const unsigned long long now = global_ns();
                if (!idle_since) idle_since = now;
                give_up = now - idle_since > sa.idle_limit_ns;
            }
            if (__syncthreads_or(give_up)) {
                if (tid == 0) atomicOr(sa.error, kStreamIdle);
                break;
            }
            __nanosleep(20000);
            continue;
        }
        if (tid == 0) idle_since = 0;
        if (a.sort_lanes) {
            // every thread that holds a trajectory needs its field now (it has
            // just started, or just accepted a step): group them by band
            const unsigned key = has ? field_band<MS>(L.gsm, L.par) : 0u;
            regroup_lanes<true>(sc, has, key, L, &s_job[tid], slot, seq, tid);
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
}

}  // namespace cor
