// cortrace.cu -- the C ABI of libcortrace.so (include/cor_trace.h) over the
// device kernels in trace.cuh.  Compiled with --fmad=false: see cor_device.cuh.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <math.h>
#include <chrono>
#include <mutex>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <vector>

#include "model_ops.h"
#include "reduce_kernels.cuh"
#include "model_prep.h"
#include "ts05_tables.h"

extern "C" {
#include "../host/coef_tables.h"
}

using namespace cor;

static_assert(sizeof(cor_job_trig) == sizeof(JobTrig), "trig layout");

namespace {

// A device buffer that only grows.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
};

}  // namespace

struct cor_ctx {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    char err[512] = {0};
    DevBuf jobs, trig, offsets, params, sites, status, records;
    int32_t n_params = 0;                 // resident DevParams blocks (cor_upload_params)
    unsigned long long* queue = nullptr;  // work-queue counter (scratch)
    DevBuf park[2];                       // parked trajectories between generations (scratch)
    GenCounters* gen = nullptr;           // per-generation counters (scratch)
    unsigned int* park_count_host = nullptr;  // pinned readback of the parked count
    unsigned long long* launches_host = nullptr;  // pinned: kernels launched by the last scan
    int generations = 0;                  // generations of the last scan (diagnostics)
    uint64_t gen_live[1024];              // live trajectories at each generation's start
    double gen_ms[1024];                  // host wall time of each generation
    std::chrono::steady_clock::time_point gen_t0;
    cor_counters* counters = nullptr;
    double* crust = nullptr;              // crustal tables: g, h, k1, k2 (packed), kd
    int crust_nmax = 0;
    int crust_n_first = 0;
    int rig_major = 1;                    // queue order for uniform grids (cor_ctx_set_queue_order)
    int sort_lanes = 1;                   // regroup lanes by field band (cor_ctx_set_lane_sort)
    int park_below = 16;                  // regroup settings (cor_ctx_set_regroup)
    int max_generations = 48;
    uint64_t min_park = 256;
    DevBuf steps;                         // trajectory dump: per-step records (cor_trace_steps)
    cor_step_record* step_dev = nullptr;  // set only while cor_trace_steps runs
    uint32_t step_cap = 0;
};

extern "C" {
const char* cor_last_error_string(const cor_ctx* ctx) { return ctx ? ctx->err : "null context"; }
int cor_abi_version(void) { return COR_TRACE_ABI_VERSION; }
}

// NVTX range over a phase of a call (scan, generation, reduction, field
// batch); a no-op unless a profiler is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

static int fail(cor_ctx* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof ctx->err, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CUDA_TRY(ctx, call)                                                                     \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? COR_ERR_NOMEM : COR_ERR_CUDA,  \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);   \
    } while (0)

static int ensure(cor_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes <= b.cap) return COR_OK;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = bytes + bytes / 4 + 256;
    CUDA_TRY(ctx, cudaMalloc(&b.p, want));
    b.cap = want;
    return COR_OK;
}

extern "C" int cor_ctx_create(int device, cor_ctx** out) {
    if (!out) return COR_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return COR_ERR_NODEV;
    }
    if (device < 0 || device >= n) return COR_ERR_INVALID;
    cor_ctx* ctx = new cor_ctx();
    ctx->device = device;
    int rc = COR_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { rc = COR_ERR_CUDA; break; }
        if (cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) { rc = COR_ERR_CUDA; break; }
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = COR_ERR_CUDA; break; }
        if (cudaMalloc(&ctx->queue, 256) != cudaSuccess) { rc = COR_ERR_NOMEM; break; }
        if (cudaMalloc(&ctx->counters, sizeof(cor_counters)) != cudaSuccess) { rc = COR_ERR_NOMEM; break; }
        if (cudaMalloc(&ctx->gen, sizeof(GenCounters)) != cudaSuccess) { rc = COR_ERR_NOMEM; break; }
        if (cudaMallocHost(&ctx->park_count_host, sizeof(unsigned int)) != cudaSuccess) { rc = COR_ERR_NOMEM; break; }
        if (cudaMallocHost(&ctx->launches_host, sizeof(unsigned long long)) != cudaSuccess) { rc = COR_ERR_NOMEM; break; }
        T96Tables tt;
        t96_tables(&tt);
        TS05Tables t5;
        ts05_tables(&t5);
        const ModelOps* all[] = {&ops_igrf, &ops_igrf_t96, &ops_t96, &ops_igrf_ts05, &ops_ts05, &ops_crustal};
        for (const ModelOps* o : all)
            if (o->upload_tables(&tt, &t5) != cudaSuccess) rc = COR_ERR_CUDA;
        if (rc != COR_OK) break;
    } while (0);
    if (rc != COR_OK) {
        cor_ctx_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return COR_OK;
}

extern "C" int cor_ctx_destroy(cor_ctx* ctx) {
    if (!ctx) return COR_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    DevBuf* bufs[] = {&ctx->jobs,   &ctx->trig,    &ctx->offsets, &ctx->params,  &ctx->sites,
                      &ctx->status, &ctx->records, &ctx->park[0], &ctx->park[1], &ctx->steps};
    if (ctx->gen) cudaFree(ctx->gen);
    if (ctx->park_count_host) cudaFreeHost(ctx->park_count_host);
    if (ctx->launches_host) cudaFreeHost(ctx->launches_host);
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (ctx->queue) cudaFree(ctx->queue);
    if (ctx->counters) cudaFree(ctx->counters);
    if (ctx->crust) cudaFree(ctx->crust);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return COR_OK;
}

extern "C" int cor_batch_count(const cor_scan_job* jobs, int32_t n_jobs, uint64_t* n_traj, uint64_t* offsets) {
    if ((!jobs && n_jobs > 0) || n_jobs < 0) return COR_ERR_INVALID;
    uint64_t tot = 0;
    for (int32_t j = 0; j < n_jobs; j++) {
        const cor_scan_job& jb = jobs[j];
        if (!(jb.del > 0.) || !isfinite(jb.rig) || !isfinite(jb.rk)) return COR_ERR_INVALID;
        // The step loop needs a positive nk1 (the turn-angle halving doubles
        // nk0 while nk0 <= 50000) and a finite, non-zero charge and start
        // vectors; the reference does not check these and runs on with
        // inf/NaN or wrapped integers.
        if (jb.nk1 <= 0 || !(jb.zn != 0.) || !isfinite(jb.zn) || !isfinite(jb.r0) || !isfinite(jb.the0) ||
            !isfinite(jb.fi0) || !isfinite(jb.the1) || !isfinite(jb.fi1))
            return COR_ERR_INVALID;
        // src/trajectory.c:7,12: i = 0 .. (int)round((rk-rig)/del)
        const double nr = round((jb.rk - jb.rig) / jb.del);
        if (!(nr >= 0.) || nr > 1e8) return COR_ERR_INVALID;
        const int64_t n_grid = (int64_t)((int)nr) + 1;
        // a window of the grid: indices i_first .. i_first + i_count - 1
        if (jb.i_first < 0 || jb.i_count < 0 || jb.i_first >= n_grid) return COR_ERR_INVALID;
        const int64_t n = jb.i_count ? (int64_t)jb.i_count : n_grid - jb.i_first;
        if ((int64_t)jb.i_first + n > n_grid) return COR_ERR_INVALID;
        if (offsets) offsets[j] = tot;
        tot += (uint64_t)n;
    }
    if (offsets) offsets[n_jobs] = tot;
    if (n_traj) *n_traj = tot;
    return COR_OK;
}

extern "C" int cor_prepare_trig(const cor_scan_job* jobs, int32_t n_jobs, cor_job_trig* out) {
    if ((!jobs || !out) && n_jobs > 0) return COR_ERR_INVALID;
    for (int32_t j = 0; j < n_jobs; j++) {
        // src/trajectory.c:18-28 angles; sin/cos as in sph_to_car (src/utils.c:28-41)
        const double th0 = (90. - jobs[j].the0) * kToRad, ph0 = jobs[j].fi0 * kToRad;
        const double th1 = (90. - jobs[j].the1) * kToRad, ph1 = jobs[j].fi1 * kToRad;
        out[j].st0 = sin(th0);
        out[j].ct0 = cos(th0);
        out[j].sp0 = sin(ph0);
        out[j].cp0 = cos(ph0);
        out[j].st1 = sin(th1);
        out[j].ct1 = cos(th1);
        out[j].sp1 = sin(ph1);
        out[j].cp1 = cos(ph1);
    }
    return COR_OK;
}

// ---- exact turn-angle threshold -------------------------------------------
// The step control rejects a trial iff gc < 1 and
// atan2(sqrt((1-gc)(1+gc)), gc) >= tu_angle (src/trajectory.c:69-73).  As a
// function of the rounded double gc this predicate is a step: true up to some
// largest double, false above.  Find that double with the host C library (the
// library the reference uses) by bisection over the ordered bit patterns of
// [0, 1), then check the step over 4096 neighbours on either side; beyond that
// window the angle differs from tu_angle by far more than any rounding error.
static bool turn_predicate(double gc, double tu) {
    if (!(gc < 1.)) return false;
    const double gs = sqrt((1. - gc) * (1. + gc));
    return atan2(gs, gc) >= tu;
}

static double bits_to_d(uint64_t b) {
    double d;
    memcpy(&d, &b, 8);
    return d;
}

static bool find_turn_threshold(double tu, double* thr) {
    if (!(tu > 1e-6) || !(tu < 1.5)) return false;
    uint64_t lo = 0;  // bits of +0.0: predicate true (angle pi/2)
    double one_m;
    {
        const double one = 1.0;
        uint64_t b;
        memcpy(&b, &one, 8);
        one_m = bits_to_d(b - 1);
    }
    uint64_t hi;
    memcpy(&hi, &one_m, 8);
    if (!turn_predicate(bits_to_d(lo), tu) || turn_predicate(bits_to_d(hi), tu)) return false;
    while (hi - lo > 1) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (turn_predicate(bits_to_d(mid), tu)) lo = mid;
        else hi = mid;
    }
    for (uint64_t k = 0; k < 4096; k++) {
        if (lo >= k && !turn_predicate(bits_to_d(lo - k), tu)) return false;
        if (turn_predicate(bits_to_d(hi + k), tu)) return false;
    }
    *thr = bits_to_d(lo);
    return true;
}

// ---- dispatch over the compile-time model sets ---------------------------
static bool model_set_ok(const cor_model_set& m) {
    const bool in_ok = m.internal_model == COR_INTERNAL_NONE || m.internal_model == COR_INTERNAL_SH;
    const bool ex_ok = m.external_model == COR_EXTERNAL_NONE || m.external_model == COR_EXTERNAL_T96 ||
                       m.external_model == COR_EXTERNAL_TS05;
    const bool cr_ok = m.crustal_model == COR_CRUSTAL_NONE || m.crustal_model == COR_CRUSTAL_CHAOS;
    const bool any = m.internal_model || m.external_model || m.crustal_model;
    return in_ok && ex_ok && cr_ok && any && m.reserved == 0;
}

// The compile-time model set matching m (model_set_ok(m) must hold).
static const ModelOps* find_ops(const cor_model_set& m) {
    if (m.crustal_model != COR_CRUSTAL_NONE) return &ops_crustal;
    const int key = m.internal_model * 100 + m.external_model * 10 + m.crustal_model;
    static const ModelOps* const all[] = {&ops_igrf, &ops_igrf_t96, &ops_t96, &ops_igrf_ts05, &ops_ts05};
    for (const ModelOps* o : all)
        if (o->key == key) return o;
    return nullptr;
}

// Generations of the scan kernel.  Generation 0 drains the work queue; every
// later one restores the trajectories the previous one parked, in a grid
// sized to their count, so the survivors run in full warps.  Each live
// trajectory count at least halves per generation (a block parks with fewer
// than park_below lanes per warp live, or when half the warps have parked), so the loop
// is short; the last generation (the context's max_generations-th, or one
// with at most min_park live trajectories) runs without parking.  The host
// reads the parked count between generations, so this call synchronises the
// stream once per generation.

static int launch_trace(cor_ctx* ctx, const ModelOps* ops, TraceArgs a, cudaStream_t s) {
    int per_sm = 0;
    CUDA_TRY(ctx, ops->occupancy(&per_sm));
    if (per_sm < 1) per_sm = 1;
    const uint64_t cap_blocks = (uint64_t)ctx->sms * (uint64_t)per_sm;
    const size_t park_bytes = sizeof(ParkedLane) * (size_t)cap_blocks * kTraceThreads;
    int rc;
    if ((rc = ensure(ctx, ctx->park[0], park_bytes)) != COR_OK) return rc;
    if ((rc = ensure(ctx, ctx->park[1], park_bytes)) != COR_OK) return rc;
    uint64_t live = a.n_traj;
    uint32_t n_restore = 0;
    int cur = 0;
    ctx->generations = 0;
    for (int g = 0; g < ctx->max_generations && live > 0; g++) {
        // as many blocks as there are warps of work, up to the resident
        // capacity, and that work spread evenly over them
        const uint64_t warps = (live + 31) / 32;
        uint64_t blocks = warps < cap_blocks ? warps : cap_blocks;
        if (blocks < 1) blocks = 1;
        uint64_t per_block = 32 * ((warps + blocks - 1) / blocks);
        if (per_block > (uint64_t)kTraceThreads) per_block = kTraceThreads;
        a.active_threads = (uint32_t)per_block;
        a.restore = g == 0 ? nullptr : (const ParkedLane*)ctx->park[cur ^ 1].p;
        a.n_restore = n_restore;
        a.park = (ParkedLane*)ctx->park[cur].p;
        a.gen = ctx->gen;
        a.allow_park = (g + 1 < ctx->max_generations && live > ctx->min_park) ? 1 : 0;
        a.park_below = ctx->park_below;
        a.launched_warps = (uint32_t)(blocks * kTraceWarps);
        CUDA_TRY(ctx, cudaMemsetAsync(ctx->gen, 0, sizeof(GenCounters), s));
        ctx->gen_t0 = std::chrono::steady_clock::now();
        ctx->gen_live[g] = live;
        ctx->gen_ms[g] = -1.;
        {
            NvtxRange r(g == 0 ? "cor: scan generation 0" : "cor: scan generation (regrouped)");
            CUDA_TRY(ctx, ops->launch_generation(a, (unsigned)blocks, s));
        }
        ctx->generations = g + 1;
        if (!a.allow_park) break;
        CUDA_TRY(ctx, cudaMemcpyAsync(ctx->park_count_host, &ctx->gen->park_count, sizeof(unsigned int),
                                      cudaMemcpyDeviceToHost, s));
        CUDA_TRY(ctx, cudaStreamSynchronize(s));
        ctx->gen_ms[g] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ctx->gen_t0).count();
        n_restore = *ctx->park_count_host;
        live = n_restore;
        cur ^= 1;
    }
    return COR_OK;
}

static int launch_scan(cor_ctx* ctx, const TraceArgs& a, cor_model_set models, cor_site_result* sites, cudaStream_t s) {
    CUDA_TRY(ctx, cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), s));
    CUDA_TRY(ctx, cudaMemsetAsync(a.counters, 0, sizeof(cor_counters), s));
    unsigned long long checks = 0;
    if (a.rig_major && a.grid_ok) {
        grid_check_kernel<<<1, 256, 0, s>>>(a.offsets, a.n_jobs, a.n_traj, const_cast<unsigned int*>(a.grid_ok));
        CUDA_TRY(ctx, cudaGetLastError());
        checks = 1;
    }
    if (a.n_traj > 0) {
        const ModelOps* ops = find_ops(models);
        if (!ops) return fail(ctx, COR_ERR_UNSUPPORTED, "model set not available");
        const int rc = launch_trace(ctx, ops, a, s);
        if (rc != COR_OK) return rc;
    }
    unsigned long long launches = checks + (a.n_traj > 0 ? (unsigned long long)ctx->generations : 0ull);
    if (a.n_jobs > 0) {
        const int threads = 256;
        const int blocks = (int)(((int64_t)a.n_jobs * 32 + threads - 1) / threads);
        reduce_kernel<<<blocks, threads, 0, s>>>(a.jobs, a.offsets, a.n_jobs, a.n_traj, a.status, sites);
        CUDA_TRY(ctx, cudaGetLastError());
        launches += 1;
    }
    // the pinned staging value is read by the copy before the next call can
    // change it: every call on a context synchronises its stream first
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    if (ctx->generations > 0 && ctx->gen_ms[ctx->generations - 1] < 0.)
        ctx->gen_ms[ctx->generations - 1] =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ctx->gen_t0).count();
    *ctx->launches_host = launches;
    CUDA_TRY(ctx, cudaMemcpyAsync(&a.counters->kernel_launches, ctx->launches_host, sizeof(unsigned long long),
                                  cudaMemcpyHostToDevice, s));
    return COR_OK;
}

// ---- crustal model tables --------------------------------------------------
// One device block, built on the host by crustal_block (model_prep.h).
static int upload_crustal(cor_ctx* ctx, const double* g, const double* h, int32_t nmax) {
    if (nmax < 2 || nmax > kChaosMaxN)
        return fail(ctx, COR_ERR_RANGE, "crustal table nmax %d outside [2, %d]", nmax, kChaosMaxN);
    const size_t total = crustal_block_size(nmax);
    double* host = (double*)calloc(total, sizeof(double));
    if (!host) return fail(ctx, COR_ERR_NOMEM, "host allocation");
    const int n_first = crustal_block(g, h, nmax, host);
    int rc = COR_OK;
    double* dev = nullptr;
    do {
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e == cudaSuccess) e = cudaMalloc(&dev, sizeof(double) * total);
        if (e != cudaSuccess) { rc = fail(ctx, COR_ERR_NOMEM, "crustal table: %s", cudaGetErrorString(e)); break; }
        e = cudaMemcpyAsync(dev, host, sizeof(double) * total, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = fail(ctx, COR_ERR_CUDA, "crustal table: %s", cudaGetErrorString(e)); break; }
        if (ctx->crust) cudaFree(ctx->crust);
        ctx->crust = dev;
        dev = nullptr;
        ctx->crust_nmax = nmax;
        ctx->crust_n_first = n_first;
    } while (0);
    if (dev) cudaFree(dev);
    free(host);
    return rc;
}

// The crustal tables for a launch of model set m; the first launch with the
// crustal model uploads the CHAOS-7.16 table unless cor_upload_crustal gave one.
static int crustal_tables(cor_ctx* ctx, const cor_model_set& m, CrustalTables* t) {
    memset(t, 0, sizeof *t);
    if (m.crustal_model == COR_CRUSTAL_NONE) return COR_OK;
    if (!ctx->crust) {
        const int rc = upload_crustal(ctx, cor_chaos716.g, cor_chaos716.h, cor_chaos716.nmax);
        if (rc != COR_OK) return rc;
    }
    const size_t nt = (size_t)ctx->crust_nmax * (size_t)(ctx->crust_nmax + 1) / 2;
    t->g = ctx->crust;
    t->h = ctx->crust + nt;
    t->k1 = ctx->crust + 2 * nt;
    t->k2 = ctx->crust + 3 * nt;
    t->kd = ctx->crust + 4 * nt;
    t->nmax = ctx->crust_nmax;
    t->n_first = ctx->crust_n_first;
    t->internal = m.internal_model;
    t->external = m.external_model;
    return COR_OK;
}

extern "C" int cor_upload_crustal(cor_ctx* ctx, const double* g, const double* h, int32_t nmax) {
    if (!ctx) return COR_ERR_INVALID;
    if (!g || !h) return fail(ctx, COR_ERR_INVALID, "null crustal table");
    return upload_crustal(ctx, g, h, nmax);
}

extern "C" int32_t cor_ctx_generation_log(const cor_ctx* ctx, int32_t cap, uint64_t* live, double* ms) {
    if (!ctx) return COR_ERR_INVALID;
    const int n = ctx->generations;
    for (int g = 0; g < n && g < cap; g++) {
        if (live) live[g] = ctx->gen_live[g];
        if (ms) ms[g] = ctx->gen_ms[g];
    }
    return n;
}

extern "C" int cor_ctx_set_lane_sort(cor_ctx* ctx, int32_t on) {
    if (!ctx) return COR_ERR_INVALID;
    if (on != 0 && on != 1) return fail(ctx, COR_ERR_INVALID, "lane sort must be 0 or 1");
    ctx->sort_lanes = on;
    return COR_OK;
}

extern "C" int cor_ctx_set_queue_order(cor_ctx* ctx, int32_t rigidity_major) {
    if (!ctx) return COR_ERR_INVALID;
    if (rigidity_major < 0 || rigidity_major > 2) return fail(ctx, COR_ERR_INVALID, "queue order must be 0, 1 or 2");
    ctx->rig_major = rigidity_major;
    return COR_OK;
}

extern "C" int cor_ctx_set_regroup(cor_ctx* ctx, int32_t park_below, int32_t max_generations, int64_t min_park) {
    if (!ctx) return COR_ERR_INVALID;
    if (park_below < 0 || park_below > 32 || max_generations < 1 || max_generations > 1024 || min_park < 0)
        return fail(ctx, COR_ERR_INVALID, "regroup settings out of range");
    ctx->park_below = park_below;
    ctx->max_generations = max_generations;
    ctx->min_park = (uint64_t)min_park;
    return COR_OK;
}

extern "C" int cor_upload_params(cor_ctx* ctx, const cor_model_params* params, int32_t n_params) {
    if (!ctx) return COR_ERR_INVALID;
    if (n_params < 1 || !params) return fail(ctx, COR_ERR_INVALID, "no parameter block");
    DevParams* host = (DevParams*)malloc(sizeof(DevParams) * (size_t)n_params);
    if (!host) return fail(ctx, COR_ERR_NOMEM, "host allocation");
    prepare_params(params, n_params, host);
    int rc = COR_OK;
    do {
        if (cudaSetDevice(ctx->device) != cudaSuccess) { rc = fail(ctx, COR_ERR_CUDA, "cudaSetDevice"); break; }
        if ((rc = ensure(ctx, ctx->params, sizeof(DevParams) * (size_t)n_params)) != COR_OK) break;
        cudaError_t e = cudaMemcpyAsync(ctx->params.p, host, sizeof(DevParams) * (size_t)n_params,
                                        cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) { rc = fail(ctx, COR_ERR_CUDA, "parameter upload: %s", cudaGetErrorString(e)); break; }
        ctx->n_params = n_params;
    } while (0);
    free(host);
    return rc;
}

static int check_req(cor_ctx* ctx, const cor_model_set& models, int32_t n_params, uint64_t step_limit, double tu,
                     double mass) {
    if (!model_set_ok(models))
        return fail(ctx, COR_ERR_UNSUPPORTED, "model set {%d,%d,%d} not available", models.internal_model,
                    models.external_model, models.crustal_model);
    if (n_params < 1) return fail(ctx, COR_ERR_INVALID, "no parameter block");
    if (!(tu > 0.) || !(mass > 0.)) return fail(ctx, COR_ERR_INVALID, "tu_angle and particle_mass must be > 0");
    if (step_limit > 0xffffffffull) return fail(ctx, COR_ERR_INVALID, "step_limit above 2^32-1");
    return COR_OK;
}

extern "C" int cor_trace_batch_device(cor_ctx* ctx, const cor_scan_job* jobs_dev, const cor_job_trig* trig_dev,
                                      int32_t n_jobs, const uint64_t* offsets_dev, uint64_t n_traj,
                                      cor_model_set models,
                                      uint64_t step_limit, double tu_angle, double particle_mass,
                                      cor_site_result* sites_dev, uint8_t* status_dev, cor_traj_record* records_dev,
                                      cor_counters* counters_dev, uint32_t flags, void* stream) {
    NvtxRange nvtx_range("cor_trace_batch_device");
    if (!ctx) return COR_ERR_INVALID;
    int rc = check_req(ctx, models, ctx->n_params, step_limit, tu_angle, particle_mass);
    if (rc != COR_OK) return rc;
    if (n_jobs < 0 || (n_jobs > 0 && (!jobs_dev || !trig_dev || !offsets_dev || !sites_dev || !status_dev)))
        return fail(ctx, COR_ERR_INVALID, "missing device buffer (status is required on the device path)");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    TraceArgs a;
    memset(&a, 0, sizeof a);
    a.sort_lanes = ctx->sort_lanes;
    a.step_records = ctx->step_dev;
    a.step_cap = ctx->step_cap;
    a.jobs = jobs_dev;
    a.trig = reinterpret_cast<const JobTrig*>(trig_dev);
    a.offsets = offsets_dev;
    a.n_jobs = n_jobs;
    a.n_traj = n_traj;
    a.params = (const DevParams*)ctx->params.p;
    a.step_limit = step_limit;
    a.tu_angle = tu_angle;
    a.gc_reject = 0.;
    a.turn_exact = find_turn_threshold(tu_angle, &a.gc_reject) ? 1 : 0;
    a.rig_major = 0;
    a.n_rig = 0;
    if (n_jobs > 0 && n_traj % (uint64_t)n_jobs == 0) {
        // rigidity-major queue order needs every scan to have the same count;
        // the uniform-grid check is made on the offsets by the caller
        a.n_rig = (uint32_t)(n_traj / (uint64_t)n_jobs);
    }
    a.mass = particle_mass;
    a.status = status_dev;
    a.records = records_dev;
    a.queue = ctx->queue;
    a.counters = counters_dev ? counters_dev : ctx->counters;
    {
        const int rc = crustal_tables(ctx, models, &a.crust);
        if (rc != COR_OK) return rc;
    }
    a.rig_major = ((flags & COR_FLAG_UNIFORM_GRID) && a.n_rig > 0) ? 1 : 0;
    // the flag is checked on the device against the offsets (grid_check_kernel)
    // in the 256-byte scratch block of the work-queue counter
    a.grid_ok = a.rig_major ? reinterpret_cast<const unsigned int*>(ctx->queue + 1) : nullptr;
    return launch_scan(ctx, a, models, sites_dev, (cudaStream_t)stream);
}

extern "C" int cor_trace_batch(cor_ctx* ctx, const cor_batch_req* req, cor_batch_result* out) {
    NvtxRange nvtx_range("cor_trace_batch");
    if (!ctx || !req || !out) return COR_ERR_INVALID;
    int rc = check_req(ctx, req->models, req->n_params, req->step_limit, req->tu_angle, req->particle_mass);
    if (rc != COR_OK) return rc;
    if (req->n_jobs < 0 || (req->n_jobs > 0 && (!req->jobs || !req->params || !out->sites)))
        return fail(ctx, COR_ERR_INVALID, "missing host buffer");
    for (int32_t j = 0; j < req->n_jobs; j++)
        if (req->jobs[j].param_index < 0 || req->jobs[j].param_index >= req->n_params)
            return fail(ctx, COR_ERR_INVALID, "job %d: param_index %d out of range", j, req->jobs[j].param_index);
    const int32_t nj = req->n_jobs;
    uint64_t* offsets = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)nj + 1));
    cor_job_trig* trig = (cor_job_trig*)malloc(sizeof(cor_job_trig) * ((size_t)nj + 1));
    if (!offsets || !trig) {
        free(offsets);
        free(trig);
        return fail(ctx, COR_ERR_NOMEM, "host allocation");
    }
    uint64_t n_traj = 0;
    rc = cor_batch_count(req->jobs, nj, &n_traj, offsets);
    bool uniform = rc == COR_OK && nj > 0;
    for (int32_t j = 0; uniform && j < nj; j++)
        uniform = offsets[j + 1] - offsets[j] == offsets[1] - offsets[0];

    if (rc == COR_OK) rc = cor_prepare_trig(req->jobs, nj, trig);
    if (rc != COR_OK) {
        free(offsets);
        free(trig);
        return fail(ctx, rc, "invalid job: rigidity grid or window, nk1 <= 0, zero charge or non-finite start");
    }
    cudaStream_t s = ctx->stream;
    do {
        if (cudaSetDevice(ctx->device) != cudaSuccess) { rc = fail(ctx, COR_ERR_CUDA, "cudaSetDevice"); break; }
        if ((rc = ensure(ctx, ctx->jobs, sizeof(cor_scan_job) * (size_t)nj)) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->trig, sizeof(cor_job_trig) * (size_t)nj)) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->offsets, sizeof(uint64_t) * ((size_t)nj + 1))) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->sites, sizeof(cor_site_result) * (size_t)nj)) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->status, (size_t)n_traj)) != COR_OK) break;
        if (out->records && (rc = ensure(ctx, ctx->records, sizeof(cor_traj_record) * (size_t)n_traj)) != COR_OK) break;
#define TRY(call)                                                                                   \
    if ((call) != cudaSuccess) {                                                                    \
        rc = fail(ctx, COR_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(cudaGetLastError()));      \
        break;                                                                                      \
    }
        TRY(cudaMemcpyAsync(ctx->jobs.p, req->jobs, sizeof(cor_scan_job) * (size_t)nj, cudaMemcpyHostToDevice, s));
        TRY(cudaMemcpyAsync(ctx->trig.p, trig, sizeof(cor_job_trig) * (size_t)nj, cudaMemcpyHostToDevice, s));
        TRY(cudaMemcpyAsync(ctx->offsets.p, offsets, sizeof(uint64_t) * ((size_t)nj + 1), cudaMemcpyHostToDevice, s));
        if ((rc = cor_upload_params(ctx, req->params, req->n_params)) != COR_OK) break;
        rc = cor_trace_batch_device(ctx, (const cor_scan_job*)ctx->jobs.p, (const cor_job_trig*)ctx->trig.p, nj,
                                    (const uint64_t*)ctx->offsets.p, n_traj, req->models, req->step_limit,
                                    req->tu_angle, req->particle_mass,
                                    (cor_site_result*)ctx->sites.p, (uint8_t*)ctx->status.p,
                                    out->records ? (cor_traj_record*)ctx->records.p : nullptr, ctx->counters,
                                    (uniform && ctx->rig_major) ? COR_FLAG_UNIFORM_GRID : 0u, s);
        if (rc != COR_OK) break;
        TRY(cudaMemcpyAsync(out->sites, ctx->sites.p, sizeof(cor_site_result) * (size_t)nj, cudaMemcpyDeviceToHost, s));
        if (out->status) TRY(cudaMemcpyAsync(out->status, ctx->status.p, (size_t)n_traj, cudaMemcpyDeviceToHost, s));
        if (out->records)
            TRY(cudaMemcpyAsync(out->records, ctx->records.p, sizeof(cor_traj_record) * (size_t)n_traj,
                                cudaMemcpyDeviceToHost, s));
        TRY(cudaMemcpyAsync(&out->counters, ctx->counters, sizeof(cor_counters), cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
#undef TRY
    } while (0);
    free(offsets);
    free(trig);
    return rc;
}

extern "C" int cor_trace_steps(cor_ctx* ctx, const cor_batch_req* req, cor_batch_result* out, cor_step_record* steps,
                               uint32_t step_capacity) {
    NvtxRange nvtx_range("cor_trace_steps");
    if (!ctx || !req || !out) return COR_ERR_INVALID;
    if (!steps || step_capacity == 0) return fail(ctx, COR_ERR_INVALID, "no step record buffer");
    uint64_t n_traj = 0;
    if (cor_batch_count(req->jobs, req->n_jobs, &n_traj, nullptr) != COR_OK)
        return fail(ctx, COR_ERR_INVALID, "invalid job: rigidity grid or window, nk1 <= 0, zero charge or non-finite start");
    const size_t bytes = sizeof(cor_step_record) * (size_t)n_traj * step_capacity;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int rc = ensure(ctx, ctx->steps, bytes ? bytes : 1);
    if (rc != COR_OK) return rc;
    CUDA_TRY(ctx, cudaMemsetAsync(ctx->steps.p, 0, bytes, ctx->stream));
    ctx->step_dev = (cor_step_record*)ctx->steps.p;
    ctx->step_cap = step_capacity;
    rc = cor_trace_batch(ctx, req, out);
    ctx->step_dev = nullptr;
    ctx->step_cap = 0;
    if (rc != COR_OK) return rc;
    CUDA_TRY(ctx, cudaMemcpy(steps, ctx->steps.p, bytes, cudaMemcpyDeviceToHost));
    return COR_OK;
}

extern "C" int cor_field_batch(cor_ctx* ctx, cor_model_set models, const cor_model_params* params, int32_t n_params,
                               const int32_t* param_index, const double* gsm_pos, int64_t n, double* geo_field) {
    NvtxRange nvtx_range("cor_field_batch");
    if (!ctx) return COR_ERR_INVALID;
    if (!model_set_ok(models))
        return fail(ctx, COR_ERR_UNSUPPORTED, "model set {%d,%d,%d} not available", models.internal_model,
                    models.external_model, models.crustal_model);
    if (n < 0 || n_params < 1 || !params || (n > 0 && (!gsm_pos || !geo_field)))
        return fail(ctx, COR_ERR_INVALID, "bad field request");
    for (int64_t i = 0; param_index && i < n; i++)
        if (param_index[i] < 0 || param_index[i] >= n_params)
            return fail(ctx, COR_ERR_INVALID, "point %lld: param_index %d out of range", (long long)i, param_index[i]);
    if (n == 0) return COR_OK;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    void *dp = nullptr, *dpos = nullptr, *dout = nullptr, *didx = nullptr;
    int rc = COR_OK;
    do {
        if (cudaMalloc(&dp, sizeof(DevParams) * (size_t)n_params) != cudaSuccess ||
            cudaMalloc(&dpos, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
            cudaMalloc(&dout, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
            (param_index && cudaMalloc(&didx, sizeof(int32_t) * (size_t)n) != cudaSuccess)) {
            rc = fail(ctx, COR_ERR_NOMEM, "device allocation for the field batch");
            break;
        }
        DevParams* hp = (DevParams*)malloc(sizeof(DevParams) * (size_t)n_params);
        if (!hp) {
            rc = fail(ctx, COR_ERR_NOMEM, "host allocation");
            break;
        }
        prepare_params(params, n_params, hp);
        cudaMemcpyAsync(dp, hp, sizeof(DevParams) * (size_t)n_params, cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
        free(hp);
        cudaMemcpyAsync(dpos, gsm_pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s);
        if (param_index) cudaMemcpyAsync(didx, param_index, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s);
        CrustalTables crust;
        if ((rc = crustal_tables(ctx, models, &crust)) != COR_OK) break;
        find_ops(models)->launch_field((const DevParams*)dp, n_params, (const int32_t*)didx, (const double*)dpos, n,
                                       (double*)dout, crust, s);
        cudaMemcpyAsync(geo_field, dout, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, s);
        cudaError_t e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) rc = fail(ctx, COR_ERR_CUDA, "field batch: %s", cudaGetErrorString(e));
    } while (0);
    if (dp) cudaFree(dp);
    if (dpos) cudaFree(dpos);
    if (dout) cudaFree(dout);
    if (didx) cudaFree(didx);
    return rc;
}

// ---- FP64 peak probe -------------------------------------------------------
// Eight independent DFMA chains per thread, all operands in registers.
__global__ void fp64_peak_kernel(double* out, int iters, double s) {
    double a[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) a[c] = 1.0 + 1e-9 * (threadIdx.x + c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 8; ++c) a[c] = __fma_rn(a[c], s, 1e-12);
    }
    double t = 0.;
#pragma unroll
    for (int c = 0; c < 8; ++c) t += a[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = t;
}

extern "C" int cor_probe_fp64_peak(cor_ctx* ctx, double* flops_per_s) {
    if (!ctx || !flops_per_s) return COR_ERR_INVALID;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int blocks = ctx->sms * 8, threads = 256, iters = 4000;
    double* out = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, 100, 0.999999);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0, ctx->stream);
        fp64_peak_kernel<<<blocks, threads, 0, ctx->stream>>>(out, iters, 0.999999);
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return fail(ctx, COR_ERR_CUDA, "fp64 probe: %s", cudaGetErrorString(e));
    *flops_per_s = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3);
    return COR_OK;
}

// ---- cost of CUDA's FP64 functions in FMA units ------------------------------
// Each thread evaluates one function on COR_FN_CHAINS independent argument
// streams (seeded host values, stepped by a tiny increment each call) and sums
// the results, so the kernel is throughput-bound like the scan.  Function 0
// is the identity: its time is the loop's own cost (the two adds per call),
// subtracted from every other.
constexpr int kFnChains = 4;
constexpr int kFnArgs = 4096;
constexpr int kFnCount = 11;   // identity, exp, log, sin, cos, atan, asin, atan2, pow, div, sqrt

template <int F>
__device__ __forceinline__ double probe_fn(double x, double y) {
    if constexpr (F == 0) return x;
    else if constexpr (F == 1) return exp(x);
    else if constexpr (F == 2) return log(x);
    else if constexpr (F == 3) return sin(x);
    else if constexpr (F == 4) return cos(x);
    else if constexpr (F == 5) return atan(x);
    else if constexpr (F == 6) return asin(x);
    else if constexpr (F == 7) return atan2(x, y);
    else if constexpr (F == 8) return pow(x, y);
    else if constexpr (F == 9) return x / y;
    else return sqrt(x);
}

template <int F>
__global__ void fp64_fn_kernel(const double* __restrict__ xs, const double* __restrict__ ys, int iters,
                               double* __restrict__ out) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    double x[kFnChains], y[kFnChains], acc[kFnChains];
#pragma unroll
    for (int c = 0; c < kFnChains; ++c) {
        x[c] = xs[(tid * kFnChains + c) % kFnArgs];
        y[c] = ys[(tid * kFnChains + c) % kFnArgs];
        acc[c] = 0.;
    }
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < kFnChains; ++c) {
            acc[c] += probe_fn<F>(x[c], y[c]);
            x[c] += 1e-12;
        }
    }
    double t = 0.;
#pragma unroll
    for (int c = 0; c < kFnChains; ++c) t += acc[c];
    out[tid] = t;
}

using FnKernel = void (*)(const double*, const double*, int, double*);
static const FnKernel kFnKernels[kFnCount] = {fp64_fn_kernel<0>, fp64_fn_kernel<1>, fp64_fn_kernel<2>,
                                              fp64_fn_kernel<3>, fp64_fn_kernel<4>, fp64_fn_kernel<5>,
                                              fp64_fn_kernel<6>, fp64_fn_kernel<7>, fp64_fn_kernel<8>,
                                              fp64_fn_kernel<9>, fp64_fn_kernel<10>};

extern "C" int cor_probe_fp64_functions(cor_ctx* ctx, double* flops_per_call) {
    if (!ctx || !flops_per_call) return COR_ERR_INVALID;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // arguments in the ranges the field models use them (seeded LCG)
    static const double lo[kFnCount] = {-1., -10., 0.05, -12., -12., -10., -0.99, -5., 0.1, -50., 0.};
    static const double hi[kFnCount] = {1., 2., 200., 12., 12., 10., 0.99, 5., 10., 50., 1000.};
    static const double ylo[kFnCount] = {0., 0., 0., 0., 0., 0., 0., -5., -2., 0.5, 0.};
    static const double yhi[kFnCount] = {0., 0., 0., 0., 0., 0., 0., 5., 2., 20., 0.};
    const int blocks = ctx->sms * 8, threads = 256, iters = 256;
    const size_t n_out = (size_t)blocks * threads;
    double *d = nullptr, *hx = nullptr;
    CUDA_TRY(ctx, cudaMalloc(&d, sizeof(double) * (2 * kFnArgs + n_out)));
    hx = (double*)malloc(sizeof(double) * 2 * kFnArgs);
    if (!hx) {
        cudaFree(d);
        return fail(ctx, COR_ERR_NOMEM, "host allocation");
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms[kFnCount];
    cudaError_t e = cudaSuccess;
    uint64_t state = 0x9E3779B97F4A7C15ull;
    for (int f = 0; f < kFnCount && e == cudaSuccess; ++f) {
        for (int k = 0; k < 2 * kFnArgs; ++k) {
            state = state * 6364136223846793005ull + 1442695040888963407ull;
            const double u = (double)(state >> 11) * (1.0 / 9007199254740992.0);
            hx[k] = k < kFnArgs ? lo[f] + u * (hi[f] - lo[f]) : ylo[f] + u * (yhi[f] - ylo[f]);
        }
        e = cudaMemcpy(d, hx, sizeof(double) * 2 * kFnArgs, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) break;
        kFnKernels[f]<<<blocks, threads, 0, ctx->stream>>>(d, d + kFnArgs, 16, d + 2 * kFnArgs);  // warm-up
        float best = 1e30f;
        for (int r = 0; r < 3; r++) {
            cudaEventRecord(e0, ctx->stream);
            kFnKernels[f]<<<blocks, threads, 0, ctx->stream>>>(d, d + kFnArgs, iters, d + 2 * kFnArgs);
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (t < best) best = t;
        }
        ms[f] = best;
        e = cudaGetLastError();
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    free(hx);
    cudaFree(d);
    if (e != cudaSuccess) return fail(ctx, COR_ERR_CUDA, "fp64 function probe: %s", cudaGetErrorString(e));
    double peak = 0.;
    const int rc = cor_probe_fp64_peak(ctx, &peak);
    if (rc != COR_OK) return rc;
    const double calls = (double)n_out * kFnChains * iters;
    flops_per_call[0] = 0.;
    for (int f = 1; f < kFnCount; ++f) flops_per_call[f] = (ms[f] - ms[0]) * 1e-3 * peak / calls;
    return COR_OK;
}

// ---- scan without allocation ------------------------------------------------
// cor_trace_batch_device_noalloc keeps its scratch in one file-scope device
// array instead of context buffers: the work-queue counter, the generation
// counters and the counters block (first 256 bytes), then the per-trajectory
// termination classes the reduction reads (COR_NOALLOC_MAX_TRAJ bytes).  It
// runs the scan as a single generation (no park buffers: those scale with the
// resident threads, ~25 MB) and never calls cudaMalloc or cudaFree.  Every call
// on every context of a device shares the array, so calls that overlap on the
// GPU race on it.
struct NoAllocHead {
    unsigned long long queue;
    unsigned long long pad0[7];
    GenCounters gen;
    unsigned long long pad1[6];
    cor_counters counters;
};
static_assert(sizeof(NoAllocHead) <= 256, "no-alloc scratch header exceeds 256 bytes");
constexpr size_t kNoAllocHead = 256;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocHead + COR_NOALLOC_MAX_TRAJ];

constexpr int kNoAllocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static unsigned char* g_noalloc_ptr[kNoAllocMaxDevices];

// Device address of the scratch array on ctx's device (current); looked up once
// per device, which also loads this library's device code there.
static int noalloc_scratch(cor_ctx* ctx, unsigned char** out) {
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return fail(ctx, COR_ERR_RANGE, "device %d beyond the %d the no-alloc path tracks", ctx->device,
                    kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[ctx->device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return fail(ctx, COR_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
        g_noalloc_ptr[ctx->device] = (unsigned char*)p;
    }
    *out = g_noalloc_ptr[ctx->device];
    return COR_OK;
}

__global__ void noalloc_launches_kernel(cor_counters* c, unsigned long long launches) { c->kernel_launches = launches; }

extern "C" int cor_trace_batch_device_noalloc(cor_ctx* ctx, const cor_scan_job* jobs_dev, const cor_job_trig* trig_dev,
                                              int32_t n_jobs, const uint64_t* offsets_dev, uint64_t n_traj,
                                              cor_model_set models, uint64_t step_limit, double tu_angle,
                                              double particle_mass, cor_site_result* sites_dev,
                                              cor_traj_record* records_dev, cor_counters* counters_dev,
                                              uint32_t flags, void* stream) {
    if (!ctx) return COR_ERR_INVALID;
    int rc = check_req(ctx, models, ctx->n_params, step_limit, tu_angle, particle_mass);
    if (rc != COR_OK) return rc;
    if (n_traj > (uint64_t)COR_NOALLOC_MAX_TRAJ)
        return fail(ctx, COR_ERR_RANGE, "%llu trajectories exceed the no-alloc maximum of %d per call",
                    (unsigned long long)n_traj, COR_NOALLOC_MAX_TRAJ);
    if (n_jobs < 0 || (n_jobs > 0 && (!jobs_dev || !trig_dev || !offsets_dev || !sites_dev)))
        return fail(ctx, COR_ERR_INVALID, "missing device buffer");
    if (models.crustal_model != COR_CRUSTAL_NONE && !ctx->crust)
        return fail(ctx, COR_ERR_INVALID, "crustal table not resident: call cor_upload_crustal first");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    unsigned char* scratch = nullptr;
    if ((rc = noalloc_scratch(ctx, &scratch)) != COR_OK) return rc;
    NoAllocHead* head = (NoAllocHead*)scratch;
    uint8_t* status = scratch + kNoAllocHead;
    cudaStream_t s = (cudaStream_t)stream;

    TraceArgs a;
    memset(&a, 0, sizeof a);
    a.sort_lanes = ctx->sort_lanes;
    a.jobs = jobs_dev;
    a.trig = reinterpret_cast<const JobTrig*>(trig_dev);
    a.offsets = offsets_dev;
    a.n_jobs = n_jobs;
    a.n_traj = n_traj;
    a.params = (const DevParams*)ctx->params.p;
    a.step_limit = step_limit;
    a.tu_angle = tu_angle;
    a.gc_reject = 0.;
    a.turn_exact = find_turn_threshold(tu_angle, &a.gc_reject) ? 1 : 0;
    a.n_rig = 0;
    if (n_jobs > 0 && n_traj % (uint64_t)n_jobs == 0) a.n_rig = (uint32_t)(n_traj / (uint64_t)n_jobs);
    a.rig_major = ((flags & COR_FLAG_UNIFORM_GRID) && a.n_rig > 0) ? 1 : 0;
    a.grid_ok = a.rig_major ? reinterpret_cast<const unsigned int*>(&head->pad0[0]) : nullptr;
    a.mass = particle_mass;
    a.status = status;
    a.records = records_dev;
    a.queue = &head->queue;
    a.counters = counters_dev ? counters_dev : &head->counters;
    a.gen = &head->gen;
    if ((rc = crustal_tables(ctx, models, &a.crust)) != COR_OK) return rc;
    a.restore = nullptr;
    a.n_restore = 0;
    a.park = nullptr;
    a.allow_park = 0;
    a.park_below = 0;

    // the header keeps the previous call's values: clear it
    CUDA_TRY(ctx, cudaMemsetAsync(scratch, 0, kNoAllocHead, s));
    if (counters_dev) CUDA_TRY(ctx, cudaMemsetAsync(counters_dev, 0, sizeof(cor_counters), s));
    unsigned long long launches = 0;
    if (a.rig_major) {
        grid_check_kernel<<<1, 256, 0, s>>>(offsets_dev, n_jobs, n_traj, reinterpret_cast<unsigned int*>(&head->pad0[0]));
        CUDA_TRY(ctx, cudaGetLastError());
        launches++;
    }
    if (n_traj > 0) {
        const ModelOps* ops = find_ops(models);
        if (!ops) return fail(ctx, COR_ERR_UNSUPPORTED, "model set not available");
        int per_sm = 0;
        CUDA_TRY(ctx, ops->occupancy(&per_sm));
        if (per_sm < 1) per_sm = 1;
        const uint64_t cap = (uint64_t)ctx->sms * (uint64_t)per_sm;
        const uint64_t warps = (n_traj + 31) / 32;
        uint64_t blocks = warps < cap ? warps : cap;
        uint64_t per_block = 32 * ((warps + blocks - 1) / blocks);
        if (per_block > (uint64_t)kTraceThreads) per_block = kTraceThreads;
        a.active_threads = (uint32_t)per_block;
        a.launched_warps = (uint32_t)(blocks * kTraceWarps);
        CUDA_TRY(ctx, ops->launch_generation(a, (unsigned)blocks, s));
        launches++;
    }
    if (n_jobs > 0) {
        const int threads = 256;
        const int blocks = (int)(((int64_t)n_jobs * 32 + threads - 1) / threads);
        reduce_kernel<<<blocks, threads, 0, s>>>(jobs_dev, offsets_dev, n_jobs, n_traj, status, sites_dev);
        CUDA_TRY(ctx, cudaGetLastError());
        launches++;
    }
    noalloc_launches_kernel<<<1, 1, 0, s>>>(a.counters, launches + 1);
    CUDA_TRY(ctx, cudaGetLastError());
    return COR_OK;
}

// ---- persistent scan stream (stream.cuh) ------------------------------------
// One launch of stream_kernel serves every segment the caller publishes until
// cor_stream_close (or a restart when the launch's parameter pool or segment
// table is full).  The host writes a segment's inputs and its descriptor with
// copies on the copy stream, waits for them, and only then moves the
// published end forward with a release store into mapped pinned memory; the
// kernel reads that end with an acquire load.  The kernel writes each
// segment's completion record into mapped pinned memory with a release store.
// Nothing here launches other kernels or allocates once the stream exists:
// the stream kernel may hold every SM.

namespace {

struct StreamSlot {
    // device buffers of cor_stream_submit segments, and per-segment scratch
    cor_scan_job* jobs = nullptr;
    JobTrig* trig = nullptr;
    uint64_t* off = nullptr;
    cor_site_result* sites = nullptr;
    uint8_t* status = nullptr;
    cor_traj_record* records = nullptr;
    uint32_t* order = nullptr;
    unsigned int* job_done = nullptr;
    unsigned long long* acc = nullptr;
    // pinned staging
    cor_scan_job* h_jobs = nullptr;
    JobTrig* h_trig = nullptr;
    uint64_t* h_off = nullptr;
    cor_site_result* h_sites = nullptr;
    uint8_t* h_status = nullptr;
    cor_traj_record* h_records = nullptr;
    uint32_t* h_order = nullptr;
    StreamSeg* h_seg = nullptr;
    unsigned long long* h_end = nullptr;
    // state
    int64_t seq = -1;
    bool busy = false;   // submitted and not yet collected
    bool own = false;    // outputs in this slot's buffers (cor_stream_submit)
    bool empty = false;  // a segment without scans: complete at once
    int32_t n_jobs = 0;
    uint64_t n_traj = 0;
};

}  // namespace

struct cor_stream {
    cor_ctx* ctx = nullptr;
    const ModelOps* ops = nullptr;
    cor_stream_config cfg;
    cudaStream_t ks = nullptr;   // the stream kernel
    cudaStream_t cs = nullptr;   // copies
    unsigned blocks = 0;
    StreamSlot* slots = nullptr;
    StreamSeg* segs_dev = nullptr;
    unsigned long long* seg_end_dev = nullptr;
    DevParams* pool_dev = nullptr;     // [fixed_params blocks | pool_params blocks]
    DevParams* h_params = nullptr;     // pinned staging
    int32_t h_params_cap = 0;
    int32_t n_fixed = 0, pool_used = 0;
    unsigned long long* queue_dev = nullptr;
    unsigned long long* h_queue = nullptr;
    void* mapped = nullptr;            // control block, completion records, error word
    StreamCtl* ctl_h = nullptr;
    StreamCtl* ctl_d = nullptr;
    StreamDone* done_h = nullptr;
    StreamDone* done_d = nullptr;
    unsigned int* err_h = nullptr;
    unsigned int* err_d = nullptr;
    bool running = false;
    int64_t next_seq = 0, first_seq = 0;
    uint64_t published = 0, first_index = 0;
    unsigned char* last_params = nullptr;  // the previous submit's blocks (host copy) for reuse
    int32_t last_n = 0, last_base = -1;
    StreamArgs args;
    cor_scan_event* events_h = nullptr;        // mapped: slots x max_jobs per-scan results (scan_events)
    cor_scan_event* events_d = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the current launch, on ks
    bool timed = false;                        // ev0/ev1 hold a launch not yet drained
    bool pending_launch = false;               // launch_on_drain: segments wait for cor_stream_drain
};

extern "C" void cor_stream_config_default(cor_stream_config* c) {
    if (!c) return;
    c->slots = 8;
    c->max_jobs = 16384;
    c->max_trajectories = 2097152;
    c->max_params = 64;
    c->want_records = 0;
    c->reserve_sms = 0;
    c->fixed_params = 256;
    c->pool_params = 4096;
    c->segments_per_launch = 65536;
    c->idle_limit_s = 60.;
    c->launch_on_drain = 0;
    c->scan_events = 0;
    c->sort_lanes = 1;
}

static void stream_free(cor_stream* s) {
    if (!s) return;
    cudaSetDevice(s->ctx->device);
    if (s->slots) {
        for (int k = 0; k < s->cfg.slots; k++) {
            StreamSlot& sl = s->slots[k];
            void* dev[] = {sl.jobs, sl.trig, sl.off, sl.sites, sl.status, sl.records, sl.order, sl.job_done, sl.acc};
            for (void* p : dev)
                if (p) cudaFree(p);
            void* host[] = {sl.h_jobs,    sl.h_trig,  sl.h_off, sl.h_sites, sl.h_status,
                            sl.h_records, sl.h_order, sl.h_seg, sl.h_end};
            for (void* p : host)
                if (p) cudaFreeHost(p);
        }
        delete[] s->slots;
    }
    void* dev[] = {s->segs_dev, s->seg_end_dev, s->pool_dev, s->queue_dev};
    for (void* p : dev)
        if (p) cudaFree(p);
    void* host[] = {s->h_params, s->h_queue, s->mapped, s->events_h};
    for (void* p : host)
        if (p) cudaFreeHost(p);
    free(s->last_params);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->ks) cudaStreamDestroy(s->ks);
    if (s->cs) cudaStreamDestroy(s->cs);
    delete s;
}

extern "C" int cor_stream_create(cor_ctx* ctx, cor_model_set models, uint64_t step_limit, double tu_angle,
                                 double particle_mass, const cor_stream_config* cfg_in, cor_stream** out) {
    if (!ctx || !out) return COR_ERR_INVALID;
    *out = nullptr;
    int rc = check_req(ctx, models, 1, step_limit, tu_angle, particle_mass);
    if (rc != COR_OK) return rc;
    cor_stream_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else cor_stream_config_default(&cfg);
    if (cfg.slots < 1 || cfg.slots > 1024 || cfg.max_jobs < 1 || cfg.max_trajectories < 1 ||
        cfg.max_trajectories > 0xffffffffll || cfg.max_params < 1 ||
        cfg.fixed_params < 0 || cfg.pool_params < cfg.max_params || cfg.segments_per_launch < 1 ||
        cfg.reserve_sms < 0 || cfg.reserve_sms >= ctx->sms || !(cfg.idle_limit_s > 0.) ||
        cfg.idle_limit_s > 86400. || (cfg.want_records != 0 && cfg.want_records != 1) ||
        (cfg.launch_on_drain != 0 && cfg.launch_on_drain != 1) || (cfg.scan_events != 0 && cfg.scan_events != 1) ||
        (cfg.sort_lanes != 0 && cfg.sort_lanes != 1))
        return fail(ctx, COR_ERR_INVALID, "stream configuration out of range");
    const ModelOps* ops = find_ops(models);
    if (!ops) return fail(ctx, COR_ERR_UNSUPPORTED, "model set not available");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int per_sm = 0;
    CUDA_TRY(ctx, ops->stream_occupancy(&per_sm));
    if (per_sm < 1) return fail(ctx, COR_ERR_CUDA, "the stream kernel does not fit on an SM");
    cor_stream* s = new cor_stream();
    s->ctx = ctx;
    s->ops = ops;
    s->cfg = cfg;
    s->blocks = (unsigned)((ctx->sms - cfg.reserve_sms) * per_sm);
    rc = COR_OK;
    do {
#define SALLOC(call)                                                                                \
    if ((call) != cudaSuccess) {                                                                    \
        cudaGetLastError();                                                                         \
        rc = fail(ctx, COR_ERR_NOMEM, "stream allocation: %s", #call);                              \
        break;                                                                                      \
    }
        SALLOC(cudaStreamCreateWithFlags(&s->ks, cudaStreamNonBlocking));
        SALLOC(cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking));
        SALLOC(cudaEventCreate(&s->ev0));
        SALLOC(cudaEventCreate(&s->ev1));
        const size_t nj = (size_t)cfg.max_jobs, nt = (size_t)cfg.max_trajectories;
        SALLOC(cudaMalloc(&s->segs_dev, sizeof(StreamSeg) * (size_t)cfg.slots));
        SALLOC(cudaMalloc(&s->seg_end_dev, sizeof(unsigned long long) * (size_t)cfg.segments_per_launch));
        SALLOC(cudaMalloc(&s->pool_dev, sizeof(DevParams) * (size_t)(cfg.fixed_params + cfg.pool_params)));
        SALLOC(cudaMalloc(&s->queue_dev, 256));
        s->h_params_cap = cfg.max_params > cfg.fixed_params ? cfg.max_params : cfg.fixed_params;
        if (s->h_params_cap < 1) s->h_params_cap = 1;
        SALLOC(cudaHostAlloc(&s->h_params, sizeof(DevParams) * (size_t)s->h_params_cap, cudaHostAllocDefault));
        SALLOC(cudaHostAlloc(&s->h_queue, sizeof(unsigned long long), cudaHostAllocDefault));
        const size_t mbytes = sizeof(StreamCtl) + sizeof(StreamDone) * (size_t)cfg.slots + 64;
        SALLOC(cudaHostAlloc(&s->mapped, mbytes, cudaHostAllocMapped));
        memset(s->mapped, 0, mbytes);
        void* dmapped = nullptr;
        SALLOC(cudaHostGetDevicePointer(&dmapped, s->mapped, 0));
        s->ctl_h = (StreamCtl*)s->mapped;
        s->ctl_d = (StreamCtl*)dmapped;
        s->done_h = (StreamDone*)((char*)s->mapped + sizeof(StreamCtl));
        s->done_d = (StreamDone*)((char*)dmapped + sizeof(StreamCtl));
        s->err_h = (unsigned int*)((char*)s->done_h + sizeof(StreamDone) * (size_t)cfg.slots);
        s->err_d = (unsigned int*)((char*)s->done_d + sizeof(StreamDone) * (size_t)cfg.slots);
        s->ctl_h->stop_at = ~0ull;
        if (cfg.scan_events) {
            const size_t eb = sizeof(cor_scan_event) * (size_t)cfg.slots * nj;
            SALLOC(cudaHostAlloc(&s->events_h, eb, cudaHostAllocMapped));
            memset(s->events_h, 0, eb);
            void* ed = nullptr;
            SALLOC(cudaHostGetDevicePointer(&ed, s->events_h, 0));
            s->events_d = (cor_scan_event*)ed;
        }
        s->last_params = (unsigned char*)malloc(sizeof(cor_model_params) * (size_t)cfg.max_params);
        s->slots = new StreamSlot[cfg.slots];
        if (!s->last_params) {
            rc = fail(ctx, COR_ERR_NOMEM, "host allocation");
            break;
        }
        for (int k = 0; k < cfg.slots && rc == COR_OK; k++) {
            StreamSlot& sl = s->slots[k];
            SALLOC(cudaMalloc(&sl.jobs, sizeof(cor_scan_job) * nj));
            SALLOC(cudaMalloc(&sl.trig, sizeof(JobTrig) * nj));
            SALLOC(cudaMalloc(&sl.off, sizeof(uint64_t) * (nj + 1)));
            SALLOC(cudaMalloc(&sl.sites, sizeof(cor_site_result) * nj));
            SALLOC(cudaMalloc(&sl.status, nt));
            if (cfg.want_records) SALLOC(cudaMalloc(&sl.records, sizeof(cor_traj_record) * nt));
            SALLOC(cudaMalloc(&sl.order, sizeof(uint32_t) * nt));
            SALLOC(cudaMalloc(&sl.job_done, sizeof(unsigned int) * nj));
            SALLOC(cudaMalloc(&sl.acc, 8 * sizeof(unsigned long long)));
            SALLOC(cudaMemset(sl.job_done, 0, sizeof(unsigned int) * nj));
            SALLOC(cudaMemset(sl.acc, 0, 8 * sizeof(unsigned long long)));
            SALLOC(cudaHostAlloc(&sl.h_jobs, sizeof(cor_scan_job) * nj, cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_trig, sizeof(JobTrig) * nj, cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_off, sizeof(uint64_t) * (nj + 1), cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_sites, sizeof(cor_site_result) * nj, cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_status, nt, cudaHostAllocDefault));
            if (cfg.want_records)
                SALLOC(cudaHostAlloc(&sl.h_records, sizeof(cor_traj_record) * nt, cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_order, sizeof(uint32_t) * nt, cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_seg, sizeof(StreamSeg), cudaHostAllocDefault));
            SALLOC(cudaHostAlloc(&sl.h_end, sizeof(unsigned long long), cudaHostAllocDefault));
        }
        if (rc != COR_OK) break;
        SALLOC(cudaDeviceSynchronize());
#undef SALLOC
        StreamArgs& sa = s->args;
        memset(&sa, 0, sizeof sa);
        sa.a.params = s->pool_dev;
        sa.a.step_limit = step_limit;
        sa.a.tu_angle = tu_angle;
        sa.a.gc_reject = 0.;
        sa.a.turn_exact = find_turn_threshold(tu_angle, &sa.a.gc_reject) ? 1 : 0;
        sa.a.mass = particle_mass;
        if ((rc = crustal_tables(ctx, models, &sa.a.crust)) != COR_OK) break;
        sa.ctl = s->ctl_d;
        sa.done = s->done_d;
        sa.error = s->err_d;
        sa.segs = s->segs_dev;
        sa.n_slots = (uint32_t)cfg.slots;
        sa.seg_end = s->seg_end_dev;
        sa.queue = s->queue_dev;
        sa.idle_limit_ns = (unsigned long long)(cfg.idle_limit_s * 1e9);
        sa.seg_cap = cfg.segments_per_launch;
        sa.n_params = cfg.fixed_params + cfg.pool_params;
        sa.a.sort_lanes = cfg.sort_lanes;
    } while (0);
    if (rc != COR_OK) {
        stream_free(s);
        return rc;
    }
    *out = s;
    return COR_OK;
}

// The stream's failure recorded by its kernel in the mapped error word, if any.
static int stream_error(cor_stream* s) {
    const unsigned e = __atomic_load_n(s->err_h, __ATOMIC_ACQUIRE);
    if (e & kStreamBadChain) return fail(s->ctx, COR_ERR_CUDA, "stream kernel found its segment table out of order");
    if (e & kStreamBadParam)
        return fail(s->ctx, COR_ERR_INVALID, "a job's param_index was outside the stream's parameter pool");
    if (e & kStreamIdle)
        return fail(s->ctx, COR_ERR_WATCHDOG, "stream kernel gave up waiting for work (idle limit)");
    return COR_OK;
}

// Lets the running launch finish every published segment, then waits for it.
static int stream_stop(cor_stream* s) {
    if (!s->running) return COR_OK;
    __atomic_store_n(&s->ctl_h->stop_at, s->published, __ATOMIC_RELEASE);
    const cudaError_t e = cudaStreamSynchronize(s->ks);
    s->running = false;
    if (e != cudaSuccess) return fail(s->ctx, COR_ERR_CUDA, "stream kernel: %s", cudaGetErrorString(e));
    return stream_error(s);
}

// Before publishing segment `seq` that brings n_params new parameter blocks:
// restarts the kernel when this launch's segment table or parameter pool is
// full, and fixes the new launch's first segment and queue index.
static int stream_prepare_launch(cor_stream* s, int64_t seq, int32_t n_params_new) {
    const bool full = (seq - s->first_seq) >= (int64_t)s->cfg.segments_per_launch ||
                      s->pool_used + n_params_new > s->cfg.pool_params;
    if (s->pending_launch) {
        // launch_on_drain: the staged segments belong to the next launch
        if (full) return fail(s->ctx, COR_ERR_BUSY, "the staged launch is full: drain it first");
        return COR_OK;
    }
    if (s->running && full) {
        const int rc = stream_stop(s);
        if (rc != COR_OK) return rc;
    }
    if (!s->running) {
        const int rc = stream_error(s);
        if (rc != COR_OK) return rc;
        s->first_seq = seq;
        s->first_index = s->published;
        s->pool_used = 0;
        s->last_base = -1;
    }
    return COR_OK;
}

// Launches the stream kernel from the launch's first segment and queue index,
// with the stop index given (~0: running until stopped), between two events.
static int stream_launch(cor_stream* s, unsigned long long stop_at) {
    cor_ctx* ctx = s->ctx;
    *s->h_queue = s->first_index;
    __atomic_store_n(s->err_h, 0u, __ATOMIC_RELAXED);
    __atomic_store_n(&s->ctl_h->stop_at, stop_at, __ATOMIC_RELEASE);
    CUDA_TRY(ctx, cudaMemcpyAsync(s->queue_dev, s->h_queue, sizeof(unsigned long long), cudaMemcpyHostToDevice, s->ks));
    s->args.first_seq = (unsigned long long)s->first_seq;
    s->args.first_index = s->first_index;
    CUDA_TRY(ctx, cudaEventRecord(s->ev0, s->ks));
    CUDA_TRY(ctx, s->ops->launch_stream(s->args, s->blocks, s->ks));
    CUDA_TRY(ctx, cudaEventRecord(s->ev1, s->ks));
    s->running = true;
    s->timed = true;
    return COR_OK;
}

// Copies the segment's descriptor and end (and, for cor_stream_submit, its
// inputs, already queued on cs), waits for the copies, launches the kernel if
// needed and moves the published end.
static int stream_publish(cor_stream* s, StreamSlot& sl, int64_t seq, uint64_t n_traj) {
    cor_ctx* ctx = s->ctx;
    const unsigned slot = (unsigned)(seq % s->cfg.slots);
    *sl.h_end = s->published + n_traj;
    CUDA_TRY(ctx, cudaMemcpyAsync(s->segs_dev + slot, sl.h_seg, sizeof(StreamSeg), cudaMemcpyHostToDevice, s->cs));
    CUDA_TRY(ctx, cudaMemcpyAsync(s->seg_end_dev + (seq - s->first_seq), sl.h_end, sizeof(unsigned long long),
                                  cudaMemcpyHostToDevice, s->cs));
    CUDA_TRY(ctx, cudaStreamSynchronize(s->cs));
    if (!s->running && !s->cfg.launch_on_drain) {
        const int rc = stream_launch(s, ~0ull);
        if (rc != COR_OK) return rc;
    }
    s->published += n_traj;
    __atomic_store_n(&s->ctl_h->published, s->published, __ATOMIC_RELEASE);
    if (s->cfg.launch_on_drain) s->pending_launch = true;
    sl.seq = seq;
    sl.busy = true;
    sl.n_traj = n_traj;
    s->next_seq = seq + 1;
    return COR_OK;
}

// Warp-wide chunk of the queue orders that keep neighbouring rigidities of a
// scan together (cor_ctx_set_queue_order mode 2).
constexpr uint32_t kQueueChunk = 32;

// The batch's trajectories (offsets space) in ascending rigidity, lowest
// first, in chunks of `chunk` consecutive trajectories of one scan (the
// chunk's key is its first rigidity; chunk 1 = trajectory by trajectory);
// ties keep the batch order.
static void rigidity_order(const cor_scan_job* jobs, int32_t n_jobs, const uint64_t* off, uint32_t chunk,
                           uint32_t* order) {
    std::vector<std::pair<double, uint64_t>> keys;   // (first rigidity, first trajectory) per chunk
    for (int32_t j = 0; j < n_jobs; j++)
        for (uint64_t k = 0; k < off[j + 1] - off[j]; k += chunk)
            keys.emplace_back(jobs[j].rig + (int)(k + (uint64_t)jobs[j].i_first) * jobs[j].del, off[j] + k);
    std::stable_sort(keys.begin(), keys.end(),
                     [](const std::pair<double, uint64_t>& a, const std::pair<double, uint64_t>& b) {
                         return a.first < b.first;
                     });
    uint64_t o = 0;
    for (const auto& kv : keys) {
        const int32_t j = (int32_t)(std::upper_bound(off, off + n_jobs + 1, kv.second) - off) - 1;
        const uint64_t end = std::min<uint64_t>(kv.second + chunk, off[j + 1]);
        for (uint64_t t = kv.second; t < end; t++) order[o++] = (uint32_t)t;
    }
}

static bool offsets_uniform(const uint64_t* off, int32_t n_jobs) {
    if (n_jobs < 1) return false;
    for (int32_t j = 0; j < n_jobs; j++)
        if (off[j + 1] - off[j] != off[1] - off[0]) return false;
    return true;
}

extern "C" int cor_stream_submit(cor_stream* s, const cor_scan_job* jobs, int32_t n_jobs,
                                 const cor_model_params* params, int32_t n_params, int64_t* ticket) {
    if (!s || !ticket) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    NvtxRange nvtx_range("cor_stream_submit");
    if (n_jobs < 0 || n_jobs > s->cfg.max_jobs || (n_jobs > 0 && (!jobs || !params)) || n_params < 0 ||
        n_params > s->cfg.max_params || (n_jobs > 0 && n_params < 1))
        return fail(ctx, COR_ERR_INVALID, "stream submit: %d scans, %d parameter blocks (limits %d, %d)", n_jobs,
                    n_params, s->cfg.max_jobs, s->cfg.max_params);
    for (int32_t j = 0; j < n_jobs; j++)
        if (jobs[j].param_index < 0 || jobs[j].param_index >= n_params)
            return fail(ctx, COR_ERR_INVALID, "job %d: param_index %d out of range", j, jobs[j].param_index);
    const int64_t seq = s->next_seq;
    StreamSlot& sl = s->slots[seq % s->cfg.slots];
    if (sl.busy) return fail(ctx, COR_ERR_BUSY, "stream slot of segment %lld still holds uncollected segment %lld",
                             (long long)seq, (long long)sl.seq);
    uint64_t n_traj = 0;
    if (cor_batch_count(jobs, n_jobs, &n_traj, sl.h_off) != COR_OK)
        return fail(ctx, COR_ERR_INVALID, "invalid job: rigidity grid or window, nk1 <= 0, zero charge or non-finite start");
    if (n_traj > (uint64_t)s->cfg.max_trajectories)
        return fail(ctx, COR_ERR_RANGE, "%llu trajectories exceed the stream's %lld per segment",
                    (unsigned long long)n_traj, (long long)s->cfg.max_trajectories);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    sl.own = true;
    sl.n_jobs = n_jobs;
    if (n_jobs == 0) {
        // no trajectories: complete at once, but keep the segment chain the
        // kernel walks whole (its end equals its base)
        int rc = stream_prepare_launch(s, seq, 0);
        if (rc != COR_OK) return rc;
        *sl.h_end = s->published;
        CUDA_TRY(ctx, cudaMemcpyAsync(s->seg_end_dev + (seq - s->first_seq), sl.h_end, sizeof(unsigned long long),
                                      cudaMemcpyHostToDevice, s->cs));
        CUDA_TRY(ctx, cudaStreamSynchronize(s->cs));
        sl.empty = true;
        sl.busy = true;
        sl.seq = seq;
        sl.n_traj = 0;
        s->next_seq = seq + 1;
        *ticket = seq;
        return COR_OK;
    }
    sl.empty = false;
    const size_t pbytes = sizeof(cor_model_params) * (size_t)n_params;
    const bool reuse = s->running && s->last_base >= 0 && s->last_n == n_params &&
                       memcmp(s->last_params, params, pbytes) == 0 &&
                       (seq - s->first_seq) < (int64_t)s->cfg.segments_per_launch;
    int rc = stream_prepare_launch(s, seq, reuse ? 0 : n_params);
    if (rc != COR_OK) return rc;
    int32_t base;
    if (reuse && s->last_base >= 0) {
        base = s->last_base;
    } else {
        base = s->cfg.fixed_params + s->pool_used;
        prepare_params(params, n_params, s->h_params);
        CUDA_TRY(ctx, cudaMemcpyAsync(s->pool_dev + base, s->h_params, sizeof(DevParams) * (size_t)n_params,
                                      cudaMemcpyHostToDevice, s->cs));
        s->pool_used += n_params;
        memcpy(s->last_params, params, pbytes);
        s->last_n = n_params;
        s->last_base = base;
    }
    memcpy(sl.h_jobs, jobs, sizeof(cor_scan_job) * (size_t)n_jobs);
    for (int32_t j = 0; j < n_jobs; j++) sl.h_jobs[j].param_index += base;
    cor_prepare_trig(jobs, n_jobs, reinterpret_cast<cor_job_trig*>(sl.h_trig));
    StreamSeg& g = *sl.h_seg;
    g.jobs = sl.jobs;
    g.trig = sl.trig;
    g.offsets = sl.off;
    g.status = sl.status;
    g.records = sl.records;
    g.sites = sl.sites;
    g.job_done = sl.job_done;
    g.acc = sl.acc;
    g.base = s->published;
    g.n_traj = n_traj;
    g.seq = (unsigned long long)seq;
    g.n_jobs = n_jobs;
    g.n_rig = (offsets_uniform(sl.h_off, n_jobs) && s->ctx->rig_major) ? (uint32_t)(sl.h_off[1] - sl.h_off[0]) : 0u;
    g.chunk = (g.n_rig && s->ctx->rig_major == 2) ? kQueueChunk : 0u;
    g.order = nullptr;
    g.events = s->events_d ? s->events_d + (size_t)(seq % s->cfg.slots) * (size_t)s->cfg.max_jobs : nullptr;
    if (!g.n_rig && s->ctx->rig_major && n_jobs > 1) {
        // scans of different lengths: hand out all their trajectories in
        // ascending rigidity, as the rigidity-major order does for a uniform
        // grid (the lowest rigidities are the longest trajectories)
        rigidity_order(jobs, n_jobs, sl.h_off, s->ctx->rig_major == 2 ? kQueueChunk : 1u, sl.h_order);
        CUDA_TRY(ctx, cudaMemcpyAsync(sl.order, sl.h_order, sizeof(uint32_t) * n_traj, cudaMemcpyHostToDevice, s->cs));
        g.order = sl.order;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(sl.jobs, sl.h_jobs, sizeof(cor_scan_job) * (size_t)n_jobs, cudaMemcpyHostToDevice, s->cs));
    CUDA_TRY(ctx, cudaMemcpyAsync(sl.trig, sl.h_trig, sizeof(JobTrig) * (size_t)n_jobs, cudaMemcpyHostToDevice, s->cs));
    CUDA_TRY(ctx, cudaMemcpyAsync(sl.off, sl.h_off, sizeof(uint64_t) * ((size_t)n_jobs + 1), cudaMemcpyHostToDevice, s->cs));
    if ((rc = stream_publish(s, sl, seq, n_traj)) != COR_OK) return rc;
    *ticket = seq;
    return COR_OK;
}

extern "C" int cor_stream_upload_params(cor_stream* s, const cor_model_params* params, int32_t n_params,
                                        int32_t* first_index) {
    if (!s || !first_index) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    if (!params || n_params < 1 || n_params > s->cfg.fixed_params - s->n_fixed)
        return fail(ctx, COR_ERR_RANGE, "%d parameter blocks do not fit the stream's fixed pool (%d of %d used)",
                    n_params, s->n_fixed, s->cfg.fixed_params);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    prepare_params(params, n_params, s->h_params);
    CUDA_TRY(ctx, cudaMemcpyAsync(s->pool_dev + s->n_fixed, s->h_params, sizeof(DevParams) * (size_t)n_params,
                                  cudaMemcpyHostToDevice, s->cs));
    CUDA_TRY(ctx, cudaStreamSynchronize(s->cs));
    *first_index = s->n_fixed;
    s->n_fixed += n_params;
    return COR_OK;
}

extern "C" int cor_stream_submit_device(cor_stream* s, const cor_scan_job* jobs_dev, const cor_job_trig* trig_dev,
                                        const uint64_t* offsets_dev, const uint64_t* offsets_host, int32_t n_jobs,
                                        cor_site_result* sites_dev, uint8_t* status_dev,
                                        cor_traj_record* records_dev, int64_t* ticket) {
    if (!s || !ticket) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    NvtxRange nvtx_range("cor_stream_submit_device");
    if (n_jobs < 1 || n_jobs > s->cfg.max_jobs || !jobs_dev || !trig_dev || !offsets_dev || !offsets_host ||
        !sites_dev || !status_dev)
        return fail(ctx, COR_ERR_INVALID, "stream device submit: missing buffer or %d scans (limit %d)", n_jobs,
                    s->cfg.max_jobs);
    if (s->n_fixed < 1) return fail(ctx, COR_ERR_INVALID, "no parameter blocks: call cor_stream_upload_params first");
    if (offsets_host[0] != 0) return fail(ctx, COR_ERR_INVALID, "offsets must start at 0");
    for (int32_t j = 0; j < n_jobs; j++)
        if (offsets_host[j + 1] <= offsets_host[j])
            return fail(ctx, COR_ERR_INVALID, "offsets must increase (scan %d has no trajectory)", j);
    const uint64_t n_traj = offsets_host[n_jobs];
    const int64_t seq = s->next_seq;
    StreamSlot& sl = s->slots[seq % s->cfg.slots];
    if (sl.busy) return fail(ctx, COR_ERR_BUSY, "stream slot of segment %lld still holds uncollected segment %lld",
                             (long long)seq, (long long)sl.seq);
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    int rc = stream_prepare_launch(s, seq, 0);
    if (rc != COR_OK) return rc;
    sl.own = false;
    sl.empty = false;
    sl.n_jobs = n_jobs;
    StreamSeg& g = *sl.h_seg;
    g.jobs = jobs_dev;
    g.trig = reinterpret_cast<const JobTrig*>(trig_dev);
    g.offsets = offsets_dev;
    g.status = status_dev;
    g.records = records_dev;
    g.sites = sites_dev;
    g.job_done = sl.job_done;
    g.acc = sl.acc;
    g.base = s->published;
    g.n_traj = n_traj;
    g.seq = (unsigned long long)seq;
    g.n_jobs = n_jobs;
    g.n_rig = (offsets_uniform(offsets_host, n_jobs) && s->ctx->rig_major) ? (uint32_t)offsets_host[1] : 0u;
    g.chunk = (g.n_rig && s->ctx->rig_major == 2) ? kQueueChunk : 0u;
    g.order = nullptr;
    g.events = nullptr;
    if ((rc = stream_publish(s, sl, seq, n_traj)) != COR_OK) return rc;
    *ticket = seq;
    return COR_OK;
}

extern "C" int cor_stream_wait(cor_stream* s, int64_t ticket, int32_t timeout_ms, cor_batch_result* out,
                               uint64_t* t_done_ns) {
    if (!s) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    if (ticket < 0 || ticket >= s->next_seq) return fail(ctx, COR_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
    const unsigned slot = (unsigned)(ticket % s->cfg.slots);
    StreamSlot& sl = s->slots[slot];
    if (!sl.busy || sl.seq != ticket)
        return fail(ctx, COR_ERR_INVALID, "ticket %lld is not outstanding", (long long)ticket);
    if (sl.own && !sl.empty && (!out || !out->sites))
        return fail(ctx, COR_ERR_INVALID, "a submitted segment's results need out->sites");
    if (sl.empty) {
        if (out) memset(&out->counters, 0, sizeof(cor_counters));
        if (t_done_ns) *t_done_ns = 0;
        sl.busy = false;
        return COR_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        if (__atomic_load_n(&s->done_h[slot].seq1, __ATOMIC_ACQUIRE) == (unsigned long long)ticket + 1) break;
        if (__atomic_load_n(s->err_h, __ATOMIC_ACQUIRE)) return stream_error(s);
        if (s->pending_launch)
            return fail(ctx, COR_ERR_INVALID, "segment %lld waits for cor_stream_drain (launch_on_drain)",
                        (long long)ticket);
        if (s->running) {
            const cudaError_t e = cudaStreamQuery(s->ks);
            if (e == cudaSuccess) {
                s->running = false;
                if (__atomic_load_n(&s->done_h[slot].seq1, __ATOMIC_ACQUIRE) == (unsigned long long)ticket + 1) break;
                return fail(ctx, COR_ERR_CUDA, "stream kernel ended before segment %lld completed", (long long)ticket);
            }
            if (e != cudaErrorNotReady) return fail(ctx, COR_ERR_CUDA, "stream kernel: %s", cudaGetErrorString(e));
        } else {
            return fail(ctx, COR_ERR_CUDA, "stream kernel is not running and segment %lld did not complete",
                        (long long)ticket);
        }
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (timeout_ms >= 0 && ms >= (double)timeout_ms) return COR_PENDING;
        timespec ts = {0, 20000};
        nanosleep(&ts, nullptr);
    }
    if (__atomic_load_n(s->err_h, __ATOMIC_ACQUIRE) & kStreamBadParam) {
        sl.busy = false;
        return stream_error(s);
    }
    const StreamDone& d = s->done_h[slot];
    if (t_done_ns) *t_done_ns = d.t_ns;
    if (out) {
        out->counters.accepted_steps = d.steps;
        out->counters.trials = d.trials;
        out->counters.trajectories = d.traj;
        out->counters.watchdog = d.watchdog;
        out->counters.kernel_launches = 1;
        if (sl.own) {
            CUDA_TRY(ctx, cudaSetDevice(ctx->device));
            CUDA_TRY(ctx, cudaMemcpyAsync(sl.h_sites, sl.sites, sizeof(cor_site_result) * (size_t)sl.n_jobs,
                                          cudaMemcpyDeviceToHost, s->cs));
            if (out->status)
                CUDA_TRY(ctx, cudaMemcpyAsync(sl.h_status, sl.status, sl.n_traj, cudaMemcpyDeviceToHost, s->cs));
            if (out->records && sl.h_records)
                CUDA_TRY(ctx, cudaMemcpyAsync(sl.h_records, sl.records, sizeof(cor_traj_record) * sl.n_traj,
                                              cudaMemcpyDeviceToHost, s->cs));
            CUDA_TRY(ctx, cudaStreamSynchronize(s->cs));
            memcpy(out->sites, sl.h_sites, sizeof(cor_site_result) * (size_t)sl.n_jobs);
            if (out->status) memcpy(out->status, sl.h_status, sl.n_traj);
            if (out->records && sl.h_records) memcpy(out->records, sl.h_records, sizeof(cor_traj_record) * sl.n_traj);
        }
    }
    sl.busy = false;
    return COR_OK;
}

extern "C" int cor_stream_poll_scans(cor_stream* s, int64_t ticket, int32_t first, int32_t count, uint8_t* done,
                                     cor_scan_event* events) {
    if (!s) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    if (!s->events_h) return fail(ctx, COR_ERR_INVALID, "the stream was created without scan_events");
    if (ticket < 0 || ticket >= s->next_seq) return fail(ctx, COR_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
    const unsigned slot = (unsigned)(ticket % s->cfg.slots);
    const StreamSlot& sl = s->slots[slot];
    if (!sl.busy || sl.seq != ticket || !sl.own)
        return fail(ctx, COR_ERR_INVALID, "ticket %lld is not an outstanding cor_stream_submit segment",
                    (long long)ticket);
    if (first < 0 || count < 0 || (int64_t)first + count > sl.n_jobs)
        return fail(ctx, COR_ERR_INVALID, "scans %d .. %d outside the segment's %d", first, first + count - 1,
                    sl.n_jobs);
    const cor_scan_event* base = s->events_h + (size_t)slot * (size_t)s->cfg.max_jobs;
    int n = 0;
    for (int32_t k = 0; k < count; k++) {
        const cor_scan_event* e = base + first + k;
        const bool d = sl.empty ? false
                                : __atomic_load_n(&e->seq1, __ATOMIC_ACQUIRE) == (unsigned long long)ticket + 1;
        if (done) done[k] = d ? 1 : 0;
        if (d) {
            n++;
            if (events) memcpy(&events[k], e, sizeof(cor_scan_event));
        }
    }
    return n;
}

extern "C" int cor_stream_drain(cor_stream* s, double* launch_ms) {
    if (!s) return COR_ERR_INVALID;
    cor_ctx* ctx = s->ctx;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (launch_ms) *launch_ms = 0.;
    if (s->pending_launch) {
        s->pending_launch = false;
        const int rc = stream_launch(s, s->published);
        if (rc != COR_OK) return rc;
    }
    const int rc = stream_stop(s);
    if (rc != COR_OK) return rc;
    if (s->timed) {
        float ms = 0.f;
        CUDA_TRY(ctx, cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        s->timed = false;
        if (launch_ms) *launch_ms = ms;
    }
    return COR_OK;
}

extern "C" int cor_stream_close(cor_stream* s) {
    if (!s) return COR_OK;
    cudaSetDevice(s->ctx->device);
    int rc = COR_OK;
    if (s->pending_launch) {
        // staged segments of a launch_on_drain stream still run, so that the
        // caller's device buffers are never left half written
        s->pending_launch = false;
        rc = stream_launch(s, s->published);
    }
    const int rc2 = stream_stop(s);
    if (rc == COR_OK) rc = rc2;
    stream_free(s);
    return rc;
}
