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

#include "model_ops.h"
#include "reduce.cuh"
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
    if (a.n_traj > 0) {
        const ModelOps* ops = find_ops(models);
        if (!ops) return fail(ctx, COR_ERR_UNSUPPORTED, "model set not available");
        const int rc = launch_trace(ctx, ops, a, s);
        if (rc != COR_OK) return rc;
    }
    unsigned long long launches = a.n_traj > 0 ? (unsigned long long)ctx->generations : 0ull;
    if (a.n_jobs > 0) {
        const int threads = 256;
        const int blocks = (int)(((int64_t)a.n_jobs * 32 + threads - 1) / threads);
        reduce_kernel<<<blocks, threads, 0, s>>>(a.jobs, a.offsets, a.n_jobs, a.status, sites);
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

extern "C" int cor_ctx_set_queue_order(cor_ctx* ctx, int32_t rigidity_major) {
    if (!ctx) return COR_ERR_INVALID;
    if (rigidity_major != 0 && rigidity_major != 1) return fail(ctx, COR_ERR_INVALID, "queue order must be 0 or 1");
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
        reduce_kernel<<<blocks, threads, 0, s>>>(jobs_dev, offsets_dev, n_jobs, status, sites_dev);
        CUDA_TRY(ctx, cudaGetLastError());
        launches++;
    }
    noalloc_launches_kernel<<<1, 1, 0, s>>>(a.counters, launches + 1);
    CUDA_TRY(ctx, cudaGetLastError());
    return COR_OK;
}
