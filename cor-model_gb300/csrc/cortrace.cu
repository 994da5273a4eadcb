// cortrace.cu -- the C ABI of libcortrace.so (include/cor_trace.h) over the
// device kernels in trace.cuh.  Compiled with --fmad=false: see cor_device.cuh.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "trace.cuh"

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
    unsigned long long* queue = nullptr;  // work-queue counter (scratch)
    cor_counters* counters = nullptr;
    const double* crust_g = nullptr;      // device copies of the crustal table
    const double* crust_h = nullptr;
    int crust_nmax = 0;
};

extern "C" {
const char* cor_last_error_string(const cor_ctx* ctx) { return ctx ? ctx->err : "null context"; }
int cor_abi_version(void) { return COR_TRACE_ABI_VERSION; }
}

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
    DevBuf* bufs[] = {&ctx->jobs, &ctx->trig, &ctx->offsets, &ctx->params, &ctx->sites, &ctx->status, &ctx->records};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (ctx->queue) cudaFree(ctx->queue);
    if (ctx->counters) cudaFree(ctx->counters);
    if (ctx->crust_g) cudaFree((void*)ctx->crust_g);
    if (ctx->crust_h) cudaFree((void*)ctx->crust_h);
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
        // src/trajectory.c:7,12: i = 0 .. (int)round((rk-rig)/del)
        const double nr = round((jb.rk - jb.rig) / jb.del);
        if (!(nr >= 0.) || nr > 1e8) return COR_ERR_INVALID;
        if (offsets) offsets[j] = tot;
        tot += (uint64_t)((int)nr) + 1;
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

// ---- dispatch over the compile-time model sets ---------------------------
static bool model_set_ok(const cor_model_set& m) {
    return m.internal_model == COR_INTERNAL_SH && m.external_model == COR_EXTERNAL_NONE &&
           m.crustal_model == COR_CRUSTAL_NONE && m.reserved == 0;
}

template <class MS>
static int launch_trace(cor_ctx* ctx, const TraceArgs& a, cudaStream_t s) {
    int per_sm = 0;
    CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trace_kernel<MS>, 128, 0));
    if (per_sm < 1) per_sm = 1;
    uint64_t blocks = (uint64_t)ctx->sms * (uint64_t)per_sm;
    const uint64_t need = (a.n_traj + 127) / 128;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    trace_kernel<MS><<<(unsigned)blocks, 128, 0, s>>>(a);
    CUDA_TRY(ctx, cudaGetLastError());
    return COR_OK;
}

static int launch_scan(cor_ctx* ctx, const TraceArgs& a, cor_model_set models, cor_site_result* sites, cudaStream_t s) {
    CUDA_TRY(ctx, cudaMemsetAsync(a.queue, 0, sizeof(unsigned long long), s));
    CUDA_TRY(ctx, cudaMemsetAsync(a.counters, 0, sizeof(cor_counters), s));
    if (a.n_traj > 0) {
        int rc = COR_ERR_UNSUPPORTED;
        if (models.internal_model == COR_INTERNAL_SH && models.external_model == COR_EXTERNAL_NONE &&
            models.crustal_model == COR_CRUSTAL_NONE)
            rc = launch_trace<ModelSet<1, 0, 0>>(ctx, a, s);
        if (rc != COR_OK) return rc;
    }
    if (a.n_jobs > 0) {
        const int threads = 256;
        const int blocks = (int)(((int64_t)a.n_jobs * 32 + threads - 1) / threads);
        reduce_kernel<<<blocks, threads, 0, s>>>(a.jobs, a.offsets, a.n_jobs, a.status, sites);
        CUDA_TRY(ctx, cudaGetLastError());
    }
    return COR_OK;
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
                                      const cor_model_params* params_dev, int32_t n_params, cor_model_set models,
                                      uint64_t step_limit, double tu_angle, double particle_mass,
                                      cor_site_result* sites_dev, uint8_t* status_dev, cor_traj_record* records_dev,
                                      cor_counters* counters_dev, void* stream) {
    if (!ctx) return COR_ERR_INVALID;
    int rc = check_req(ctx, models, n_params, step_limit, tu_angle, particle_mass);
    if (rc != COR_OK) return rc;
    if (n_jobs < 0 || (n_jobs > 0 && (!jobs_dev || !trig_dev || !offsets_dev || !sites_dev || !status_dev)))
        return fail(ctx, COR_ERR_INVALID, "missing device buffer (status is required on the device path)");
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    TraceArgs a;
    a.jobs = jobs_dev;
    a.trig = reinterpret_cast<const JobTrig*>(trig_dev);
    a.offsets = offsets_dev;
    a.n_jobs = n_jobs;
    a.n_traj = n_traj;
    a.params = params_dev;
    a.step_limit = step_limit;
    a.tu_angle = tu_angle;
    a.mass = particle_mass;
    a.status = status_dev;
    a.records = records_dev;
    a.queue = ctx->queue;
    a.counters = counters_dev ? counters_dev : ctx->counters;
    a.crust = CrustalTables{ctx->crust_g, ctx->crust_h, ctx->crust_nmax};
    return launch_scan(ctx, a, models, sites_dev, (cudaStream_t)stream);
}

extern "C" int cor_trace_batch(cor_ctx* ctx, const cor_batch_req* req, cor_batch_result* out) {
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
    if (rc == COR_OK) rc = cor_prepare_trig(req->jobs, nj, trig);
    if (rc != COR_OK) {
        free(offsets);
        free(trig);
        return fail(ctx, rc, "invalid rigidity grid in a job");
    }
    cudaStream_t s = ctx->stream;
    do {
        if (cudaSetDevice(ctx->device) != cudaSuccess) { rc = fail(ctx, COR_ERR_CUDA, "cudaSetDevice"); break; }
        if ((rc = ensure(ctx, ctx->jobs, sizeof(cor_scan_job) * (size_t)nj)) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->trig, sizeof(cor_job_trig) * (size_t)nj)) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->offsets, sizeof(uint64_t) * ((size_t)nj + 1))) != COR_OK) break;
        if ((rc = ensure(ctx, ctx->params, sizeof(cor_model_params) * (size_t)req->n_params)) != COR_OK) break;
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
        TRY(cudaMemcpyAsync(ctx->params.p, req->params, sizeof(cor_model_params) * (size_t)req->n_params,
                            cudaMemcpyHostToDevice, s));
        rc = cor_trace_batch_device(ctx, (const cor_scan_job*)ctx->jobs.p, (const cor_job_trig*)ctx->trig.p, nj,
                                    (const uint64_t*)ctx->offsets.p, n_traj, (const cor_model_params*)ctx->params.p,
                                    req->n_params, req->models, req->step_limit, req->tu_angle, req->particle_mass,
                                    (cor_site_result*)ctx->sites.p, (uint8_t*)ctx->status.p,
                                    out->records ? (cor_traj_record*)ctx->records.p : nullptr, ctx->counters, s);
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

extern "C" int cor_field_batch(cor_ctx* ctx, cor_model_set models, const cor_model_params* params, int32_t n_params,
                               const int32_t* param_index, const double* gsm_pos, int64_t n, double* geo_field) {
    if (!ctx) return COR_ERR_INVALID;
    if (!model_set_ok(models))
        return fail(ctx, COR_ERR_UNSUPPORTED, "model set {%d,%d,%d} not available", models.internal_model,
                    models.external_model, models.crustal_model);
    if (n < 0 || n_params < 1 || !params || (n > 0 && (!gsm_pos || !geo_field)))
        return fail(ctx, COR_ERR_INVALID, "bad field request");
    if (n == 0) return COR_OK;
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    void *dp = nullptr, *dpos = nullptr, *dout = nullptr, *didx = nullptr;
    int rc = COR_OK;
    do {
        if (cudaMalloc(&dp, sizeof(cor_model_params) * (size_t)n_params) != cudaSuccess ||
            cudaMalloc(&dpos, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
            cudaMalloc(&dout, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
            (param_index && cudaMalloc(&didx, sizeof(int32_t) * (size_t)n) != cudaSuccess)) {
            rc = fail(ctx, COR_ERR_NOMEM, "device allocation for the field batch");
            break;
        }
        cudaMemcpyAsync(dp, params, sizeof(cor_model_params) * (size_t)n_params, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(dpos, gsm_pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, s);
        if (param_index) cudaMemcpyAsync(didx, param_index, sizeof(int32_t) * (size_t)n, cudaMemcpyHostToDevice, s);
        const int threads = 128;
        const unsigned blocks = (unsigned)((n + threads - 1) / threads);
        field_kernel<ModelSet<1, 0, 0>><<<blocks, threads, 0, s>>>(
            (const cor_model_params*)dp, n_params, (const int32_t*)didx, (const double*)dpos, n, (double*)dout,
            CrustalTables{ctx->crust_g, ctx->crust_h, ctx->crust_nmax});
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
