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
    int32_t n_params = 0;                 // resident DevParams blocks (cor_upload_params)
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

// ---- host-derived model constants -----------------------------------------
// Per-condition quantities of t96_gsm that depend only on PARMOD
// (lib/t96/t96.c:5-31, :52-58), with the reference's expressions and the
// host C library.
static void t96_prepare(const double* parmod, T96Cond* c) {
    const double pdyn = parmod[0];
    const double depr = 0.8 * parmod[1] - 13.0 * sqrt(pdyn);
    const double byimf = parmod[2], bzimf = parmod[3];
    const double bt = sqrt(byimf * byimf + bzimf * bzimf);
    double theta = 0.0;
    if (byimf != 0.0 || bzimf != 0.0) {
        theta = atan2(byimf, bzimf);
        if (theta <= 0.0) theta += 6.2831853;
    }
    c->ct = cos(theta);
    c->st = sin(theta);
    const double eps = 718.5 * sqrt(pdyn) * bt * sin(theta / 2.);
    c->kimfy = 0.7850 * byimf;
    c->kimfz = 0.7850 * bzimf;
    c->xappa = pow(pdyn / 2.0, 0.14);
    c->xappa3 = c->xappa * c->xappa * c->xappa;
    c->am = 70.0 / c->xappa;
    c->c548 = 5.48 / c->xappa;
    c->asq = c->am * c->am;
    c->four_asq = 4.0 * c->asq;
    c->two_asq = 2.0 * c->asq;
    c->r_two_asq = 1.0 / c->two_asq;
    const double factes = eps / 3630.7 - 1.0;
    const double factpd = sqrt(pdyn / 2.0) - 1.0;
    c->rcampl = -1.162 * depr;
    c->tampl2 = 22.344 + 18.50 * factpd + 2.602 * factes;
    c->tampl3 = 6.903 + 5.287 * factpd;
    c->b1ampl = 0.5790 + 0.4462 * factes;
    c->b2ampl = 20.0 * c->b1ampl;
    c->rimfampl = 0.7850 * bt;
}

// Position-independent constants of the T96 terms: the square roots of the
// shielding mode scales (shlcar3x3_t96 :514, birk1shld :1045, birk2shl :1208,
// intercon :255), sin/cos of the fixed loop tilts (crosslp :890, loops4
// :1446), and the r2sheet factors (:1513-1551).
static void t96_tables(T96Tables* t) {
    const double P[3][3] = {{12.75434981, 11.37659788, 636.4346279},
                            {5.187666221, 6.802472048, 39.13543412},
                            {19.69877970, 20.30095680, 86.45407420}};
    const double R[3][3] = {{1.752483754, 3.604231143, 12.83078674},
                            {2.784722096, 6.979576616, 25.71716760},
                            {22.50403727, 23.41617329, 48.48140573}};
    for (int m = 0; m < 3; m++)
        for (int i = 0; i < 3; i++) {
            const double pp = 1.0 / (P[m][i] * P[m][i]);
            for (int k = 0; k < 3; k++) t->shl_sq[m][3 * i + k] = sqrt(pp + 1.0 / (R[m][k] * R[m][k]));
        }
    const double PS[4] = {5.303648988, 10.40368955, 69.65230348, 466.5099509};
    const double RS[4] = {1.645049286, 3.825838190, 11.66675599, 558.9781177};
    for (int i = 0; i < 4; i++) {
        const double rpi = 1.0 / PS[i];
        const double rpi2 = rpi * rpi;
        for (int k = 0; k < 4; k++) {
            const double rk = 1.0 / RS[k];
            t->b1s_sq[4 * i + k] = sqrt(rpi2 + rk * rk);
        }
    }
    const double AI[2] = {13.85650567, 14.90554500}, AK[2] = {10.21914434, 10.09021632};
    for (int i = 0; i < 2; i++) {
        const double aiai = 1.0 / (AI[i] * AI[i]);
        for (int k = 0; k < 2; k++) t->b2s_sq[2 * i + k] = sqrt(aiai + 1.0 / (AK[k] * AK[k]));
    }
    const double RP[3] = {0.12503844191332988, 0.071597395204476152, 0.011080976889832743};
    const double RR[3] = {0.059675527522452816, 0.00098459526668325296, 0.00064371058922777988};
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) t->ic_sq[3 * i + k] = sqrt(RP[i] * RP[i] + RR[k] * RR[k]);
    const double AL[4] = {1.00891, 0.0031, 0.1375, 0.9625};
    for (int i = 0; i < 4; i++) {
        t->cross_cs[i][0] = cos(AL[i]);
        t->cross_cs[i][1] = sin(AL[i]);
    }
    const double TH[2] = {.8573, 0.4312}, PH[2] = {3.0986, 1.55};
    for (int i = 0; i < 2; i++) {
        t->loop_cs[i][0] = sin(TH[i]);
        t->loop_cs[i][1] = cos(TH[i]);
        t->loop_cs[i][2] = sin(PH[i]);
        t->loop_cs[i][3] = cos(PH[i]);
    }
    const double stmp = -2. * 2.718281828459;
    t->r2s_k[0] = sqrt(stmp * -19.0969);
    t->r2s_k[1] = sqrt(stmp * -9.28828);
    t->r2s_k[2] = sqrt(stmp * -0.129687);
    t->r2s_k[3] = sqrt(stmp * -13.6750);
    t->r2s_k[4] = sqrt(stmp * -6.70625);
    t->r2s_k[5] = pow(0.579023e-01, 4);
    t->r2s_k[6] = pow(0.567500e-01, 4);
    t->r2s_k[7] = pow(0.538750e-01, 4);
}

static void prepare_params(const cor_model_params* in, int32_t n, DevParams* out) {
    for (int32_t i = 0; i < n; i++) {
        memset(&out[i], 0, sizeof(DevParams));
        out[i].p = in[i];
        t96_prepare(in[i].parmod, &out[i].t96);
    }
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
        T96Tables tt;
        t96_tables(&tt);
        if (cudaMemcpyToSymbol(c_t96, &tt, sizeof tt) != cudaSuccess) { rc = COR_ERR_CUDA; break; }
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
    const bool ex_ok = m.external_model == COR_EXTERNAL_NONE || m.external_model == COR_EXTERNAL_T96;
    const bool cr_ok = m.crustal_model == COR_CRUSTAL_NONE;
    const bool any = m.internal_model || m.external_model || m.crustal_model;
    return in_ok && ex_ok && cr_ok && any && m.reserved == 0;
}

// Calls fn.template operator()<ModelSet<...>>() for the compile-time set
// matching m (model_set_ok(m) must hold).
template <class F>
static int dispatch_models(const cor_model_set& m, F&& fn) {
    const int key = m.internal_model * 100 + m.external_model * 10 + m.crustal_model;
    switch (key) {
        case 100: return fn(ModelSet<1, 0, 0>{});
        case 110: return fn(ModelSet<1, 1, 0>{});
        case 10: return fn(ModelSet<0, 1, 0>{});
        default: return COR_ERR_UNSUPPORTED;
    }
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
        const int rc = dispatch_models(models, [&](auto ms) { return launch_trace<decltype(ms)>(ctx, a, s); });
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
    if (!ctx) return COR_ERR_INVALID;
    int rc = check_req(ctx, models, ctx->n_params, step_limit, tu_angle, particle_mass);
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
    a.crust = CrustalTables{ctx->crust_g, ctx->crust_h, ctx->crust_nmax};
    a.rig_major = ((flags & COR_FLAG_UNIFORM_GRID) && a.n_rig > 0) ? 1 : 0;
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
    bool uniform = rc == COR_OK && nj > 0;
    for (int32_t j = 0; uniform && j < nj; j++)
        uniform = offsets[j + 1] - offsets[j] == offsets[1] - offsets[0];

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
                                    uniform ? COR_FLAG_UNIFORM_GRID : 0u, s);
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
        const int threads = 128;
        const unsigned blocks = (unsigned)((n + threads - 1) / threads);
        const CrustalTables crust{ctx->crust_g, ctx->crust_h, ctx->crust_nmax};
        dispatch_models(models, [&](auto ms) {
            field_kernel<decltype(ms)><<<blocks, threads, 0, s>>>((const DevParams*)dp, n_params, (const int32_t*)didx,
                                                                   (const double*)dpos, n, (double*)dout, crust);
            return COR_OK;
        });
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
