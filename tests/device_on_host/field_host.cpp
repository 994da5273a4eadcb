// field_host.cpp -- TEST INFRASTRUCTURE: the device field code, RK step and
// per-trajectory scan logic of libcortrace compiled as host C++ (cuda_shim.h)
// with the reference's
// floating-point flags, so that its expression trees can be compared with
// the reference bit for bit: here the transcendental functions are the host
// C library's, as in the reference, where on the GPU they are CUDA's.
// tests/test_device_code_on_host.py builds this file and calls it via ctypes.
#include "cuda_shim.h"

#include "../../cor-model_gb300/csrc/model_prep.h"
#include "../../cor-model_gb300/csrc/trace.cuh"

using namespace cor;

namespace {
DevParams g_dp;
template <int I, int E>
Vec3 field_of(const Vec3 gsm_m) {
    const CrustalTables none{};
    return calculate_field<ModelSet<I, E, 0>>(true, gsm_m, &g_dp, none);
}
template <int I, int E>
void trace_all(const TraceArgs& a) {
    const CrustalTables none{};
    for (uint64_t t = 0; t < a.n_traj; t++) {
        Lane L;
        lane_init(L, a, t, false);
        for (;;) {
            L.field = calculate_field<ModelSet<I, E, 0>>(true, L.gsm, L.par, none);
            L.b = 1.E-09 * sqrt(L.field.x * L.field.x + L.field.y * L.field.y + L.field.z * L.field.z);
            const int st = lane_advance(L, a);
            if (st != 0) {
                lane_finish(L, a, st);
                break;
            }
        }
    }
}

}  // namespace

extern "C" {

// The position-independent tables, as cor_ctx_create uploads them.
void host_tables(void) {
    t96_tables(&c_t96);
    ts05_tables(&c_ts05);
}

// internal_geo at n GEO points [R_E] with the parameter block p.
void host_internal_geo(const cor_model_params* p, const double* pts, int64_t n, double* out) {
    for (int64_t i = 0; i < n; i++) {
        const Vec3 b = internal_geo(Vec3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, p);
        out[3 * i] = b.x;
        out[3 * i + 1] = b.y;
        out[3 * i + 2] = b.z;
    }
}

// t96_field / ts05_field at n GSM points [R_E] for PARMOD (10 values).
void host_external(int external, const double* parmod, const double* pts, int64_t n, double* out) {
    T96Cond c96;
    TS05Cond c05;
    memset(&c96, 0, sizeof c96);
    memset(&c05, 0, sizeof c05);
    t96_prepare(parmod, &c96);
    ts05_prepare(parmod, &c05);
    for (int64_t i = 0; i < n; i++) {
        const Vec3 x{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        const Vec3 b = external == COR_EXTERNAL_T96 ? t96_field(c96, x) : ts05_field(c05, x);
        out[3 * i] = b.x;
        out[3 * i + 1] = b.y;
        out[3 * i + 2] = b.z;
    }
}

// calculate_field<ModelSet> (GSM metres -> GEO nT) for the model sets
// without the crustal field; returns -1 for a set it does not cover.
int host_calculate_field(int internal, int external, const cor_model_params* p, const double* pts, int64_t n,
                         double* out) {
    prepare_params(p, 1, &g_dp);
    for (int64_t i = 0; i < n; i++) {
        const Vec3 x{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        Vec3 b;
        if (internal && external == COR_EXTERNAL_NONE) b = field_of<1, 0>(x);
        else if (internal && external == COR_EXTERNAL_T96) b = field_of<1, 1>(x);
        else if (internal && external == COR_EXTERNAL_TS05) b = field_of<1, 2>(x);
        else if (!internal && external == COR_EXTERNAL_T96) b = field_of<0, 1>(x);
        else if (!internal && external == COR_EXTERNAL_TS05) b = field_of<0, 2>(x);
        else return -1;
        out[3 * i] = b.x;
        out[3 * i + 1] = b.y;
        out[3 * i + 2] = b.z;
    }
    return 0;
}

// The scan kernel's work for every trajectory of a batch, one after the other:
// lane_init, then the kernel loop of trace_kernel -- the field at the lane's
// GSM position whenever it needs one, lane_advance, lane_finish at the
// termination -- for the model sets without the crustal field.  The turn test
// is the reference's atan2 predicate (turn_exact = 0), which on the host is
// the reference's own decision.  status/records get n_traj entries; returns
// -1 for a model set it does not cover.
int host_trace(int internal, int external, const cor_scan_job* jobs, const cor_job_trig* trig, int32_t n_jobs,
               const uint64_t* offsets, uint64_t n_traj, const cor_model_params* params, int32_t n_params,
               uint64_t step_limit, double tu_angle, double mass, uint8_t* status, cor_traj_record* records) {
    DevParams* dp = (DevParams*)calloc((size_t)n_params, sizeof(DevParams));
    if (!dp) return -2;
    prepare_params(params, n_params, dp);
    TraceArgs a;
    memset(&a, 0, sizeof a);
    a.jobs = jobs;
    a.trig = reinterpret_cast<const JobTrig*>(trig);
    a.offsets = offsets;
    a.n_jobs = n_jobs;
    a.n_traj = n_traj;
    a.params = dp;
    a.step_limit = step_limit;
    a.tu_angle = tu_angle;
    a.turn_exact = 0;
    a.mass = mass;
    a.status = status;
    a.records = records;
    int rc = 0;
    if (internal && external == COR_EXTERNAL_NONE) trace_all<1, 0>(a);
    else if (internal && external == COR_EXTERNAL_T96) trace_all<1, 1>(a);
    else if (internal && external == COR_EXTERNAL_TS05) trace_all<1, 2>(a);
    else if (!internal && external == COR_EXTERNAL_T96) trace_all<0, 1>(a);
    else if (!internal && external == COR_EXTERNAL_TS05) trace_all<0, 2>(a);
    else rc = -1;
    free(dp);
    return rc;
}

// chaos_geo_warp at n GEO points [R_E] for the packed tables g/h of nmax
// degrees (the tables built by crustal_block, as cor_upload_crustal builds
// them), 32 points at a time by an emulated warp (the last one partly idle).
int host_chaos(const double* g, const double* h, int32_t nmax, const double* pts, int64_t n, double* out) {
    std::vector<double> block(crustal_block_size(nmax), 0.);
    const int n_first = crustal_block(g, h, nmax, block.data());
    const size_t nt = (size_t)nmax * (size_t)(nmax + 1) / 2;
    const double* b0 = block.data();
    const CrustalTables t{b0, b0 + nt, b0 + 2 * nt, b0 + 3 * nt, b0 + 4 * nt, nmax, n_first, 1, 0};
    ShimWarp w;
    shim_warp = &w;
    for (int64_t base = 0; base < n; base += 32) {
        std::thread lanes[32];
        for (int l = 0; l < 32; l++)
            lanes[l] = std::thread([&, l] {
                threadIdx.x = (unsigned)l;
                const int64_t i = base + l;
                const bool want = i < n;
                const Vec3 x = want ? Vec3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]} : Vec3{0., 0., 0.};
                const Vec3 f = chaos_geo_warp(want, x, t);
                if (want) {
                    out[3 * i] = f.x;
                    out[3 * i + 1] = f.y;
                    out[3 * i + 2] = f.z;
                }
            });
        for (std::thread& th : lanes) th.join();
    }
    shim_warp = nullptr;
    return 0;
}

// calculate_field of the crustal model set (internal and external chosen at
// run time, as the one crustal instantiation does) at n GSM points [m], 32
// points at a time by an emulated warp.
int host_calculate_field_crustal(int internal, int external, const cor_model_params* p, const double* g,
                                 const double* h, int32_t nmax, const double* pts, int64_t n, double* out) {
    prepare_params(p, 1, &g_dp);
    std::vector<double> block(crustal_block_size(nmax), 0.);
    const int n_first = crustal_block(g, h, nmax, block.data());
    const size_t nt = (size_t)nmax * (size_t)(nmax + 1) / 2;
    const double* b0 = block.data();
    const CrustalTables t{b0, b0 + nt, b0 + 2 * nt, b0 + 3 * nt, b0 + 4 * nt, nmax, n_first, internal, external};
    ShimWarp w;
    shim_warp = &w;
    for (int64_t base = 0; base < n; base += 32) {
        std::thread lanes[32];
        for (int l = 0; l < 32; l++)
            lanes[l] = std::thread([&, l] {
                threadIdx.x = (unsigned)l;
                const int64_t i = base + l;
                const bool want = i < n;
                const Vec3 x = want ? Vec3{pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]} : Vec3{0., 0., 0.};
                const Vec3 f =
                    calculate_field<ModelSet<kModelAtRunTime, kModelAtRunTime, 1>>(want, x, &g_dp, t);
                if (want) {
                    out[3 * i] = f.x;
                    out[3 * i + 1] = f.y;
                    out[3 * i + 2] = f.z;
                }
            });
        for (std::thread& th : lanes) th.join();
    }
    shim_warp = nullptr;
    return 0;
}

// One RK step (rk_velocity then rk_position): vel and pos in/out.
void host_rk_step(double h, double d, const double* field, double* vel, double* pos) {
    const Vec3 f{field[0], field[1], field[2]};
    const Vec3 v{vel[0], vel[1], vel[2]};
    const Vec3 x{pos[0], pos[1], pos[2]};
    const Vec3 nv = rk_velocity(h, d, f, v);
    const Vec3 nx = rk_position(h, v, x);
    vel[0] = nv.x;
    vel[1] = nv.y;
    vel[2] = nv.z;
    pos[0] = nx.x;
    pos[1] = nx.y;
    pos[2] = nx.z;
}

// regroup_lanes (trace.cuh) on one emulated 256-thread block.  Thread t starts
// with a trajectory tagged t (traj = t, step = 1000 + t, slot = t, seq =
// 100000 + t, rig = t + 0.5, its job = jobs[t] with zn = t + 1 and nk1 = 7 + t)
// when part[t] is set, and takes part with key[t].  job_copy selects the
// stream kernel's form (each thread keeps its own copy of its scan's job) or
// the batch kernel's (the job pointer moves).  out[t] gets, for the
// trajectory thread t holds afterwards: traj, step, slot, seq, rig, zn, nk1,
// and whether its job pointer is the thread's own copy.
int host_regroup(const unsigned* key, const int32_t* part, int32_t job_copy, double* out) {
    static cor_scan_job jobs[kTraceThreads], own[kTraceThreads];
    static RegroupScratch sc;
    for (int t = 0; t < kTraceThreads; t++) {
        memset(&jobs[t], 0, sizeof(cor_scan_job));
        jobs[t].zn = t + 1.0;
        jobs[t].nk1 = 7 + t;
        own[t] = jobs[t];
    }
    ShimBlock block;
    shim_block = &block;
    std::vector<std::thread> threads;
    for (int t = 0; t < kTraceThreads; t++)
        threads.emplace_back([&, t] {
            threadIdx.x = (unsigned)t;
            Lane L;
            memset(&L, 0, sizeof L);
            L.traj = (uint64_t)t;
            L.step = 1000u + (uint32_t)t;
            L.rig = t + 0.5;
            L.job = job_copy ? &own[t] : &jobs[t];
            unsigned slot = (unsigned)t;
            unsigned long long seq = 100000ull + (unsigned long long)t;
            if (job_copy) regroup_lanes<true>(sc, part[t] != 0, key[t], L, &own[t], slot, seq, t);
            else regroup_lanes<false>(sc, part[t] != 0, key[t], L, nullptr, slot, seq, t);
            double* o = out + 8 * t;
            o[0] = (double)L.traj;
            o[1] = (double)L.step;
            o[2] = (double)slot;
            o[3] = (double)seq;
            o[4] = L.rig;
            o[5] = L.job->zn;
            o[6] = (double)L.job->nk1;
            o[7] = L.job == &own[t] ? 1.0 : 0.0;
        });
    for (std::thread& th : threads) th.join();
    shim_block = nullptr;
    return 0;
}

}  // extern "C"
