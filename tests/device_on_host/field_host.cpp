// field_host.cpp -- TEST INFRASTRUCTURE: the device field code and RK step of
// libcortrace compiled as host C++ (cuda_shim.h) with the reference's
// floating-point flags, so that its expression trees can be compared with
// the reference bit for bit: here the transcendental functions are the host
// C library's, as in the reference, where on the GPU they are CUDA's.
// tests/test_device_code_on_host.py builds this file and calls it via ctypes.
#include "cuda_shim.h"

#include "../../cor-model_gb300/csrc/model_prep.h"

using namespace cor;

namespace {
DevParams g_dp;
template <int I, int E>
Vec3 field_of(const Vec3 gsm_m) {
    const CrustalTables none{};
    return calculate_field<ModelSet<I, E, 0>>(true, gsm_m, &g_dp, none);
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

}  // extern "C"
