// field.cuh -- field composition on the device, calculate_field
// (src/models.c:194-207) with the model list fixed at compile time.
#pragma once

#include "cor_device.cuh"
#include "chaos.cuh"
#include "t96.cuh"
#include "ts05.cuh"

namespace cor {

// Compile-time model set: internal (0/1), external (0 none, 1 T96, 2 TS05),
// crustal (0/1).  The kernels are instantiated per set so the step loop
// carries no model dispatch.  kModelAtRunTime for internal or external reads
// the choice from the crustal tables' internal/external members instead (the
// one instantiation that serves every set with a crustal model).
constexpr int kModelAtRunTime = -1;

template <int INTERNAL, int EXTERNAL, int CRUSTAL>
struct ModelSet {
    static constexpr int internal = INTERNAL;
    static constexpr int external = EXTERNAL;
    static constexpr int crustal = CRUSTAL;
};

// Device copy of one parameter block: the ABI block (ModelsParams) plus the
// per-condition constants of the external models, derived on the host.
struct DevParamsBody {
    cor_model_params p;
    T96Cond t96;
    TS05Cond ts05;
};
// Padded to a multiple of 256 bytes, so that in an array of blocks no cache
// line holds parts of two blocks (the scan stream appends blocks while its
// kernel runs and reads them through the read-only path).
struct DevParams {
    cor_model_params p;
    T96Cond t96;
    TS05Cond ts05;
    unsigned char pad[256 - sizeof(DevParamsBody) % 256];
};
static_assert(sizeof(DevParams) % 256 == 0, "parameter blocks are whole 256-byte units");

// GSM position in metres -> GEO field in nT, for the lanes with `want` set
// (the others get zeros and never read dp).  With the crustal model every
// lane of the warp must make the call together, converged: the crustal sum
// is evaluated by the whole warp (chaos_geo_warp).  Without it, a caller may
// call for its wanting lanes alone.
template <class MS>
__device__ __forceinline__ Vec3 calculate_field(const bool want, const Vec3 gsm_pos, const DevParams* __restrict__ dp,
                                                const CrustalTables& crust) {
    Vec3 tot = {0., 0., 0.};
    Vec3 pos = {0., 0., 0.};
    const cor_model_params* __restrict__ p = nullptr;
    if (want) {
        p = &dp->p;
        pos = {DIVRE(gsm_pos.x), DIVRE(gsm_pos.y), DIVRE(gsm_pos.z)};
        const bool internal = MS::internal == kModelAtRunTime ? crust.internal != 0 : MS::internal != 0;
        const int external = MS::external == kModelAtRunTime ? crust.external : MS::external;
        if (internal) {
            // internal_calc, src/models.c:146-160
            const Vec3 geo = gsm_to_geo(pos, p);
            const Vec3 bg = internal_geo(geo, p);
            const Vec3 bs = geo_to_gsm(bg, p);
            tot.x += bs.x;
            tot.y += bs.y;
            tot.z += bs.z;
        }
        if (external == COR_EXTERNAL_T96) {
            const Vec3 b = t96_field(dp->t96, pos);  // t96_calc, src/models.c:171-177
            tot.x += b.x;
            tot.y += b.y;
            tot.z += b.z;
        } else if (external == COR_EXTERNAL_TS05) {
            const Vec3 b = ts05_field(dp->ts05, pos);  // ts05_calc, src/models.c:162-169
            tot.x += b.x;
            tot.y += b.y;
            tot.z += b.z;
        }
    }
    if constexpr (MS::crustal != 0) {
        // chaos_7_16_calc, src/models.c:179-192
        const Vec3 geo = want ? gsm_to_geo(pos, p) : Vec3{0., 0., 0.};
        const Vec3 bg = chaos_geo_warp(want, geo, crust);
        if (want) {
            const Vec3 bs = geo_to_gsm(bg, p);
            tot.x += bs.x;
            tot.y += bs.y;
            tot.z += bs.z;
        }
    }
    return want ? gsm_to_geo(tot, p) : tot;
}

// Which branches of the field code a GSM position (metres) takes, as a sort
// key: lanes with equal keys run the same call sites of the expensive
// sub-models, so a warp of them issues each sub-model once.  The key only
// places lanes and never enters a result, so a position it misjudges costs
// time, not bits.  With T96 the leading part is the band of the Region-2
// field (r2_birk's xksi bands, lib/t96/t96.c:1265-1314), whose outer, sheet
// and inner fields dominate the divergent work; then, for every model set,
// the radius in whole R_E (the internal field's degree and T96/TS05's inner
// structures change with it) and |z|/r in twelfths (latitude bands).
template <class MS>
__device__ __forceinline__ unsigned field_band(const Vec3 gsm_pos, const DevParams* __restrict__ dp) {
    constexpr double kInvRe = 1.0 / kRe;
    const double x = gsm_pos.x * kInvRe, y = gsm_pos.y * kInvRe, z = gsm_pos.z * kInvRe;
    const double r = sqrt(x * x + y * y + z * z);
    const unsigned ri = r < 31.0 ? (unsigned)r : 31u;
    const double zr = r > 0.0 ? fabs(z) / r : 0.0;
    const unsigned lat = zr < 1.0 ? (unsigned)(zr * 12.0) : 12u;
    unsigned band = 0;
    if constexpr (MS::external == COR_EXTERNAL_T96) {
        const double xa = dp->t96.xappa;
        const double xks = t96_xksi(x * xa, y * xa, z * xa);
        band = xks < -0.045 ? 0u : xks < -0.015 ? 1u : xks < 0.015 ? 2u : xks < 0.045 ? 3u : 4u;
    }
    return (band << 9) | (ri << 4) | lat;
}

}  // namespace cor
