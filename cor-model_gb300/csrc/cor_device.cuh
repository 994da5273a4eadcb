// cor_device.cuh -- FP64 device building blocks of the rigidity scan.
//
// Every function here keeps the reference's expression order.  The units of
// the IGRF-only model set and the C ABI are compiled with --fmad=false (the
// reference is built with -ffp-contract=off, CMakeLists.txt:17), so each
// result there is the correctly rounded IEEE value of the same expression
// tree: bit-identical to the reference wherever only + - * / sqrt are
// involved.  The units with an external or crustal model (whose C-library
// functions differ from CUDA's anyway) are compiled with FMA contraction;
// div_c/div_r spell out their roundings (__dmul_rn, __fma_rn), so they stay
// exact there too.
#pragma once

#include <stdint.h>

#include "../../include/cor_trace.h"

namespace cor {

// Legacy-truncated constants of src/common.h:4-11.
constexpr double kPi = 3.141592654;
constexpr double k2Pi = 6.28318531;
constexpr double kRe = 6.3712e+06;
constexpr double kToRad = kPi / 180.;
constexpr double kQ = 1.6021e-19;
constexpr double kC = 2.99725e+08;

// Boundary refinement bound (the reference doubles nk0 without one,
// src/trajectory.c:126-130).
constexpr int kNk0Cap = 1 << 30;

struct Vec3 {
    double x, y, z;
};

// Correctly rounded x / c for a constant c, given rc = RN(1/c).  q0 = RN(x*rc)
// is within one ulp of x/c, so r = x - q0*c is exact in one FMA, and
// RN(q0 + r*rc) is the correctly rounded quotient (Markstein's theorem for
// a correctly rounded reciprocal and a faithful first quotient).  Three FP64
// operations instead of a full division; the result equals x / c bit for bit
// (checked for every constant used here in the test suite).
__device__ __forceinline__ double div_c(const double x, const double c, const double rc) {
    const double q0 = __dmul_rn(x, rc);
    const double r = __fma_rn(-q0, c, x);
    return __fma_rn(r, rc, q0);
}
#define DIV3(x) ::cor::div_c((x), 3., 1. / 3.)
#define DIV25(x) ::cor::div_c((x), 25., 1. / 25.)
#define DIV81(x) ::cor::div_c((x), 81., 1. / 81.)
#define DIV75(x) ::cor::div_c((x), 75., 1. / 75.)
#define DIV192(x) ::cor::div_c((x), 192., 1. / 192.)
#define DIV4(x) ((x)*0.25)  // exact: 0.25 is a power of two
#define DIVRE(x) ::cor::div_c((x), ::cor::kRe, 1. / ::cor::kRe)

// Correctly rounded x / b given the correctly rounded reciprocal rb = 1/b of
// a run-time divisor (same theorem as div_c), for several quotients that
// share one divisor.
__device__ __forceinline__ double div_r(const double x, const double b, const double rb) {
    const double q0 = __dmul_rn(x, rb);
    const double r = __fma_rn(-q0, b, x);
    return __fma_rn(r, rb, q0);
}

// geo_to_gsm, src/utils.c:75-87 (rows of A).
__device__ __forceinline__ Vec3 geo_to_gsm(const Vec3 g, const cor_model_params* __restrict__ p) {
    Vec3 s;
    s.x = __ldg(&p->a1[0]) * g.x + __ldg(&p->a1[1]) * g.y + __ldg(&p->a1[2]) * g.z;
    s.y = __ldg(&p->a2[0]) * g.x + __ldg(&p->a2[1]) * g.y + __ldg(&p->a2[2]) * g.z;
    s.z = __ldg(&p->a3[0]) * g.x + __ldg(&p->a3[1]) * g.y + __ldg(&p->a3[2]) * g.z;
    return s;
}

// gsm_to_geo, src/utils.c:89-101 (columns of A).
__device__ __forceinline__ Vec3 gsm_to_geo(const Vec3 s, const cor_model_params* __restrict__ p) {
    Vec3 g;
    g.x = __ldg(&p->a1[0]) * s.x + __ldg(&p->a2[0]) * s.y + __ldg(&p->a3[0]) * s.z;
    g.y = __ldg(&p->a1[1]) * s.x + __ldg(&p->a2[1]) * s.y + __ldg(&p->a3[1]) * s.z;
    g.z = __ldg(&p->a1[2]) * s.x + __ldg(&p->a2[2]) * s.y + __ldg(&p->a3[2]) * s.z;
    return g;
}

// Out-of-line C-library functions for the field models.  The inline
// expansion of a CUDA double-precision function is tens to hundreds of
// instructions, and the T96/TS05 models call them at many sites inside
// unrolled loops; calling one out-of-line copy instead keeps each kernel's
// field code small enough for the instruction caches.  Same functions, same
// results.
struct SinCos {
    double s, c;
};
static __device__ __noinline__ double ol_exp(const double x) { return exp(x); }
static __device__ __noinline__ double ol_log(const double x) { return log(x); }
static __device__ __noinline__ double ol_sin(const double x) { return sin(x); }
static __device__ __noinline__ double ol_cos(const double x) { return cos(x); }
static __device__ __noinline__ double ol_atan(const double x) { return atan(x); }
static __device__ __noinline__ double ol_asin(const double x) { return asin(x); }
static __device__ __noinline__ double ol_atan2(const double y, const double x) { return atan2(y, x); }
static __device__ __noinline__ double ol_pow(const double x, const double y) { return pow(x, y); }
static __device__ __noinline__ SinCos ol_sincos_v(const double x) {
    SinCos r;
    sincos(x, &r.s, &r.c);
    return r;
}
__device__ __forceinline__ void ol_sincos(const double x, double* s, double* c) {
    const SinCos r = ol_sincos_v(x);
    *s = r.s;
    *c = r.c;
}

// Spherical-harmonic internal field, internal_geo (lib/internal/internal.c:182-275).
// Degree truncated by radius, NM = min(13, 3 + 30/((int)R + 2)) (:201-205).
// The (m, n) double loop is unrolled with compile-time indices so the
// powers of 1/R stay in registers; the loop exits at the lane's own degree.
__device__ __forceinline__ Vec3 internal_geo(const Vec3 x, const cor_model_params* __restrict__ p) {
    const double rho2 = x.x * x.x + x.y * x.y;
    const double R = sqrt(rho2 + x.z * x.z);
    const double pp = 1. / R;
    const double C = div_r(x.z, R, pp);
    const double rho = sqrt(rho2);
    const double S = div_r(rho, R, pp);
    const bool pole = S < 1.E-5;
    double cf, sf;
    if (pole) {
        cf = 1.;
        sf = 0.;
    } else {
        cf = x.x / rho;
        sf = x.y / rho;
    }
    int nm = 3 + 30 / ((int)R + 2);
    if (nm > 13) nm = 13;
    const int K = nm + 1;

    double pw[14], pwn[14];
    {
        double pr = pp;
#pragma unroll
        for (int n = 1; n <= 14; n++) {
            pr = pr * pp;
            pw[n - 1] = pr;
            pwn[n - 1] = pr * n;
        }
    }

    const double* __restrict__ G = p->g;
    const double* __restrict__ H = p->h;
    const double* __restrict__ REC = p->rec;
    double pmm = 1., dmm = 0.;
    double br = 0., bt = 0., bf = 0.;
    double cm = 0., sm = 1.;
#pragma unroll
    for (int m = 1; m <= 14; m++) {
        if (m > K) break;
        if (m != 1) {
            const double w = cm;
            cm = w * cf + sm * sf;
            sm = sm * cf - w * sf;
        }
        double q = pmm, zz = dmm, bi = 0., p2 = 0., d2 = 0.;
#pragma unroll
        for (int n = m; n <= 14; n++) {
            if (n > K) break;
            const double an = pw[n - 1];
            const int mn = n * (n - 1) / 2 + m - 1;
            const double e = __ldg(&G[mn]);
            const double hh = __ldg(&H[mn]);
            const double w = e * sm + hh * cm;
            br = br + pwn[n - 1] * w * q;
            bt = bt - an * w * zz;
            if (m != 1) {
                const double qq = pole ? zz : q;
                bi = bi + an * (e * cm - hh * sm) * qq;
            }
            const double xk = __ldg(&REC[mn]);
            const double dp = C * zz - S * q - xk * d2;
            const double pm = C * q - xk * p2;
            d2 = zz;
            p2 = q;
            zz = dp;
            q = pm;
        }
        dmm = S * dmm + C * pmm;
        pmm = S * pmm;
        if (m != 1) {
            bi = bi * (m - 1);
            bf = bf + bi;
        }
    }
    double bphi;
    if (pole) {
        if (C < 0.) bf = -bf;
        bphi = bf;
    } else {
        bphi = bf / S;
    }
    const double he = br * S + bt * C;
    Vec3 b;
    b.x = he * cf - bphi * sf;
    b.y = he * sf + bphi * cf;
    b.z = br * C - bt * S;
    return b;
}

// Velocity half of calculate_position_and_speed (src/trajectory.c:277-329,
// :350-352): six stages of dv/dt = d (v x B) with B frozen.  Returns the
// updated velocity; the position half is separate because a trial rejected
// by the turn-angle test never uses it.
__device__ __forceinline__ Vec3 rk_velocity(const double h, const double d, const Vec3 f, const Vec3 v) {
#define CX(Y, Z) (h * (d * ((Y)*f.z - (Z)*f.y)))
#define CY(X, Z) (h * (d * ((Z)*f.x - (X)*f.z)))
#define CZ(X, Y) (h * (d * ((X)*f.y - (Y)*f.x)))
    const double a1 = CX(v.y, v.z), b1 = CY(v.x, v.z), c1 = CZ(v.x, v.y);
    const double sx2 = v.x + DIV3(a1), sy2 = v.y + DIV3(b1), sz2 = v.z + DIV3(c1);
    const double a2 = CX(sy2, sz2), b2 = CY(sx2, sz2), c2 = CZ(sx2, sy2);
    const double sx3 = v.x + DIV25(4. * a1 + 6. * a2);
    const double sy3 = v.y + DIV25(4. * b1 + 6. * b2);
    const double sz3 = v.z + DIV25(4. * c1 + 6. * c2);
    const double a3 = CX(sy3, sz3), b3 = CY(sx3, sz3), c3 = CZ(sx3, sy3);
    const double sx4 = v.x + DIV4(a1 - 12. * a2 + 15. * a3);
    const double sy4 = v.y + DIV4(b1 - 12. * b2 + 15. * b3);
    const double sz4 = v.z + DIV4(c1 - 12. * c2 + 15. * c3);
    const double a4 = CX(sy4, sz4), b4 = CY(sx4, sz4), c4 = CZ(sx4, sy4);
    const double sx5 = v.x + DIV81(6. * a1 + 90. * a2 - 50. * a3 + 8. * a4);
    const double sy5 = v.y + DIV81(6. * b1 + 90. * b2 - 50. * b3 + 8. * b4);
    const double sz5 = v.z + DIV81(6. * c1 + 90. * c2 - 50. * c3 + 8. * c4);
    const double a5 = CX(sy5, sz5), b5 = CY(sx5, sz5), c5 = CZ(sx5, sy5);
    const double sx6 = v.x + DIV75(6. * a1 + 36. * a2 + 10. * a3 + 8. * a4);
    const double sy6 = v.y + DIV75(6. * b1 + 36. * b2 + 10. * b3 + 8. * b4);
    const double sz6 = v.z + DIV75(6. * c1 + 36. * c2 + 10. * c3 + 8. * c4);
    const double a6 = CX(sy6, sz6), b6 = CY(sx6, sz6), c6 = CZ(sx6, sy6);
#undef CX
#undef CY
#undef CZ
    Vec3 o;
    o.x = v.x + DIV192(23. * a1 + 125. * a3 - 81. * a5 + 125. * a6);
    o.y = v.y + DIV192(23. * b1 + 125. * b3 - 81. * b5 + 125. * b6);
    o.z = v.z + DIV192(23. * c1 + 125. * c3 - 81. * c5 + 125. * c6);
    return o;
}

// Position half of calculate_position_and_speed (src/trajectory.c:331-348,
// :353-355): the same tableau on h*v with the unrotated velocity.
__device__ __forceinline__ double rk_position_1(const double h, const double vc, const double xc) {
    const double k1 = h * vc;
    const double k2 = h * (vc + DIV3(k1));
    const double k3 = h * (vc + DIV25(4. * k1 + 6. * k2));
    const double k4 = h * (vc + DIV4(k1 - 12. * k2 + 15. * k3));
    const double k5 = h * (vc + DIV81(6. * k1 + 90. * k2 - 50. * k3 + 8. * k4));
    const double k6 = h * (vc + DIV75(6. * k1 + 36. * k2 + 10. * k3 + 8. * k4));
    return xc + DIV192(23. * k1 + 125. * k3 - 81. * k5 + 125. * k6);
}

__device__ __forceinline__ Vec3 rk_position(const double h, const Vec3 v, const Vec3 x) {
    Vec3 o;
    o.x = rk_position_1(h, v.x, x.x);
    o.y = rk_position_1(h, v.y, x.y);
    o.z = rk_position_1(h, v.z, x.z);
    return o;
}

}  // namespace cor
