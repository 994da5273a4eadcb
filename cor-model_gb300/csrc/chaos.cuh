// chaos.cuh -- the crustal field chaos_geo (lib/chaos/chaos.c:120-226, the
// branch built without OLD_CODE) on the device, evaluated by a whole warp.
//
// The terms are the reference's: fully normalised P_n^m and dP_n^m/dtheta
// from the recursion of chaos.c:159-196 and the (n, m) terms of :201-216.
// What differs is who computes them and the order of the final summation:
//  * every lane of the warp calls chaos_geo_warp; the positions of the lanes
//    that want a field are taken one after another, each by all 32 lanes, so
//    a lone trajectory (a long one at the end of a scan) costs 1/32 of a full
//    warp's work per step instead of all of it;
//  * for one position, lane l takes the orders m = l, 63-l, 64+l, 127-l, ...
//    (a snake over the lanes, which evens out the column lengths nmax - m)
//    and walks each column down the degrees with the column recursion
//    (P(n,m) needs only P(n-1,m) and P(n-2,m)), the diagonal P(m,m) and the
//    radial powers (a/r)^(n+1) carried along as the reference's sequential
//    products; sin(m*phi), cos(m*phi) once per column;
//  * the recursion factors k = sqrt((2n-1)/2n), k1 = (2n-1)/sqrt(n^2-m^2),
//    k2 = sqrt(((n-1)^2-m^2)/(n^2-m^2)) come from tables the host built with
//    the same expressions (IEEE division and square root are correctly
//    rounded on both sides, so they hold the reference's values);
//  * the three sums are taken per column, then across the lanes, where the
//    reference sums degree by degree.
// The device atan2/sin/cos are not glibc's either, so results agree with the
// reference to a few ulp of the crustal field, not bit for bit.
#pragma once

#include "cor_device.cuh"

namespace cor {

constexpr int kChaosMaxN = 192;      // largest nmax (table rows) accepted
constexpr double kChaosReKm = 6371.2;              // lib/chaos/chaos.h:6
constexpr double kChaos2Pi = 6.283185307179586;    // lib/chaos/chaos.h:7
constexpr double kChaosPi = 3.141592653589793;     // lib/chaos/chaos.h:8

// Device tables of the crustal model.  g, h, k1, k2 are packed lower
// triangles (index n(n+1)/2 + m); kd holds k per degree.  n_first is the
// first degree with a non-zero coefficient: lower degrees add exactly +0 to
// sums that are +0, so their terms are skipped (their rows are still built).
// The kernels of sets with a crustal model choose the internal and external
// models at run time (the crustal sum dwarfs the dispatch), from `internal`
// and `external` (COR_INTERNAL_*, COR_EXTERNAL_*).
struct CrustalTables {
    const double* g;
    const double* h;
    const double* k1;
    const double* k2;
    const double* kd;
    int nmax;
    int n_first;
    int internal;
    int external;
};

// Called by all 32 lanes of a warp together; a lane with `want` set gets
// chaos_geo at its own GEO position x [R_E].
static __device__ __noinline__ Vec3 chaos_geo_warp(const bool want, const Vec3 x, const CrustalTables& t) {
    const int lane = threadIdx.x & 31;
    const int nmax = t.nmax;
    const double* __restrict__ G = t.g;
    const double* __restrict__ H = t.h;
    unsigned todo = __ballot_sync(0xffffffffu, want);
    Vec3 mine = {0., 0., 0.};
    while (todo) {
        const int q = __ffs(todo) - 1;
        todo &= todo - 1;
        const double px = __shfl_sync(0xffffffffu, x.x, q);
        const double py = __shfl_sync(0xffffffffu, x.y, q);
        const double pz = __shfl_sync(0xffffffffu, x.z, q);
        // geometry, chaos.c:128-140 (every lane computes the same values)
        const double rho2 = px * px + py * py;
        const double R = sqrt(rho2 + pz * pz);
        const double C = pz / R;
        const double r = R * kChaosReKm;
        double theta = 0., phi = 0., S = 0., cf = 1., sf = 0.;
        if (rho2 != 0.) {
            const double rho = sqrt(rho2);
            S = rho / R;
            cf = px / rho;
            sf = py / rho;
            phi = atan2(py, px);
            theta = atan2(rho, pz);
            if (phi < 0.) phi += kChaos2Pi;
        } else if (pz < 0.) {
            theta = kChaosPi;
        }
        const double st = sin(theta);
        const double ct = cos(theta);
        const double tem = kChaosReKm / r;
        const double rr = 1. / r;
        double br = 0., bt = 0., bp = 0.;
        // diagonal P(d,d), dP(d,d) and the radial power ar[d] = tem^(d+1)
        double pd = 1., dpd = 0., rnd = tem;
        int d = 0;
        for (int c = 0;; c++) {
            const int m = c * 32 + ((c & 1) ? 31 - lane : lane);
            if (m >= nmax) break;
            while (d < m) {                       // chaos.c:159-170
                d++;
                rnd = rnd * tem;                  // :142-152, ar[d] = ar[d-1] * tem
                if (d == 1) {
                    pd = st;
                    dpd = ct;
                } else {
                    const double k = __ldg(t.kd + d);
                    const double kp = k * pd;
                    dpd = ct * kp + st * k * dpd;
                    pd = st * kp;
                }
            }
            double sm, cm;
            sincos(m * phi, &sm, &cm);
            const double md = (double)m;
            double p1 = pd, dp1 = dpd, p2 = 0., dp2 = 0.;   // P(n-1,m), P(n-2,m); P(m-1,m) = 0
            double rn = rnd;
            for (int n = m; n < nmax; n++) {
                double pnm, dpnm;
                if (n == m) {
                    pnm = p1;
                    dpnm = dp1;
                } else {
                    if (n == 1) {                 // P(1,0), dP(1,0) are set directly, :161-163
                        pnm = ct;
                        dpnm = -st;
                    } else {                      // :172-194
                        const int idx = n * (n + 1) / 2 + m;
                        const double k1 = __ldg(t.k1 + idx);
                        const double k2 = __ldg(t.k2 + idx);
                        pnm = k1 * ct * p1 - k2 * p2;
                        dpnm = k1 * (-st * p1 + ct * dp1) - k2 * dp2;
                    }
                    p2 = p1;
                    dp2 = dp1;
                    p1 = pnm;
                    dp1 = dpnm;
                    rn = rn * tem;
                }
                if (n >= t.n_first) {             // :201-216
                    const double drn = div_r(-(double)(n + 1) * rn, r, rr);
                    const int idx = n * (n + 1) / 2 + m;
                    const double g = __ldg(G + idx);
                    const double h = __ldg(H + idx);
                    const double tt = g * cm + h * sm;
                    br += tt * pnm * drn;
                    bt += tt * dpnm * rn;
                    bp += (-g * md * sm + h * md * cm) * pnm * rn;
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            br += __shfl_xor_sync(0xffffffffu, br, o);
            bt += __shfl_xor_sync(0xffffffffu, bt, o);
            bp += __shfl_xor_sync(0xffffffffu, bp, o);
        }
        bt = -bt * kChaosReKm / r;          // :218-220
        bp = -bp * kChaosReKm / (r * st);
        br = -br * kChaosReKm;
        const double he = br * S + bt * C;
        if (lane == q) mine = Vec3{he * cf - bp * sf, he * sf + bp * cf, br * C - bt * S};
    }
    return mine;
}

}  // namespace cor
