// chaos.cuh -- the crustal field chaos_geo (lib/chaos/chaos.c:120-226, the
// branch built without OLD_CODE) on the device.
//
// The sum is the reference's: degrees n = 0 .. nmax-1 outer, orders m = 0 .. n
// inner, with fully normalised P_n^m and dP_n^m/dtheta from the recursion of
// chaos.c:159-196 and the terms of :201-216 accumulated in the same order.
// What differs is where the values come from, not what they are:
//  * sin(m*phi) and cos(m*phi) depend on m only; they are evaluated once per
//    order into a per-thread table instead of once per (n, m) term;
//  * the recursion factors k = sqrt((2n-1)/2n), k1 = (2n-1)/sqrt(n^2-m^2) and
//    k2 = sqrt(((n-1)^2-m^2)/(n^2-m^2)) are read from tables the host built
//    with the same expressions (IEEE division and square root are correctly
//    rounded on both sides, so the tables hold the reference's values);
//  * only the rows n-1 and n-2 of P and dP are kept (rows of equal parity
//    share storage, a new row overwriting the one two degrees back);
//  * the radial powers (a/r)^(n+1) and their r-derivative are carried from
//    degree to degree (chaos.c:142-152 computes the same sequence up front).
// The device atan2/sin/cos are not glibc's, so results agree with the
// reference to a few ulp of those values, not bit for bit.
#pragma once

#include "cor_device.cuh"

namespace cor {

constexpr int kChaosMaxN = 192;      // largest nmax (table rows) a thread's scratch holds
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

static __device__ __noinline__ Vec3 chaos_geo(const Vec3 x, const CrustalTables& t) {
    const double rho2 = x.x * x.x + x.y * x.y;
    const double R = sqrt(rho2 + x.z * x.z);
    const double C = x.z / R;
    const double r = R * kChaosReKm;
    double theta = 0., phi = 0., S = 0., cf = 1., sf = 0.;
    if (rho2 != 0.) {
        const double rho = sqrt(rho2);
        S = rho / R;
        cf = x.x / rho;
        sf = x.y / rho;
        phi = atan2(x.y, x.x);
        theta = atan2(rho, x.z);
        if (phi < 0.) phi += kChaos2Pi;
    } else if (x.z < 0.) {
        theta = kChaosPi;
    }
    const int nmax = t.nmax;

    double sm[kChaosMaxN], cm[kChaosMaxN];
    for (int m = 0; m < nmax; m++) sincos(m * phi, &sm[m], &cm[m]);
    // P and dP of degrees n-2 / n-1, in rows (n & 1); entries a row of that
    // parity never wrote read as zero, as the reference's calloc'd table does
    double P[2][kChaosMaxN], dP[2][kChaosMaxN];
    for (int m = 0; m < nmax; m++) {
        P[0][m] = 0.;
        P[1][m] = 0.;
        dP[0][m] = 0.;
        dP[1][m] = 0.;
    }

    const double st = sin(theta);
    const double ct = cos(theta);
    const double tem = kChaosReKm / r;
    double rn = tem;                // ar[n]
    double drn = -tem / r;          // dar[n]
    double br = 0., bt = 0., bp = 0.;
    const double* __restrict__ G = t.g;
    const double* __restrict__ H = t.h;

    auto term = [&](int idx, int m, double pnm, double dpnm) {
        const double md = (double)m;
        const double g = __ldg(G + idx);
        const double h = __ldg(H + idx);
        const double tt = g * cm[m] + h * sm[m];
        br += tt * pnm * drn;
        bt += tt * dpnm * rn;
        bp += (-g * md * sm[m] + h * md * cm[m]) * pnm * rn;
    };

    for (int n = 0; n < nmax; n++) {
        if (n > 0) {
            const double tn = rn * tem;
            rn = tn;
            drn = -(double)(n + 1) * tn / r;
        }
        const int base = n * (n + 1) / 2;
        double* __restrict__ Pn = P[n & 1];         // row n (overwrites row n-2)
        double* __restrict__ dPn = dP[n & 1];
        const double* __restrict__ P1 = P[(n + 1) & 1];   // row n-1
        const double* __restrict__ dP1 = dP[(n + 1) & 1];
        const bool sum = n >= t.n_first;
        if (n == 0) {
            Pn[0] = 1.;
            dPn[0] = 0.;
            if (sum) term(0, 0, 1., 0.);
            continue;
        }
        if (n == 1) {
            Pn[0] = ct;
            Pn[1] = st;
            dPn[0] = -st;
            dPn[1] = ct;
            if (sum) {
                term(1, 0, ct, -st);
                term(2, 1, st, ct);
            }
            continue;
        }
        // diagonal first (chaos.c:166-170), then m < n (:172-194)
        const double k = __ldg(t.kd + n);
        const double kp = k * P1[n - 1];
        const double pnn = st * kp;
        const double dpnn = ct * kp + st * k * dP1[n - 1];
        for (int m = 0; m < n; m++) {
            const double k1 = __ldg(t.k1 + base + m);
            const double k2 = __ldg(t.k2 + base + m);
            const double pp = P1[m];
            const double pnm = k1 * ct * pp - k2 * Pn[m];
            const double dpnm = k1 * (-st * pp + ct * dP1[m]) - k2 * dPn[m];
            Pn[m] = pnm;
            dPn[m] = dpnm;
            if (sum) term(base + m, m, pnm, dpnm);
        }
        Pn[n] = pnn;
        dPn[n] = dpnn;
        if (sum) term(base + n, n, pnn, dpnn);
    }
    bt = -bt * kChaosReKm / r;          // chaos.c:218-220
    bp = -bp * kChaosReKm / (r * st);
    br = -br * kChaosReKm;
    const double he = br * S + bt * C;
    return Vec3{he * cf - bp * sf, he * sf + bp * cf, br * C - bt * S};
}

}  // namespace cor
