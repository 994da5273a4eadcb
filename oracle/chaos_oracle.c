/*
 * chaos_oracle.c -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU restatement of chaos_geo (lib/chaos/chaos.c:120-226, the branch compiled
 * when OLD_CODE is not defined): a spherical-harmonic sum with fully
 * normalised Legendre functions P_n^m and dP_n^m/dtheta built by the
 * recursion of :175-196, and a sin/cos(m*phi) call per (n,m) term (:201-216).
 * The reference keeps the two nmax x nmax tables on the stack; here they live
 * in per-thread heap scratch.  Same operation order, same C library calls.
 */
#include "cor_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define O_RE_KM 6371.2              /* lib/chaos/chaos.h:6 */
#define O_2PI_D 6.283185307179586   /* lib/chaos/chaos.h:7 */
#define O_PI_D 3.141592653589793    /* lib/chaos/chaos.h:8 */

void orc_chaos_geo(double x, double y, double z, const double *G, const double *H, int nmax,
                   double *bx, double *by, double *bz) {
    const double rho2 = x * x + y * y;
    const double R = sqrt(rho2 + z * z);
    const double C = z / R;
    const double r = R * O_RE_KM;
    double theta = 0., phi = 0., S = 0., cf = 1., sf = 0.;
    if (rho2 != 0.) {
        const double rho = sqrt(rho2);
        S = rho / R;
        cf = x / rho;
        sf = y / rho;
        phi = atan2(y, x);
        theta = atan2(rho, z);
        if (phi < 0.) phi += O_2PI_D;
    } else if (z < 0.) {
        theta = O_PI_D;
    }

    double *ar = (double *)malloc(sizeof(double) * (size_t)nmax * 2);
    double *P = (double *)calloc((size_t)nmax * nmax, sizeof(double));
    double *dP = (double *)calloc((size_t)nmax * nmax, sizeof(double));
    double *dar = ar + nmax;
    if (!ar || !P || !dP) {
        free(ar); free(P); free(dP);
        *bx = *by = *bz = NAN;
        return;
    }
#define IX(n, m) ((size_t)(n) * nmax + (m))
    /* radial powers (a/r)^(n+1) and their r-derivative, :142-152 */
    const double tem = O_RE_KM / r;
    ar[0] = tem;
    dar[0] = -tem / r;
    for (int i = 1; i < nmax; i++) {
        const double t = ar[i - 1] * tem;
        ar[i] = t;
        dar[i] = -(i + 1) * t / r;
    }
    /* Legendre recursion, :159-196 */
    const double st = sin(theta);
    const double ct = cos(theta);
    P[IX(0, 0)] = 1.;
    P[IX(1, 0)] = ct;
    P[IX(1, 1)] = st;
    dP[IX(0, 0)] = 0.;
    dP[IX(1, 0)] = -st;
    dP[IX(1, 1)] = ct;
    for (int n = 2; n < nmax; n++) {
        const double n2 = n * 2;
        const double n21 = n2 - 1;
        const int n1 = n - 1;
        const double k = sqrt(n21 / n2);
        const double kp = k * P[IX(n1, n1)];
        P[IX(n, n)] = st * kp;
        dP[IX(n, n)] = ct * kp + st * k * dP[IX(n1, n1)];
        const int n_2 = n - 2;
        const double nn = (double)n * n;
        for (int m = 0; m < n; m++) {
            const double mm = m * m;
            const double nnmm = nn - mm;
            const double k1 = n21 / sqrt(nnmm);
            const double k2 = sqrt((n1 * n1 - mm) / nnmm);
            const double pp = P[IX(n1, m)];
            P[IX(n, m)] = k1 * ct * pp - k2 * P[IX(n_2, m)];
            dP[IX(n, m)] = k1 * (-st * pp + ct * dP[IX(n1, m)]) - k2 * dP[IX(n_2, m)];
        }
    }
    /* the sum, :201-216 */
    double br = 0., bt = 0., bp = 0.;
    for (int n = 0; n < nmax; n++) {
        for (int m = 0; m <= n; m++) {
            const double mphi = m * phi;
            const double smp = sin(mphi);
            const double cmp = cos(mphi);
            const double g = G[IX(n, m)];
            const double h = H[IX(n, m)];
            const double t = g * cmp + h * smp;
            const double pnm = P[IX(n, m)];
            const double rn = ar[n];
            br += t * pnm * dar[n];
            bt += t * dP[IX(n, m)] * rn;
            bp += (-g * m * smp + h * m * cmp) * pnm * rn;
        }
    }
#undef IX
    free(ar); free(P); free(dP);
    bt = -bt * O_RE_KM / r;                                /* :218-220 */
    bp = -bp * O_RE_KM / (r * st);
    br = -br * O_RE_KM;
    const double he = br * S + bt * C;
    *bx = he * cf - bp * sf;
    *by = he * sf + bp * cf;
    *bz = br * C - bt * S;
}
