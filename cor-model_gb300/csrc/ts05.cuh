// ts05.cuh -- the zero-tilt TS05 external field on the device (ts05_gsm,
// lib/ts05/ts05.c:7-134 with lib/ts05/{deformed,birk_tot,full_rc}.c;
// Tsyganenko-Sitnov 2005 with its fitted constants).
//
// Same terms and expression order as the reference, except that:
//   * every quantity that depends on PARMOD only (pow(Pdyn/2, ...), the
//     current amplitudes, the shifted shielding coefficients of shlcar5x5,
//     birk_shl and rc_shield, ...) comes from TS05Cond, filled on the host;
//   * square roots of constant expressions and sin/cos of the fixed quadrupole
//     angle come from the TS05Tables constant block, also host-computed;
//   * sin/cos of a shared argument are taken once;
//   * birk_tot's R12 and R22 modes, which ts05_gsm never uses
//     (ts05.c:82-83 vs :112-114), are not evaluated.
// Transcendentals are CUDA's FP64 library; pow(x, 2) is x*x.
#pragma once

#include "cor_device.cuh"

namespace cor {

struct TS05Cond {
    double xappa, xappa3, am, x0, asq, four_asq, two_asq, r_two_asq;
    double byimf, bzimf, oimfy_k, oimfz_k;   // oimf = b*imf * A[19]
    double dx1, dx2, d, xk1, xk2, scsy, scpr;
    double tamp1, tamp2, a_src, a_prc, a_r11, a_r21;
    double coef1[25], coef2[25];             // shlcar5x5: A[2l] + A[2l+1]*DXSHIFT
    double amp11[9], amp21[9];               // birk_shl amplitudes at X_SC
    double amp_sy[9], amp_pr[9];             // rc_shield amplitudes at X_SC
    double fac_sy, fac_pr;                   // rc_shield (X_SC + 1)^3
};

struct TS05Tables {
    double s3_sq[9], s3_rsq[3];              // shlcar3x3 sqrt(1/P^2 + 1/R^2); 1/sqrt of the R3 modes
    double s5_rp[2][5], s5_rr[2][5], s5_sq[2][25];
    double bs_p[2][3], bs_r[2][3], bs_sq[2][9];   // birk_shl tables SH11, SH21
    double rc_p[2][3], rc_r[2][3], rc_sq[2][9];   // rc_shield tables C_SY, C_PR
    double cphi, sphi;                       // cos/sin of the partial-ring quadrupole angle A[37]
    double rs_sq[2][20];                     // A[k]*A[k] of r_s / theta_s for the A11 and A21 tables
};

static __constant__ TS05Tables c_ts05;

// Region-1/Region-2 cone tables, birk_tot.c:126-164 (MODE 1 only)
static __constant__ double c_ts05_a11[31] = {
    .1618068350, -.1797957553, 2.999642482, -.9322708978, -.6811059760, .2099057262, -8.358815746,
    -14.86033550, .3838362986, -16.30945494, 4.537022847, 2.685836007, 27.97833029, 6.330871059,
    1.876532361, 18.95619213, .9651528100, .4217195118, -.08957770020, -1.823555887, .7457045438,
    -.5785916524, -1.010200918, .01112389357, .09572927448, -.3599292276, 8.713700514, .9763932955,
    3.834602998, 2.492118385, .7113544659};
static __constant__ double c_ts05_a21[31] = {
    .1278764024, -.2320034273, 1.805623266, -32.37241440, -.9931490648, .3175085630, -2.492465814,
    -16.21600096, .2695393416, -6.752691265, 3.971794901, 14.54477563, 41.10158386, 7.912889730,
    1.258297372, 9.583547721, 1.014141963, .5104134759, -.1790430468, -1.756358428, .7561986717,
    -.6775248254, -.04014016420, .01446794851, .1200521731, -.2203584559, 4.508963850, .8221623576,
    1.779933730, 1.102649543, .8867880020};

// ---- deformed.c ------------------------------------------------------------
static __device__ __noinline__ Vec3 ts05_taildisk(const double D0, const double DELTADX, const double x, const double y,
                                             const double z) {
    constexpr double F[5] = {-71.09346626, -1014.308601, -1272.939359, -3224.935936, -44546.86232};
    constexpr double B[5] = {10.90101242, 12.68393898, 13.51791954, 14.86775017, 15.12306404};
    constexpr double Cc[5] = {.7954069972, .6716601849, 1.174866319, 2.565249920, 10.01986790};
    const double rho = sqrt(x * x + y * y);
    const double rr = 1. / rho;
    const double drhodx = div_r(x, rho, rr), drhody = div_r(y, rho, rr);
    const double dex = ol_exp(div_c(x, 7., 1. / 7.));
    const double y20 = div_c(y, 20., 1. / 20.);
    const double d = D0 + 4.7 * y20 * y20 + DELTADX * dex;
    const double dddy = 4.7 * y * 0.005;
    const double dddx = div_c(DELTADX, 7., 1. / 7.) * dex;
    const double dzeta = sqrt(z * z + d * d);
    const double rdz = 1. / dzeta;
    const double ddzdx = div_r(d * dddx, dzeta, rdz), ddzdy = div_r(d * dddy, dzeta, rdz), ddzdz = div_r(z, dzeta, rdz);
    double bx = 0., by = 0., bz = 0.;
#pragma unroll
    for (int i = 0; i < 5; i++) {
        const double bi = B[i], ci = Cc[i];
        const double dzc = dzeta + ci;
        const double dzc2 = dzc * dzc;
        const double rpb = rho + bi, rmb = rho - bi;
        const double s1 = sqrt(rpb * rpb + dzc2), s2 = sqrt(rmb * rmb + dzc2);
        const double r1 = 1. / s1, r2 = 1. / s2;
        const double ds1dr = div_r(rho + bi, s1, r1), ds2dr = div_r(rho - bi, s2, r2);
        const double ds1dz = div_r(dzc, s1, r1), ds2dz = div_r(dzc, s2, r2);
        const double ds1dx = ds1dr * drhodx + ds1dz * ddzdx, ds1dy = ds1dr * drhody + ds1dz * ddzdy;
        const double ds1dzz = ds1dz * ddzdz;
        const double ds2dx = ds2dr * drhodx + ds2dz * ddzdx, ds2dy = ds2dr * drhody + ds2dz * ddzdy;
        const double ds2dzz = ds2dz * ddzdz;
        const double s12 = s1 * s2, sp = s1 + s2, sp2 = sp * sp;
        const double bi2 = 2. * bi;
        const double fac1 = sqrt(sp2 - bi2 * bi2);
        const double as = fac1 / (s12 * sp2);
        const double rsp = 1. / sp;
        const double asp = div_r(as, sp, rsp);
        const double das1 = (1. / (fac1 * s2) - asp * (s2 * s2 + s1 * (3. * s1 + 4. * s2))) / (s1 * sp);
        const double das2 = (1. / (fac1 * s1) - asp * (s1 * s1 + s2 * (3. * s2 + 4. * s1))) / (s2 * sp);
        const double dasdx = das1 * ds1dx + das2 * ds2dx;
        const double dasdy = das1 * ds1dy + das2 * ds2dy;
        const double dasdz = das1 * ds1dzz + das2 * ds2dzz;
        bx = bx - F[i] * x * dasdz;
        by = by - F[i] * y * dasdz;
        bz = bz + F[i] * (2. * as + x * dasdx + y * dasdy);
    }
    return {bx, by, bz};
}

// shlcar5x5, deformed.c:169-208, table t (0: A1 of unwarped, 1: A2)
static __device__ __noinline__ Vec3 ts05_shlcar5x5(const int t, const double* __restrict__ coef, const double x,
                                              const double y, const double z) {
    double szk[5], czk[5];
#pragma unroll
    for (int k = 0; k < 5; k++) ol_sincos(z * c_ts05.s5_rr[t][k], &szk[k], &czk[k]);
    double hx = 0., hy = 0., hz = 0.;
#pragma unroll
    for (int i = 0; i < 5; i++) {
        const double rp = c_ts05.s5_rp[t][i];
        double sy, cy;
        ol_sincos(y * rp, &sy, &cy);
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const double rr = c_ts05.s5_rr[t][k];
            const double sq = c_ts05.s5_sq[t][5 * i + k];
            const double e = ol_exp(x * sq);
            const double c = coef[5 * i + k];
            hx = hx + c * (-sq * e * cy * szk[k]);
            hy = hy + c * (rp * e * sy * szk[k]);
            hz = hz + c * (-rr * e * cy * czk[k]);
        }
    }
    return {hx, hy, hz};
}

// warped + unwarped, deformed.c:4-92
static __device__ __noinline__ void ts05_warped(const TS05Cond& c, const double x, const double y, const double z, Vec3& b1,
                                            Vec3& b2) {
    const double rho2 = y * y + z * z;
    const double rho = sqrt(rho2);
    double phi = 0., cphi = 1., sphi = 0.;
    if (y != 0. || z != 0.) {
        phi = ol_atan2(z, y);
        const double rr = 1. / rho;
        cphi = div_r(y, rho, rr);
        sphi = div_r(z, rho, rr);
    }
    double sf, cf;
    ol_sincos(phi, &sf, &cf);
    const double yy = rho * cf, zz = rho * sf;
    const Vec3 f1 = ts05_taildisk(c.d * 1.1, 1., (x - 6. - c.dx1) * 1.1 + 1.2, yy * 1.1, zz * 1.1);
    const Vec3 h1 = ts05_shlcar5x5(0, c.coef1, x, yy, zz);
    const Vec3 f2 = ts05_taildisk(c.d * 0.25, 0., (x - 4. - c.dx2) * 0.25 - 9., yy * 0.25, zz * 0.25);
    const Vec3 h2 = ts05_shlcar5x5(1, c.coef2, x, yy, zz);
    const Vec3 u1 = {f1.x + h1.x, f1.y + h1.y, f1.z + h1.z};
    const Vec3 u2 = {f2.x + h2.x, f2.y + h2.y, f2.z + h2.z};
    double br = u1.y * cf + u1.z * sf;
    double bp = -u1.y * sf + u1.z * cf;
    b1 = {u1.x, br * cphi - bp * sphi, br * sphi + bp * cphi};
    br = u2.y * cf + u2.z * sf;
    bp = -u2.y * sf + u2.z * cf;
    b2 = {u2.x, br * cphi - bp * sphi, br * sphi + bp * cphi};
}

// ---- birk_tot.c ---------------------------------------------------------------
__device__ __forceinline__ double ts05_r_s(const double* __restrict__ A, const double* __restrict__ q, const double R,
                                           const double cth, const double c2th) {
    const double R2 = R * R;
    const double R2aa = R2 + q[15];
    const double rr = 1. / R;
    return R + div_r(A[1], R, rr) + A[2] * R / sqrt(R2 + q[10]) + A[3] * R / (R2 + q[11]) +
           (A[4] + div_r(A[5], R, rr) + A[6] * R / sqrt(R2 + q[12]) + A[7] * R / (R2 + q[13])) * cth +
           (A[8] * R / sqrt(R2 + q[14]) + A[9] * R / (R2aa * R2aa)) * c2th;
}

__device__ __forceinline__ double ts05_theta_s(const double* __restrict__ A, const double* __restrict__ q,
                                               const double R, const double TH, const double sth, const double s2th,
                                               const double s3th) {
    const double R2 = R * R;
    const double rr = 1. / R;
    return TH + (A[16] + div_r(A[17], R, rr) + A[18] / R2 + A[19] * R / sqrt(R2 + q[26 - 10])) * sth +
           (A[20] + A[21] * R / sqrt(R2 + q[27 - 10]) + A[22] * R / (R2 + q[28 - 10])) * s2th +
           (A[23] + div_r(A[24], R, rr) + A[25] * R / (R2 + q[29 - 10])) * s3th;
}

// fialcos, birk_tot.c:311-372, MODE = 1
static __device__ __noinline__ void ts05_fialcos1(const double R, const double TH, const double sf, const double cfi,
                                              const double th0, const double dt, double& bt, double& bp) {
    double st, ctt;
    ol_sincos(TH, &st, &ctt);
    const double ro = R * st;
    const double tg = st / (1. + ctt);
    const double ctg = st / (1. - ctt);
    const double tnp = th0 + dt, tnm = th0 - dt;
    double tgp = 0., tgm = 0., tgm2 = 0., tgp2 = 0.;
    if (TH >= tnm) {
        tgp = tan(tnp * 0.5);
        tgm = tan(tnm * 0.5);
        tgm2 = tgm * tgm;
        tgp2 = tgp * tgp;
    }
    const double tm = 1. * tg;
    const double ccos = 1. * cfi - 0. * sf;
    const double ssin = 0. * cfi + 1. * sf;
    double t, dtt;
    if (TH < tnm) {
        t = tm;
        dtt = 0.5 * 1 * tm * (tg + ctg);
    } else if (TH < tnp) {
        const double tgm2m = 1. * tgm2;
        const double fc = 1. / (tgp - tgm);
        const double fc1 = 1. / (2 * 1 + 1);
        const double tgm2m1 = tgm2m * tgm;
        const double tg21 = 1. + tg * tg;
        t = fc * (tm * (tgp - tg) + fc1 * (tm * tg - tgm2m1 / tm));
        dtt = 0.5 * 1 * fc * tg21 * (tm / tg * (tgp - tg) - fc1 * (tm - tgm2m1 / (tm * tg)));
    } else {
        const double tgp2m = 1. * tgp2, tgm2m = 1. * tgm2;
        const double fc = 1. / (tgp - tgm);
        const double fc1 = 1. / (2 * 1 + 1);
        t = fc * fc1 * (tgp2m * tgp - tgm2m * tgm) / tm;
        dtt = -t * 1 * 0.5 * (tg + ctg);
    }
    bt = (1 * t * ccos / ro) * 800.;
    bp = (-dtt * ssin / R) * 800.;
}

// one_cone, birk_tot.c:248-291 (MODE 1)
static __device__ __noinline__ Vec3 ts05_one_cone(const double* __restrict__ A, const double* __restrict__ q,
                                             const double x, const double y, const double z, const double dth) {
    const double th0 = A[30];
    const double rho2 = x * x + y * y;
    const double rho = sqrt(rho2);
    const double R = sqrt(rho2 + z * z);
    const double TH = ol_atan2(rho, z);
    const double PHI = ol_atan2(y, x);
    double sth, cth, s2, c2, s3;
    ol_sincos(TH, &sth, &cth);
    ol_sincos(2. * TH, &s2, &c2);
    s3 = ol_sin(3. * TH);
    const double rs = ts05_r_s(A, q, R, cth, c2);
    const double ths = ts05_theta_s(A, q, R, TH, sth, s2, s3);
    double sf, cfi;
    ol_sincos(PHI, &sf, &cfi);
    double btast, bfast;
    ts05_fialcos1(rs, ths, sf, cfi, th0, dth, btast, bfast);
    const double rr = 1. / R;
    const double rsr = div_r(rs, R, rr);
    const double stsst = ol_sin(ths) / sth;
    const double rdp = R + 1E-6, rdm = R - 1E-6;
    const double drsdr = div_c(ts05_r_s(A, q, rdp, cth, c2) - ts05_r_s(A, q, rdm, cth, c2), 2E-6, 1. / 2E-6);
    const double tdp = TH + 1E-6, tdm = TH - 1E-6;
    double sp, cp, sm, cm, s2p, c2p, s2m, c2m;
    ol_sincos(tdp, &sp, &cp);
    ol_sincos(tdm, &sm, &cm);
    ol_sincos(2. * tdp, &s2p, &c2p);
    ol_sincos(2. * tdm, &s2m, &c2m);
    const double drsdt = div_c(ts05_r_s(A, q, R, cp, c2p) - ts05_r_s(A, q, R, cm, c2m), 2E-6, 1. / 2E-6);
    const double dtsdr = div_c(ts05_theta_s(A, q, rdp, TH, sth, s2, s3) - ts05_theta_s(A, q, rdm, TH, sth, s2, s3),
                               2E-6, 1. / 2E-6);
    const double dtsdt = div_c(ts05_theta_s(A, q, R, tdp, sp, s2p, ol_sin(3. * tdp)) -
                                   ts05_theta_s(A, q, R, tdm, sm, s2m, ol_sin(3. * tdm)),
                               2E-6, 1. / 2E-6);
    const double br = -div_r(rsr, R, rr) * stsst * btast * drsdt;
    const double bth = rsr * stsst * btast * drsdr;
    const double bph = rsr * bfast * (drsdr * dtsdt - drsdt * dtsdr);
    const double s = div_r(rho, R, rr), c = div_r(z, R, rr);
    const double rrho = 1. / rho;
    const double sfv = div_r(y, rho, rrho), cfv = div_r(x, rho, rrho);
    const double be = br * s + bth * c;
    return {A[0] * (be * cfv - bph * sfv), A[0] * (be * sfv + bph * cfv), A[0] * (br * c - bth * s)};
}

// birk_1n2, birk_tot.c:125-234 (MODE 1), numb 1 -> R11, 2 -> R21
static __device__ __noinline__ Vec3 ts05_birk_1n2(const int numb, const double x, const double y, const double z,
                                             const double xkappa) {
    const double dphi = numb == 1 ? 0.055 : 0.030;
    const double dth = numb == 1 ? 0.06 : 0.09;
    const double xs_ = x * xkappa, ys = y * xkappa, zs_ = z * xkappa;
    const double xs2 = xs_ * xs_, zs2 = zs_ * zs_;
    const double rho = sqrt(xs2 + zs2);
    const double rho2 = rho * rho;
    double phi = 0.;
    if (xs_ != 0. || zs_ != 0.) phi = ol_atan2(-zs_, xs_);
    double sphic, cphic;
    ol_sincos(phi, &sphic, &cphic);
    const double r02 = 49. + rho2;
    const double brack = dphi + 0.5 * 49. / 50. * (rho2 - 1.) / r02;
    const double phis = phi - brack * sphic;
    const double dpsp = 1. - brack * cphic;
    const double dpsr = -2. * 0.5 * 49. * rho / (r02 * r02) * sphic;
    double sphics, cphics;
    ol_sincos(phis, &sphics, &cphics);
    const double xs = rho * cphics, zs = -rho * sphics;
    const double* A = numb == 1 ? c_ts05_a11 : c_ts05_a21;
    const double* q = c_ts05.rs_sq[numb - 1];
    const Vec3 bn = ts05_one_cone(A, q, xs, ys, zs, dth);
    const Vec3 bs = ts05_one_cone(A, q, xs, -ys, -zs, dth);
    const double bxs = bn.x - bs.x, byas = bn.y + bs.y, bzs = bn.z + bs.z;
    const double brhoas = bxs * cphics - bzs * sphics;
    const double bphias = -bxs * sphics - bzs * cphics;
    const double brho_s = brhoas * dpsp * xkappa;
    const double bphi_s = (bphias - rho * (brhoas * dpsr)) * xkappa;
    const double by_s = byas * dpsp * xkappa;
    return {brho_s * cphic - bphi_s * sphic, by_s, -brho_s * sphic - bphi_s * cphic};
}

// birk_shl (birk_tot.c:374-403, fac = 1) and rc_shield (full_rc.c:690-721):
// 3x3 Cartesian shields with condition-dependent amplitudes.
static __device__ __noinline__ Vec3 ts05_shield3(const double* __restrict__ P, const double* __restrict__ Rr,
                                            const double* __restrict__ SQ, const double* __restrict__ amp,
                                            const double fac, const bool has_fac, const double x, const double y,
                                            const double z) {
    double szk[3], czk[3];
#pragma unroll
    for (int k = 0; k < 3; k++) ol_sincos(z / Rr[k], &szk[k], &czk[k]);
    double gx = 0., gy = 0., gz = 0.;
#pragma unroll
    for (int j = 0; j < 3; j++) {
        const double p = P[j];
        double sy, cy;
        ol_sincos(y / p, &sy, &cy);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const double sq = SQ[3 * j + k];
            const double e = ol_exp(x * sq);
            const double a = amp[3 * j + k];
            if (has_fac) {
                gx += (-sq * e * cy * szk[k] * fac) * a;
                gy += (e * sy * szk[k] / p * fac) * a;
                gz += (-e * cy * czk[k] / Rr[k] * fac) * a;
            } else {
                gx += (-sq * e * cy * szk[k]) * a;
                gy += (e * sy * szk[k] / p) * a;
                gz += (-e * cy * czk[k] / Rr[k]) * a;
            }
        }
    }
    return {gx, gy, gz};
}

// ---- full_rc.c ------------------------------------------------------------------
__device__ __forceinline__ void ts05_ellip(const double xk2s, double& elk, double& ele) {
    const double dl = ol_log(1. / xk2s);
    elk = 1.38629436112 + xk2s * (0.09666344259 + xk2s * (0.03590092383 + xk2s * (0.03742563713 + xk2s * 0.01451196212))) +
          dl * (0.5 + xk2s * (0.12498593597 + xk2s * (0.06880248576 + xk2s * (0.03328355346 + xk2s * 0.00441787012))));
    ele = 1. + xk2s * (0.44325141463 + xk2s * (0.0626060122 + xk2s * (0.04757383546 + xk2s * 0.01736506451))) +
          dl * xk2s * (0.2499836831 + xk2s * (0.09200180037 + xk2s * (0.04069697526 + xk2s * 0.00526449639)));
}

static __device__ __noinline__ double ts05_two_loops(const double alpha_s, const double gamma_s, const double rrc1,
                                                 const double dd1, const double rrc2, const double dd2,
                                                 const double a1, const double a2) {
    const double gs2 = gamma_s * gamma_s;
    const double alsqh = (alpha_s * alpha_s) * 0.5;
    const double F = 64. / 27. * gs2 + (alsqh * alsqh);
    const double Q = ol_pow((sqrt(F) + alsqh), (1. / 3.));
    const double g13 = ol_pow(gs2, (1. / 3.));
    double C = Q - 4. * g13 / (3. * Q);
    if (C < 0.) C = 0.;
    const double G = sqrt(C * C + 4. * g13);
    const double RS = 4. / ((sqrt(2. * G - C) + sqrt(C)) * (G + C));
    const double costs = gamma_s * (RS * RS);
    const double sints = sqrt(1. - costs * costs);
    const double rhos = RS * sints;
    const double zs = RS * costs;
    const double zs2 = zs * zs;
    const double srh = sqrt(rhos);
    double elk, ele;
    const double r1 = rrc1 + rhos;
    double P = r1 * r1 + zs2 + dd1 * dd1;
    double xk2 = 4. * rrc1 * rhos / P;
    double xkr = sqrt(xk2) * srh;
    ts05_ellip(1. - xk2, elk, ele);
    const double aphi1 = ((1. - xk2 * 0.5) * elk - ele) / xkr;
    const double r2 = rrc2 + rhos;
    P = r2 * r2 + zs2 + dd2 * dd2;
    xk2 = 4. * rrc2 * rhos / P;
    xkr = sqrt(xk2) * srh;
    ts05_ellip(1. - xk2, elk, ele);
    const double aphi2 = ((1. - xk2 * 0.5) * elk - ele) / xkr;
    return a1 * aphi1 + a2 * aphi2;
}

static __device__ __noinline__ double ts05_ap(const double R, const double sint, const double cost) {
    bool prox = false;
    double s1 = sint, c1 = cost;
    if (s1 < 1.E-2) {
        s1 = 1.E-2;
        c1 = .99994999875;
        prox = true;
    }
    const double q1 = div_c(R - 3.746064740, 1.508802177, 1. / 1.508802177);
    const double q2 = div_c(R - 4.993638842, 3.324180497, 1. / 3.324180497);
    const double q3 = div_c(R - 2.969226745, 2.243367377, 1. / 2.243367377);
    const double l1 = div_c(c1, 0.5873525737, 1. / 0.5873525737), l2 = div_c(c1, 0.4368407663, 1. / 0.4368407663);
    const double arg1 = -(q1 * q1) - (l1 * l1);
    const double arg2 = -(q2 * q2) - (l2 * l2);
    const double arg3 = -(q3 * q3);
    const double e1 = arg1 >= -500. ? ol_exp(arg1) : 0.;
    const double e2 = arg2 >= -500. ? ol_exp(arg2) : 0.;
    const double e3 = arg3 >= -500. ? ol_exp(arg3) : 0.;
    const double alpha = (s1 * s1) / R;
    const double alpha_s = alpha * (1. + -0.2291904607 * e1 + 0.1556236119 * e2 + 0.1855957207 * e3);
    const double gamma = c1 / (R * R);
    double ap = ts05_two_loops(alpha_s, gamma, 4.274684950, 2.439528329, 3.367557287, 3.146382545, -456.5289941,
                               375.9055332);
    if (prox) ap = ap * sint / s1;
    return ap;
}

static __device__ __noinline__ double ts05_apprc(const double R, const double sint, const double cost) {
    constexpr double P1 = .3058309043, ALPHA1 = .1817139853, DAL1 = .1257532909, BETA1 = 3.422509402, DG1 = .04742939676;
    constexpr double P2 = -4.800458958, ALPHA2 = -.02845643596, DAL2 = .2188114228, BETA2 = 2.545944574, DG2 = .00813272793;
    constexpr double BETA3 = .35868244, P3 = 103.1601001, ALPHA3 = -.00764731187, DAL3 = .1046487459;
    constexpr double BETA4 = 2.958863546, DG3 = .01172314188, BETA5 = .4382872938, Q0 = .01134908150;
    constexpr double Q1 = 14.51339943, ALPHA4 = .2647095287, DAL4 = .07091230197, DG4 = .01512963586;
    constexpr double Q2 = 6.861329631, ALPHA5 = .1677400816, DAL5 = .04433648846, DG5 = .05553741389;
    constexpr double BETA6 = .7665599464, BETA7 = .7277854652;
    bool prox = false;
    double s1 = sint, c1 = cost;
    if (s1 < 1.E-2) {
        s1 = 1.E-2;
        c1 = .99994999875;
        prox = true;
    }
    const double alpha = (s1 * s1) / R;
    const double gamma = c1 / (R * R);
    const double g1 = div_c(gamma, DG1, 1. / DG1), g4 = div_c(gamma, DG4, 1. / DG4);
    const double a4 = div_c(alpha - ALPHA4, DAL4, 1. / DAL4);
    const double arg1 = -(g1 * g1);
    const double arg2 = -(a4 * a4) - (g4 * g4);
    const double e1 = arg1 >= -500. ? ol_exp(arg1) : 0.;
    const double e2 = arg2 >= -500. ? ol_exp(arg2) : 0.;
    const double u1 = div_c(alpha - ALPHA1, DAL1, 1. / DAL1);
    const double u2 = div_c(alpha - ALPHA2, DAL2, 1. / DAL2);
    const double u3 = div_c(alpha - ALPHA3, DAL3, 1. / DAL3);
    const double u5 = div_c(alpha - ALPHA5, DAL5, 1. / DAL5);
    const double v2 = div_c(gamma, DG2, 1. / DG2), v3 = div_c(gamma, DG3, 1. / DG3), v5 = div_c(gamma, DG5, 1. / DG5);
    const double am3 = alpha - ALPHA3;
    const double alpha_s = alpha * (1. + P1 / ol_pow((1. + u1 * u1), BETA1) * e1 +
                                    P2 * (alpha - ALPHA2) / ol_pow((1. + u2 * u2), BETA2) / ol_pow((1. + v2 * v2), BETA3) +
                                    P3 * (am3 * am3) / ol_pow((1. + u3 * u3), BETA4) / ol_pow((1. + v3 * v3), BETA5));
    const double gamma_s = gamma * (1. + Q0 + Q1 * (alpha - ALPHA4) * e2 +
                                    Q2 * (alpha - ALPHA5) / ol_pow((1. + u5 * u5), BETA6) / ol_pow((1. + v5 * v5), BETA7));
    double ap = ts05_two_loops(alpha_s, gamma_s, 6.560486035, 1.930711037, 3.827208119, .7789990504, -80.11202281,
                               12.58246758);
    if (prox) ap = ap * sint / s1;
    return ap;
}

// rc_symm (full_rc.c:116-152) and prc_symm (:264-300)
template <bool PRC>
static __device__ __noinline__ Vec3 ts05_symm(const double x, const double y, const double z) {
    constexpr double DS = 1.E-2, DC = 0.99994999875, D = 1.E-4, DRD = 5E3;
    const double rho2 = x * x + y * y;
    const double r2 = rho2 + z * z;
    const double R = sqrt(r2);
    const double rp = R + D, rm = R - D;
    const double rr = 1. / R;
    const double sint = div_r(sqrt(rho2), R, rr);
    const double cost = div_r(z, R, rr);
    double fxy, bz;
    if (sint < DS) {
        const double A = (PRC ? ts05_apprc(R, DS, DC) : ts05_ap(R, DS, DC)) / DS;
        const double dardr = (rp * (PRC ? ts05_apprc(rp, DS, DC) : ts05_ap(rp, DS, DC)) -
                              rm * (PRC ? ts05_apprc(rm, DS, DC) : ts05_ap(rm, DS, DC))) *
                             DRD;
        fxy = z * (2. * A - dardr) / (R * r2);
        bz = div_r(2. * A * (cost * cost) + dardr * (sint * sint), R, rr);
    } else {
        const double th = ol_atan2(sint, cost);
        double stp, ctp, stm, ctm;
        ol_sincos(th + D, &stp, &ctp);
        ol_sincos(th - D, &stm, &ctm);
        const double br = (stp * (PRC ? ts05_apprc(R, stp, ctp) : ts05_ap(R, stp, ctp)) -
                           stm * (PRC ? ts05_apprc(R, stm, ctm) : ts05_ap(R, stm, ctm))) /
                          (R * sint) * DRD;
        const double bt = div_r(rm * (PRC ? ts05_apprc(rm, sint, cost) : ts05_ap(rm, sint, cost)) -
                                    rp * (PRC ? ts05_apprc(rp, sint, cost) : ts05_ap(rp, sint, cost)),
                                R, rr) *
                          DRD;
        fxy = div_r(br + bt * cost / sint, R, rr);
        bz = br * cost - bt * sint;
    }
    return {fxy * x, fxy * y, bz};
}

__device__ __forceinline__ void ts05_ffs(const double A, const double A0, const double DA, double& F, double& FA,
                                         double& FS) {
    const double da2 = DA * DA;
    const double p = A + A0, m = A - A0;
    const double sq1 = sqrt(p * p + da2), sq2 = sqrt(m * m + da2);
    FA = 2. / (sq1 + sq2);
    F = FA * A;
    FS = 0.5 * (sq1 + sq2) / (sq1 * sq2) * (1. - F * F);
}

static __device__ __noinline__ double ts05_br_prc_q(const double R, const double sint, const double cost) {
    const double sint2 = sint * sint, cost2 = cost * cost, sc = sint * cost;
    const double alpha = sint2 / R;
    const double gamma = cost / (R * R);
    double F, FA, FS;
    ts05_ffs(alpha, .1417519429, .6388013110E-02, F, FA, FS);
    const double d1 = sc * ol_pow(F, 2.318824273) / (ol_pow(div_c(R, 5.303934488, 1. / 5.303934488), 4.213397467) + 1.);
    const double d2 = d1 * cost2;
    ts05_ffs(alpha, .1401142771, .2306094179E-01, F, FA, FS);
    const double d3 = sc * ol_pow(FS, .7955534018) / (ol_pow(div_c(R, 3.462235072, 1. / 3.462235072), 2.568743010) + 1.);
    const double d4 = d3 * cost2;
    ts05_ffs(alpha, .1485233485, .2319676273E-01, F, FA, FS);
    const double d5 = sc * (ol_pow(alpha, 3.477425908)) * (ol_pow(FS, 1.922155110)) /
                      (ol_pow(div_c(R, 7.830223587, 1. / 7.830223587), 8.492933868) + 1.);
    const double d6 = d5 * cost2;
    const double a4 = div_c(alpha - .1295221828, .01753008801, 1. / .01753008801);
    const double g1 = div_c(gamma, .01125504083, 1. / .01125504083);
    double arga = a4 * a4 + 1.;
    double argg = 1. + g1 * g1;
    double ra = 1. / arga;
    const double d7 = sc / arga / argg, d8 = div_r(d7, arga, ra), d9 = div_r(d8, arga, ra), d10 = div_r(d9, arga, ra);
    const double a5 = div_c(alpha - .1811846095, .04841237481, 1. / .04841237481);
    const double g2 = div_c(gamma, .01981805097, 1. / .01981805097);
    arga = a5 * a5 + 1.;
    argg = 1. + g2 * g2;
    ra = 1. / arga;
    const double d11 = sc / arga / argg, d12 = div_r(d11, arga, ra), d13 = div_r(d12, arga, ra),
                 d14 = div_r(d13, arga, ra);
    const double r4 = R * R * R * R;
    constexpr double C1 = 6.557801891, C2 = 6.348576071, C3 = 5.744436687;
    const double d15 = sc / (r4 + C1 * C1 * C1 * C1);
    const double d16 = sc / (r4 + C2 * C2 * C2 * C2) * cost2;
    const double d17 = sc / (r4 + C3 * C3 * C3 * C3) * (cost2 * cost2);
    ts05_ffs(alpha, .2265212965, .1301957209, F, FA, FS);
    const double rd = div_c(R - 1.2, .5654023158, 1. / .5654023158);
    const double d18 = sc * FS / (1. + rd * rd);
    return -21.2666329 * d1 + 32.24527521 * d2 + -6.062894078 * d3 + 7.515660734 * d4 + 233.7341288 * d5 +
           -227.1195714 * d6 + 8.483233889 * d7 + 16.80642754 * d8 + -24.63534184 * d9 + 9.067120578 * d10 +
           -1.052686913 * d11 + -12.08384538 * d12 + 18.61969572 * d13 + -12.71686069 * d14 + 47017.35679 * d15 +
           -50646.71204 * d16 + 7746.058231 * d17 + 1.531069371 * d18;
}

static __device__ __noinline__ double ts05_bt_prc_q(const double R, const double sint, const double cost) {
    const double sint2 = sint * sint, cost2 = cost * cost;
    const double alpha = sint2 / R;
    const double gamma = cost / (R * R);
    double F, FA, FS;
    ts05_ffs(alpha, .2071721360, .05030555417, F, FA, FS);
    const double d1 = ol_pow(F, 1.243288286) / (ol_pow(div_c(R, 7.471332374, 1. / 7.471332374), 3.180533613) + 1.);
    const double d2 = d1 * cost2;
    ts05_ffs(alpha, .1568504222, .02092910682, F, FA, FS);
    const double d3 = ol_pow(FA, 1.376743507) / ol_pow(R, 1.985148197);
    const double d4 = d3 * cost2;
    ts05_ffs(alpha, .1701395257, .1019870070, F, FA, FS);
    const double d5 = ol_pow(FS, .3157139940) * ol_pow(alpha, 1.056309517) /
                      (ol_pow(div_c(R, 6.293740981, 1. / 6.293740981), 5.671824276) + 1.);
    const double d6 = d5 * cost2;
    ts05_ffs(gamma, 0., .01040696080, F, FA, FS);
    const double a4 = div_c(alpha - .1280772299, .02189060799, 1. / .02189060799);
    const double fcc = (1. + a4 * a4);
    const double rf = 1. / fcc;
    const double d7 = rf * FS, d8 = div_r(d7, fcc, rf), d9 = div_r(d8, fcc, rf), d10 = div_r(d9, fcc, rf);
    const double a5 = div_c(alpha - .1648265607, .04701592613, 1. / .04701592613);
    const double g2 = div_c(gamma, .01526400086, 1. / .01526400086);
    const double arg = 1. + a5 * a5;
    const double ra = 1. / arg;
    const double d11 = ra / (1. + g2 * g2), d12 = div_r(d11, arg, ra), d13 = div_r(d12, arg, ra),
                 d14 = div_r(d13, arg, ra);
    const double r4 = R * R * R * R;
    constexpr double C1 = 12.88384229, C2 = 3.361775101, C3 = 23.44173897;
    const double d15 = 1. / (r4 + C1 * C1);
    const double d16 = cost2 / (r4 + C2 * C2);
    const double d17 = (cost2 * cost2) / (r4 + C3 * C3);
    return 12.74640393 * d1 + -7.516393516 * d2 + -5.476233865 * d3 + 3.212704645 * d4 + -59.10926169 * d5 +
           46.62198189 * d6 + -.01644280062 * d7 + .1234229112 * d8 + -.08579198697 * d9 + .01321366966 * d10 +
           .8970494003 * d11 + 9.136186247 * d12 + -38.19301215 * d13 + 21.73775846 * d14 + -410.0783424 * d15 +
           -69.90832690 * d16 + -848.8543440 * d17;
}

// prc_quad, full_rc.c:425-481
static __device__ __noinline__ Vec3 ts05_prc_quad(const double x, const double y, const double z) {
    constexpr double D = 1.E-4, DD = 2.E-4, DS = 1.E-2, DC = 0.99994999875;
    const double rho2 = x * x + y * y;
    const double R = sqrt(rho2 + z * z);
    const double rho = sqrt(rho2);
    const double rr = 1. / R;
    const double sint = div_r(rho, R, rr), cost = div_r(z, R, rr);
    const double rp = R + D, rm = R - D;
    if (sint > DS) {
        const double rrho = 1. / rho;
        const double cphi = div_r(x, rho, rrho), sphi = div_r(y, rho, rrho);
        const double br = ts05_br_prc_q(R, sint, cost);
        const double bt = ts05_bt_prc_q(R, sint, cost);
        const double dbrr = div_c(ts05_br_prc_q(rp, sint, cost) - ts05_br_prc_q(rm, sint, cost), DD, 1. / DD);
        const double th = ol_atan2(sint, cost);
        double stp, ctp, stm, ctm;
        ol_sincos(th + D, &stp, &ctp);
        ol_sincos(th - D, &stm, &ctm);
        const double dbtt = div_c(ts05_bt_prc_q(R, stp, ctp) - ts05_bt_prc_q(R, stm, ctm), DD, 1. / DD);
        return {sint * (br + (br + R * dbrr + dbtt) * (sphi * sphi)) + cost * bt,
                -sint * sphi * cphi * (br + R * dbrr + dbtt), (br * cost - bt * sint) * cphi};
    }
    const double st = DS;
    const double ct = z < 0. ? -DC : DC;
    const double th = ol_atan2(st, ct);
    double stp, ctp, stm, ctm;
    ol_sincos(th + D, &stp, &ctp);
    ol_sincos(th - D, &stm, &ctm);
    const double br = ts05_br_prc_q(R, st, ct);
    const double bt = ts05_bt_prc_q(R, st, ct);
    const double dbrr = div_c(ts05_br_prc_q(rp, st, ct) - ts05_br_prc_q(rm, st, ct), DD, 1. / DD);
    const double dbtt = div_c(ts05_bt_prc_q(R, stp, ctp) - ts05_bt_prc_q(R, stm, ctm), DD, 1. / DD);
    const double fcxy = R * dbrr + dbtt;
    const double rst = R * st;
    const double rst2 = rst * rst;
    const double y2 = y * y;
    const double rr2 = 1. / rst2;
    return {div_r(br * (x * x + 2. * y2) + fcxy * y2, rst2, rr2) + bt * cost, div_r(-(br + fcxy) * x * y, rst2, rr2),
            div_r((br * cost / st - bt) * x, R, rr)};
}

// ---- ts05.c ---------------------------------------------------------------------
// shlcar3x3, ts05.c:136-235
static __device__ __noinline__ Vec3 ts05_shlcar3x3(const double x, const double y, const double z) {
    constexpr double PS[3] = {9.620648151, 6.082014949, 27.75216226};
    constexpr double R1 = 12.44199571, R2 = 5.122226936, R3 = 6.982039615;
    constexpr double r32 = R3 * R3;
    constexpr double AM[9] = {-901.2327248 + 895.8011176, 817.6208321 - 845.5880889, -83.73539535 + 86.58542841,
                              336.8781402 - 329.3619944,  -311.2947120 + 308.6011161, 31.94469304 - 31.30824526,
                              125.8739681 - 372.3384278,  -235.4720434 + 286.7594095, 21.86305585 - 27.42344605};
    const double z1 = div_c(z, R1, 1. / R1), z2 = div_c(z, R2, 1. / R2), z3 = div_c(z, R3, 1. / R3);
    double s1, c1, s2, c2, s3, c3;
    ol_sincos(z1, &s1, &c1);
    ol_sincos(z2, &s2, &c2);
    ol_sincos(z3, &s3, &c3);
    const double s3r = div_c(s3, R3, 1. / R3);
    const double xr3 = div_c(x, R3, 1. / R3);
    const double xr32 = div_c(x, r32, 1. / r32);
    double bx = 0., by = 0., bz = 0.;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double P = PS[i];
        double syp, cyp;
        ol_sincos(div_c(y, P, 1. / P), &syp, &cyp);
        double h[9];
        double sq = c_ts05.s3_sq[3 * i];
        double e = ol_exp(sq * x);
        const double ep = div_c(e, P, 1. / P);
        h[0] = -sq * e * cyp * s1;
        h[1] = ep * syp * s1;
        h[2] = div_c(-e * cyp, R1, 1. / R1) * c1;
        sq = c_ts05.s3_sq[3 * i + 1];
        e = ol_exp(sq * x);
        const double ep2 = div_c(e, P, 1. / P);
        h[3] = -sq * e * cyp * s2;
        h[4] = ep2 * syp * s2;
        h[5] = div_c(-e * cyp, R2, 1. / R2) * c2;
        sq = c_ts05.s3_sq[3 * i + 2];
        const double rsq = c_ts05.s3_rsq[i];
        e = ol_exp(sq * x);
        const double ep3 = div_c(e, P, 1. / P);
        h[6] = -e * cyp * (sq * z * c3 + s3r * (x + rsq));
        h[7] = ep3 * syp * (z * c3 + div_r(xr3 * s3, sq, rsq));
        h[8] = -e * cyp * (c3 * (1. + div_r(xr32, sq, rsq)) - z3 * s3);
        const double a0 = AM[3 * i], a1 = AM[3 * i + 1], a2 = AM[3 * i + 2];
        if (i == 0) {
            bx = a0 * h[0];
            by = a0 * h[1];
            bz = a0 * h[2];
        } else {
            bx = bx + a0 * h[0];
            by = by + a0 * h[1];
            bz = bz + a0 * h[2];
        }
        bx = bx + a1 * h[3];
        by = by + a1 * h[4];
        bz = bz + a1 * h[5];
        bx = bx + a2 * h[6];
        by = by + a2 * h[7];
        bz = bz + a2 * h[8];
    }
    return {bx, by, bz};
}

__device__ __forceinline__ Vec3 ts05_dipole(const double x, const double y, const double z) {
    const double p = x * x, u = z * z, t = y * y;
    const double sq = sqrt(p + t + u);
    const double q = 30115. / (sq * sq * sq * sq * sq);
    return {q * 3. * z * x, q * -3. * z * y, q * (p + t - 2. * u)};
}

// ts05_gsm, ts05.c:7-134.  X = GSM position [R_E].
static __device__ __noinline__ Vec3 ts05_field(const TS05Cond& c, const Vec3 X) {
    const double x = X.x, y = X.y, z = X.z;
    const double oimfy = c.oimfy_k, oimfz = c.oimfz_k;
    double xmxm = c.am + x - c.x0;
    if (xmxm < 0) xmxm = 0.;
    const double axx0 = xmxm * xmxm;
    const double rho2 = y * y + z * z;
    const double aro = (c.asq + rho2) + axx0;
    const double sigma = sqrt(div_r(aro + sqrt(aro * aro - c.four_asq * axx0), c.two_asq, c.r_two_asq));
    if (!(sigma < 1.1960 + 0.005)) {
        const Vec3 q = ts05_dipole(x, y, z);
        return {-q.x, oimfy - q.y, oimfz - q.z};
    }
    const double xx = x * c.xappa, yy = y * c.xappa, zz = z * c.xappa;
    const Vec3 cf = ts05_shlcar3x3(xx, yy, zz);
    Vec3 t1, t2;
    ts05_warped(c, xx, yy, zz, t1, t2);
    // birk_tot (R11 and R21)
    const Vec3 f11 = ts05_birk_1n2(1, xx, yy, zz, c.xk1);
    const Vec3 h11 = ts05_shield3(c_ts05.bs_p[0], c_ts05.bs_r[0], c_ts05.bs_sq[0], c.amp11, 1., false, xx, yy, zz);
    const Vec3 f21 = ts05_birk_1n2(2, xx, yy, zz, c.xk2);
    const Vec3 h21 = ts05_shield3(c_ts05.bs_p[1], c_ts05.bs_r[1], c_ts05.bs_sq[1], c.amp21, 1., false, xx, yy, zz);
    const Vec3 r11 = {f11.x + h11.x, f11.y + h11.y, f11.z + h11.z};
    const Vec3 r21 = {f21.x + h21.x, f21.y + h21.y, f21.z + h21.z};
    // full_rc
    const double rsy = 1. / c.scsy, rpr = 1. / c.scpr;
    const Vec3 bs = ts05_symm<false>(div_r(xx, c.scsy, rsy), div_r(yy, c.scsy, rsy), div_r(zz, c.scsy, rsy));
    const double xta = div_r(xx, c.scpr, rpr), yta = div_r(yy, c.scpr, rpr), zta = div_r(zz, c.scpr, rpr);
    const Vec3 bas = ts05_symm<true>(xta, yta, zta);
    const double cp = c_ts05.cphi, sp = c_ts05.sphi;
    const Vec3 bq = ts05_prc_quad(xta * cp - yta * sp, xta * sp + yta * cp, zta);
    const double bxq = bq.x * cp + bq.y * sp;
    const double byq = -bq.x * sp + bq.y * cp;
    const Vec3 fs = ts05_shield3(c_ts05.rc_p[0], c_ts05.rc_r[0], c_ts05.rc_sq[0], c.amp_sy, c.fac_sy, true, xx, yy, zz);
    const Vec3 fp = ts05_shield3(c_ts05.rc_p[1], c_ts05.rc_r[1], c_ts05.rc_sq[1], c.amp_pr, c.fac_pr, true, xx, yy, zz);
    const Vec3 src = {bs.x + fs.x, bs.y + fs.y, bs.z + fs.z};
    const Vec3 prc = {(bas.x + bxq) + fp.x, (bas.y + byq) + fp.y, (bas.z + bq.z) + fp.z};
    constexpr double A19 = 0.452536;
    const double bbx = 1.00000 * (cf.x * c.xappa3) + c.tamp1 * t1.x + c.tamp2 * t2.x + c.a_src * src.x +
                       c.a_prc * prc.x + c.a_r11 * r11.x + c.a_r21 * r21.x + A19 * 0.;
    const double bby = 1.00000 * (cf.y * c.xappa3) + c.tamp1 * t1.y + c.tamp2 * t2.y + c.a_src * src.y +
                       c.a_prc * prc.y + c.a_r11 * r11.y + c.a_r21 * r21.y + A19 * c.byimf;
    const double bbz = 1.00000 * (cf.z * c.xappa3) + c.tamp1 * t1.z + c.tamp2 * t2.z + c.a_src * src.z +
                       c.a_prc * prc.z + c.a_r11 * r11.z + c.a_r21 * r21.z + A19 * c.bzimf;
    if (sigma < 1.1960 - 0.005) return {bbx, bby, bbz};
    const Vec3 q = ts05_dipole(x, y, z);
    const double fint = 0.5 * (1. - div_c(sigma - 1.1960, 0.005, 1. / 0.005));
    const double fext = 0.5 * (1. + div_c(sigma - 1.1960, 0.005, 1. / 0.005));
    return {(bbx + q.x) * fint - q.x, (bby + q.y) * fint + oimfy * fext - q.y, (bbz + q.z) * fint + oimfz * fext - q.z};
}

}  // namespace cor
