// model_prep.h -- host-side derivation of the model constants the device
// field code reads: the per-condition quantities of T96 and TS05 (from
// PARMOD) and the position-independent tables of both models, computed with
// the reference's expressions and the host C library.  Host code only: the
// C ABI (cortrace.cu) fills DevParams blocks and the __constant__ tables from
// it, and the host build of the field code that the tests compare with the
// reference uses the same functions.
#pragma once

#include <math.h>
#include <string.h>

#include "field.cuh"
#include "ts05_tables.h"

namespace cor {

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

// Per-condition quantities of ts05_gsm that depend only on PARMOD
// (lib/ts05/ts05.c:19-110), and the condition-dependent shield amplitudes
// (shlcar5x5 deformed.c:196-197, birk_shl birk_tot.c:393, rc_shield
// full_rc.c:691-711), with the reference's expressions.
static void ts05_shield_amps(const double* T, double xsc, double* amp) {
    for (int m = 0; m < 9; m++) {
        const int l = 4 * m;
        amp[m] = T[l] + xsc * T[l + 1] + T[l + 2] + xsc * T[l + 3];
    }
}

static void ts05_prepare(const double* parmod, TS05Cond* c) {
    using namespace ts05h;
    const double pdyn = parmod[0];
    const double dst = parmod[1] * 0.8 - 13. * sqrt(pdyn);
    const double w1 = parmod[4], w2 = parmod[5], w3 = parmod[6], w4 = parmod[7], w5 = parmod[8], w6 = parmod[9];
    c->byimf = parmod[2];
    c->bzimf = parmod[3];
    c->xappa = pow((pdyn / 2.), A[22]);
    c->xappa3 = c->xappa * c->xappa * c->xappa;
    c->am = 34.586 / c->xappa;
    c->x0 = 3.4397 / c->xappa;
    c->oimfy_k = c->byimf * A[19];
    c->oimfz_k = c->bzimf * A[19];
    c->asq = c->am * c->am;
    c->four_asq = 4. * c->asq;
    c->two_asq = 2. * c->asq;
    c->r_two_asq = 1. / c->two_asq;
    double dstt = -20.;
    if (dst < dstt) dstt = dst;
    double znam = pow(fabs(dstt), 0.37);
    c->dx1 = A[23] - A[24] / znam;
    c->dx2 = A[25] - A[26] / znam;
    c->d = A[35] * exp(-w1 / A[36]) + A[68];
    znam = fabs(dst);
    if (dst >= -20.) znam = 20.;
    c->xk1 = A[31] * pow(znam / 20., A[32]);
    c->xk2 = A[33] * pow(znam / 20., A[34]);
    c->scsy = A[27] * pow((20. / znam), A[28]) * c->xappa;
    c->scpr = A[29] * pow((20. / znam), A[30]) * c->xappa;
    const double dlp1 = pow((pdyn / 2.), A[20]);
    const double dlp2 = pow((pdyn / 2.), A[21]);
    c->tamp1 = A[1] + A[2] * dlp1 + A[3] * (A[38] * w1) / sqrt(w1 * w1 + A[38] * A[38]);
    c->tamp2 = A[5] + A[6] * dlp2 + A[7] * (A[39] * w2) / sqrt(w2 * w2 + A[39] * A[39]);
    c->a_src = A[9] + A[10] * (A[40] * w3) / sqrt(w3 * w3 + A[40] * A[40]) + A[11] * dst;
    c->a_prc = A[12] + A[13] * (A[41] * w4) / sqrt(w4 * w4 + A[41] * A[41]) + A[14] * dst;
    c->a_r11 = A[15] + A[16] * (A[42] * w5) / sqrt(w5 * w5 + A[42] * A[42]);
    c->a_r21 = A[17] + A[18] * (A[43] * w6) / sqrt(w6 * w6 + A[43] * A[43]);
    for (int l = 0; l < 25; l++) {
        c->coef1[l] = U1[2 * l] + U1[2 * l + 1] * c->dx1;
        c->coef2[l] = U2[2 * l] + U2[2 * l + 1] * c->dx2;
    }
    ts05_shield_amps(SH11, c->xk1 - 1.1, c->amp11);
    ts05_shield_amps(SH21, c->xk2 - 1.0, c->amp21);
    const double xs_sy = c->scsy - 1., xs_pr = c->scpr - 1.;
    ts05_shield_amps(CSY, xs_sy, c->amp_sy);
    ts05_shield_amps(CPR, xs_pr, c->amp_pr);
    const double f1 = xs_sy + 1., f2 = xs_pr + 1.;
    c->fac_sy = f1 * f1 * f1;
    c->fac_pr = f2 * f2 * f2;
}

// Position-independent constants of the TS05 terms (shlcar3x3 ts05.c:137-217,
// shlcar5x5 deformed.c:178-186, birk_shl birk_tot.c:379-390, rc_shield
// full_rc.c:697-708, src_prc full_rc.c:91-92, r_s/theta_s birk_tot.c:294-308).
static void ts05_tables(TS05Tables* t) {
    using namespace ts05h;
    const double PS[3] = {9.620648151, 6.082014949, 27.75216226};
    const double R1 = 12.44199571, R2 = 5.122226936, R3 = 6.982039615;
    const double r12 = 1. / (R1 * R1), r22 = 1. / (R2 * R2), r32_1 = 1. / (R3 * R3);
    for (int i = 0; i < 3; i++) {
        const double pp = 1. / (PS[i] * PS[i]);
        t->s3_sq[3 * i] = sqrt(pp + r12);
        t->s3_sq[3 * i + 1] = sqrt(pp + r22);
        t->s3_sq[3 * i + 2] = sqrt(pp + r32_1);
        t->s3_rsq[i] = 1. / t->s3_sq[3 * i + 2];
    }
    const double* U[2] = {U1, U2};
    for (int m = 0; m < 2; m++) {
        for (int i = 0; i < 5; i++) t->s5_rp[m][i] = 1. / U[m][50 + i];
        for (int k = 0; k < 5; k++) t->s5_rr[m][k] = 1. / U[m][55 + k];
        for (int i = 0; i < 5; i++)
            for (int k = 0; k < 5; k++)
                t->s5_sq[m][5 * i + k] = sqrt(t->s5_rp[m][i] * t->s5_rp[m][i] + t->s5_rr[m][k] * t->s5_rr[m][k]);
    }
    const double* SH[2] = {SH11, SH21};
    const double* RC[2] = {CSY, CPR};
    for (int m = 0; m < 2; m++) {
        for (int j = 0; j < 3; j++) {
            t->bs_p[m][j] = SH[m][72 + j];
            t->bs_r[m][j] = SH[m][75 + j];
            t->rc_p[m][j] = RC[m][72 + j];
            t->rc_r[m][j] = RC[m][75 + j];
        }
        for (int j = 0; j < 3; j++) {
            const double pb = 1. / (t->bs_p[m][j] * t->bs_p[m][j]);
            const double pr = 1. / (t->rc_p[m][j] * t->rc_p[m][j]);
            for (int k = 0; k < 3; k++) {
                t->bs_sq[m][3 * j + k] = sqrt(pb + 1. / (t->bs_r[m][k] * t->bs_r[m][k]));
                t->rc_sq[m][3 * j + k] = sqrt(pr + 1. / (t->rc_r[m][k] * t->rc_r[m][k]));
            }
        }
    }
    t->cphi = cos(A[37]);
    t->sphi = sin(A[37]);
    const double* AC[2] = {A11, A21};
    for (int m = 0; m < 2; m++) {
        for (int k = 0; k < 20; k++) t->rs_sq[m][k] = 0.;
        for (int k = 10; k <= 15; k++) t->rs_sq[m][k] = AC[m][k] * AC[m][k];
        for (int k = 26; k <= 29; k++) t->rs_sq[m][k - 10] = AC[m][k] * AC[m][k];
    }
}

static void prepare_params(const cor_model_params* in, int32_t n, DevParams* out) {
    for (int32_t i = 0; i < n; i++) {
        memset(&out[i], 0, sizeof(DevParams));
        out[i].p = in[i];
        t96_prepare(in[i].parmod, &out[i].t96);
        ts05_prepare(in[i].parmod, &out[i].ts05);
    }
}

// The crustal model's tables, as one block: g, h, k1, k2 (packed lower
// triangles of nmax(nmax+1)/2 entries each), then kd (nmax entries).  k1, k2
// and kd are the recursion factors of lib/chaos/chaos.c:163-180, computed with
// its expressions.  `host` holds crustal_block_size(nmax) zeroed doubles.
// Returns the first degree with a non-zero coefficient (nmax if none).
static size_t crustal_block_size(int32_t nmax) {
    return 4 * ((size_t)nmax * (size_t)(nmax + 1) / 2) + (size_t)nmax;
}

static int crustal_block(const double* g, const double* h, int32_t nmax, double* host) {
    const size_t nt = (size_t)nmax * (size_t)(nmax + 1) / 2;
    double* hk1 = host + 2 * nt;
    double* hk2 = host + 3 * nt;
    double* hkd = host + 4 * nt;
    memcpy(host, g, sizeof(double) * nt);
    memcpy(host + nt, h, sizeof(double) * nt);
    int n_first = nmax;
    for (int n = 0; n < nmax && n_first == nmax; n++)
        for (int m = 0; m <= n; m++)
            if (g[n * (n + 1) / 2 + m] != 0. || h[n * (n + 1) / 2 + m] != 0.) {
                n_first = n;
                break;
            }
    for (int n = 2; n < nmax; n++) {
        const double n2 = n * 2;
        const double n21 = n2 - 1;
        const int n1 = n - 1;
        hkd[n] = sqrt(n21 / n2);
        const double nn = (double)n * n;
        for (int m = 0; m < n; m++) {
            const double mm = m * m;
            const double nnmm = nn - mm;
            hk1[n * (n + 1) / 2 + m] = n21 / sqrt(nnmm);
            hk2[n * (n + 1) / 2 + m] = sqrt((n1 * n1 - mm) / nnmm);
        }
    }
    return n_first;
}

}  // namespace cor
