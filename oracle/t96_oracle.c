/*
 * t96_oracle.c -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU restatement of the zero-tilt T96 external field as the reference
 * implements it (lib/t96/t96.c:4-1656; Tsyganenko 1996 data-based model with
 * its fitted constants).  Structure is regrouped (loops over the shielding
 * modes, one table per fitted block) but every term keeps the reference's
 * expression order, so with -ffp-contract=off and the same C library the
 * values are the reference's bit for bit.  Reference quirks kept on purpose:
 * the dipole of dipole_t96 (:1645-1656) uses sin(psi) = cos(psi) = 1 in its
 * x component; cylhar1 (:165) is unused and not restated.
 */
#include "cor_oracle.h"

#include <math.h>

/* ---- Bessel approximations, lib/t96/t96.c:211-234 --------------------- */
static double t_bes0(double x) {
    if (fabs(x) < 3.0) {
        const double x32 = (x / 3.0) * (x / 3.0);
        return 1.0 - x32 * (2.2499997 - x32 * (1.2656208 - x32 * (0.3163866 - x32 * (0.0444479 - x32 * (0.0039444 - x32 * 0.00021)))));
    }
    const double xd3 = 3.0 / x;
    const double f0 = 0.79788456 - xd3 * (0.00000077 + xd3 * (0.00552740 + xd3 * (0.00009512 - xd3 * (0.00137237 - xd3 * (0.00072805 - xd3 * 0.00014476)))));
    const double t0 = x - 0.78539816 - xd3 * (0.04166397 + xd3 * (0.00003954 - xd3 * (0.00262573 - xd3 * (0.00054125 + xd3 * (0.00029333 - xd3 * 0.00013558)))));
    return f0 / sqrt(x) * cos(t0);
}

static double t_bes1(double x) {
    if (fabs(x) < 3.0) {
        const double x32 = (x / 3.0) * (x / 3.0);
        const double b = 0.5 - x32 * (0.56249985 - x32 * (0.21093573 - x32 * (0.03954289 - x32 * (0.00443319 - x32 * (0.00031761 - x32 * 0.00001109)))));
        return b * x;
    }
    const double xd3 = 3.0 / x;
    const double f1 = 0.79788456 + xd3 * (0.00000156 + xd3 * (0.01659667 + xd3 * (0.00017105 - xd3 * (0.00249511 - xd3 * (0.00113653 - xd3 * 0.00020033)))));
    const double t1 = x - 2.35619449 + xd3 * (0.12499612 + xd3 * (0.0000565 - xd3 * (0.00637879 - xd3 * (0.00074348 + xd3 * (0.00079824 - xd3 * 0.00029166)))));
    return f1 / sqrt(x) * cos(t1);
}

/* ---- Chapman-Ferraro field, cylindrical harmonics (:113-163) ---------- */
static void t_cylharm(double x, double y, double z, double b[3]) {
    static const double A[12] = { 0.24777, -27.003, -0.46815, 7.0637, -1.5918, -0.90317E-01,
                                  57.522, 13.757, 2.0100, 10.458, 4.5798, 2.1695 };
    double rho = sqrt(y * y + z * z), sf, cf;
    if (rho < 1.0e-8) { sf = 1.0; cf = 0.0; rho = 1.0e-8; }
    else { sf = z / rho; cf = y / rho; }
    const double sf2 = sf * sf;
    const double s2c2 = sf2 - cf * cf;
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 3; ++i) {
        const double dz = rho / A[i + 6];
        const double j0 = t_bes0(dz), j1 = t_bes1(dz);
        const double e = exp(x / A[i + 6]);
        bx -= A[i] * j1 * e * sf;
        by += A[i] * (2.0 * j1 / dz - j0) * e * sf * cf;
        bz += A[i] * (j1 / dz * s2c2 - j0 * sf2) * e;
    }
    for (int i = 3; i < 6; ++i) {
        const double dz = rho / A[i + 6];
        const double xk = x / A[i + 6];
        const double j0 = t_bes0(dz), j1 = t_bes1(dz);
        const double e = exp(xk);
        const double brho = (xk * j0 - (dz * dz + xk - 1.0) * j1 / dz) * e * sf;
        const double bphi = (j0 + j1 / dz * (xk - 1.0)) * e * cf;
        bx += A[i] * (dz * j0 + xk * j1) * e * sf;
        by += A[i] * (brho * cf - bphi * sf);
        bz += A[i] * (brho * sf + bphi * cf);
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* ---- IMF interconnection field (:236-271) ----------------------------- */
static void t_intercon(double x, double y, double z, double b[3]) {
    static const double A[9] = { -8.411078731, 5932254.951, -9073284.93, -11.68794634, 6027598.824,
                                 -9218378.368, -6.508798398, -11824.42793, 18015.66212 };
    static const double RP[3] = { 0.12503844191332988, 0.071597395204476152, 0.011080976889832743 };
    static const double RR[3] = { 0.059675527522452816, 0.00098459526668325296, 0.00064371058922777988 };
    double bx = 0.0, by = 0.0, bz = 0.0;
    int l = 0;
    for (int i = 0; i < 3; i++) {
        const double cy = cos(y * RP[i]), sy = sin(y * RP[i]);
        for (int k = 0; k < 3; k++) {
            const double sz = sin(z * RR[k]), cz = cos(z * RR[k]);
            const double sq = sqrt(RP[i] * RP[i] + RR[k] * RR[k]);
            const double e = exp(x * sq);
            bx += A[l] * (-sq * e * cy * sz);
            by += A[l] * (RP[i] * e * sy * sz);
            bz += A[l] * (-RR[k] * e * cy * cz);
            l++;
        }
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* ---- 3x3 Cartesian shielding harmonics (:500-617) --------------------- */
/* a[0..17] amplitudes as 9 summed pairs, a[18..20] P scales, a[21..23] R scales */
static void t_shlcar3x3(const double *a, double x, double y, double z, double h[3]) {
    double hx = 0.0, hy = 0.0, hz = 0.0;
    for (int i = 0; i < 3; i++) {
        const double p = a[18 + i];
        const double pp = 1.0 / (p * p);
        const double yp = y / p;
        const double sy = sin(yp), cy = cos(yp);
        for (int k = 0; k < 3; k++) {
            const double r = a[21 + k];
            const double zr = z / r;
            const double sz = sin(zr), cz = cos(zr);
            const double sq = sqrt(pp + 1.0 / (r * r));
            const double e = exp(x * sq);
            const double amp = a[2 * (3 * i + k)] + a[2 * (3 * i + k) + 1];
            hx += (-sq * e * cy * sz) * amp;
            hy += (e / p * sy * sz) * amp;
            hz += (-e / r * cy * cz) * amp;
        }
    }
    h[0] = hx; h[1] = hy; h[2] = hz;
}

/* ---- ring current (:323-381) ------------------------------------------ */
static void t_ringcurr(double x, double y, double z, double b[3]) {
    static const double F[2] = { 569.895366, -1603.386993 };
    static const double BETA[2] = { 2.722188, 3.766875 };
    const double dzs = sqrt(z * z + 4.0);
    const double rhos = sqrt(x * x + y * y);
    const double ddz = z / dzs;
    double drx = 0.0, dry = (y >= 0) ? 1.0 : -1.0;
    if (rhos >= 1.0e-5) { drx = x / rhos; dry = y / rhos; }
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 2; ++i) {
        const double bi = BETA[i];
        const double dzb = dzs + bi, rp = rhos + bi, rm = rhos - bi;
        const double dzb2 = dzb * dzb;
        const double bi2 = 2.0 * bi;
        const double s1 = sqrt(dzb2 + rp * rp), s2 = sqrt(dzb2 + rm * rm);
        const double ds1dz = dzb / s1, ds2dz = dzb / s2;
        const double ds1dr = rp / s1, ds2dr = rm / s2;
        const double s12 = s1 * s2, sp = s1 + s2, sp2 = sp * sp;
        const double fac1 = sqrt(sp2 - bi2 * bi2);
        const double as = fac1 / (s12 * sp2);
        const double term1 = 1.0 / (s12 * sp * fac1);
        const double fac2 = as / sp2;
        const double das1 = term1 - fac2 / s1 * (s2 * s2 + s1 * (3.0 * s1 + 4.0 * s2));
        const double das2 = term1 - fac2 / s2 * (s1 * s1 + s2 * (3.0 * s2 + 4.0 * s1));
        const double dasdx = das1 * (ds1dr * drx) + das2 * (ds2dr * drx);
        const double dasdy = das1 * (ds1dr * dry) + das2 * (ds2dr * dry);
        const double dasdz = das1 * (ds1dz * ddz) + das2 * (ds2dz * ddz);
        bx += -F[i] * x * dasdz;
        by -= F[i] * y * dasdz;
        bz += F[i] * ((2.0 * as + y * dasdy) + x * dasdx);
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* ---- tail disk (:383-443) --------------------------------------------- */
static void t_taildisk(double x, double y, double z, double b[3]) {
    static const double F[4] = { -745796.7338, 1176470.141, -444610.529, -57508.01028 };
    static const double BETA[4] = { 7.9250000, 8.0850000, 8.4712500, 27.89500 };
    const double y20 = y / 20.0;
    const double d = 2.0 + 10.0 * (y20 * y20);
    const double dzs = sqrt(z * z + d * d);
    const double ddy = (d * 10.0 * y * 0.005) / dzs;
    const double ddz = z / dzs;
    const double xs = x - 4.5;
    const double rhos = sqrt(xs * xs + y * y);
    double drx = 0.0, dry = (y >= 0) ? 1.0 : -1.0;
    if (rhos >= 1.0e-5) { drx = xs / rhos; dry = y / rhos; }
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 4; ++i) {
        const double bi = BETA[i];
        const double bi1 = 2.0 * bi;
        const double dzb = dzs + bi, rp = rhos + bi, rm = rhos - bi;
        const double s1 = sqrt(dzb * dzb + rp * rp), s2 = sqrt(dzb * dzb + rm * rm);
        const double ds1dz = dzb / s1, ds2dz = dzb / s2;
        const double ds1dr = rp / s1, ds2dr = rm / s2;
        const double s12 = s1 * s2, sp = s1 + s2, sp2 = sp * sp;
        const double fac1 = sqrt(sp2 - bi1 * bi1);
        const double as = fac1 / (s12 * sp2);
        const double term1 = 1.0 / (s12 * sp * fac1);
        const double fac2 = as / sp2;
        const double das1 = term1 - fac2 / s1 * (s2 * s2 + s1 * (3.0 * s1 + 4.0 * s2));
        const double das2 = term1 - fac2 / s2 * (s1 * s1 + s2 * (3.0 * s2 + 4.0 * s1));
        const double dasdx = das1 * (ds1dr * drx) + das2 * (ds2dr * drx);
        const double dasdy = das1 * (ds1dz * ddy + ds1dr * dry) + das2 * (ds2dz * ddy + ds2dr * dry);
        const double dasdz = das1 * (ds1dz * ddz) + das2 * (ds2dz * ddz);
        bx += F[i] * ((4.5 - x) * dasdz);
        by -= F[i] * y * dasdz;
        bz += F[i] * ((2.0 * as + y * dasdy) + xs * dasdx);
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* ---- T87-type tail sheet (:445-498), three mirrored wires per line ---- */
static void t_tail87(double x, double z, double *bxo, double *bzo) {
    const double zp = z - 40.0, zm = z + 40.0;
    const double xnx = -10.0 - x;
    const double xnx2 = xnx * xnx;
    const double xc1 = x + 1.261, xc2 = x + 0.663;
    const double xc22 = xc2 * xc2;
    const double xr2 = xc2 * -0.1071;
    const double xc12 = xc1 * xc1;
    const double d2 = 3.0 * 3.0;
    const double b20 = z * z + d2, b2p = zp * zp + d2, b2m = zm * zm + d2;
    const double b = sqrt(b20), bp = sqrt(b2p), bm = sqrt(b2m);
    const double xa1 = xc12 + b20, xap1 = xc12 + b2p, xam1 = xc12 + b2m;
    const double xa2 = 1. / (xc22 + b20), xap2 = 1. / (xc22 + b2p), xam2 = 1. / (xc22 + b2m);
    const double xna = xnx2 + b20, xnap = xnx2 + b2p, xnam = xnx2 + b2m;
    const double f = b20 - xc22, fp = b2p - xc22, fm = b2m - xc22;
    const double xln1 = log(76.37 / xna), xlnp1 = log(76.37 / xnap), xlnm1 = log(76.37 / xnam);
    const double xln2 = xln1 + 0.13238005, xlnp2 = xlnp1 + 0.13238005, xlnm2 = xlnm1 + 0.13238005;
    const double aln = 0.25 * (xlnp1 + xlnm1 - 2. * xln1);
    const double s0 = (atan(xnx / b) + 1.5707963) / b;
    const double s0p = (atan(xnx / bp) + 1.5707963) / bp;
    const double s0m = (atan(xnx / bm) + 1.5707963) / bm;
    const double s1 = (xln1 * .5 + xc1 * s0) / xa1;
    const double s1p = (xlnp1 * .5 + xc1 * s0p) / xap1;
    const double s1m = (xlnm1 * .5 + xc1 * s0m) / xam1;
    const double s2 = (xc2 * xa2 * xln2 + 0.1071 - f * xa2 * s0) * xa2;
    const double s2p = (xc2 * xap2 * xlnp2 + 0.1071 - fp * xap2 * s0p) * xap2;
    const double s2m = (xc2 * xam2 * xlnm2 + 0.1071 - fm * xam2 * s0m) * xam2;
    const double g1 = (b20 * s0 - 0.5 * xc1 * xln1) / xa1;
    const double g1p = (b2p * s0p - 0.5 * xc1 * xlnp1) / xap1;
    const double g1m = (b2m * s0m - 0.5 * xc1 * xlnm1) / xam1;
    const double g2 = ((0.5 * f * xln2 + 2. * s0 * b20 * xc2) * xa2 + xr2) * xa2;
    const double g2p = ((0.5 * fp * xlnp2 + 2. * s0p * b2p * xc2) * xap2 + xr2) * xap2;
    const double g2m = ((0.5 * fm * xlnm2 + 2. * s0m * b2m * xc2) * xam2 + xr2) * xam2;
    *bxo = 0.391734 * (z * s0 - 0.5 * (zp * s0p + zm * s0m)) + 5.89715 * (z * s1 - 0.5 * (zp * s1p + zm * s1m)) +
           24.6833 * (z * s2 - 0.5 * (zp * s2p + zm * s2m));
    *bzo = 0.391734 * aln + 5.89715 * (g1 - 0.5 * (g1p + g1m)) + 24.6833 * (g2 - 0.5 * (g2p + g2m));
}

/* ---- ring current + tail modes with their shields (:273-321) ---------- */
static void t_tailrc(double x, double y, double z, double rc[3], double t2[3], double t3[3]) {
    static const double ARC[24] = {
        -3.087699646, 3.516259114, 18.81380577, -13.95772338, -5.497076303, 0.1712890838, 2.392629189,
        -2.728020808, -14.79349936, 11.08738083, 4.388174084, 0.2492163197E-01, 0.7030375685, -.7966023165,
        -3.835041334, 2.642228681, -0.2405352424, -0.7297705678, 12.75434981, 11.37659788, 636.4346279,
        1.752483754, 3.604231143, 12.83078674 };
    static const double AT2[24] = {
        0.8747515218, -0.9116821411, 2.209365387, -2.159059518, -7.059828867, 5.924671028, -1.916935691,
        1.996707344, -3.877101873, 3.947666061, 11.38715899, -8.343210833, 1.194109867, -1.244316975,
        3.73895491, -4.406522465, -20.66884863, 3.020952989, 5.187666221, 6.802472048, 39.13543412,
        2.784722096, 6.979576616, 25.71716760 };
    static const double AT3[24] = {
        -19091.95061, -3011.613928, 20582.16203, 4242.918430, -2377.091102, -1504.820043, 19884.04650,
        2725.150544, -21389.04845, -3990.475093, 2401.610097, 1548.171792, -946.5493963, 490.1528941,
        986.9156625, -489.3265930, -67.99278499, 8.711175710, 19.69877970, 20.30095680, 86.45407420,
        22.50403727, 23.41617329, 48.48140573 };
    double h[3], w[3];
    t_ringcurr(x, y, z, h);
    t_shlcar3x3(ARC, x, y, z, w);
    rc[0] = w[0] + h[0]; rc[1] = w[1] + h[1]; rc[2] = w[2] + h[2];
    t_shlcar3x3(AT2, x, y, z, w);
    t_taildisk(x, y, z, h);
    t2[0] = w[0] + h[0]; t2[1] = w[1] + h[1]; t2[2] = w[2] + h[2];
    t_shlcar3x3(AT3, x, y, z, w);
    double hx, hz;
    t_tail87(x, z, &hx, &hz);
    t3[0] = w[0] + hx; t3[1] = w[1]; t3[2] = w[2] + hz;
}

/* ---- current loops (:857-907) ----------------------------------------- */
static void t_circle(double x, double y, double z, double rl, double b[3]) {
    const double rho2 = x * x + y * y;
    const double rho = sqrt(rho2);
    const double rr = rho + rl;
    const double r22 = z * z + rr * rr;
    const double r2 = sqrt(r22);
    const double r12 = r22 - 4.0 * rho * rl;
    const double r32 = 0.5 * (r12 + r22);
    const double xk2 = 1.0 - r12 / r22;
    const double xk2s = 1.0 - xk2;
    const double dl = log(1.0 / xk2s);
    const double K = 1.38629436112 + xk2s * (0.09666344259 + xk2s * (0.03590092383 + xk2s * (0.03742563713 + xk2s * 0.01451196212))) +
                     dl * (0.5 + xk2s * (0.12498593597 + xk2s * (0.06880248576 + xk2s * (0.03328355346 + xk2s * 0.00441787012))));
    const double E = 1.0 + xk2s * (0.44325141463 + xk2s * (0.0626060122 + xk2s * (0.04757383546 + xk2s * 0.01736506451))) +
                     dl * xk2s * (0.2499836831 + xk2s * (0.09200180037 + xk2s * (0.04069697526 + xk2s * 0.00526449639)));
    double brho;
    if (rho > 1e-6) brho = z / (rho2 * r2) * (r32 / r12 * E - K);
    else brho = 3.141592654 * rl / r2 * (rl - rho) / r12 * z / (r32 - rho2);
    b[0] = brho * x;
    b[1] = brho * y;
    b[2] = (K - E * (r32 - 2.0 * rl * rl) / r12) / r2;
}

static void t_crosslp(double x, double y, double z, double b[3], double xc, double rl, double al) {
    const double cal = (cos)(al), sal = (sin)(al);
    const double y1 = y * cal - z * sal, z1 = y * sal + z * cal;
    const double y2 = y * cal + z * sal, z2 = -y * sal + z * cal;
    double b1[3], b2[3];
    t_circle(x - xc, y1, z1, rl, b1);
    t_circle(x - xc, y2, z2, rl, b2);
    b[0] = b1[0] + b2[0];
    b[1] = (b1[1] + b2[1]) * cal + (b1[2] - b2[2]) * sal;
    b[2] = -(b1[1] - b2[1]) * sal + (b1[2] + b2[2]) * cal;
}

/* dipole field gradient terms (:909-928): out[0..2] = x-dipole, [3..5] y, [6..8] z */
static void t_dipxyz(double x, double y, double z, double o[9]) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    const double xmr5 = 30574.0 / (r2 * r2 * sqrt(r2));
    const double xmr53 = 3.0 * xmr5;
    o[0] = xmr5 * (3.0 * x2 - r2);
    o[1] = xmr53 * x * y;
    o[2] = xmr53 * x * z;
    o[3] = o[1];
    o[4] = xmr5 * (3.0 * y2 - r2);
    o[5] = xmr53 * y * z;
    o[6] = o[2];
    o[7] = o[5];
    o[8] = xmr5 * (3.0 * z2 - r2);
}

/* ---- Region-1 basis: dipole loops near noon (:809-855) ---------------- */
static void t_diploop1(double x, double y, double z, double D[3][14]) {
    static const double XX[12] = { -11.0, -7.0, -7.0, -3.0, -3.0, 1.0, 1.0, 1.0, 5.0, 5.0, 9.0, 9.0 };
    static const double YY[12] = { 2.0, 0.0, 4.0, 2.0, 6.0, 0.0, 4.0, 8.0, 2.0, 6.0, 0.0, 4.0 };
    const double z2 = z * z;
    for (int i = 0; i < 12; i++) {
        const double dy = YY[i] * 0.945719;
        const double dx = XX[i] * 1.12541;
        const double xd = x - dx;
        double yd = y - dy;
        double r2 = xd * xd + yd * yd + z2;
        double xmr5 = 30574.0 / (r2 * r2 * sqrt(r2));
        double xmr53 = 3.0 * xmr5;
        const double b1x = xmr53 * xd * z, b1y = xmr53 * yd * z, b1z = xmr5 * (3.0 * z2 - r2);
        double b2x = 0.0, b2y = 0.0, b2z = 0.0;
        if (fabs(dy) > 1.0e-10) {
            yd = y + dy;
            r2 = xd * xd + yd * yd + z2;
            xmr5 = 30574.0 / (r2 * r2 * sqrt(r2));
            xmr53 = 3.0 * xmr5;
            b2x = xmr53 * xd * z;
            b2y = xmr53 * yd * z;
            b2z = xmr5 * (3.0 * z2 - r2);
        }
        D[0][i] = b1x + b2x;
        D[1][i] = b1y + b2y;
        D[2][i] = b1z + b2z;
    }
    double b[3];
    t_crosslp(x, y, z, b, 2.28397, 1.86106, 1.00891);
    D[0][12] = b[0]; D[1][12] = b[1]; D[2][12] = b[2];
    t_circle(x + 5.60831, y, z, 7.83281, b);
    D[0][13] = b[0]; D[1][13] = b[1]; D[2][13] = b[2];
}

/* ---- Region-1 basis: conical harmonics and dipole pairs (:930-1028) ---- */
static void t_condip1(double x, double y, double z, double D[3][42]) {
    static const double XX[14] = { -10.0, -7.0, -4.0, -4.0, 0.0, 4.0, 4.0, 7.0, 10.0, 0.0, 0.0, 0.0, 0.0, 0.0 };
    static const double YY[14] = { 3.0, 6.0, 3.0, 9.0, 6.0, 3.0, 9.0, 6.0, 3.0, 0.0, 0.0, 0.0, 0.0, 0.0 };
    static const double ZZ[14] = { 20.0, 20.0, 4.0, 20.0, 4.0, 4.0, 20.0, 20.0, 20.0, 2.0, 3.0, 4.50, 7.0, 10.0 };
    const double xsm = x + 0.16;
    const double ro2 = xsm * xsm + y * y;
    const double ro = sqrt(ro2);
    double cf[5], sf[5];
    cf[0] = xsm / ro;
    sf[0] = y / ro;
    cf[1] = cf[0] * cf[0] - sf[0] * sf[0];
    sf[1] = 2.0 * sf[0] * cf[0];
    for (int m = 2; m < 5; m++) {
        cf[m] = cf[m - 1] * cf[0] - sf[m - 1] * sf[0];
        sf[m] = sf[m - 1] * cf[0] + cf[m - 1] * sf[0];
    }
    const double r2 = ro2 + z * z;
    const double r = sqrt(r2);
    const double c = z / r, s = ro / r;
    const double ch = sqrt(0.5 * (1.0 + c)), sh = sqrt(0.5 * (1.0 - c));
    const double tnh = sh / ch, cnh = 1.0 / tnh;
    for (int m = 0; m < 5; m++) {
        const double mn = m + 1;
        const double bt = mn * cf[m] / (r * s) * (pow(tnh, mn) + pow(cnh, mn));
        const double bf = -0.5 * mn * sf[m] / r * (pow(tnh, m) / (ch * ch) - pow(cnh, m) / (sh * sh));
        D[0][m] = bt * c * cf[0] - bf * sf[0];
        D[1][m] = bt * c * sf[0] + bf * cf[0];
        D[2][m] = -bt * s;
    }
    for (int i = 0; i < 9; i++) {
        double xd, yd;
        if (i == 2 || i == 4 || i == 5) { xd = XX[i] * 0.08; yd = YY[i] * 0.08; }
        else { xd = XX[i] * 0.4; yd = YY[i] * 0.4; }
        const double zd = ZZ[i];
        double b1[9], b2[9], b3[9], b4[9];
        t_dipxyz(x - xd, y - yd, z - zd, b1);
        t_dipxyz(x - xd, y + yd, z - zd, b2);
        t_dipxyz(x - xd, y - yd, z + zd, b3);
        t_dipxyz(x - xd, y + yd, z + zd, b4);
        const int ix = (i + 1) * 3 + 2, iy = ix + 1, iz = iy + 1;
        for (int c3 = 0; c3 < 3; c3++) {
            D[c3][ix] = b1[c3] + b2[c3] - b3[c3] - b4[c3];
            D[c3][iy] = b1[3 + c3] - b2[3 + c3] - b3[3 + c3] + b4[3 + c3];
            D[c3][iz] = b1[6 + c3] + b2[6 + c3] + b3[6 + c3] + b4[6 + c3];
        }
    }
    for (int i = 1; i <= 5; i++) {
        const double zd = ZZ[i + 8];
        double b1[9], b2[9];
        t_dipxyz(x, y, z - zd, b1);
        t_dipxyz(x, y, z + zd, b2);
        const int ix = 30 + i * 2, iz = ix + 1;
        for (int c3 = 0; c3 < 3; c3++) {
            D[c3][ix] = b1[c3] - b2[c3];
            D[c3][iz] = b1[6 + c3] + b2[6 + c3];
        }
    }
}

/* ---- Region-1 shield (:1030-1194): 4 P x 4 R modes -------------------- */
static void t_birk1shld(double x, double y, double z, double b[3]) {
    static const double PS[4] = { 5.303648988, 10.40368955, 69.65230348, 466.5099509 };
    static const double RS[4] = { 1.645049286, 3.825838190, 11.66675599, 558.9781177 };
    /* the 16 amplitudes, each the sum of the reference's two fitted halves */
    static const double A1[16] = { 1.174198045, 4.840161537, 82.18368896, -4122.331796,
                                   -21.54975037, -72.81365728, 40.08073706, 1955.348537,
                                   794.0496433, 1889.837171, -1260.543238, -293.5942373,
                                   -773.7002492, -1824.143669, 1192.484774, 89.15537624 };
    static const double A2[16] = { -1.463820502, -3.674506864, -94.94071588, 4670.278676,
                                   26.72661293, 44.09887902, -51.23563510, -1940.971550,
                                   -982.2441344, -558.9779727, 1260.063802, 344.7250789,
                                   957.0094135, 520.7994379, -1192.184565, -98.52042999 };
    double rk[4], rk2[4], szk[4], czk[4];
    for (int k = 0; k < 4; k++) {
        rk[k] = 1.0 / RS[k];
        const double zr = z * rk[k];
        szk[k] = sin(zr);
        czk[k] = cos(zr);
        rk2[k] = rk[k] * rk[k];
    }
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 4; i++) {
        const double rpi = 1.0 / PS[i];
        const double rpi2 = rpi * rpi;
        const double ry = rpi * y;
        const double sy = sin(ry), cy = cos(ry);
        for (int k = 0; k < 4; k++) {
            const double sq = sqrt(rpi2 + rk2[k]);
            const double e = exp(x * sq);
            const double aa = A1[4 * i + k] + A2[4 * i + k];
            bx += (-sq * e * cy * szk[k]) * aa;
            by += (rpi * e * sy * szk[k]) * aa;
            bz += (-rk[k] * e * cy * czk[k]) * aa;
        }
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* ---- Region-1 total (:619-807) ---------------------------------------- */
static void t_sum_d1(const double D[3][14], double b[3]) {
    static const double C1[14] = { -0.911582E-03, -0.376654E-02, -0.727423E-02, -0.270084E-02, -0.123899E-02,
                                   -0.154387E-02, -0.340040E-02, -0.191858E-01, -0.518979E-01, 0.635061E-01,
                                   0.440680, -0.396570, -89.5587, 23.2806 };
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 14; i++) { bx += C1[i] * D[0][i]; by += C1[i] * D[1][i]; bz += C1[i] * D[2][i]; }
    b[0] = bx; b[1] = by; b[2] = bz;
}

static void t_sum_d2(const double D[3][42], double b[3]) {
    static const double C2[42] = {
        6.04133, 0.305415, 0.606066E-02, 0.128379E-03, -0.179406E-04, 1.41714, -27.2586, -4.28833, -1.30675,
        35.5607, 8.95792, 0.961617E-03, -0.801477E-03, -0.782795E-03, -1.65242, -16.5242, -5.33798,
        0.424878E-03, 0.331787E-03, -0.704305E-03, 0.844342E-03, 0.953682E-04, 0.886271E-03, 25.1120,
        20.9299, 5.14569, -44.1670, -51.0672, -1.87725, 20.2998, 48.7505, -2.97415, 0.174615E-03,
        -0.789777E-06, 0.686047E-03, 0.460104E-04, -0.345216E-02, 0.221871E-02, 0.110078E-01,
        -0.661373E-02, 0.249201E-02, 0.343978E-01 };
    double bx = 0.0, by = 0.0, bz = 0.0;
    for (int i = 0; i < 42; i++) { bx += C2[i] * D[0][i]; by += C2[i] * D[1][i]; bz += C2[i] * D[2][i]; }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* Field of the blend zone between the two Region-1 bases at tet0 near
 * t1..t2; south selects the sign of the cosines and which basis is first. */
static void t_birk1_blend(double x, double y, double z, double r, double r3, double pas, double t1, double t2,
                          int south, double b[3]) {
    const double sqr = sqrt(r);
    const double s1 = sin(t1);
    const double st01 = sqr / pow(r3 + 1.0 / (s1 * s1 * s1 * s1 * s1 * s1) - 1.0, 0.1666666667);
    const double s2 = sin(t2);
    const double st02 = sqr / pow(r3 + 1.0 / (s2 * s2 * s2 * s2 * s2 * s2) - 1.0, 0.1666666667);
    double ct01 = sqrt(1.0 - st01 * st01), ct02 = sqrt(1.0 - st02 * st02);
    if (south) { ct01 = -ct01; ct02 = -ct02; }
    const double x1 = r * st01 * cos(pas), y1 = r * st01 * sin(pas), z1 = r * ct01;
    double b1[3], b2[3];
    if (!south) {
        double D1[3][14];
        t_diploop1(x1, y1, z1, D1);
        t_sum_d1(D1, b1);
    } else {
        double D2[3][42];
        t_condip1(x1, y1, z1, D2);
        t_sum_d2(D2, b1);
    }
    const double x2 = r * st02 * cos(pas), y2 = r * st02 * sin(pas), z2 = r * ct02;
    if (!south) {
        double D2[3][42];
        t_condip1(x2, y2, z2, D2);
        t_sum_d2(D2, b2);
    } else {
        double D1[3][14];
        t_diploop1(x2, y2, z2, D1);
        t_sum_d1(D1, b2);
    }
    const double dx2 = x2 - x1, dy2 = y2 - y1, dz2 = z2 - z1;
    const double ss = sqrt(dx2 * dx2 + dy2 * dy2 + dz2 * dz2);
    const double dx = x - x1, dy = y - y1, dz = z - z1;
    const double ds = sqrt(dx * dx + dy * dy + dz * dz);
    const double frac = ds / ss;
    for (int c = 0; c < 3; c++) b[c] = b1[c] * (1.0 - frac) + b2[c] * frac;
}

static void t_birk1tot(double x, double y, double z, double b[3]) {
    const double tnoonn = 12.0 * 0.01745329;
    const double tnoons = 3.141592654 - tnoonn;
    const double r2 = x * x + y * y + z * z;
    const double r = sqrt(r2);
    const double r3 = r * r2;
    double pas = 0.0;
    if (x != 0.0 || y != 0.0) pas = atan2(y, x);
    const double tas = atan2(sqrt(x * x + y * y), z);
    const double stas = sin(tas);
    double tet0 = asin(stas / pow((stas * stas * stas * stas * stas * stas) * (1.0 - r3) + r3, 0.1666666667));
    if (tas > 1.5707963) tet0 = 3.141592654 - tet0;
    const double dtet = (8.0 * 0.01745329) * (sin(pas * 0.5) * sin(pas * 0.5));
    const double tr1n = tnoonn + dtet, tr1s = tnoons - dtet;
    const double t01n = tr1n - 0.034906, t01s = tr1s - 0.034906;
    const double t02s = tr1s + 0.034906, t02n = tr1n + 0.034906;
    double bx = 0.0, by = 0.0, bz = 0.0, t[3];
    if (tet0 < t01n || tet0 > t02s) {
        double D1[3][14];
        t_diploop1(x, y, z, D1);
        t_sum_d1(D1, t);
        bx += t[0]; by += t[1]; bz += t[2];
    }
    if (tet0 > t02n && tet0 < t01s) {
        double D2[3][42];
        t_condip1(x, y, z, D2);
        t_sum_d2(D2, t);
        bx += t[0]; by += t[1]; bz += t[2];
    }
    if (tet0 >= t01n && tet0 <= t02n) {
        t_birk1_blend(x, y, z, r, r3, pas, t01n, t02n, 0, t);
        bx = t[0]; by = t[1]; bz = t[2];
    }
    if (tet0 >= t01s && tet0 <= t02s) {
        t_birk1_blend(x, y, z, r, r3, pas, t01s, t02s, 1, t);
        bx = t[0]; by = t[1]; bz = t[2];
    }
    double bs[3];
    t_birk1shld(x, y, z, bs);
    b[0] = bx + bs[0]; b[1] = by + bs[1]; b[2] = bz + bs[2];
}

/* ---- Region-2 shield (:1196-1263): 2 P x 2 R modes -------------------- */
static void t_birk2shl(double x, double y, double z, double h[3]) {
    static const double PI_[2] = { 13.85650567, 14.90554500 };
    static const double RK[2] = { 10.21914434, 10.09021632 };
    static const double A1[4] = { -111.6371348, 110.3735178, 111.9448247, -110.7586562 };
    static const double A2[4] = { 124.5402702, -122.0095905, -129.1957743, 126.5649012 };
    double hx = 0.0, hy = 0.0, hz = 0.0;
    for (int i = 0; i < 2; i++) {
        const double ai = PI_[i];
        const double ya = y / ai;
        const double cy = cos(ya);
        double aiai = 0.0;
        for (int k = 0; k < 2; k++) {
            const double ak = RK[k];
            const double za = z / ak;
            const double sz = sin(za), cz = cos(za);
            const double sy = sin(ya);
            if (k == 0) aiai = 1.0 / (ai * ai);
            const double sq = sqrt(aiai + 1.0 / (ak * ak));
            const double e = exp(x * sq);
            const double as = A1[2 * i + k] + A2[2 * i + k];
            hx += (-sq * e * cy * sz) * as;
            hy += (e / ai * sy * sz) * as;
            hz += (-e / ak * cy * cz) * as;
        }
    }
    h[0] = hx; h[1] = hy; h[2] = hz;
}

/* ---- Region-2 pieces (:1265-1643) ------------------------------------- */
static double t_xksi(double x, double y, double z) {
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double r2 = x2 + y2 + z2;
    const double r = sqrt(r2);
    const double xr = x / r, yr = y / r, zr = z / r;
    const double dr = 7.50937;
    const double dr2 = dr * dr;
    const double r0 = 1.21563;
    double pr = 0.0;
    if (r >= r0) pr = sqrt((r - r0) * (r - r0) + dr2) - dr;
    const double f = x + pr * (0.305662 + -0.383593 * xr + 0.2677733 * xr * xr + -0.097656 * yr * yr + -0.636034 * zr * zr);
    const double g = y + pr * (-0.359862 * yr + 0.424706 * xr * yr);
    const double h = z + pr * (-0.126366 * zr + 0.292578 * xr * zr);
    const double g2 = g * g;
    const double fgh = f * f + g2 + h * h;
    const double sq = sqrt(fgh);
    const double fgh32 = sq * sq * sq;
    const double fg2 = (f * f) + g2;
    if (fg2 < 1.0e-5) return -1.0;
    const double th = sin(0.3665191 + 0.5 * 0.09599309 * (1.0 - f / sqrt(fg2)));
    return (fg2 / fgh32) - (th * th);
}

static double t_tksi(double xk, double x0, double dx) {
    const double tdz3 = 2.0 * dx * dx * dx;
    if (xk - x0 < -dx) return 0.0;
    if (xk - x0 >= dx) return 1.0;
    if (xk >= x0 - dx && xk < x0) {
        const double d = xk - x0 + dx;
        const double br3 = d * d * d;
        return 1.5 * br3 / (tdz3 + br3);
    }
    const double d = xk - x0 - dx;
    const double br3 = d * d * d;
    return 1.0 + 1.5 * br3 / (tdz3 - br3);
}

static void t_bconic(double x, double y, double z, double cbx[5], double cby[5], double cbz[5]) {
    const double ro2 = x * x + y * y;
    const double ro = sqrt(ro2);
    const double cf = x / ro, sf = y / ro;
    const double r2 = ro2 + z * z;
    const double r = sqrt(r2);
    const double c = z / r, s = ro / r;
    const double ch = sqrt(0.5 * (1.0 + c)), sh = sqrt(0.5 * (1.0 - c));
    double tnhm1 = 1.0, cnhm1 = 1.0;
    const double tnh = sh / ch, cnh = 1.0 / tnh;
    double cfm1 = 1.0, sfm1 = 0.0;
    for (int m = 0; m < 5; m++) {
        const double cfm = cfm1 * cf - sfm1 * sf;
        const double sfm = cfm1 * sf + sfm1 * cf;
        cfm1 = cfm; sfm1 = sfm;
        const double tnhm = tnhm1 * tnh, cnhm = cnhm1 * cnh;
        const double bt = (m + 1) * cfm / (r * s) * (tnhm + cnhm);
        const double bf = -0.5 * (m + 1) * sfm / r * (tnhm1 / (ch * ch) - cnhm1 / (sh * sh));
        tnhm1 = tnhm; cnhm1 = cnhm;
        cbx[m] = bt * c * cf - bf * sf;
        cby[m] = bt * c * sf + bf * cf;
        cbz[m] = -bt * s;
    }
}

static void t_dipdistr(double x, double y, double z, double b[3], int mode) {
    const double x2 = x * x;
    const double rho2 = x2 + y * y;
    if (mode == 0) {
        const double r2 = rho2 + z * z;
        const double r3 = r2 * sqrt(r2);
        b[0] = z / (rho2 * rho2) * (r2 * (y * y - x2) - rho2 * x2) / r3;
        b[1] = -x * y * z / (rho2 * rho2) * (2.0 * r2 + rho2) / r3;
        b[2] = x / r3;
        return;
    }
    b[0] = z / (rho2 * rho2) * (y * y - x2);
    b[1] = -2.0 * x * y * z / (rho2 * rho2);
    b[2] = x / rho2;
}

static void t_loops4(double x, double y, double z, double b[3], double xc, double yc, double zc, double R,
                     double theta, double phi) {
    const double st = (sin)(theta), ct = (cos)(theta), sp = (sin)(phi), cp = (cos)(phi);
    double xs, yss, zs, xss, zss, bxs, q[3];
    xs = (x - xc) * cp + (y - yc) * sp;
    yss = (y - yc) * cp - (x - xc) * sp;
    zs = z - zc;
    xss = xs * ct - zs * st;
    zss = zs * ct + xs * st;
    t_circle(xss, yss, zss, R, q);
    bxs = q[0] * ct + q[2] * st;
    const double bz1 = q[2] * ct - q[0] * st;
    const double bx1 = bxs * cp - q[1] * sp;
    const double by1 = bxs * sp + q[1] * cp;
    xs = (x - xc) * cp - (y + yc) * sp;
    yss = (y + yc) * cp + (x - xc) * sp;
    zs = z - zc;
    xss = xs * ct - zs * st;
    zss = zs * ct + xs * st;
    t_circle(xss, yss, zss, R, q);
    bxs = q[0] * ct + q[2] * st;
    const double bz2 = q[2] * ct - q[0] * st;
    const double bx2 = bxs * cp + q[1] * sp;
    const double by2 = -bxs * sp + q[1] * cp;
    xs = -(x - xc) * cp + (y + yc) * sp;
    yss = -(y + yc) * cp - (x - xc) * sp;
    zs = z + zc;
    xss = xs * ct - zs * st;
    zss = zs * ct + xs * st;
    t_circle(xss, yss, zss, R, q);
    bxs = q[0] * ct + q[2] * st;
    const double bz3 = q[2] * ct - q[0] * st;
    const double bx3 = -bxs * cp - q[1] * sp;
    const double by3 = bxs * sp - q[1] * cp;
    xs = -(x - xc) * cp - (y - yc) * sp;
    yss = -(y - yc) * cp + (x - xc) * sp;
    zs = z + zc;
    xss = xs * ct - zs * st;
    zss = zs * ct + xs * st;
    t_circle(xss, yss, zss, R, q);
    bxs = q[0] * ct + q[2] * st;
    b[0] = bx1 + bx2 + bx3 + (-bxs * cp + q[1] * sp);
    b[1] = by1 + by2 + by3 + (-bxs * sp - q[1] * cp);
    b[2] = bz1 + bz2 + bz3 + (q[2] * ct - q[0] * st);
}

static void t_r2inner(double x, double y, double z, double b[3]) {
    double cbx[5], cby[5], cbz[5], d8[3], d6[3], d7[3];
    t_bconic(x, y, z, cbx, cby, cbz);
    t_loops4(x, y, z, d8, -8.1902, 6.5239, 5.504, 7.7815, .8573, 3.0986);
    t_dipdistr(x - .0774, y, z, d6, 0);
    t_dipdistr(x + .038, y, z, d7, 1);
    const double *cb[3] = { cbx, cby, cbz };
    for (int c = 0; c < 3; c++)
        b[c] = 154.185 * cb[c][0] + -2.12446 * cb[c][1] + 0.601735E-01 * cb[c][2] + -.153954E-02 * cb[c][3] +
               .355077E-04 * cb[c][4] + 29.9996 * d6[c] + 262.886 * d7[c] + 99.9132 * d8[c];
}

static void t_r2outer(double x, double y, double z, double b[3]) {
    double d1[3], d2[3], d3[3], d4[3], d5[3];
    t_crosslp(x, y, z, d1, 0.55, 0.694, 0.0031);
    t_crosslp(x, y, z, d2, 1.55, 2.8, 0.1375);
    t_crosslp(x, y, z, d3, -0.7, 0.2, 0.9625);
    t_circle(x + 2.994, y, z, 2.925, d4);
    t_loops4(x, y, z, d5, -1.775, 4.3, -0.275, 2.7, 0.4312, 1.55);
    for (int c = 0; c < 3; c++)
        b[c] = -34.105 * d1[c] + -2.00019 * d2[c] + 628.639 * d3[c] + 73.4847 * d4[c] + 12.5162 * d5[c];
}

/* Region-2 sheet (:1511-1593): tables of the 5 latitudinal modes x 4
 * longitudinal modes x {1, T1, T2, T3} for each component. */
static void t_r2sheet(double x, double y, double z, double b[3]) {
    static const double CX[5][4][4] = {
        { { 8.07190, -7.39582, -7.62341, 0.684671 }, { -13.5672, 11.6681, 13.1154, -0.890217 },
          { 7.78726, -5.38346, -8.08738, 0.609385 }, { -2.70410, 3.53741, 3.15549, -1.11069 } },
        { { -8.47555, 0.278122, 2.73514, 4.55625 }, { 13.1134, 1.15848, -3.52648, -8.24698 },
          { -6.85710, -2.81369, 2.03795, 4.64383 }, { 2.49309, -1.22041, -1.67432, -0.422526 } },
        { { -5.39796, 7.10326, 5.53730, -13.1918 }, { 4.67853, -7.60329, -2.53066, 7.76338 },
          { 5.60165, 5.34816, -4.56441, 7.05976 }, { -2.62723, -0.529078, 1.42019, -2.93919 } },
        { { 55.6338, -1.55181, 39.8311, -80.6561 }, { -46.9655, 32.8925, -6.32296, 19.7841 },
          { 124.731, 10.4347, -30.7581, 102.680 }, { -47.4037, -3.31278, 9.37141, -50.0268 } },
        { { -533.319, 110.426, 1000.20, -1051.40 }, { 1619.48, 589.855, -1462.73, 1087.10 },
          { -1994.73, -1654.12, 1263.33, -260.210 }, { 1424.84, 1255.71, -956.733, 219.946 } } };
    static const double CY[5][4][4] = {
        { { -9.08427, 10.6777, 10.3288, -0.969987 }, { 6.45257, -8.42508, -7.97464, 1.41996 },
          { -1.92490, 3.93575, 2.83283, -1.48621 }, { 0.244033, -0.757941, -0.386557, 0.344566 } },
        { { 9.56674, -2.5365, -3.32916, -5.86712 }, { -6.19625, 1.83879, 2.52772, 4.34417 },
          { 1.87268, -2.13213, -1.69134, -0.176379 }, { -0.261359, 0.566419, 0.3138, -0.134699 } },
        { { -3.83086, -8.4154, 4.77005, -9.31479 }, { 37.5715, 19.3992, -17.9582, 36.4604 },
          { -14.9993, -3.1442, 6.17409, -15.5519 }, { 2.28621, -0.00891549, -0.462912, 2.47314 } },
        { { 41.7555, 208.614, -45.7861, -77.8687 }, { 239.357, -67.9226, 66.8743, 238.534 },
          { -112.136, 16.2069, -40.4706, -134.328 }, { 21.56, -0.201725, 2.21, 32.5855 } },
        { { -108.217, -1005.98, 585.753, 323.668 }, { -817.056, 235.750, -560.965, -576.892 },
          { 684.193, 85.0275, 168.394, 477.776 }, { -289.253, -123.216, 75.6501, -178.605 } } };
    static const double CZ[5][4][4] = {
        { { 1167.61, -917.782, -1253.2, -274.128 }, { -1538.75, 1257.62, 1745.07, 113.479 },
          { 393.326, -426.858, -641.1, 190.833 }, { -29.9435, -1.04881, 117.125, -25.7663 } },
        { { -1168.16, 910.247, 1239.31, 289.515 }, { 1540.56, -1248.29, -1727.61, -131.785 },
          { -394.577, 426.163, 637.422, -187.965 }, { 30.0348, 0.221898, -116.68, 26.0291 } },
        { { 12.6804, 4.84091, 1.18166, -2.75946 }, { -17.9822, -6.80357, -1.47134, 3.02266 },
          { 4.79648, 0.665255, -0.256229, -0.0857282 }, { -0.588997, 0.0634812, 0.164303, -0.15285 } },
        { { 22.2524, -22.4376, -3.85595, 6.07625 }, { -105.959, -41.6698, 0.378615, 1.55958 },
          { 44.3981, 18.8521, 3.19466, 5.89142 }, { -8.63227, -2.36418, -1.027, -2.31515 } },
        { { 1035.38, 2040.66, -131.881, -744.533 }, { -3274.93, -4845.61, 482.438, 1567.43 },
          { 1354.02, 2040.47, -151.653, -845.012 }, { -111.723, -265.343, -26.1171, 216.632 } } };
    const double xks = t_xksi(x, y, z);
    const double xks2 = xks * xks;
    const double t1x = xks / sqrt(xks2 + 0.483750e-01 * 0.483750e-01);
    const double px72 = 0.396953e-01 * 0.396953e-01;
    const double qx = sqrt(xks2 + px72);
    const double t2x = (px72 * 0.396953e-01) / (qx * qx * qx);
    const double t3x = xks / pow(sqrt(xks2 + 0.579023e-01 * 0.579023e-01), 5) * 3.493856 * (pow)(0.579023e-01, 4);
    const double t1y = xks / sqrt(xks2 + 0.478750e-01 * 0.478750e-01);
    const double py72 = 0.363750e-01 * 0.363750e-01;
    const double qy = sqrt(xks2 + py72);
    const double t2y = (py72 * 0.363750e-01) / (qy * qy * qy);
    const double t3y = xks / pow(sqrt(xks2 + 0.567500e-01 * 0.567500e-01), 5) * 3.493856 * (pow)(0.567500e-01, 4);
    const double t1z = xks / sqrt(xks2 + 0.355625e-01 * 0.355625e-01);
    const double pz72 = 0.318750e-01 * 0.318750e-01;
    const double qz = sqrt(xks2 + pz72);
    const double t2z = (pz72 * 0.318750e-01) / (qz * qz * qz);
    const double t3z = xks / pow(sqrt(xks2 + 0.538750e-01 * 0.538750e-01), 5) * 3.493856 * (pow)(0.538750e-01, 4);
    const double rho2 = x * x + y * y;
    const double r = sqrt(rho2 + z * z);
    const double rho = sqrt(rho2);
    const double c1p = x / rho, s1p = y / rho;
    const double s2p = 2.0 * s1p * c1p;
    const double c2p = c1p * c1p - s1p * s1p;
    const double s3p = s2p * c1p + c2p * s1p;
    const double c3p = c2p * c1p - s2p * s1p;
    const double s4p = s3p * c1p + c3p * s1p;
    const double ct = z / r;
    const double ct2 = ct * ct;
    const double ct2m1 = ct2 - 1.0;
    const double stmp = -2. * 2.718281828459;
    double s[5];
    /* x component */
    s[0] = sqrt(stmp * -19.0969) * ct * exp(-19.0969 * ct2);
    s[1] = sqrt(stmp * -9.28828) * ct * exp(-9.28828 * ct2);
    s[2] = sqrt(stmp * -0.129687) * ct * exp(-0.129687 * ct2);
    s[3] = ct * exp(5.58594 * ct2m1);
    s[4] = ct * exp(22.5055 * ct2m1);
    double acc = 0.0;
    for (int l = 0; l < 5; l++) {
        const double (*c)[4] = CX[l];
        const double term = (c[0][0] + c[0][1] * t1x + c[0][2] * t2x + c[0][3] * t3x) +
                            c1p * (c[1][0] + c[1][1] * t1x + c[1][2] * t2x + c[1][3] * t3x) +
                            c2p * (c[2][0] + c[2][1] * t1x + c[2][2] * t2x + c[2][3] * t3x) +
                            c3p * (c[3][0] + c[3][1] * t1x + c[3][2] * t2x + c[3][3] * t3x);
        acc = (l == 0) ? s[l] * term : acc + s[l] * term;
    }
    b[0] = acc;
    /* y component */
    s[0] = sqrt(stmp * -13.6750) * ct * exp(-13.6750 * ct2);
    s[1] = sqrt(stmp * -6.70625) * ct * exp(-6.70625 * ct2);
    s[2] = ct * exp(2.31875 * ct2m1);
    s[3] = ct * exp(11.4062 * ct2m1);
    s[4] = ct * exp(20.4562 * ct2m1);
    acc = 0.0;
    for (int l = 0; l < 5; l++) {
        const double (*c)[4] = CY[l];
        const double term = s1p * (c[0][0] + c[0][1] * t1y + c[0][2] * t2y + c[0][3] * t3y) +
                            s2p * (c[1][0] + c[1][1] * t1y + c[1][2] * t2y + c[1][3] * t3y) +
                            s3p * (c[2][0] + c[2][1] * t1y + c[2][2] * t2y + c[2][3] * t3y) +
                            s4p * (c[3][0] + c[3][1] * t1y + c[3][2] * t2y + c[3][3] * t3y);
        acc = (l == 0) ? s[l] * term : acc + s[l] * term;
    }
    b[1] = acc;
    /* z component */
    s[0] = exp(-16.7125 * ct2);
    s[1] = exp(-16.4625 * ct2);
    s[2] = exp(-0.1625 * ct2);
    s[3] = exp(5.1 * (ct2 - 1.0));
    s[4] = exp(23.7125 * (ct2 - 1.0));
    acc = 0.0;
    for (int l = 0; l < 5; l++) {
        const double (*c)[4] = CZ[l];
        const double term = (c[0][0] + c[0][1] * t1z + c[0][2] * t2z + c[0][3] * t3z) +
                            c1p * (c[1][0] + c[1][1] * t1z + c[1][2] * t2z + c[1][3] * t3z) +
                            c2p * (c[2][0] + c[2][1] * t1z + c[2][2] * t2z + c[2][3] * t3z) +
                            c3p * (c[3][0] + c[3][1] * t1z + c[3][2] * t2z + c[3][3] * t3z);
        acc = (l == 0) ? s[l] * term : acc + s[l] * term;
    }
    b[2] = acc;
}

static void t_r2birk(double x, double y, double z, double b[3]) {
    const double dl = 0.03, dl1 = 0.015;
    const double xks = t_xksi(x, y, z);
    double bx = 0.0, by = 0.0, bz = 0.0, q1[3], q2[3];
    if (xks < -(dl + dl1)) {
        t_r2outer(x, y, z, q1);
        bx = q1[0] * -0.02; by = q1[1] * -0.02; bz = q1[2] * -0.02;
    }
    if (xks >= -(dl + dl1) && xks < -dl + dl1) {
        t_r2outer(x, y, z, q1);
        t_r2sheet(x, y, z, q2);
        const double f2 = -0.02 * t_tksi(xks, -dl, dl1);
        const double f1 = -0.02 - f2;
        bx = q1[0] * f1 + q2[0] * f2; by = q1[1] * f1 + q2[1] * f2; bz = q1[2] * f1 + q2[2] * f2;
    }
    if (xks >= -dl + dl1 && xks < dl - dl1) {
        t_r2sheet(x, y, z, q1);
        bx = q1[0] * -0.02; by = q1[1] * -0.02; bz = q1[2] * -0.02;
    }
    if (xks >= dl - dl1 && xks < dl + dl1) {
        t_r2inner(x, y, z, q1);
        t_r2sheet(x, y, z, q2);
        const double f1 = -0.02 * t_tksi(xks, dl, dl1);
        const double f2 = -0.02 - f1;
        bx = q1[0] * f1 + q2[0] * f2; by = q1[1] * f1 + q2[1] * f2; bz = q1[2] * f1 + q2[2] * f2;
    }
    if (xks >= dl + dl1) {
        t_r2inner(x, y, z, q1);
        bx = -q1[0] * 0.02; by = -q1[1] * 0.02; bz = -q1[2] * 0.02;
    }
    b[0] = bx; b[1] = by; b[2] = bz;
}

/* dipole_t96 (:1645-1656) */
static void t_dipole(double x, double y, double z, double b[3]) {
    const double p = x * x, u = z * z, v = 3.0 * z * x, t = y * y;
    const double ptu = sqrt(p + t + u);
    const double q = 30574.0 / (ptu * ptu * ptu * ptu * ptu);
    b[0] = q * ((t + u - 2.0 * p) - v);
    b[1] = -3.0 * y * q * z;
    b[2] = q * (p + t - 2.0 * u);
}

/* ---- t96_gsm, lib/t96/t96.c:4-111 ------------------------------------- */
void orc_t96_gsm(const double *parmod, double x, double y, double z, double *bxo, double *byo, double *bzo) {
    const double pdyn = parmod[0];
    const double depr = 0.8 * parmod[1] - 13.0 * sqrt(pdyn);
    const double byimf = parmod[2], bzimf = parmod[3];
    const double bt = sqrt(byimf * byimf + bzimf * bzimf);
    double theta = 0.0;
    if (byimf != 0.0 || bzimf != 0.0) {
        theta = (atan2)(byimf, bzimf);
        if (theta <= 0.0) theta += 6.2831853;
    }
    const double ct = (cos)(theta), st = (sin)(theta);
    const double eps = 718.5 * sqrt(pdyn) * bt * (sin)(theta / 2.);
    const double ys = y * ct - z * st, zs = z * ct + y * st;
    const double ysd = ys / 10.0;
    const double factimf = exp(x / 20.0 - ysd * ysd);
    const double oimfy = 0.7850 * byimf * factimf, oimfz = 0.7850 * bzimf * factimf;
    const double xappa = (pow)(pdyn / 2.0, 0.14);
    const double xappa3 = xappa * xappa * xappa;
    const double am = 70.0 / xappa;
    const double rho2 = y * y + z * z;
    const double asq = am * am;
    double xmxm = am + x - (5.48 / xappa);
    if (xmxm < 0.0) xmxm = 0.0;
    const double axx0 = xmxm * xmxm;
    const double aro = asq + rho2;
    const double aa = aro + axx0;
    const double sigma = sqrt((aro + axx0 + sqrt(aa * aa - 4.0 * asq * axx0)) / (2.0 * asq));
    double q[3];
    if (sigma >= 1.08 + 0.005) {
        t_dipole(x, y, z, q);
        *bxo = -q[0];
        *byo = oimfy - q[1];
        *bzo = oimfz - q[2];
        return;
    }
    const double factes = eps / 3630.7 - 1.0;
    const double factpd = sqrt(pdyn / 2.0) - 1.0;
    const double rcampl = -1.162 * depr;
    const double tampl2 = 22.344 + 18.50 * factpd + 2.602 * factes;
    const double tampl3 = 6.903 + 5.287 * factpd;
    const double b1ampl = 0.5790 + 0.4462 * factes;
    const double b2ampl = 20.0 * b1ampl;
    const double xx = x * xappa, yy = y * xappa, zz = z * xappa;
    double cf[3], rc[3], t2[3], t3[3], r1[3], r2[3], r2h[3], im[3];
    t_cylharm(xx, yy, zz, cf);
    t_tailrc(xx, yy, zz, rc, t2, t3);
    t_birk1tot(xx, yy, zz, r1);
    t_birk2shl(xx, yy, zz, r2);
    t_r2birk(xx, yy, zz, r2h);
    r2[0] += r2h[0]; r2[1] += r2h[1]; r2[2] += r2h[2];
    t_intercon(xx, ys * xappa, zs * xappa, im);
    const double rimfy = im[1] * ct + im[2] * st;
    const double rimfz = im[2] * ct - im[1] * st;
    const double rimfampl = 0.7850 * bt;
    const double fx = cf[0] * xappa3 + rcampl * rc[0] + tampl2 * t2[0] + tampl3 * t3[0] + b1ampl * r1[0] + b2ampl * r2[0] + rimfampl * im[0];
    const double fy = cf[1] * xappa3 + rcampl * rc[1] + tampl2 * t2[1] + tampl3 * t3[1] + b1ampl * r1[1] + b2ampl * r2[1] + rimfampl * rimfy;
    const double fz = cf[2] * xappa3 + rcampl * rc[2] + tampl2 * t2[2] + tampl3 * t3[2] + b1ampl * r1[2] + b2ampl * r2[2] + rimfampl * rimfz;
    if (sigma < 1.08 - 0.005) {
        *bxo = fx; *byo = fy; *bzo = fz;
        return;
    }
    const double fint = 0.5 * (1.0 - (sigma - 1.08) / 0.005);
    const double fext = 0.5 * (1.0 + (sigma - 1.08) / 0.005);
    t_dipole(x, y, z, q);
    *bxo = (fx + q[0]) * fint - q[0];
    *byo = (fy + q[1]) * fint + oimfy * fext - q[1];
    *bzo = (fz + q[2]) * fint + oimfz * fext - q[2];
}
