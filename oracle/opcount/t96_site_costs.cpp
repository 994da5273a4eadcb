// t96_site_costs.cpp -- TEST INFRASTRUCTURE: the cost of every expensive call
// site of the T96 field at given positions, and the bands that decide which
// sites a position reaches, from the op-counting oracle (flop.hpp).
//
// Built by warp_divergence.py with -include flop.hpp; oracle/t96_oracle.c is
// included here so that its static functions (the reference's sub-models,
// lib/t96/t96.c) can be called one at a time.  Costs are weighted FP64
// operations: + - * 1, and division, square root and every C-library function
// at the cost measured on the GPU (cor_probe_fp64_functions).
//
// usage: t96_site_costs <positions.bin> <out.bin> <pdyn> <dst> <byimf> <bzimf>
//   positions.bin: n x 3 doubles, GSM metres; out.bin: n x kCols doubles.
#include "../t96_oracle.c"
#undef double

thread_local FlopTally g_tally;

namespace {
// add, mul, div, sqrt, exp, log, sin, cos, tan, atan, asin, atan2, pow, fmod
const double kWeight[FC_N] = {1, 1, 14.7, 15.2, 30.0, 58.4, 35.3, 35.3, 35.3, 55.3, 82.4, 76.4, 170.6, 50.0};

double take() {
    double c = 0;
    for (int k = 0; k < FC_N; k++) c += kWeight[k] * (double)g_tally.by_class[k];
    g_tally = FlopTally();
    return c;
}

// Output columns.
enum Col {
    kWhole,     // orc_t96_gsm at the point
    kSigma,     // 0 inside the magnetopause, 1 boundary layer, 2 outside
    kCylharm, kTailrc, kBirk2shl, kIntercon, kBirk1shld,
    kBirk1Pre,  // birk1tot_02 up to its band decision
    kBirk1Band, // 0 loops basis at the point, 1 conical basis at the point, 2 north blend, 3 south blend
    kLoopsAt, kCondipAt,                    // each basis at the point
    kBlend,                                 // the whole blend (band 2/3 only)
    kLoopsE1, kCondipE1, kLoopsE2, kCondipE2,  // each basis at the two edge points (band 2/3 only)
    kXksi,
    kR2Band,    // r2_birk's five xksi bands
    kR2Outer, kR2Sheet, kR2Inner,
    kR2Birk, kBirk1Tot,
    kRadius,    // |x| in R_E
    kRingcurr, kShlcar, kTaildisk, kTail87,  // the parts of tailrc96 (one shield: all three cost alike)
    kCols
};
}  // namespace

#define COST(...) ([&] { g_tally = FlopTally(); __VA_ARGS__; return take(); }())

int main(int argc, char** argv) {
    if (argc < 7) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    fseek(f, 0, SEEK_END);
    const long n = ftell(f) / 24;
    fseek(f, 0, SEEK_SET);
    double* s = (double*)malloc(24 * (size_t)n);
    if (fread(s, 24, n, f) != (size_t)n) return 4;
    fclose(f);
    const flop_t parmod[10] = {atof(argv[3]), atof(argv[4]), atof(argv[5]), atof(argv[6]), 0, 0, 0, 0, 0, 0};
    const flop_t pdyn = parmod[0];
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 5;
    for (long i = 0; i < n; i++) {
        const flop_t x = s[3 * i] / 6.3712e+06, y = s[3 * i + 1] / 6.3712e+06, z = s[3 * i + 2] / 6.3712e+06;
        double out[kCols] = {0};
        flop_t bx, by, bz, b[3];
        out[kWhole] = COST(orc_t96_gsm(parmod, x, y, z, &bx, &by, &bz));
        // magnetopause (lib/t96/t96.c:4-111)
        const flop_t xappa = pow(pdyn / 2.0, 0.14);
        const flop_t am = 70.0 / xappa, asq = am * am;
        flop_t xmxm = am + x - (5.48 / xappa);
        if (xmxm < 0.0) xmxm = 0.0;
        const flop_t axx0 = xmxm * xmxm, aro = asq + y * y + z * z, aa = aro + axx0;
        const flop_t sigma = sqrt((aro + axx0 + sqrt(aa * aa - 4.0 * asq * axx0)) / (2.0 * asq));
        out[kSigma] = sigma >= 1.085 ? 2 : (sigma < 1.075 ? 0 : 1);
        const flop_t xx = x * xappa, yy = y * xappa, zz = z * xappa;
        flop_t rc[3], t2[3], t3[3];
        out[kCylharm] = COST(t_cylharm(xx, yy, zz, b));
        out[kTailrc] = COST(t_tailrc(xx, yy, zz, rc, t2, t3));
        out[kBirk2shl] = COST(t_birk2shl(xx, yy, zz, b));
        out[kIntercon] = COST(t_intercon(xx, yy, zz, b));
        out[kBirk1shld] = COST(t_birk1shld(xx, yy, zz, b));
        // birk1tot_02's band decision (lib/t96/t96.c:619-689)
        flop_t tet0, pas, r, r3, t01n, t02n, t01s, t02s;
        out[kBirk1Pre] = COST({
            const flop_t tnoonn = 12.0 * 0.01745329, tnoons = 3.141592654 - tnoonn;
            const flop_t r2 = xx * xx + yy * yy + zz * zz;
            r = sqrt(r2);
            r3 = r * r2;
            pas = 0.0;
            if (xx != 0.0 || yy != 0.0) pas = atan2(yy, xx);
            const flop_t tas = atan2(sqrt(xx * xx + yy * yy), zz);
            const flop_t stas = sin(tas);
            tet0 = asin(stas / pow((stas * stas * stas * stas * stas * stas) * (1.0 - r3) + r3, 0.1666666667));
            if (tas > 1.5707963) tet0 = 3.141592654 - tet0;
            const flop_t dtet = (8.0 * 0.01745329) * (sin(pas * 0.5) * sin(pas * 0.5));
            const flop_t tr1n = tnoonn + dtet, tr1s = tnoons - dtet;
            t01n = tr1n - 0.034906;
            t01s = tr1s - 0.034906;
            t02s = tr1s + 0.034906;
            t02n = tr1n + 0.034906;
        });
        int band;
        if (tet0 < t01n || tet0 > t02s) band = 0;
        else if (tet0 > t02n && tet0 < t01s) band = 1;
        else if (tet0 >= t01n && tet0 <= t02n) band = 2;
        else band = 3;
        out[kBirk1Band] = band;
        {
            flop_t D1[3][14], D2[3][42], t[3];
            out[kLoopsAt] = COST(t_diploop1(xx, yy, zz, D1); t_sum_d1(D1, t));
            out[kCondipAt] = COST(t_condip1(xx, yy, zz, D2); t_sum_d2(D2, t));
        }
        if (band >= 2) {
            const bool south = band == 3;
            const flop_t t1 = south ? t01s : t01n, t2b = south ? t02s : t02n;
            const flop_t sqr = sqrt(r);
            const flop_t s1 = sin(t1), s2 = sin(t2b);
            const flop_t st01 = sqr / pow(r3 + 1.0 / (s1 * s1 * s1 * s1 * s1 * s1) - 1.0, 0.1666666667);
            const flop_t st02 = sqr / pow(r3 + 1.0 / (s2 * s2 * s2 * s2 * s2 * s2) - 1.0, 0.1666666667);
            flop_t ct01 = sqrt(1.0 - st01 * st01), ct02 = sqrt(1.0 - st02 * st02);
            if (south) {
                ct01 = -ct01;
                ct02 = -ct02;
            }
            const flop_t x1 = r * st01 * cos(pas), y1 = r * st01 * sin(pas), z1 = r * ct01;
            const flop_t x2 = r * st02 * cos(pas), y2 = r * st02 * sin(pas), z2 = r * ct02;
            flop_t D1[3][14], D2[3][42], t[3];
            out[kBlend] = COST(t_birk1_blend(xx, yy, zz, r, r3, pas, t1, t2b, south, t));
            out[kLoopsE1] = COST(t_diploop1(x1, y1, z1, D1); t_sum_d1(D1, t));
            out[kCondipE1] = COST(t_condip1(x1, y1, z1, D2); t_sum_d2(D2, t));
            out[kLoopsE2] = COST(t_diploop1(x2, y2, z2, D1); t_sum_d1(D1, t));
            out[kCondipE2] = COST(t_condip1(x2, y2, z2, D2); t_sum_d2(D2, t));
        }
        // r2_birk's bands (lib/t96/t96.c:1265-1314)
        flop_t xks;
        out[kXksi] = COST(xks = t_xksi(xx, yy, zz));
        const double dl = 0.03, dl1 = 0.015;
        out[kR2Band] = xks < -(dl + dl1) ? 0 : xks < -dl + dl1 ? 1 : xks < dl - dl1 ? 2 : xks < dl + dl1 ? 3 : 4;
        out[kR2Outer] = COST(t_r2outer(xx, yy, zz, b));
        out[kR2Sheet] = COST(t_r2sheet(xx, yy, zz, b));
        out[kR2Inner] = COST(t_r2inner(xx, yy, zz, b));
        out[kR2Birk] = COST(t_r2birk(xx, yy, zz, b));
        out[kBirk1Tot] = COST(t_birk1tot(xx, yy, zz, b));
        out[kRadius] = std::sqrt(s[3 * i] * s[3 * i] + s[3 * i + 1] * s[3 * i + 1] + s[3 * i + 2] * s[3 * i + 2]) /
                       6.3712e+06;
        {
            // a shield's cost does not depend on its coefficient values
            flop_t coef[24];
            for (int k = 0; k < 24; k++) coef[k] = 1.0 + 0.1 * k;
            flop_t hx, hz;
            out[kRingcurr] = COST(t_ringcurr(xx, yy, zz, b));
            out[kShlcar] = COST(t_shlcar3x3(coef, xx, yy, zz, b));
            out[kTaildisk] = COST(t_taildisk(xx, yy, zz, b));
            out[kTail87] = COST(t_tail87(xx, zz, &hx, &hz));
        }
        fwrite(out, sizeof(double), kCols, o);
    }
    fclose(o);
    free(s);
    return 0;
}
