/*
 * setup.c -- host-side set-up of the internal field and the GSM frame.
 *
 * Runs once per condition on the host (microseconds) and fills the parameter
 * block the kernels read.  Restates internal_recalc
 * (lib/internal/internal.c:89-180) with its helpers interpolate / extrapolate
 * (:12-36), interpolate_or_extrapolate (:64-87) and sun (:38-62).  Built with
 * -ffp-contract=off like the reference, so g/h/rec/a1..a3 equal the
 * reference's bit for bit.
 */
#include <math.h>
#include <string.h>

#include "../../include/cor_trace.h"
#include "coef_tables.h"

#define S_TO_DEG 57.295779513 /* DEF_TO_DEG, lib/internal/internal.h:6 */

const cor_sh_table *cor_find_sh_table(const char *version) {
    if (!version) return NULL;
    for (int i = 0; i < cor_sh_table_count; i++)
        if (strcmp(cor_sh_tables[i].version, version) == 0) return &cor_sh_tables[i];
    return NULL;
}

/* Linear interpolation between two epochs, lib/internal/internal.c:12-22. */
static void s_interpolate(double *g, double *h, const double *gx, const double *hx,
                          const double *gy, const double *hy, int edge_year, int year, int iday,
                          double step) {
    const double f2 = (year + (iday - 1) / 365.25 - edge_year) / step;
    const double f1 = 1. - f2;
    for (int i = 0; i < COR_SH_COEFS; ++i) {
        g[i] = gx[i] * f1 + gy[i] * f2;
        h[i] = hx[i] * f1 + hy[i] * f2;
    }
}

/* Secular-variation extrapolation of the first 46 terms,
 * lib/internal/internal.c:24-36. */
static void s_extrapolate(double *g, double *h, const double *gx, const double *hx,
                          const double *gy, const double *hy, int max_year, int year, int iday,
                          double step) {
    const double dt = year + (iday - 1) / 365.25 - (max_year - step);
    for (int i = 0; i < COR_SH_COEFS; ++i) {
        g[i] = gx[i];
        h[i] = hx[i];
        if (i > 45) continue;
        g[i] += gy[i] * dt;
        h[i] += hy[i] * dt;
    }
}

/* Sun position and Greenwich sidereal time, lib/internal/internal.c:38-62. */
static void s_sun(int iyear, int iday, int ihour, int min, int isec, double *gst, double *slong,
                  double *srasn, double *sdec) {
    const double fday = (ihour * 3600 + min * 60 + isec) / 86400.;
    const double dj = 365 * (iyear - 1900) + (int)((iyear - 1901) / 4) + iday - 0.5 + fday;
    const double t = dj / 36525.;
    *gst = fmod(279.690983 + 0.9856473354 * dj + 360. * fday + 180., 360.) / S_TO_DEG;
    const double vl = fmod(279.696678 + 0.9856473354 * dj, 360.);
    const double g = fmod(358.475845 + 0.985600267 * dj, 360.) / S_TO_DEG;
    *slong = (vl + (1.91946 - 0.004789 * t) * sin(g) + 0.020094 * sin(2. * g)) / S_TO_DEG;
    if (*slong > 6.2831853) *slong = *slong - 6.2831853;
    else if (*slong < 0) *slong = *slong + 6.2831853;
    const double obliq = (23.45229 - 0.0130125 * t) / S_TO_DEG;
    const double slp = *slong - 9.924E-5;
    const double sob = sin(obliq);
    const double sind = sob * sin(slp);
    const double cosd = sqrt(1. - sind * sind);
    const double sc = sind / cosd;
    *sdec = atan(sc);
    *srasn = 3.141592654 - atan2(cos(obliq) / sob * sc, -cos(slp) / cosd);
}

/* Epoch selection, lib/internal/internal.c:64-87.  The index arithmetic is
 * unsigned like the reference's uint32_t fields. */
static int s_epoch_coefs(const cor_sh_table *t, int year, int iday, double *g, double *h) {
    const double *const *gh = t->gh;
    const unsigned n = (unsigned)t->n_arrays, step = (unsigned)t->years_step;
    const unsigned min_year = (unsigned)t->min_year, max_year = (unsigned)t->max_year;
    if (t->extrapolate && max_year - year <= step) {
        s_extrapolate(g, h, gh[n - 4], gh[n - 3], gh[n - 2], gh[n - 1], (int)max_year, year, iday, step);
        return 0;
    }
    if ((unsigned)year >= max_year) return -1;
    int idx;
    if ((unsigned)year <= min_year) idx = (int)(max_year / step - (min_year + 1) / step);
    else idx = (int)(max_year / step - year / step);
    const int pos = (int)n - 2 * idx - 1;
    const int edge_year = (int)(min_year + ((pos - 1) / 2) * step);
    s_interpolate(g, h, gh[pos - 1], gh[pos], gh[pos + 1], gh[pos + 2], edge_year, year, iday, step);
    return 0;
}

/* GEO->GSM rows from the dipole (g10, g11, h11) and the sun,
 * lib/internal/internal.c:129-178. */
static void s_gsm_axes(const double *g, const double *h, const int32_t tm[7], double *a1, double *a2,
                       double *a3) {
    const double g10 = -g[1];
    const double g11 = g[2];
    const double h11 = h[2];
    const double sq = g11 * g11 + h11 * h11;
    const double sqq = sqrt(sq);
    const double sqr = sqrt(g10 * g10 + sq);
    double gst = 0., slong = 0., srasn = 0., sdec = 0.;
    if (tm[0] > 1900 && tm[0] < 2100) s_sun(tm[0], tm[3], tm[4], tm[5], tm[6], &gst, &slong, &srasn, &sdec);
    const double ct0 = g10 / sqr;
    const double cl0 = -g11 / sqq;
    const double sl0 = -h11 / sqq;
    const double st0 = sqq / sqr;
    const double stcl = st0 * cl0;
    const double stsl = st0 * sl0;
    const double cgst = cos(gst);
    const double sgst = sin(gst);
    const double dip1 = stcl * cgst - stsl * sgst;
    const double dip2 = stcl * sgst + stsl * cgst;
    const double dip3 = ct0;
    const double csdec = cos(sdec);
    const double s1 = cos(srasn) * csdec;
    const double s2 = sin(srasn) * csdec;
    const double s3 = sin(sdec);
    double y1 = dip2 * s3 - dip3 * s2;
    double y2 = dip3 * s1 - dip1 * s3;
    double y3 = dip1 * s2 - dip2 * s1;
    const double y = sqrt(y1 * y1 + y2 * y2 + y3 * y3);
    y1 = y1 / y;
    y2 = y2 / y;
    y3 = y3 / y;
    const double z1 = s2 * y3 - s3 * y2;
    const double z2 = s3 * y1 - s1 * y3;
    const double z3 = s1 * y2 - s2 * y1;
    a1[0] = s1 * cgst + s2 * sgst;
    a1[1] = -s1 * sgst + s2 * cgst;
    a1[2] = s3;
    a2[0] = y1 * cgst + y2 * sgst;
    a2[1] = -y1 * sgst + y2 * cgst;
    a2[2] = y3;
    a3[0] = z1 * cgst + z2 * sgst;
    a3[1] = -z1 * sgst + z2 * cgst;
    a3[2] = z3;
}

static int s_recalc(const cor_sh_table *t, const int32_t tm[7], cor_model_params *out) {
    if (tm[0] > t->max_year || tm[0] < t->min_year) return COR_ERR_RANGE;  /* :90-92 */
    /* Legendre recursion factors, :94-103 */
    double n2;
    for (int i = 1; i < 15; ++i) {
        n2 = 2 * i - 1;
        n2 = n2 * (n2 - 2);
        for (int j = 1; j < i + 1; ++j) {
            const int mn = i * (i - 1) / 2 + j - 1;
            out->rec[mn] = ((i - j) * (i + j - 2)) / n2;
        }
    }
    if (s_epoch_coefs(t, tm[0], tm[3], out->g, out->h) != 0) return COR_ERR_RANGE;
    /* Schmidt semi-normalisation folded into G/H, :109-127 */
    double s = 1., p, aa;
    for (int i = 2; i <= 14; ++i) {
        const int mn = (i * (i - 1) / 2 + 1) - 1;
        s = s * (2 * i - 3) / (i - 1);
        out->g[mn] *= s;
        out->h[mn] *= s;
        p = s;
        for (int j = 2; j <= i; j++) {
            aa = 1.;
            if (j == 2) aa = 2.;
            p = p * sqrt(aa * (i - j + 1) / (i + j - 2));
            const int mnn = mn + j - 1;
            out->g[mnn] *= p;
            out->h[mnn] *= p;
        }
    }
    s_gsm_axes(out->g, out->h, tm, out->a1, out->a2, out->a3);
    return COR_OK;
}

int cor_internal_setup(const char *version, const int32_t time[7], cor_model_params *out) {
    if (!out || !time) return COR_ERR_INVALID;
    const cor_sh_table *t = cor_find_sh_table(version);
    if (!t) return COR_ERR_INVALID;
    return s_recalc(t, time, out);
}

int cor_gsm_setup(const int32_t time[7], cor_model_params *out) {
    if (!out || !time) return COR_ERR_INVALID;
    cor_model_params tmp;
    const int rc = s_recalc(&cor_sh_tables[0], time, &tmp);
    if (rc != COR_OK) return rc;
    memcpy(out->a1, tmp.a1, sizeof tmp.a1);
    memcpy(out->a2, tmp.a2, sizeof tmp.a2);
    memcpy(out->a3, tmp.a3, sizeof tmp.a3);
    return COR_OK;
}
