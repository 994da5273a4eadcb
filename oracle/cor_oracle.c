/*
 * cor_oracle.c -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU restatement of the reference's rigidity scan: geometry, the
 * spherical-harmonic internal field, field composition, the 6-stage RK step and
 * the scan loop with its step control and terminations.  Each function cites
 * the reference file:line it restates.  Operation order follows the reference
 * expression by expression, and the file is compiled with -ffp-contract=off
 * like the reference (CMakeLists.txt:17), so the results are the reference's
 * bit for bit on the same C library.  Only tests/, smoke() and bench.py's CPU
 * baseline load it.
 */
#include "cor_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* Physical constants, legacy-truncated as in src/common.h:4-11. */
#define O_PI 3.141592654
#define O_2PI 6.28318531
#define O_RE 6.3712e+06
#define O_TO_RAD (O_PI / 180.)
#define O_Q 1.6021e-19
#define O_C 2.99725e+08

/* Boundary refinement doubles nk0 without a bound in the reference
 * (src/trajectory.c:126-130); its int nk0 would overflow past 2^31.  Both the
 * oracle and the kernels stop at this value and report COR_TRAJ_WATCHDOG. */
#define O_NK0_CAP (1 << 30)

/* ---- geometry: src/utils.c:28-101 ------------------------------------- */
static void o_sph_to_car(double r, double theta, double phi, double car[3]) {
    /* src/utils.c:28-41.  The parenthesised names keep these calls out of the
     * one-ulp libm perturbation build (nudge/), as the device takes them from
     * the host C library. */
    const double sq = r * (sin)(theta);
    car[0] = sq * (cos)(phi);
    car[1] = sq * (sin)(phi);
    car[2] = r * (cos)(theta);
}

static void o_car_to_sph(const double car[3], double sph[3]) {
    /* src/utils.c:43-73 */
    const double x = car[0], y = car[1], z = car[2];
    const double sq = x * x + y * y;
    const double r = sqrt(sq + z * z);
    if (sq != 0.) {
        double phi = atan2(y, x);
        const double theta = atan2(sqrt(sq), z);
        if (phi < 0.) phi += O_2PI;
        sph[0] = r; sph[1] = theta; sph[2] = phi;
        return;
    }
    sph[0] = r;
    sph[1] = (z < 0.) ? O_PI : 0.;
    sph[2] = 0.;
}

static void o_geo_to_gsm(const double g[3], double out[3], const cor_model_params *p) {
    /* src/utils.c:75-87: rows of A */
    const double x = g[0], y = g[1], z = g[2];
    out[0] = p->a1[0] * x + p->a1[1] * y + p->a1[2] * z;
    out[1] = p->a2[0] * x + p->a2[1] * y + p->a2[2] * z;
    out[2] = p->a3[0] * x + p->a3[1] * y + p->a3[2] * z;
}

static void o_gsm_to_geo(const double s[3], double out[3], const cor_model_params *p) {
    /* src/utils.c:89-101: columns of A */
    const double x = s[0], y = s[1], z = s[2];
    out[0] = p->a1[0] * x + p->a2[0] * y + p->a3[0] * z;
    out[1] = p->a1[1] * x + p->a2[1] * y + p->a3[1] * z;
    out[2] = p->a1[2] * x + p->a2[2] * y + p->a3[2] * z;
}

/* ---- internal field: lib/internal/internal.c:182-275 ------------------- */
static int o_internal_degree(double R) {
    /* truncation by radius, lib/internal/internal.c:201-205 */
    int nm = 3 + 30 / ((int)R + 2);
    return nm > 13 ? 13 : nm;
}

void orc_internal_geo(double x, double y, double z, const double *g, const double *h,
                      const double *rec, double *bx, double *by, double *bz) {
    double pw[14], pwn[14];  /* A[] and B[] of the reference: (1/R)^(n+2), times n+1 */
    const double rho2 = x * x + y * y;
    const double R = sqrt(rho2 + z * z);
    const double C = z / R;
    const double rho = sqrt(rho2);
    const double S = rho / R;
    const int pole = S < 1.E-5;
    double cf, sf;
    if (pole) { cf = 1.; sf = 0.; } else { cf = x / rho; sf = y / rho; }

    const double pp = 1. / R;
    double p = pp;
    const int K = o_internal_degree(R) + 1;
    for (int n = 1; n <= K; n++) {
        p = p * pp;
        pw[n - 1] = p;
        pwn[n - 1] = p * n;
    }

    /* m-outer, n-inner recursion of the reference (:214-258): the order of
     * the running sums is what fixes the rounding, so it is kept. */
    double pmm = 1., dmm = 0.;           /* P and D carried between m columns */
    double br = 0., bt = 0., bf = 0.;
    double cm = 0., sm = 1.;             /* X, Y: sin/cos recursion in m */
    for (int m = 1; m <= K; m++) {
        if (m != 1) {
            const double w = cm;
            cm = w * cf + sm * sf;
            sm = sm * cf - w * sf;
        }
        double q = pmm, zz = dmm, bi = 0., p2 = 0., d2 = 0.;
        for (int n = m; n <= K; n++) {
            const double an = pw[n - 1];
            const int mn = n * (n - 1) / 2 + m - 1;
            const double e = g[mn];
            const double hh = h[mn];
            const double w = e * sm + hh * cm;
            br = br + pwn[n - 1] * w * q;
            bt = bt - an * w * zz;
            if (m != 1) {
                const double qq = pole ? zz : q;
                bi = bi + an * (e * cm - hh * sm) * qq;
            }
            const double xk = rec[mn];
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
    *bx = he * cf - bphi * sf;
    *by = he * sf + bphi * cf;
    *bz = br * C - bt * S;
}

int64_t orc_internal_geo_flops(double R) {
    /* Operation count of orc_internal_geo off the pole, counting + - * / sqrt
     * as one each: set-up 12, power table 2 per n, 6 per m column for the
     * sin/cos recursion (m>1), 4 per column update, 2 per column for bi (m>1),
     * 23 per (n,m) term with m>1 and 17 with m=1, 13 for the components. */
    const int K = o_internal_degree(R) + 1;
    int64_t f = 12 + 2 * K + 13;
    for (int m = 1; m <= K; m++) {
        const int terms = K - m + 1;
        f += 4;                                   /* dmm, pmm */
        if (m != 1) f += 6 + 2 + terms * 23;
        else f += terms * 17;
    }
    return f;
}

/* ---- field composition: src/models.c:146-207 -------------------------- */
static const double *g_crust_g = NULL, *g_crust_h = NULL;
static int g_crust_nmax = 0;

void orc_set_crustal_table(const double *g, const double *h, int nmax) {
    g_crust_g = g; g_crust_h = h; g_crust_nmax = nmax;
}

void orc_calculate_field(const double gsm_pos[3], cor_model_set models,
                         const cor_model_params *p, double geo_field[3]) {
    const double pos[3] = { gsm_pos[0] / O_RE, gsm_pos[1] / O_RE, gsm_pos[2] / O_RE };
    double tot[3] = { 0., 0., 0. };
    if (models.internal_model == COR_INTERNAL_SH) {
        /* internal_calc, src/models.c:146-160 */
        double geo[3], bg[3], bs[3];
        o_gsm_to_geo(pos, geo, p);
        orc_internal_geo(geo[0], geo[1], geo[2], p->g, p->h, p->rec, &bg[0], &bg[1], &bg[2]);
        o_geo_to_gsm(bg, bs, p);
        tot[0] += bs[0]; tot[1] += bs[1]; tot[2] += bs[2];
    }
    if (models.external_model == COR_EXTERNAL_T96) {
        /* t96_calc, src/models.c:171-177 */
        double b[3];
        orc_t96_gsm(p->parmod, pos[0], pos[1], pos[2], &b[0], &b[1], &b[2]);
        tot[0] += b[0]; tot[1] += b[1]; tot[2] += b[2];
    } else if (models.external_model == COR_EXTERNAL_TS05) {
        /* ts05_calc, src/models.c:162-169 */
        double b[3];
        orc_ts05_gsm(p->parmod, pos[0], pos[1], pos[2], &b[0], &b[1], &b[2]);
        tot[0] += b[0]; tot[1] += b[1]; tot[2] += b[2];
    }
    if (models.crustal_model == COR_CRUSTAL_CHAOS && g_crust_g) {
        /* chaos_7_16_calc, src/models.c:179-192 */
        double geo[3], bg[3], bs[3];
        o_gsm_to_geo(pos, geo, p);
        orc_chaos_geo(geo[0], geo[1], geo[2], g_crust_g, g_crust_h, g_crust_nmax, &bg[0], &bg[1], &bg[2]);
        o_geo_to_gsm(bg, bs, p);
        tot[0] += bs[0]; tot[1] += bs[1]; tot[2] += bs[2];
    }
    o_gsm_to_geo(tot, geo_field, p);
}

/* ---- RK step: src/trajectory.c:275-356 -------------------------------- */
/* Velocity: dv/dt = d (v x B) with B frozen, six stages with the weights
 * (23, 0, 125, 0, -81, 125)/192.  Position: the same tableau applied to h*v. */
void orc_rk_step(double h, double d, const double f[3], double vel[3], double pos[3]) {
    const double vx = vel[0], vy = vel[1], vz = vel[2];
    const double fx = f[0], fy = f[1], fz = f[2];
#define CROSS_X(Y, Z) (h * (d * ((Y) * fz - (Z) * fy)))
#define CROSS_Y(X, Z) (h * (d * ((Z) * fx - (X) * fz)))
#define CROSS_Z(X, Y) (h * (d * ((X) * fy - (Y) * fx)))
    const double a1 = CROSS_X(vy, vz), b1 = CROSS_Y(vx, vz), c1 = CROSS_Z(vx, vy);
    /* stage 2: v + k1/3 */
    const double sx2 = vx + a1 / 3., sy2 = vy + b1 / 3., sz2 = vz + c1 / 3.;
    const double a2 = CROSS_X(sy2, sz2), b2 = CROSS_Y(sx2, sz2), c2 = CROSS_Z(sx2, sy2);
    /* stage 3: v + (4 k1 + 6 k2)/25 */
    const double sx3 = vx + (4. * a1 + 6. * a2) / 25.;
    const double sy3 = vy + (4. * b1 + 6. * b2) / 25.;
    const double sz3 = vz + (4. * c1 + 6. * c2) / 25.;
    const double a3 = CROSS_X(sy3, sz3), b3 = CROSS_Y(sx3, sz3), c3 = CROSS_Z(sx3, sy3);
    /* stage 4: v + (k1 - 12 k2 + 15 k3)/4 */
    const double sx4 = vx + (a1 - 12. * a2 + 15. * a3) / 4.;
    const double sy4 = vy + (b1 - 12. * b2 + 15. * b3) / 4.;
    const double sz4 = vz + (c1 - 12. * c2 + 15. * c3) / 4.;
    const double a4 = CROSS_X(sy4, sz4), b4 = CROSS_Y(sx4, sz4), c4 = CROSS_Z(sx4, sy4);
    /* stage 5: v + (6 k1 + 90 k2 - 50 k3 + 8 k4)/81 */
    const double sx5 = vx + (6. * a1 + 90. * a2 - 50. * a3 + 8. * a4) / 81.;
    const double sy5 = vy + (6. * b1 + 90. * b2 - 50. * b3 + 8. * b4) / 81.;
    const double sz5 = vz + (6. * c1 + 90. * c2 - 50. * c3 + 8. * c4) / 81.;
    const double a5 = CROSS_X(sy5, sz5), b5 = CROSS_Y(sx5, sz5), c5 = CROSS_Z(sx5, sy5);
    /* stage 6: v + (6 k1 + 36 k2 + 10 k3 + 8 k4)/75 */
    const double sx6 = vx + (6. * a1 + 36. * a2 + 10. * a3 + 8. * a4) / 75.;
    const double sy6 = vy + (6. * b1 + 36. * b2 + 10. * b3 + 8. * b4) / 75.;
    const double sz6 = vz + (6. * c1 + 36. * c2 + 10. * c3 + 8. * c4) / 75.;
    const double a6 = CROSS_X(sy6, sz6), b6 = CROSS_Y(sx6, sz6), c6 = CROSS_Z(sx6, sy6);
#undef CROSS_X
#undef CROSS_Y
#undef CROSS_Z
    /* position stages on the unrotated velocity (:331-348) */
    double pk[3][6];
    const double vv[3] = { vx, vy, vz };
    for (int c = 0; c < 3; c++) {
        const double k1 = h * vv[c];
        const double k2 = h * (vv[c] + k1 / 3.);
        const double k3 = h * (vv[c] + (4. * k1 + 6. * k2) / 25.);
        const double k4 = h * (vv[c] + (k1 - 12. * k2 + 15. * k3) / 4.);
        const double k5 = h * (vv[c] + (6. * k1 + 90. * k2 - 50. * k3 + 8. * k4) / 81.);
        const double k6 = h * (vv[c] + (6. * k1 + 36. * k2 + 10. * k3 + 8. * k4) / 75.);
        pk[c][0] = k1; pk[c][2] = k3; pk[c][4] = k5; pk[c][5] = k6;
    }
    vel[0] += (23. * a1 + 125. * a3 - 81. * a5 + 125. * a6) / 192.;
    vel[1] += (23. * b1 + 125. * b3 - 81. * b5 + 125. * b6) / 192.;
    vel[2] += (23. * c1 + 125. * c3 - 81. * c5 + 125. * c6) / 192.;
    for (int c = 0; c < 3; c++)
        pos[c] += (23. * pk[c][0] + 125. * pk[c][2] - 81. * pk[c][4] + 125. * pk[c][5]) / 192.;
}

/* ---- scan: src/trajectory.c:6-161 ------------------------------------- */
static int64_t o_n_rig(const cor_scan_job *job) {
    return (int64_t)(int)round((job->rk - job->rig) / job->del) + 1;  /* :7,12 */
}

/* Indices traced: the whole grid, or the window i_first .. i_first+i_count-1
 * of it (cor_trace.h); -1 for an invalid window. */
static int64_t o_n_traced(const cor_scan_job *job) {
    const int64_t n = o_n_rig(job);
    if (job->i_first < 0 || job->i_count < 0 || job->i_first >= n) return -1;
    const int64_t m = job->i_count ? job->i_count : n - job->i_first;
    return job->i_first + m > n ? -1 : m;
}

/* One trajectory, src/trajectory.c:13-153.  Returns the COR_TRAJ_* class. */
static int o_trace_one(const cor_scan_job *job, const cor_model_params *p, cor_model_set models,
                       uint64_t step_limit, double tu_angle, double mass, double rig,
                       cor_traj_record *rec, cor_step_record *steps, uint32_t step_cap) {
    int nk0 = job->nk1;
    double alength = 0., time = 0.;
    const double a = rig * 1.0e+09 * job->zn * O_Q / (mass * O_C * O_C);
    const double vr0 = O_C * sqrt(1. - 1. / (1. + a * a));
    double pos[3], vel[3], gsm[3], field[3];
    o_sph_to_car(job->r0 * O_RE, (90. - job->the0) * O_TO_RAD, job->fi0 * O_TO_RAD, pos);
    o_geo_to_gsm(pos, gsm, p);
    orc_calculate_field(gsm, models, p, field);
    double b = 1.E-09 * sqrt(field[0] * field[0] + field[1] * field[1] + field[2] * field[2]);
    o_sph_to_car(vr0, (90. - job->the1) * O_TO_RAD, job->fi1 * O_TO_RAD, vel);
    double v = vr0;
    unsigned int step = 0;
    uint32_t trials = 0;
    int status;

    for (;;) {
        step++;
        const double vc = v / O_C;
        if (vc > 1.) { status = COR_TRAJ_SUPERLUM; break; }            /* :48-54 */
        const double hm = mass / sqrt(1. - vc * vc);                   /* :56-60 */
        const double t = (2. * O_PI * hm) / (fabs(job->zn) * O_Q * b);
        const double h = t / nk0;
        const double d = (1.E-09 * job->zn * O_Q) / hm;
        const double prev_pos[3] = { pos[0], pos[1], pos[2] };
        const double prev_vel[3] = { vel[0], vel[1], vel[2] };
        const double vprev = v;
        orc_rk_step(h, d, field, vel, pos);                            /* :65 */
        trials++;
        v = sqrt(vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
        const double gc = (vel[0] * prev_vel[0] + vel[1] * prev_vel[1] + vel[2] * prev_vel[2]) / (v * vprev);
        if (gc < 1.) {                                                 /* :69-79 */
            const double gs = sqrt((1. - gc) * (1. + gc));
            const double gu = atan2(gs, gc);
            if (gu >= tu_angle && nk0 <= 50000) {
                nk0 *= 2;
                memcpy(pos, prev_pos, sizeof pos);
                memcpy(vel, prev_vel, sizeof vel);
                step--;
                continue;
            }
        }
        double sph[3];
        o_car_to_sph(pos, sph);                                        /* :81-82 */
        o_geo_to_gsm(pos, gsm, p);
        const double pax = (gsm[0] / O_RE + 25.3) / 36.08;             /* :84-87 */
        const double paz = (gsm[1] * gsm[1] + gsm[2] * gsm[2]) / (O_RE * O_RE);
        const double r = sph[0] / O_RE;
        const double paus = pax * pax + paz / 459.6736;
        if (r >= 25. || paus > 1.) {                                   /* :89-131 */
            if ((r >= 25. && fabs(r - 25.) < 0.002) || (r <= 25. && paus > 1. && fabs(paus - 1.) < 0.002)) {
                status = COR_TRAJ_ALLOWED;
                break;
            }
            if (nk0 >= O_NK0_CAP) { status = COR_TRAJ_WATCHDOG; break; }
            nk0 *= 2;
            memcpy(pos, prev_pos, sizeof pos);
            memcpy(vel, prev_vel, sizeof vel);
            step--;
            continue;
        }
        if (r < 1.) { status = COR_TRAJ_REENTRY; break; }              /* :133-138 */
        if (step > step_limit || sph[2] > 31.4) {                      /* :140-145 */
            status = COR_TRAJ_STEP_LIMIT;
            break;
        }
        orc_calculate_field(gsm, models, p, field);                    /* :147-148 */
        b = 1.E-09 * sqrt(field[0] * field[0] + field[1] * field[1] + field[2] * field[2]);
        time = time + t / nk0;                                         /* :150-152 */
        alength += sqrt((pos[0] - prev_pos[0]) * (pos[0] - prev_pos[0]) +
                        (pos[1] - prev_pos[1]) * (pos[1] - prev_pos[1]) +
                        (pos[2] - prev_pos[2]) * (pos[2] - prev_pos[2]));
        if (steps && step <= step_cap) {                               /* trajectory mode, :254-258 */
            cor_step_record *o = &steps[step - 1];
            memcpy(o->gsm, gsm, sizeof gsm);
            memcpy(o->pos, pos, sizeof pos);
            o->v = v;
            o->time = time;
            o->length = alength;
            o->step = step;
            o->reserved = 0;
        }
        nk0 = job->nk1;
    }
    if (rec) {
        memcpy(rec->pos, pos, sizeof pos);
        memcpy(rec->vel, vel, sizeof vel);
        rec->v = v;
        rec->time = time;
        rec->length = alength;
        rec->steps = (status == COR_TRAJ_ALLOWED) ? step - 1 : step;
        rec->trials = trials;
        rec->status = status;
        rec->reserved = 0;
    }
    return status;
}

/* The reduction of src/trajectory.c:156-160 over the classes of one scan's
 * traced trajectories (status[0..n-1] = grid indices i_first..), in ascending
 * rigidity, i.e. the reference's serial result (its OpenMP fmin/fmax). */
static void o_reduce_job(const cor_scan_job *job, const uint8_t *status, int64_t n, cor_site_result *site) {
    int nza = job->i_first;  /* a window's untraced lower indices count as forbidden */
    double rmx1 = 0., rmx2 = 0., rmi = job->rk;                        /* :8-9 */
    for (int64_t k = 0; k < n; k++) {
        const int64_t i = job->i_first + k;
        const double rig = job->rig + i * job->del;                    /* :14 */
        const int st = status[k];
        if (st == COR_TRAJ_ALLOWED) {
            rmi = fmin(rmi, rig);                                      /* :115 */
        } else if (st == COR_TRAJ_REENTRY || st == COR_TRAJ_SUPERLUM) {
            nza += 1;
            rmx1 = fmax(rmx1, rig);                                    /* :52,136 */
        } else {
            nza += 1;
            rmx2 = fmax(rmx2, rig);                                    /* :143 */
        }
    }
    double rmx = fmax(rmx1, rmx2);                                     /* :156-159 */
    const double zan = nza - (rmi - job->rig) / job->del;
    const double rms = rmi + zan * job->del;
    rmx = rmx + job->del;
    site->r_lower = rmi;
    site->r_upper = rmx;
    site->r_cutoff = rms;
    site->n_forbidden = nza;
    site->n_traj = (int32_t)n;
}

int orc_scan_job(const cor_scan_job *job, const cor_model_params *params, cor_model_set models,
                 uint64_t step_limit, double tu_angle, double particle_mass,
                 cor_site_result *site, uint8_t *status, cor_traj_record *records,
                 cor_counters *counters) {
    if (!(job->del > 0.)) return COR_ERR_INVALID;
    const int64_t n = o_n_traced(job);
    if (n < 0) return COR_ERR_INVALID;
    uint8_t *st_buf = status ? status : (uint8_t *)malloc(n > 0 ? (size_t)n : 1);
    if (!st_buf) return COR_ERR_NOMEM;
    uint64_t steps = 0, trials = 0, wd = 0;
    for (int64_t k = 0; k < n; k++) {
        const double rig = job->rig + (job->i_first + k) * job->del;  /* :14 */
        cor_traj_record r;
        const int st = o_trace_one(job, params, models, step_limit, tu_angle, particle_mass, rig, &r, NULL, 0);
        wd += st == COR_TRAJ_WATCHDOG;
        steps += r.steps;
        trials += r.trials;
        st_buf[k] = (uint8_t)st;
        if (records) records[k] = r;
    }
    if (site) o_reduce_job(job, st_buf, n, site);
    if (st_buf != status) free(st_buf);
    if (counters) {
        counters->accepted_steps += steps;
        counters->trials += trials;
        counters->trajectories += (uint64_t)n;
        counters->watchdog += wd;
    }
    return COR_OK;
}

/* ---- batch over host threads ------------------------------------------ */
/* Work items are chunks of ORC_CHUNK consecutive rigidities of one scan,
 * handed out from a shared counter in scan order: every host thread stays
 * busy until the batch's last chunk, as the reference's schedule(dynamic,1)
 * over the rigidities of a scan keeps its team busy (src/trajectory.c:11).
 * The per-scan reductions run after every chunk has finished. */
#define ORC_CHUNK 4

typedef struct {
    const cor_batch_req *req;
    const uint64_t *offsets;
    const uint64_t *chunk_off;   /* n_jobs + 1 prefix of chunks per scan */
    uint8_t *status;
    cor_traj_record *records;
    uint64_t next;
    pthread_mutex_t lock;
    cor_counters total;
    int err;
} o_pool;

static void *o_worker(void *arg) {
    o_pool *pl = (o_pool *)arg;
    const int32_t nj = pl->req->n_jobs;
    cor_counters local = { 0, 0, 0, 0, 0 };
    int j = 0;
    for (;;) {
        const uint64_t c = __atomic_fetch_add(&pl->next, 1, __ATOMIC_RELAXED);
        if (c >= pl->chunk_off[nj]) break;
        while (pl->chunk_off[j + 1] <= c) j++;   /* a thread's claims only ever move forward */
        const cor_scan_job *job = &pl->req->jobs[j];
        const uint64_t n = pl->offsets[j + 1] - pl->offsets[j];
        const uint64_t k0 = (c - pl->chunk_off[j]) * ORC_CHUNK;
        const uint64_t k1 = k0 + ORC_CHUNK < n ? k0 + ORC_CHUNK : n;
        const cor_model_params *par = &pl->req->params[job->param_index];
        for (uint64_t k = k0; k < k1; k++) {
            const double rig = job->rig + (int64_t)(job->i_first + (int64_t)k) * job->del;  /* :14 */
            cor_traj_record r;
            const int st = o_trace_one(job, par, pl->req->models, pl->req->step_limit, pl->req->tu_angle,
                                       pl->req->particle_mass, rig, &r, NULL, 0);
            pl->status[pl->offsets[j] + k] = (uint8_t)st;
            if (pl->records) pl->records[pl->offsets[j] + k] = r;
            local.accepted_steps += r.steps;
            local.trials += r.trials;
            local.trajectories += 1;
            local.watchdog += st == COR_TRAJ_WATCHDOG;
        }
    }
    pthread_mutex_lock(&pl->lock);
    pl->total.accepted_steps += local.accepted_steps;
    pl->total.trials += local.trials;
    pl->total.trajectories += local.trajectories;
    pl->total.watchdog += local.watchdog;
    pthread_mutex_unlock(&pl->lock);
    return NULL;
}

int orc_scan_batch(const cor_batch_req *req, const uint64_t *offsets, int threads,
                   cor_site_result *sites, uint8_t *status, cor_traj_record *records,
                   cor_counters *counters) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    const int32_t nj = req->n_jobs;
    for (int32_t j = 0; j < nj; j++) {
        const cor_scan_job *job = &req->jobs[j];
        if (job->param_index < 0 || job->param_index >= req->n_params || !(job->del > 0.) ||
            o_n_traced(job) != (int64_t)(offsets[j + 1] - offsets[j]))
            return COR_ERR_INVALID;
    }
    uint64_t *chunk_off = (uint64_t *)malloc(sizeof(uint64_t) * ((size_t)nj + 1));
    uint8_t *st_buf = status ? status : (uint8_t *)malloc(offsets[nj] > 0 ? (size_t)offsets[nj] : 1);
    if (!chunk_off || !st_buf) {
        free(chunk_off);
        if (st_buf != status) free(st_buf);
        return COR_ERR_NOMEM;
    }
    chunk_off[0] = 0;
    for (int32_t j = 0; j < nj; j++)
        chunk_off[j + 1] = chunk_off[j] + (offsets[j + 1] - offsets[j] + ORC_CHUNK - 1) / ORC_CHUNK;
    o_pool pl;
    memset(&pl, 0, sizeof pl);
    pl.req = req; pl.offsets = offsets; pl.chunk_off = chunk_off; pl.status = st_buf; pl.records = records;
    pthread_mutex_init(&pl.lock, NULL);
    pthread_t tid[1024];
    int started = 0;
    for (int t = 1; t < threads; t++)
        if (pthread_create(&tid[started], NULL, o_worker, &pl) == 0) started++;
    o_worker(&pl);
    for (int t = 0; t < started; t++) pthread_join(tid[t], NULL);
    pthread_mutex_destroy(&pl.lock);
    if (sites)
        for (int32_t j = 0; j < nj; j++)
            o_reduce_job(&req->jobs[j], st_buf + offsets[j], (int64_t)(offsets[j + 1] - offsets[j]), &sites[j]);
    free(chunk_off);
    if (st_buf != status) free(st_buf);
    if (counters) *counters = pl.total;
    return pl.err;
}

/* trajectory_simulation (src/trajectory.c:163-273) for the first traced
 * rigidity of a job: every accepted step into steps[0 .. step_cap-1]; returns
 * the number recorded (or a negative COR_ERR_*). */
int orc_trace_steps(const cor_scan_job *job, const cor_model_params *params, cor_model_set models,
                    uint64_t step_limit, double tu_angle, double particle_mass,
                    cor_step_record *steps, uint32_t step_cap, cor_traj_record *rec) {
    if (!(job->del > 0.) || o_n_traced(job) < 1) return COR_ERR_INVALID;
    const double rig = job->rig + (int64_t)job->i_first * job->del;
    cor_traj_record r;
    memset(steps, 0, sizeof(cor_step_record) * step_cap);
    o_trace_one(job, params, models, step_limit, tu_angle, particle_mass, rig, &r, steps, step_cap);
    if (rec) *rec = r;
    uint32_t n = 0;
    while (n < step_cap && steps[n].step == n + 1) n++;
    return (int)n;
}
