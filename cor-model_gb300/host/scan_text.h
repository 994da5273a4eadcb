/*
 * scan_text.h -- the text of one rigidity scan as trajectory_simulation_cutoff
 * prints it (src/trajectory.c:81-122 for an allowed row, :160 for the CUTOFF
 * line), from the records libcortrace returns.  The angles are taken with the
 * host C library, as the reference does, so the text equals the reference's
 * wherever the final states do.  Shared by the drop-in `cor` program
 * (cli_scan.c) and the link-in replacement of the reference's own function
 * (trajectory_shim.c); it names nothing of either program's types.
 */
#ifndef COR_SCAN_TEXT_H
#define COR_SCAN_TEXT_H

#include <math.h>
#include <stdio.h>

#include "../../include/cor_trace.h"

/* the legacy-truncated constants of src/common.h:4-11 */
#define COR_TXT_PI 3.141592654
#define COR_TXT_2PI 6.28318531
#define COR_TXT_RE 6.3712e+06
#define COR_TXT_TO_RAD (COR_TXT_PI / 180.)
#define COR_TXT_C 2.99725e+08

/* car_to_sph, src/utils.c:43-73 */
static inline void cor_txt_car_to_sph(const double car[3], double sph[3]) {
    const double x = car[0], y = car[1], z = car[2];
    const double sq = x * x + y * y;
    const double r = sqrt(sq + z * z);
    if (sq != 0.) {
        double phi = atan2(y, x);
        const double theta = atan2(sqrt(sq), z);
        if (phi < 0.) phi += COR_TXT_2PI;
        sph[0] = r; sph[1] = theta; sph[2] = phi;
        return;
    }
    sph[0] = r;
    sph[1] = z < 0. ? COR_TXT_PI : 0.;
    sph[2] = 0.;
}

/* One allowed row, src/trajectory.c:81-122. */
static inline void cor_txt_allowed_row(FILE *out, double rig, const cor_traj_record *r) {
    double sph[3];
    cor_txt_car_to_sph(r->pos, sph);
    const double rr = sph[0] / COR_TXT_RE;
    const double td = 90. - (sph[1] / COR_TXT_TO_RAD);
    const double fei = sph[2] / COR_TXT_TO_RAD;
    const double s = sin(sph[1]), c = cos(sph[1]), sf = sin(sph[2]), cf = cos(sph[2]);
    const double be = r->vel[0] * cf + r->vel[1] * sf;
    const double vr = be * s + r->vel[2] * c;
    const double vt = be * c - r->vel[2] * s;
    const double vp = -r->vel[0] * sf + r->vel[1] * cf;
    const double va = vt * c + vr * s;
    const double dm = sqrt(vt * vt + va * va);
    const double ast = atan2(-vt * s + vr * c, dm) / COR_TXT_TO_RAD;
    double asf = (sph[2] + atan2(vp, va)) / COR_TXT_TO_RAD;
    if (asf > 360.) asf -= 360.;
    fprintf(out, "%10.6f%15.10f%12.6f%10.3f%10.3f%10.3f%10.3f%12.6f%16.2f\n", rig, r->v / COR_TXT_C, rr, td, fei, ast,
            asf, r->time, r->length / 1000.);
}

/* The allowed rows in ascending rigidity, then the CUTOFF line (:160) of a
 * scan over rig + i*del, i = 0 .. n-1.  Returns 0, or -1 if a write failed. */
static inline int cor_txt_scan(FILE *out, double rig, double del, int64_t n, const cor_site_result *site,
                               const uint8_t *status, const cor_traj_record *records) {
    for (int64_t i = 0; i < n; i++)
        if (status[i] == COR_TRAJ_ALLOWED) cor_txt_allowed_row(out, rig + (int)i * del, &records[i]);
    return fprintf(out, "  CUTOFF with rigidities P(S),P(C),P(M) are:\n%12.5f%12.5f%12.5f\n\n", site->r_lower,
                   site->r_upper, site->r_cutoff) < 0
               ? -1
               : 0;
}

#endif /* COR_SCAN_TEXT_H */
