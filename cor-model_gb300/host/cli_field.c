/*
 * cli_field.c -- `cor -m field` (src/field.c:6-53): the field on a
 * latitude/longitude grid at one radius, evaluated on the GPU in one
 * cor_field_batch call.
 *
 * The grid and its quirks are the reference's: rows j = 0 .. n_the
 * (inclusive), columns i = 0 .. n_phi - 1 (exclusive), n = (int)(span/step),
 * a zero step giving a single row or no columns.  Start positions are made on
 * the host with the C library (sph_to_car, src/utils.c:28-41) and rotated to
 * GSM with the reference's expression order (geo_to_gsm, :75-87), so the
 * device evaluates calculate_field at the reference's points; rows are
 * printed in the reference's order and format.
 */
#include <math.h>
#include <stdlib.h>

#include "cli.h"

int field_simulation(const InfileHeader *h, const ModelsParams *p, const Model **models, FILE *out) {
    const double del_the = h->the1 - h->the0, del_phi = h->fi1 - h->fi0;
    int n_the = 0, n_phi = 0;
    if (h->lat_step > 0.) n_the = (int)(del_the / h->lat_step);
    if (h->lon_step > 0.) n_phi = (int)(del_phi / h->lon_step);
    if (n_the < 0 || n_phi <= 0) return 0;
    const int64_t n = (int64_t)(n_the + 1) * n_phi;
    double *gsm = malloc(sizeof(double) * 3 * (size_t)n);
    double *geo = malloc(sizeof(double) * 3 * (size_t)n);
    double *lat = malloc(sizeof(double) * (size_t)n);
    double *lon = malloc(sizeof(double) * (size_t)n);
    if (!gsm || !geo || !lat || !lon) {
        fprintf(stderr, "Error: out of memory\n");
        return 1;
    }
    const double r = h->r0 * DEF_RE;
    int64_t k = 0;
    for (int j = 0; j <= n_the; j++) {
        const double the0a = h->the0 + (double)(j * h->lat_step);
        for (int i = 0; i < n_phi; i++, k++) {
            const double phi0a = h->fi0 + (double)(i * h->lon_step);
            const double theta = (90. - the0a) * DEF_TO_RAD, phi = phi0a * DEF_TO_RAD;
            const double sq = r * sin(theta);
            const double x = sq * cos(phi), y = sq * sin(phi), z = r * cos(theta);
            gsm[3 * k + 0] = p->a1[0] * x + p->a1[1] * y + p->a1[2] * z;
            gsm[3 * k + 1] = p->a2[0] * x + p->a2[1] * y + p->a2[2] * z;
            gsm[3 * k + 2] = p->a3[0] * x + p->a3[1] * y + p->a3[2] * z;
            lat[k] = the0a;
            lon[k] = phi0a;
        }
    }
    cor_ctx *ctx;
    int rc = cli_context(&ctx);
    if (rc == COR_OK) rc = cor_field_batch(ctx, models_device_set(models), p, 1, NULL, gsm, n, geo);
    if (rc != COR_OK) {
        fprintf(stderr, "Error: field evaluation failed: %s\n", cor_last_error_string(ctx));
        free(gsm); free(geo); free(lat); free(lon);
        return 1;
    }
    for (k = 0; k < n; k++) {
        const double bx = geo[3 * k], by = geo[3 * k + 1], bz = geo[3 * k + 2];
        const double b = sqrt(bx * bx + by * by + bz * bz);
        fprintf(out, "%9.2f%9.2f%11.2f%11.2f%11.2f%11.2f\n", lat[k], lon[k], b, bx, by, bz);
    }
    free(gsm); free(geo); free(lat); free(lon);
    return 0;
}
