/*
 * sanitize_harness.c -- TEST INFRASTRUCTURE: drives the host-side C of
 * libcortrace (model set-up, INFILE parsing, model registry) and the C oracle
 * under AddressSanitizer and UndefinedBehaviorSanitizer (tests/test_sanitize.py
 * builds and runs it); any sanitizer report, or a wrong return code, fails.
 * It includes malformed inputs: truncated INFILEs, dates outside every
 * coefficient table, missing external-field parameter lines.
 */
#define _GNU_SOURCE
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../cor-model_gb300/host/cli.h"
#include "../cor-model_gb300/host/coef_tables.h"
#include "../oracle/cor_oracle.h"

static int failures = 0;
#define CHECK(cond, ...)                      \
    do {                                      \
        if (!(cond)) {                        \
            fprintf(stderr, __VA_ARGS__);     \
            fputc('\n', stderr);              \
            failures++;                       \
        }                                     \
    } while (0)

static FILE *mem(const char *text) { return fmemopen((void *)text, strlen(text), "r"); }

int main(void) {
    cor_model_params p;
    /* 1. set-up of every internal model at dates inside, at the ends of and
     * outside its table */
    for (int k = 0; k < cor_sh_table_count; k++) {
        const cor_sh_table *t = &cor_sh_tables[k];
        const int years[5] = {t->min_year, (t->min_year + t->max_year) / 2, t->max_year, t->max_year + 3,
                              t->min_year - 50};
        for (int y = 0; y < 5; y++) {
            const int32_t tm[7] = {years[y], 6, 21, 173, 12, 0, 0};
            memset(&p, 0, sizeof p);
            const int rc = cor_internal_setup(t->version, tm, &p);
            CHECK(rc == COR_OK || rc == COR_ERR_RANGE, "%s %d: set-up returned %d", t->version, years[y], rc);
        }
    }
    const int32_t tm[7] = {2020, 6, 21, 173, 12, 0, 0};
    CHECK(cor_internal_setup("no-such-model", tm, &p) != COR_OK, "unknown model accepted");
    CHECK(cor_gsm_setup(tm, &p) == COR_OK, "GSM set-up failed");

    /* 2. INFILE parsing: valid and truncated cutoff and field headers */
    InfileHeader h;
    FILE *f = mem("0.05 1 20\n1.0031391260673028 50 15\n50 15\n2020 1 1 1 0 0 0\n100 0 0 0.05\n");
    CHECK(read_cutoff_infile_header(f, &h) == 0 && h.del == 0.05 && h.nk1 == 100, "cutoff header");
    fclose(f);
    f = mem("");
    CHECK(read_cutoff_infile_header(f, &h) != 0, "empty cutoff INFILE accepted");
    fclose(f);
    f = mem("0.05 1 20\n1.0031391260673028 50 15\n50 15\n2020 1 1\n");
    CHECK(read_cutoff_infile_header(f, &h) != 0, "cutoff header cut short accepted");
    fclose(f);
    f = mem("1.0 -90 0\n10 10 90\n");
    CHECK(read_field_infile_header(f, &h) != 0, "field header cut short accepted");
    fclose(f);
    f = mem("1.0 -90 0\n10 10 90 360\n2020 1 1 1 0 0 0\n");
    CHECK(read_field_infile_header(f, &h) == 0 && h.lat_step == 10. && h.fi1 == 360., "field header");
    fclose(f);

    /* 3. the model registry: set-up with and without the external lines */
    const Model *t96 = get_model(external_models, "t96");
    const Model *ts05 = get_model(external_models, "ts05");
    const Model *igrf = get_model(internal_models, "igrf14");
    CHECK(t96 && ts05 && igrf && !get_model(external_models, "t01"), "model registry");
    const Model *m1[3] = {igrf, t96, NULL};
    h.iy = 2020; h.mes = 6; h.ide = 21; h.id = 173; h.ih = 12; h.min = 0; h.is = 0;
    f = mem("-20 2 0 -1\n");
    CHECK(models_setup(m1, f, &h, &p) == 0 && p.parmod[0] == 2. && p.parmod[1] == -20., "T96 parameters");
    fclose(f);
    f = mem("-20 2\n");
    CHECK(models_setup(m1, f, &h, &p) != 0, "truncated T96 parameters accepted");
    fclose(f);
    const Model *m2[2] = {ts05, NULL};        /* external model alone: GSM axes from the date */
    f = mem("-20 2 0 -1\n1 1 1 1 1 1\n");
    CHECK(models_setup(m2, f, &h, &p) == 0 && p.parmod[9] == 1., "TS05 parameters");
    fclose(f);

    /* 4. the oracle: short scans with every external model, the crustal field */
    cor_model_params q;
    CHECK(cor_internal_setup("igrf14", tm, &q) == COR_OK, "igrf14 set-up");
    q.parmod[0] = 2.; q.parmod[1] = -20.; q.parmod[2] = 0.; q.parmod[3] = -1.;
    for (int k = 4; k < 10; k++) q.parmod[k] = 1.;
    cor_scan_job job;
    memset(&job, 0, sizeof job);
    job.r0 = 1.0031391260673028; job.the0 = 40.; job.fi0 = 20.; job.the1 = 40.; job.fi1 = 20.;
    job.rig = 6.; job.del = 1.; job.rk = 9.; job.zn = 1.; job.nk1 = 100;
    for (int ext = 0; ext <= 2; ext++) {
        cor_model_set ms = {COR_INTERNAL_SH, ext, COR_CRUSTAL_NONE, 0};
        cor_site_result site;
        uint8_t status[4];
        cor_traj_record rec[4];
        cor_counters c;
        memset(&c, 0, sizeof c);
        const int rc = orc_scan_job(&job, &q, ms, 3000, 0.01, 1.6725e-27, &site, status, rec, &c);
        CHECK(rc == COR_OK && site.n_traj == 4, "oracle scan with external model %d: %d", ext, rc);
    }
    job.i_first = 1; job.i_count = 2;          /* a window of the grid */
    {
        cor_model_set ms = {COR_INTERNAL_SH, COR_EXTERNAL_T96, COR_CRUSTAL_NONE, 0};
        cor_site_result site;
        uint8_t status[2];
        CHECK(orc_scan_job(&job, &q, ms, 3000, 0.01, 1.6725e-27, &site, status, NULL, NULL) == COR_OK &&
                  site.n_traj == 2, "oracle window scan");
        job.i_count = 9;                       /* past the end of the grid */
        CHECK(orc_scan_job(&job, &q, ms, 3000, 0.01, 1.6725e-27, &site, status, NULL, NULL) != COR_OK,
              "window past the grid accepted");
        job.i_first = 0; job.i_count = 0;
        cor_step_record steps[16];              /* far fewer than the trajectory's steps: truncated */
        cor_traj_record rec;
        const int n = orc_trace_steps(&job, &q, ms, 3000, 0.01, 1.6725e-27, steps, 16, &rec);
        CHECK(n == 16 && steps[15].step == 16, "step records truncated at the capacity: %d", n);
    }
    {
        const int nmax = cor_chaos716.nmax;
        double *G = calloc((size_t)nmax * nmax, sizeof(double)), *H = calloc((size_t)nmax * nmax, sizeof(double));
        for (int n = 0; n < nmax; n++)
            for (int m = 0; m <= n; m++) {
                G[n * nmax + m] = cor_chaos716.g[n * (n + 1) / 2 + m];
                H[n * nmax + m] = cor_chaos716.h[n * (n + 1) / 2 + m];
            }
        double bx, by, bz;
        orc_chaos_geo(1.2, 0.3, -0.4, G, H, nmax, &bx, &by, &bz);
        CHECK(bx == bx && by == by && bz == bz, "CHAOS field is NaN");
        free(G);
        free(H);
    }
    if (failures) {
        fprintf(stderr, "%d check(s) failed\n", failures);
        return 1;
    }
    printf("sanitize ok\n");
    return 0;
}
