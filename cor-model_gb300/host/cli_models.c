/*
 * cli_models.c -- the model registry of src/models.c:22-144 for the device
 * path: the same names, versions and lookup order; set-up goes through
 * cor_internal_setup (internal_recalc) and the PARMOD readers of cli_io.c.
 */
#include <string.h>

#include "cli.h"

static const Model igrf_14 = { "IGRF-14", "igrf14", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model igrf_13 = { "IGRF-13", "igrf13", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model igrf_12 = { "IGRF-12", "igrf12", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model igrf_11 = { "IGRF-11", "igrf11", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model igrf_10 = { "IGRF-10", "igrf10", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model igrf_9 = { "IGRF-9", "igrf9", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model hist = { "Historical (0-1968 CE)", "hist", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model cals10k_2 = { "Historical (CALS10k.2)", "cals10k.2", MODEL_INTERNAL, COR_INTERNAL_SH, 0 };
static const Model ts_05 = { "Tsyganenko-Sitnov 05", "ts05", MODEL_EXTERNAL, COR_EXTERNAL_TS05, 10 };
static const Model t_96 = { "Tsyganenko 96", "t96", MODEL_EXTERNAL, COR_EXTERNAL_T96, 4 };
static const Model chaos_7_16 = { "CHAOS-7.16", "chaos7.16", MODEL_CRUSTAL, COR_CRUSTAL_CHAOS, 0 };

/* src/models.c:110-112 */
const Model *internal_models[] = { &igrf_14, &igrf_13, &igrf_12, &igrf_11, &igrf_10, &igrf_9, &hist, &cals10k_2, NULL };
const Model *external_models[] = { &ts_05, &t_96, NULL };
const Model *crustal_models[] = { &chaos_7_16, NULL };

const Model *get_model(const Model **models, const char *version) {
    /* src/models.c:114-122 */
    for (int i = 0; models[i] != NULL; i++)
        if (strcmp(models[i]->version, version) == 0) return models[i];
    return NULL;
}

/* The setup_fun loop of cutoff() (src/main.c:51-61): internal_recalc for the
 * internal model, PARMOD from the INFILE for the external one.  Without an
 * internal model the GSM axes come from the IGRF-14 dipole at the date (the
 * reference leaves them uninitialised, src/main.c:51). */
int models_setup(const Model **models, FILE *f, const InfileHeader *h, ModelsParams *p) {
    const int32_t t[7] = { h->iy, h->mes, h->ide, h->id, h->ih, h->min, h->is };
    int have_internal = 0;
    for (int i = 0; models[i]; i++) {
        const Model *m = models[i];
        if (m->kind == MODEL_INTERNAL) {
            if (cor_internal_setup(m->version, t, p) != COR_OK) return -1;
            have_internal = 1;
        } else if (m->kind == MODEL_EXTERNAL) {
            const int rc = m->code == COR_EXTERNAL_TS05 ? read_ts05_params(f, p) : read_t96_params(f, p);
            if (rc != 0) return -1;
        }
    }
    if (!have_internal && cor_gsm_setup(t, p) != COR_OK) return -1;
    return 0;
}

cor_model_set models_device_set(const Model **models) {
    cor_model_set s = { COR_INTERNAL_NONE, COR_EXTERNAL_NONE, COR_CRUSTAL_NONE, 0 };
    for (int i = 0; models[i]; i++) {
        if (models[i]->kind == MODEL_INTERNAL) s.internal_model = models[i]->code;
        else if (models[i]->kind == MODEL_EXTERNAL) s.external_model = models[i]->code;
        else s.crustal_model = models[i]->code;
    }
    return s;
}
