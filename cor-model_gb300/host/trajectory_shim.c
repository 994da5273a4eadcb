/*
 * trajectory_shim.c -- trajectory_simulation_cutoff with exactly the
 * reference's signature (src/trajectory.h:10), running the scan on the GPU
 * through libcortrace.  It is meant to be compiled INSIDE the reference's
 * build, against the reference's own headers (common.h for InfileHeader,
 * models.h for Model and ModelsParams), in place of the definition in
 * src/trajectory.c: the reference's main(), INFILE reader, model registry and
 * set-up (src/main.c, src/io.c, src/models.c) then run unchanged and call this
 * function for `cor -m cutoff` (src/main.c:86).  oracle/build.py's build_shim()
 * is the recipe: it renames the reference's own definition away
 * (-Dtrajectory_simulation_cutoff=...) and links this file and libcortrace.so
 * into the reference's program.
 *
 * What it does: the INFILE header becomes one cor_scan_job, ModelsParams is
 * the parameter block (the same members in the same order as
 * cor_model_params), the model array (NULL-terminated, in main()'s order) is
 * mapped to a device model set by Model.version (src/models.c:22-108), and
 * the rows and CUTOFF line are printed from the returned records
 * (scan_text.h).  `parallel` (-p) is ignored: the scan always runs on the GPU.
 * Errors go to stderr and end the program with status 1, as the reference's
 * main() does for its own errors.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "models.h"
#include "trajectory.h"

#include "cor_trace.h"
#include "scan_text.h"

/* ModelsParams and cor_model_params must be the same block */
_Static_assert(sizeof(ModelsParams) == sizeof(cor_model_params), "ModelsParams layout");
_Static_assert(sizeof(((ModelsParams *)0)->G) == sizeof(((cor_model_params *)0)->g), "Gauss table size");

static cor_ctx *g_shim_ctx = NULL;

static cor_model_set shim_model_set(const Model **models) {
    cor_model_set s = { COR_INTERNAL_NONE, COR_EXTERNAL_NONE, COR_CRUSTAL_NONE, 0 };
    for (int i = 0; models[i]; i++) {
        const char *v = models[i]->version;
        if (strcmp(v, "t96") == 0) s.external_model = COR_EXTERNAL_T96;
        else if (strcmp(v, "ts05") == 0) s.external_model = COR_EXTERNAL_TS05;
        else if (strcmp(v, "chaos7.16") == 0) s.crustal_model = COR_CRUSTAL_CHAOS;
        else s.internal_model = COR_INTERNAL_SH;   /* igrf9..igrf14, hist, cals10k.2 */
    }
    return s;
}

void trajectory_simulation_cutoff(InfileHeader *header, const Model **models, ModelsParams *models_params,
                                  FILE *outfile, uint64_t step_limit, double tu_angle, double particle_mass,
                                  uint32_t parallel) {
    (void)parallel;
    if (!g_shim_ctx) {
        const int rc = cor_ctx_create(0, &g_shim_ctx);
        if (rc != COR_OK) {
            fprintf(stderr, "Error: no usable CUDA device for the GPU scan (code %d)\n", rc);
            exit(1);
        }
    }
    cor_scan_job job;
    memset(&job, 0, sizeof job);
    job.r0 = header->r0;
    job.the0 = header->the0;
    job.fi0 = header->fi0;
    job.the1 = header->the1;
    job.fi1 = header->fi1;
    job.rig = header->rig;
    job.del = header->del;
    job.rk = header->rk;
    job.zn = header->zn;
    job.nk1 = header->nk1;
    uint64_t n = 0;
    if (cor_batch_count(&job, 1, &n, NULL) != COR_OK) {
        fprintf(stderr, "Error: invalid rigidity grid\n");
        exit(1);
    }
    cor_model_params params;
    memcpy(&params, models_params, sizeof params);
    cor_site_result site;
    uint8_t *status = (uint8_t *)malloc((size_t)n);
    cor_traj_record *records = (cor_traj_record *)malloc(sizeof(cor_traj_record) * (size_t)n);
    if (!status || !records) {
        fprintf(stderr, "Error: out of memory\n");
        exit(1);
    }
    cor_batch_req req;
    memset(&req, 0, sizeof req);
    req.jobs = &job;
    req.n_jobs = 1;
    req.params = &params;
    req.n_params = 1;
    req.models = shim_model_set(models);
    req.step_limit = step_limit;
    req.tu_angle = tu_angle;
    req.particle_mass = particle_mass;
    cor_batch_result res;
    memset(&res, 0, sizeof res);
    res.sites = &site;
    res.status = status;
    res.records = records;
    if (cor_trace_batch(g_shim_ctx, &req, &res) != COR_OK) {
        fprintf(stderr, "Error: %s\n", cor_last_error_string(g_shim_ctx));
        exit(1);
    }
    cor_txt_scan(outfile, job.rig, job.del, (int64_t)n, &site, status, records);
    free(status);
    free(records);
}
