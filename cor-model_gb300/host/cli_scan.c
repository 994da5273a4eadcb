/*
 * cli_scan.c -- trajectory_simulation_cutoff (src/trajectory.c:6-161) on the
 * GPU: the scan of one INFILE goes to libcortrace as a batch of one, and the
 * allowed rows and the CUTOFF line are printed from the returned records with
 * the reference's formulas and formats (src/trajectory.c:90-122, :160), using
 * the host C library, so the text equals the reference's wherever the final
 * states do.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cli.h"
#include "scan_text.h"

static cor_ctx *g_ctx = NULL;

int cli_context(cor_ctx **ctx) {
    if (!g_ctx) {
        const int rc = cor_ctx_create(0, &g_ctx);
        if (rc != COR_OK) {
            fprintf(stderr, "Error: no usable CUDA device (code %d)\n", rc);
            return rc;
        }
    }
    *ctx = g_ctx;
    return COR_OK;
}

static void job_from_header(const InfileHeader *h, cor_scan_job *j) {
    j->r0 = h->r0;
    j->the0 = h->the0;
    j->fi0 = h->fi0;
    j->the1 = h->the1;
    j->fi1 = h->fi1;
    j->rig = h->rig;
    j->del = h->del;
    j->rk = h->rk;
    j->zn = h->zn;
    j->nk1 = h->nk1;
    j->param_index = 0;
    j->i_first = 0;  /* the whole grid */
    j->i_count = 0;
}

int cli_write_scan(FILE *out, const InfileHeader *h, const cor_site_result *site, const uint8_t *status,
                   const cor_traj_record *records) {
    const int n = (int)round((h->rk - h->rig) / h->del);
    return cor_txt_scan(out, h->rig, h->del, (int64_t)n + 1, site, status, records);
}

void trajectory_simulation_cutoff(InfileHeader *header, const Model **models, ModelsParams *models_params,
                                  FILE *outfile, uint64_t step_limit, double tu_angle, double particle_mass,
                                  uint32_t parallel) {
    (void)parallel; /* the scan always runs on the GPU */
    cor_ctx *ctx = NULL;
    if (cli_context(&ctx) != COR_OK) exit(1);
    cor_scan_job job;
    job_from_header(header, &job);
    uint64_t n = 0;
    if (cor_batch_count(&job, 1, &n, NULL) != COR_OK) {
        fprintf(stderr, "Error: invalid rigidity grid\n");
        exit(1);
    }
    cor_site_result site;
    uint8_t *status = (uint8_t *)malloc(n);
    cor_traj_record *records = (cor_traj_record *)malloc(sizeof(cor_traj_record) * n);
    if (!status || !records) {
        fprintf(stderr, "Error: out of memory\n");
        exit(1);
    }
    cor_batch_req req;
    memset(&req, 0, sizeof req);
    req.jobs = &job;
    req.n_jobs = 1;
    req.params = models_params;
    req.n_params = 1;
    req.models = models_device_set(models);
    req.step_limit = step_limit;
    req.tu_angle = tu_angle;
    req.particle_mass = particle_mass;
    cor_batch_result res;
    memset(&res, 0, sizeof res);
    res.sites = &site;
    res.status = status;
    res.records = records;
    const int rc = cor_trace_batch(ctx, &req, &res);
    if (rc != COR_OK) {
        fprintf(stderr, "Error: %s\n", cor_last_error_string(ctx));
        exit(1);
    }
    cli_write_scan(outfile, header, &site, status, records);
    free(status);
    free(records);
}

/* `cor -m trajectory` (src/trajectory.c:163-273): every accepted step of each
 * rigidity, traced on the GPU with the scan's integrator and recorded there
 * (cor_trace_steps), printed here in the reference's two formats. */
#define TRAJ_MAX_RECORDED 4000000u

int trajectory_simulation(InfileHeader *header, const Model **models, ModelsParams *models_params, FILE *tragsm,
                          FILE *trasph, uint64_t step_limit, double tu_angle, double particle_mass) {
    cor_ctx *ctx;
    if (cli_context(&ctx) != COR_OK) return 1;
    cor_scan_job job;
    job_from_header(header, &job);
    uint64_t n = 0;
    if (cor_batch_count(&job, 1, &n, NULL) != COR_OK) {
        fprintf(stderr, "Error: invalid rigidity grid\n");
        return 1;
    }
    const uint32_t cap = step_limit < TRAJ_MAX_RECORDED ? (uint32_t)(step_limit ? step_limit : 1) : TRAJ_MAX_RECORDED;
    cor_step_record *steps = (cor_step_record *)malloc(sizeof(cor_step_record) * (size_t)cap * (size_t)n);
    cor_traj_record *records = (cor_traj_record *)malloc(sizeof(cor_traj_record) * (size_t)n);
    uint8_t *status = (uint8_t *)malloc((size_t)n);
    if (!steps || !records || !status) {
        fprintf(stderr, "Error: out of memory\n");
        return 1;
    }
    cor_site_result site;
    cor_batch_req req;
    memset(&req, 0, sizeof req);
    req.jobs = &job;
    req.n_jobs = 1;
    req.params = models_params;
    req.n_params = 1;
    req.models = models_device_set(models);
    req.step_limit = step_limit;
    req.tu_angle = tu_angle;
    req.particle_mass = particle_mass;
    cor_batch_result res;
    memset(&res, 0, sizeof res);
    res.sites = &site;
    res.status = status;
    res.records = records;
    if (cor_trace_steps(ctx, &req, &res, steps, cap) != COR_OK) {
        fprintf(stderr, "Error: %s\n", cor_last_error_string(ctx));
        return 1;
    }
    for (uint64_t t = 0; t < n; t++) {
        const cor_step_record *s = steps + t * cap;
        for (uint32_t k = 0; k < cap && s[k].step == k + 1; k++) {
            double sph[3];
            cor_txt_car_to_sph(s[k].pos, sph);
            const double r = sph[0] / DEF_RE;
            const double td = 90. - (sph[1] / DEF_TO_RAD);
            const double fei = sph[2] / DEF_TO_RAD;
            fprintf(tragsm, "%6d%17.5f%17.5f%17.5f%14.2f%15.10f%18.2f\n", (int)s[k].step, s[k].gsm[0], s[k].gsm[1],
                    s[k].gsm[2], s[k].v, s[k].time, s[k].length);
            fprintf(trasph, "%6d%17.5f%17.5f%17.5f%14.2f%15.10f%18.2f\n", (int)s[k].step, r, td, fei, s[k].v,
                    s[k].time, s[k].length);
        }
    }
    free(steps);
    free(records);
    free(status);
    return 0;
}
