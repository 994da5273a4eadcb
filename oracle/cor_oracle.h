/*
 * cor_oracle.h -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU restatement of the reference's rigidity scan (`cor -m cutoff`), used only
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
 * checker for libcortrace.  It shares the ABI structs of include/cor_trace.h so
 * the same inputs feed both.  Parity of this restatement with the reference is
 * pinned by tests/golden/ (fixtures produced by the reference built from source
 * by oracle/build.py).
 */
#ifndef COR_ORACLE_H
#define COR_ORACLE_H

#include <stdint.h>
#include "../include/cor_trace.h"

#ifdef __cplusplus
extern "C" {
#endif

/* internal_geo, lib/internal/internal.c:182-275 */
void orc_internal_geo(double x, double y, double z, const double *g, const double *h,
                      const double *rec, double *bx, double *by, double *bz);

/* t96_gsm, lib/t96/t96.c:4-111 */
void orc_t96_gsm(const double *parmod, double x, double y, double z,
                 double *bx, double *by, double *bz);

/* ts05_gsm, lib/ts05/ts05.c:7-134 */
void orc_ts05_gsm(const double *parmod, double x, double y, double z,
                  double *bx, double *by, double *bz);

/* chaos_geo, lib/chaos/chaos.c:120-226; g/h are dense nmax x nmax tables. */
void orc_chaos_geo(double x, double y, double z, const double *g, const double *h, int nmax,
                   double *bx, double *by, double *bz);

/* calculate_field, src/models.c:194-207: GSM position [m] -> GEO field [nT]. */
void orc_calculate_field(const double gsm_pos[3], cor_model_set models,
                         const cor_model_params *p, double geo_field[3]);

/* calculate_position_and_speed, src/trajectory.c:275-356 */
void orc_rk_step(double h, double d, const double field[3], double vel[3], double pos[3]);

/* Crustal table used by orc_calculate_field when models.crustal_model is set. */
void orc_set_crustal_table(const double *g, const double *h, int nmax);

/* trajectory_simulation_cutoff, src/trajectory.c:6-161, serial semantics,
 * for one scan.  records/status have round((rk-rig)/del)+1 entries (either may
 * be NULL).  Counters are added to *counters when not NULL. */
/* Per-step records of the first traced rigidity of a job (trajectory mode). */
int orc_trace_steps(const cor_scan_job *job, const cor_model_params *params, cor_model_set models,
                    uint64_t step_limit, double tu_angle, double particle_mass,
                    cor_step_record *steps, uint32_t step_cap, cor_traj_record *rec);

int orc_scan_job(const cor_scan_job *job, const cor_model_params *params, cor_model_set models,
                 uint64_t step_limit, double tu_angle, double particle_mass,
                 cor_site_result *site, uint8_t *status, cor_traj_record *records,
                 cor_counters *counters);

/* A batch of scans over `threads` host threads: chunks of 4 consecutive
 * rigidities are handed out from a shared counter (the reference balances its
 * OpenMP team per rigidity, src/trajectory.c:11), and each scan is reduced
 * once all of its chunks are done.  offsets as from cor_batch_count. */
int orc_scan_batch(const cor_batch_req *req, const uint64_t *offsets, int threads,
                   cor_site_result *sites, uint8_t *status, cor_traj_record *records,
                   cor_counters *counters);

/* Count of floating-point operations of one orc_internal_geo call at radius R
 * (for the roofline's algorithmic work unit). */
int64_t orc_internal_geo_flops(double R);

#ifdef __cplusplus
}
#endif

#endif
