/*
 * cor_trace.h -- C ABI of the GB300 cutoff-rigidity tracer (libcortrace.so).
 *
 * The library replaces the rigidity scan of `cor -m cutoff`:
 *   trajectory_simulation_cutoff()   src/trajectory.c:6-161   (scan, step control, RK, terminations)
 *   calculate_field()                src/models.c:194-207     (field composition, GSM<->GEO)
 *   internal_geo()                   lib/internal/internal.c:182-275 (spherical-harmonic field)
 *   t96_gsm() / ts05_gsm()           lib/t96/t96.c:4, lib/ts05/ts05.c:7 (external fields)
 *   chaos_geo()                      lib/chaos/chaos.c:120-226 (high-degree SH field)
 * and the host-side set-up that feeds it:
 *   internal_recalc()                lib/internal/internal.c:89-180
 *
 * Every entry point takes plain pointers and sizes; no C++ or framework types
 * cross the boundary.  All functions return COR_OK (0) or a negative COR_ERR_*
 * code; cor_last_error_string() gives a one-line reason for the last failure on
 * a context.  Buffers are owned by the caller.  A context is bound to one CUDA
 * device and is not safe for concurrent use from several host threads; use one
 * context per thread.
 */
#ifndef COR_TRACE_H
#define COR_TRACE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COR_TRACE_ABI_VERSION 3

/* Number of Gauss coefficients of the degree-13 internal models
 * (INTERNAL_COEFS_SIZE, lib/internal/coefs/coefs.h:6). */
#define COR_SH_COEFS 105

/* ---- error codes ------------------------------------------------------ */
#define COR_OK               0
#define COR_ERR_INVALID     -1  /* bad argument, bad size, unknown model     */
#define COR_ERR_NOMEM       -2  /* device or host allocation failed          */
#define COR_ERR_CUDA        -3  /* a CUDA runtime call failed                */
#define COR_ERR_WATCHDOG    -4  /* a kernel gave up on a bounded wait        */
#define COR_ERR_NODEV       -5  /* no CUDA device / library built without it */
#define COR_ERR_UNSUPPORTED -6  /* combination of models not available       */
#define COR_ERR_RANGE       -7  /* epoch outside the coefficient table       */
#define COR_ERR_BUSY        -8  /* no free stream slot: collect a ticket first */
#define COR_PENDING          1  /* cor_stream_wait: the segment is not done yet */

/* ---- field models ----------------------------------------------------- */
/* main() builds models[] in the order internal, external, crustal
 * (src/main.c:269-299); calculate_field sums them in that order. */
#define COR_INTERNAL_NONE 0
#define COR_INTERNAL_SH   1   /* any of igrf9..igrf14, hist, cals10k.2 */
#define COR_EXTERNAL_NONE 0
#define COR_EXTERNAL_T96  1   /* -e t96  */
#define COR_EXTERNAL_TS05 2   /* -e ts05 */
#define COR_CRUSTAL_NONE  0
#define COR_CRUSTAL_CHAOS 1   /* -c chaos7.16 */

typedef struct {
    int32_t internal_model;   /* COR_INTERNAL_* */
    int32_t external_model;   /* COR_EXTERNAL_* */
    int32_t crustal_model;    /* COR_CRUSTAL_*  */
    int32_t reserved;         /* must be 0      */
} cor_model_set;

/* Per-condition parameter block: the ModelsParams struct of src/models.h:9-17
 * with the same members and meaning.  g/h are the Schmidt-scaled Gauss
 * coefficients at the epoch, rec the Legendre recursion factors, a1..a3 the
 * rows of the GEO->GSM rotation, parmod the external-field parameters
 * {Pdyn, Dst, ByIMF, BzIMF, W1..W6} (src/io.c:98-127). */
typedef struct {
    double parmod[10];
    double g[COR_SH_COEFS];
    double h[COR_SH_COEFS];
    double rec[COR_SH_COEFS];
    double a1[3];
    double a2[3];
    double a3[3];
} cor_model_params;

/* One rigidity scan = one INFILE of `cor -m cutoff` (InfileHeader,
 * src/common.h:26-54; read by read_cutoff_infile_header, src/io.c:4-20).
 * The scan's grid is rig + i*del for i = 0 .. N-1, N = round((rk-rig)/del) + 1
 * (src/trajectory.c:7,14).  i_first / i_count select a window of that grid
 * (no counterpart in the reference; zero = the reference's whole scan): the
 * indices i_first .. i_first + i_count - 1 are traced with the same
 * rigidities rig + i*del as the whole scan, and the reduction counts the
 * untraced indices below the window as forbidden and those above it as
 * allowed, so a window that holds the whole penumbra gives the whole scan's
 * P(S), P(C), P(M) bit for bit. */
typedef struct {
    double r0;     /* start radius [R_E]                              */
    double the0;   /* start geographic latitude [deg]                 */
    double fi0;    /* start geographic longitude [deg]                */
    double the1;   /* latitude of the initial velocity vector [deg]   */
    double fi1;    /* longitude of the initial velocity vector [deg]  */
    double rig;    /* first rigidity [GV]                             */
    double del;    /* rigidity step [GV], > 0                         */
    double rk;     /* last rigidity [GV]                              */
    double zn;     /* charge number, non-zero                         */
    int32_t nk1;   /* steps per gyro period (initial), > 0            */
    int32_t param_index; /* which cor_model_params block this scan uses */
    int32_t i_first; /* first grid index traced (0: from the grid's start) */
    int32_t i_count; /* indices traced (0: to the grid's end)             */
} cor_scan_job;

/* Termination class of one trajectory (src/trajectory.c:48-145). */
#define COR_TRAJ_NONE        0  /* not traced                                    */
#define COR_TRAJ_ALLOWED     1  /* escaped at r = 25 R_E or the magnetopause      */
#define COR_TRAJ_REENTRY     2  /* r < 1 R_E                  (forbidden, rmx1)   */
#define COR_TRAJ_SUPERLUM    3  /* v/c > 1                    (forbidden, rmx1)   */
#define COR_TRAJ_STEP_LIMIT  4  /* step > step_limit          (forbidden, rmx2)   */
#define COR_TRAJ_WATCHDOG    5  /* boundary refinement ran past nk0 = 2^30;
                                   the reference has no bound here (its int nk0
                                   would overflow).  Counted as forbidden, rmx2. */

/* Final state of one trajectory.  For allowed trajectories the host derives
 * the printed row (eth, efi, ath, afi; src/trajectory.c:91-122) from pos/vel
 * with the C library, so the text output matches the reference digit for digit. */
typedef struct {
    double pos[3];     /* final GEO position [m]                 */
    double vel[3];     /* final GEO velocity [m/s]               */
    double v;          /* |vel| as carried by the integrator     */
    double time;       /* accumulated time [s]                   */
    double length;     /* accumulated path length [m]            */
    uint32_t steps;    /* accepted steps                         */
    uint32_t trials;   /* RK trials, accepted and rejected       */
    int32_t status;    /* COR_TRAJ_*                             */
    int32_t reserved;
} cor_traj_record;

/* Per-scan reduction (src/trajectory.c:156-160): P(S)=r_lower, P(C)=r_upper,
 * P(M)=r_cutoff, exactly as printed on the CUTOFF line. */
typedef struct {
    double r_lower;     /* rmi  */
    double r_upper;     /* rmx  = max(rmx1, rmx2) + del */
    double r_cutoff;    /* rms  = rmi + zan*del */
    int32_t n_forbidden;  /* nza (a window's untraced lower indices count as forbidden) */
    int32_t n_traj;       /* trajectories traced                                   */
} cor_site_result;

typedef struct {
    uint64_t accepted_steps;  /* = field evaluations after the initial one */
    uint64_t trials;          /* RK trials (accepted + rejected)           */
    uint64_t trajectories;
    uint64_t watchdog;        /* trajectories that ended COR_TRAJ_WATCHDOG */
    uint64_t kernel_launches; /* kernels the call launched: the scan's generations, the uniform-grid
                                 check (when the rigidity-major order was asked for) and the reduction;
                                 cor_trace_batch_device_noalloc also counts the kernel that writes
                                 this block; a stream segment counts its stream launch (1) */
} cor_counters;

typedef struct {
    const cor_scan_job *jobs;          /* n_jobs scans                        */
    int32_t n_jobs;
    int32_t n_params;
    const cor_model_params *params;    /* n_params parameter blocks           */
    cor_model_set models;
    uint64_t step_limit;               /* -s, default 25000 (src/main.c:13)   */
    double tu_angle;                   /* -u, default 0.01 (src/main.c:19)    */
    double particle_mass;              /* -t, proton 1.6725e-27 kg            */
} cor_batch_req;

typedef struct {
    cor_site_result *sites;     /* n_jobs, required                              */
    uint8_t *status;            /* n_trajectories, optional (NULL = not written) */
    cor_traj_record *records;   /* n_trajectories, optional                      */
    cor_counters counters;      /* filled by the call                            */
} cor_batch_result;

typedef struct cor_ctx cor_ctx;

/* ---- context ---------------------------------------------------------- */
/* No counterpart in the reference, which keeps no state between INFILEs and
 * reports errors by printing to stderr and returning 1 from main
 * (src/main.c:14-49).  A context holds one device's stream, the resident
 * parameter blocks and crustal table, and reusable buffers; every call on it
 * sets the string cor_last_error_string returns when it fails. */
int cor_ctx_create(int device, cor_ctx **out);
int cor_ctx_destroy(cor_ctx *ctx);
const char *cor_last_error_string(const cor_ctx *ctx);
int cor_abi_version(void);

/* Number of trajectories of a batch and, optionally, the exclusive prefix
 * offsets of each job's trajectories (offsets has n_jobs+1 entries).  A scan
 * has (int)round((rk-rig)/del)+1 of them, as the loop of src/trajectory.c:7,12
 * counts, or i_count for a window.  Also the one check of every job: it
 * returns COR_ERR_INVALID for a bad grid or window, nk1 <= 0, a zero charge
 * or a non-finite start value. */
int cor_batch_count(const cor_scan_job *jobs, int32_t n_jobs,
                    uint64_t *n_trajectories, uint64_t *offsets);

/* sin/cos of the start colatitude/longitude and of the velocity direction of
 * each scan, (90-the0), fi0, (90-the1), fi1 in radians (src/trajectory.c:18-28).
 * Taken from the host C library so the start vectors on the device equal the
 * reference's; cor_trace_batch computes them itself. */
typedef struct {
    double st0, ct0, sp0, cp0;
    double st1, ct1, sp1, cp1;
} cor_job_trig;

int cor_prepare_trig(const cor_scan_job *jobs, int32_t n_jobs, cor_job_trig *out);

/* ---- scan ------------------------------------------------------------- */
/* Replaces trajectory_simulation_cutoff (src/trajectory.c:6) for a batch of
 * scans.  Host buffers in and out; copies are done inside the call.  Blocks
 * until the results are on the host. */
int cor_trace_batch(cor_ctx *ctx, const cor_batch_req *req, cor_batch_result *out);

/* cor_trace_batch_device flags */
#define COR_FLAG_UNIFORM_GRID 1u  /* every job has the same number of rigidities:
                                     the work queue then hands out the lowest
                                     rigidities of all jobs first.  The device
                                     checks the offsets before the scan and
                                     keeps the scan-by-scan order when they are
                                     not uniform: a wrong flag costs the order,
                                     never a result or a write out of bounds */

/* Uploads n_params parameter blocks to the device, where they stay for the
 * following cor_trace_batch_device calls (cor_trace_batch uploads its own).
 * Each block is the ModelsParams the reference passes to
 * trajectory_simulation_cutoff (src/models.h:9-17, filled by the setup_fun
 * loop of src/main.c:51-61).  Per-condition constants of the external models
 * are derived here on the host. */
int cor_upload_params(cor_ctx *ctx, const cor_model_params *params, int32_t n_params);

/* Regrouping of the scan kernel on this context (no counterpart in the
 * reference; an autotuner's knobs).  After the work queue drains, a block
 * parks its live trajectories for the next kernel generation when fewer than
 * park_below lanes per warp are live (0..32; default 16), or once half of the
 * generation's warps have parked; at most max_generations generations run
 * (1..1024; default 48; 1 = never regroup), and a generation with at most
 * min_park live trajectories (default 256) runs them to the end.  Results
 * do not depend on these settings, only the time does. */
int cor_ctx_set_regroup(cor_ctx *ctx, int32_t park_below, int32_t max_generations, int64_t min_park);

/* Diagnostics of the last scan on this context (no counterpart in the
 * reference): for each kernel generation, the live trajectories it started
 * with and its host wall time [ms] (generation 0 drains the work queue; the
 * later ones run regrouped tails).  Fills up to cap entries and returns the
 * number of generations (negative COR_ERR_* for a null context). */
int32_t cor_ctx_generation_log(const cor_ctx *ctx, int32_t cap, uint64_t *live, double *ms);

/* Work-queue order on this context (no counterpart in the reference; an
 * autotuner's knob).  1 (default): the lowest rigidity of every scan first
 * (longest trajectories first); 0: scan by scan, consecutive rigidities of one
 * scan to neighbouring lanes, whose paths start out alike; 2 (streams only;
 * the batch path takes it as 1): chunks of 32 consecutive rigidities of one
 * scan, one warp's worth, the chunks in ascending rigidity -- neighbouring
 * lanes alike and the longest trajectories early.  cor_trace_batch uses it
 * when every job has the same number of rigidities; the batch device path
 * takes the order from its flags (COR_FLAG_UNIFORM_GRID); stream segments of
 * unequal scans (windows) are handed out in ascending rigidity by trajectory
 * (1) or by chunk (2).  Results do not depend on it. */
int cor_ctx_set_queue_order(cor_ctx *ctx, int32_t rigidity_major);

/* 1 (the default): before each field evaluation, every block of the scan
 * kernel of cor_trace_batch, cor_trace_batch_device(_noalloc) and
 * cor_trace_steps regroups its trajectories by the branches of the field
 * code their positions take, so that a warp's lanes run the same sub-models;
 * 0: never.  Results do not depend on it (a stream takes the same choice from
 * cor_stream_config.sort_lanes).  Other values give COR_ERR_INVALID.  No
 * counterpart in the reference (its OpenMP threads run one trajectory each,
 * src/trajectory.c:11). */
int cor_ctx_set_lane_sort(cor_ctx *ctx, int32_t on);

/* Replaces the crustal model's coefficient table on this context: G and H as
 * packed lower triangles (index n*(n+1)/2 + m, degrees n = 0 .. nmax-1), the
 * layout of lib/chaos/coefs/chaos_7_16.h read by chaos_geo
 * (lib/chaos/chaos.c:120-226).  Without this call the first scan or field
 * batch with COR_CRUSTAL_CHAOS uploads the built-in CHAOS-7.16 table
 * (nmax 186).  nmax outside [2, 192] gives COR_ERR_RANGE.  The reference
 * has no counterpart: its table is a compile-time constant. */
int cor_upload_crustal(cor_ctx *ctx, const double *g, const double *h, int32_t nmax);

/* trajectory_simulation_cutoff (src/trajectory.c:6-161), as cor_trace_batch,
 * with every buffer already in device memory (jobs, trig from
 * cor_prepare_trig, offsets from cor_batch_count, sites, status, records),
 * using the parameter blocks of the last cor_upload_params.  The jobs are not
 * checked again here: they must be ones that cor_batch_count accepted, and
 * offsets_dev[n_jobs] must equal n_trajectories (writes and reads stay below
 * n_trajectories either way).
 * `stream` is a cudaStream_t (NULL = the legacy default stream).  The scan runs in
 * generations: between two of them the host reads how many trajectories the
 * kernel parked for regrouping, so the call synchronises `stream` a few
 * times and returns with the last generation and the reduction queued.
 * Counters go to the device buffer `counters_dev` (a cor_counters; NULL =
 * internal). */
int cor_trace_batch_device(cor_ctx *ctx,
                           const cor_scan_job *jobs_dev, const cor_job_trig *trig_dev,
                           int32_t n_jobs, const uint64_t *offsets_dev, uint64_t n_trajectories,
                           cor_model_set models, uint64_t step_limit,
                           double tu_angle, double particle_mass,
                           cor_site_result *sites_dev, uint8_t *status_dev,
                           cor_traj_record *records_dev, cor_counters *counters_dev,
                           uint32_t flags, void *stream);

/* Largest n_trajectories one cor_trace_batch_device_noalloc call accepts. */
#define COR_NOALLOC_MAX_TRAJ 1048576

/* The scan of cor_trace_batch_device without any device allocation: it calls
 * no cudaMalloc, cudaFree or other allocating routine.  It has no counterpart
 * in the reference.  Its scratch is one file-scope device array of
 * 256 + COR_NOALLOC_MAX_TRAJ bytes (the work-queue counter, the generation and
 * counter blocks, and the per-trajectory termination classes the reduction
 * reads), so the per-trajectory classes are not returned (there is no
 * status_dev); n_trajectories above COR_NOALLOC_MAX_TRAJ gives COR_ERR_RANGE
 * before any GPU work.  It runs the scan as one kernel generation (no
 * regrouping, whose park buffers would need memory), then the reduction, and
 * returns with both queued on `stream` without synchronising it.  Results
 * (sites, records, counters) are identical to cor_trace_batch_device's.
 * Preconditions: the parameter blocks are resident (cor_upload_params) and,
 * for a model set with the crustal model, so is its table (cor_upload_crustal)
 * -- otherwise COR_ERR_INVALID; offsets_dev[n_jobs] equals n_trajectories
 * (the kernels never touch the array at or beyond n_trajectories in any case).
 * counters_dev->kernel_launches counts every kernel of the call: the
 * uniform-grid check (with COR_FLAG_UNIFORM_GRID), the scan, the reduction
 * and the kernel that writes the count (4 for a uniform batch).
 * The first call on a device looks up the array's device address there
 * (cudaGetSymbolAddress, which may load this library's device code onto that
 * device); make that first call before any stream capture on the device.
 * Every call, on every context of the device, shares the array and finds the
 * previous call's contents in it (the call clears what must start at zero):
 * calls whose work overlaps on the GPU race on it and must be serialised by
 * the caller, e.g. by issuing them all on one stream. */
int cor_trace_batch_device_noalloc(cor_ctx *ctx,
                                   const cor_scan_job *jobs_dev, const cor_job_trig *trig_dev,
                                   int32_t n_jobs, const uint64_t *offsets_dev, uint64_t n_trajectories,
                                   cor_model_set models, uint64_t step_limit,
                                   double tu_angle, double particle_mass,
                                   cor_site_result *sites_dev, cor_traj_record *records_dev,
                                   cor_counters *counters_dev, uint32_t flags, void *stream);

/* ---- persistent scan stream -------------------------------------------- */
/* No counterpart in the reference, which runs one INFILE per process and
 * waits for its whole scan (trajectory_simulation_cutoff, src/trajectory.c:6-161,
 * called once from cutoff(), src/main.c:86).  A stream keeps ONE launch of the
 * scan kernel resident on the device and feeds it batches of scans
 * ("segments") as the caller submits them: every trajectory is traced and
 * every scan reduced exactly as cor_trace_batch does (same flags, cutoffs and
 * records, bit for bit), but a lane whose trajectory ends takes the next
 * trajectory of any published segment, so the device never waits for one
 * batch's last long trajectories before starting the next batch.
 *
 * Each segment's inputs are copied to the device (or already there, for
 * cor_stream_submit_device), published through a control block in mapped
 * pinned host memory, and reduced on the device by the warp that finishes a
 * scan's last trajectory; the segment's completion is written back to mapped
 * host memory, where cor_stream_wait reads it.  While a stream runs, its
 * kernel occupies every SM but cfg.reserve_sms: other kernels on the device
 * (the caller's, or libraries') run only on the reserved SMs, so a caller
 * that launches device work between submits must reserve some.
 * A stream is used from one host thread at a time. */
typedef struct cor_stream cor_stream;

typedef struct {
    int32_t slots;             /* segments submitted and not yet collected, at most (ring size; default 8)  */
    int32_t max_jobs;          /* scans per segment (default 16384)                                          */
    int64_t max_trajectories;  /* trajectories per segment (default 2097152, at most 2^32-1)                 */
    int32_t max_params;        /* parameter blocks per cor_stream_submit (default 64)                        */
    int32_t want_records;      /* 1: cor_stream_submit segments keep per-trajectory final records (default 0) */
    int32_t reserve_sms;       /* SMs the stream kernel leaves free for other kernels (default 0)            */
    int32_t fixed_params;      /* capacity of cor_stream_upload_params (default 256)                         */
    int32_t pool_params;       /* parameter blocks of cor_stream_submit per launch (default 4096)            */
    int32_t segments_per_launch; /* segments per launch (default 65536)                                      */
    double idle_limit_s;       /* a block of the kernel with nothing to trace for this long gives up and the
                                  stream fails with COR_ERR_WATCHDOG (default 60 s); cor_stream_drain and
                                  cor_stream_close are the normal ways to end a launch                      */
    int32_t launch_on_drain;   /* 1: submits only stage and publish; cor_stream_drain launches the kernel
                                  with everything published and the stop index already set, so the launch
                                  never waits on the host (at most `slots` segments per launch; default 0) */
    int32_t scan_events;       /* 1: each cor_stream_submit scan's result is also written to mapped host
                                  memory as soon as it is reduced (cor_stream_poll_scans; default 0)     */
    int32_t sort_lanes;        /* 1: before each field evaluation a block regroups its trajectories by the
                                  branches of the field code their positions take, so a warp's lanes run
                                  the same sub-models (results are unchanged; default 1); 0: never      */
} cor_stream_config;

void cor_stream_config_default(cor_stream_config *cfg);

/* A stream on ctx's device for one model set and one step control
 * (step_limit, tu_angle, particle_mass as in cor_batch_req).  Allocates every
 * buffer it will use (device ring slots, pinned staging, mapped control
 * block); no call on the stream allocates afterwards.  The kernel is launched
 * by the first submit and relaunched when a launch's parameter pool or
 * segment capacity is used up (after its published segments finish). */
int cor_stream_create(cor_ctx *ctx, cor_model_set models, uint64_t step_limit, double tu_angle,
                      double particle_mass, const cor_stream_config *cfg, cor_stream **out);

/* Publishes a batch of scans from host buffers: jobs (checked as by
 * cor_batch_count; param_index into params[0 .. n_params-1]) and their
 * parameter blocks.  Returns at once with a ticket (the segment's sequence
 * number); cor_stream_wait collects the results.  COR_ERR_BUSY when the ring
 * slot the segment needs still holds an uncollected segment.  With the
 * context's rigidity-major queue order (the default), a batch of equal scans
 * is handed out lowest rigidity first across its scans, and a batch of
 * unequal scans (windows) in ascending rigidity over all its trajectories:
 * the longest trajectories start first. */
int cor_stream_submit(cor_stream *s, const cor_scan_job *jobs, int32_t n_jobs, const cor_model_params *params,
                      int32_t n_params, int64_t *ticket);

/* The result of one scan of a segment as the stream kernel reports it the
 * moment the scan's last trajectory is reduced, before the rest of its
 * segment has finished (cor_stream_poll_scans). */
typedef struct {
    cor_site_result site;   /* P(S), P(C), P(M) as cor_trace_batch gives them              */
    uint8_t first_class;    /* COR_TRAJ_* of the scan's first traced rigidity              */
    uint8_t last_class;     /* COR_TRAJ_* of its last                                      */
    uint16_t reserved;
    uint32_t reserved2;
    uint64_t seq1;          /* the segment's ticket + 1 once this record is the scan's     */
} cor_scan_event;

/* Which scans of an outstanding cor_stream_submit segment have finished so
 * far (the stream must have been created with scan_events = 1): for scans
 * first .. first+count-1 of the segment, done[k] is set to 1 when scan
 * first+k has finished, and then events[k] holds its result (either array may
 * be NULL to skip it).  Returns the number of finished scans in the range.
 * No counterpart in the reference: it lets a caller act on a scan (a window
 * edge hit, a small request inside a big segment) without waiting for the
 * whole segment. */
int cor_stream_poll_scans(cor_stream *s, int64_t ticket, int32_t first, int32_t count, uint8_t *done,
                          cor_scan_event *events);

/* Parameter blocks for cor_stream_submit_device: appended to the stream's
 * fixed pool, where they stay for the stream's lifetime; *first_index is the
 * pool index of params[0] (device jobs use first_index + k as param_index). */
int cor_stream_upload_params(cor_stream *s, const cor_model_params *params, int32_t n_params, int32_t *first_index);

/* Publishes a batch whose buffers are already in device memory: jobs_dev
 * (param_index into the fixed pool), trig_dev (cor_prepare_trig),
 * offsets_dev (cor_batch_count), and the outputs sites_dev, status_dev
 * (required) and records_dev (optional).  offsets_host is the host copy of
 * the same offsets: the trajectory count and the queue order are taken from
 * it (rigidity-major when every scan has the same count); offsets_dev must
 * hold the same values.  The buffers must stay valid until the ticket is
 * collected. */
int cor_stream_submit_device(cor_stream *s, const cor_scan_job *jobs_dev, const cor_job_trig *trig_dev,
                             const uint64_t *offsets_dev, const uint64_t *offsets_host, int32_t n_jobs,
                             cor_site_result *sites_dev, uint8_t *status_dev, cor_traj_record *records_dev,
                             int64_t *ticket);

/* Waits up to timeout_ms (0: just look; negative: no limit) for a ticket.
 * COR_PENDING if it is not done yet; COR_OK once done, with out->counters
 * filled and, for a cor_stream_submit segment, out->sites (required),
 * out->status and out->records (optional, NULL = not copied) filled from
 * the device; the ticket is then collected and its slot free.  t_done_ns,
 * if not NULL, gets the device's %globaltimer at the segment's completion.
 * COR_ERR_WATCHDOG if the kernel gave up waiting for work (idle_limit_s),
 * COR_ERR_CUDA if it failed. */
int cor_stream_wait(cor_stream *s, int64_t ticket, int32_t timeout_ms, cor_batch_result *out, uint64_t *t_done_ns);

/* Ends the current launch once every published segment has finished (their
 * results stay collectable) and writes the launch's duration in ms, measured
 * with CUDA events recorded on the kernel's stream around it, to *launch_ms
 * (if not NULL; 0 when nothing ran).  The next submit starts a new launch. */
int cor_stream_drain(cor_stream *s, double *launch_ms);

/* Stops the kernel after every published segment has finished (uncollected
 * results are dropped) and frees the stream. */
int cor_stream_close(cor_stream *s);

/* ---- trajectory dump (`cor -m trajectory`) ----------------------------- */
/* One accepted step of a traced trajectory: what trajectory_simulation
 * (src/trajectory.c:163-273) prints per step to its tragsm_ and trasph_ files
 * (the host derives r, latitude and longitude from pos with the C library). */
typedef struct {
    double gsm[3];    /* GSM position [m]                 */
    double pos[3];    /* GEO position [m]                 */
    double v;         /* speed [m/s]                      */
    double time;      /* accumulated time [s]             */
    double length;    /* accumulated path length [m]      */
    uint32_t step;    /* accepted step number (1-based)   */
    uint32_t reserved;
} cor_step_record;

/* Replaces trajectory_simulation (src/trajectory.c:163-273, `cor -m
 * trajectory`).  Traces every rigidity of the jobs like cor_trace_batch and also records
 * each accepted step: trajectory t (in batch order) writes its steps 1..k to
 * steps[t * step_capacity .. t * step_capacity + k - 1] for k up to
 * step_capacity (steps beyond the capacity are traced but not recorded).
 * out->records, when given, holds each trajectory's final state, whose
 * `steps` is the number of accepted steps.  The reference's trajectory mode
 * traces one rigidity per INFILE (rig == rk). */
int cor_trace_steps(cor_ctx *ctx, const cor_batch_req *req, cor_batch_result *out, cor_step_record *steps,
                    uint32_t step_capacity);

/* ---- field ------------------------------------------------------------ */
/* calculate_field (src/models.c:194-207) at n points: gsm_pos is n x 3 GSM
 * positions in metres; geo_field gets n x 3 GEO field components in nT.
 * param_index gives, per point, the parameter block (NULL = block 0); an
 * index outside 0 .. n_params-1 gives COR_ERR_INVALID before any GPU work. */
int cor_field_batch(cor_ctx *ctx, cor_model_set models,
                    const cor_model_params *params, int32_t n_params,
                    const int32_t *param_index, const double *gsm_pos,
                    int64_t n, double *geo_field);

/* ---- host set-up ------------------------------------------------------ */
/* internal_recalc (lib/internal/internal.c:89-180) for a named internal
 * model ("igrf14", "igrf13", ..., "hist", "cals10k.2"; src/models.c:22-84).
 * time = {iy, mes, ide, id, ih, min, is} as in the INFILE.  Fills g, h, rec,
 * a1..a3 of *out and leaves parmod untouched.  Host only; needs no GPU. */
int cor_internal_setup(const char *version, const int32_t time[7], cor_model_params *out);

/* GEO->GSM rotation alone (a1..a3), for runs without an internal model.
 * The reference leaves these uninitialised in that case (src/main.c:51);
 * here they are computed from the date with the IGRF-14 dipole. */
int cor_gsm_setup(const int32_t time[7], cor_model_params *out);

/* ---- measurement -------------------------------------------------------- */
/* Measures the device's FP64 FMA throughput with a register-resident DFMA
 * loop on every SM (an FMA counts as 2 flops) and writes flops/s.  The
 * denominator of the scan's FP64 roofline; no counterpart in the reference. */
int cor_probe_fp64_peak(cor_ctx *ctx, double *flops_per_s);

/* The throughput cost of the device's FP64 functions in units of the peak
 * above: flops_per_call[k] = (time per call, the probe loop's own cost taken
 * out) x (cor_probe_fp64_peak flops/s), for k = 1 exp, 2 log, 3 sin, 4 cos,
 * 5 atan, 6 asin, 7 atan2, 8 pow, 9 division, 10 sqrt ([0] = 0, the loop).
 * Arguments are seeded values in the ranges the field models use.  These are
 * the measured weights of the transcendentals in the scan's roofline
 * numerator (the reference's C library functions it calls per step); no
 * counterpart in the reference. */
int cor_probe_fp64_functions(cor_ctx *ctx, double *flops_per_call);

#ifdef __cplusplus
}
#endif

#endif /* COR_TRACE_H */
