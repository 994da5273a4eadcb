/*
 * cli.h -- types of the drop-in `cor` command-line program.
 *
 * The program keeps the reference's command line (src/args.c:11-23), INFILE
 * and output formats (src/io.c) and model registry (src/models.c:22-112), so
 * these types carry the same members with the same meaning as the
 * reference's InfileHeader (src/common.h:26-54), ModelsParams
 * (src/models.h:9-17) and Model (src/models.h:19-25).  The model table holds
 * a device model-set entry instead of a field function pointer, because the
 * field is evaluated on the GPU.
 */
#ifndef COR_CLI_H
#define COR_CLI_H

#include <stdint.h>
#include <stdio.h>

#include "../../include/cor_trace.h"

#define DEF_PI 3.141592654
#define DEF_2PI 6.28318531
#define DEF_RE 6.3712e+06
#define DEF_TO_RAD (DEF_PI / 180.)
#define DEF_Q 1.6021e-19
#define DEF_C 2.99725e+08
#define DEF_HM0_E 9.1093826e-31
#define DEF_HM0_P 1.6725e-27

#define OPT_PARALLEL 1

typedef struct {
    double r0, the0, fi0, the1, fi1;
    int iy, mes, ide, id, ih, min, is;
    double zn;
    int nk1, iopt, ist;
    double rig, del, rk;
    double lat_step, lon_step;   /* field mode (src/io.c:52-67) */
} InfileHeader;

typedef cor_model_params ModelsParams;

typedef enum { MODEL_INTERNAL, MODEL_EXTERNAL, MODEL_CRUSTAL } ModelKind;

typedef struct {
    const char *name;
    const char *version;
    ModelKind kind;
    int code;               /* COR_INTERNAL_SH / COR_EXTERNAL_T96 / ... */
    int needs_params;       /* 4 (T96) or 10 (TS05) PARMOD values follow the header */
} Model;

typedef struct {
    char *input_file_name;
    char *output_file_name;
    char *external_model_name;
    char *internal_model_name;
    char *crustal_model_name;
    char *steps_count;
    char *tu_angle;
    char *mode;
    char *particle_type;
    char *batch_file_name;  /* -b: manifest of "INFILE OUTFILE" lines, traced in one GPU call */
    uint32_t options;
} CLIArguments;

/* cli_io.c -- src/io.c */
int read_cutoff_infile_header(FILE *input_file, InfileHeader *h);
int write_cutoff_outfile_header(FILE *output_file, const InfileHeader *h, const Model **models, uint64_t steps_count);
int read_ts05_params(FILE *input_file, ModelsParams *params);
int read_t96_params(FILE *input_file, ModelsParams *params);
int read_field_infile_header(FILE *input_file, InfileHeader *h);
int write_field_outfile_header(FILE *output_file, const InfileHeader *h, const Model **models);

/* cli_models.c -- src/models.c */
extern const Model *internal_models[];
extern const Model *external_models[];
extern const Model *crustal_models[];
const Model *get_model(const Model **models, const char *version);
int models_setup(const Model **models, FILE *input_file, const InfileHeader *h, ModelsParams *params);
cor_model_set models_device_set(const Model **models);

/* cli_scan.c -- src/trajectory.c */
int cli_context(cor_ctx **ctx);
void trajectory_simulation_cutoff(InfileHeader *header, const Model **models, ModelsParams *models_params,
                                  FILE *outfile, uint64_t step_limit, double tu_angle, double particle_mass,
                                  uint32_t parallel);
int cli_write_scan(FILE *outfile, const InfileHeader *h, const cor_site_result *site, const uint8_t *status,
                   const cor_traj_record *records);

int trajectory_simulation(InfileHeader *header, const Model **models, ModelsParams *models_params, FILE *tragsm,
                          FILE *trasph, uint64_t step_limit, double tu_angle, double particle_mass);

/* cli_field.c -- src/field.c */
int field_simulation(const InfileHeader *header, const ModelsParams *params, const Model **models, FILE *outfile);

#endif
