/*
 * cli_main.c -- the drop-in `cor` program: the reference's command line
 * (src/args.c:11-78) and cutoff() driver (src/main.c:12-94, :257-315), with
 * the rigidity scan on the GPU through libcortrace.  One extra option, -b
 * MANIFEST, traces many INFILEs in a single GPU call (each manifest line is
 * "INFILE OUTFILE"; every output file has the single-run format).
 */
#include <argp.h>
#include <errno.h>
#include <limits.h>
#include <stdlib.h>
#include <string.h>

#include "cli.h"

const char *argp_program_version = "cor-model 3.0 (GB300 scan)";

static const char doc[] = "Trajectory simulation of cosmic ray particle in Earth's magnetosphere";
static const char args_doc[] = "INFILE";

static struct argp_option options[] = {
    { "par", 'p', 0, 0, "Parallel computation (the scan always runs on the GPU)" },
    { "output", 'o', "FILE", 0, "Output to FILE instead of standard output." },
    { "steps-count", 's', "COUNT", 0, "Maximal single trajectory steps count (default: 25000)" },
    { "tu-angle", 'u', "RAD", 0, "TU angle, specifies the precision of the trajectory calculation (default: 0.01 rad)" },
    { "mode", 'm', "MODE", 0, "Calculation mode: cutoff, field, trajectory (default: cutoff)" },
    { "particle-type", 't', "TYPE", 0, "Particle type: electron or proton (default: proton)" },
    { "batch", 'b', "MANIFEST", 0, "Trace every 'INFILE OUTFILE' pair listed in MANIFEST in one GPU call" },
    { 0, 0, 0, 0, "Geomagnetic field models:" },
    { "internal-field", 'i', "MODEL", 0, "Use internal field model: igrf9-14, hist, cals10k.2 (default: igrf14)" },
    { "external-field", 'e', "MODEL", 0, "Use external field model: ts05, t96 (default: none)" },
    { "crustal-field", 'c', "MODEL", 0, "Use crustal field model: chaos7.16 (default: none)" },
    { 0 }
};

static error_t parse_opt(int key, char *arg, struct argp_state *state) {
    CLIArguments *a = state->input;
    switch (key) {
        case 'p': a->options |= OPT_PARALLEL; break;
        case 'o': a->output_file_name = arg; break;
        case 's': a->steps_count = arg; break;
        case 'u': a->tu_angle = arg; break;
        case 'm': a->mode = arg; break;
        case 't': a->particle_type = arg; break;
        case 'b': a->batch_file_name = arg; break;
        case 'i': a->internal_model_name = arg; break;
        case 'e': a->external_model_name = arg; break;
        case 'c': a->crustal_model_name = arg; break;
        case ARGP_KEY_ARG:
            if (state->arg_num >= 1) argp_usage(state);
            a->input_file_name = arg;
            break;
        case ARGP_KEY_END:
            if (state->arg_num < 1 && !a->batch_file_name) argp_usage(state);
            break;
        default: return ARGP_ERR_UNKNOWN;
    }
    return 0;
}

/* src/utils.c:8-26 */
static int string_to_uint64(const char *s, uint64_t *num) {
    char *end;
    errno = 0;
    *num = strtoul(s, &end, 10);
    if (end == s || *end != '\0' || errno == ERANGE) return -1;
    return 0;
}

static int string_to_double(const char *s, double *num) {
    char *end;
    errno = 0;
    *num = strtod(s, &end);
    if (end == s || *end != '\0' || errno == ERANGE) return -1;
    return 0;
}

typedef struct {
    uint64_t steps;
    double tu_angle;
    double mass;
} RunOptions;

static int run_options(const CLIArguments *args, RunOptions *o) {
    o->steps = 25000; /* src/main.c:13 */
    if (args->steps_count && string_to_uint64(args->steps_count, &o->steps) == -1) {
        fprintf(stderr, "Error: Invalid steps count '%s'\n", args->steps_count);
        return 1;
    }
    o->tu_angle = .01; /* src/main.c:19 */
    if (args->tu_angle && string_to_double(args->tu_angle, &o->tu_angle) == -1) {
        fprintf(stderr, "Error: Invalid TU angle '%s'\n", args->tu_angle);
        return 1;
    }
    o->mass = DEF_HM0_P;
    if (strcmp(args->particle_type, "electron") == 0) o->mass = DEF_HM0_E;
    return 0;
}

/* Reads one INFILE with its model parameters (src/main.c:32-67). */
static int load_infile(const char *path, const Model **models, InfileHeader *h, ModelsParams *p) {
    FILE *f = fopen(path, "r");
    if (!f) {
        perror("Error: Cannot open input file for reading");
        return 1;
    }
    memset(p, 0, sizeof *p);
    if (read_cutoff_infile_header(f, h) != 0) {
        fprintf(stderr, "Error: Invalid input file\n");
        fclose(f);
        return 1;
    }
    if (h->del <= 0.) {
        fprintf(stderr, "Error: Rigidity step size must be bigger than 0\n");
        fclose(f);
        return 1;
    }
    if (models_setup(models, f, h, p) != 0) {
        fprintf(stderr, "Error: Invalid input file\n");
        fclose(f);
        return 1;
    }
    if (fclose(f) != 0) {
        perror("Error: Cannot close input file");
        return 1;
    }
    return 0;
}

static int cutoff(const CLIArguments *args, const Model **models) {
    RunOptions o;
    if (run_options(args, &o)) return 1;
    InfileHeader h = {0};
    ModelsParams p;
    if (load_infile(args->input_file_name, models, &h, &p)) return 1;
    FILE *out = stdout;
    if (args->output_file_name) {
        out = fopen(args->output_file_name, "w");
        if (!out) {
            perror("Error: Cannot open output file for writing");
            return 1;
        }
    }
    if (write_cutoff_outfile_header(out, &h, models, o.steps) != 0) {
        fprintf(stderr, "Error: Cannot write output file header\n");
        if (out != stdout) fclose(out);
        return 1;
    }
    trajectory_simulation_cutoff(&h, models, &p, out, o.steps, o.tu_angle, o.mass, args->options & OPT_PARALLEL);
    if (out != stdout && fclose(out) != 0) {
        perror("Error: Cannot close output file");
        return 1;
    }
    return 0;
}

/* `-m field` (src/main.c:96-155): the field on a latitude/longitude grid. */
static int field(const CLIArguments *args, const Model **models) {
    FILE *f = fopen(args->input_file_name, "r");
    if (!f) {
        perror("Error: Cannot open input file for reading");
        return 1;
    }
    InfileHeader h = {0};
    ModelsParams p;
    memset(&h, 0, sizeof h);
    memset(&p, 0, sizeof p);
    if (read_field_infile_header(f, &h) != 0 || models_setup(models, f, &h, &p) != 0) {
        fprintf(stderr, "Error: Invalid input file\n");
        fclose(f);
        return 1;
    }
    if (fclose(f) != 0) {
        perror("Error: Cannot close input file");
        return 1;
    }
    FILE *out = stdout;
    if (args->output_file_name) {
        out = fopen(args->output_file_name, "w");
        if (!out) {
            perror("Error: Cannot open output file for writing");
            return 1;
        }
    }
    if (write_field_outfile_header(out, &h, models) != 0) {
        fprintf(stderr, "Error: Cannot write output file header\n");
        if (out != stdout) fclose(out);
        return 1;
    }
    const int rc = field_simulation(&h, &p, models, out);
    if (out != stdout && fclose(out) != 0) {
        perror("Error: Cannot close output file");
        return 1;
    }
    return rc;
}

/* `-m trajectory` (src/main.c:157-252): one INFILE with rig == rk, every
 * accepted step to tragsm_<OUTPUT> (GSM) and trasph_<OUTPUT> (spherical). */
static int trajectory(const CLIArguments *args, const Model **models) {
    if (!args->output_file_name) {
        fprintf(stderr, "Error: Output file name is required for trajectory calculation mode\n");
        return 1;
    }
    RunOptions o;
    if (run_options(args, &o)) return 1;
    FILE *f = fopen(args->input_file_name, "r");
    if (!f) {
        perror("Error: Cannot open input file for reading");
        return 1;
    }
    InfileHeader h = {0};
    ModelsParams p;
    memset(&h, 0, sizeof h);
    memset(&p, 0, sizeof p);
    if (read_cutoff_infile_header(f, &h) != 0) {
        fprintf(stderr, "Error: Invalid input file\n");
        fclose(f);
        return 1;
    }
    if (h.rig != h.rk) {
        fprintf(stderr, "Error: Invalid input file - starting and ending rigidity must be the same for trajectory "
                        "calculation mode\n");
        fclose(f);
        return 1;
    }
    if (models_setup(models, f, &h, &p) != 0) {
        fprintf(stderr, "Error: Invalid input file\n");
        fclose(f);
        return 1;
    }
    if (fclose(f) != 0) {
        perror("Error: Cannot close input file");
        return 1;
    }
    /* one rigidity: the step only sizes the single-point grid.  A zero step
     * makes the reference's grid count round(0/0), which yields no rigidity;
     * a negative one still gives the single point. */
    const int none = !(h.del != 0.) || h.del != h.del;
    if (h.del < 0.) h.del = -h.del;
    const size_t len = strlen(args->output_file_name);
    char *gsm_name = malloc(len + 8), *sph_name = malloc(len + 8);
    if (!gsm_name || !sph_name) return 1;
    strcpy(gsm_name, "tragsm_");
    strcat(gsm_name, args->output_file_name);
    strcpy(sph_name, "trasph_");
    strcat(sph_name, args->output_file_name);
    FILE *g = fopen(gsm_name, "w");
    if (!g) {
        perror("Error: Cannot open tragsm output file for writing");
        return 1;
    }
    FILE *s = fopen(sph_name, "w");
    if (!s) {
        fclose(g);
        perror("Error: Cannot open trasfer output file for writing");
        return 1;
    }
    const int rc = none ? 0 : trajectory_simulation(&h, models, &p, g, s, o.steps, o.tu_angle, o.mass);
    free(gsm_name);
    free(sph_name);
    if (fclose(g) != 0 || fclose(s) != 0) {
        perror("Error: Cannot close output file");
        return 1;
    }
    return rc;
}

/* -b MANIFEST: all scans in one cor_trace_batch call, one parameter block per
 * INFILE (each INFILE has its own date and external-field parameters). */
static int batch(const CLIArguments *args, const Model **models) {
    RunOptions o;
    if (run_options(args, &o)) return 1;
    FILE *mf = fopen(args->batch_file_name, "r");
    if (!mf) {
        perror("Error: Cannot open manifest");
        return 1;
    }
    int cap = 64, n = 0;
    char (*in)[4096] = malloc(sizeof(*in) * cap), (*outn)[4096] = malloc(sizeof(*outn) * cap);
    while (in && outn && fscanf(mf, "%4095s %4095s", in[n], outn[n]) == 2) {
        if (++n == cap) {
            cap *= 2;
            in = realloc(in, sizeof(*in) * cap);
            outn = realloc(outn, sizeof(*outn) * cap);
        }
    }
    fclose(mf);
    if (!in || !outn) return 1;
    InfileHeader *hs = calloc(n ? n : 1, sizeof(InfileHeader));
    ModelsParams *ps = calloc(n ? n : 1, sizeof(ModelsParams));
    cor_scan_job *jobs = calloc(n ? n : 1, sizeof(cor_scan_job));
    uint64_t *off = calloc(n + 1, sizeof(uint64_t));
    for (int i = 0; i < n; i++) {
        if (load_infile(in[i], models, &hs[i], &ps[i])) return 1;
        cor_scan_job *j = &jobs[i];
        j->r0 = hs[i].r0; j->the0 = hs[i].the0; j->fi0 = hs[i].fi0; j->the1 = hs[i].the1; j->fi1 = hs[i].fi1;
        j->rig = hs[i].rig; j->del = hs[i].del; j->rk = hs[i].rk; j->zn = hs[i].zn; j->nk1 = hs[i].nk1;
        j->param_index = i;
    }
    uint64_t total = 0;
    if (cor_batch_count(jobs, n, &total, off) != COR_OK) {
        fprintf(stderr, "Error: invalid rigidity grid in the manifest\n");
        return 1;
    }
    cor_site_result *sites = calloc(n ? n : 1, sizeof(cor_site_result));
    uint8_t *status = malloc(total ? total : 1);
    cor_traj_record *records = malloc(sizeof(cor_traj_record) * (total ? total : 1));
    cor_ctx *ctx;
    if (!sites || !status || !records || cli_context(&ctx) != COR_OK) return 1;
    cor_batch_req req = { jobs, n, n, ps, models_device_set(models), o.steps, o.tu_angle, o.mass };
    cor_batch_result res;
    memset(&res, 0, sizeof res);
    res.sites = sites;
    res.status = status;
    res.records = records;
    if (n > 0 && cor_trace_batch(ctx, &req, &res) != COR_OK) {
        fprintf(stderr, "Error: %s\n", cor_last_error_string(ctx));
        return 1;
    }
    for (int i = 0; i < n; i++) {
        FILE *out = fopen(outn[i], "w");
        if (!out) {
            perror("Error: Cannot open output file for writing");
            return 1;
        }
        write_cutoff_outfile_header(out, &hs[i], models, o.steps);
        cli_write_scan(out, &hs[i], &sites[i], status + off[i], records + off[i]);
        fclose(out);
    }
    fprintf(stderr, "traced %d scans, %llu trajectories, %llu accepted steps\n", n,
            (unsigned long long)res.counters.trajectories, (unsigned long long)res.counters.accepted_steps);
    free(in); free(outn); free(hs); free(ps); free(jobs); free(off); free(sites); free(status); free(records);
    return 0;
}

int main(int argc, char **argv) {
    CLIArguments args;
    memset(&args, 0, sizeof args);
    args.mode = "cutoff";
    args.particle_type = "proton";
    struct argp argp = { options, parse_opt, args_doc, doc, 0, 0, 0 };
    argp_parse(&argp, argc, argv, 0, NULL, &args);
    if (!args.internal_model_name && !args.external_model_name && !args.crustal_model_name)
        args.internal_model_name = "igrf14"; /* src/main.c:264-266 */
    int index = 0;
    const Model *models[4] = { NULL };
    if (args.internal_model_name) {
        const Model *m = get_model(internal_models, args.internal_model_name);
        if (!m) {
            fprintf(stderr, "Error: Invalid internal geomagnetic field model: '%s'\n", args.internal_model_name);
            return 1;
        }
        models[index++] = m;
    }
    if (args.external_model_name) {
        const Model *m = get_model(external_models, args.external_model_name);
        if (!m) {
            fprintf(stderr, "Error: Invalid external geomagnetic field model: '%s'\n", args.external_model_name);
            return 1;
        }
        models[index++] = m;
    }
    if (args.crustal_model_name) {
        const Model *m = get_model(crustal_models, args.crustal_model_name);
        if (!m) {
            fprintf(stderr, "Error: Invalid crustal geomagnetic field model: '%s'\n", args.crustal_model_name);
            return 1;
        }
        models[index++] = m;
    }
    if (strcmp(args.mode, "field") == 0) return field(&args, models);
    if (strcmp(args.mode, "trajectory") == 0) return trajectory(&args, models);
    if (strcmp(args.mode, "cutoff") != 0) {
        fprintf(stderr, "Error: Invalid calculation mode\n");
        return 1;
    }
    return args.batch_file_name ? batch(&args, models) : cutoff(&args, models);
}
