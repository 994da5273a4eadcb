// count_main.cpp -- TEST INFRASTRUCTURE: runs the op-counting oracle on a
// sample of single-rigidity scans read from a binary file and prints the
// totals (accepted steps, RK trials, FP64 operations, transcendentals).
//
// usage: count_ops <jobs.bin> <params.bin> <internal> <external> <crustal>
#include <stdio.h>

#include "../cor_oracle.h"

thread_local FlopTally g_tally;

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    FILE* fj = fopen(argv[1], "rb");
    FILE* fp = fopen(argv[2], "rb");
    if (!fj || !fp) return 3;
    fseek(fj, 0, SEEK_END);
    const long nj = ftell(fj) / (long)sizeof(cor_scan_job);
    fseek(fj, 0, SEEK_SET);
    cor_scan_job* jobs = (cor_scan_job*)malloc(sizeof(cor_scan_job) * nj);
    cor_model_params params;
    if (fread(jobs, sizeof(cor_scan_job), nj, fj) != (size_t)nj) return 4;
    if (fread(&params, sizeof params, 1, fp) != 1) return 5;
    cor_model_set ms = {atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), 0};
    uint64_t steps = 0, trials = 0, ops = 0, trans = 0, by_class[FC_N] = {0};
    for (long j = 0; j < nj; j++) {
        cor_counters c;
        memset(&c, 0, sizeof c);
        cor_site_result site;
        g_tally = FlopTally();
        orc_scan_job(&jobs[j], &params, ms, 25000, 0.01, 1.6725e-27, &site, NULL, NULL, &c);
        steps += c.accepted_steps;
        trials += c.trials;
        ops += g_tally.ops;
        trans += g_tally.trans;
        for (int k = 0; k < FC_N; k++) by_class[k] += g_tally.by_class[k];
    }
    static const char* names[FC_N] = {"add", "mul", "div", "sqrt", "exp", "log", "sin", "cos", "tan", "atan", "asin",
                                      "atan2", "pow", "fmod"};
    printf("{\"scans\": %ld, \"accepted_steps\": %llu, \"trials\": %llu, \"ops\": %llu, \"transcendentals\": %llu",
           nj, (unsigned long long)steps, (unsigned long long)trials, (unsigned long long)ops,
           (unsigned long long)trans);
    printf(", \"by_class\": {");
    for (int k = 0; k < FC_N; k++) printf("%s\"%s\": %llu", k ? ", " : "", names[k], (unsigned long long)by_class[k]);
    printf("}}\n");
    return 0;
}
