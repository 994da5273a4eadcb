// depth_main.cpp -- TEST INFRASTRUCTURE: runs the depth-tracking oracle
// (depth.hpp) on single-rigidity scans read from a binary file and prints,
// per trajectory, its accepted steps, its FP64 instructions and the length
// of its longest dependent chain, as JSON lines.
//
// usage: count_depth <jobs.bin> <params.bin> <internal> <external> <crustal>
#include <stdio.h>

#include "../cor_oracle.h"

thread_local DepTally g_dep;
const DepWeights g_w;

// The ABI layouts with plain doubles, as the files hold them.
struct RawJob {
    raw_double r0, the0, fi0, the1, fi1, rig, del, rk, zn;
    int32_t nk1, param_index, i_first, i_count;
};
struct RawParams {
    raw_double parmod[10], g[COR_SH_COEFS], h[COR_SH_COEFS], rec[COR_SH_COEFS], a1[3], a2[3], a3[3];
};
static_assert(sizeof(RawJob) == 88 && sizeof(RawParams) == 8 * (10 + 3 * COR_SH_COEFS + 9), "ABI layouts");

int main(int argc, char** argv) {
    if (argc < 6) return 2;
    FILE* fj = fopen(argv[1], "rb");
    FILE* fp = fopen(argv[2], "rb");
    if (!fj || !fp) return 3;
    fseek(fj, 0, SEEK_END);
    const long nj = ftell(fj) / (long)sizeof(RawJob);
    fseek(fj, 0, SEEK_SET);
    RawJob* raw = (RawJob*)malloc(sizeof(RawJob) * nj);
    RawParams rp;
    if (fread(raw, sizeof(RawJob), nj, fj) != (size_t)nj) return 4;
    if (fread(&rp, sizeof rp, 1, fp) != 1) return 5;
    cor_model_params p;
    for (int k = 0; k < 10; k++) p.parmod[k] = rp.parmod[k];
    for (int k = 0; k < COR_SH_COEFS; k++) {
        p.g[k] = rp.g[k];
        p.h[k] = rp.h[k];
        p.rec[k] = rp.rec[k];
    }
    for (int k = 0; k < 3; k++) {
        p.a1[k] = rp.a1[k];
        p.a2[k] = rp.a2[k];
        p.a3[k] = rp.a3[k];
    }
    const cor_model_set ms = {atoi(argv[3]), atoi(argv[4]), atoi(argv[5]), 0};
    for (long j = 0; j < nj; j++) {
        const RawJob& r = raw[j];
        cor_scan_job job;
        job.r0 = r.r0; job.the0 = r.the0; job.fi0 = r.fi0; job.the1 = r.the1; job.fi1 = r.fi1;
        job.rig = r.rig; job.del = r.del; job.rk = r.rk; job.zn = r.zn;
        job.nk1 = r.nk1; job.param_index = r.param_index; job.i_first = r.i_first; job.i_count = r.i_count;
        cor_counters c;
        memset(&c, 0, sizeof c);
        cor_site_result site;
        g_dep = DepTally();
        orc_scan_job(&job, &p, ms, 25000, 0.01, 1.6725e-27, &site, NULL, NULL, &c);
        printf("{\"steps\": %llu, \"trials\": %llu, \"issue\": %.1f, \"critical\": %.1f, \"ops\": %llu}\n",
               (unsigned long long)c.accepted_steps, (unsigned long long)c.trials, g_dep.issue, g_dep.max,
               (unsigned long long)g_dep.ops);
    }
    return 0;
}
