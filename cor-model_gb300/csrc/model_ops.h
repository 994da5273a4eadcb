// model_ops.h -- per-model-set entry points.  Each compile-time model set
// (internal / external / crustal combination) is instantiated in its own
// translation unit (inst_*.cu) so they compile in parallel; the host code
// reaches them through this table.
#pragma once

#include <cuda_runtime.h>

#include "stream.cuh"

namespace cor {

struct ModelOps {
    int key;  // internal*100 + external*10 + crustal (negative for run-time choices)
    cudaError_t (*occupancy)(int* blocks_per_sm);
    cudaError_t (*launch_generation)(const TraceArgs& a, unsigned blocks, cudaStream_t s);
    cudaError_t (*launch_field)(const DevParams* params, int n_params, const int32_t* pidx, const double* pos,
                                int64_t n, double* out, CrustalTables crust, cudaStream_t s);
    // copies the host-derived constant blocks into this unit's constant memory
    cudaError_t (*upload_tables)(const T96Tables* t96, const TS05Tables* ts05);
    // the persistent stream kernel (stream.cuh)
    cudaError_t (*stream_occupancy)(int* blocks_per_sm);
    cudaError_t (*launch_stream)(const StreamArgs& a, unsigned blocks, cudaStream_t s);
};

extern const ModelOps ops_igrf, ops_igrf_t96, ops_t96, ops_igrf_ts05, ops_ts05, ops_crustal;

}  // namespace cor
