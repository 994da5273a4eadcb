// inst.cuh -- instantiates the kernels of one model set and its ModelOps.
#pragma once

#include "model_ops.h"

#define COR_MODEL_INSTANCE(NAME, I, E, C)                                                                  \
    namespace cor {                                                                                        \
    using MS_##NAME = ModelSet<I, E, C>;                                                                   \
    static cudaError_t occ_##NAME(int* n) {                                                                \
        cudaError_t e = cudaFuncSetAttribute(trace_kernel<MS_##NAME>,                                      \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRegroupSmem); \
        if (e != cudaSuccess) return e;                                                                    \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, trace_kernel<MS_##NAME>, kTraceThreads,    \
                                                             kRegroupSmem);                                \
    }                                                                                                      \
    static cudaError_t gen_##NAME(const TraceArgs& a, unsigned blocks, cudaStream_t s) {                   \
        cudaError_t e = cudaFuncSetAttribute(trace_kernel<MS_##NAME>,                                      \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRegroupSmem); \
        if (e != cudaSuccess) return e;                                                                    \
        trace_kernel<MS_##NAME><<<blocks, kTraceThreads, kRegroupSmem, s>>>(a);                            \
        return cudaGetLastError();                                                                         \
    }                                                                                                      \
    static cudaError_t socc_##NAME(int* n) {                                                               \
        cudaError_t e = cudaFuncSetAttribute(stream_kernel<MS_##NAME>,                                     \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRegroupSmem); \
        if (e != cudaSuccess) return e;                                                                    \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stream_kernel<MS_##NAME>, kTraceThreads,   \
                                                             kRegroupSmem);                              \
    }                                                                                                      \
    static cudaError_t stream_##NAME(const StreamArgs& a, unsigned blocks, cudaStream_t s) {               \
        cudaError_t e = cudaFuncSetAttribute(stream_kernel<MS_##NAME>,                                     \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRegroupSmem); \
        if (e != cudaSuccess) return e;                                                                    \
        stream_kernel<MS_##NAME><<<blocks, kTraceThreads, kRegroupSmem, s>>>(a);                         \
        return cudaGetLastError();                                                                         \
    }                                                                                                      \
    static cudaError_t field_##NAME(const DevParams* p, int np, const int32_t* idx, const double* pos,     \
                                    int64_t n, double* out, CrustalTables crust, cudaStream_t s) {         \
        const unsigned blocks = (unsigned)((n + 127) / 128);                                               \
        field_kernel<MS_##NAME><<<blocks, 128, 0, s>>>(p, np, idx, pos, n, out, crust);                    \
        return cudaGetLastError();                                                                         \
    }                                                                                                      \
    static cudaError_t tables_##NAME(const T96Tables* t96, const TS05Tables* ts05) {                       \
        cudaError_t e = cudaMemcpyToSymbol(c_t96, t96, sizeof(T96Tables));                                 \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ts05, ts05, sizeof(TS05Tables));                    \
        return e;                                                                                          \
    }                                                                                                      \
    const ModelOps ops_##NAME = {I * 100 + E * 10 + C, occ_##NAME, gen_##NAME, field_##NAME, tables_##NAME, \
                                 socc_##NAME, stream_##NAME};                                               \
    }
