// cuda_shim.h -- TEST INFRASTRUCTURE: the few CUDA qualifiers and intrinsics
// the device code uses, defined for a host C++ compiler, so that the field
// models and the scan's per-trajectory functions (cor-model_gb300/csrc/*.cuh)
// compile as host code (tests/device_on_host/field_host.cpp).  Every standard header is included
// before the qualifier macros are defined, so the macros never reach a
// library header.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <barrier>
#include <cmath>
#include <thread>
#include <vector>

#define __host__
#define __device__
#define __global__
#define __constant__
#define __forceinline__ inline __attribute__((always_inline))
#define __noinline__ __attribute__((noinline))
#define __restrict__ __restrict
#define __shared__
#define __align__(n) __attribute__((aligned(n)))
#define __launch_bounds__(...)

template <class T>
static inline T __ldg(const T* p) { return *p; }
// Each operation rounded once, as on the device: the file is compiled with
// -ffp-contract=off, so a*b is never fused into a neighbouring add.
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }

// Warp emulation for the crustal field's warp-cooperative sum (chaos.cuh):
// 32 host threads stand for the lanes of one warp (each sets its own
// threadIdx.x), and while they run, shim_warp points at their exchange
// slots and barrier.  Shuffles and ballots write the lane's value to its
// slot, wait for all 32 lanes, read, and wait again before the slots are
// reused: the semantics of a converged warp, which chaos_geo_warp requires.
struct ShimDim3 {
    unsigned x, y, z;
};
static thread_local ShimDim3 threadIdx = {0, 0, 0};
static const ShimDim3 blockIdx = {0, 0, 0}, blockDim = {32, 1, 1};

struct ShimWarp {
    std::barrier<> bar{32};
    uint64_t slot[32];
};
static ShimWarp* shim_warp = nullptr;

// Block emulation for the lane regrouping (regroup_lanes, trace.cuh): 256
// host threads stand for a block's threads; __syncthreads waits on the block
// barrier and each warp's ballots go through its own ShimWarp.  While
// shim_block is set it takes the place of shim_warp.
struct ShimBlock {
    std::barrier<> bar{256};
    ShimWarp warps[8];
};
static ShimBlock* shim_block = nullptr;
static inline ShimWarp* shim_my_warp() { return shim_block ? &shim_block->warps[(threadIdx.x >> 5) & 7] : shim_warp; }

template <class T>
static inline T shim_exchange(T v, int src) {
    static_assert(sizeof(T) <= 8, "exchange of at most 8 bytes");
    ShimWarp* w = shim_my_warp();
    if (!w) abort();
    uint64_t b = 0;
    memcpy(&b, &v, sizeof(T));
    w->slot[threadIdx.x & 31] = b;
    w->bar.arrive_and_wait();
    const uint64_t r = w->slot[src & 31];
    w->bar.arrive_and_wait();
    T out;
    memcpy(&out, &r, sizeof(T));
    return out;
}
template <class T>
static inline T __shfl_sync(unsigned, T v, int src, int = 32) { return shim_exchange(v, src); }
template <class T>
static inline T __shfl_xor_sync(unsigned, T v, int o, int = 32) { return shim_exchange(v, (int)(threadIdx.x & 31) ^ o); }
static inline unsigned __ballot_sync(unsigned, int p) {
    ShimWarp* w = shim_my_warp();
    if (!w) abort();
    w->slot[threadIdx.x & 31] = p != 0;
    w->bar.arrive_and_wait();
    unsigned m = 0;
    for (int l = 0; l < 32; l++)
        if (w->slot[l]) m |= 1u << l;
    w->bar.arrive_and_wait();
    return m;
}
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }

// The scan kernel's queue and block-wide decisions (trace.cuh) are not run
// on the host (field_host.cpp drives the per-trajectory functions directly);
// these let the header compile and abort if they are ever called.
template <class T>
static inline T __shfl_down_sync(unsigned, T, unsigned, int = 32) { abort(); }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
static inline void __syncwarp(unsigned = 0xffffffffu) { abort(); }
static inline int __syncthreads_count(int) { abort(); }
static inline int __syncthreads_or(int) { abort(); }
static inline void __syncthreads() {
    if (!shim_block) abort();
    shim_block->bar.arrive_and_wait();
}
template <class T>
static inline T atomicAdd(T*, T) { abort(); }
