// cuda_shim.h -- TEST INFRASTRUCTURE: the few CUDA qualifiers and intrinsics
// the device field code uses, defined for a host C++ compiler, so that
// cor-model_gb300/csrc/{cor_device,t96,ts05,field}.cuh compile as host code
// (tests/device_on_host/field_host.cpp).  Every standard header is included
// before the qualifier macros are defined, so the macros never reach a
// library header.
#pragma once

#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>

#define __host__
#define __device__
#define __global__
#define __constant__
#define __forceinline__ inline __attribute__((always_inline))
#define __noinline__ __attribute__((noinline))
#define __restrict__ __restrict
#define __launch_bounds__(...)

template <class T>
static inline T __ldg(const T* p) { return *p; }
// Each operation rounded once, as on the device: the file is compiled with
// -ffp-contract=off, so a*b is never fused into a neighbouring add.
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }

// Warp and block intrinsics of the crustal field's warp-cooperative sum
// (chaos.cuh) and of the scan kernel's queue and block-wide decisions
// (trace.cuh).  They let those headers compile; neither the crustal model nor
// the kernel runs on the host (field_host.cpp drives the per-trajectory
// functions directly), and these abort if they ever are called.
struct ShimDim3 {
    unsigned x, y, z;
};
static const ShimDim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1};
static inline unsigned __ballot_sync(unsigned, int) { abort(); }
static inline int __ffs(unsigned) { abort(); }
template <class T>
static inline T __shfl_sync(unsigned, T, int, int = 32) { abort(); }
template <class T>
static inline T __shfl_xor_sync(unsigned, T, int, int = 32) { abort(); }
template <class T>
static inline T __shfl_down_sync(unsigned, T, unsigned, int = 32) { abort(); }
static inline int __popc(unsigned) { abort(); }
static inline void __syncwarp(unsigned = 0xffffffffu) { abort(); }
static inline int __syncthreads_count(int) { abort(); }
static inline int __syncthreads_or(int) { abort(); }
template <class T>
static inline T atomicAdd(T*, T) { abort(); }
