// common.cuh -- shared device helpers for the 2CLOWNS-3D GB300 pressure solve.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "clowns_gpu.h"

namespace clowns {

constexpr int kWarp = 32;
constexpr int kNumSMs = 152;   // GB300: 2 dies x 76 SMs

// Fixed constants of the reference (src2LOWNS/0mod-variables.F90:32-44).
constexpr double kTiny = 1.0e-15;
constexpr double kSmall = 1.0e-9;

#define CLOWNS_CUDA_TRY(expr)                                                      \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            clowns::set_last_error(_e, #expr, __FILE__, __LINE__);                 \
            return CLOWNS_ERR_CUDA;                                                \
        }                                                                          \
    } while (0)

void set_last_error(cudaError_t e, const char* what, const char* file, int line);
void set_last_error_msg(const char* msg);

static inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
static inline int div_up(long a, long b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// Warp / block reductions (fixed tree order => deterministic for a fixed launch)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums of two values over a warp at the cost of one: lanes exchange across the
// half-warps first, so that lanes 0-15 go on summing a and lanes 16-31 summing b
// (5 additions per lane instead of 10).  Returns a's total in lanes 0-15 and b's
// in lanes 16-31.  Fixed order: deterministic.
template <typename A>
__device__ __forceinline__ A warp_pair_sum(A a, A b) {
    const bool hi = (threadIdx.x & 16) != 0;
    A keep = hi ? b : a;
    const A send = hi ? a : b;
    keep += __shfl_xor_sync(0xffffffffu, send, 16);
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
    return keep;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* >= 32*NV */) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) smem[q * 32 + wid] = v[q];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double t = lane < nw ? smem[q * 32 + lane] : 0.0;
            v[q] = warp_sum(t);
        }
    }
    __syncthreads();
}

// Sum `count` partial records of NV doubles (stride NV) in a fixed order with one
// warp.  Every lane returns the same totals.
template <int NV>
__device__ __forceinline__ void warp_sum_partials(const double* partials, int count, double (&out)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = 0.0;
    for (int b = lane; b < count; b += 32) {
#pragma unroll
        for (int q = 0; q < NV; q++) out[q] += __ldcg(partials + (size_t)b * NV + q);
    }
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = warp_sum(out[q]);
}

// Streaming loads that should not displace the vectors held in L2.
__device__ __forceinline__ double ld_stream(const double* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float* p) { return __ldcs(p); }

}  // namespace clowns
