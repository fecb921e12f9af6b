// common.cuh -- shared device helpers for the GB300 FEM-H1 / SPG-QP library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <float.h>

#include "pasc_gb300.h"

namespace pasc {

// Largest K the register-resident (fused) kernels are instantiated for; larger K runs the
// lane-group kernels.
constexpr int KMAX_FUSED = 8;
// Largest K any kernel accepts (lane-group projection holds one value per lane).
constexpr int KMAX_GROUP = 32;
// Largest K the plain FP64 projection accepts (its sort buffer is thread-local).
constexpr int KMAX_PLAIN = 128;
// Largest GLL memory length.
constexpr int MMAX = 64;

// ---------------------------------------------------------------------------------------
// Block-level reductions (deterministic: fixed shuffle tree, fixed warp order).
// ---------------------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV])
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int q = 0; q < NV; q++) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
    }
}

// Sums v over the block; the result is valid in thread 0.  scratch: NV * (blockDim/32) doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    warp_sum<NV>(v);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) scratch[q * nw + warp] = v[q];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) v[q] = lane < nw ? scratch[q * nw + lane] : 0.0;
        warp_sum<NV>(v);
    }
    __syncthreads();
}

// Compensated (Neumaier) FP32 accumulator: per-thread sums stay in FP32 arithmetic (FP64
// throughput on this part is a small fraction of FP32) while keeping about twice the
// significand; it is widened to FP64 for the block and grid stages.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float v)
    {
        float t = __fadd_rn(s, v);
        if (fabsf(s) >= fabsf(v)) c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, t), v));
        else c = __fadd_rn(c, __fadd_rn(__fsub_rn(v, t), s));
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

// Last-block-done ticket: returns true in every thread of the block that finished last.
// partials must already be written and fenced by the caller.
__device__ __forceinline__ bool last_block_done(unsigned int *counter)
{
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int ticket = atomicAdd(counter, 1u);
        am_last = (ticket == gridDim.x - 1);
    }
    __syncthreads();
    if (am_last) __threadfence();
    return am_last;
}

// Same for a counter shared by n participants (e.g. the segments of one signal): true in the
// block that arrives n-th.
__device__ __forceinline__ bool last_block_done_count(unsigned int *counter, unsigned int n)
{
    __shared__ bool am_last_n;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last_n = (atomicAdd(counter, 1u) == n - 1);
    __syncthreads();
    if (am_last_n) __threadfence();
    return am_last_n;
}

}  // namespace pasc
