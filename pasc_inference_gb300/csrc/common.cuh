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

// Float-float sums for the block and grid stages of the sweeps.  A value is the unevaluated
// sum hi + lo of two FP32 numbers (about 48 significant bits); two of them are added with
// Knuth's TwoSum on the high parts, the low parts folded into the error term, and Dekker's
// Fast2Sum to renormalise (the "double-float" addition of Dekker 1971 and of Bailey's
// double-double libraries, in FP32).  FP64 arithmetic on this part issues at a small fraction of
// the FP32 rate, and every block of a sweep reduces at the same moment, at the end of its
// tiles: eleven FP32 additions per pair keep that stage off the FP64 pipe.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_make(float v) { return FF{v, 0.f}; }

__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bv = __fsub_rn(s, a.hi);
    const float av = __fsub_rn(s, bv);
    float e = __fadd_rn(__fsub_rn(a.hi, av), __fsub_rn(b.hi, bv));  // s + e = a.hi + b.hi exactly
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    return FF{hi, __fsub_rn(e, __fsub_rn(hi, s))};
}

__device__ __forceinline__ double ff_value(FF a) { return (double)a.hi + (double)a.lo; }

template <int NV>
__device__ __forceinline__ void warp_sum_ff(FF (&v)[NV])
{
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const FF o{__shfl_down_sync(0xffffffffu, v[q].hi, off), __shfl_down_sync(0xffffffffu, v[q].lo, off)};
            v[q] = ff_add(v[q], o);
        }
    }
}

// Sums v over the block; the result is valid in thread 0.  scratch: NV * (blockDim/32) pairs.
template <int NV>
__device__ __forceinline__ void block_sum_ff(FF (&v)[NV], float2 *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    warp_sum_ff<NV>(v);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) scratch[q * nw + warp] = make_float2(v[q].hi, v[q].lo);
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            const float2 p = lane < nw ? scratch[q * nw + lane] : make_float2(0.f, 0.f);
            v[q] = FF{p.x, p.y};
        }
        warp_sum_ff<NV>(v);
    }
    __syncthreads();
}

// Block stage of a sweep's four sums (objective, d'd, neighbour differences of d, g'd) into
// the block's slot of partials (four float-float pairs, 32 bytes); then, in the block that
// finishes last, the grid stage over the nslot slots slot0 + b * stride (b < nslot) in that
// order.  Returns true in thread 0 of that block with the four sums in w.  snap_src/snap_dst
// (nullable): the last block also copies snap_bytes (a multiple of 8) from snap_src (global)
// to snap_dst (shared), all threads at once, visible to thread 0 on return.  BATCH: slots whose
// loads a thread issues before adding them (the additions stay in slot order, so the sums do
// not depend on it): one L2 latency per BATCH slots, for kernels with registers to spare.
template <int BATCH = 1>
__device__ __forceinline__ bool sweep_grid_sum4(const KahanF &f, float dd, float dAd, float gd, float2 *partials,
                                               long slot, unsigned int *ticket, unsigned int nslot, long slot0,
                                               long stride, float2 *scratch, double (&w)[4],
                                               const void *snap_src = nullptr, void *snap_dst = nullptr,
                                               int snap_bytes = 0)
{
    FF v[4] = {FF{f.s, f.c}, ff_make(dd), ff_make(dAd), ff_make(gd)};
    block_sum_ff<4>(v, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++) partials[slot * 4 + q] = make_float2(v[q].hi, v[q].lo);
    }
    __shared__ bool am_last4;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last4 = (atomicAdd(ticket, 1u) == nslot - 1);
    __syncthreads();
    if (!am_last4) return false;
    __threadfence();
    if (snap_dst) {
        const unsigned long long *src = reinterpret_cast<const unsigned long long *>(snap_src);
        unsigned long long *dst = reinterpret_cast<unsigned long long *>(snap_dst);
        for (int q = threadIdx.x; q < snap_bytes / 8; q += blockDim.x) dst[q] = __ldcg(src + q);
    }
    FF u[4] = {ff_make(0.f), ff_make(0.f), ff_make(0.f), ff_make(0.f)};
    if constexpr (BATCH == 1) {
        for (long b = threadIdx.x; b < (long)nslot; b += blockDim.x) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const float2 p = __ldcg(partials + (slot0 + b * stride) * 4 + q);
                u[q] = ff_add(u[q], FF{p.x, p.y});
            }
        }
    } else {
        for (long b0 = threadIdx.x; b0 < (long)nslot; b0 += BATCH * (long)blockDim.x) {
            float2 p[BATCH][4];
#pragma unroll
            for (int r = 0; r < BATCH; r++) {
                const long b = b0 + r * (long)blockDim.x;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    p[r][q] = b < (long)nslot ? __ldcg(partials + (slot0 + b * stride) * 4 + q) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int r = 0; r < BATCH; r++) {
                if (b0 + r * (long)blockDim.x >= (long)nslot) break;
#pragma unroll
                for (int q = 0; q < 4; q++) u[q] = ff_add(u[q], FF{p[r][q].x, p[r][q].y});
            }
        }
    }
    block_sum_ff<4>(u, scratch);
    if (threadIdx.x != 0) return false;
#pragma unroll
    for (int q = 0; q < 4; q++) w[q] = ff_value(u[q]);
    return true;
}

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
