// project.cuh -- per-timestep Euclidean projection onto the K-simplex {y >= 0, sum y = 1}.
//
// Algorithm of the reference (include/general/algebra/feasibleset/simplex_local.h:176-246,
// device version src/petscvector/algebra/feasibleset/simplex_local.cu:70-139):
//   a block that is already feasible (no entry < 0 and an exact sum of 1) is left untouched;
//   otherwise sort ascending, scan i = K-1 .. 1 for the first t_i = (sum_{j>=i} y_j - 1)/(K-i)
//   with t_i >= y_{i-1}; if none, t = (sum(x) - 1)/K; result max(x - t, 0).
//
// Three GB300 forms:
//   project_ref_f64   FP64, the reference's exact operation order (bubble sort, suffix sums
//                     recomputed from y_i upwards); used by the plain FP64 path, bit-identical
//                     to the CPU restatement.
//   project_reg<K>    FP32, one thread per timestep, K values in registers, sorting network
//                     and an incremental suffix sum; used inside the fused SPG sweep.
//   project_group<G>  FP32, G lanes per timestep (one value per lane), ranks, suffix sums and
//                     the threshold choice exchanged with warp shuffles; used for K > 8.
#pragma once

#include "common.cuh"

namespace pasc {

// ---------------------------------------------------------------------------------------
// FP64, reference operation order.  y: caller scratch of K doubles.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ void project_ref_f64(double *x, int K, double *y)
{
    bool inside = true;
    double sum = 0.0;
    for (int k = 0; k < K; k++) {
        if (x[k] < 0.0) inside = false;
        sum = __dadd_rn(sum, x[k]);
    }
    if (sum != 1.0) inside = false;
    if (inside) return;

    for (int k = 0; k < K; k++) y[k] = x[k];
    // bubble sort with last-swap bound (simplex_local.cu:48-68)
    int m = K;
    while (m > 0) {
        int mnew = 0;
        for (int i = 1; i < m; i++) {
            if (y[i] < y[i - 1]) {
                double sw = y[i];
                y[i] = y[i - 1];
                y[i - 1] = sw;
                mnew = i;
            }
        }
        m = mnew;
    }
    double t_hat = 0.0;
    int i = K - 1;
    while (i >= 1) {
        double sum_y = 0.0;
        for (int j = i; j < K; j++) sum_y = __dadd_rn(sum_y, y[j]);
        double ti = __ddiv_rn(__dsub_rn(sum_y, 1.0), (double)(K - i));
        if (ti >= y[i - 1]) {
            t_hat = ti;
            i = -1;
        } else {
            i = i - 1;
        }
    }
    if (i == 0) t_hat = __ddiv_rn(__dsub_rn(sum, 1.0), (double)K);
    for (int k = 0; k < K; k++) {
        double ti = __dsub_rn(x[k], t_hat);
        x[k] = ti > 0.0 ? ti : 0.0;
    }
}

// ---------------------------------------------------------------------------------------
// FP32, one thread per timestep, compile-time K.
// ---------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void cswap(float (&s)[K], int a, int b)
{
    float lo = fminf(s[a], s[b]), hi = fmaxf(s[a], s[b]);
    s[a] = lo;
    s[b] = hi;
}

template <int K>
__device__ __forceinline__ void sort_net(float (&s)[K])
{
    // odd-even transposition network: K rounds, fully unrolled
#pragma unroll
    for (int r = 0; r < K; r++) {
#pragma unroll
        for (int a = (r & 1); a + 1 < K; a += 2) cswap<K>(s, a, a + 1);
    }
}

// The reference's threshold (the first t_i from the top with t_i >= y_{i-1}) equals the
// largest of all candidates t_i = (sum of the K-i largest entries - 1)/(K-i): every candidate
// is a lower bound of the threshold (sum_k max(y_k - t, 0) >= 1 at t = t_i) and the one of the
// active set attains it.  Taking the maximum needs no search and no branch; for K <= 3 it
// needs no sort either (the largest, the sum minus the smallest, the sum).  An already
// feasible block yields t = 0 and is returned unchanged, as in the reference's early exit.
// The divisions are multiplications by compile-time reciprocals (within one ulp), fused with
// the subtraction of 1.
template <int K>
__device__ __forceinline__ void project_reg(float (&x)[K])
{
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) sum += x[k];
    // (s - 1)/j is taken as fmaf(s, 1/j, -1/j): one rounding of the exact c*s - c (zero at
    // s = 1 exactly, so a feasible block keeps t = 0).  fmaxf drops NaN operands: the last
    // candidate, the one over all K entries, is merged by a comparison instead, so that a block
    // holding a NaN (a NaN sum) gets a NaN threshold and becomes all zeros, as in the reference
    // (whose comparisons with NaN all fail).
    float tau;
    if (K == 1) {
        tau = sum - 1.f;
    } else if (K == 2) {
        const float t1 = fmaxf(x[0], x[1]) - 1.f, t2 = fmaf(sum, 0.5f, -0.5f);
        tau = t1 >= t2 ? t1 : t2;
    } else if (K == 3) {
        const float mx = fmaxf(fmaxf(x[0], x[1]), x[2]);
        const float mn = fminf(fminf(x[0], x[1]), x[2]);
        const float t12 = fmaxf(mx - 1.f, fmaf(sum - mn, 0.5f, -0.5f));
        const float t3 = fmaf(sum, 1.f / 3.f, -1.f / 3.f);
        tau = t12 >= t3 ? t12 : t3;
    } else {
        float s[K];
#pragma unroll
        for (int k = 0; k < K; k++) s[k] = x[k];
        sort_net<K>(s);
        float acc = 0.f;
        tau = -FLT_MAX;
#pragma unroll
        for (int i = K - 1; i >= 1; i--) {
            acc += s[i];
            tau = fmaxf(tau, fmaf(acc, 1.f / (float)(K - i), -1.f / (float)(K - i)));
        }
        const float tk = fmaf(sum, 1.f / (float)K, -1.f / (float)K);
        tau = tau >= tk ? tau : tk;
    }
#pragma unroll
    for (int k = 0; k < K; k++) x[k] = fmaxf(x[k] - tau, 0.f);
}

// ---------------------------------------------------------------------------------------
// FP32, G lanes per timestep (G a power of two, 2..32), lane k of the group holds x_k for
// k < K.  All lanes of the warp must call it (shuffles use the full mask); lanes whose group
// has no valid timestep pass valid = false.
// ---------------------------------------------------------------------------------------
template <int G>
__device__ __forceinline__ float project_group(float v, int K, bool valid)
{
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);            // lane within group
    const int base = lane & ~(G - 1);         // first lane of group
    const bool act = valid && gl < K;

    // feasibility and total sum (butterfly within the group: identical result in every lane)
    float sum = act ? v : 0.f;
    int neg = (act && v < 0.f) ? 1 : 0;
#pragma unroll
    for (int off = 1; off < G; off <<= 1) {
        sum = __fadd_rn(sum, __shfl_xor_sync(0xffffffffu, sum, off));
        neg |= __shfl_xor_sync(0xffffffffu, neg, off);
    }
    const bool inside = (neg == 0) && (sum == 1.f);

    // stable ascending rank of this lane's value among the K valid lanes
    int rank = 0;
    for (int j = 0; j < G; j++) {
        float vj = __shfl_sync(0xffffffffu, v, base + j);
        if (j < K && act) {
            if (vj < v || (vj == v && j < gl)) rank++;
        }
    }
    // suffix sum over ranks >= my rank, and the value of rank-1
    float suf = 0.f, below = -FLT_MAX;
    for (int j = 0; j < G; j++) {
        float vj = __shfl_sync(0xffffffffu, v, base + j);
        int rj = __shfl_sync(0xffffffffu, rank, base + j);
        if (j < K && act) {
            if (rj >= rank) suf = __fadd_rn(suf, vj);
            if (rj == rank - 1) below = vj;
        }
    }
    // candidate: rank r >= 1 with t_r >= y_{r-1}; the reference takes the largest such r
    float tr = act && rank >= 1 ? __fdiv_rn(__fsub_rn(suf, 1.f), (float)(K - rank)) : 0.f;
    int cand = (act && rank >= 1 && tr >= below) ? rank : -1;
    int best = cand;
#pragma unroll
    for (int off = 1; off < G; off <<= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, off));
    // broadcast t of the winning lane
    float tau = __fdiv_rn(__fsub_rn(sum, 1.f), (float)K);
    for (int j = 0; j < G; j++) {
        float tj = __shfl_sync(0xffffffffu, tr, base + j);
        int cj = __shfl_sync(0xffffffffu, cand, base + j);
        if (best >= 0 && cj == best) tau = tj;
    }
    if (!act || inside) return v;
    float r = __fsub_rn(v, tau);
    return r > 0.f ? r : 0.f;
}

}  // namespace pasc
