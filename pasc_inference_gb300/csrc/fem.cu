// fem.cu -- FEM temporal coarsening (GraphH1FEMModel with fem_reduce < 1): the gamma QP is
// solved on T2 = ceil(T*fem_reduce) timesteps; gamma and the residual are reduced onto the
// coarse grid before the solve and the solution is prolongated back after it.
//
//   type 0, FEM-SUM (src/petscvector/common/fem.cpp:32-115, 124-210): diff = T1/T2; coarse t2
//     sums the fine t in [round(t2*diff), round((t2+1)*diff)); prolongation copies it back.
//   type 1, FEM-HAT (src/petscvector/common/femhat.cpp:27-215, include/general/common/
//     femhat.h:154-195): diff = (T1-1)/(T2-1); reduction weights the fine values by the hat
//     function centred at t2*diff (the reference's loop bounds, which start at floor of the
//     hat's left end, kept as they are); prolongation interpolates linearly between the two
//     coarse neighbours (a neighbour past the last coarse point counts as 0).
// One thread per (coarse or fine timestep, cluster); the index arithmetic is FP64 with the
// reference's expressions and no contraction, so the block bounds are the reference's.  (The
// reference's own CUDA FEM kernels are declared under other names than the ones it calls and
// do not link; its sequential code defines the behaviour restated here.)
#include <math.h>

#include "common.cuh"
#include "internal.h"

namespace pasc {

__device__ __forceinline__ double fem_mul(long a, double b) { return __dmul_rn((double)a, b); }

// value of the fine field at (t, k): a stored field, or the residual (x_t - theta_k)^2
template <typename TIn>
struct FineField {
    const TIn *g;          // T1*K, or null
    const double *data;    // T1 (residual form)
    const double *theta;   // K
    int K;
    __device__ __forceinline__ double operator()(long t, int k) const
    {
        if (g) return (double)g[t * K + k];
        const double r = data[t] - theta[k];
        return r * r;
    }
};

template <typename TIn, typename TOut>
__global__ void fem_reduce_kernel(FineField<TIn> f, TOut *g2, long T1, long T2, int K, int type, double diff,
                                  long right_t1_idx, double scale)
{
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= T2 * K) return;
    const long t2 = idx / K;
    const int k = (int)(idx - t2 * K);
    double mysum = 0.0;
    if (type == 0) {
        const long lo = (long)round(fem_mul(t2, diff)), hi = (long)round(fem_mul(t2 + 1, diff));
        for (long i = lo; i < hi; i++) mysum = __dadd_rn(mysum, f(i, k));
    } else {
        const double center = fem_mul(t2, diff), left = fem_mul(t2 - 1, diff), right = fem_mul(t2 + 1, diff);
        long t1 = (long)floor(left), id = t1;
        while ((double)t1 <= center) {
            const double phi = __ddiv_rn(__dsub_rn((double)t1, left), __dsub_rn(center, left));
            if (id >= 0) mysum = __dadd_rn(mysum, __dmul_rn(phi, f(id, k)));
            t1 += 1;
            id += 1;
        }
        while ((double)t1 < right) {
            const double phi = __ddiv_rn(__dsub_rn((double)t1, right), __dsub_rn(center, right));
            if (id < right_t1_idx) mysum = __dadd_rn(mysum, __dmul_rn(phi, f(id, k)));
            t1 += 1;
            id += 1;
        }
    }
    g2[idx] = (TOut)__dmul_rn(mysum, scale);
}

template <typename TIn, typename TOut>
__global__ void fem_prolongate_kernel(const TIn *g2, TOut *g1, long T1, long T2, int K, int type, double diff)
{
    if (type == 0) {
        // one thread per coarse (t2, k), writing its block
        const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
        if (idx >= T2 * K) return;
        const long t2 = idx / K;
        const int k = (int)(idx - t2 * K);
        const long lo = (long)round(fem_mul(t2, diff)), hi = (long)round(fem_mul(t2 + 1, diff));
        const TIn v = g2[idx];
        for (long i = lo; i < hi; i++) g1[i * K + k] = (TOut)v;
        return;
    }
    const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (idx >= T1 * K) return;
    const long t1 = idx / K;
    const int k = (int)(idx - t1 * K);
    const long l = (long)floor(__ddiv_rn((double)t1, diff)), r = l + 1;
    const double t1_left = fem_mul(l, diff), t1_right = fem_mul(r, diff);
    const double phi_l = __ddiv_rn(__dsub_rn((double)t1, t1_left), __dsub_rn(t1_right, t1_left));
    const double phi_r = __ddiv_rn(__dsub_rn((double)t1, t1_right), __dsub_rn(t1_left, t1_right));
    const double gr = r < T2 ? (double)g2[r * K + k] : 0.0;
    const double gl = l < T2 ? (double)g2[l * K + k] : 0.0;
    double v = 0.0;
    v = __dadd_rn(v, __dmul_rn(phi_l, gr));
    v = __dadd_rn(v, __dmul_rn(phi_r, gl));
    g1[idx] = (TOut)v;
}

static double fem_diff(long T1, long T2, int type)
{
    return type == 0 ? (double)T1 / (double)T2 : (double)(T1 - 1) / (double)(T2 - 1);
}

static long fem_right_t1_idx(long T2, double diff) { return (long)floor(diff * (double)(T2 - 1)); }

static unsigned int fem_grid(long n) { return (unsigned int)((n + 255) / 256); }

template <typename TIn, typename TOut>
cudaError_t launch_fem_reduce(const TIn *g1, const double *data, const double *theta, TOut *g2, long T1, long T2,
                              int K, int type, double scale, cudaStream_t s)
{
    if (T2 * K == 0) return cudaSuccess;
    const double diff = fem_diff(T1, T2, type);
    FineField<TIn> f{g1, data, theta, K};
    fem_reduce_kernel<TIn, TOut><<<fem_grid(T2 * K), 256, 0, s>>>(f, g2, T1, T2, K, type, diff,
                                                                  fem_right_t1_idx(T2, diff), scale);
    return cudaGetLastError();
}

template <typename TIn, typename TOut>
cudaError_t launch_fem_prolongate(const TIn *g2, TOut *g1, long T1, long T2, int K, int type, cudaStream_t s)
{
    const double diff = fem_diff(T1, T2, type);
    const long n = type == 0 ? T2 * K : T1 * K;
    if (n == 0) return cudaSuccess;
    fem_prolongate_kernel<TIn, TOut><<<fem_grid(n), 256, 0, s>>>(g2, g1, T1, T2, K, type, diff);
    return cudaGetLastError();
}

template cudaError_t launch_fem_reduce<double, double>(const double *, const double *, const double *, double *, long,
                                                       long, int, int, double, cudaStream_t);
template cudaError_t launch_fem_reduce<float, float>(const float *, const double *, const double *, float *, long,
                                                     long, int, int, double, cudaStream_t);
template cudaError_t launch_fem_prolongate<double, double>(const double *, double *, long, long, int, int,
                                                           cudaStream_t);
template cudaError_t launch_fem_prolongate<float, float>(const float *, float *, long, long, int, int, cudaStream_t);

long fem_T_reduced(long T, double fem_reduce) { return fem_reduce < 1.0 ? (long)ceil((double)T * fem_reduce) : T; }

}  // namespace pasc

using namespace pasc;

extern "C" {

int pasc_gb300_fem_reduce_f64(const double *g1_dev, double *g2_dev, long T1, long T2, int K, int fem_type,
                              void *stream)
{
    if ((!g1_dev || !g2_dev) && T1 > 0) { record_error("fem_reduce: NULL argument"); return PASC_ERR_ARG; }
    if (T1 < 1 || T2 < 1 || T2 > T1 || K < 1 || (fem_type != 0 && fem_type != 1) || (fem_type == 1 && T2 < 2)) {
        record_error("fem_reduce: need 1 <= T2 <= T1, K >= 1, fem_type 0 or 1 (FEM-HAT: T2 >= 2)");
        return PASC_ERR_ARG;
    }
    if (launch_fem_reduce<double, double>(g1_dev, nullptr, nullptr, g2_dev, T1, T2, K, fem_type, 1.0,
                                          (cudaStream_t)stream) != cudaSuccess) {
        record_error("fem_reduce: kernel launch failed");
        return PASC_ERR_CUDA;
    }
    return PASC_OK;
}

int pasc_gb300_fem_prolongate_f64(const double *g2_dev, double *g1_dev, long T1, long T2, int K, int fem_type,
                                  void *stream)
{
    if ((!g1_dev || !g2_dev) && T1 > 0) { record_error("fem_prolongate: NULL argument"); return PASC_ERR_ARG; }
    if (T1 < 1 || T2 < 1 || T2 > T1 || K < 1 || (fem_type != 0 && fem_type != 1) || (fem_type == 1 && T2 < 2)) {
        record_error("fem_prolongate: need 1 <= T2 <= T1, K >= 1, fem_type 0 or 1 (FEM-HAT: T2 >= 2)");
        return PASC_ERR_ARG;
    }
    if (launch_fem_prolongate<double, double>(g2_dev, g1_dev, T1, T2, K, fem_type, (cudaStream_t)stream) !=
        cudaSuccess) {
        record_error("fem_prolongate: kernel launch failed");
        return PASC_ERR_CUDA;
    }
    return PASC_OK;
}

}  // extern "C"
