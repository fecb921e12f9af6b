// kernels_plain.cu -- FP64 kernels of the plain path: one kernel per operation of the
// reference's PETSc solve (src/petscvector/solver/spgqpsolver.cpp:55-345), in the
// reference's arithmetic (no fused multiply-add: every product and sum is rounded, as in the
// host VecAXPY/VecDot/MatMult loops), with deterministic two-stage reductions.
#include "common.cuh"
#include "project.cuh"
#include "internal.h"

namespace pasc {

constexpr int PLAIN_NT = 256;

static int num_sms()
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

static int grid_elems(long n, int per_sm = 8)
{
    long blocks = (n + PLAIN_NT - 1) / PLAIN_NT;
    long cap = (long)num_sms() * per_sm;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

// Grid of the reduction kernels: fixed so that results do not depend on the problem size's
// rounding of the grid (deterministic for a given device).
static int grid_reduce() { return num_sms() * 4; }

size_t dot_partials_size() { return (size_t)4096 * 8 + 64; }

// ---------------------------------------------------------------------------------------
// projection (simplex_local.cu:70-139), thread per timestep, reference order, no scratch.
// ---------------------------------------------------------------------------------------
template <int KB>
__global__ void project_f64_kernel(double *x, long T, int K)
{
    double y[KB];
    const long stride = (long)gridDim.x * blockDim.x;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += stride)
        project_ref_f64(x + t * K, K, y);
}

cudaError_t launch_project_f64(double *x, long T, int K, cudaStream_t s)
{
    if (T <= 0) return cudaSuccess;
    const int g = grid_elems(T);
    if (K <= 8) project_f64_kernel<8><<<g, PLAIN_NT, 0, s>>>(x, T, K);
    else if (K <= 32) project_f64_kernel<32><<<g, PLAIN_NT, 0, s>>>(x, T, K);
    else if (K <= KMAX_PLAIN) project_f64_kernel<KMAX_PLAIN><<<g, 128, 0, s>>>(x, T, K);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// FEM-H1 operator: assembled row (blockgraphsparse.cpp:51-109, R = 1) summed over ascending
// columns from 0.0 like MatMult, then VecScale by coeff (spgqpsolver.cpp:122-123).
// ---------------------------------------------------------------------------------------
// the assembled row t of A_hat applied to column k of x (x points at element (t, k))
__device__ __forceinline__ double ahat_row_f64(const double *x, long t, long T, int K)
{
    double sum = 0.0;
    if (T == 1) {
        sum = __dadd_rn(sum, __dmul_rn(0.0, x[0]));
    } else {
        const double w = (t == 0 || t == T - 1) ? 2.0 : 4.0;
        if (t > 0) sum = __dadd_rn(sum, __dmul_rn(-2.0, x[-K]));
        sum = __dadd_rn(sum, __dmul_rn(w, x[0]));
        if (t < T - 1) sum = __dadd_rn(sum, __dmul_rn(-2.0, x[K]));
    }
    return sum;
}

// kc != null: block k scaled by kc[k] (BlockGraphSparseMatrix with coefficients,
// blockgraphsparse.cpp:161-185: VecScale of block k by alpha*theta_k*theta_k)
__global__ void matmult_f64_kernel(const double *x, double *y, long T, int K, double coeff, const double *kc)
{
    const long n = T * K;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long t = i / K;
        const double sum = ahat_row_f64(x + i, t, T, K);
        y[i] = __dmul_rn(kc ? kc[i - t * K] : coeff, sum);
    }
}

cudaError_t launch_matmult_f64(const double *x, double *y, long T, int K, double coeff, cudaStream_t s,
                               const double *kc)
{
    if (T <= 0) return cudaSuccess;
    matmult_f64_kernel<<<grid_elems(T * K), PLAIN_NT, 0, s>>>(x, y, T, K, coeff, kc);
    return cudaGetLastError();
}

// ck64[k] = (coeff * theta_k) * theta_k (the order of blockgraphsparse.cpp:177), kw32[k] = theta_k^2
__global__ void tp_coeffs_kernel(const double *theta, double coeff, int K, double *ck64, float *kw32)
{
    const int k = threadIdx.x;
    if (k >= K) return;
    const double th = theta[k];
    ck64[k] = __dmul_rn(__dmul_rn(coeff, th), th);
    if (kw32) kw32[k] = (float)__dmul_rn(th, th);
}

cudaError_t launch_tp_coeffs(const double *theta64, double coeff, int K, double *ck64, float *kw32, cudaStream_t s)
{
    tp_coeffs_kernel<<<1, 32 * ((K + 31) / 32), 0, s>>>(theta64, coeff, K, ck64, kw32);
    return cudaGetLastError();
}

// y = y + a*x  (VecAXPY)
__global__ void axpy_f64_kernel(double *y, double a, const double *x, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        y[i] = __dadd_rn(y[i], __dmul_rn(a, x[i]));
}

cudaError_t launch_axpy_f64(double *y, double a, const double *x, long n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    axpy_f64_kernel<<<grid_elems(n), PLAIN_NT, 0, s>>>(y, a, x, n);
    return cudaGetLastError();
}

// d = x + (-a)*g  (VecCopy(x, d) followed by VecAXPY(d, -a, g), spgqpsolver.cpp:146-147)
__global__ void xmay_f64_kernel(double *d, const double *x, double a, const double *g, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        d[i] = __dadd_rn(x[i], __dmul_rn(-a, g[i]));
}

cudaError_t launch_xmay_f64(double *d, const double *x, double a, const double *g, long n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    xmay_f64_kernel<<<grid_elems(n), PLAIN_NT, 0, s>>>(d, x, a, g, n);
    return cudaGetLastError();
}

// b_tk = bscale * ((x_t - theta_k)*(x_t - theta_k))  (graphh1fem.cpp:258-286)
__global__ void residual_f64_kernel(const double *data, const double *theta, double *b, long T, int K,
                                    double bscale)
{
    const long n = T * K;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long t = i / K;
        const int k = (int)(i - t * K);
        const double r = __dsub_rn(data[t], theta[k]);
        b[i] = __dmul_rn(bscale, __dmul_rn(r, r));
    }
}

cudaError_t launch_residual_f64(const double *data, const double *theta, double *b, long T, int K,
                                double bscale, cudaStream_t s)
{
    if (T <= 0) return cudaSuccess;
    residual_f64_kernel<<<grid_elems(T * K), PLAIN_NT, 0, s>>>(data, theta, b, T, K, bscale);
    return cudaGetLastError();
}

// blocked k*T+t -> interleaved t*K+k  (decomposition.cpp:266-356, R = 1)
// T blocks = Tt timesteps x R nodes; block s = t*R + r comes from k*R*Tt + r*Tt + t
// (with R > 1, Decomposition::permute_TRblocksize, decomposition.cpp:260-340)
template <typename F>
__global__ void permute_kernel(const F *src, F *dst, long T, int K, long R)
{
    const long n = T * K;
    const long Tt = T / R;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long s = i / K;
        const int k = (int)(i - s * K);
        const long t = s / R, r = s - t * R;
        dst[i] = src[(long)k * T + r * Tt + t];
    }
}

cudaError_t launch_permute_f64(const double *src, double *dst, long T, int K, cudaStream_t s, long R)
{
    if (T <= 0) return cudaSuccess;
    permute_kernel<double><<<grid_elems(T * K), PLAIN_NT, 0, s>>>(src, dst, T, K, R);
    return cudaGetLastError();
}

cudaError_t launch_permute_f32(const float *src, float *dst, long T, int K, cudaStream_t s, long R)
{
    if (T <= 0) return cudaSuccess;
    permute_kernel<float><<<grid_elems(T * K), PLAIN_NT, 0, s>>>(src, dst, T, K, R);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// deterministic reductions: stage 1 (fixed grid, per-thread FP64 sums over a grid-stride
// range, block tree) writes partials; the last block sums them in index order.
// ---------------------------------------------------------------------------------------
struct DotPtrs {
    const double *a[3];
    const double *b[3];
};

template <int NQ, int MODE>  // MODE 0: dots; MODE 1: x*(g - b) in slot 0
__global__ void __launch_bounds__(PLAIN_NT) dots_f64_kernel(DotPtrs p, long n, double *scratch, double *out)
{
    __shared__ double s_red[NQ * (PLAIN_NT / 32)];
    double v[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) v[q] = 0.0;
    const long stride = (long)gridDim.x * PLAIN_NT;
    for (long i = (long)blockIdx.x * PLAIN_NT + threadIdx.x; i < n; i += stride) {
        if (MODE == 1) {
            v[0] = __dadd_rn(v[0], __dmul_rn(p.a[0][i], __dsub_rn(p.a[1][i], p.b[0][i])));
        } else {
#pragma unroll
            for (int q = 0; q < NQ; q++) v[q] = __dadd_rn(v[q], __dmul_rn(p.a[q][i], p.b[q][i]));
        }
    }
    block_sum<NQ>(v, s_red);
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + 4096 * 4);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) scratch[blockIdx.x * NQ + q] = v[q];
    }
    if (!last_block_done(counter)) return;
    double w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += PLAIN_NT) {
#pragma unroll
        for (int q = 0; q < NQ; q++) w[q] = __dadd_rn(w[q], __ldcg(scratch + b * NQ + q));
    }
    block_sum<NQ>(w, s_red);
    if (threadIdx.x == 0) {
        *counter = 0;
#pragma unroll
        for (int q = 0; q < NQ; q++) out[q] = w[q];
    }
}

cudaError_t launch_dots_f64(int nq, const double *a0, const double *b0, const double *a1,
                            const double *b1, const double *a2, const double *b2, long n,
                            double *scratch, double *out, cudaStream_t s)
{
    DotPtrs p = {{a0, a1, a2}, {b0, b1, b2}};
    const int g = grid_reduce();
    if (g > 4096 / 3) return cudaErrorInvalidValue;
    if (nq == 1) dots_f64_kernel<1, 0><<<g, PLAIN_NT, 0, s>>>(p, n, scratch, out);
    else if (nq == 2) dots_f64_kernel<2, 0><<<g, PLAIN_NT, 0, s>>>(p, n, scratch, out);
    else if (nq == 3) dots_f64_kernel<3, 0><<<g, PLAIN_NT, 0, s>>>(p, n, scratch, out);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

cudaError_t launch_fx_f64(const double *x, const double *g, const double *b, long n,
                          double *scratch, double *out, cudaStream_t s)
{
    DotPtrs p = {{x, g, nullptr}, {b, nullptr, nullptr}};
    dots_f64_kernel<1, 1><<<grid_reduce(), PLAIN_NT, 0, s>>>(p, n, scratch, out);
    return cudaGetLastError();
}

// theta_k = sum_t gamma_tk x_t / sum_t gamma_tk (graphh1fem.cpp:347-380), KB clusters per pass.
// TP (usethetainpenalty, graphh1fem.cpp:318-372): theta is set to 1, Agamma = A gamma with that
// theta (block k scaled by alpha), and theta_k = g'x / (sum g + gamma_k'Agamma_k / 2).
template <int KB, bool TP>
__global__ void __launch_bounds__(PLAIN_NT) theta_f64_kernel(const double *gamma, const double *data,
                                                             double *theta, long T, int K, int k0,
                                                             double *scratch, double alpha)
{
    constexpr int NQ = (TP ? 3 : 2) * KB;
    __shared__ double s_red[NQ * (PLAIN_NT / 32)];
    double v[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) v[q] = 0.0;
    const int nk = min(KB, K - k0);
    const long stride = (long)gridDim.x * PLAIN_NT;
    for (long t = (long)blockIdx.x * PLAIN_NT + threadIdx.x; t < T; t += stride) {
        const double x = data[t];
#pragma unroll
        for (int q = 0; q < KB; q++) {
            if (q < nk) {
                const double gk = gamma[t * K + k0 + q];
                v[q] = __dadd_rn(v[q], __dmul_rn(x, gk));
                v[KB + q] = __dadd_rn(v[KB + q], gk);
                if (TP) {
                    const double agk = __dmul_rn(alpha, ahat_row_f64(gamma + t * K + k0 + q, t, T, K));
                    v[(TP ? 2 * KB : 0) + q] = __dadd_rn(v[(TP ? 2 * KB : 0) + q], __dmul_rn(gk, agk));
                }
            }
        }
    }
    block_sum<NQ>(v, s_red);
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + 4096 * 4);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) scratch[blockIdx.x * NQ + q] = v[q];
    }
    if (!last_block_done(counter)) return;
    double w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += PLAIN_NT) {
#pragma unroll
        for (int q = 0; q < NQ; q++) w[q] = __dadd_rn(w[q], __ldcg(scratch + b * NQ + q));
    }
    block_sum<NQ>(w, s_red);
    if (threadIdx.x == 0) {
        *counter = 0;
        for (int q = 0; q < nk; q++) {
            if (TP) {
                const double den = 1.0 * w[KB + q] + 0.5 * w[(TP ? 2 * KB : 0) + q];
                theta[k0 + q] = den != 0.0 ? (1.0 * w[q]) / den : 0.0;
            } else {
                theta[k0 + q] = (w[KB + q] != 0.0) ? w[q] / w[KB + q] : 0.0;
            }
        }
    }
}

cudaError_t launch_theta_f64(const double *gamma, const double *data, double *theta, long T, int K,
                             double *scratch, cudaStream_t s, bool tp, double pen_alpha)
{
    // 4096*4 doubles of partials: grid * 3*KB must fit
    const int g = min(grid_reduce(), 4096 * 4 / (3 * 8));
    for (int k0 = 0; k0 < K; k0 += 8) {
        if (tp) theta_f64_kernel<8, true><<<g, PLAIN_NT, 0, s>>>(gamma, data, theta, T, K, k0, scratch, pen_alpha);
        else theta_f64_kernel<8, false><<<g, PLAIN_NT, 0, s>>>(gamma, data, theta, T, K, k0, scratch, 0.0);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// || -solution + sum_k theta_k gamma_k ||_1 (signal1Ddata.cpp:157-186)
__global__ void __launch_bounds__(PLAIN_NT) abserr_kernel(const double *gamma, const double *theta,
                                                          const double *sol, long T, int K,
                                                          double *scratch, double *out)
{
    __shared__ double s_red[PLAIN_NT / 32];
    double v[1] = {0.0};
    const long stride = (long)gridDim.x * PLAIN_NT;
    for (long t = (long)blockIdx.x * PLAIN_NT + threadIdx.x; t < T; t += stride) {
        double r = -sol[t];
        for (int k = 0; k < K; k++) r = __dadd_rn(r, __dmul_rn(theta[k], gamma[t * K + k]));
        v[0] = __dadd_rn(v[0], fabs(r));
    }
    block_sum<1>(v, s_red);
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + 4096 * 4);
    if (threadIdx.x == 0) scratch[blockIdx.x] = v[0];
    if (!last_block_done(counter)) return;
    double w[1] = {0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += PLAIN_NT) w[0] = __dadd_rn(w[0], __ldcg(scratch + b));
    block_sum<1>(w, s_red);
    if (threadIdx.x == 0) {
        *counter = 0;
        *out = w[0];
    }
}

cudaError_t launch_recon_abserr(const double *gamma, const double *theta, const double *sol,
                                long T, int K, double *scratch, double *out, cudaStream_t s)
{
    abserr_kernel<<<grid_reduce(), PLAIN_NT, 0, s>>>(gamma, theta, sol, T, K, scratch, out);
    return cudaGetLastError();
}

__global__ void argmax_kernel(const double *gamma, int *labels, long T, int K)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += stride) {
        int best = 0;
        double bv = gamma[t * K];
        for (int k = 1; k < K; k++) {
            const double v = gamma[t * K + k];
            if (v > bv) { bv = v; best = k; }
        }
        labels[t] = best;
    }
}

cudaError_t launch_argmax(const double *gamma, int *labels, long T, int K, cudaStream_t s)
{
    if (T <= 0) return cudaSuccess;
    argmax_kernel<<<grid_elems(T), PLAIN_NT, 0, s>>>(gamma, labels, T, K);
    return cudaGetLastError();
}

}  // namespace pasc
