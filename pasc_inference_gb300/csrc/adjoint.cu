// adjoint.cu -- derivatives of a loss through the converged gamma-step QP (no counterpart in
// the reference, which only solves).
//
// The QP  min 1/2 x'Ax - b'x  over the product of K-simplices has A = coeff * (A_hat (x) I_K)
// (coeff = epssqr/T) and b_tk = bscale * (x_t - theta_k)^2 (bscale = -1/T), as formed by
// GraphH1FEMModel (src/petscvector/model/graphh1fem.cpp:146-151, 237-289).  At a solution
// gamma the free set of timestep t is F_t = {k : gamma_tk > act_tol}; S = {v : v_tk = 0 for k
// outside F_t, sum_k v_tk = 0} is the space gamma can move in without changing the active
// set, and P (per timestep: zero outside F_t, subtract the mean over F_t) is the orthogonal
// projection onto it.  The free set is read from one projected-gradient step,
// z = Proj(gamma - a (A gamma - b)) with a = 1/(8 coeff + |bscale|) (1/||A|| when A dominates):
// at an exact solution z = gamma, and on an FP32 end point (x^c + beta d, not exactly on the
// active face) entries held at zero by a positive multiplier are projected away instead of
// being mistaken for free ones.  The optimality conditions on S, P(A gamma - b) = 0, differentiated at
// a fixed active set give  P A P gamma' = -P(A' gamma - b'),  so for a loss l(gamma)
//     l' = -lambda'(A' gamma - b'),   lambda in S solving  P A P lambda = P dl/dgamma.
// lambda is found by conjugate gradients on S: two kernels per CG iteration (apply P A P to the
// search direction and reduce p'q; update lambda and r and reduce r'r), the scalars kept on
// the device (last block of each launch), launched in CUDA-graph chunks with the host polling
// a status word in between.  The fp64 problem runs them in FP64.  The mixed problem runs them
// in FP32 inside FP64 iterative refinement (this part's FP64 rate, not HBM, bounds an FP64 CG
// iteration): the FP64 residual rhs - P A P lambda is rounded to FP32, an FP32 CG reduces it
// by 1e-4, its correction is added to the FP64 lambda, and the loop repeats until the FP64
// residual meets cg_tol; the solution is FP64-accurate, the iterations stream FP32.  The gradients then follow in one pass:
//     dl/d epssqr  = -(d coeff/d epssqr) * sum_tk lambda_tk (A_hat gamma)_tk
//     dl/d x_t     =  sum_k lambda_tk * 2 bscale (x_t - theta_k)
//     dl/d theta_k = -sum_t lambda_tk * 2 bscale (x_t - theta_k)      (through b only)
// All reductions sum fixed per-block partials in block order (deterministic).
#include <math.h>
#include <string.h>
#include <algorithm>
#include <string>

#include "common.cuh"
#include "internal.h"
#include "problem.h"
#include "project.cuh"

namespace pasc {

constexpr int ADJ_NT = 256;
constexpr int ADJ_CHUNK = 16;  // CG iterations per captured graph

enum { ADJ_RUNNING = 0, ADJ_CONVERGED = 1, ADJ_MAXIT = 2, ADJ_BREAKDOWN = 4, ADJ_INNER_DONE = 8 };

constexpr double ADJ_INNER_TOL = 1e-4;  // residual reduction of one FP32 refinement step
constexpr int ADJ_MAX_OUTER = 20;

struct AdjDevState {
    double rr, rr0, pq, alpha, beta, tol;
    double free_dims;
    int it, maxit, status, pcur;
    unsigned int counter;
    double rr_in0;  // FP32 refinement: r'r at the start of the current inner solve
    int outer;
    unsigned int fall;  // clusters free at every timestep (their cluster-constant, zero-sum
                        // vectors are the null space of P A P on S)
    double nullc[8];    // component of lambda along that null space, per cluster
    double rr64;        // FP32 refinement: FP64 r'r of the last residual
    double rscale;      // FP32 refinement: the residual is handed to the FP32 solve times this
                        // (its rms brought to 1: a small residual would otherwise lose its
                        // products p'q to FP32 underflow), the correction divided by it
};

struct AdjointWork {
    int K = 0, grid = 0;
    long T = 0;
    double *gam = nullptr;           // N: FP64 gamma (the mixed path converts into it)
    double *gl = nullptr;            // N: dl/dgamma
    double *lam = nullptr, *r = nullptr, *pb[2] = {nullptr, nullptr}, *q = nullptr;  // N each
    float *r32 = nullptr, *pb32[2] = {nullptr, nullptr}, *q32 = nullptr, *d32 = nullptr;  // N each (mixed)
    cudaGraphExec_t chunk32 = nullptr;
    unsigned int *mask = nullptr;    // T: free clusters of each timestep (bit k)
    double *clean = nullptr, *dX = nullptr;  // T each
    double *partials = nullptr;      // grid * 16
    double *out = nullptr;           // 16: results of the one-pass kernels
    double *out_h = nullptr;         // pinned mirror
    AdjDevState *st = nullptr, *st_h = nullptr;
    unsigned int *ticket = nullptr;  // last-block ticket of the one-pass kernels
    cudaGraphExec_t chunk = nullptr;
    double gtheta_direct[8] = {0};   // direct d loss/d theta of the last recon_mse
    bool have_gl = false;
};

void adjoint_free(AdjointWork *w)
{
    if (!w) return;
    if (w->chunk) cudaGraphExecDestroy(w->chunk);
    if (w->chunk32) cudaGraphExecDestroy(w->chunk32);
    void *dev[] = {w->gam, w->gl, w->lam, w->r, w->pb[0], w->pb[1], w->q, w->mask, w->clean, w->dX,
                   w->partials, w->out, w->st, w->ticket, w->r32, w->pb32[0], w->pb32[1], w->q32, w->d32};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (w->out_h) cudaFreeHost(w->out_h);
    if (w->st_h) cudaFreeHost(w->st_h);
    delete w;
}

// ---------------------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------------------

// orthogonal projection onto S at one timestep (free clusters: bits of m)
template <int K>
__device__ __forceinline__ void proj_free(double (&v)[K], unsigned int m)
{
    const int nf = __popc(m);
    if (nf <= 1) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = 0.0;
        return;
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < K; k++) s += ((m >> k) & 1u) ? v[k] : 0.0;
    const double mean = s / nf;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = ((m >> k) & 1u) ? v[k] - mean : 0.0;
}

// Writes the block's NV sums to partials[blockIdx.x * 16 + j]; the last block to finish
// (ticket) sums them in block order and returns true with the totals in w (thread 0).
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *partials, unsigned int *ticket,
                                         double *scratch, double (&w)[NV])
{
    block_sum<NV>(v, scratch);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int j = 0; j < NV; j++) partials[blockIdx.x * 16 + j] = v[j];
    }
    if (!last_block_done(ticket)) return false;
#pragma unroll
    for (int j = 0; j < NV; j++) w[j] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
#pragma unroll
        for (int j = 0; j < NV; j++) w[j] += __ldcg(partials + b * 16 + j);
    }
    block_sum<NV>(w, scratch);
    if (threadIdx.x == 0) *ticket = 0;
    return true;
}

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------

// l = 1/T sum_t (sum_k gamma_tk theta_k - c_t)^2, dl/dgamma_tk = 2/T e_t theta_k and the
// direct dl/dtheta_k = 2/T sum_t e_t gamma_tk (e = reconstruction - clean).
template <int K>
__global__ void __launch_bounds__(ADJ_NT) recon_mse_kernel(const double *gam, const double *theta,
                                                           const double *clean, long T, double *gl,
                                                           double *partials, unsigned int *ticket, double *out)
{
    __shared__ double scratch[(K + 1) * (ADJ_NT / 32)];
    const double invT = 1.0 / (double)T;
    double th[K];
#pragma unroll
    for (int k = 0; k < K; k++) th[k] = theta[k];
    double v[K + 1];
#pragma unroll
    for (int j = 0; j <= K; j++) v[j] = 0.0;
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        double g[K], rec = 0.0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            g[k] = gam[t * K + k];
            rec += g[k] * th[k];
        }
        const double e = rec - clean[t];
        v[0] += e * e;
#pragma unroll
        for (int k = 0; k < K; k++) {
            gl[t * K + k] = 2.0 * invT * e * th[k];
            v[1 + k] += 2.0 * invT * e * g[k];
        }
    }
    double w[K + 1];
    if (!grid_sum<K + 1>(v, partials, ticket, scratch, w)) return;
    if (threadIdx.x == 0) {
        out[0] = w[0] * invT;
#pragma unroll
        for (int k = 0; k < K; k++) out[1 + k] = w[1 + k];
    }
}

// free sets (from z = Proj(gamma - a g), see the head of the file), r = P dl/dgamma
// (POLISH: r = -P g, the face-Newton step's right-hand side), lambda = 0, both
// search-direction buffers 0, r'r and dim S.
template <int K, bool POLISH = false>
__global__ void __launch_bounds__(ADJ_NT) adj_setup_kernel(const double *gam, const double *gl, const double *data,
                                                           const double *theta, long T, double coeff, double bscale,
                                                           double act_tol, unsigned int *mask, double *lam,
                                                           double *r, double *p0, double *p1,
                                                           double *partials, AdjDevState *st)
{
    __shared__ double scratch[(3 + K) * (ADJ_NT / 32)];
    const double a = 1.0 / (8.0 * coeff + fabs(bscale));
    double v2[3 + K];
#pragma unroll
    for (int j = 0; j < 3 + K; j++) v2[j] = 0.0;
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        const double x = data[t];
        double z[K], zs[K], grad[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double gc = gam[t * K + k];
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gc - gam[(t - 1) * K + k]);
            if (t < T - 1) ag += 2.0 * (gc - gam[(t + 1) * K + k]);
            const double res = x - theta[k];
            grad[k] = coeff * ag - bscale * res * res;
            v2[2 + K] += (bscale * res * res) * (bscale * res * res);
            z[k] = gc - a * grad[k];
        }
        unsigned int m = 0u;
        double v[K];
        if (POLISH) {
            m = mask[t];  // the face gamma was snapped onto (adj_polish_mask_kernel, adj_polish_snap_kernel)
#pragma unroll
            for (int k = 0; k < K; k++) v[k] = -grad[k];
        } else {
            project_ref_f64(z, K, zs);
#pragma unroll
            for (int k = 0; k < K; k++) {
                m |= (z[k] > act_tol ? 1u : 0u) << k;
                v[k] = gl[t * K + k];
            }
            mask[t] = m;
        }
        proj_free<K>(v, m);
#pragma unroll
        for (int k = 0; k < K; k++) {
            r[t * K + k] = v[k];
            lam[t * K + k] = 0.0;
            p0[t * K + k] = 0.0;
            p1[t * K + k] = 0.0;
            v2[0] += v[k] * v[k];
        }
        const int nf = __popc(m);
        v2[1] += nf > 1 ? (double)(nf - 1) : 0.0;
#pragma unroll
        for (int k = 0; k < K; k++) v2[2 + k] += (double)((m >> k) & 1u);
    }
    double w[3 + K];
    if (!grid_sum<3 + K>(v2, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        st->rr = st->rr0 = w[0];
        st->free_dims = w[1];
        unsigned int fall = 0u;
#pragma unroll
        for (int k = 0; k < K; k++) fall |= (w[2 + k] == (double)T ? 1u : 0u) << k;
        st->fall = fall;
        st->it = 0;
        st->beta = 0.0;
        st->pcur = 0;
        st->status = (w[0] > 0.0) ? ADJ_RUNNING : ADJ_CONVERGED;
        // POLISH: a projected gradient at the rounding level of b (||P g|| <= 1e-12 ||b||) is
        // stationary already; a solve on it would only fit noise
        if (POLISH && w[0] <= 1e-24 * w[2 + K]) st->status = ADJ_CONVERGED;
        if (!isfinite(w[0])) st->status = ADJ_BREAKDOWN;
    }
}

// p_new = r + beta p_old (at t and its neighbours), q = P A p_new, p'q; alpha = r'r / p'q.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_apply_kernel(const unsigned int *mask, const double *r,
                                                           double *pb0, double *pb1, double *q, long T,
                                                           double coeff, double *partials, AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    if (st->status != ADJ_RUNNING) return;  // uniform
    const int pc = st->pcur;
    const double beta = st->beta;
    const double *pold = pc ? pb1 : pb0;
    double *pnew = pc ? pb0 : pb1;
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        double pc_[K], y[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            pc_[k] = r[t * K + k] + beta * pold[t * K + k];
            y[k] = 0.0;
        }
        if (t > 0) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const double pl = r[(t - 1) * K + k] + beta * pold[(t - 1) * K + k];
                y[k] += 2.0 * (pc_[k] - pl);
            }
        }
        if (t < T - 1) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const double pr = r[(t + 1) * K + k] + beta * pold[(t + 1) * K + k];
                y[k] += 2.0 * (pc_[k] - pr);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) y[k] *= coeff;
        proj_free<K>(y, mask[t]);
#pragma unroll
        for (int k = 0; k < K; k++) {
            pnew[t * K + k] = pc_[k];
            q[t * K + k] = y[k];
            v[0] += pc_[k] * y[k];
        }
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        st->pq = w[0];
        if (w[0] > 0.0 && isfinite(w[0])) {
            st->alpha = st->rr / w[0];
        } else {
            st->alpha = 0.0;
            st->status = ADJ_BREAKDOWN;  // P A P is only semi-definite: r left its range
        }
    }
}

// lambda += alpha p, r -= alpha q, r'r; beta, convergence.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_update_kernel(double *lam, double *r, const double *pb0,
                                                            const double *pb1, const double *q, long T,
                                                            double *partials, AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    if (st->status != ADJ_RUNNING) return;
    const double alpha = st->alpha;
    const double *p = st->pcur ? pb0 : pb1;  // written by the apply kernel
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const long i = t * K + k;
            lam[i] += alpha * p[i];
            const double rn = r[i] - alpha * q[i];
            r[i] = rn;
            v[0] += rn * rn;
        }
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        const double rr = w[0];
        st->beta = rr / st->rr;
        st->rr = rr;
        st->it += 1;
        st->pcur ^= 1;
        if (!isfinite(rr)) st->status = ADJ_BREAKDOWN;
        else if (rr <= st->tol * st->tol * st->rr0) st->status = ADJ_CONVERGED;
        else if (st->it >= st->maxit) st->status = ADJ_MAXIT;
    }
}

// ---- FP32 refinement (mixed problems) ----

template <int K>
__device__ __forceinline__ void proj_free_f(float (&v)[K], unsigned int m)
{
    const int nf = __popc(m);
    if (nf <= 1) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = 0.f;
        return;
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) s += ((m >> k) & 1u) ? v[k] : 0.f;
    const float mean = s / (float)nf;
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = ((m >> k) & 1u) ? v[k] - mean : 0.f;
}

// FP64 residual r = rhs - P A P lambda (lambda with its neighbours), rounded into r32; the
// correction d32 and both FP32 search directions restart at 0.  Last block: r'r, the outer
// convergence test, and the inner solve's start.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_residual_kernel(const unsigned int *mask, const double *lam,
                                                              const double *rhs, float *r32, float *p0, float *p1,
                                                              float *d32, long T, double coeff, double *partials,
                                                              AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    const double rscale = st->rscale;
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        double y[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double lc = lam[t * K + k];
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (lc - lam[(t - 1) * K + k]);
            if (t < T - 1) ag += 2.0 * (lc - lam[(t + 1) * K + k]);
            y[k] = coeff * ag;
        }
        proj_free<K>(y, mask[t]);
#pragma unroll
        for (int k = 0; k < K; k++) {
            const long i = t * K + k;
            const double rv = rhs[i] - y[k];
            r32[i] = (float)(rv * rscale);
            p0[i] = 0.f;
            p1[i] = 0.f;
            d32[i] = 0.f;
            v[0] += rv * rv;
        }
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        st->rr64 = w[0];
        st->rr = w[0] * rscale * rscale;  // r'r of the scaled FP32 residual the inner solve starts from
        st->rr_in0 = st->rr;
        st->beta = 0.0;
        st->pcur = 0;
        if (!isfinite(w[0])) st->status = ADJ_BREAKDOWN;
        else if (w[0] <= st->tol * st->tol * st->rr0) st->status = ADJ_CONVERGED;
        else if (st->outer >= ADJ_MAX_OUTER || st->it >= st->maxit) st->status = ADJ_MAXIT;
        else st->status = ADJ_RUNNING;
        st->outer += 1;
    }
}

// FP32 form of adj_apply_kernel (p = r + beta p_old, q = P A p, p'q summed in FP64)
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_apply32_kernel(const unsigned int *mask, const float *r,
                                                             float *pb0, float *pb1, float *q, long T, float coeff,
                                                             double *partials, AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    if (st->status != ADJ_RUNNING) return;  // uniform
    const int pc = st->pcur;
    const float beta = (float)st->beta;
    const float *pold = pc ? pb1 : pb0;
    float *pnew = pc ? pb0 : pb1;
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        float pc_[K], y[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            pc_[k] = fmaf(beta, pold[t * K + k], r[t * K + k]);
            y[k] = 0.f;
        }
        if (t > 0) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float pl = fmaf(beta, pold[(t - 1) * K + k], r[(t - 1) * K + k]);
                y[k] += 2.f * (pc_[k] - pl);
            }
        }
        if (t < T - 1) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float pr = fmaf(beta, pold[(t + 1) * K + k], r[(t + 1) * K + k]);
                y[k] += 2.f * (pc_[k] - pr);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) y[k] *= coeff;
        proj_free_f<K>(y, mask[t]);
        float part = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            pnew[t * K + k] = pc_[k];
            q[t * K + k] = y[k];
            part = fmaf(pc_[k], y[k], part);
        }
        v[0] += (double)part;
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        st->pq = w[0];
        if (w[0] > 0.0 && isfinite(w[0])) {
            st->alpha = st->rr / w[0];
        } else {
            st->alpha = 0.0;
            st->status = ADJ_BREAKDOWN;
        }
    }
}

// FP32 form of adj_update_kernel on the correction d32; the inner solve ends when r'r has
// dropped by ADJ_INNER_TOL^2
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_update32_kernel(float *d, float *r, const float *pb0, const float *pb1,
                                                              const float *q, long T, double *partials,
                                                              AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    if (st->status != ADJ_RUNNING) return;
    const float alpha = (float)st->alpha;
    const float *p = st->pcur ? pb0 : pb1;
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        float part = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const long i = t * K + k;
            d[i] = fmaf(alpha, p[i], d[i]);
            const float rn = fmaf(-alpha, q[i], r[i]);
            r[i] = rn;
            part = fmaf(rn, rn, part);
        }
        v[0] += (double)part;
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        const double rr = w[0];
        st->beta = rr / st->rr;
        st->rr = rr;
        st->it += 1;
        st->pcur ^= 1;
        if (!isfinite(rr)) st->status = ADJ_BREAKDOWN;
        else if (rr <= ADJ_INNER_TOL * ADJ_INNER_TOL * st->rr_in0 || st->it >= st->maxit) st->status = ADJ_INNER_DONE;
    }
}

// lambda = P(lambda + d32): FP64 accumulation of the FP32 correction, projected back onto S
// (the FP32 correction leaves S by its rounding, and a component outside S would be
// amplified by the solve of the next step)
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_accum_kernel(double *lam, const float *d, const unsigned int *mask,
                                                           long T, const AdjDevState *st)
{
    const double inv = 1.0 / st->rscale;
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        double v[K];
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = lam[t * K + k] + (double)d[t * K + k] * inv;
        proj_free<K>(v, mask[t]);
#pragma unroll
        for (int k = 0; k < K; k++) lam[t * K + k] = v[k];
    }
}

// The null space of P A P on S: v_tk = c_k for all t with c supported on the clusters free at
// every timestep and summing to 0 (A_hat annihilates constants in t).  Conjugate gradients
// from 0 stay orthogonal to it; the FP32 steps of the refinement do not quite (the rounded
// right-hand side has a component there), and that component moves dl/dx (not dl/depssqr).
// lambda is returned orthogonal to the null space, the minimum-norm solution.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_nullmean_kernel(const double *lam, long T, double *partials,
                                                              AdjDevState *st)
{
    __shared__ double scratch[K * (ADJ_NT / 32)];
    double v[K];
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = 0.0;
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] += lam[t * K + k];
    }
    double w[K];
    if (!grid_sum<K>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        const unsigned int f = st->fall;
        const int nf = __popc(f);
        double mean = 0.0;
        for (int k = 0; k < K; k++) mean += ((f >> k) & 1u) ? w[k] / (double)T : 0.0;
        mean = nf > 0 ? mean / nf : 0.0;
        for (int k = 0; k < K; k++) st->nullc[k] = (nf >= 2 && ((f >> k) & 1u)) ? w[k] / (double)T - mean : 0.0;
    }
}

template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_nullsub_kernel(double *lam, long T, const AdjDevState *st)
{
    double c[K];
#pragma unroll
    for (int k = 0; k < K; k++) c[k] = st->nullc[k];
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
#pragma unroll
        for (int k = 0; k < K; k++) lam[t * K + k] -= c[k];
    }
}

// gradients from lambda (see the head of the file).  dX may be null.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_output_kernel(const double *lam, const double *gam,
                                                            const double *data, const double *theta, long T,
                                                            double dcoeff, double bscale, double *dX,
                                                            double *partials, unsigned int *ticket, double *out)
{
    __shared__ double scratch[(K + 1) * (ADJ_NT / 32)];
    double th[K];
#pragma unroll
    for (int k = 0; k < K; k++) th[k] = theta[k];
    double v[K + 1];
#pragma unroll
    for (int j = 0; j <= K; j++) v[j] = 0.0;
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        const double x = data[t];
        double dx = 0.0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double lk = lam[t * K + k];
            const double gc = gam[t * K + k];
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gc - gam[(t - 1) * K + k]);
            if (t < T - 1) ag += 2.0 * (gc - gam[(t + 1) * K + k]);
            v[0] += lk * ag;
            const double db = 2.0 * bscale * (x - th[k]);  // d b_tk / d x_t = -d b_tk / d theta_k
            dx += lk * db;
            v[1 + k] -= lk * db;
        }
        if (dX) dX[t] = dx;
    }
    double w[K + 1];
    if (!grid_sum<K + 1>(v, partials, ticket, scratch, w)) return;
    if (threadIdx.x == 0) {
        out[0] = -dcoeff * w[0];
#pragma unroll
        for (int k = 0; k < K; k++) out[1 + k] = w[1 + k];
    }
}

// Polish, first pass: the free set of every timestep from one projected-gradient step (as in
// adj_setup_kernel).
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_polish_mask_kernel(const double *gam, const double *data,
                                                                 const double *theta, long T, double coeff,
                                                                 double bscale, double act_tol, unsigned int *mask)
{
    const double a = 1.0 / (8.0 * coeff + fabs(bscale));
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        const double x = data[t];
        double z[K], zs[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double gc = gam[t * K + k];
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gc - gam[(t - 1) * K + k]);
            if (t < T - 1) ag += 2.0 * (gc - gam[(t + 1) * K + k]);
            const double res = x - theta[k];
            z[k] = gc - a * (coeff * ag - bscale * res * res);
        }
        project_ref_f64(z, K, zs);
        unsigned int m = 0u;
#pragma unroll
        for (int k = 0; k < K; k++) m |= (z[k] > act_tol ? 1u : 0u) << k;
        mask[t] = m;
    }
}

// Polish, second pass: gamma onto its face -- entries outside the free set to 0, their mass
// spread evenly over the free ones (the sum stays 1); the Newton step then starts on the face.
// (A timestep with no free entry -- not possible for z on the simplex with act_tol < 1/K --
// is left as it is.)
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_polish_snap_kernel(double *gam, const unsigned int *mask, long T)
{
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        const unsigned int m = mask[t];
        const int nf = __popc(m);
        if (nf == 0 || nf == K) continue;
        double y[K], out = 0.0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            y[k] = gam[t * K + k];
            if (!((m >> k) & 1u)) out += y[k];
        }
        const double share = out / nf;
#pragma unroll
        for (int k = 0; k < K; k++) gam[t * K + k] = ((m >> k) & 1u) ? y[k] + share : 0.0;
    }
}

// Polish: gamma += delta (delta = lambda of the face-Newton solve, in S: zero off the free
// set, zero sum per timestep); a timestep with a negative entry left its face and is projected
// back onto the simplex (FP64, the reference's order).  x32: the FP32 state, rounded from the
// result (mixed problems; may be null).  out[0..2] = projected timesteps, sum delta^2,
// sum gamma^2.
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_polish_apply_kernel(const double *lam, double *gam, float *x32, long T,
                                                                  double *partials, unsigned int *ticket, double *out)
{
    __shared__ double scratch[3 * (ADJ_NT / 32)];
    double v[3] = {0.0, 0.0, 0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        double y[K], ys[K], d2 = 0.0;
        bool neg = false;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double dk = lam[t * K + k];
            y[k] = gam[t * K + k] + dk;
            d2 += dk * dk;
            neg |= !(y[k] >= 0.0);
        }
        if (neg) project_ref_f64(y, K, ys);
#pragma unroll
        for (int k = 0; k < K; k++) {
            gam[t * K + k] = y[k];
            if (x32) x32[t * K + k] = (float)y[k];
            v[2] += y[k] * y[k];
        }
        v[0] += neg ? 1.0 : 0.0;
        v[1] += d2;
    }
    double w[3];
    if (!grid_sum<3>(v, partials, ticket, scratch, w)) return;
    if (threadIdx.x == 0) {
        out[0] = w[0];
        out[1] = w[1];
        out[2] = w[2];
    }
}

// Polish: the right-hand side -P g minus its component in the null space of P A P (the
// st->nullc adj_nullmean_kernel found for it); r'r starts the solve.  Where clusters are free
// at every timestep, moving their weights by constants that sum to zero changes f only
// linearly, g'v, which vanishes at the optimum: the Newton step on the face ignores it (the
// solve needs a right-hand side in the range of P A P).
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_polish_rhs_kernel(double *r, long T, double *partials, AdjDevState *st)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    double c[K];
#pragma unroll
    for (int k = 0; k < K; k++) c[k] = st->nullc[k];
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double y = r[t * K + k] - c[k];
            r[t * K + k] = y;
            v[0] += y * y;
        }
    }
    double w[1];
    if (!grid_sum<1>(v, partials, &st->counter, scratch, w)) return;
    if (threadIdx.x == 0) {
        st->rr = st->rr0 = w[0];
        st->status = (w[0] > 0.0) ? ADJ_RUNNING : ADJ_CONVERGED;
        if (!isfinite(w[0])) st->status = ADJ_BREAKDOWN;
    }
}

// out[0] = 1/2 gamma'A gamma - b'gamma in FP64 (A = coeff A_hat, b = bscale (x - theta)^2)
template <int K>
__global__ void __launch_bounds__(ADJ_NT) adj_objective_kernel(const double *gam, const double *data,
                                                               const double *theta, long T, double coeff,
                                                               double bscale, double *partials,
                                                               unsigned int *ticket, double *out)
{
    __shared__ double scratch[1 * (ADJ_NT / 32)];
    double v[1] = {0.0};
    for (long t = blockIdx.x * (long)ADJ_NT + threadIdx.x; t < T; t += (long)gridDim.x * ADJ_NT) {
        const double x = data[t];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const double gc = gam[t * K + k];
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gc - gam[(t - 1) * K + k]);
            if (t < T - 1) ag += 2.0 * (gc - gam[(t + 1) * K + k]);
            const double res = x - theta[k];
            v[0] += gc * (0.5 * coeff * ag - bscale * res * res);
        }
    }
    double w[1];
    if (!grid_sum<1>(v, partials, ticket, scratch, w)) return;
    if (threadIdx.x == 0) out[0] = w[0];
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------

static int afail(int code, const std::string &msg)
{
    record_error(msg.c_str());
    return code;
}

#define ACU(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return afail(PASC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define ACHK(call)                     \
    do {                               \
        int r_ = (call);               \
        if (r_ != PASC_OK) return r_;  \
    } while (0)

#define PASC_ADJ_DISPATCH(K, ...)                                             \
    switch (K) {                                                              \
        case 1: { constexpr int KK = 1; __VA_ARGS__; } break;                 \
        case 2: { constexpr int KK = 2; __VA_ARGS__; } break;                 \
        case 3: { constexpr int KK = 3; __VA_ARGS__; } break;                 \
        case 4: { constexpr int KK = 4; __VA_ARGS__; } break;                 \
        case 5: { constexpr int KK = 5; __VA_ARGS__; } break;                 \
        case 6: { constexpr int KK = 6; __VA_ARGS__; } break;                 \
        case 7: { constexpr int KK = 7; __VA_ARGS__; } break;                 \
        case 8: { constexpr int KK = 8; __VA_ARGS__; } break;                 \
        default: break;                                                       \
    }

static int ensure_work(pasc_gb300_problem *p)
{
    if (p->adj) return PASC_OK;
    if (p->K > 8) return afail(PASC_ERR_NOTSUPP, "adjoint: K > 8 is not supported");
    if (p->xdim > 1) return afail(PASC_ERR_NOTSUPP, "adjoint: 1-D signals only");
    if (p->fem_inner) return afail(PASC_ERR_NOTSUPP, "adjoint: reduced (fem_reduce < 1) problems are not supported");
    if (p->tp) return afail(PASC_ERR_NOTSUPP, "adjoint: theta in the penalty is not supported");
    if (p->graph) return afail(PASC_ERR_NOTSUPP, "adjoint: graph (R > 1) problems are not supported");
    AdjointWork *w = new AdjointWork();
    w->K = p->K;
    w->T = p->T;
    const long N = p->N, T = p->T;
    w->grid = (int)std::max(1L, std::min((T + ADJ_NT - 1) / ADJ_NT, (long)p->sms * 4));
    auto dal = [&](void **ptr, size_t bytes) { return cudaMalloc(ptr, bytes > 0 ? bytes : 1) == cudaSuccess; };
    bool ok = dal((void **)&w->gl, sizeof(double) * N) && dal((void **)&w->lam, sizeof(double) * N) &&
              dal((void **)&w->r, sizeof(double) * N) && dal((void **)&w->pb[0], sizeof(double) * N) &&
              dal((void **)&w->pb[1], sizeof(double) * N) && dal((void **)&w->q, sizeof(double) * N) &&
              dal((void **)&w->mask, sizeof(unsigned int) * T) && dal((void **)&w->clean, sizeof(double) * T) &&
              dal((void **)&w->dX, sizeof(double) * T) && dal((void **)&w->partials, sizeof(double) * 16 * w->grid) &&
              dal((void **)&w->out, sizeof(double) * 16) && dal((void **)&w->st, sizeof(AdjDevState)) &&
              dal((void **)&w->ticket, sizeof(unsigned int));
    if (ok && p->precision == PASC_PREC_MIXED)
        ok = dal((void **)&w->gam, sizeof(double) * N) && dal((void **)&w->r32, sizeof(float) * N) &&
             dal((void **)&w->pb32[0], sizeof(float) * N) && dal((void **)&w->pb32[1], sizeof(float) * N) &&
             dal((void **)&w->q32, sizeof(float) * N) && dal((void **)&w->d32, sizeof(float) * N);
    if (ok) ok = cudaMallocHost((void **)&w->out_h, sizeof(double) * 16) == cudaSuccess &&
                 cudaMallocHost((void **)&w->st_h, sizeof(AdjDevState)) == cudaSuccess;
    if (!ok) {
        adjoint_free(w);
        return afail(PASC_ERR_ALLOC, "adjoint: device allocation failed");
    }
    cudaMemsetAsync(w->ticket, 0, sizeof(unsigned int), p->stream);
    cudaMemsetAsync(w->st, 0, sizeof(AdjDevState), p->stream);
    p->adj = w;
    return PASC_OK;
}

// FP64 gamma of the problem (converted from the FP32 state on the mixed path)
static int adj_gamma(pasc_gb300_problem *p, const double **g)
{
    if (p->precision == PASC_PREC_FP64) {
        *g = p->x;
        return PASC_OK;
    }
    ACU(launch_f32_to_f64(p->xb[p->cur], p->adj->gam, p->N, p->stream));
    *g = p->adj->gam;
    return PASC_OK;
}

static int ensure_adj_graph(pasc_gb300_problem *p)
{
    AdjointWork *w = p->adj;
    if (w->chunk) return PASC_OK;
    ACU(cudaStreamSynchronize(p->stream));
    cudaGraph_t g;
    ACU(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    const double coeff = p->coeffA;
    for (int i = 0; i < ADJ_CHUNK; i++) {
        PASC_ADJ_DISPATCH(p->K, {
            adj_apply_kernel<KK><<<w->grid, ADJ_NT, 0, p->stream>>>(w->mask, w->r, w->pb[0], w->pb[1], w->q,
                                                                    p->T, coeff, w->partials, w->st);
            adj_update_kernel<KK><<<w->grid, ADJ_NT, 0, p->stream>>>(w->lam, w->r, w->pb[0], w->pb[1], w->q,
                                                                     p->T, w->partials, w->st);
        });
    }
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    if (e != cudaSuccess) return afail(PASC_ERR_CUDA, std::string("adjoint capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&w->chunk, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        w->chunk = nullptr;
        return afail(PASC_ERR_CUDA, std::string("adjoint graph: ") + cudaGetErrorString(e));
    }
    return PASC_OK;
}

// CUDA graph of ADJ_CHUNK FP32 CG iterations (mixed problems)
static int ensure_adj_graph32(pasc_gb300_problem *p)
{
    AdjointWork *w = p->adj;
    if (w->chunk32) return PASC_OK;
    ACU(cudaStreamSynchronize(p->stream));
    cudaGraph_t g;
    ACU(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    const float coeff = (float)p->coeffA;
    for (int i = 0; i < ADJ_CHUNK; i++) {
        PASC_ADJ_DISPATCH(p->K, {
            adj_apply32_kernel<KK><<<w->grid, ADJ_NT, 0, p->stream>>>(w->mask, w->r32, w->pb32[0], w->pb32[1],
                                                                      w->q32, p->T, coeff, w->partials, w->st);
            adj_update32_kernel<KK><<<w->grid, ADJ_NT, 0, p->stream>>>(w->d32, w->r32, w->pb32[0], w->pb32[1],
                                                                       w->q32, p->T, w->partials, w->st);
        });
    }
    cudaError_t e = cudaStreamEndCapture(p->stream, &g);
    if (e != cudaSuccess) return afail(PASC_ERR_CUDA, std::string("adjoint capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&w->chunk32, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        w->chunk32 = nullptr;
        return afail(PASC_ERR_CUDA, std::string("adjoint graph: ") + cudaGetErrorString(e));
    }
    return PASC_OK;
}

// FP32 conjugate gradients inside FP64 iterative refinement (mixed problems): w->r holds the
// FP64 right-hand side P dl/dgamma, lambda starts at 0
static int adj_refine(pasc_gb300_problem *p, AdjDevState *h, int *launches)
{
    AdjointWork *w = p->adj;
    cudaStream_t s = p->stream;
    double rr_last = h->rr0;  // FP64 r'r of the last residual (the right-hand side's at first)
    auto residual = [&]() -> int {
        // scale of the next FP32 solve from the last residual: its rms about 1 (then 1e-4 after
        // each further inner solve, well inside the FP32 range)
        h->rscale = rr_last > 0.0 && isfinite(rr_last) ? 1.0 / sqrt(rr_last / (double)p->N) : 1.0;
        ACU(cudaMemcpyAsync(&w->st->rscale, &h->rscale, sizeof(double), cudaMemcpyHostToDevice, s));
        PASC_ADJ_DISPATCH(p->K, (adj_residual_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(
                                    w->mask, w->lam, w->r, w->r32, w->pb32[0], w->pb32[1], w->d32, p->T, p->coeffA,
                                    w->partials, w->st)));
        ACU(cudaGetLastError());
        *launches += 1;
        ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
        ACU(cudaStreamSynchronize(s));
        rr_last = h->rr64;
        return PASC_OK;
    };
    ACHK(residual());  // lambda = 0: r32 = the right-hand side
    while (h->status == ADJ_RUNNING) {
        while (h->status == ADJ_RUNNING) {
            ACU(cudaGraphLaunch(w->chunk32, s));
            *launches += 2 * ADJ_CHUNK;
            ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
            ACU(cudaStreamSynchronize(s));
        }
        if (h->status != ADJ_INNER_DONE) break;  // breakdown
        PASC_ADJ_DISPATCH(p->K, (adj_accum_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->lam, w->d32, w->mask, p->T,
                                                                                   w->st)));
        ACU(cudaGetLastError());
        *launches += 1;
        ACHK(residual());
    }
    return PASC_OK;
}

}  // namespace pasc

using namespace pasc;

extern "C" {

void pasc_gb300_adjoint_default_opts(pasc_gb300_adjoint_opts *o)
{
    if (!o) return;
    o->act_tol = 1e-7;
    o->cg_tol = 1e-10;
    o->cg_maxit = 20000;
}

int pasc_gb300_recon_mse(pasc_gb300_problem *p, const double *clean, double *loss)
{
    if (!p || !clean || !loss) return afail(PASC_ERR_ARG, "recon_mse: NULL argument");
    ACU(cudaSetDevice(p->device));
    ACHK(ensure_work(p));
    AdjointWork *w = p->adj;
    const double *g = nullptr;
    ACHK(adj_gamma(p, &g));
    ACU(cudaMemcpyAsync(w->clean, clean, sizeof(double) * p->T, cudaMemcpyHostToDevice, p->stream));
    PASC_ADJ_DISPATCH(p->K, (recon_mse_kernel<KK><<<w->grid, ADJ_NT, 0, p->stream>>>(
                                g, p->theta64, w->clean, p->T, w->gl, w->partials, w->ticket, w->out)));
    ACU(cudaGetLastError());
    ACU(cudaMemcpyAsync(w->out_h, w->out, sizeof(double) * (1 + p->K), cudaMemcpyDeviceToHost, p->stream));
    ACU(cudaStreamSynchronize(p->stream));
    *loss = w->out_h[0];
    for (int k = 0; k < p->K; k++) w->gtheta_direct[k] = w->out_h[1 + k];
    w->have_gl = true;
    return PASC_OK;
}

int pasc_gb300_adjoint(pasc_gb300_problem *p, const double *dloss_dgamma, const pasc_gb300_adjoint_opts *o,
                       double *dloss_depssqr, double *dloss_ddata, double *dloss_dtheta,
                       pasc_gb300_adjoint_stats *stats)
{
    if (!p) return afail(PASC_ERR_ARG, "adjoint: NULL problem");
    pasc_gb300_adjoint_opts od;
    pasc_gb300_adjoint_default_opts(&od);
    if (!o) o = &od;
    if (o->cg_maxit < 0 || !(o->cg_tol >= 0.0)) return afail(PASC_ERR_ARG, "adjoint: bad options");
    ACU(cudaSetDevice(p->device));
    ACHK(ensure_work(p));
    AdjointWork *w = p->adj;
    cudaStream_t s = p->stream;
    const bool stored = dloss_dgamma == nullptr;
    if (stored && !w->have_gl)
        return afail(PASC_ERR_STATE, "adjoint: no dloss/dgamma given and none stored by recon_mse");
    if (!stored) {
        ACU(cudaMemcpyAsync(w->gl, dloss_dgamma, sizeof(double) * p->N, cudaMemcpyHostToDevice, s));
        w->have_gl = false;  // the stored MSE gradient is overwritten
    }
    const double *g = nullptr;
    ACHK(adj_gamma(p, &g));
    const bool mixed = p->precision == PASC_PREC_MIXED;
    if (mixed) ACHK(ensure_adj_graph32(p));
    else ACHK(ensure_adj_graph(p));
    ACU(cudaEventRecord(p->ev0, s));

    AdjDevState *h = w->st_h;
    memset(h, 0, sizeof *h);
    h->tol = o->cg_tol;
    h->maxit = o->cg_maxit;
    ACU(cudaMemcpyAsync(w->st, h, sizeof *h, cudaMemcpyHostToDevice, s));
    PASC_ADJ_DISPATCH(p->K, (adj_setup_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(
                                g, w->gl, p->data64, p->theta64, p->T, p->coeffA, p->coeffB, o->act_tol,
                                w->mask, w->lam, w->r, w->pb[0], w->pb[1], w->partials, w->st)));
    ACU(cudaGetLastError());
    int launches = 1;
    ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
    ACU(cudaStreamSynchronize(s));
    if (h->status == ADJ_RUNNING && o->cg_maxit == 0) h->status = ADJ_MAXIT;
    if (mixed && h->status == ADJ_RUNNING) {
        ACHK(adj_refine(p, h, &launches));
    } else {
        while (h->status == ADJ_RUNNING) {
            ACU(cudaGraphLaunch(w->chunk, s));
            launches += 2 * ADJ_CHUNK;
            ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
            ACU(cudaStreamSynchronize(s));
        }
    }
    if (h->status != ADJ_BREAKDOWN && __builtin_popcount(h->fall) >= 2) {
        // lambda orthogonal to the null space of P A P (see adj_nullmean_kernel)
        PASC_ADJ_DISPATCH(p->K, {
            adj_nullmean_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->lam, p->T, w->partials, w->st);
            adj_nullsub_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->lam, p->T, w->st);
        });
        ACU(cudaGetLastError());
        launches += 2;
    }
    const double dcoeff = p->scalef ? 1.0 / (double)p->T : 1.0;  // d coeff / d epssqr
    PASC_ADJ_DISPATCH(p->K, (adj_output_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(
                                w->lam, g, p->data64, p->theta64, p->T, dcoeff, p->coeffB, w->dX, w->partials,
                                w->ticket, w->out)));
    ACU(cudaGetLastError());
    launches++;
    ACU(cudaMemcpyAsync(w->out_h, w->out, sizeof(double) * (1 + p->K), cudaMemcpyDeviceToHost, s));
    if (dloss_ddata) ACU(cudaMemcpyAsync(dloss_ddata, w->dX, sizeof(double) * p->T, cudaMemcpyDeviceToHost, s));
    ACU(cudaEventRecord(p->ev1, s));
    ACU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    if (dloss_depssqr) *dloss_depssqr = w->out_h[0];
    if (dloss_dtheta) {
        for (int k = 0; k < p->K; k++) dloss_dtheta[k] = w->out_h[1 + k] + (stored ? w->gtheta_direct[k] : 0.0);
    }
    if (stats) {
        stats->cg_it = h->it;
        stats->status = h->status;
        stats->kernel_launches = launches;
        stats->free_dims = (long)h->free_dims;
        stats->cg_relres = h->rr0 > 0.0 ? sqrt((mixed ? h->rr64 : h->rr) / h->rr0) : 0.0;
        stats->time_s = ms * 1e-3;
    }
    if (h->status == ADJ_BREAKDOWN)
        return afail(PASC_ERR_STATE, "adjoint: conjugate gradients broke down (non-finite values, or the "
                                     "right-hand side has a component in the null space of P A P)");
    return PASC_OK;
}

void pasc_gb300_polish_default_opts(pasc_gb300_polish_opts *o)
{
    if (!o) return;
    o->rounds = 4;
    o->act_tol = 0.0;
    o->cg_tol = 1e-6;
    o->cg_maxit = 2000;
}

int pasc_gb300_polish(pasc_gb300_problem *p, const pasc_gb300_polish_opts *o, pasc_gb300_polish_stats *stats)
{
    if (!p) return afail(PASC_ERR_ARG, "polish: NULL problem");
    pasc_gb300_polish_opts od;
    pasc_gb300_polish_default_opts(&od);
    if (!o) o = &od;
    if (o->rounds < 0 || o->cg_maxit < 0 || !(o->cg_tol >= 0.0)) return afail(PASC_ERR_ARG, "polish: bad options");
    ACU(cudaSetDevice(p->device));
    ACHK(ensure_work(p));
    AdjointWork *w = p->adj;
    cudaStream_t s = p->stream;
    const bool mixed = p->precision == PASC_PREC_MIXED;
    // the FP64 gamma the rounds refine: the problem's own (fp64) or a widened copy of the FP32
    // state, written back rounded once at the end (mixed)
    double *gam = mixed ? w->gam : p->x;
    double *backup = w->gl;  // gamma at the start of a round (a kept dloss/dgamma is dropped anyway)
    if (mixed) ACU(launch_f32_to_f64(p->xb[p->cur], gam, p->N, s));
    if (mixed) ACHK(ensure_adj_graph32(p));
    else ACHK(ensure_adj_graph(p));
    ACU(cudaEventRecord(p->ev0, s));
    AdjDevState *h = w->st_h;
    int launches = mixed ? 1 : 0, rounds = 0, cg_it = 0, cg_status = 0;
    double face_changes = 0.0, step_rel = 0.0, cg_relres = 0.0;
    auto objective = [&](double *f) -> int {
        PASC_ADJ_DISPATCH(p->K, (adj_objective_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(
                                    gam, p->data64, p->theta64, p->T, p->coeffA, p->coeffB, w->partials, w->ticket,
                                    w->out)));
        ACU(cudaGetLastError());
        launches++;
        ACU(cudaMemcpyAsync(w->out_h, w->out, sizeof(double), cudaMemcpyDeviceToHost, s));
        ACU(cudaStreamSynchronize(s));
        *f = w->out_h[0];
        return PASC_OK;
    };
    double f = 0.0;
    ACHK(objective(&f));
    for (int r = 0; r < o->rounds; r++) {
        memset(h, 0, sizeof *h);
        h->tol = o->cg_tol;
        h->maxit = o->cg_maxit;
        ACU(cudaMemcpyAsync(w->st, h, sizeof *h, cudaMemcpyHostToDevice, s));
        ACU(cudaMemcpyAsync(backup, gam, sizeof(double) * p->N, cudaMemcpyDeviceToDevice, s));
        PASC_ADJ_DISPATCH(p->K, {
            adj_polish_mask_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(gam, p->data64, p->theta64, p->T, p->coeffA,
                                                                  p->coeffB, o->act_tol, w->mask);
            adj_polish_snap_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(gam, w->mask, p->T);
        });
        ACU(cudaGetLastError());
        launches += 2;
        PASC_ADJ_DISPATCH(p->K, (adj_setup_kernel<KK, true><<<w->grid, ADJ_NT, 0, s>>>(
                                    gam, nullptr, p->data64, p->theta64, p->T, p->coeffA, p->coeffB, o->act_tol,
                                    w->mask, w->lam, w->r, w->pb[0], w->pb[1], w->partials, w->st)));
        ACU(cudaGetLastError());
        launches++;
        ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
        ACU(cudaStreamSynchronize(s));
        if (h->status == ADJ_RUNNING && __builtin_popcount(h->fall) >= 2) {
            PASC_ADJ_DISPATCH(p->K, {
                adj_nullmean_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->r, p->T, w->partials, w->st);
                adj_polish_rhs_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->r, p->T, w->partials, w->st);
            });
            ACU(cudaGetLastError());
            launches += 2;
            ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
            ACU(cudaStreamSynchronize(s));
        }
        if (h->status == ADJ_CONVERGED) {  // stationary on the face (to rounding): keep the snap if it did not raise f
            double fs = 0.0;
            ACHK(objective(&fs));
            if (fs <= f + 1e-15 * fabs(f)) f = fs;
            else ACU(cudaMemcpyAsync(gam, backup, sizeof(double) * p->N, cudaMemcpyDeviceToDevice, s));
            face_changes = 0.0;
            break;
        }
        if (h->status != ADJ_RUNNING) return afail(PASC_ERR_STATE, "polish: non-finite gradient");
        const double rr0 = h->rr0;
        if (mixed) {
            ACHK(adj_refine(p, h, &launches));
        } else {
            while (h->status == ADJ_RUNNING) {
                ACU(cudaGraphLaunch(w->chunk, s));
                launches += 2 * ADJ_CHUNK;
                ACU(cudaMemcpyAsync(h, w->st, sizeof *h, cudaMemcpyDeviceToHost, s));
                ACU(cudaStreamSynchronize(s));
            }
        }
        cg_it += h->it;
        cg_status = h->status == ADJ_INNER_DONE ? ADJ_CONVERGED : h->status;
        cg_relres = h->rr0 > 0.0 ? sqrt((mixed ? h->rr64 : h->rr) / h->rr0) : 0.0;
        // conjugate gradients stop short (p'q <= 0) only where the residual has reached the
        // rounding level of the operator: lambda is then the last iterate (fp64; it is kept
        // only if it reduced the residual) or the corrections of the completed refinement
        // steps (mixed)
        if (h->status == ADJ_BREAKDOWN && !mixed && !(h->rr < rr0)) break;
        if (__builtin_popcount(h->fall) >= 2) {  // the step orthogonal to the null space, as in the adjoint
            PASC_ADJ_DISPATCH(p->K, {
                adj_nullmean_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->lam, p->T, w->partials, w->st);
                adj_nullsub_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(w->lam, p->T, w->st);
            });
            ACU(cudaGetLastError());
            launches += 2;
        }
        PASC_ADJ_DISPATCH(p->K, (adj_polish_apply_kernel<KK><<<w->grid, ADJ_NT, 0, s>>>(
                                    w->lam, gam, nullptr, p->T, w->partials, w->ticket, w->out)));
        ACU(cudaGetLastError());
        launches++;
        ACU(cudaMemcpyAsync(w->out_h, w->out, sizeof(double) * 3, cudaMemcpyDeviceToHost, s));
        ACU(cudaStreamSynchronize(s));
        const double fc = w->out_h[0], sr = w->out_h[2] > 0.0 ? sqrt(w->out_h[1] / w->out_h[2]) : 0.0;
        double fnew = 0.0;
        ACHK(objective(&fnew));
        if (!(fnew <= f + 1e-15 * fabs(f))) {  // no descent: keep the round's starting gamma and stop
            ACU(cudaMemcpyAsync(gam, backup, sizeof(double) * p->N, cudaMemcpyDeviceToDevice, s));
            break;
        }
        f = fnew;
        rounds = r + 1;
        face_changes = fc;
        step_rel = sr;
        if (face_changes == 0.0) break;  // the step stayed on its face: a further round would only
                                         // repeat the solve to its tolerance
    }
    if (mixed) {
        ACU(launch_f64_to_f32(gam, p->xb[p->cur], p->N, s));
        launches++;
        ACU(launch_f32_to_f64(p->xb[p->cur], gam, p->N, s));
        ACHK(objective(&f));  // of the gamma kept: the FP32 rounding of the polished one
    }
    ACU(cudaEventRecord(p->ev1, s));
    ACU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    p->fx_last = f;
    p->have_fx = true;
    w->have_gl = false;  // a stored dloss/dgamma belongs to the gamma before the polish
    if (stats) {
        stats->rounds = rounds;
        stats->cg_it = cg_it;
        stats->kernel_launches = launches;
        stats->face_changes = (long)face_changes;
        stats->cg_status = cg_status;
        stats->cg_relres = cg_relres;
        stats->step_rel = step_rel;
        stats->fx = f;
        stats->time_s = ms * 1e-3;
    }
    return PASC_OK;
}

}  // extern "C"
