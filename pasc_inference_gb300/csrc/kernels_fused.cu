// kernels_fused.cu -- mixed-precision (FP32 state, FP64 reductions) SPG-QP kernels.
//
// One HBM sweep per SPG iteration, and only gamma (x) is stored.  The reference iteration
// (src/petscvector/solver/spgqpsolver.cpp:140-216)
//     d = P(x - alpha g) - x ; Ad = coeff*A_hat d ; dd, dAd, gd ; beta (GLL) ;
//     x += beta d ; g += beta Ad ; f = 1/2 (g - b)'x ; alpha = dd/dAd
// keeps the gradient in memory and updates it recursively.  Here the gradient is recomputed
// on chip from x, g = coeff*A_hat x - b (the same value in exact arithmetic; the stencil has
// the footprint the recursive update needs anyway), so nothing but x crosses HBM and FP32
// rounding cannot accumulate in g over the iterations.  b is formed in registers from the
// data and theta (b_tk = bscale*(x_t - theta_k)^2, src/petscvector/model/graphh1fem.cpp:258-286),
// or, for multichannel data (BMAT), read from the T x K array the residual kernel wrote once per
// outer iteration (K values per timestep instead of n channels).
//
// The sweep is re-timed so that one pass finishes iteration c+1 and starts iteration c+2:
// it reads x^c, forms g^c, d_{c+1}, x^{c+1} = x^c + beta_{c+1} d_{c+1}, g^{c+1}, f^{c+1},
// then d_{c+2} and its dots.  The halo (2 timesteps before a tile, 3 after) is recomputed,
// never stored; x^{c+1} goes to the other half of a ping-pong pair.  HBM traffic per
// iteration: read x and the data, write x = 8*K*T + 4*T bytes.
//
// Reductions: per thread in compensated FP32, per block and per grid in FP64 (fixed order,
// deterministic for a fixed grid).  The last block applies the step-length and GLL rules in
// FP64 and advances the device state; the host only polls the status word between chunks
// of sweeps.  d'Ad is accumulated in the difference form 2*coeff*sum (d_{t+1}-d_t)^2, equal
// to d'(A d) for the FEM-H1 matrix but free of the cancellation the dot form has in FP32.
#include "common.cuh"
#include "project.cuh"
#include "internal.h"
#include "sweep_common.cuh"

namespace pasc {

// K consecutive floats of one timestep: 16-byte loads when K % 4 == 0, 8-byte when K % 2 == 0
// (the buffers are 16-byte aligned and t*K*4 bytes keeps that alignment).  STREAM: evict-first.
template <int K, bool STREAM>
__device__ __forceinline__ void load_row(const float *p, float (&v)[K])
{
    if (K % 4 == 0) {
#pragma unroll
        for (int q = 0; q < K / 4; q++) {
            const float4 w = STREAM ? __ldcs(reinterpret_cast<const float4 *>(p) + q)
                                    : __ldg(reinterpret_cast<const float4 *>(p) + q);
            v[4 * q] = w.x; v[4 * q + 1] = w.y; v[4 * q + 2] = w.z; v[4 * q + 3] = w.w;
        }
    } else if (K % 2 == 0) {
#pragma unroll
        for (int q = 0; q < K / 2; q++) {
            const float2 w = STREAM ? __ldcs(reinterpret_cast<const float2 *>(p) + q)
                                    : __ldg(reinterpret_cast<const float2 *>(p) + q);
            v[2 * q] = w.x; v[2 * q + 1] = w.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = STREAM ? __ldcs(p + k) : __ldg(p + k);
    }
}

template <int K>
__device__ __forceinline__ void store_row(float *p, const float (&v)[K])
{
    if (K % 4 == 0) {
#pragma unroll
        for (int q = 0; q < K / 4; q++)
            __stcs(reinterpret_cast<float4 *>(p) + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
    } else if (K % 2 == 0) {
#pragma unroll
        for (int q = 0; q < K / 2; q++) __stcs(reinterpret_cast<float2 *>(p) + q, make_float2(v[2 * q], v[2 * q + 1]));
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) __stcs(p + k, v[k]);
    }
}

constexpr int SWEEP_NT = 256;  // threads per block = timesteps per tile incl. halo
constexpr int SWEEP_HL = 2;    // halo timesteps before the owned range
constexpr int SWEEP_HR = 3;    // halo timesteps after it
constexpr int SWEEP_W = SWEEP_NT - SWEEP_HL - SWEEP_HR;  // owned timesteps per tile

int sweep_tile_width() { return SWEEP_W; }

// TP: theta in the penalty, block k of A is coeff * a.kw[k] * A_hat (usethetainpenalty)
template <int K, bool INIT, bool BMAT, bool TP = false>
__global__ void __launch_bounds__(SWEEP_NT, K <= 4 ? 6 : (K <= 6 ? 4 : 3)) spg_sweep_kernel(SweepArgs a)
{
    __shared__ float s_x[SWEEP_NT * K];  // x^c (zero outside 0 <= t < T)
    __shared__ float s_y[SWEEP_NT * K];  // x^{c+1}
    __shared__ float s_d[SWEEP_NT * K];  // d_{c+2}
    __shared__ double s_red[4 * (SWEEP_NT / 32)];

    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;  // uniform across the grid

    const int cur = st->cur;
    const float *__restrict__ xin = cur ? a.xb1 : a.xb0;
    float *__restrict__ xout = cur ? a.xb0 : a.xb1;
    const float a0 = (float)st->alpha_prev;
    const float beta = (float)st->beta;
    const float a1 = (float)st->alpha_cur;
    const float coeff = (float)st->coeff;
    const float bscale = (float)st->bscale;
    const int T = (int)a.T;  // K*T < 2^31 (checked at creation)

    float theta[K], ck[K], kw[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        theta[k] = BMAT ? 0.f : a.theta[k];
        kw[k] = TP ? a.kw[k] : 1.f;
        ck[k] = TP ? coeff * kw[k] : coeff;
    }

    KahanF acc_f;  // the objective keeps a compensated sum; the dots need less
    float acc_dd = 0.f, acc_dAd = 0.f, acc_gd = 0.f;
    const int i = threadIdx.x;
    // neighbour slots, clamped so that the edge threads (whose results are discarded) stay
    // inside the shared arrays
    const int il = (i > 0 ? i - 1 : 0) * K, ir = (i < SWEEP_NT - 1 ? i + 1 : i) * K;
    const int ntiles = (T + SWEEP_W - 1) / SWEEP_W;

    // the next tile's x and data are loaded into registers while the current one is computed
    float xn[K], dvn = 0.f, bn[K];
    {
        const int t = blockIdx.x * SWEEP_W - SWEEP_HL + i;
        const bool in = (int)blockIdx.x < ntiles && (unsigned)t < (unsigned)T;
        if (in) {
            load_row<K, true>(xin + t * K, xn);
            if (BMAT) load_row<K, false>(a.bmat + t * K, bn);
            else dvn = __ldg(a.data + t);
        } else {
#pragma unroll
            for (int k = 0; k < K; k++) {
                xn[k] = 0.f;
                bn[k] = 0.f;
            }
        }
    }

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int t = tile * SWEEP_W - SWEEP_HL + i;
        const bool in = (unsigned)t < (unsigned)T;
        // FEM-H1 row (blockgraphsparse.cpp:51-109, R = 1) in difference form:
        // (A_hat x)_t = 2 [t > 0] (x_t - x_{t-1}) + 2 [t < T-1] (x_t - x_{t+1}), equal to the
        // assembled row (centre 4, 2 at an end, neighbours -2) but exact where neighbours agree
        const float ml = t > 0 ? 2.f : 0.f, mr = t < T - 1 ? 2.f : 0.f;

        // phase A: x^c (INIT: the projected start point) and b_t in registers
        float xc[K], bk[K];
        const float dv = dvn;
#pragma unroll
        for (int k = 0; k < K; k++) {
            xc[k] = xn[k];
            if (BMAT) bk[k] = bn[k];
        }
        {
            const int tn = t + (int)gridDim.x * SWEEP_W;
            const bool inn = tile + (int)gridDim.x < ntiles && (unsigned)tn < (unsigned)T;
            if (inn) {
                load_row<K, true>(xin + tn * K, xn);
                if (BMAT) load_row<K, false>(a.bmat + tn * K, bn);
                else dvn = __ldg(a.data + tn);
            } else {
#pragma unroll
                for (int k = 0; k < K; k++) {
                    xn[k] = 0.f;
                    bn[k] = 0.f;
                }
                dvn = 0.f;
            }
        }
        if (INIT) project_reg<K>(xc);
#pragma unroll
        for (int k = 0; k < K; k++) {
            if (!BMAT) {
                const float r = dv - theta[k];
                bk[k] = bscale * (r * r);
            }
            s_x[i * K + k] = in ? xc[k] : 0.f;
        }
        __syncthreads();

        // phase B: g^c = coeff*A_hat x^c - b, d_{c+1} = P(x^c - alpha g^c) - x^c,
        //          x^{c+1} = x^c + beta d_{c+1}    (INIT: x^{c+1} = x^c)
        float x1[K];
        const bool inB = in && i >= 1 && i <= SWEEP_NT - 2;
        if (INIT) {
#pragma unroll
            for (int k = 0; k < K; k++) x1[k] = xc[k];
        } else {
            float z[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float S = ml * (xc[k] - s_x[il + k]) + mr * (xc[k] - s_x[ir + k]);
                const float g = ck[k] * S - bk[k];
                z[k] = xc[k] - a0 * g;
            }
            project_reg<K>(z);
#pragma unroll
            for (int k = 0; k < K; k++) x1[k] = xc[k] + beta * (z[k] - xc[k]);
        }
#pragma unroll
        for (int k = 0; k < K; k++) s_y[i * K + k] = (INIT ? in : inB) ? x1[k] : 0.f;
        __syncthreads();

        // phase C: g^{c+1}, objective contribution, d_{c+2} = P(x^{c+1} - alpha' g^{c+1}) - x^{c+1}
        const bool inC = in && i >= 2 && i <= SWEEP_NT - 3;
        const bool own = in && i >= SWEEP_HL && i < SWEEP_NT - SWEEP_HR;
        float g1[K], d1[K];
        {
            float fpart = 0.f;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float S = ml * (x1[k] - s_y[il + k]) + mr * (x1[k] - s_y[ir + k]);
                g1[k] = ck[k] * S - bk[k];
                fpart += (g1[k] - bk[k]) * x1[k];
                d1[k] = x1[k] - a1 * g1[k];
            }
            if (own) acc_f.add(fpart);
            project_reg<K>(d1);
#pragma unroll
            for (int k = 0; k < K; k++) {
                d1[k] = inC ? d1[k] - x1[k] : 0.f;
                s_d[i * K + k] = d1[k];
            }
        }
        __syncthreads();

        // phase D: dots of d_{c+2}; write x^{c+1}
        if (own) {
            const bool right = t < T - 1;
#pragma unroll
            for (int k = 0; k < K; k++) {
                acc_dd += d1[k] * d1[k];
                acc_gd += g1[k] * d1[k];
                const float df = right ? s_d[ir + k] - d1[k] : 0.f;
                acc_dAd += TP ? kw[k] * df * df : df * df;
            }
            store_row<K>(xout + t * K, x1);
        }
    }

    // block and grid reductions (float-float; the step logic in FP64)
    double w[4];
    if (!sweep_grid_sum4(acc_f, acc_dd, acc_dAd, acc_gd, reinterpret_cast<float2 *>(a.partials), blockIdx.x,
                         &st->counter, gridDim.x, 0, 1, reinterpret_cast<float2 *>(s_red), w))
        return;
    spg_finish_sweep<INIT>(st, cur, w);
}

template <int K, bool INIT>
static int blocks_per_sm_t(bool tp)
{
    int nb = 0;
    if (tp) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_sweep_kernel<K, INIT, false, true>, SWEEP_NT, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_sweep_kernel<K, INIT, false>, SWEEP_NT, 0);
    return nb > 0 ? nb : 1;
}

int sweep_blocks_per_sm(int K, bool init, bool tp)
{
    switch (K) {
#define PASC_CASE(KK) case KK: return init ? blocks_per_sm_t<KK, true>(tp) : blocks_per_sm_t<KK, false>(tp);
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 1;
    }
}

cudaError_t launch_sweep(int K, bool init, int grid, const SweepArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK)                                                                   \
    case KK:                                                                            \
        if (a.bmat) {                                                                   \
            if (init) spg_sweep_kernel<KK, true, true><<<grid, SWEEP_NT, 0, s>>>(a);    \
            else spg_sweep_kernel<KK, false, true><<<grid, SWEEP_NT, 0, s>>>(a);        \
        } else if (a.kw) {                                                              \
            if (init) spg_sweep_kernel<KK, true, false, true><<<grid, SWEEP_NT, 0, s>>>(a); \
            else spg_sweep_kernel<KK, false, false, true><<<grid, SWEEP_NT, 0, s>>>(a); \
        } else {                                                                        \
            if (init) spg_sweep_kernel<KK, true, false><<<grid, SWEEP_NT, 0, s>>>(a);   \
            else spg_sweep_kernel<KK, false, false><<<grid, SWEEP_NT, 0, s>>>(a);       \
        }                                                                               \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// theta update (graphh1fem.cpp:347-380): theta_k = sum_t gamma_tk x_t / sum_t gamma_tk.
// FP32 gamma/data, compensated FP32 per thread, FP64 per block and grid; the last block
// writes theta in FP64 and FP32.
// TP (usethetainpenalty, graphh1fem.cpp:318-372): theta_k = g'x / (sum g + g'(alpha A_hat)g / 2)
// with gamma_k'A_hat gamma_k taken in the difference form 2 sum_t (g_{t+1} - g_t)^2.
// ---------------------------------------------------------------------------------------
constexpr int THETA_NT = 256;

template <int K, bool TP = false>
__global__ void __launch_bounds__(THETA_NT) theta_kernel(ThetaArgs a)
{
    constexpr int NQ = TP ? 3 * K : 2 * K;
    __shared__ double s_red[NQ * (THETA_NT / 32)];
    const float *gam = a.cur ? a.xb1 : a.xb0;
    KahanF sx[K], sg[K], sa[TP ? K : 1];
    const long stride = (long)gridDim.x * THETA_NT;
    for (long t = (long)blockIdx.x * THETA_NT + threadIdx.x; t < a.T; t += stride) {
        const float x = __ldg(a.data + t);
        const bool right = TP && t + 1 < a.T;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float gk = __ldcs(gam + t * K + k);
            sg[k].add(gk);
            sx[k].add(__fmul_rn(x, gk));
            if (TP && right) {
                const float df = __ldg(gam + (t + 1) * K + k) - gk;
                sa[TP ? k : 0].add(df * df);
            }
        }
    }
    double v[NQ];
#pragma unroll
    for (int k = 0; k < K; k++) {
        v[k] = sx[k].value();
        v[K + k] = sg[k].value();
        if (TP) v[(TP ? 2 * K : 0) + k] = sa[TP ? k : 0].value();
    }
    block_sum<NQ>(v, s_red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) a.partials[blockIdx.x * NQ + q] = v[q];
    }
    if (!last_block_done(&a.st->counter2)) return;
    double w[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += THETA_NT) {
#pragma unroll
        for (int q = 0; q < NQ; q++) w[q] += __ldcg(a.partials + b * NQ + q);
    }
    block_sum<NQ>(w, s_red);
    if (threadIdx.x == 0) {
        a.st->counter2 = 0;
#pragma unroll
        for (int k = 0; k < K; k++) {
            double th;
            if (TP) {
                const double gAg = a.pen_alpha * (2.0 * w[(TP ? 2 * K : 0) + k]);
                const double den = 1.0 * w[K + k] + 0.5 * gAg;
                th = den != 0.0 ? (1.0 * w[k]) / den : 0.0;
            } else {
                th = (w[K + k] != 0.0) ? w[k] / w[K + k] : 0.0;
            }
            a.theta64[k] = th;
            a.theta32[k] = (float)th;
        }
    }
}

cudaError_t launch_theta_f32(int K, int grid, const ThetaArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK)                                                          \
    case KK:                                                                   \
        if (a.tp) theta_kernel<KK, true><<<grid, THETA_NT, 0, s>>>(a);         \
        else theta_kernel<KK><<<grid, THETA_NT, 0, s>>>(a);                    \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// standalone FP32 projection and operator (device-pointer entry points)
// ---------------------------------------------------------------------------------------
template <int K>
__global__ void project_f32_reg_kernel(float *x, long T)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < T; t += stride) {
        float v[K];
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = x[t * K + k];
        project_reg<K>(v);
#pragma unroll
        for (int k = 0; k < K; k++) x[t * K + k] = v[k];
    }
}

template <int G>
__global__ void project_f32_group_kernel(float *x, long T, int K)
{
    const int per_warp = 32 / G;
    const long warp_global = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (long w = warp_global; w * per_warp < T; w += nwarps) {
        const long t = w * per_warp + lane / G;
        const int k = lane & (G - 1);
        const bool valid = t < T;
        const bool act = valid && k < K;
        float v = act ? x[t * K + k] : 0.f;
        float r = project_group<G>(v, K, valid);
        if (act) x[t * K + k] = r;
    }
}

static int grid_for(long work, int threads)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long blocks = (work + threads - 1) / threads;
    long cap = (long)sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

cudaError_t launch_project_f32(float *x, long T, int K, cudaStream_t s)
{
    if (T <= 0) return cudaSuccess;
    switch (K) {
#define PASC_CASE(KK) case KK: project_f32_reg_kernel<KK><<<grid_for(T, 256), 256, 0, s>>>(x, T); break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default:
            if (K <= 16) project_f32_group_kernel<16><<<grid_for(T * 16, 256), 256, 0, s>>>(x, T, K);
            else if (K <= 32) project_f32_group_kernel<32><<<grid_for(T * 32, 256), 256, 0, s>>>(x, T, K);
            else return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

__global__ void matmult_f32_kernel(const float *x, float *y, long T, int K, float coeff)
{
    const long n = T * K;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += stride) {
        const long t = idx / K;
        float sum = 0.f;
        if (T > 1) {
            const float w = (t == 0 || t == T - 1) ? 2.f : 4.f;
            if (t > 0) sum = __fmul_rn(-2.f, x[idx - K]);
            sum = __fadd_rn(sum, __fmul_rn(w, x[idx]));
            if (t < T - 1) sum = __fadd_rn(sum, __fmul_rn(-2.f, x[idx + K]));
        }
        y[idx] = __fmul_rn(coeff, sum);
    }
}

cudaError_t launch_matmult_f32(const float *x, float *y, long T, int K, float coeff, cudaStream_t s)
{
    if (T <= 0) return cudaSuccess;
    matmult_f32_kernel<<<grid_for(T * K, 256), 256, 0, s>>>(x, y, T, K, coeff);
    return cudaGetLastError();
}

__global__ void f64_to_f32_kernel(const double *src, float *dst, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = (float)src[i];
}

__global__ void f32_to_f64_kernel(const float *src, double *dst, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = (double)src[i];
}

cudaError_t launch_f64_to_f32(const double *src, float *dst, long n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    f64_to_f32_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t launch_f32_to_f64(const float *src, double *dst, long n, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    f32_to_f64_kernel<<<grid_for(n, 256), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace pasc
