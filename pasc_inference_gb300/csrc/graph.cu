// graph.cu -- graph (R > 1) and image mode of the FEM-H1 model: BlockGraphSparseMatrix on a
// graph of R nodes (src/petscvector/algebra/matrix/blockgraphsparse.cpp:7-103) and the graphs
// the reference builds (BGMGraph::process, src/petscvector/algebra/graph/bgmgraph.cpp:73-152;
// BGMGraphGrid1D / BGMGraphGrid2D::process_grid, include/general/algebra/graph/
// bgmgraphgrid{1D,2D}.h).
//
// Layout: T timesteps, R nodes, K clusters; gamma block s = t*R + r holds K values
// (index s*K + k, Decomposition with DDR_size = 1); data has T*R values (index s).
// The operator couples (t, r) with (t+-1, r) by -2 and with (t, r'), (t+-1, r') by -1 for every
// graph neighbour r'; the diagonal makes every row sum to zero.  In difference form:
//   (A_hat x)_s = sum over couplings (s, s', w) of w (x_s - x_s').
//
// Kernels:
//   graph_matmult_f64_kernel   the assembled row in PETSc's sorted column order (FP64; the
//                              fp64 solver path and the standalone entry point)
//   graph_sweep_a_kernel       mixed path, one SPG iteration, part 1: x^{c+1} = x^c + beta d
//                              (INIT: the projected start point), g^{c+1} in difference form,
//                              f, d_{c+2} = P(x^{c+1} - alpha g^{c+1}) - x^{c+1}, d'd, g'd;
//                              writes x^{c+1} and d_{c+2}
//   graph_sweep_b_kernel       part 2: d'A d from the stored d_{c+2} (edge form, every
//                              coupling counted from both ends), and on the last block the
//                              step-length / GLL / stop logic of the 1-D sweeps
// A general graph cannot be tiled with a bounded halo the way the 1-D chain is (g^{c+1} needs
// x^{c+1} of the neighbours, d'Ad needs d_{c+2} of the neighbours), so the mixed path keeps
// x and d in HBM and makes two passes per iteration: 5 FP32 vectors of traffic per iteration
// (read x, d; write x, d; read d) plus the data, against 2 for the 1-D fused sweep.  Neighbour
// reads of an image grid hit L1/L2.
#include <math.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "project.cuh"
#include "sweep_common.cuh"
#include "internal.h"

namespace pasc {

// ---------------------------------------------------------------------------------------
// FP64 operator, assembled order
// ---------------------------------------------------------------------------------------
__global__ void graph_matmult_f64_kernel(const double *x, double *y, long T, long R, int K, double coeff,
                                         const double *kc, const int *ptr, const int *idx)
{
    const long n = T * R * K;
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long s = i / K;
        const int k = (int)(i - s * K);
        const long t = s / R, r = s - t * R;
        const int q0 = ptr[r], q1 = ptr[r + 1], m = q1 - q0;
        double wsum;
        if (t == 0 || t == T - 1) wsum = T > 1 ? (double)(2 * m + 2) : (double)m;
        else wsum = (double)(3 * m + 4);
        double sum = 0.0;
        for (long tt = t - 1; tt <= t + 1; tt++) {
            if (tt < 0 || tt >= T) continue;
            int q = q0;
            bool self = false;
            while (q < q1 || !self) {
                long rn;
                double v;
                if (!self && (q >= q1 || idx[q] > r)) {
                    rn = r;
                    v = tt == t ? wsum : -2.0;
                    self = true;
                } else {
                    rn = idx[q++];
                    v = -1.0;
                }
                sum = __dadd_rn(sum, __dmul_rn(v, x[(tt * R + rn) * K + k]));
            }
        }
        y[i] = __dmul_rn(kc ? kc[k] : coeff, sum);
    }
}

static int graph_grid(long work, int threads)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long blocks = (work + threads - 1) / threads;
    const long cap = (long)sms * 8;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

cudaError_t launch_graph_matmult_f64(const double *x, double *y, long T, long R, int K, double coeff,
                                     const int *ptr, const int *idx, cudaStream_t s, const double *kc)
{
    if (T * R <= 0) return cudaSuccess;
    graph_matmult_f64_kernel<<<graph_grid(T * R * K, 256), 256, 0, s>>>(x, y, T, R, K, coeff, kc, ptr, idx);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// Mixed path: two kernels per SPG iteration
// ---------------------------------------------------------------------------------------
constexpr int GRAPH_NT = 256;

// x^{c+1} of block s: x + beta d, or (INIT) the projected start point
template <int K, bool INIT>
__device__ __forceinline__ void next_x(const float *__restrict__ xin, const float *__restrict__ din, long s,
                                       float beta, float (&v)[K])
{
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = __ldg(xin + s * K + k);
    if (INIT) {
        project_reg<K>(v);
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = fmaf(beta, __ldg(din + s * K + k), v[k]);
    }
}

// calls f(s', w) for every coupling of block s = t*R + r
template <typename F>
__device__ __forceinline__ void for_each_coupling(long t, long r, long T, long R, const int *__restrict__ ptr,
                                                  const int *__restrict__ idx, F f)
{
    const int q0 = __ldg(ptr + r), q1 = __ldg(ptr + r + 1);
    for (int q = q0; q < q1; q++) f(t * R + __ldg(idx + q), 1.f);
    if (t > 0) {
        f((t - 1) * R + r, 2.f);
        for (int q = q0; q < q1; q++) f((t - 1) * R + __ldg(idx + q), 1.f);
    }
    if (t < T - 1) {
        f((t + 1) * R + r, 2.f);
        for (int q = q0; q < q1; q++) f((t + 1) * R + __ldg(idx + q), 1.f);
    }
}

template <int K, bool INIT>
__global__ void __launch_bounds__(GRAPH_NT) graph_sweep_a_kernel(GraphSweepArgs a)
{
    __shared__ double s_red[3 * (GRAPH_NT / 32)];
    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;  // uniform across the grid
    const int cur = st->cur;
    const float *__restrict__ xin = cur ? a.xb1 : a.xb0;
    float *__restrict__ xout = cur ? a.xb0 : a.xb1;
    const float *__restrict__ din = cur ? a.db1 : a.db0;
    float *__restrict__ dout = cur ? a.db0 : a.db1;
    const float beta = (float)st->beta, a1 = (float)st->alpha_cur;
    const float coeff = (float)st->coeff, bscale = (float)st->bscale;
    const long T = a.T, R = a.R, NB = T * R;
    float theta[K];
#pragma unroll
    for (int k = 0; k < K; k++) theta[k] = a.theta[k];

    KahanF acc_f;
    float acc_dd = 0.f, acc_gd = 0.f;
    const long stride = (long)gridDim.x * GRAPH_NT;
    for (long s = (long)blockIdx.x * GRAPH_NT + threadIdx.x; s < NB; s += stride) {
        const long t = s / R, r = s - t * R;
        float x1[K], S[K];
        next_x<K, INIT>(xin, din, s, beta, x1);
#pragma unroll
        for (int k = 0; k < K; k++) S[k] = 0.f;
        for_each_coupling(t, r, T, R, a.ptr, a.idx, [&](long sn, float w) {
            float xn[K];
            next_x<K, INIT>(xin, din, sn, beta, xn);
#pragma unroll
            for (int k = 0; k < K; k++) S[k] = fmaf(w, x1[k] - xn[k], S[k]);
        });
        const float dv = __ldg(a.data + s);
        float g1[K], d1[K], fpart = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float rr = dv - theta[k];
            const float bk = bscale * (rr * rr);
            g1[k] = fmaf(coeff, S[k], -bk);
            fpart += (g1[k] - bk) * x1[k];
            d1[k] = fmaf(-a1, g1[k], x1[k]);
        }
        acc_f.add(fpart);
        project_reg<K>(d1);
#pragma unroll
        for (int k = 0; k < K; k++) {
            d1[k] -= x1[k];
            acc_dd = fmaf(d1[k], d1[k], acc_dd);
            acc_gd = fmaf(g1[k], d1[k], acc_gd);
            __stcg(xout + s * K + k, x1[k]);
            __stcg(dout + s * K + k, d1[k]);
        }
    }
    double v[3] = {acc_f.value(), (double)acc_dd, (double)acc_gd};
    block_sum<3>(v, s_red);
    if (threadIdx.x == 0) {
        a.partials[blockIdx.x * 4 + 0] = v[0];
        a.partials[blockIdx.x * 4 + 1] = v[1];
        a.partials[blockIdx.x * 4 + 3] = v[2];
    }
}

template <int K, bool INIT>
__global__ void __launch_bounds__(GRAPH_NT) graph_sweep_b_kernel(GraphSweepArgs a)
{
    __shared__ double s_red[4 * (GRAPH_NT / 32)];
    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;
    const int cur = st->cur;
    const float *__restrict__ dn = cur ? a.db0 : a.db1;  // d_{c+2}, written by part 1
    const long T = a.T, R = a.R, NB = T * R;
    float acc = 0.f;
    const long stride = (long)gridDim.x * GRAPH_NT;
    for (long s = (long)blockIdx.x * GRAPH_NT + threadIdx.x; s < NB; s += stride) {
        const long t = s / R, r = s - t * R;
        float d[K];
#pragma unroll
        for (int k = 0; k < K; k++) d[k] = __ldcg(dn + s * K + k);
        for_each_coupling(t, r, T, R, a.ptr, a.idx, [&](long sn, float w) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float df = d[k] - __ldcg(dn + sn * K + k);
                acc = fmaf(w * df, df, acc);
            }
        });
    }
    // d'A_hat d = 1/2 sum_s sum_couplings w (d_s - d_s')^2; the finish step takes
    // dAd = 2 coeff w[2], so w[2] carries a quarter of the double sum
    double v[1] = {0.25 * (double)acc};
    block_sum<1>(v, s_red);
    if (threadIdx.x == 0) a.partials[blockIdx.x * 4 + 2] = v[0];
    if (!last_block_done(&st->counter)) return;
    double w[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += GRAPH_NT) {
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] += __ldcg(a.partials + b * 4 + q);
    }
    block_sum<4>(w, s_red);
    if (threadIdx.x != 0) return;
    spg_finish_sweep<INIT>(st, cur, w);
}

int graph_sweep_grid(long nblocks)
{
    return graph_grid(nblocks, GRAPH_NT);
}

template <int K, bool INIT>
static cudaError_t launch_graph_t(int grid, const GraphSweepArgs &a, cudaStream_t s)
{
    graph_sweep_a_kernel<K, INIT><<<grid, GRAPH_NT, 0, s>>>(a);
    graph_sweep_b_kernel<K, INIT><<<grid, GRAPH_NT, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_graph_sweep(int K, bool init, int grid, const GraphSweepArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK) \
    case KK: return init ? launch_graph_t<KK, true>(grid, a, s) : launch_graph_t<KK, false>(grid, a, s);
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------------------
// Host: graphs and their checks
// ---------------------------------------------------------------------------------------
const char *graph_check(long R, const int *ptr, const int *idx)
{
    if (R < 1) return "R must be >= 1";
    if (!ptr) return "NULL neighbour offsets";
    if (ptr[0] != 0) return "nbr_ptr[0] must be 0";
    for (long r = 0; r < R; r++)
        if (ptr[r + 1] < ptr[r]) return "nbr_ptr must be non-decreasing";
    if (ptr[R] > 0 && !idx) return "NULL neighbour indices";
    for (long r = 0; r < R; r++) {
        for (int q = ptr[r]; q < ptr[r + 1]; q++) {
            const int j = idx[q];
            if (j < 0 || j >= R) return "neighbour index out of range";
            if (j == r) return "a node cannot be its own neighbour";
            if (q > ptr[r] && idx[q - 1] >= j) return "neighbour lists must be sorted ascending without duplicates";
            // symmetry: r must appear in j's list
            if (!std::binary_search(idx + ptr[j], idx + ptr[j + 1], (int)r)) return "the graph must be symmetric";
        }
    }
    return nullptr;
}

// true when the lists are those of BGMGraphGrid2D(W, H) with H >= 2 (node i*W + j)
bool graph_is_grid2d(long R, const int *ptr, const int *idx, int *W, int *H)
{
    if (R < 4 || ptr[1] - ptr[0] < 1 || idx[ptr[0]] != 1) return false;
    long w;
    if (ptr[1] - ptr[0] == 2 && idx[ptr[0] + 1] >= 2) w = idx[ptr[0] + 1];
    else return false;
    if (R % w != 0 || R / w < 2) return false;
    const long h = R / w;
    long q = 0;
    for (long id = 0; id < R; id++) {
        const long i = id / w, j = id - i * w;
        if (ptr[id] != q) return false;
        if (i > 0 && idx[q++] != id - w) return false;
        if (j > 0 && idx[q++] != id - 1) return false;
        if (j < w - 1 && idx[q++] != id + 1) return false;
        if (i < h - 1 && idx[q++] != id + w) return false;
    }
    if (ptr[R] != q || w > 2000000000L || h > 2000000000L) return false;
    *W = (int)w;
    *H = (int)h;
    return true;
}

}  // namespace pasc

using namespace pasc;

extern "C" {

int pasc_gb300_graph_grid1d(int width, int *nbr_ptr, int *nbr_idx)
{
    if (width < 1 || !nbr_ptr || (width > 1 && !nbr_idx)) {
        record_error("graph_grid1d: width >= 1 and non-NULL outputs needed");
        return PASC_ERR_ARG;
    }
    int q = 0;
    for (int i = 0; i < width; i++) {
        nbr_ptr[i] = q;
        if (i > 0) nbr_idx[q++] = i - 1;
        if (i < width - 1) nbr_idx[q++] = i + 1;
    }
    nbr_ptr[width] = q;
    return PASC_OK;
}

int pasc_gb300_graph_grid2d(int width, int height, int *nbr_ptr, int *nbr_idx)
{
    if (width < 1 || height < 1 || (long)width * height > 2000000000L || !nbr_ptr ||
        ((width > 1 || height > 1) && !nbr_idx)) {
        record_error("graph_grid2d: width, height >= 1 and non-NULL outputs needed");
        return PASC_ERR_ARG;
    }
    const int n = width * height;
    int q = 0;
    for (int id = 0; id < n; id++) {
        const int i = id / width, j = id - i * width;  // row, column
        nbr_ptr[id] = q;
        if (i > 0) nbr_idx[q++] = id - width;           // down
        if (j > 0) nbr_idx[q++] = id - 1;               // left
        if (j < width - 1) nbr_idx[q++] = id + 1;       // right
        if (i < height - 1) nbr_idx[q++] = id + width;  // up
    }
    nbr_ptr[n] = q;
    return PASC_OK;
}

int pasc_gb300_graph_threshold(const double *coords, int n, int dim, double threshold, int *nbr_ptr, int *nbr_idx,
                               long idx_capacity, long *nnz)
{
    if (!coords || n < 1 || dim < 1 || !nbr_ptr || !nnz) {
        record_error("graph_threshold: coords, n >= 1, dim >= 1, nbr_ptr and nnz needed");
        return PASC_ERR_ARG;
    }
    const double thr2 = threshold * threshold;
    auto close = [&](int i, int j) {
        double s = 0.0;
        for (int d = 0; d < dim; d++) {
            const double df = coords[i + (long)d * n] - coords[j + (long)d * n];
            s += df * df;
        }
        return s < thr2;
    };
    std::vector<long> cnt((size_t)n, 0);
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (close(i, j)) {
                cnt[i]++;
                cnt[j]++;
            }
    long q = 0;
    for (int i = 0; i < n; i++) {
        if (q > 2000000000L) {
            record_error("graph_threshold: too many edges");
            return PASC_ERR_ARG;
        }
        nbr_ptr[i] = (int)q;
        q += cnt[i];
    }
    if (q > 2000000000L) {
        record_error("graph_threshold: too many edges");
        return PASC_ERR_ARG;
    }
    nbr_ptr[n] = (int)q;
    *nnz = q;
    if (!nbr_idx) return PASC_OK;  // sizes only
    if (idx_capacity < q) {
        record_error("graph_threshold: nbr_idx holds fewer than nnz entries");
        return PASC_ERR_ARG;
    }
    for (int i = 0; i < n; i++) cnt[i] = nbr_ptr[i];
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++)
            if (close(i, j)) {
                nbr_idx[cnt[i]++] = j;
                nbr_idx[cnt[j]++] = i;
            }
    return PASC_OK;
}

int pasc_gb300_graph_matmult_f64(const double *x_dev, double *y_dev, long T, long R, int K, double coeff,
                                 const int *nbr_ptr_dev, const int *nbr_idx_dev, void *stream)
{
    if (!x_dev || !y_dev || !nbr_ptr_dev || T < 1 || R < 1 || K < 1) {
        record_error("graph_matmult_f64: NULL argument or T, R, K < 1");
        return PASC_ERR_ARG;
    }
    if (launch_graph_matmult_f64(x_dev, y_dev, T, R, K, coeff, nbr_ptr_dev, nbr_idx_dev, (cudaStream_t)stream,
                                 nullptr) != cudaSuccess) {
        record_error("graph_matmult_f64: kernel launch failed");
        return PASC_ERR_CUDA;
    }
    return PASC_OK;
}

}  // extern "C"
