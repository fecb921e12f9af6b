// image.cu -- the fused mixed-precision SPG sweep for image data: one timestep (T = 1) on the
// 4-neighbour pixel grid (BGMGraphGrid2D, include/general/algebra/graph/bgmgraphgrid2D.h:88-142)
// with the operator of blockgraphsparse.cpp:48-103 at T = 1: (A_hat x)_p = sum over the
// in-image neighbours n of p of (x_p - x_n).
//
// The general graph path (graph.cu) keeps x and d in HBM and makes two passes per iteration;
// on the grid a tile with a halo of 3 pixels holds everything one SPG iteration needs, so this
// kernel does what the 1-D bulk-copy sweep does, in two dimensions: one pass over HBM per
// iteration, x the only state (read x and data, write x).
//
// One block takes a 26 x 26 tile of owned pixels at a time and stages the 32 x 32 region around
// it in shared memory (structure of arrays, one plane per cluster; one warp lane per column,
// so no index arithmetic beyond row and lane; tiles away from the image border run without
// range checks):
//   A  x^c of the region (INIT: projected), data of the region;
//   B  on the region less 1 pixel: g^c = coeff A_hat x^c - b, x^{c+1} = x^c + beta d_{c+1}
//      with d_{c+1} = P(x^c - alpha g^c) - x^c   (INIT: x^{c+1} = x^c);
//   C  on the region less 2 pixels: g^{c+1}, d_{c+2} = P(x^{c+1} - alpha' g^{c+1}) - x^{c+1}
//      (stored over x^c), and on owned pixels the objective, d'd and g'd;
//   D  on owned pixels: d'A_hat d in edge form (each neighbour pair counted from both ends)
//      and the store of x^{c+1}.
// Pixels outside the image hold zeros and are no one's neighbours.  The last block applies the
// step-length / GLL / stop logic of the 1-D sweeps (sweep_common.cuh).
#include "common.cuh"
#include "project.cuh"
#include "sweep_common.cuh"
#include "internal.h"

namespace pasc {

constexpr int IMG_NT = 256;                       // 8 warps
constexpr int IMG_S = 32, IMG_HALO = 3;            // staged region 32 x 32 (one warp lane per column)
constexpr int IMG_TW = IMG_S - 2 * IMG_HALO;       // 26 x 26 owned pixels per tile
constexpr int IMG_NS = IMG_S * IMG_S;
constexpr int IMG_ROWS_PER_WARP = IMG_S / (IMG_NT / 32);

template <int K>
struct ImgSmem {
    float xs[K * IMG_NS];  // x^c, then d_{c+2} (plane k at k*IMG_NS, row-major 32 x 32)
    float ys[K * IMG_NS];  // x^{c+1}
    float dat[IMG_NS];
    double red[4 * (IMG_NT / 32)];
};

size_t image_sweep_smem(int K)
{
    switch (K) {
#define PASC_CASE(KK) case KK: return sizeof(ImgSmem<KK>);
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 0;
    }
}

// sum over the in-image neighbours n of staged pixel s (image coordinates gx, gy) of
// (v_s - v_n); EDGE = false: all four neighbours exist
template <bool EDGE>
__device__ __forceinline__ float grid_diff(const float *v, int s, int gx, int gy, int W, int H)
{
    const float c = v[s];
    if (!EDGE) return ((c - v[s - 1]) + (c - v[s + 1])) + ((c - v[s - IMG_S]) + (c - v[s + IMG_S]));
    float S = 0.f;
    if (gx > 0) S += c - v[s - 1];
    if (gx < W - 1) S += c - v[s + 1];
    if (gy > 0) S += c - v[s - IMG_S];
    if (gy < H - 1) S += c - v[s + IMG_S];
    return S;
}

// One tile: phases A-D for the 26 x 26 pixels owned by the tile with staged origin (ox, oy).
// Warp w takes the staged rows w, w+8, w+16, w+24; lane l the column l.
template <int K, bool INIT, bool EDGE>
__device__ __forceinline__ void image_tile(ImgSmem<K> &sm, const ImageSweepArgs &a, const float *__restrict__ xin,
                                           float *__restrict__ xout, int ox, int oy, const float (&theta)[K],
                                           float a0, float beta, float a1, float coeff, float bscale, KahanF &acc_f,
                                           float &acc_dd, float &acc_gd, float &acc_dad)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int W = a.W, H = a.H;
    const int gx = ox + lane;
    const bool colin = !EDGE || (unsigned)gx < (unsigned)W;

    // A: stage x^c (INIT: projected) and the data
#pragma unroll
    for (int j = 0; j < IMG_ROWS_PER_WARP; j++) {
        const int r = warp + j * (IMG_NT / 32), gy = oy + r, s = r * IMG_S + lane;
        const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
        const long pix = (long)gy * W + gx;
        float v[K];
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = in ? __ldcs(xin + pix * K + k) : 0.f;
        if (INIT && in) project_reg<K>(v);
#pragma unroll
        for (int k = 0; k < K; k++) sm.xs[k * IMG_NS + s] = v[k];
        sm.dat[s] = in ? __ldg(a.data + pix) : 0.f;
    }
    __syncthreads();

    // B: x^{c+1} on rows / columns 1..30
    if (lane >= 1 && lane <= IMG_S - 2) {
#pragma unroll
        for (int j = 0; j < IMG_ROWS_PER_WARP; j++) {
            const int r = warp + j * (IMG_NT / 32);
            if (r < 1 || r > IMG_S - 2) continue;
            const int gy = oy + r, s = r * IMG_S + lane;
            const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
            float x1[K];
            if (INIT) {
#pragma unroll
                for (int k = 0; k < K; k++) x1[k] = sm.xs[k * IMG_NS + s];
            } else {
                float xc[K], z[K];
                const float dv = sm.dat[s];
#pragma unroll
                for (int k = 0; k < K; k++) {
                    xc[k] = sm.xs[k * IMG_NS + s];
                    const float S = grid_diff<EDGE>(sm.xs + k * IMG_NS, s, gx, gy, W, H);
                    const float rr = dv - theta[k];
                    const float g = fmaf(coeff, S, -(bscale * (rr * rr)));
                    z[k] = fmaf(-a0, g, xc[k]);
                }
                project_reg<K>(z);
#pragma unroll
                for (int k = 0; k < K; k++) x1[k] = fmaf(beta, z[k] - xc[k], xc[k]);
            }
#pragma unroll
            for (int k = 0; k < K; k++) sm.ys[k * IMG_NS + s] = in ? x1[k] : 0.f;
        }
    }
    __syncthreads();

    // C: g^{c+1}, d_{c+2} on rows / columns 2..29 (d over x^c); owned (3..28): f, d'd, g'd
    if (lane >= 2 && lane <= IMG_S - 3) {
        const bool owncol = lane >= IMG_HALO && lane < IMG_HALO + IMG_TW;
#pragma unroll
        for (int j = 0; j < IMG_ROWS_PER_WARP; j++) {
            const int r = warp + j * (IMG_NT / 32);
            if (r < 2 || r > IMG_S - 3) continue;
            const int gy = oy + r, s = r * IMG_S + lane;
            const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
            const bool own = in && owncol && r >= IMG_HALO && r < IMG_HALO + IMG_TW;
            float y[K], g1[K], d1[K], fpart = 0.f;
            const float dv = sm.dat[s];
#pragma unroll
            for (int k = 0; k < K; k++) {
                y[k] = sm.ys[k * IMG_NS + s];
                const float S = grid_diff<EDGE>(sm.ys + k * IMG_NS, s, gx, gy, W, H);
                const float rr = dv - theta[k];
                const float bk = bscale * (rr * rr);
                g1[k] = fmaf(coeff, S, -bk);
                fpart += (g1[k] - bk) * y[k];
                d1[k] = fmaf(-a1, g1[k], y[k]);
            }
            project_reg<K>(d1);
#pragma unroll
            for (int k = 0; k < K; k++) {
                d1[k] = in ? d1[k] - y[k] : 0.f;
                sm.xs[k * IMG_NS + s] = d1[k];
            }
            if (own) {
                acc_f.add(fpart);
#pragma unroll
                for (int k = 0; k < K; k++) {
                    acc_dd = fmaf(d1[k], d1[k], acc_dd);
                    acc_gd = fmaf(g1[k], d1[k], acc_gd);
                }
            }
        }
    }
    __syncthreads();

    // D: owned pixels: d'A_hat d (edge form) and the store of x^{c+1}
    if (lane >= IMG_HALO && lane < IMG_HALO + IMG_TW) {
#pragma unroll
        for (int j = 0; j < IMG_ROWS_PER_WARP; j++) {
            const int r = warp + j * (IMG_NT / 32);
            if (r < IMG_HALO || r >= IMG_HALO + IMG_TW) continue;
            const int gy = oy + r, s = r * IMG_S + lane;
            if (EDGE && !(colin && (unsigned)gy < (unsigned)H)) continue;
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float *dk = sm.xs + k * IMG_NS;
                const float c = dk[s];
                const float dl = c - dk[s - 1], dr = c - dk[s + 1], dd = c - dk[s - IMG_S], du = c - dk[s + IMG_S];
                if (!EDGE || gx > 0) acc_dad = fmaf(dl, dl, acc_dad);
                if (!EDGE || gx < W - 1) acc_dad = fmaf(dr, dr, acc_dad);
                if (!EDGE || gy > 0) acc_dad = fmaf(dd, dd, acc_dad);
                if (!EDGE || gy < H - 1) acc_dad = fmaf(du, du, acc_dad);
            }
            const long pix = (long)gy * W + gx;
#pragma unroll
            for (int k = 0; k < K; k++) __stcs(xout + pix * K + k, sm.ys[k * IMG_NS + s]);
        }
    }
    __syncthreads();  // the next tile restages the buffers
}

template <int K, bool INIT>
__global__ void __launch_bounds__(IMG_NT) image_sweep_kernel(ImageSweepArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ImgSmem<K> &sm = *reinterpret_cast<ImgSmem<K> *>(smem_raw);
    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;  // uniform across the grid
    const int cur = st->cur;
    const float *__restrict__ xin = cur ? a.xb1 : a.xb0;
    float *__restrict__ xout = cur ? a.xb0 : a.xb1;
    const float a0 = (float)st->alpha_prev, beta = (float)st->beta, a1 = (float)st->alpha_cur;
    const float coeff = (float)st->coeff, bscale = (float)st->bscale;
    const int W = a.W, H = a.H;
    float theta[K];
#pragma unroll
    for (int k = 0; k < K; k++) theta[k] = a.theta[k];
    const int tiles_x = (W + IMG_TW - 1) / IMG_TW, tiles_y = (H + IMG_TW - 1) / IMG_TW;
    const int ntiles = tiles_x * tiles_y;

    KahanF acc_f;
    float acc_dd = 0.f, acc_gd = 0.f, acc_dad = 0.f;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
        const int ox = tx * IMG_TW - IMG_HALO, oy = ty * IMG_TW - IMG_HALO;  // staged origin
        if (ox >= 0 && oy >= 0 && ox + IMG_S <= W && oy + IMG_S <= H)
            image_tile<K, INIT, false>(sm, a, xin, xout, ox, oy, theta, a0, beta, a1, coeff, bscale, acc_f, acc_dd,
                                       acc_gd, acc_dad);
        else
            image_tile<K, INIT, true>(sm, a, xin, xout, ox, oy, theta, a0, beta, a1, coeff, bscale, acc_f, acc_dd,
                                      acc_gd, acc_dad);
    }

    // d'A_hat d = 1/2 sum_p sum_n (d_p - d_n)^2; the finish step takes dAd = 2 coeff w[2]
    double v[4] = {acc_f.value(), (double)acc_dd, 0.25 * (double)acc_dad, (double)acc_gd};
    block_sum<4>(v, sm.red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++) a.partials[blockIdx.x * 4 + q] = v[q];
    }
    if (!last_block_done(&st->counter)) return;
    double w[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += IMG_NT) {
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] += __ldcg(a.partials + b * 4 + q);
    }
    block_sum<4>(w, sm.red);
    if (threadIdx.x != 0) return;
    spg_finish_sweep<INIT>(st, cur, w);
}

template <int K, bool INIT>
static int image_blocks_t()
{
    const size_t smem = sizeof(ImgSmem<K>);
    cudaFuncSetAttribute(image_sweep_kernel<K, INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, image_sweep_kernel<K, INIT>, IMG_NT, smem);
    return nb > 0 ? nb : 1;
}

// sets the shared-memory limit of both forms and returns the blocks per SM of the regular one
int image_sweep_blocks_per_sm(int K)
{
    switch (K) {
#define PASC_CASE(KK) case KK: image_blocks_t<KK, true>(); return image_blocks_t<KK, false>();
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 0;
    }
}

int image_sweep_tiles(int W, int H)
{
    return ((W + IMG_TW - 1) / IMG_TW) * ((H + IMG_TW - 1) / IMG_TW);
}

cudaError_t launch_image_sweep(int K, bool init, int grid, const ImageSweepArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK)                                                                                  \
    case KK:                                                                                           \
        if (init) image_sweep_kernel<KK, true><<<grid, IMG_NT, sizeof(ImgSmem<KK>), s>>>(a);           \
        else image_sweep_kernel<KK, false><<<grid, IMG_NT, sizeof(ImgSmem<KK>), s>>>(a);               \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pasc
