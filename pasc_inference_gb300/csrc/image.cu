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
// Each warp takes a strip tile: 32 columns (one per lane; the middle 26 owned) by IMG_TH + 6
// rows (the middle IMG_TH owned), walked top to bottom with everything in registers:
//   A  load x^c of the next row (INIT: projected) and its data;
//   B  on the row above it: g^c = coeff A_hat x^c - b, x^{c+1} = x^c + beta d_{c+1} with
//      d_{c+1} = P(x^c - alpha g^c) - x^c   (INIT: x^{c+1} = x^c);
//   C  one row higher: g^{c+1}, d_{c+2} = P(x^{c+1} - alpha' g^{c+1}) - x^{c+1}, and on owned
//      pixels the objective, d'd and g'd;
//   D  one row higher again, on owned pixels: d'A_hat d in edge form (each neighbour pair
//      counted from both ends) and the store of x^{c+1}.
// Left and right neighbours come from the adjacent lanes (shuffles), up and down from the
// three-row windows; there is no shared memory and no block barrier in the sweep.  Strip tiles
// away from the image border run without range checks.
// Pixels outside the image hold zeros and are no one's neighbours.  The last block applies the
// step-length / GLL / stop logic of the 1-D sweeps (sweep_common.cuh).
#include "common.cuh"
#include "project.cuh"
#include "sweep_common.cuh"
#include "internal.h"

namespace pasc {

constexpr int IMG_NT = 256;                  // 8 warps, each on its own strip tile
constexpr int IMG_HALO = 3;
constexpr int IMG_TW = 32 - 2 * IMG_HALO;     // 26 owned columns per warp (one lane per column)
constexpr int IMG_TH = 63;                    // owned rows per strip tile (staged rows a multiple of 3)
constexpr int IMG_SH = IMG_TH + 2 * IMG_HALO; // staged rows
constexpr int IMG_PF = 3;                     // rows in flight per warp (a multiple of the 3-row windows)

// x^c and data of staged row i of a strip tile (zeros outside the image)
template <int K, bool EDGE>
__device__ __forceinline__ void image_load_row(const ImageSweepArgs &a, const float *__restrict__ xin, int i, int oy,
                                               int gx, bool colin, int H, int W, float (&x)[K], float &d)
{
    const int gy = oy + i;
    const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
    const long pix = (long)gy * W + gx;
#pragma unroll
    for (int k = 0; k < K; k++) x[k] = in ? __ldcs(xin + pix * K + k) : 0.f;
    d = in ? __ldg(a.data + pix) : 0.f;
}

struct ImgSmem {
    double red[4 * (IMG_NT / 32)];
};

// sum over the in-image neighbours of (v_c - v_n); l, r from the neighbouring lanes, u, d from
// the rows above and below.  EDGE = false: all four neighbours exist.
template <bool EDGE>
__device__ __forceinline__ float grid_diff(float c, float l, float r, float u, float d, int gx, int gy, int W,
                                           int H)
{
    if (!EDGE) return ((c - l) + (c - r)) + ((c - u) + (c - d));
    float S = 0.f;
    if (gx > 0) S += c - l;
    if (gx < W - 1) S += c - r;
    if (gy > 0) S += c - u;
    if (gy < H - 1) S += c - d;
    return S;
}

// One strip tile of a warp: columns ox .. ox+31 (lane = column; 26 owned in the middle), staged
// rows oy .. oy+IMG_SH-1 (IMG_TH owned in the middle), walked top to bottom.  At step i the
// warp loads row i and computes, in registers, phase B on row i-1, phase C on row i-2 and
// phase D on row i-3, keeping three-row windows of x^c (X), x^{c+1} (Y) and d_{c+2} (D);
// left and right neighbours come from the adjacent lanes.  Lanes and rows near the tile's
// border compute values that only their inner neighbours use (halo of 3).
template <int K, bool INIT, bool EDGE>
__device__ __forceinline__ void image_strip(const ImageSweepArgs &a, const float *__restrict__ xin,
                                            float *__restrict__ xout, int ox, int oy, const float (&theta)[K],
                                            float a0, float beta, float a1, float coeff, float bscale, KahanF &acc_f,
                                            float &acc_dd, float &acc_gd, float &acc_dad)
{
    const int lane = threadIdx.x & 31;
    const int W = a.W, H = a.H;
    const int gx = ox + lane;
    const bool colin = !EDGE || (unsigned)gx < (unsigned)W;
    const bool laneB = lane >= 1 && lane <= 30, laneC = lane >= 2 && lane <= 29;
    const bool laneD = lane >= IMG_HALO && lane < IMG_HALO + IMG_TW;
    float X0[K], X1[K], X2[K], Y0[K], Y1[K], Y2[K], D0[K], D1[K], D2[K];
    float dat1 = 0.f, dat2 = 0.f;  // data of rows i-1 and i
    float datC = 0.f;              // data of row i-2
#pragma unroll
    for (int k = 0; k < K; k++) {
        X0[k] = X1[k] = X2[k] = 0.f;
        Y0[k] = Y1[k] = Y2[k] = 0.f;
        D0[k] = D1[k] = D2[k] = 0.f;
    }
    // rows are prefetched IMG_PF ahead (ring of registers, static slots through the unrolled
    // inner loop) so that each warp keeps several row loads in flight
    float PX[IMG_PF][K], PD[IMG_PF];
#pragma unroll
    for (int q = 0; q < IMG_PF; q++) image_load_row<K, EDGE>(a, xin, q, oy, gx, colin, H, W, PX[q], PD[q]);
#pragma unroll 1
    for (int i0 = 0; i0 < IMG_SH; i0 += IMG_PF) {
#pragma unroll
        for (int q = 0; q < IMG_PF; q++) {
            const int i = i0 + q;
            if (i >= IMG_SH) break;  // uniform
            // row i arrives from slot q; slot q is refilled with row i + IMG_PF
            {
#pragma unroll
                for (int k = 0; k < K; k++) {
                    X0[k] = X1[k];
                    X1[k] = X2[k];
                    X2[k] = PX[q][k];
                }
                datC = dat1;
                dat1 = dat2;
                dat2 = PD[q];
                if (INIT && colin && (!EDGE || (unsigned)(oy + i) < (unsigned)H)) project_reg<K>(X2);
                if (i + IMG_PF < IMG_SH) image_load_row<K, EDGE>(a, xin, i + IMG_PF, oy, gx, colin, H, W, PX[q], PD[q]);
            }
            // B on row i-1: x^{c+1}
            {
                const int r = i - 1, gy = oy + r;
                const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
                float y[K];
                if (INIT) {
#pragma unroll
                    for (int k = 0; k < K; k++) y[k] = X1[k];
                } else {
                    float z[K];
#pragma unroll
                    for (int k = 0; k < K; k++) {
                        const float l = __shfl_up_sync(0xffffffffu, X1[k], 1), rr_ = __shfl_down_sync(0xffffffffu, X1[k], 1);
                        const float S = grid_diff<EDGE>(X1[k], l, rr_, X0[k], X2[k], gx, gy, W, H);
                        const float rr = dat1 - theta[k];
                        const float g = fmaf(coeff, S, -(bscale * (rr * rr)));
                        z[k] = fmaf(-a0, g, X1[k]);
                    }
                    project_reg<K>(z);
#pragma unroll
                    for (int k = 0; k < K; k++) y[k] = fmaf(beta, z[k] - X1[k], X1[k]);
                }
                const bool ok = in && laneB && r >= 1;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    Y0[k] = Y1[k];
                    Y1[k] = Y2[k];
                    Y2[k] = ok ? y[k] : 0.f;
                }
            }
            // C on row i-2: g^{c+1}, d_{c+2}; owned: f, d'd, g'd
            {
                const int r = i - 2, gy = oy + r;
                const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
                float g1[K], d1[K], fpart = 0.f;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const float l = __shfl_up_sync(0xffffffffu, Y1[k], 1), rr_ = __shfl_down_sync(0xffffffffu, Y1[k], 1);
                    const float S = grid_diff<EDGE>(Y1[k], l, rr_, Y0[k], Y2[k], gx, gy, W, H);
                    const float rr = datC - theta[k];
                    const float bk = bscale * (rr * rr);
                    g1[k] = fmaf(coeff, S, -bk);
                    fpart += (g1[k] - bk) * Y1[k];
                    d1[k] = fmaf(-a1, g1[k], Y1[k]);
                }
                project_reg<K>(d1);
                const bool ok = in && laneC && r >= 2;
                const bool own = ok && laneD && r >= IMG_HALO && r < IMG_HALO + IMG_TH;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    d1[k] = ok ? d1[k] - Y1[k] : 0.f;
                    D0[k] = D1[k];
                    D1[k] = D2[k];
                    D2[k] = d1[k];
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
            // D on row i-3: d'A_hat d (edge form), store x^{c+1} (Y0 holds row i-3)
            {
                const int r = i - 3, gy = oy + r;
                const bool in = colin && (!EDGE || (unsigned)gy < (unsigned)H);
                const bool own = in && laneD && r >= IMG_HALO && r < IMG_HALO + IMG_TH;
                float part = 0.f;
#pragma unroll
                for (int k = 0; k < K; k++) {
                    const float l = __shfl_up_sync(0xffffffffu, D1[k], 1), rr_ = __shfl_down_sync(0xffffffffu, D1[k], 1);
                    const float c = D1[k];
                    const float dl = c - l, dr = c - rr_, du = c - D0[k], dd = c - D2[k];
                    if (!EDGE || gx > 0) part = fmaf(dl, dl, part);
                    if (!EDGE || gx < W - 1) part = fmaf(dr, dr, part);
                    if (!EDGE || gy > 0) part = fmaf(du, du, part);
                    if (!EDGE || gy < H - 1) part = fmaf(dd, dd, part);
                }
                if (own) {
                    acc_dad += part;
                    const long pix = (long)gy * W + gx;
#pragma unroll
                    for (int k = 0; k < K; k++) __stcs(xout + pix * K + k, Y0[k]);
                }
            }
        }
    }
}

template <int K, bool INIT>
__global__ void __launch_bounds__(IMG_NT) image_sweep_kernel(ImageSweepArgs a)
{
    __shared__ ImgSmem sm;
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
    const int tiles_x = (W + IMG_TW - 1) / IMG_TW, tiles_y = (H + IMG_TH - 1) / IMG_TH;
    const int ntiles = tiles_x * tiles_y;
    const int warps = IMG_NT / 32, warp = threadIdx.x >> 5;

    KahanF acc_f;
    float acc_dd = 0.f, acc_gd = 0.f, acc_dad = 0.f;
    for (int tile = blockIdx.x * warps + warp; tile < ntiles; tile += gridDim.x * warps) {
        const int ty = tile / tiles_x, tx = tile - ty * tiles_x;
        const int ox = tx * IMG_TW - IMG_HALO, oy = ty * IMG_TH - IMG_HALO;  // staged origin
        if (ox >= 0 && oy >= 0 && ox + 32 <= W && oy + IMG_SH <= H)
            image_strip<K, INIT, false>(a, xin, xout, ox, oy, theta, a0, beta, a1, coeff, bscale, acc_f, acc_dd,
                                        acc_gd, acc_dad);
        else
            image_strip<K, INIT, true>(a, xin, xout, ox, oy, theta, a0, beta, a1, coeff, bscale, acc_f, acc_dd,
                                       acc_gd, acc_dad);
    }

    // d'A_hat d = 1/2 sum_p sum_n (d_p - d_n)^2; the finish step takes dAd = 2 coeff w[2]
    // (the factor 1/4 is exact in FP32)
    double w[4];
    if (!sweep_grid_sum4(acc_f, acc_dd, 0.25f * acc_dad, acc_gd, reinterpret_cast<float2 *>(a.partials), blockIdx.x,
                         &st->counter, gridDim.x, 0, 1, reinterpret_cast<float2 *>(sm.red), w))
        return;
    spg_finish_sweep<INIT>(st, cur, w);
}

template <int K, bool INIT>
static int image_blocks_t()
{
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, image_sweep_kernel<K, INIT>, IMG_NT, 0);
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

// blocks with work: each takes IMG_NT / 32 strip tiles at a time
int image_sweep_tiles(int W, int H)
{
    const int tiles = ((W + IMG_TW - 1) / IMG_TW) * ((H + IMG_TH - 1) / IMG_TH);
    return (tiles + IMG_NT / 32 - 1) / (IMG_NT / 32);
}

cudaError_t launch_image_sweep(int K, bool init, int grid, const ImageSweepArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK)                                                                                  \
    case KK:                                                                                           \
        if (init) image_sweep_kernel<KK, true><<<grid, IMG_NT, 0, s>>>(a);                             \
        else image_sweep_kernel<KK, false><<<grid, IMG_NT, 0, s>>>(a);                                 \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace pasc
