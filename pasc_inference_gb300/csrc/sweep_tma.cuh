// sweep_tma.cuh -- the bulk-copy form of the fused SPG sweep, as reusable pieces: PTX helpers
// for mbarriers and 1-D bulk copies, the shared-memory stage layout, and the computation of
// one tile (phases A-D of the sweep for 4 timesteps per thread).  Used by the single-problem
// kernel (kernels_sweep_tma.cu) and the batched kernel (kernels_batch.cu).
//
// A tile is P = NT*4 consecutive timesteps of one signal starting at t0 (a multiple of 4
// minus the 4-timestep halo): thread 0 and thread NT-1 compute halo only, threads 1..NT-2
// own 4 timesteps each (W = P - 8 owned timesteps).  Gamma and data of the tile arrive in
// stage s of a two-stage shared buffer through bulk copies that complete on the stage's
// mbarrier; buffers carry zero pads so that every copy is in bounds.
#pragma once

#include "common.cuh"
#include "project.cuh"
#include "internal.h"

namespace pasc {

constexpr int TMA_R = 4;          // timesteps per thread
constexpr int TMA_HALO = 4;       // halo timesteps on each side of a tile
constexpr unsigned int TMA_WAIT_LIMIT = 1u << 24;  // try_wait rounds before giving up
constexpr int TMA_NO_REFILL = -(1 << 30);

__device__ __forceinline__ unsigned int smem_addr(const void *p)
{
    return (unsigned int)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned int bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared; src, dst 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned int bytes, unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Waits for the phase `parity` of the barrier to complete; false if it did not within the limit.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned int parity)
{
    const unsigned int a = smem_addr(bar);
    for (unsigned int it = 0; it < TMA_WAIT_LIMIT; it++) {
        unsigned int done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Shared memory of a block, sized for up to KB clusters.  BM: the stages carry the tile's b
// (P*K values, materialised for multichannel data) instead of its data values.  R: timesteps
// per thread (4, or 2 for large K, whose per-thread arrays would not fit the registers).
template <int KB, int NT, bool BM = false, int R = TMA_R>
struct TmaSmem {
    static constexpr int P = NT * R;
    alignas(16) float x[2][P * KB];  // gamma tile, two stages (stride K for K <= KB)
    alignas(16) float dat[2][BM ? P * KB : P];  // data tile (BM: b tile), two stages
    // x^{c+1} of each thread's first / last timestep and d_{c+2} of its first timestep (layout:
    // nbr_idx), double buffered by tile parity: one block barrier per tile separates their
    // writes from their reads (tma_tile_body)
    float yl[2][NT * KB], yr[2][NT * KB];
    float dl[2][NT * KB];
    double red[4 * (NT / 32)];
    unsigned long long bar[2];
    int job;                          // batched kernel: the work item this block took
};

// Slot of cluster k of thread i in the neighbour arrays yl, yr, dl.  Thread-major (i*K + k)
// for odd K, whose stride meets every bank once per 32 threads; cluster-major (k*NT + i) for
// even K >= 4, where a stride of K floats would put 2-8 lanes of a warp on one bank.
template <int K, int NT>
__device__ __forceinline__ int nbr_idx(int i, int k)
{
    return (K % 2 == 0 && K >= 4) ? k * NT + i : i * K + k;
}

// Scalars of one signal's sweep.
template <int K>
struct TileScalars {
    float a0, beta, a1, coeff, bscale;
    float theta[K];
    float kw[K];  // TP: block weights theta_k^2 (block k of A is coeff * kw[k] * A_hat)
    int T;
    const float *xin;
    float *xout;
    const float *data;  // BM: the materialised b (T*K, zero pads like gamma)
    // SWZ tiles (R*K == 16): tensor maps of xin and of the materialised b over 64-byte rows,
    // and the row of timestep 0 (the front pad's rows)
    const CUtensorMap *tmx = nullptr, *tmb = nullptr;
    int roff = 0;
};

// 2-D tiled TMA load of one box into shared memory, completing on `bar` (complete_tx).
// x is the innermost coordinate (elements); x * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, unsigned long long *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// SWZ tiles: thread i's R*K = 16 values (64 bytes) are row i of the stage, brought in by a
// tensor copy with the 64-byte swizzle, which stores 16-byte chunk c of row i at chunk
// c ^ ((i >> 1) & 3) of that row (the stage base is 512-byte aligned).  Unswizzled, the rows
// 64 bytes apart put a warp's 16-byte loads of one chunk on two of the eight 16-byte bank
// groups (16 wavefronts instead of 4); swizzled, every group once per 8 lanes.
__device__ __forceinline__ int swz_chunk(int row, int c) { return c ^ ((row >> 1) & 3); }

struct TileAcc {
    KahanF f;
    float dd = 0.f, dAd = 0.f, gd = 0.f;
};

// The d'Ad term of the pair (last timestep of this thread, first timestep of the next thread)
// of a tile, left for after the next block barrier (the next tile's, or the one that ends the
// block's tiles) so that the tile needs no barrier between writing d_{c+2} and reading it.
template <int K>
struct TilePending {
    float dlast[K];
    int j;       // tile parity whose dl buffer holds the neighbour's value
    bool valid;  // this thread owns the pair and both timesteps lie in the signal
};

// Adds the pending pair term; call after a block barrier that follows the tile's phase C.
template <int K, int KB, int NT, bool BM, bool TP, int R>
__device__ __forceinline__ void tma_flush_pending(const TmaSmem<KB, NT, BM, R> &sm, const TileScalars<K> &sc,
                                                  TileAcc &acc, TilePending<K> &pend)
{
    if (pend.valid) {
        const int ri = threadIdx.x + 1;  // owners are never the last thread
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float df = sm.dl[pend.j & 1][nbr_idx<K, NT>(ri, k)] - pend.dlast[k];
            acc.dAd = fmaf(TP ? df * sc.kw[k] : df, df, acc.dAd);
        }
    }
    pend.valid = false;
}

// Thread 0: bring the tile starting at timestep t0 into stage s.
template <int K, int KB, int NT, bool BM, int R>
__device__ __forceinline__ void tma_issue(TmaSmem<KB, NT, BM, R> &sm, int s, const float *xin, const float *data,
                                          int t0)
{
    constexpr int P = NT * R;
    const unsigned int bytes_x = P * K * sizeof(float), bytes_d = (BM ? P * K : P) * sizeof(float);
    mbar_expect_tx(&sm.bar[s], bytes_x + bytes_d);
    bulk_g2s(sm.x[s], xin + (long)t0 * K, bytes_x, &sm.bar[s]);
    bulk_g2s(sm.dat[s], data + (long)t0 * (BM ? K : 1), bytes_d, &sm.bar[s]);
}

// Thread 0: the same tile by tensor copies with the 64-byte swizzle (gamma, and b when BM; the
// data values of a 1-D signal by a plain bulk copy).  The box is NT rows of 16 floats, row
// (t0 * K) / 16 + roff of the map (t0 is a multiple of 4 and of 2 for K = 4 and 8, so this
// is exact); rows past the end of a map read as zeros and count in the transaction bytes.
template <int K, int KB, int NT, bool BM, int R>
__device__ __forceinline__ void tma_issue_swz(TmaSmem<KB, NT, BM, R> &sm, int s, const TileScalars<K> &sc, int t0)
{
    static_assert(R * K == 16 && KB == K, "swizzled tiles hold one 64-byte row per thread");
    constexpr int P = NT * R;
    const unsigned int bytes_x = P * K * sizeof(float), bytes_d = (BM ? P * K : P) * sizeof(float);
    const int row = (t0 * K) / 16 + sc.roff;
    mbar_expect_tx(&sm.bar[s], bytes_x + bytes_d);
    tma_load_2d(sm.x[s], sc.tmx, 0, row, &sm.bar[s]);
    if (BM) tma_load_2d(sm.dat[s], sc.tmb, 0, row, &sm.bar[s]);
    else bulk_g2s(sm.dat[s], sc.data + (long)t0, bytes_d, &sm.bar[s]);
}

// One tile (the block's j-th) in stage s: phases A-D of the sweep.  `arrived`: this thread saw
// the stage's copy complete (its own bounded mbarrier wait).  The tile has ONE block barrier,
// after phase B, which also votes on `arrived`: if any thread's wait gave up, every thread
// returns false there (before any further copy is issued).  After the barrier thread 0 refills
// stage s with the tile at refill_t0 unless it is TMA_NO_REFILL (phase A was the stage's last
// reader), and the pending pair term of the block's previous tile is added.  The neighbour
// arrays are double buffered by j: a tile writes its parity's buffers before (yl, yr) or after
// (dl) its barrier and they are read after that barrier, while the next tile writes the other
// parity.  All threads of the block must call it.
//
// The FEM-H1 row is formed from shared neighbour differences: with D_j = x_{tb+j} -
// x_{tb+j-1} (zero when the pair crosses an end of the signal, t_j <= 0 or t_j > T-1),
// (A_hat x)_r = 2 (D_r - D_{r+1}), which is bit for bit the difference form
// 2[t>0](x_t - x_{t-1}) + 2[t<T-1](x_t - x_{t+1}) and needs one subtraction per neighbour
// pair.  EDGE: the tile touches t <= 0 or t >= T-1 and needs the range masks; interior tiles
// (all but the first and last of a signal) run without them.  TP: theta in the penalty, the
// operator of cluster k is scaled by sc.kw[k] (and so is its share of d'Ad).
template <int K, int KB, int NT, bool INIT, bool BM, bool EDGE, bool TP = false, int R = TMA_R, bool SWZ = false>
__device__ __forceinline__ bool tma_tile_body(TmaSmem<KB, NT, BM, R> &sm, int s, int j, bool arrived, int t0,
                                              const TileScalars<K> &sc, TileAcc &acc, TilePending<K> &pend,
                                              int refill_t0)
{
    const int jb = j & 1;
    constexpr int HT = TMA_HALO / R;  // halo threads at each end of the tile
    const int i = threadIdx.x;
    const int li = i > 0 ? i - 1 : i, ri = i < NT - 1 ? i + 1 : i;  // clamped neighbours
    const bool owner = i >= HT && i <= NT - 1 - HT;                  // owns its R timesteps
    const int T = sc.T;
    const int tb = t0 + i * R;  // first timestep of this thread
    const float c2 = 2.f * sc.coeff;

    // range masks: in[r] (0 <= t_r < T) and dm[j] (the pair (t_j - 1, t_j) lies in the signal)
    bool in[R], dm[R + 1];
#pragma unroll
    for (int r = 0; r < R; r++) in[r] = EDGE ? (unsigned)(tb + r) < (unsigned)T : true;
#pragma unroll
    for (int j = 0; j <= R; j++) dm[j] = EDGE ? (unsigned)(tb + j - 1) < (unsigned)(T - 1) : true;

    // phase A: this thread's 4 timesteps of x^c and b, plus the neighbours' edge values
    float xc[R][K], bk[R][K], xlft[K], xrgt[K];
    {
        float dv[R];
        if (!BM) {
            if constexpr (R == 4) {
                const float4 d4 = *reinterpret_cast<const float4 *>(&sm.dat[s][i * R]);
                dv[0] = d4.x; dv[1] = d4.y; dv[2] = d4.z; dv[3] = d4.w;
            } else {
                const float2 d2 = *reinterpret_cast<const float2 *>(&sm.dat[s][i * R]);
                dv[0] = d2.x; dv[1] = d2.y;
            }
        }
        if constexpr ((R * K) % 4 == 0) {
            const float4 *src = reinterpret_cast<const float4 *>(&sm.x[s][i * R * K]);
#pragma unroll
            for (int q = 0; q < R * K / 4; q++) {
                const float4 v = src[SWZ ? swz_chunk(i, q) : q];
                const int e = 4 * q;
                xc[(e + 0) / K][(e + 0) % K] = v.x;
                xc[(e + 1) / K][(e + 1) % K] = v.y;
                xc[(e + 2) / K][(e + 2) % K] = v.z;
                xc[(e + 3) / K][(e + 3) % K] = v.w;
            }
        } else {
            const float2 *src = reinterpret_cast<const float2 *>(&sm.x[s][i * R * K]);
#pragma unroll
            for (int q = 0; q < R * K / 2; q++) {
                const float2 v = src[q];
                const int e = 2 * q;
                xc[(e + 0) / K][(e + 0) % K] = v.x;
                xc[(e + 1) / K][(e + 1) % K] = v.y;
            }
        }
        // the neighbours' edge rows: vector loads for K = 4, 6, 8 (rows 16 or 8 bytes aligned),
        // which also spread a warp's loads over more banks (the rows lie R*K floats apart)
        const float *nl = &sm.x[s][(li * R + R - 1) * K], *nr = &sm.x[s][(ri * R) * K];
        if constexpr (SWZ) {
            // rows li and ri: the chunks of the left neighbour's last timestep, of the right
            // neighbour's first, each at its swizzled place
            const float4 *rl = reinterpret_cast<const float4 *>(&sm.x[s][li * 16]);
            const float4 *rr = reinterpret_cast<const float4 *>(&sm.x[s][ri * 16]);
            constexpr int c0 = (R - 1) * K / 4;
#pragma unroll
            for (int q = 0; q < K / 4; q++) {
                const float4 a = rl[swz_chunk(li, c0 + q)];
                const float4 c = rr[swz_chunk(ri, q)];
                xlft[4 * q] = a.x; xlft[4 * q + 1] = a.y; xlft[4 * q + 2] = a.z; xlft[4 * q + 3] = a.w;
                xrgt[4 * q] = c.x; xrgt[4 * q + 1] = c.y; xrgt[4 * q + 2] = c.z; xrgt[4 * q + 3] = c.w;
            }
        } else if constexpr (K % 4 == 0) {
#pragma unroll
            for (int q = 0; q < K / 4; q++) {
                const float4 a = reinterpret_cast<const float4 *>(nl)[q];
                const float4 c = reinterpret_cast<const float4 *>(nr)[q];
                xlft[4 * q] = a.x; xlft[4 * q + 1] = a.y; xlft[4 * q + 2] = a.z; xlft[4 * q + 3] = a.w;
                xrgt[4 * q] = c.x; xrgt[4 * q + 1] = c.y; xrgt[4 * q + 2] = c.z; xrgt[4 * q + 3] = c.w;
            }
        } else if constexpr (K % 2 == 0 && K >= 4) {
#pragma unroll
            for (int q = 0; q < K / 2; q++) {
                const float2 a = reinterpret_cast<const float2 *>(nl)[q];
                const float2 c = reinterpret_cast<const float2 *>(nr)[q];
                xlft[2 * q] = a.x; xlft[2 * q + 1] = a.y;
                xrgt[2 * q] = c.x; xrgt[2 * q + 1] = c.y;
            }
        } else {
#pragma unroll
            for (int k = 0; k < K; k++) {
                xlft[k] = nl[k];
                xrgt[k] = nr[k];
            }
        }
        if (BM) {
            // this thread's R*K values of b, in vector loads as x (scalar loads at a stride of
            // R*K floats would hit the same banks from most lanes of a warp)
            if constexpr ((R * K) % 4 == 0) {
                const float4 *b4 = reinterpret_cast<const float4 *>(&sm.dat[s][i * R * K]);
#pragma unroll
                for (int q = 0; q < R * K / 4; q++) {
                    const float4 v = b4[SWZ ? swz_chunk(i, q) : q];
                    const int e = 4 * q;
                    bk[(e + 0) / K][(e + 0) % K] = v.x;
                    bk[(e + 1) / K][(e + 1) % K] = v.y;
                    bk[(e + 2) / K][(e + 2) % K] = v.z;
                    bk[(e + 3) / K][(e + 3) % K] = v.w;
                }
            } else {
                const float2 *b2 = reinterpret_cast<const float2 *>(&sm.dat[s][i * R * K]);
#pragma unroll
                for (int q = 0; q < R * K / 2; q++) {
                    const float2 v = b2[q];
                    const int e = 2 * q;
                    bk[(e + 0) / K][(e + 0) % K] = v.x;
                    bk[(e + 1) / K][(e + 1) % K] = v.y;
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (!BM) {
                    const float rr = dv[r] - sc.theta[k];
                    bk[r][k] = sc.bscale * (rr * rr);
                }
            }
    }
    if (INIT) {
        // the start point is projected; its neighbours are projected the same way
#pragma unroll
        for (int r = 0; r < R; r++) project_reg<K>(xc[r]);
        project_reg<K>(xlft);
        project_reg<K>(xrgt);
    }
    if (EDGE) {
        // zero outside the signal (the pads hold zeros; projection of a zero block does not)
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int k = 0; k < K; k++) xc[r][k] = in[r] ? xc[r][k] : 0.f;
        const bool inl = (unsigned)(tb - 1) < (unsigned)T, inr = (unsigned)(tb + R) < (unsigned)T;
#pragma unroll
        for (int k = 0; k < K; k++) {
            xlft[k] = inl ? xlft[k] : 0.f;
            xrgt[k] = inr ? xrgt[k] : 0.f;
        }
    }

    // phase B: x^{c+1}
    float x1[R][K];
    if (INIT) {
#pragma unroll
        for (int r = 0; r < R; r++)
#pragma unroll
            for (int k = 0; k < K; k++) x1[r][k] = xc[r][k];
    } else {
#pragma unroll
        for (int k = 0; k < K; k++) {
            float D[R + 1];
            D[0] = xc[0][k] - xlft[k];
#pragma unroll
            for (int r = 1; r < R; r++) D[r] = xc[r][k] - xc[r - 1][k];
            D[R] = xrgt[k] - xc[R - 1][k];
#pragma unroll
            for (int j = 0; j <= R; j++) D[j] = dm[j] ? D[j] : 0.f;
#pragma unroll
            for (int r = 0; r < R; r++) {
                const float g = fmaf(TP ? c2 * sc.kw[k] : c2, D[r] - D[r + 1], -bk[r][k]);
                x1[r][k] = fmaf(-sc.a0, g, xc[r][k]);  // z before the projection
            }
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            project_reg<K>(x1[r]);
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float v = fmaf(sc.beta, x1[r][k] - xc[r][k], xc[r][k]);
                x1[r][k] = in[r] ? v : 0.f;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        sm.yl[jb][nbr_idx<K, NT>(i, k)] = x1[0][k];
        sm.yr[jb][nbr_idx<K, NT>(i, k)] = x1[R - 1][k];
    }
    if (!__syncthreads_and(arrived)) return false;

    // the stage is free (phase A was its last reader): refill it
    if (i == 0 && refill_t0 != TMA_NO_REFILL) {
        fence_proxy_async_smem();
        if constexpr (SWZ) tma_issue_swz<K>(sm, s, sc, refill_t0);
        else tma_issue<K>(sm, s, sc.xin, sc.data, refill_t0);
    }
    // the previous tile's d_{c+2} was written before this barrier
    tma_flush_pending<K, KB, NT, BM, TP, R>(sm, sc, acc, pend);

    // phase C: g^{c+1}, objective, d_{c+2}
    float g1[R][K], d1[R][K];
    {
        float fpart = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) {
            float E[R + 1];
            E[0] = x1[0][k] - sm.yr[jb][nbr_idx<K, NT>(li, k)];
#pragma unroll
            for (int r = 1; r < R; r++) E[r] = x1[r][k] - x1[r - 1][k];
            E[R] = sm.yl[jb][nbr_idx<K, NT>(ri, k)] - x1[R - 1][k];
#pragma unroll
            for (int j = 0; j <= R; j++) E[j] = dm[j] ? E[j] : 0.f;
#pragma unroll
            for (int r = 0; r < R; r++) {
                g1[r][k] = fmaf(TP ? c2 * sc.kw[k] : c2, E[r] - E[r + 1], -bk[r][k]);
                const float fk = (g1[r][k] - bk[r][k]) * x1[r][k];
                fpart += in[r] ? fk : 0.f;
                d1[r][k] = fmaf(-sc.a1, g1[r][k], x1[r][k]);
            }
        }
        if (owner) acc.f.add(fpart);
#pragma unroll
        for (int r = 0; r < R; r++) {
            project_reg<K>(d1[r]);
#pragma unroll
            for (int k = 0; k < K; k++) d1[r][k] = in[r] ? d1[r][k] - x1[r][k] : 0.f;
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) sm.dl[jb][nbr_idx<K, NT>(i, k)] = d1[0][k];

    // phase D: dots of d_{c+2} and the store of x^{c+1}; the pair with the next thread's first
    // timestep waits for the next barrier (TilePending)
    if (owner) {
#pragma unroll
        for (int k = 0; k < K; k++) {
#pragma unroll
            for (int r = 0; r < R; r++) {
                acc.dd = fmaf(d1[r][k], d1[r][k], acc.dd);
                acc.gd = fmaf(g1[r][k], d1[r][k], acc.gd);
                if (r < R - 1) {
                    const float df = dm[r + 1] ? d1[r + 1][k] - d1[r][k] : 0.f;  // pair (t_r, t_r + 1) inside
                    acc.dAd = fmaf(TP ? df * sc.kw[k] : df, df, acc.dAd);
                }
            }
            pend.dlast[k] = d1[R - 1][k];
        }
        pend.valid = dm[R];
        pend.j = j;
        if (!EDGE || in[R - 1]) {
            // all R timesteps inside: 16-byte stores when R*K is a multiple of 4 (tb*K*4 bytes is
            // then a multiple of 16: tb is a multiple of R), 8-byte stores otherwise
            if constexpr ((R * K) % 4 == 0) {
                float4 *dst = reinterpret_cast<float4 *>(sc.xout + (long)tb * K);
#pragma unroll
                for (int q = 0; q < R * K / 4; q++) {
                    const int e = 4 * q;
                    dst[q] = make_float4(x1[(e + 0) / K][(e + 0) % K], x1[(e + 1) / K][(e + 1) % K],
                                         x1[(e + 2) / K][(e + 2) % K], x1[(e + 3) / K][(e + 3) % K]);
                }
            } else {
                float2 *dst = reinterpret_cast<float2 *>(sc.xout + (long)tb * K);
#pragma unroll
                for (int q = 0; q < R * K / 2; q++) {
                    const int e = 2 * q;
                    dst[q] = make_float2(x1[(e + 0) / K][(e + 0) % K], x1[(e + 1) / K][(e + 1) % K]);
                }
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; r++)
                if (in[r])
#pragma unroll
                    for (int k = 0; k < K; k++) sc.xout[(long)(tb + r) * K + k] = x1[r][k];
        }
    }
    return true;
}

template <int K, int KB, int NT, bool INIT, bool BM = false, bool TP = false, int R = TMA_R, bool SWZ = false>
__device__ __forceinline__ bool tma_tile(TmaSmem<KB, NT, BM, R> &sm, int s, int j, bool arrived, int t0,
                                         const TileScalars<K> &sc, TileAcc &acc, TilePending<K> &pend, int refill_t0)
{
    constexpr int P = NT * R;
    if (t0 >= 1 && t0 + P <= sc.T - 1)
        return tma_tile_body<K, KB, NT, INIT, BM, false, TP, R, SWZ>(sm, s, j, arrived, t0, sc, acc, pend, refill_t0);
    return tma_tile_body<K, KB, NT, INIT, BM, true, TP, R, SWZ>(sm, s, j, arrived, t0, sc, acc, pend, refill_t0);
}

}  // namespace pasc
