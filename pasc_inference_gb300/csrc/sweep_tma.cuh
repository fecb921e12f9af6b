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
// (P*K values, materialised for multichannel data) instead of its data values.
template <int KB, int NT, bool BM = false>
struct TmaSmem {
    static constexpr int P = NT * TMA_R;
    alignas(16) float x[2][P * KB];  // gamma tile, two stages (stride K for K <= KB)
    alignas(16) float dat[2][BM ? P * KB : P];  // data tile (BM: b tile), two stages
    float yl[NT * KB], yr[NT * KB];  // x^{c+1} of each thread's first / last timestep
    float dl[NT * KB];               // d_{c+2} of each thread's first timestep
    double red[4 * (NT / 32)];
    unsigned long long bar[2];
    int job;                          // batched kernel: the work item this block took
};

// Scalars of one signal's sweep.
template <int K>
struct TileScalars {
    float a0, beta, a1, coeff, bscale;
    float theta[K];
    int T;
    const float *xin;
    float *xout;
    const float *data;  // BM: the materialised b (T*K, zero pads like gamma)
};

struct TileAcc {
    KahanF f;
    float dd = 0.f, dAd = 0.f, gd = 0.f;
};

// Thread 0: bring the tile starting at timestep t0 into stage s.
template <int K, int KB, int NT, bool BM>
__device__ __forceinline__ void tma_issue(TmaSmem<KB, NT, BM> &sm, int s, const float *xin, const float *data, int t0)
{
    constexpr int P = NT * TMA_R;
    const unsigned int bytes_x = P * K * sizeof(float), bytes_d = (BM ? P * K : P) * sizeof(float);
    mbar_expect_tx(&sm.bar[s], bytes_x + bytes_d);
    bulk_g2s(sm.x[s], xin + (long)t0 * K, bytes_x, &sm.bar[s]);
    bulk_g2s(sm.dat[s], data + (long)t0 * (BM ? K : 1), bytes_d, &sm.bar[s]);
}

// One tile whose stage s has arrived: phases A-D of the sweep.  After the stage's last read
// (phase B; phase C when b comes from the stage) thread 0 refills stage s with the tile at
// refill_t0 unless it is TMA_NO_REFILL.  Contains three __syncthreads(); all threads of the
// block must call it.
template <int K, int KB, int NT, bool INIT, bool BM = false>
__device__ __forceinline__ void tma_tile(TmaSmem<KB, NT, BM> &sm, int s, int t0, const TileScalars<K> &sc,
                                         TileAcc &acc, int refill_t0)
{
    constexpr int R = TMA_R;
    const int i = threadIdx.x;
    const int li = i > 0 ? i - 1 : i, ri = i < NT - 1 ? i + 1 : i;  // clamped neighbours
    const bool owner = i >= 1 && i <= NT - 2;                        // owns its 4 timesteps
    const int T = sc.T;
    const int tb = t0 + i * R;  // first timestep of this thread

    // phase A: this thread's 4 timesteps of x^c and data, plus the neighbours' edge values
    float xc[R][K], dv[R], xlft[K], xrgt[K];
    const float *bt = &sm.dat[s][i * R * K];  // BM: this thread's R*K values of b
    if (!BM) {
        const float4 d4 = *reinterpret_cast<const float4 *>(&sm.dat[s][i * R]);
        dv[0] = d4.x; dv[1] = d4.y; dv[2] = d4.z; dv[3] = d4.w;
    }
    {
        const float4 *src = reinterpret_cast<const float4 *>(&sm.x[s][i * R * K]);
#pragma unroll
        for (int q = 0; q < K; q++) {
            const float4 v = src[q];
            const int e = 4 * q;
            xc[(e + 0) / K][(e + 0) % K] = v.x;
            xc[(e + 1) / K][(e + 1) % K] = v.y;
            xc[(e + 2) / K][(e + 2) % K] = v.z;
            xc[(e + 3) / K][(e + 3) % K] = v.w;
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            xlft[k] = sm.x[s][(li * R + R - 1) * K + k];
            xrgt[k] = sm.x[s][(ri * R) * K + k];
        }
    }
    bool in[R];
    float ml[R], mr[R];  // FEM-H1 row in difference form: 2[t>0](x_t-x_{t-1}) + 2[t<T-1](x_t-x_{t+1})
#pragma unroll
    for (int r = 0; r < R; r++) {
        const int t = tb + r;
        in[r] = (unsigned)t < (unsigned)T;
        ml[r] = t > 0 ? 2.f : 0.f;
        mr[r] = t < T - 1 ? 2.f : 0.f;
    }
    if (INIT) {
        // the start point is projected; its neighbours are projected the same way
#pragma unroll
        for (int r = 0; r < R; r++) project_reg<K>(xc[r]);
        project_reg<K>(xlft);
        project_reg<K>(xrgt);
    }
    // zero outside the signal (the pads hold zeros; projection of a zero block does not)
#pragma unroll
    for (int r = 0; r < R; r++)
#pragma unroll
        for (int k = 0; k < K; k++) xc[r][k] = in[r] ? xc[r][k] : 0.f;
    {
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
        for (int r = 0; r < R; r++) {
            float z[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float left = r == 0 ? xlft[k] : xc[r > 0 ? r - 1 : 0][k];
                const float right = r == R - 1 ? xrgt[k] : xc[r < R - 1 ? r + 1 : R - 1][k];
                const float S = ml[r] * (xc[r][k] - left) + mr[r] * (xc[r][k] - right);
                float bk;
                if (BM) {
                    bk = bt[r * K + k];
                } else {
                    const float rr = dv[r] - sc.theta[k];
                    bk = sc.bscale * (rr * rr);
                }
                const float g = sc.coeff * S - bk;
                z[k] = xc[r][k] - sc.a0 * g;
            }
            project_reg<K>(z);
#pragma unroll
            for (int k = 0; k < K; k++) x1[r][k] = in[r] ? xc[r][k] + sc.beta * (z[k] - xc[r][k]) : 0.f;
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        sm.yl[i * K + k] = x1[0][k];
        sm.yr[i * K + k] = x1[R - 1][k];
    }
    __syncthreads();

    // the stage is free (phase A was its last reader): refill it
    if (!BM && i == 0 && refill_t0 != TMA_NO_REFILL) {
        fence_proxy_async_smem();
        tma_issue<K>(sm, s, sc.xin, sc.data, refill_t0);
    }

    // phase C: g^{c+1}, objective, d_{c+2}
    float g1[R][K], d1[R][K];
    {
        float yl[K], yr[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            yl[k] = sm.yr[li * K + k];
            yr[k] = sm.yl[ri * K + k];
        }
        float fpart = 0.f;
#pragma unroll
        for (int r = 0; r < R; r++) {
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float left = r == 0 ? yl[k] : x1[r > 0 ? r - 1 : 0][k];
                const float right = r == R - 1 ? yr[k] : x1[r < R - 1 ? r + 1 : R - 1][k];
                const float S = ml[r] * (x1[r][k] - left) + mr[r] * (x1[r][k] - right);
                float bk;
                if (BM) {
                    bk = bt[r * K + k];
                } else {
                    const float rr = dv[r] - sc.theta[k];
                    bk = sc.bscale * (rr * rr);
                }
                g1[r][k] = sc.coeff * S - bk;
                fpart += in[r] ? (g1[r][k] - bk) * x1[r][k] : 0.f;
                d1[r][k] = x1[r][k] - sc.a1 * g1[r][k];
            }
            project_reg<K>(d1[r]);
#pragma unroll
            for (int k = 0; k < K; k++) d1[r][k] = in[r] ? d1[r][k] - x1[r][k] : 0.f;
        }
        if (owner) acc.f.add(fpart);
    }
#pragma unroll
    for (int k = 0; k < K; k++) sm.dl[i * K + k] = d1[0][k];
    __syncthreads();
    // BM: phase C was the stage's last reader
    if (BM && i == 0 && refill_t0 != TMA_NO_REFILL) {
        fence_proxy_async_smem();
        tma_issue<K>(sm, s, sc.xin, sc.data, refill_t0);
    }

    // phase D: dots of d_{c+2} and the store of x^{c+1}
    if (owner) {
        float dnext[K];
#pragma unroll
        for (int k = 0; k < K; k++) dnext[k] = sm.dl[ri * K + k];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const bool pair = in[r] && (tb + r) < T - 1;
#pragma unroll
            for (int k = 0; k < K; k++) {
                acc.dd += d1[r][k] * d1[r][k];
                acc.gd += g1[r][k] * d1[r][k];
                const float nb = r == R - 1 ? dnext[k] : d1[r < R - 1 ? r + 1 : R - 1][k];
                const float df = pair ? nb - d1[r][k] : 0.f;
                acc.dAd += df * df;
            }
        }
        if (in[R - 1]) {
            // all four timesteps inside: 16-byte stores (tb is a multiple of 4)
            float4 *dst = reinterpret_cast<float4 *>(sc.xout + (long)tb * K);
#pragma unroll
            for (int q = 0; q < K; q++) {
                const int e = 4 * q;
                dst[q] = make_float4(x1[(e + 0) / K][(e + 0) % K], x1[(e + 1) / K][(e + 1) % K],
                                     x1[(e + 2) / K][(e + 2) % K], x1[(e + 3) / K][(e + 3) % K]);
            }
        } else {
#pragma unroll
            for (int r = 0; r < R; r++)
                if (in[r])
#pragma unroll
                    for (int k = 0; k < K; k++) sc.xout[(long)(tb + r) * K + k] = x1[r][k];
        }
    }
    // the neighbour arrays are rewritten by the next tile's phase B only after its own
    // __syncthreads-separated phase A, so no barrier is needed here
}

}  // namespace pasc
