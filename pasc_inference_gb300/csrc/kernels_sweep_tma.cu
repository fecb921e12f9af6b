// kernels_sweep_tma.cu -- the fused mixed-precision SPG sweep, Blackwell form: four timesteps
// per thread, tiles of gamma and data brought into shared memory by bulk asynchronous copies
// (cp.async.bulk, completion on an mbarrier), double buffered so that the next tile is in
// flight while the current one is computed.
//
// The arithmetic is that of kernels_fused.cu (one sweep = the end of SPG iteration c+1 and the
// start of iteration c+2, gradient recomputed on chip, x the only state in HBM); only the
// mapping differs:
//   - a tile is P = NT*4 consecutive timesteps: 4 halo timesteps on each side (thread 0 and
//     thread NT-1 compute halo only) and W = P - 8 owned timesteps;
//   - one thread issues a bulk copy of the tile's P*K gamma values and P data values (16-byte
//     aligned: tiles start at multiples of 4 timesteps, buffers carry zero pads of 4 timesteps
//     in front and MAXP behind, so every copy is in bounds and needs no edge case);
//   - each thread reads its 4*K values with 16-byte shared loads (conflict-free), keeps them in
//     registers, and exchanges only its first and last timestep with its neighbours;
//   - x^{c+1} goes from registers straight to HBM with 16-byte stores.
// Every wait on an mbarrier is bounded: a wait that gives up sets the error word of the
// device state (the host then reports PASC_ERR_TIMEOUT), the block waits once more, bounded,
// for the copies it has in flight, and leaves its tile loop.
#include "common.cuh"
#include "project.cuh"
#include "internal.h"
#include "sweep_common.cuh"

namespace pasc {

constexpr int TMA_R = 4;          // timesteps per thread
constexpr int TMA_HALO = 4;       // halo timesteps on each side of a tile
constexpr unsigned int TMA_WAIT_LIMIT = 1u << 24;  // try_wait rounds before giving up

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

template <int K, int NT>
struct TmaSmem {
    static constexpr int P = NT * TMA_R;
    alignas(16) float x[2][P * K];   // gamma tile, two stages
    alignas(16) float dat[2][P];     // data tile, two stages
    float yl[NT * K], yr[NT * K];    // x^{c+1} of each thread's first / last timestep
    float dl[NT * K];                // d_{c+2} of each thread's first timestep
    double red[4 * (NT / 32)];
    unsigned long long bar[2];
};

template <int K, int NT, bool INIT>
__global__ void __launch_bounds__(NT) spg_sweep_tma_kernel(SweepArgs a)
{
    constexpr int R = TMA_R;
    constexpr int P = NT * R;
    constexpr int W = P - 2 * TMA_HALO;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TmaSmem<K, NT> &sm = *reinterpret_cast<TmaSmem<K, NT> *>(smem_raw);

    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;  // uniform across the grid

    const int cur = st->cur;
    const float *xin = cur ? a.xb1 : a.xb0;
    float *xout = cur ? a.xb0 : a.xb1;
    const float a0 = (float)st->alpha_prev;
    const float beta = (float)st->beta;
    const float a1 = (float)st->alpha_cur;
    const float coeff = (float)st->coeff;
    const float bscale = (float)st->bscale;
    const int T = (int)a.T;
    const int ntiles = (T + W - 1) / W;
    const int i = threadIdx.x;

    float theta[K];
#pragma unroll
    for (int k = 0; k < K; k++) theta[k] = a.theta[k];

    const unsigned int bytes_x = P * K * sizeof(float), bytes_d = P * sizeof(float);
    if (i == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (i == 0) {
#pragma unroll
        for (int s = 0; s < 2; s++) {
            const int tile = blockIdx.x + s * gridDim.x;
            if (tile < ntiles) {
                const int t0 = tile * W - TMA_HALO;  // >= -4: inside the front pad
                mbar_expect_tx(&sm.bar[s], bytes_x + bytes_d);
                bulk_g2s(sm.x[s], xin + (long)t0 * K, bytes_x, &sm.bar[s]);
                bulk_g2s(sm.dat[s], a.data + t0, bytes_d, &sm.bar[s]);
            }
        }
    }

    KahanF acc_f;
    float acc_dd = 0.f, acc_dAd = 0.f, acc_gd = 0.f;
    unsigned int parity = 0u;  // bit s: phase parity of stage s
    const int li = i > 0 ? i - 1 : i, ri = i < NT - 1 ? i + 1 : i;  // clamped neighbours
    const bool owner = i >= 1 && i <= NT - 2;                        // thread owns its 4 timesteps

    int j = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, j++) {
        const int s = j & 1;
        const bool arrived = mbar_wait(&sm.bar[s], (parity >> s) & 1u);
        if (!__syncthreads_and(arrived)) {
            // a bulk copy did not arrive in time: record it, wait (bounded) once more for the
            // copies this block has in flight, and leave the tile loop
            if (i == 0) atomicExch(&st->error, 1);
            mbar_wait(&sm.bar[s], (parity >> s) & 1u);
            if (tile + (int)gridDim.x < ntiles) mbar_wait(&sm.bar[s ^ 1], (parity >> (s ^ 1)) & 1u);
            break;
        }
        parity ^= 1u << s;
        const int tb = tile * W - TMA_HALO + i * R;  // first timestep of this thread

        // phase A: this thread's 4 timesteps of x^c and data, plus the neighbours' edge values
        float xc[R][K], dv[R], xlft[K], xrgt[K];
        {
            const float4 d4 = *reinterpret_cast<const float4 *>(&sm.dat[s][i * R]);
            dv[0] = d4.x; dv[1] = d4.y; dv[2] = d4.z; dv[3] = d4.w;
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
        float ml[R], mr[R];  // difference-form FEM-H1 row weights (see kernels_fused.cu)
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
                    const float rr = dv[r] - theta[k];
                    const float g = coeff * S - bscale * (rr * rr);
                    z[k] = xc[r][k] - a0 * g;
                }
                project_reg<K>(z);
#pragma unroll
                for (int k = 0; k < K; k++) x1[r][k] = in[r] ? xc[r][k] + beta * (z[k] - xc[r][k]) : 0.f;
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            sm.yl[i * K + k] = x1[0][k];
            sm.yr[i * K + k] = x1[R - 1][k];
        }
        __syncthreads();

        // the stage is free (phase A was its last reader): refill it with the tile after next
        if (i == 0 && tile + 2 * (int)gridDim.x < ntiles) {
            fence_proxy_async_smem();
            const int t0 = (tile + 2 * gridDim.x) * W - TMA_HALO;
            mbar_expect_tx(&sm.bar[s], bytes_x + bytes_d);
            bulk_g2s(sm.x[s], xin + (long)t0 * K, bytes_x, &sm.bar[s]);
            bulk_g2s(sm.dat[s], a.data + t0, bytes_d, &sm.bar[s]);
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
                    const float rr = dv[r] - theta[k];
                    const float bk = bscale * (rr * rr);
                    g1[r][k] = coeff * S - bk;
                    fpart += in[r] ? (g1[r][k] - bk) * x1[r][k] : 0.f;
                    d1[r][k] = x1[r][k] - a1 * g1[r][k];
                }
                project_reg<K>(d1[r]);
#pragma unroll
                for (int k = 0; k < K; k++) d1[r][k] = in[r] ? d1[r][k] - x1[r][k] : 0.f;
            }
            if (owner) acc_f.add(fpart);
        }
#pragma unroll
        for (int k = 0; k < K; k++) sm.dl[i * K + k] = d1[0][k];
        __syncthreads();

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
                    acc_dd += d1[r][k] * d1[r][k];
                    acc_gd += g1[r][k] * d1[r][k];
                    const float nb = r == R - 1 ? dnext[k] : d1[r < R - 1 ? r + 1 : R - 1][k];
                    const float df = pair ? nb - d1[r][k] : 0.f;
                    acc_dAd += df * df;
                }
            }
            if (in[R - 1]) {
                // all four timesteps inside: 16-byte stores (tb is a multiple of 4)
                float4 *dst = reinterpret_cast<float4 *>(xout + (long)tb * K);
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
                        for (int k = 0; k < K; k++) xout[(long)(tb + r) * K + k] = x1[r][k];
            }
        }
    }

    // block and grid reductions
    double v[4] = {acc_f.value(), (double)acc_dd, (double)acc_dAd, (double)acc_gd};
    block_sum<4>(v, sm.red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; q++) a.partials[blockIdx.x * 4 + q] = v[q];
    }
    if (!last_block_done(&st->counter)) return;

    double w[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += NT) {
#pragma unroll
        for (int q = 0; q < 4; q++) w[q] += __ldcg(a.partials + b * 4 + q);
    }
    block_sum<4>(w, sm.red);
    if (threadIdx.x != 0) return;
    spg_finish_sweep<INIT>(st, cur, w);
}

template <int K, int NT, bool INIT>
static cudaError_t launch_tma_t(int grid, const SweepArgs &a, cudaStream_t s)
{
    // the dynamic shared memory limit was raised by tma_blocks_per_sm_t at problem creation
    // (no attribute call here: launches may be inside a stream capture)
    const size_t smem = sizeof(TmaSmem<K, NT>);
    spg_sweep_tma_kernel<K, NT, INIT><<<grid, NT, smem, s>>>(a);
    return cudaGetLastError();
}

template <int K, int NT, bool INIT>
static int tma_blocks_per_sm_t()
{
    const size_t smem = sizeof(TmaSmem<K, NT>);
    cudaFuncSetAttribute(spg_sweep_tma_kernel<K, NT, INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_sweep_tma_kernel<K, NT, INIT>, NT, smem);
    return nb > 0 ? nb : 1;
}

constexpr int TMA_NT = 128;

int sweep_tma_tile_width() { return TMA_NT * TMA_R - 2 * TMA_HALO; }
int sweep_tma_max_tile() { return TMA_NT * TMA_R; }

bool sweep_tma_supported(int K) { return K >= 1 && K <= 8; }

int sweep_tma_blocks_per_sm(int K, bool init)
{
    switch (K) {
#define PASC_CASE(KK) \
    case KK: return init ? tma_blocks_per_sm_t<KK, TMA_NT, true>() : tma_blocks_per_sm_t<KK, TMA_NT, false>();
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 1;
    }
}

cudaError_t launch_sweep_tma(int K, bool init, int grid, const SweepArgs &a, cudaStream_t s)
{
    switch (K) {
#define PASC_CASE(KK)                                                                    \
    case KK:                                                                             \
        return init ? launch_tma_t<KK, TMA_NT, true>(grid, a, s) : launch_tma_t<KK, TMA_NT, false>(grid, a, s);
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pasc
