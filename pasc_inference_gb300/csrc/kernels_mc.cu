// kernels_mc.cu -- multichannel data (X_t in R^n, n = xdim > 1): the residuals
// b_tk = bscale * ||X_t - theta_k||^2 and the theta update theta_k = sum_t gamma_tk X_t /
// sum_t gamma_tk.  The reference's GraphH1FEM uses scalar data (src/petscvector/model/
// graphh1fem.cpp:258-286, 347-380) while sizing theta K*xdim (graphh1fem.cpp:23); these kernels
// are the natural extension: squared Euclidean distances and K-means centroids.
//
// X is held in HBM as BF16 (T x n, row-major, 2 bytes per value): it is the largest array of
// the problem (256 MB at T = 1e6, n = 128) and is read once per outer iteration by each of
// the two kernels.  ||X_t||^2 is computed once, when the data is set.
//
// Residual on the tensor cores (n a multiple of 64, n <= 256): R = X Theta^T with
// tcgen05.mma (kind::f16, BF16 operands, FP32 accumulation in tensor memory), then
// b_tk = bscale * (||X_t||^2 - 2 R_tk + ||theta_k||^2) in the epilogue.  Theta enters as three
// BF16 parts (theta = t1 + t2 + t3 to 24 bits, stacked as 3K rows of the B operand, N = 32),
// so R carries the precision of the FP32 theta rather than of BF16; every product of two BF16
// values is exact in FP32.  One 128-timestep tile per step: TMA brings the tile's n/64 boxes
// of 128 x 64 values (128-byte swizzle) into a 4-stage ring, one thread issues n/16 MMAs
// (M = 128, N = 32, K = 16 each) and commits them to an mbarrier, and the four warps read
// their 32 tensor-memory lanes (one timestep per thread) for the epilogue.
// Other n: the same formula on the CUDA cores in FP32 (mc_residual_simt_kernel), which also
// serves as an independent check of the tensor-core kernel.
//
// Theta update on the CUDA cores in FP32 (products of FP32 gamma and BF16 X, FP32 partial sums
// folded into float-float pairs, common.cuh), per-block float-float partials, then one block per
// cluster sums them in a fixed order and prepares what the residual needs: the BF16 split, the
// FP32 copy and ||theta_k||^2.  No FP64 arithmetic runs in the sums: on this part a dependent
// FP64 add takes 63 cycles, and the folds of every block ran at the same moment.
#include <cuda_bf16.h>
#include <string.h>
#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace pasc {

// ---------------------------------------------------------------------------------------
// data: FP64 -> BF16 (round to nearest even), ||X_t||^2 of the rounded values
// ---------------------------------------------------------------------------------------
// One rounding from FP64 to the nearest value with 8 significant bits (ties to even), then an
// exact conversion of that value (normal BF16 range; zero, infinities and NaN pass through).
__device__ __forceinline__ unsigned short bf16_rn_from_f64(double x)
{
    if (x == 0.0 || !isfinite(x)) return __bfloat16_as_ushort(__double2bfloat16(x));
    int e;
    frexp(x, &e);
    const double r = ldexp(rint(ldexp(x, 8 - e)), e - 8);
    return __bfloat16_as_ushort(__double2bfloat16(r));
}

__global__ void mc_convert_kernel(const double *x64, unsigned short *xbf, long n_total)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n_total; i += (long)gridDim.x * blockDim.x)
        xbf[i] = bf16_rn_from_f64(x64[i]);
}

// one warp per timestep
__global__ void mc_xnorm_kernel(const unsigned short *xbf, float *xnorm, long T, int n)
{
    const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long t = warp; t < T; t += nw) {
        double s = 0.0;
        for (int j = lane; j < n; j += 32) {
            const double v = (double)__bfloat162float(__ushort_as_bfloat16(xbf[t * n + j]));
            s += v * v;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) xnorm[t] = (float)s;
    }
}

cudaError_t launch_mc_convert(const double *x64, unsigned short *xbf, float *xnorm, long T, int n, cudaStream_t s)
{
    const long tot = T * (long)n;
    const int g1 = (int)std::min<long>((tot + 255) / 256, 4096);
    mc_convert_kernel<<<g1, 256, 0, s>>>(x64, xbf, tot);
    const int g2 = (int)std::min<long>((T * 32 + 255) / 256, 4096);
    mc_xnorm_kernel<<<g2, 256, 0, s>>>(xbf, xnorm, T, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// residual on the tensor cores
// ---------------------------------------------------------------------------------------
constexpr int MC_TILE = 128;     // timesteps per tile (MMA M)
constexpr int MC_N = 32;         // MMA N: 3 BF16 parts x K <= 24 rows, padded
constexpr int MC_ATOM_A = MC_TILE * 128;  // bytes of one 64-column box of a tile
constexpr int MC_ATOM_B = MC_N * 128;     // bytes of one 64-column slice of the B operand

template <int NKA>
__host__ __device__ constexpr int mc_stages() { return NKA <= 2 ? 4 : 3; }

template <int NKA>
__host__ __device__ constexpr size_t mc_tc_smem()
{
    return 1024 + (size_t)mc_stages<NKA>() * NKA * MC_ATOM_A + (size_t)NKA * MC_ATOM_B + 64;
}

template <int NKA, int K>
__global__ void __launch_bounds__(128, 1) mc_residual_tc_kernel(const __grid_constant__ CUtensorMap tx, McArgs a)
{
    constexpr int S = mc_stages<NKA>();
    constexpr int STAGE = NKA * MC_ATOM_A;
    constexpr unsigned int IDESC = umma_idesc_bf16_f32<MC_TILE, MC_N>();
    static_assert(3 * K <= MC_N, "three BF16 parts of theta must fit the N of the MMA");
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_addr(smem_raw) & 1023u)) & 1023u);
    unsigned char *sA = base;
    unsigned char *sB = sA + S * STAGE;
    unsigned long long *full = reinterpret_cast<unsigned long long *>(sB + NKA * MC_ATOM_B);
    unsigned long long *mmab = full + S;
    unsigned int *tslot = reinterpret_cast<unsigned int *>(mmab + 1);

    const int tid = threadIdx.x, warp = tid >> 5;
    const long ntiles = (a.T + MC_TILE - 1) / MC_TILE;
    const int n = a.n;

    if (tid == 0) {
        for (int s = 0; s < S; s++) mbar_init(&full[s], 1);
        mbar_init(mmab, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tslot, 32);
        tmem_relinquish();
    }
    // B operand: the 32 x n BF16 rows of the theta split, in the 128-byte swizzle layout
    // (16-byte chunk c of row r of a 64-column slice sits at chunk c ^ (r % 8) of that row)
    {
        const int chunks = n / 8;
        for (int idx = tid; idx < MC_N * chunks; idx += 128) {
            const int r = idx / chunks, c16 = idx - r * chunks;
            const int atom = c16 >> 3, c = c16 & 7;
            const uint4 v = *reinterpret_cast<const uint4 *>(a.theta_split + (long)r * n + c16 * 8);
            *reinterpret_cast<uint4 *>(sB + atom * MC_ATOM_B + (r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4)) = v;
        }
    }
    fence_proxy_async_smem();  // the thread-written B operand is read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned int tmem = *tslot;

    float tn[K];
#pragma unroll
    for (int k = 0; k < K; k++) tn[k] = a.tnorm[k];
    const float bscale = a.bscale;

    auto issue = [&](int s, long tile) {
        mbar_expect_tx(&full[s], STAGE);
#pragma unroll
        for (int ka = 0; ka < NKA; ka++)
            tma_load_2d(sA + s * STAGE + ka * MC_ATOM_A, &tx, ka * 64, (int)(tile * MC_TILE), &full[s]);
    };
    unsigned int inflight = 0u;  // stages with a copy issued and not yet consumed (thread 0)
    if (tid == 0) {
        for (int s = 0; s < S; s++) {
            const long tile = blockIdx.x + (long)s * gridDim.x;
            if (tile < ntiles) {
                issue(s, tile);
                inflight |= 1u << s;
            }
        }
    }

    unsigned int ph_full = 0u, ph_mma = 0u;
    int err = 0;
    int j = 0;
    // ||X_t||^2 of this thread's timestep is loaded one tile ahead, so that its HBM latency
    // overlaps the current tile's MMAs and epilogue
    float xn_next = 0.f;
    {
        const long t = (long)blockIdx.x * MC_TILE + tid;
        if (blockIdx.x < ntiles && t < a.T) xn_next = a.xnorm[t];
    }
    for (long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, j++) {
        const int s = j % S;
        const float xn = xn_next;
        {
            const long t = (tile + gridDim.x) * MC_TILE + tid;
            xn_next = t < a.T ? a.xnorm[t] : 0.f;
        }
        bool ok = true;
        if (tid == 0) {
            ok = mbar_wait(&full[s], (ph_full >> s) & 1u);
            if (ok) {
                inflight &= ~(1u << s);
                tc_fence_after();
                const unsigned int a0 = smem_addr(sA + s * STAGE), b0 = smem_addr(sB);
#pragma unroll
                for (int ks = 0; ks < NKA * 4; ks++) {
                    const unsigned int koff = (unsigned int)(ks & 3) * 32u;  // K-step inside a 128-byte atom
                    const unsigned long long ad = umma_desc_sw128(a0 + (ks >> 2) * MC_ATOM_A + koff);
                    const unsigned long long bd = umma_desc_sw128(b0 + (ks >> 2) * MC_ATOM_B + koff);
                    umma_bf16(tmem, ad, bd, IDESC, ks > 0 ? 1u : 0u);
                }
                umma_commit(mmab);
            }
        }
        ph_full ^= 1u << s;
        if (!__syncthreads_and(ok)) {
            err = 1;
            break;
        }
        const bool mok = mbar_wait(mmab, ph_mma);
        ph_mma ^= 1u;
        if (!__syncthreads_and(mok)) {
            err = 2;
            break;
        }
        tc_fence_after();
        // the MMAs have read stage s: refill it
        if (tid == 0) {
            const long nt = tile + (long)S * gridDim.x;
            if (nt < ntiles) {
                issue(s, nt);
                inflight |= 1u << s;
            }
        }
        float d[32];
        tmem_load_32cols(tmem + ((unsigned int)(32 * warp) << 16), d);
        const long t = tile * MC_TILE + tid;
        if (t < a.T) {
            float out[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float R = (d[2 * K + k] + d[K + k]) + d[k];
                out[k] = bscale * ((xn - 2.f * R) + tn[k]);
            }
            float *dst = a.bmat + t * K;
            if constexpr (K % 4 == 0) {
                // rows of K floats start 16-byte aligned
#pragma unroll
                for (int q = 0; q < K / 4; q++)
                    reinterpret_cast<float4 *>(dst)[q] = make_float4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
            } else {
#pragma unroll
                for (int k = 0; k < K; k++) dst[k] = out[k];
            }
        }
        tc_fence_before();
        __syncthreads();  // tensor memory is rewritten by the next tile's MMAs
    }

    if (err) {
        // a copy or the MMAs did not complete in time: record it, wait (bounded) once more for
        // whatever this block still has in flight, release tensor memory and leave
        if (tid == 0) {
            atomicExch(a.err, err);
            if (err == 2) mbar_wait(mmab, ph_mma);
            for (int s = 0; s < S; s++)
                if (inflight & (1u << s)) mbar_wait(&full[s], (ph_full >> s) & 1u);
        }
        tc_fence_before();
        __syncthreads();
    }
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

int mc_tc_supported(int n) { return n >= 64 && n <= 256 && n % 64 == 0 && n != 192; }

typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

cudaError_t mc_make_tmap(CUtensorMap *map, const unsigned short *xbf, long T, int n)
{
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = (PFN_encodeTiled)p;
    }
    memset(map, 0, sizeof *map);
    const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)T};
    const cuuint64_t strides[1] = {(cuuint64_t)n * 2};
    const cuuint32_t box[2] = {64, (cuuint32_t)MC_TILE};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)xbf, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int NKA, int K>
static cudaError_t launch_tc_t(const CUtensorMap &map, int grid, const McArgs &a, cudaStream_t s)
{
    mc_residual_tc_kernel<NKA, K><<<grid, 128, mc_tc_smem<NKA>(), s>>>(map, a);
    return cudaGetLastError();
}

template <int NKA, int K>
static cudaError_t prepare_tc_t()
{
    return cudaFuncSetAttribute(mc_residual_tc_kernel<NKA, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)mc_tc_smem<NKA>());
}

#define PASC_MC_K_SWITCH(K, NKA, FN, ...)                                         \
    switch (K) {                                                                  \
        case 1: return FN<NKA, 1>(__VA_ARGS__);                                   \
        case 2: return FN<NKA, 2>(__VA_ARGS__);                                   \
        case 3: return FN<NKA, 3>(__VA_ARGS__);                                   \
        case 4: return FN<NKA, 4>(__VA_ARGS__);                                   \
        case 5: return FN<NKA, 5>(__VA_ARGS__);                                   \
        case 6: return FN<NKA, 6>(__VA_ARGS__);                                   \
        case 7: return FN<NKA, 7>(__VA_ARGS__);                                   \
        case 8: return FN<NKA, 8>(__VA_ARGS__);                                   \
        default: return cudaErrorInvalidValue;                                    \
    }

cudaError_t prepare_mc_residual_tc(int K, int n)
{
    switch (n / 64) {
        case 1: PASC_MC_K_SWITCH(K, 1, prepare_tc_t)
        case 2: PASC_MC_K_SWITCH(K, 2, prepare_tc_t)
        case 4: PASC_MC_K_SWITCH(K, 4, prepare_tc_t)
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_mc_residual_tc(const CUtensorMap &map, int K, int n, int grid, const McArgs &a, cudaStream_t s)
{
    switch (n / 64) {
        case 1: PASC_MC_K_SWITCH(K, 1, launch_tc_t, map, grid, a, s)
        case 2: PASC_MC_K_SWITCH(K, 2, launch_tc_t, map, grid, a, s)
        case 4: PASC_MC_K_SWITCH(K, 4, launch_tc_t, map, grid, a, s)
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------------------
// residual on the CUDA cores (any n <= 256): FP32 theta in shared memory, one timestep per
// thread, FP32 dot products
// ---------------------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(256) mc_residual_simt_kernel(McArgs a)
{
    extern __shared__ float s_th[];  // K * n
    const int n = a.n;
    for (int i = threadIdx.x; i < K * n; i += blockDim.x) s_th[i] = a.theta_f32[i];
    __syncthreads();
    float tn[K];
#pragma unroll
    for (int k = 0; k < K; k++) tn[k] = a.tnorm[k];
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < a.T; t += (long)gridDim.x * blockDim.x) {
        float R[K];
#pragma unroll
        for (int k = 0; k < K; k++) R[k] = 0.f;
        const unsigned short *row = a.xbf + t * n;
        for (int j = 0; j < n; j++) {
            const float x = __bfloat162float(__ushort_as_bfloat16(row[j]));
#pragma unroll
            for (int k = 0; k < K; k++) R[k] = fmaf(x, s_th[k * n + j], R[k]);
        }
        const float xn = a.xnorm[t];
#pragma unroll
        for (int k = 0; k < K; k++) a.bmat[t * K + k] = a.bscale * ((xn - 2.f * R[k]) + tn[k]);
    }
}

template <int NKA, int K>
static cudaError_t launch_simt_t(int grid, const McArgs &a, cudaStream_t s)
{
    mc_residual_simt_kernel<K><<<grid, 256, sizeof(float) * K * a.n, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_mc_residual_simt(int K, int grid, const McArgs &a, cudaStream_t s)
{
    PASC_MC_K_SWITCH(K, 0, launch_simt_t, grid, a, s)
}

// ---------------------------------------------------------------------------------------
// theta update
// ---------------------------------------------------------------------------------------
constexpr int MC_THETA_NT = 128;
constexpr int MC_THETA_FOLD = 64;  // timesteps summed in FP32 before folding into a pair

// partials (float-float pairs) [g * (K*n + K) + k*n + j] = sum_t gamma_tk X_tj,
// [.. + K*n + k] = sum_t gamma_tk over block g's timesteps; thread = channel (NJ channels per
// thread, n <= 128 * NJ)
template <int NJ, int K>
__global__ void __launch_bounds__(MC_THETA_NT) mc_theta_partial_kernel(McArgs a, const float *gamma)
{
    const int n = a.n;
    const long per = (a.T + gridDim.x - 1) / gridDim.x;
    const long t0 = blockIdx.x * per, t1 = t0 + per < a.T ? t0 + per : a.T;
    FF acc[NJ][K], den[K];
#pragma unroll
    for (int q = 0; q < NJ; q++)
#pragma unroll
        for (int k = 0; k < K; k++) acc[q][k] = ff_make(0.f);
#pragma unroll
    for (int k = 0; k < K; k++) den[k] = ff_make(0.f);
    for (long tb = t0; tb < t1; tb += MC_THETA_FOLD) {
        const long te = tb + MC_THETA_FOLD < t1 ? tb + MC_THETA_FOLD : t1;
        float f[NJ][K], fd[K];
#pragma unroll
        for (int q = 0; q < NJ; q++)
#pragma unroll
            for (int k = 0; k < K; k++) f[q][k] = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) fd[k] = 0.f;
        for (long t = tb; t < te; t++) {
            float g[K];
#pragma unroll
            for (int k = 0; k < K; k++) {
                g[k] = __ldg(gamma + t * K + k);
                fd[k] += g[k];
            }
#pragma unroll
            for (int q = 0; q < NJ; q++) {
                const int jj = threadIdx.x + q * MC_THETA_NT;
                const float x = jj < n ? __bfloat162float(__ushort_as_bfloat16(a.xbf[t * n + jj])) : 0.f;
#pragma unroll
                for (int k = 0; k < K; k++) f[q][k] = fmaf(g[k], x, f[q][k]);
            }
        }
#pragma unroll
        for (int q = 0; q < NJ; q++)
#pragma unroll
            for (int k = 0; k < K; k++) acc[q][k] = ff_add(acc[q][k], ff_make(f[q][k]));
#pragma unroll
        for (int k = 0; k < K; k++) den[k] = ff_add(den[k], ff_make(fd[k]));
    }
    float2 *P = reinterpret_cast<float2 *>(a.partials) + (long)blockIdx.x * (K * n + K);
#pragma unroll
    for (int q = 0; q < NJ; q++) {
        const int jj = threadIdx.x + q * MC_THETA_NT;
        if (jj < n)
#pragma unroll
            for (int k = 0; k < K; k++) P[k * n + jj] = make_float2(acc[q][k].hi, acc[q][k].lo);
    }
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; k++) P[K * n + k] = make_float2(den[k].hi, den[k].lo);
}

// Vectorised form for n in {8, 16, 32, 64, 128, 256}: a thread owns 8 consecutive channels of a
// row (one 16-byte load of BF16) and holds their K sums in FP32 over its 64 rows; TPR = n/8
// threads share a row and a block of 256 threads covers MC_THETA_ROWS consecutive rows.
// Clusters with gamma_tk == 0 contribute nothing and are skipped (near convergence most
// timesteps sit at a vertex of the simplex, so this removes most of the multiply-adds).
// Block sums: shuffles across the rows of a warp, then warps in a fixed order through shared
// memory in float-float pairs (deterministic); one partial per block in the layout of the
// kernel above.
constexpr int MC_THETA_VNT = 256;
constexpr int MC_THETA_ROWS = 1024;

template <int K, int TPR>
__global__ void __launch_bounds__(MC_THETA_VNT, K >= 7 ? 1 : 2) mc_theta_partial_vec_kernel(McArgs a, const float *gamma)
{
    constexpr int RPB = MC_THETA_VNT / TPR;  // rows per step
    constexpr int NW = MC_THETA_VNT / 32;
    const int n = TPR * 8;
    __shared__ float2 s_sum[TPR * 8 * K + K];
    const int tid = threadIdx.x, c = tid % TPR, r0 = tid / TPR;
    const long t0 = (long)blockIdx.x * MC_THETA_ROWS;
    const long t1 = t0 + MC_THETA_ROWS < a.T ? t0 + MC_THETA_ROWS : a.T;
    float acc[8][K], den[K];
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
        for (int k = 0; k < K; k++) acc[q][k] = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) den[k] = 0.f;
#pragma unroll 2
    for (long t = t0 + r0; t < t1; t += RPB) {
        const uint4 xv = __ldcs(reinterpret_cast<const uint4 *>(a.xbf + t * n) + c);
        float g[K];
#pragma unroll
        for (int k = 0; k < K; k++) g[k] = __ldg(gamma + t * K + k);
        float x[8];
        const unsigned int w[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
            x[2 * q] = __uint_as_float(w[q] << 16);
            x[2 * q + 1] = __uint_as_float(w[q] & 0xFFFF0000u);
        }
#pragma unroll
        for (int k = 0; k < K; k++) {
            den[k] += g[k];
            if (g[k] != 0.f) {
#pragma unroll
                for (int q = 0; q < 8; q++) acc[q][k] = fmaf(g[k], x[q], acc[q][k]);
            }
        }
    }
    // rows of a warp that share channel chunk c: lanes c, c + TPR, ...
#pragma unroll
    for (int off = TPR; off < 32; off <<= 1) {
#pragma unroll
        for (int q = 0; q < 8; q++)
#pragma unroll
            for (int k = 0; k < K; k++) acc[q][k] += __shfl_xor_sync(0xffffffffu, acc[q][k], off);
#pragma unroll
        for (int k = 0; k < K; k++) den[k] += __shfl_xor_sync(0xffffffffu, den[k], off);
    }
    const int lane = tid & 31, warp = tid >> 5;
    for (int w = 0; w < NW; w++) {
        if (warp == w && lane < TPR) {
#pragma unroll
            for (int q = 0; q < 8; q++)
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float2 &dst = s_sum[k * n + c * 8 + q];
                    const FF r = ff_add(w == 0 ? ff_make(0.f) : FF{dst.x, dst.y}, ff_make(acc[q][k]));
                    dst = make_float2(r.hi, r.lo);
                }
            if (c == 0)
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float2 &dst = s_sum[K * n + k];
                    const FF r = ff_add(w == 0 ? ff_make(0.f) : FF{dst.x, dst.y}, ff_make(den[k]));
                    dst = make_float2(r.hi, r.lo);
                }
        }
        __syncthreads();
    }
    float2 *P = reinterpret_cast<float2 *>(a.partials) + (long)blockIdx.x * (K * n + K);
    for (int i = tid; i < K * n + K; i += MC_THETA_VNT) P[i] = s_sum[i];
}

// Bulk-copy form (n in {8, ..., 256} as above): a block takes chunks of MC_TC_ROWS consecutive
// rows; one thread copies each chunk's X rows (n BF16 per row, contiguous) and gamma rows
// (K FP32 per row, contiguous; the gamma buffer's zero pads make every copy whole) into a
// 3-stage shared-memory ring with cp.async.bulk, so the loads in flight live in shared
// memory rather than registers.  A thread owns 4 channels of one row per step (8-byte shared
// loads, conflict-free across a row) and sums in FP32 in two levels (per chunk, then over its
// chunks); rows beyond T carry gamma = 0 from the pad and are skipped like any zero weight.
// Every wait on a copy is bounded: a timeout sets the error word, the block waits once more
// for its copies in flight and leaves without writing its partial.
constexpr int MC_TC_ROWS = 64;
constexpr int MC_TC_STAGES = 3;

template <int K, int TPR>
__host__ __device__ constexpr size_t mc_theta_tma_smem()
{
    return (size_t)MC_TC_STAGES * (MC_TC_ROWS * TPR * 4 * 2 + MC_TC_ROWS * K * 4) + (size_t)(TPR * 4 * K + K) * 8 +
           MC_TC_STAGES * 8 + 128;  // the block sums: TPR*4*K + K float-float pairs
}

template <int K, int TPR>
__global__ void __launch_bounds__(MC_THETA_VNT) mc_theta_tma_kernel(McArgs a, const float *gamma)
{
    constexpr int n = TPR * 4;                 // channels
    constexpr int RPS = MC_THETA_VNT / TPR;    // rows per step
    constexpr int NW = MC_THETA_VNT / 32;
    constexpr int XB = MC_TC_ROWS * n * 2;     // bytes of a chunk's X rows
    constexpr int GB = MC_TC_ROWS * K * 4;     // bytes of a chunk's gamma rows
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *xs = smem_raw;
    float *gs = reinterpret_cast<float *>(smem_raw + MC_TC_STAGES * XB);
    float2 *s_sum = reinterpret_cast<float2 *>(smem_raw + MC_TC_STAGES * (XB + GB));
    unsigned long long *bar = reinterpret_cast<unsigned long long *>(s_sum + n * K + K);

    const int tid = threadIdx.x, c = tid % TPR, r0 = tid / TPR;
    const long nchunks = (a.T + MC_TC_ROWS - 1) / MC_TC_ROWS;
    if (tid == 0) {
        for (int s = 0; s < MC_TC_STAGES; s++) mbar_init(&bar[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    auto issue = [&](int s, long chunk) {
        const long t0 = chunk * MC_TC_ROWS;
        const long rows = a.T - t0 < MC_TC_ROWS ? a.T - t0 : MC_TC_ROWS;
        const unsigned int xbytes = (unsigned int)(rows * n * 2);
        mbar_expect_tx(&bar[s], xbytes + GB);
        bulk_g2s(xs + s * XB, a.xbf + t0 * n, xbytes, &bar[s]);
        bulk_g2s(gs + s * (GB / 4), gamma + t0 * K, GB, &bar[s]);
    };
    unsigned int inflight = 0u;
    if (tid == 0) {
        for (int s = 0; s < MC_TC_STAGES; s++) {
            const long ch = blockIdx.x + (long)s * gridDim.x;
            if (ch < nchunks) {
                issue(s, ch);
                inflight |= 1u << s;
            }
        }
    }
    float tot[4][K], dtot[K];
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
        for (int k = 0; k < K; k++) tot[q][k] = 0.f;
#pragma unroll
    for (int k = 0; k < K; k++) dtot[k] = 0.f;
    for (int i = tid; i < n * K + K; i += MC_THETA_VNT) s_sum[i] = make_float2(0.f, 0.f);  // a row may span warps
    unsigned int parity = 0u;
    bool failed = false;
    int j = 0;
    for (long ch = blockIdx.x; ch < nchunks; ch += gridDim.x, j++) {
        const int s = j % MC_TC_STAGES;
        const bool ok = mbar_wait(&bar[s], (parity >> s) & 1u);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        parity ^= 1u << s;
        if (tid == 0) inflight &= ~(1u << s);
        const unsigned char *xc = xs + s * XB;
        const float *gc = gs + s * (GB / 4);
        float acc[4][K], den[K];
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int k = 0; k < K; k++) acc[q][k] = 0.f;
#pragma unroll
        for (int k = 0; k < K; k++) den[k] = 0.f;
#pragma unroll 4
        for (int r = r0; r < MC_TC_ROWS; r += RPS) {
            const uint2 xv = *reinterpret_cast<const uint2 *>(xc + (r * n + c * 4) * 2);
            const float x[4] = {__uint_as_float(xv.x << 16), __uint_as_float(xv.x & 0xFFFF0000u),
                                __uint_as_float(xv.y << 16), __uint_as_float(xv.y & 0xFFFF0000u)};
            float gr[K];  // the row's weights: 16-byte shared loads where the row is 16-byte aligned
            if constexpr (K % 4 == 0) {
#pragma unroll
                for (int k4 = 0; k4 < K / 4; k4++) {
                    const float4 v = reinterpret_cast<const float4 *>(gc + r * K)[k4];
                    gr[4 * k4] = v.x; gr[4 * k4 + 1] = v.y; gr[4 * k4 + 2] = v.z; gr[4 * k4 + 3] = v.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < K; k++) gr[k] = gc[r * K + k];
            }
#pragma unroll
            for (int k = 0; k < K; k++) {
                const float g = gr[k];
                den[k] += g;
                if (g != 0.f) {
#pragma unroll
                    for (int q = 0; q < 4; q++) acc[q][k] = fmaf(g, x[q], acc[q][k]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int k = 0; k < K; k++) tot[q][k] += acc[q][k];
#pragma unroll
        for (int k = 0; k < K; k++) dtot[k] += den[k];
        __syncthreads();  // every thread is done with stage s
        if (tid == 0) {
            const long nx = ch + (long)MC_TC_STAGES * gridDim.x;
            if (nx < nchunks) {
                fence_proxy_async_smem();
                issue(s, nx);
                inflight |= 1u << s;
            }
        }
    }
    if (failed) {
        if (tid == 0) {
            atomicExch(a.err, 3);
            for (int s = 0; s < MC_TC_STAGES; s++)
                if (inflight & (1u << s)) mbar_wait(&bar[s], (parity >> s) & 1u);
        }
        return;
    }
    // rows of a warp that share channel chunk c, then warps in a fixed order (float-float)
#pragma unroll
    for (int off = TPR; off < 32; off <<= 1) {
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int k = 0; k < K; k++) tot[q][k] += __shfl_xor_sync(0xffffffffu, tot[q][k], off);
#pragma unroll
        for (int k = 0; k < K; k++) dtot[k] += __shfl_xor_sync(0xffffffffu, dtot[k], off);
    }
    const int lane = tid & 31, warp = tid >> 5;
    for (int w = 0; w < NW; w++) {
        if (warp == w && lane < TPR) {
#pragma unroll
            for (int q = 0; q < 4; q++)
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float2 &dst = s_sum[k * n + c * 4 + q];
                    const FF r = ff_add(FF{dst.x, dst.y}, ff_make(tot[q][k]));
                    dst = make_float2(r.hi, r.lo);
                }
            if (c == 0)
#pragma unroll
                for (int k = 0; k < K; k++) {
                    float2 &dst = s_sum[K * n + k];
                    const FF r = ff_add(FF{dst.x, dst.y}, ff_make(dtot[k]));
                    dst = make_float2(r.hi, r.lo);
                }
        }
        __syncthreads();
    }
    float2 *P = reinterpret_cast<float2 *>(a.partials) + (long)blockIdx.x * (K * n + K);
    for (int i = tid; i < K * n + K; i += MC_THETA_VNT) P[i] = s_sum[i];
}

#define PASC_MC_TPR_SWITCH_R(r, n, FN, ...)                      \
    switch ((n) / 4) {                                           \
        case 2: r = FN<2>(__VA_ARGS__); break;                   \
        case 4: r = FN<4>(__VA_ARGS__); break;                   \
        case 8: r = FN<8>(__VA_ARGS__); break;                   \
        case 16: r = FN<16>(__VA_ARGS__); break;                 \
        case 32: r = FN<32>(__VA_ARGS__); break;                 \
        case 64: r = FN<64>(__VA_ARGS__); break;                 \
        default: r = -1; break;                                  \
    }

#define PASC_MC_TPR_SWITCH(n, FN, ...)                           \
    switch ((n) / 4) {                                           \
        case 2: return FN<2>(__VA_ARGS__);                       \
        case 4: return FN<4>(__VA_ARGS__);                       \
        case 8: return FN<8>(__VA_ARGS__);                       \
        case 16: return FN<16>(__VA_ARGS__);                     \
        case 32: return FN<32>(__VA_ARGS__);                     \
        case 64: return FN<64>(__VA_ARGS__);                     \
        default: return -1;                                      \
    }

template <int K>
struct ThetaTma {
    template <int TPR>
    static int blocks()
    {
        const size_t smem = mc_theta_tma_smem<K, TPR>();
        if (cudaFuncSetAttribute(mc_theta_tma_kernel<K, TPR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return -1;
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, mc_theta_tma_kernel<K, TPR>, MC_THETA_VNT, smem);
        return nb;
    }
    template <int TPR>
    static int launch(int grid, const McArgs &a, const float *gamma, cudaStream_t s)
    {
        mc_theta_tma_kernel<K, TPR><<<grid, MC_THETA_VNT, mc_theta_tma_smem<K, TPR>(), s>>>(a, gamma);
        return 0;
    }
};

// blocks per SM of the bulk-copy theta kernel (sets its shared-memory limit); 0: not available
int mc_theta_tma_blocks_per_sm(int K, int n)
{
    int r = -1;
    switch (K) {
#define PASC_CASE(KK) \
    case KK: r = [&]() -> int { PASC_MC_TPR_SWITCH(n, ThetaTma<KK>::template blocks) }(); break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: break;
    }
    return r > 0 ? r : 0;
}

int mc_theta_vec_supported(int n) { return n == 8 || n == 16 || n == 32 || n == 64 || n == 128 || n == 256; }
int mc_theta_vec_grid(long T) { return (int)((T + MC_THETA_ROWS - 1) / MC_THETA_ROWS); }

// One block per cluster k: blockDim = nb * S, nb = n rounded up to a multiple of 32, S slices.
// from_partials: theta_k from the float-float partial sums of `nparts` blocks -- slice s sums
// the parts s, s + S, ... in order, then the S slice sums are added in slice order (fixed
// order, deterministic; S dependent chains of nparts/S additions instead of one of nparts),
// and one FP64 division per channel; otherwise theta64 as given (S = 1).  Then, in slice 0: the
// FP32 copy, the three BF16 parts (rows k, K + k, 2K + k of theta_split) and ||theta_k||^2.
constexpr int MC_PREP_MAX_THREADS = 1024;
constexpr int MC_PREP_BATCH = 8;

template <int K>
__global__ void __launch_bounds__(MC_PREP_MAX_THREADS) mc_theta_prepare_kernel(McArgs a, int nparts, int from_partials)
{
    __shared__ double s_red[32];
    __shared__ float2 s_part[MC_PREP_MAX_THREADS + 8];
    const int k = blockIdx.x, n = a.n, nb = (n + 31) / 32 * 32;
    const int j = threadIdx.x % nb, sl = threadIdx.x / nb, S = blockDim.x / nb;
    double th = 0.0;
    if (from_partials) {
        const float2 *P = reinterpret_cast<const float2 *>(a.partials);
        FF num = ff_make(0.f), den = ff_make(0.f);
        // the loads of MC_PREP_BATCH parts are issued before their additions (the additions stay
        // in part order): one memory latency per batch instead of one per part
        for (int g0 = sl; g0 < nparts; g0 += MC_PREP_BATCH * S) {
            float2 pn[MC_PREP_BATCH], pd[MC_PREP_BATCH];
#pragma unroll
            for (int u = 0; u < MC_PREP_BATCH; u++) {
                const int g = g0 + u * S;
                const float2 *Pg = P + (long)g * (K * n + K);
                pn[u] = (g < nparts && j < n) ? Pg[k * n + j] : make_float2(0.f, 0.f);
                pd[u] = (g < nparts && j == 0) ? Pg[K * n + k] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < MC_PREP_BATCH; u++) {
                if (g0 + u * S >= nparts) break;
                if (j < n) num = ff_add(num, FF{pn[u].x, pn[u].y});
                if (j == 0) den = ff_add(den, FF{pd[u].x, pd[u].y});
            }
        }
        s_part[threadIdx.x] = make_float2(num.hi, num.lo);
        if (j == 0) s_part[MC_PREP_MAX_THREADS + (sl & 7)] = make_float2(den.hi, den.lo);
        __syncthreads();
        if (sl == 0) {
            num = ff_make(0.f);
            den = ff_make(0.f);
            for (int q = 0; q < S; q++) {
                num = ff_add(num, FF{s_part[q * nb + j].x, s_part[q * nb + j].y});
                den = ff_add(den, FF{s_part[MC_PREP_MAX_THREADS + q].x, s_part[MC_PREP_MAX_THREADS + q].y});
            }
            const double dd = ff_value(den);
            th = (j < n && dd != 0.0) ? ff_value(num) / dd : 0.0;
            if (j < n) a.theta64[k * n + j] = th;
        }
    } else if (j < n && sl == 0) {
        th = a.theta64[k * n + j];
    }
    if (sl == 0 && j < n) {
        a.theta_f32[k * n + j] = (float)th;
        const __nv_bfloat16 p1 = __double2bfloat16(th);
        const double r1 = th - (double)__bfloat162float(p1);
        const __nv_bfloat16 p2 = __double2bfloat16(r1);
        const double r2 = r1 - (double)__bfloat162float(p2);
        const __nv_bfloat16 p3 = __double2bfloat16(r2);
        a.theta_split[(long)k * n + j] = __bfloat16_as_ushort(p1);
        a.theta_split[(long)(K + k) * n + j] = __bfloat16_as_ushort(p2);
        a.theta_split[(long)(2 * K + k) * n + j] = __bfloat16_as_ushort(p3);
    }
    double v = th * th;  // 0 outside slice 0
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (sl == 0 && (j & 31) == 0) s_red[j >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < nb / 32; w++) s += s_red[w];
        a.tnorm[k] = (float)s;
    }
}

template <int NKA, int K>
static cudaError_t launch_theta_t(int grid, const McArgs &a, const float *gamma, cudaStream_t s)
{
    const int nb = ((a.n + 31) / 32) * 32;
    const int np = nb * std::min(8, std::max(1, MC_PREP_MAX_THREADS / nb));  // prepare: up to 8 slices
    if (gamma && a.theta_tma_grid > 0) {
        int r = -1;
        PASC_MC_TPR_SWITCH_R(r, a.n, ThetaTma<K>::template launch, a.theta_tma_grid, a, gamma, s)
        if (r < 0) return cudaErrorInvalidValue;
        mc_theta_prepare_kernel<K><<<K, np, 0, s>>>(a, a.theta_tma_grid, 1);
    } else if (gamma && mc_theta_vec_supported(a.n)) {
        const int g = mc_theta_vec_grid(a.T);
        switch (a.n / 8) {
            case 1: mc_theta_partial_vec_kernel<K, 1><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            case 2: mc_theta_partial_vec_kernel<K, 2><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            case 4: mc_theta_partial_vec_kernel<K, 4><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            case 8: mc_theta_partial_vec_kernel<K, 8><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            case 16: mc_theta_partial_vec_kernel<K, 16><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            case 32: mc_theta_partial_vec_kernel<K, 32><<<g, MC_THETA_VNT, 0, s>>>(a, gamma); break;
            default: return cudaErrorInvalidValue;
        }
        mc_theta_prepare_kernel<K><<<K, np, 0, s>>>(a, g, 1);
    } else if (gamma) {
        if (a.n <= 128) mc_theta_partial_kernel<1, K><<<grid, MC_THETA_NT, 0, s>>>(a, gamma);
        else mc_theta_partial_kernel<2, K><<<grid, MC_THETA_NT, 0, s>>>(a, gamma);
        mc_theta_prepare_kernel<K><<<K, np, 0, s>>>(a, grid, 1);
    } else {
        mc_theta_prepare_kernel<K><<<K, nb, 0, s>>>(a, 0, 0);
    }
    return cudaGetLastError();
}

cudaError_t launch_mc_theta(int K, int grid, const McArgs &a, const float *gamma, cudaStream_t s)
{
    if (a.n > 256) return cudaErrorInvalidValue;
    PASC_MC_K_SWITCH(K, 0, launch_theta_t, grid, a, gamma, s)
}

size_t mc_partials_size(int K, int n, int grid, long T)
{
    const long g = mc_theta_vec_supported(n) && mc_theta_vec_grid(T) > grid ? mc_theta_vec_grid(T) : grid;
    return (size_t)g * (K * n + K);  // the bulk-copy kernel runs at most `grid` blocks
}

}  // namespace pasc
