// kernels_sweep_tma.cu -- the fused mixed-precision SPG sweep for one signal, Blackwell form:
// four timesteps per thread, tiles of gamma and data brought into shared memory by bulk
// asynchronous copies (cp.async.bulk, completion on an mbarrier), double buffered so that
// the next tile is in flight while the current one is computed (sweep_tma.cuh).
//
// The arithmetic is that of kernels_fused.cu (one sweep = the end of SPG iteration c+1 and the
// start of iteration c+2, gradient recomputed on chip, x the only state in HBM); only the
// mapping differs:
//   - a tile is P = NT*4 consecutive timesteps: 4 halo timesteps on each side (thread 0 and
//     thread NT-1 compute halo only) and W = P - 8 owned timesteps;
//   - one thread issues a bulk copy of the tile's P*K gamma values and P data values (16-byte
//     aligned: tiles start at multiples of 4 timesteps, buffers carry zero pads of 4 timesteps
//     in front and at least P behind, so every copy is in bounds and needs no edge case);
//   - each thread reads its 4*K values with 16-byte shared loads (conflict-free), keeps them in
//     registers, and exchanges only its first and last timestep with its neighbours;
//   - x^{c+1} goes from registers straight to HBM with 16-byte stores.
// MODE 0: b formed from data and theta; 1: b read from a materialised T*K array (multichannel
// data, reduced FEM problems); 2: as 0 with theta in the penalty (block k of A weighted by
// theta_k^2, GraphH1FEMModel with usethetainpenalty, blockgraphsparse.cpp:161-185).
// Every wait on an mbarrier is bounded: a wait that gives up sets the error word of the
// device state (the host then reports PASC_ERR_TIMEOUT), the block waits once more, bounded,
// for the copies it has in flight, and leaves its tile loop.
#include <string.h>

#include "sweep_tma.cuh"
#include "sweep_common.cuh"

namespace pasc {

// Timesteps per thread and threads per block of the tile: 4 x 128, or for K >= 6 (whose
// per-thread arrays of 4 timesteps need ~165 registers, 3 blocks per SM) 2 x 256; the tile is
// 512 timesteps either way.
// MinBlocks: resident blocks per SM the registers are held to (0: the compiler's choice).  At
// K <= 3 the compiler's own choice was 72 registers with a 16-byte local-memory spill (7
// blocks per SM); held to 8 blocks it fits 64 registers without one.
template <int K>
struct TmaShape {
    static constexpr int R = K >= 6 ? 2 : 4;
    static constexpr int NT = 512 / R;
    static constexpr int MinBlocks = K <= 3 ? 8 : (K == 4 ? 6 : (K == 5 ? 5 : 0));
};

// SWZ (R*K == 16 only): tiles by tensor copies with the 64-byte swizzle (sweep_tma.cuh); the
// stages then start at a 512-byte aligned shared address (512 bytes more dynamic memory).
template <int K, int NT, bool INIT, int MODE, bool SWZ = false>
__global__ void __launch_bounds__(NT, TmaShape<K>::MinBlocks) spg_sweep_tma_kernel(const __grid_constant__ SweepArgs a)
{
    constexpr bool BM = MODE == 1, TP = MODE == 2;
    constexpr int R = TmaShape<K>::R;
    constexpr int P = NT * R;
    constexpr int W = P - 2 * TMA_HALO;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *smem_base = SWZ ? smem_raw + ((512u - (smem_addr(smem_raw) & 511u)) & 511u) : smem_raw;
    TmaSmem<K, NT, BM, R> &sm = *reinterpret_cast<TmaSmem<K, NT, BM, R> *>(smem_base);

    SpgDevState *st = a.st;
    if (st->status != PASC_SPG_RUNNING) return;  // uniform across the grid

    const int cur = st->cur;
    TileScalars<K> sc;
    sc.xin = cur ? a.xb1 : a.xb0;
    sc.xout = cur ? a.xb0 : a.xb1;
    sc.data = BM ? a.bmat : a.data;
    sc.tmx = &a.tm_x[cur];
    sc.tmb = &a.tm_b;
    sc.roff = a.roff;
    sc.a0 = (float)st->alpha_prev;
    sc.beta = (float)st->beta;
    sc.a1 = (float)st->alpha_cur;
    sc.coeff = (float)st->coeff;
    sc.bscale = (float)st->bscale;
    sc.T = (int)a.T;
#pragma unroll
    for (int k = 0; k < K; k++) {
        sc.theta[k] = a.theta[k];
        sc.kw[k] = TP ? a.kw[k] : 1.f;
    }
    const int ntiles = (sc.T + W - 1) / W;
    const int i = threadIdx.x;

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
            if (tile < ntiles) {  // t0 >= -4: the front pad
                if constexpr (SWZ) tma_issue_swz<K>(sm, s, sc, tile * W - TMA_HALO);
                else tma_issue<K>(sm, s, sc.xin, sc.data, tile * W - TMA_HALO);
            }
        }
    }

    TileAcc acc;
    TilePending<K> pend;
    pend.valid = false;
    unsigned int parity = 0u;  // bit s: phase parity of stage s
    int j = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, j++) {
        const int s = j & 1;
        const bool arrived = mbar_wait(&sm.bar[s], (parity >> s) & 1u);
        const int next2 = tile + 2 * (int)gridDim.x;
        if (!tma_tile<K, K, NT, INIT, BM, TP, R, SWZ>(sm, s, j, arrived, tile * W - TMA_HALO, sc, acc, pend,
                                                 next2 < ntiles ? next2 * W - TMA_HALO : TMA_NO_REFILL)) {
            // a bulk copy did not arrive in time (the tile's barrier voted on it, before any
            // further copy was issued): record it, wait (bounded) once more for the copies this
            // block has in flight, and leave the tile loop
            if (i == 0) atomicExch(&st->error, 1);
            mbar_wait(&sm.bar[s], (parity >> s) & 1u);
            if (tile + (int)gridDim.x < ntiles) mbar_wait(&sm.bar[s ^ 1], (parity >> (s ^ 1)) & 1u);
            pend.valid = false;
            break;
        }
        parity ^= 1u << s;
    }
    __syncthreads();
    tma_flush_pending<K, K, NT, BM, TP, R>(sm, sc, acc, pend);  // the last tile's pair terms

    // block and grid reductions (float-float; the step logic in FP64)
    // the last block snapshots the state into the first stage (free: every copy was consumed)
    // for the step logic
    static_assert(sizeof(SpgDevState) <= sizeof(sm.x[0]) && sizeof(SpgDevState) % 8 == 0, "state snapshot");
    SpgDevState *snap = reinterpret_cast<SpgDevState *>(sm.x[0]);
    double w[4];
    if (!sweep_grid_sum4<4>(acc.f, acc.dd, acc.dAd, acc.gd, reinterpret_cast<float2 *>(a.partials), blockIdx.x,
                            &st->counter, gridDim.x, 0, 1, reinterpret_cast<float2 *>(sm.red), w, st, snap,
                            (int)sizeof(SpgDevState)))
        return;
    spg_finish_sweep<INIT>(st, *snap, cur, w);
}

template <int K, int NT, bool INIT, int MODE, bool SWZ>
static constexpr size_t tma_smem_bytes()
{
    return sizeof(TmaSmem<K, NT, MODE == 1, TmaShape<K>::R>) + (SWZ ? 512 : 0);
}

template <int K, int NT, bool INIT, int MODE>
static cudaError_t launch_tma_mode(int grid, const SweepArgs &a, cudaStream_t s)
{
    if constexpr (TmaShape<K>::R * K == 16) {
        if (a.swz) {
            spg_sweep_tma_kernel<K, NT, INIT, MODE, true><<<grid, NT, tma_smem_bytes<K, NT, INIT, MODE, true>(), s>>>(a);
            return cudaGetLastError();
        }
    }
    spg_sweep_tma_kernel<K, NT, INIT, MODE, false><<<grid, NT, tma_smem_bytes<K, NT, INIT, MODE, false>(), s>>>(a);
    return cudaGetLastError();
}

template <int K, int NT, bool INIT>
static cudaError_t launch_tma_t(int grid, const SweepArgs &a, cudaStream_t s)
{
    // the dynamic shared memory limit was raised by tma_blocks_per_sm_t at problem creation
    // (no attribute call here: launches may be inside a stream capture)
    if (a.bmat) return launch_tma_mode<K, NT, INIT, 1>(grid, a, s);
    if (a.kw) return launch_tma_mode<K, NT, INIT, 2>(grid, a, s);
    return launch_tma_mode<K, NT, INIT, 0>(grid, a, s);
}

template <int K, int NT, bool INIT, int MODE, bool SWZ>
static int tma_blocks_per_sm_form()
{
    const size_t smem = tma_smem_bytes<K, NT, INIT, MODE, SWZ>();
    cudaFuncSetAttribute(spg_sweep_tma_kernel<K, NT, INIT, MODE, SWZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    // all of the unified L1/shared array as shared memory: the tiles arrive by bulk copy, and
    // the default split held K = 3 to 7 blocks per SM
    cudaFuncSetAttribute(spg_sweep_tma_kernel<K, NT, INIT, MODE, SWZ>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         (int)cudaSharedmemCarveoutMaxShared);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_sweep_tma_kernel<K, NT, INIT, MODE, SWZ>, NT, smem);
    return nb > 0 ? nb : 1;
}

// occupancy of the form in use (the swizzled one where it applies: K = 4, 8); the attributes of
// both forms are set
template <int K, int NT, bool INIT, int MODE>
static int tma_blocks_per_sm_mode()
{
    const int n0 = tma_blocks_per_sm_form<K, NT, INIT, MODE, false>();
    if constexpr (TmaShape<K>::R * K == 16) return tma_blocks_per_sm_form<K, NT, INIT, MODE, true>();
    return n0;
}

// sets the shared-memory limit of the three forms; returns the occupancy of the form that
// `bm` / `tp` select
template <int K, int NT, bool INIT>
static int tma_blocks_per_sm_t(bool bm, bool tp)
{
    const int n0 = tma_blocks_per_sm_mode<K, NT, INIT, 0>();
    const int n1 = tma_blocks_per_sm_mode<K, NT, INIT, 1>();
    const int n2 = tma_blocks_per_sm_mode<K, NT, INIT, 2>();
    return bm ? n1 : (tp ? n2 : n0);
}

constexpr int TMA_P = 512;  // timesteps per tile, for every K (TmaShape)

int sweep_tma_tile_width() { return TMA_P - 2 * TMA_HALO; }

int sweep_tma_threads(int K)
{
    switch (K) {
#define PASC_CASE(KK) case KK: return TmaShape<KK>::NT;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 0;
    }
}

bool sweep_tma_rows16(int K) { return K == 4 || K == 8; }  // TmaShape<K>::R * K == 16

typedef CUresult (*PFN_encodeTiled_rows)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                         const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                         CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                         CUtensorMapFloatOOBfill);

cudaError_t sweep_tma_make_rowmap(CUtensorMap *map, const float *base, long n, int rows_per_box)
{
    static PFN_encodeTiled_rows fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess) return e;
        if (q != cudaDriverEntryPointSuccess || !p) return cudaErrorNotSupported;
        fn = (PFN_encodeTiled_rows)p;
    }
    if (n < 16 || n % 16 != 0 || rows_per_box < 1 || rows_per_box > 256) return cudaErrorInvalidValue;
    memset(map, 0, sizeof *map);
    const cuuint64_t dims[2] = {16, (cuuint64_t)(n / 16)};
    const cuuint64_t strides[1] = {64};
    const cuuint32_t box[2] = {16, (cuuint32_t)rows_per_box};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void *)base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

bool sweep_tma_supported(int K) { return K >= 1 && K <= 8; }

int sweep_tma_blocks_per_sm(int K, bool init, bool bmat, bool tp)
{
    switch (K) {
#define PASC_CASE(KK)                                                       \
    case KK:                                                                \
        return init ? tma_blocks_per_sm_t<KK, TmaShape<KK>::NT, true>(bmat, tp)       \
                    : tma_blocks_per_sm_t<KK, TmaShape<KK>::NT, false>(bmat, tp);
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
        return init ? launch_tma_t<KK, TmaShape<KK>::NT, true>(grid, a, s)                 \
                    : launch_tma_t<KK, TmaShape<KK>::NT, false>(grid, a, s);
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pasc
