// kernels_batch.cu -- many independent FEM-H1 problems (signals of different length T, cluster
// count K and epssqr) advanced by ONE launch per SPG iteration.
//
// The reference solves such problems one after another (the epssqr sweep and annealing
// restarts of examples/test_signal1D/test_signal1D.cpp:268-353, include/general/solver/
// tssolver.h:522-698; independent signals are separate runs).  Here all of them share a
// persistent grid:
//   - each signal is cut into segments of seg_tiles bulk-copy tiles (sweep_tma.cuh); the
//     segments of the signals still running, grouped into work items of m consecutive
//     segments of one signal (m sized from how many segments are running: long items while
//     the GPU is full, short ones when few signals remain), form one work list, longest
//     signals first (rebuilt whenever the signals' states are read), and blocks take items in
//     turn from an atomic counter, so long and short signals balance across the GPU;
//   - an item is computed by one block with the tile pipeline of the single-signal kernel
//     (K dispatched at run time) and leaves its four partial sums in the slot of its first
//     segment, so the sums do not depend on which block took which item (deterministic);
//   - the block that completes the last item of a signal (per-signal ticket) reduces that
//     signal's slots in order and applies the reference's step-length, GLL and stopping rules
//     to that signal alone (sweep_common.cuh): every signal converges on its own, and the
//     segments of a signal whose solve has ended are skipped (per-signal convergence mask).
// The batched theta step uses the same work list.
#include "sweep_tma.cuh"
#include "sweep_common.cuh"

namespace pasc {

constexpr int BATCH_NT = 128;
constexpr int BATCH_W = BATCH_NT * TMA_R - 2 * TMA_HALO;  // owned timesteps per tile
// tiles per segment (BatchArgs::seg_tiles) and segments per work item are set at run time
// (batch.cu: batch_layout, batch_merge)

int batch_tile_width() { return BATCH_W; }
int batch_max_tile() { return BATCH_NT * TMA_R; }

// Computes one work item of signal `q`, the m segments from `seg` on (all threads of the
// block).  j counts the tiles this block has computed (it selects the stage) and parity holds
// the stages' phase bits; both persist across items.  Returns false if a bulk copy did not
// arrive in time.
template <int K, int KB, bool INIT>
__device__ __forceinline__ bool batch_segment(TmaSmem<KB, BATCH_NT> &sm, const BatchArgs &a, int q, int seg, int m,
                                              int &j, unsigned int &parity)
{
    const BatchInstDev &I = a.inst[q];
    SpgDevState *st = a.st + q;
    const int cur = st->cur;
    TileScalars<K> sc;
    sc.xin = (cur ? a.xb1 : a.xb0) + I.xoff;
    sc.xout = (cur ? a.xb0 : a.xb1) + I.xoff;
    sc.data = a.data + I.doff;
    sc.a0 = (float)st->alpha_prev;
    sc.beta = (float)st->beta;
    sc.a1 = (float)st->alpha_cur;
    sc.coeff = (float)st->coeff;
    sc.bscale = (float)st->bscale;
    sc.T = I.T;
#pragma unroll
    for (int k = 0; k < K; k++) sc.theta[k] = I.theta[k];

    const int lseg = seg - I.seg0;
    const int tlo = lseg * a.seg_tiles;
    const int thi = min(tlo + m * a.seg_tiles, I.tiles);
    if (lseg < 0 || lseg >= I.nseg || lseg % m != 0 || tlo >= thi) {
        // not an item of this signal (a work list out of step with the segment table): issue
        // no copy, report it
        if (threadIdx.x == 0) atomicExch(&st->error, 1);
        return true;
    }
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();  // the stages were last read through the generic proxy
        tma_issue<K>(sm, j & 1, sc.xin, sc.data, tlo * BATCH_W - TMA_HALO);
        if (tlo + 1 < thi) tma_issue<K>(sm, (j + 1) & 1, sc.xin, sc.data, (tlo + 1) * BATCH_W - TMA_HALO);
    }
    TileAcc acc;
    TilePending<K> pend;
    pend.valid = false;
    for (int tile = tlo; tile < thi; tile++, j++) {
        const int s = j & 1;
        const bool arrived = mbar_wait(&sm.bar[s], (parity >> s) & 1u);
        if (!tma_tile<K, KB, BATCH_NT, INIT>(sm, s, j, arrived, tile * BATCH_W - TMA_HALO, sc, acc, pend,
                                             tile + 2 < thi ? (tile + 2) * BATCH_W - TMA_HALO : TMA_NO_REFILL)) {
            mbar_wait(&sm.bar[s], (parity >> s) & 1u);
            if (tile + 1 < thi) mbar_wait(&sm.bar[s ^ 1], (parity >> (s ^ 1)) & 1u);
            return false;
        }
        parity ^= 1u << s;
    }
    __syncthreads();
    tma_flush_pending<K, KB, BATCH_NT, false, false, TMA_R>(sm, sc, acc, pend);  // the segment's last tile: its pair terms belong to this signal

    // the block that ends the signal's sweep snapshots its state into the first stage (free:
    // this item's copies were consumed, the next item's are issued after this) for the step logic
    static_assert(sizeof(SpgDevState) <= sizeof(sm.x[0]) && sizeof(SpgDevState) % 8 == 0, "state snapshot");
    SpgDevState *snap = reinterpret_cast<SpgDevState *>(sm.x[0]);
    double w[4];
    if (sweep_grid_sum4(acc.f, acc.dd, acc.dAd, acc.gd, reinterpret_cast<float2 *>(a.partials), seg, &a.ticket[q],
                        (unsigned int)((I.nseg + m - 1) / m), I.seg0, m, reinterpret_cast<float2 *>(sm.red), w, st,
                        snap, (int)sizeof(SpgDevState))) {
        a.ticket[q] = 0;
        spg_finish_sweep<INIT>(st, *snap, cur, w);
    }
    return true;
}

// resident blocks per SM the register allocation is held to: the run-time K switch makes the
// compiler allocate for the largest case, above what any single K needs
constexpr int batch_min_blocks(int KB) { return KB <= 3 ? 5 : KB <= 5 ? 4 : KB <= 7 ? 3 : 2; }

template <int KB, bool INIT>
__global__ void __launch_bounds__(BATCH_NT, batch_min_blocks(KB)) spg_batch_sweep_kernel(BatchArgs a)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    TmaSmem<KB, BATCH_NT> &sm = *reinterpret_cast<TmaSmem<KB, BATCH_NT> *>(smem_raw);
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
    int j = 0;
    unsigned int parity = 0u;
    const int nwork = a.nwork[0], m = max(a.nwork[1], 1);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) sm.job = (int)atomicAdd(a.next_job, 1u);
        __syncthreads();
        const int job = sm.job;
        if (job >= nwork) break;
        const int seg = a.work[job];
        if ((unsigned)seg >= (unsigned)a.nseg) continue;  // never for a list of the current layout
        const int q = a.seg_inst[seg];
        if (a.st[q].status != PASC_SPG_RUNNING) continue;  // this signal's solve ended in this chunk
        bool ok = true;
        switch (a.inst[q].K) {
#define PASC_CASE(KK) \
    case KK: if (KK <= KB) ok = batch_segment<(KK <= KB ? KK : 1), KB, INIT>(sm, a, q, seg, m, j, parity); break;
            PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
            PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
            default: break;
        }
        if (!ok) {
            if (threadIdx.x == 0) atomicExch(&a.st[q].error, 1);
            return;  // the copies in flight were waited for; the signal reports an error
        }
    }
}

// ---------------------------------------------------------------------------------------
// batched theta step (graphh1fem.cpp:347-380) on the same work list: an item sums
// gamma_tk x_t and gamma_tk over its timesteps; the last item of a signal divides.
// ---------------------------------------------------------------------------------------
constexpr int BATCH_THETA_NT = 256;

template <int K>
__device__ __forceinline__ void theta_segment(const BatchArgs &a, int q, int seg, int m, double *s_red)
{
    const BatchInstDev &I = a.inst[q];
    const float *gam = (a.st[q].cur ? a.xb1 : a.xb0) + I.xoff;
    const float *dat = a.data + I.doff;
    const long seg_t = (long)a.seg_tiles * BATCH_W;
    const long t_lo = (long)(seg - I.seg0) * seg_t;
    const long t_hi = t_lo + m * seg_t < I.T ? t_lo + m * seg_t : I.T;
    const int nitems = (I.nseg + m - 1) / m;
    KahanF sx[K], sg[K];
    for (long t = t_lo + threadIdx.x; t < t_hi; t += BATCH_THETA_NT) {
        const float x = __ldg(dat + t);
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float gk = __ldg(gam + t * K + k);
            sg[k].add(gk);
            sx[k].add(x * gk);
        }
    }
    double v[2 * K];
#pragma unroll
    for (int k = 0; k < K; k++) {
        v[k] = sx[k].value();
        v[K + k] = sg[k].value();
    }
    block_sum<2 * K>(v, s_red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int r = 0; r < 2 * K; r++) a.partials[(long)seg * 16 + r] = v[r];
    }
    if (!last_block_done_count(&a.ticket[q], (unsigned int)nitems)) return;
    double w[2 * K];
#pragma unroll
    for (int r = 0; r < 2 * K; r++) w[r] = 0.0;
    for (int b = threadIdx.x; b < nitems; b += BATCH_THETA_NT) {
#pragma unroll
        for (int r = 0; r < 2 * K; r++) w[r] += __ldcg(a.partials + ((long)I.seg0 + (long)b * m) * 16 + r);
    }
    block_sum<2 * K>(w, s_red);
    if (threadIdx.x == 0) {
        a.ticket[q] = 0;
        for (int k = 0; k < K; k++) {
            const double th = (w[K + k] != 0.0) ? w[k] / w[K + k] : 0.0;
            a.theta64[q * 8 + k] = th;
            a.inst[q].theta[k] = (float)th;
        }
    }
}

__global__ void __launch_bounds__(BATCH_THETA_NT) theta_batch_kernel(BatchArgs a)
{
    __shared__ double s_red[2 * 8 * (BATCH_THETA_NT / 32)];
    __shared__ int s_job;
    const int nwork = a.nwork[0], m = max(a.nwork[1], 1);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_job = (int)atomicAdd(a.next_job, 1u);
        __syncthreads();
        const int job = s_job;
        if (job >= nwork) break;
        const int seg = a.work[job];
        if ((unsigned)seg >= (unsigned)a.nseg) continue;  // never for a list of the current layout
        const int q = a.seg_inst[seg];
        if (!a.active[q]) continue;
        if ((seg - a.inst[q].seg0) % m != 0) {  // not the first segment of an item
            if (threadIdx.x == 0) atomicExch(&a.st[q].error, 1);
            continue;
        }
        switch (a.inst[q].K) {
#define PASC_CASE(KK) case KK: theta_segment<KK>(a, q, seg, m, s_red); break;
            PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
            PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
            default: break;
        }
    }
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
template <int KB, bool INIT>
static int batch_blocks_per_sm_t()
{
    const size_t smem = sizeof(TmaSmem<KB, BATCH_NT>);
    cudaFuncSetAttribute(spg_batch_sweep_kernel<KB, INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, spg_batch_sweep_kernel<KB, INIT>, BATCH_NT, smem);
    return nb > 0 ? nb : 1;
}

int batch_blocks_per_sm(int KB, bool init)
{
    switch (KB) {
#define PASC_CASE(KK) case KK: return init ? batch_blocks_per_sm_t<KK, true>() : batch_blocks_per_sm_t<KK, false>();
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return 1;
    }
}

cudaError_t launch_batch_sweep(int KB, bool init, int grid, const BatchArgs &a, cudaStream_t s)
{
    switch (KB) {
#define PASC_CASE(KK)                                                                                       \
    case KK:                                                                                                \
        if (init) spg_batch_sweep_kernel<KK, true><<<grid, BATCH_NT, sizeof(TmaSmem<KK, BATCH_NT>), s>>>(a); \
        else spg_batch_sweep_kernel<KK, false><<<grid, BATCH_NT, sizeof(TmaSmem<KK, BATCH_NT>), s>>>(a);     \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_theta_batch(int grid, const BatchArgs &a, cudaStream_t s)
{
    theta_batch_kernel<<<grid, BATCH_THETA_NT, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pasc
