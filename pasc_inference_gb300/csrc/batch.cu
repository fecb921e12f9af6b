// batch.cu -- C ABI of the batched solver: many independent FEM-H1 signals on one GPU, one
// launch per SPG iteration for all of them (kernels_batch.cu), each signal with its own
// T, K, epssqr, step lengths, GLL memory and stopping decision.
#include <math.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"

using namespace pasc;

namespace {

constexpr int IDLE = 99;  // status of a signal that takes no part in the current solve
constexpr long BPAD_FRONT = 4;

int bfail(int code, const std::string &msg)
{
    record_error(msg.c_str());
    return code;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// device-driven loops.  The batched SPG solve and the batched TSSolver run as ONE CUDA graph
// launch each: conditional WHILE nodes repeat the SPG sweeps of the running signals and the
// outer (theta step, gamma step, |L - L_old| test) iterations, and small single-block control
// kernels decide on the device whether to go on.  Every loop is bounded: the sweep loop ends
// once `spg_maxit` sweeps have run, the outer loop after `ts_maxit` iterations, whatever the
// signals' states, and both end on a device error (a bounded bulk-copy wait that gave up).
// ---------------------------------------------------------------------------------------
namespace pasc {

struct BatchLoop {
    // settings, written by the host before each launch
    int ts_maxit, ts_relative, chunk, spg_maxit;
    double ts_eps;
    double eps, gamma, sigma1, sigma2, alphainit;
    int maxit, m, stop_difff, stop_normgp, stop_Anormgp;
    // progress
    int outer_it, sweeps, error, launches;
};

struct BatchOuter {  // one signal's outer loop (TSSolver::solve, tssolver.h:550-645)
    double L, dL;
    int done, it_last, spg_it, spg_hm, incr, pad;
};

constexpr int BL_NT = 1024;

// exclusive prefix sum over the block of one int per thread; *total gets the sum
__device__ __forceinline__ int bl_scan(int v, int *s_warp, int *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < (BL_NT / 32) ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[32 + lane] = w;  // inclusive sums of the warps
    }
    __syncthreads();
    const int before = (warp ? s_warp[32 + warp - 1] : 0) + x - v;
    *total = s_warp[32 + BL_NT / 32 - 1];
    __syncthreads();
    return before;
}

// The work list: the items of the signals with take(i), longest signals first (the same list
// update_worklist builds on the host).
template <class Take>
__device__ void bl_worklist(const BatchArgs &a, int *work, int *nwork, Take take)
{
    __shared__ int s_warp[64];
    int nseg = 0;
    for (int q0 = 0; q0 < a.ninst; q0 += BL_NT) {
        const int q = q0 + threadIdx.x;
        int total;
        bl_scan((q < a.ninst && take(a.order[q])) ? a.inst[a.order[q]].nseg : 0, s_warp, &total);
        nseg += total;
    }
    const int m = batch_merge(nseg, a.merge_target, a.merge_max);
    int base = 0;
    for (int q0 = 0; q0 < a.ninst; q0 += BL_NT) {
        const int q = q0 + threadIdx.x;
        const int i = q < a.ninst ? a.order[q] : 0;
        const int cnt = (q < a.ninst && take(i)) ? (a.inst[i].nseg + m - 1) / m : 0;
        int total;
        const int off = base + bl_scan(cnt, s_warp, &total);
        for (int c = 0; c < cnt; c++) work[off + c] = a.inst[i].seg0 + c * m;
        base += total;
    }
    if (threadIdx.x == 0) {
        nwork[0] = base;
        nwork[1] = m;
        *a.next_job = 0u;
    }
}

__device__ __forceinline__ int bl_count(int v)
{
    return __syncthreads_count(v);
}

__global__ void __launch_bounds__(BL_NT) bl_begin_kernel(BatchArgs a, BatchLoop *L, BatchOuter *O, int *active)
{
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) {
        BatchOuter o;
        o.L = DBL_MAX;
        o.dL = DBL_MAX;
        o.done = o.it_last = o.spg_it = o.spg_hm = o.incr = o.pad = 0;
        O[i] = o;
        active[i] = 1;
    }
    if (threadIdx.x == 0) {
        L->outer_it = 0;
        L->error = 0;
        L->launches = 1;
    }
}

// theta step of the signals still in their outer loop: work list and tickets
__global__ void __launch_bounds__(BL_NT) bl_theta_head_kernel(BatchArgs a, int *work, int *nwork, BatchLoop *L)
{
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) a.ticket[i] = 0u;
    bl_worklist(a, work, nwork, [&](int i) { return a.active[i] != 0; });
    if (threadIdx.x == 0) L->launches += 2;
}

// start of an SPG solve of the active signals (the set-up of spgqpsolver.cpp:104-137 is the
// INIT sweep that follows); the others are left as they are (status IDLE)
__global__ void __launch_bounds__(BL_NT) bl_spg_setup_kernel(BatchArgs a, int *work, int *nwork, BatchLoop *L,
                                                             const double *coeffA, const double *coeffB,
                                                             cudaGraphConditionalHandle h_sweeps)
{
    const BatchLoop cfg = *L;
    int nact = 0;
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) {
        SpgDevState &h = a.st[i];
        const int cur = h.cur;
        SpgDevState z;
        memset(&z, 0, sizeof z);
        z.alpha_prev = z.alpha_cur = cfg.alphainit;
        z.coeff = coeffA[i];
        z.bscale = coeffB[i];
        z.eps = cfg.eps;
        z.gamma = cfg.gamma;
        z.sigma1 = cfg.sigma1;
        z.sigma2 = cfg.sigma2;
        z.maxit = cfg.maxit;
        z.m = cfg.m;
        z.stop_difff = cfg.stop_difff;
        z.stop_normgp = cfg.stop_normgp;
        z.stop_Anormgp = cfg.stop_Anormgp;
        z.cur = cur;
        z.status = a.active[i] ? PASC_SPG_RUNNING : 99;  // 99: takes no part (batch.cu IDLE)
        h = z;
        a.ticket[i] = 0u;
        nact += a.active[i] ? 1 : 0;
    }
    nact = bl_count(nact > 0);
    bl_worklist(a, work, nwork, [&](int i) { return a.active[i] != 0; });
    if (threadIdx.x == 0) {
        L->sweeps = 0;
        L->launches += 2;  // this kernel and the INIT sweep
        cudaGraphSetConditional(h_sweeps, nact > 0 ? 1u : 0u);
    }
}

// after `chunk` sweeps: drop the signals whose solve ended from the work list and decide on
// the next chunk
__global__ void __launch_bounds__(BL_NT) bl_spg_poll_kernel(BatchArgs a, int *work, int *nwork, BatchLoop *L,
                                                            cudaGraphConditionalHandle h_sweeps)
{
    int running = 0, err = 0;
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) {
        running |= a.st[i].status == PASC_SPG_RUNNING;
        err |= a.st[i].error != 0;
    }
    running = bl_count(running);
    err = bl_count(err);
    bl_worklist(a, work, nwork, [&](int i) { return a.st[i].status == PASC_SPG_RUNNING; });
    if (threadIdx.x == 0) {
        const int sweeps = L->sweeps + L->chunk;
        L->sweeps = sweeps;
        L->launches += L->chunk + 1;
        if (err) L->error = 1;
        cudaGraphSetConditional(h_sweeps, (running > 0 && err == 0 && sweeps < L->spg_maxit) ? 1u : 0u);
    }
}

// end of a batched SPG solve: a solve still running has used its iterations
__global__ void __launch_bounds__(BL_NT) bl_spg_final_kernel(BatchArgs a, BatchLoop *L)
{
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT)
        if (a.st[i].status == PASC_SPG_RUNNING) a.st[i].status = PASC_SPG_MAXIT;
    if (threadIdx.x == 0) L->launches += 1;
}

// end of an outer iteration (tssolver.h:618-645): L, |L - L_old| and the stopping test of
// every active signal; a signal whose test holds leaves the loop
__global__ void __launch_bounds__(BL_NT) bl_outer_tail_kernel(BatchArgs a, BatchLoop *L, BatchOuter *O, int *active,
                                                              cudaGraphConditionalHandle h_outer)
{
    const int it = L->outer_it;
    const int ts_maxit = L->ts_maxit;
    int left = 0;
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) {
        if (!active[i]) continue;
        SpgDevState &h = a.st[i];
        if (h.status == PASC_SPG_RUNNING) h.status = PASC_SPG_MAXIT;
        BatchOuter o = O[i];
        o.spg_it += h.it;
        o.spg_hm += h.hessmult;
        const double L_old = o.L;
        o.L = h.fx;
        o.dL = fabs(o.L - L_old);
        if (o.L - L_old > 0) o.incr++;
        o.it_last = it;
        const bool stop = L->ts_relative ? (o.dL < L->ts_eps * fabs(o.L)) : (o.dL < L->ts_eps);
        if (stop) {
            o.done = 1;
            active[i] = 0;
        } else {
            if (it == ts_maxit - 1) o.it_last = ts_maxit;
            left = 1;
        }
        O[i] = o;
    }
    left = bl_count(left);
    int err = 0;
    for (int i = threadIdx.x; i < a.ninst; i += BL_NT) err |= a.st[i].error != 0;
    err = bl_count(err);
    if (threadIdx.x == 0) {
        L->outer_it = it + 1;
        L->launches += 1;
        if (err) L->error = 1;
        cudaGraphSetConditional(h_outer, (left > 0 && err == 0 && L->error == 0 && it + 1 < ts_maxit) ? 1u : 0u);
    }
}

}  // namespace pasc

#define BCU(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return bfail(PASC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
#define BCHK(call)                     \
    do {                               \
        int r_ = (call);               \
        if (r_ != PASC_OK) return r_;  \
    } while (0)

static constexpr int BATCH_CHUNK = 16;
static constexpr int BATCH_MIN_SEG_TILES = 2;  // the smallest segment size
// automatic work items: segments of 4 tiles merged into items of up to 32 tiles, about four
// items per resident block (measured on 256 signals of 1e3..1e6 timesteps: fixed 4-tile items
// were best for the TSSolver, whose late sweeps run few signals, fixed 16-tile items for
// long QP solves of all signals)
static constexpr int BATCH_AUTO_SEG_TILES = 4;
static constexpr int BATCH_MERGE_MAX_TILES = 32;
static constexpr int BATCH_AUTO_ITEMS_PER_BLOCK = 4;

struct pasc_gb300_batch {
    int n = 0, device = 0, sms = 0, KB = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<long> T;
    std::vector<int> K;
    std::vector<double> epssqr, coeffA, coeffB;
    std::vector<BatchInstDev> inst_h;
    std::vector<int> cur;  // buffer holding each signal's gamma
    BatchInstDev *inst_d = nullptr;
    int *seg_inst_d = nullptr;
    int nseg = 0, nseg_max = 0;
    // segments: bulk-copy tiles per segment; merge_per_block > 0: work items of up to
    // BATCH_MERGE_MAX_TILES tiles sized for about merge_per_block items per resident block of
    // the sweep grid, 0: one segment per item (a pinned size).  order: signals by decreasing T
    int seg_tiles = BATCH_AUTO_SEG_TILES, merge_per_block = BATCH_AUTO_ITEMS_PER_BLOCK;
    std::vector<int> order_h;
    int *order_d = nullptr;
    // work list: the items of the signals taking part in the next launches; nwork_d holds
    // {items, segments per item}
    int *work_d = nullptr, *nwork_d = nullptr, *work_h = nullptr;
    std::vector<char> in_work;  // signals in the uploaded list (valid while work_valid)
    bool work_valid = false;
    long nx = 0, nd = 0, maxN = 0;
    float *xb[2] = {nullptr, nullptr}, *data = nullptr;
    double *stage64 = nullptr;
    SpgDevState *st_d = nullptr, *st_h = nullptr;
    double *partials = nullptr, *theta64 = nullptr;
    unsigned int *ticket = nullptr, *next_job = nullptr;
    int *active_d = nullptr, *active_h = nullptr;
    int grid = 0, grid_init = 0, grid_theta = 0, occ = 1, occ_init = 1;
    cudaGraphExec_t chunk = nullptr;
    pasc_gb300_spgqp_opts o{};
    int launches = 0;
    // device-driven loops (one graph launch per solve): control state, per-signal outer-loop
    // records, the graphs (SPG solve; TSSolver without / with the theta step) and the capture
    // streams of the loop bodies
    int device_loop = 1;
    int loop_chunk = 4;
    BatchLoop *loop_d = nullptr, *loop_h = nullptr;
    BatchOuter *outer_d = nullptr, *outer_h = nullptr;
    double *coeffA_d = nullptr, *coeffB_d = nullptr;
    cudaGraphExec_t g_spg = nullptr, g_ts[2] = {nullptr, nullptr};
    cudaStream_t aux[2] = {nullptr, nullptr};
};


static void batch_free(pasc_gb300_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->chunk) cudaGraphExecDestroy(b->chunk);
    for (cudaGraphExec_t g : {b->g_spg, b->g_ts[0], b->g_ts[1]})
        if (g) cudaGraphExecDestroy(g);
    for (cudaStream_t q : b->aux)
        if (q) cudaStreamDestroy(q);
    if (b->loop_h) cudaFreeHost(b->loop_h);
    if (b->outer_h) cudaFreeHost(b->outer_h);
    void *dev[] = {b->inst_d, b->seg_inst_d, b->work_d, b->nwork_d, b->xb[0], b->xb[1], b->data, b->stage64, b->st_d, b->partials,
                   b->theta64, b->ticket, b->next_job, b->active_d, b->loop_d, b->outer_d, b->coeffA_d, b->coeffB_d,
                   b->order_d};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (b->st_h) cudaFreeHost(b->st_h);
    if (b->active_h) cudaFreeHost(b->active_h);
    if (b->work_h) cudaFreeHost(b->work_h);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Cuts every signal into segments of seg_tiles tiles (segment numbers in signal order, as the
// per-signal reductions expect) and sizes the grids.  Drops the cached graphs (they hold the
// launch shapes) and the uploaded work list (it numbers segments of the old layout).
static int batch_layout(pasc_gb300_batch *b, int seg_tiles)
{
    std::vector<int> seg_inst;
    // the device copy holds the theta the batched theta step wrote last
    BCU(cudaStreamSynchronize(b->stream));
    BCU(cudaMemcpy(b->inst_h.data(), b->inst_d, sizeof(BatchInstDev) * b->n, cudaMemcpyDeviceToHost));
    for (int i = 0; i < b->n; i++) {
        BatchInstDev &I = b->inst_h[i];
        I.seg0 = (int)seg_inst.size();
        I.nseg = (I.tiles + seg_tiles - 1) / seg_tiles;
        for (int s = 0; s < I.nseg; s++) seg_inst.push_back(i);
    }
    if ((int)seg_inst.size() > b->nseg_max) return bfail(PASC_ERR_STATE, "batch: segment table overflow");
    b->seg_tiles = seg_tiles;
    b->nseg = (int)seg_inst.size();
    b->grid = std::max(1, std::min(b->occ * b->sms, b->nseg));
    b->grid_init = std::max(1, std::min(b->occ_init * b->sms, b->nseg));
    b->grid_theta = std::max(1, std::min(b->sms * 4, b->nseg));
    BCU(cudaMemcpy(b->inst_d, b->inst_h.data(), sizeof(BatchInstDev) * b->n, cudaMemcpyHostToDevice));
    BCU(cudaMemcpy(b->seg_inst_d, seg_inst.data(), sizeof(int) * b->nseg, cudaMemcpyHostToDevice));
    for (cudaGraphExec_t *g : {&b->chunk, &b->g_spg, &b->g_ts[0], &b->g_ts[1]}) {
        if (*g) cudaGraphExecDestroy(*g);
        *g = nullptr;
    }
    b->work_valid = false;
    return PASC_OK;
}

static BatchArgs batch_args(pasc_gb300_batch *b)
{
    BatchArgs a;
    a.inst = b->inst_d;
    a.seg_inst = b->seg_inst_d;
    a.work = b->work_d;
    a.nwork = b->nwork_d;
    a.nseg = b->nseg;
    a.ninst = b->n;
    a.xb0 = b->xb[0];
    a.xb1 = b->xb[1];
    a.data = b->data;
    a.st = b->st_d;
    a.partials = b->partials;
    a.ticket = b->ticket;
    a.next_job = b->next_job;
    a.active = b->active_d;
    a.theta64 = b->theta64;
    a.order = b->order_d;
    a.seg_tiles = b->seg_tiles;
    a.merge_target = b->merge_per_block * b->grid;
    a.merge_max = std::max(1, BATCH_MERGE_MAX_TILES / b->seg_tiles);
    return a;
}

static int batch_check_index(pasc_gb300_batch *b, int i)
{
    if (!b) return bfail(PASC_ERR_ARG, "batch: NULL handle");
    if (i < 0 || i >= b->n) return bfail(PASC_ERR_ARG, "batch: signal index out of range");
    return PASC_OK;
}

extern "C" {

int pasc_gb300_batch_create(pasc_gb300_batch **out, int n, const long *T, const int *K, const double *epssqr,
                            int device)
{
    if (!out || !T || !K || !epssqr) return bfail(PASC_ERR_ARG, "batch_create: NULL argument");
    *out = nullptr;
    if (n < 1) return bfail(PASC_ERR_ARG, "batch_create: n must be >= 1");
    int ndev = pasc_gb300_device_count();
    if (ndev <= 0) return bfail(PASC_ERR_CUDA, "batch_create: no CUDA device available");
    if (device < 0 || device >= ndev) return bfail(PASC_ERR_ARG, "batch_create: device out of range");
    pasc_gb300_batch *b = new pasc_gb300_batch();
    auto bail = [&](int code) { batch_free(b); return code; };
    b->n = n;
    b->device = device;
    b->T.assign(T, T + n);
    b->K.assign(K, K + n);
    b->epssqr.assign(epssqr, epssqr + n);
    b->cur.assign(n, 0);
    const int W = batch_tile_width();
    const long PADB = batch_max_tile();
    b->inst_h.resize(n);
    long xo = 0, doff = 0;
    for (int i = 0; i < n; i++) {
        if (T[i] < 1 || K[i] < 1 || K[i] > 8)
            return bail(bfail(PASC_ERR_ARG, "batch_create: signal " + std::to_string(i) + " needs T >= 1 and 1 <= K <= 8"));
        if ((double)T[i] * K[i] > 1.0e9) return bail(bfail(PASC_ERR_ARG, "batch_create: signal too long"));
        b->KB = std::max(b->KB, K[i]);
        BatchInstDev &I = b->inst_h[i];
        memset(&I, 0, sizeof I);
        I.T = (int)T[i];
        I.K = K[i];
        I.xoff = xo + BPAD_FRONT * K[i];
        I.doff = doff + BPAD_FRONT;
        xo += ((BPAD_FRONT + T[i] + PADB) * K[i] + 3) / 4 * 4;  // next signal starts 16-byte aligned
        doff += (BPAD_FRONT + T[i] + PADB + 3) / 4 * 4;
        I.tiles = (int)((T[i] + W - 1) / W);
        b->nseg_max += (I.tiles + BATCH_MIN_SEG_TILES - 1) / BATCH_MIN_SEG_TILES;
        b->maxN = std::max(b->maxN, T[i] * (long)K[i]);
        double c = epssqr[i] * (1.0 / (double)T[i]);  // graphh1fem.cpp:146-151
        b->coeffA.push_back(c);
        b->coeffB.push_back(-1.0 * (1.0 / (double)T[i]));  // graphh1fem.cpp:280-283
    }
    b->nx = xo;
    b->nd = doff;
    b->order_h.resize(n);
    for (int i = 0; i < n; i++) b->order_h[i] = i;
    std::stable_sort(b->order_h.begin(), b->order_h.end(), [&](int x, int y) { return T[x] > T[y]; });
    if (cudaSetDevice(device) != cudaSuccess) return bail(bfail(PASC_ERR_CUDA, "cudaSetDevice failed"));
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)
        return bail(bfail(PASC_ERR_CUDA, "batch_create: stream/event creation failed"));
    auto dal = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes > 0 ? bytes : 1) == cudaSuccess; };
    if (!dal((void **)&b->inst_d, sizeof(BatchInstDev) * n) || !dal((void **)&b->seg_inst_d, sizeof(int) * b->nseg_max) ||
        !dal((void **)&b->xb[0], sizeof(float) * b->nx) || !dal((void **)&b->xb[1], sizeof(float) * b->nx) ||
        !dal((void **)&b->data, sizeof(float) * b->nd) || !dal((void **)&b->stage64, sizeof(double) * b->maxN) ||
        !dal((void **)&b->st_d, sizeof(SpgDevState) * n) || !dal((void **)&b->partials, sizeof(double) * 16 * b->nseg_max) ||
        !dal((void **)&b->theta64, sizeof(double) * 8 * n) || !dal((void **)&b->ticket, sizeof(unsigned int) * n) ||
        !dal((void **)&b->next_job, sizeof(unsigned int)) || !dal((void **)&b->active_d, sizeof(int) * n) ||
        !dal((void **)&b->work_d, sizeof(int) * b->nseg_max) || !dal((void **)&b->nwork_d, 2 * sizeof(int)) ||
        !dal((void **)&b->order_d, sizeof(int) * n) ||
        !dal((void **)&b->loop_d, sizeof(BatchLoop)) || !dal((void **)&b->outer_d, sizeof(BatchOuter) * n) ||
        !dal((void **)&b->coeffA_d, sizeof(double) * n) || !dal((void **)&b->coeffB_d, sizeof(double) * n))
        return bail(bfail(PASC_ERR_ALLOC, "batch_create: device allocation failed"));
    if (cudaMallocHost((void **)&b->st_h, sizeof(SpgDevState) * n) != cudaSuccess ||
        cudaMallocHost((void **)&b->active_h, sizeof(int) * n) != cudaSuccess ||
        cudaMallocHost((void **)&b->work_h, sizeof(int) * (b->nseg_max + 2)) != cudaSuccess ||
        cudaMallocHost((void **)&b->loop_h, sizeof(BatchLoop)) != cudaSuccess ||
        cudaMallocHost((void **)&b->outer_h, sizeof(BatchOuter) * n) != cudaSuccess)
        return bail(bfail(PASC_ERR_ALLOC, "batch_create: pinned allocation failed"));
    if (cudaStreamCreateWithFlags(&b->aux[0], cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->aux[1], cudaStreamNonBlocking) != cudaSuccess)
        return bail(bfail(PASC_ERR_CUDA, "batch_create: stream creation failed"));
    memset(b->loop_h, 0, sizeof(BatchLoop));
    cudaMemcpy(b->coeffA_d, b->coeffA.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(b->coeffB_d, b->coeffB.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    memset(b->st_h, 0, sizeof(SpgDevState) * n);
    cudaMemset(b->xb[0], 0, sizeof(float) * b->nx);  // pads stay zero: kernels write 0 <= t < T only
    cudaMemset(b->xb[1], 0, sizeof(float) * b->nx);
    cudaMemset(b->data, 0, sizeof(float) * b->nd);
    cudaMemset(b->st_d, 0, sizeof(SpgDevState) * n);
    cudaMemset(b->ticket, 0, sizeof(unsigned int) * n);
    cudaMemset(b->theta64, 0, sizeof(double) * 8 * n);
    cudaMemset(b->nwork_d, 0, 2 * sizeof(int));
    b->in_work.assign(n, 0);
    cudaMemcpy(b->inst_d, b->inst_h.data(), sizeof(BatchInstDev) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(b->order_d, b->order_h.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    b->occ = batch_blocks_per_sm(b->KB, false);
    b->occ_init = batch_blocks_per_sm(b->KB, true);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess ||
        batch_layout(b, b->seg_tiles) != PASC_OK || cudaDeviceSynchronize() != cudaSuccess)
        return bail(bfail(PASC_ERR_CUDA, "batch_create: initialisation failed"));
    *out = b;
    return PASC_OK;
}

int pasc_gb300_batch_destroy(pasc_gb300_batch *b)
{
    batch_free(b);
    return PASC_OK;
}

int pasc_gb300_batch_set_loop(pasc_gb300_batch *b, int device_loop, int chunk)
{
    if (!b) return bfail(PASC_ERR_ARG, "batch_set_loop: NULL handle");
    if (chunk < 1 || chunk > 64) return bfail(PASC_ERR_ARG, "batch_set_loop: chunk must be in [1, 64]");
    BCU(cudaSetDevice(b->device));
    BCU(cudaStreamSynchronize(b->stream));
    if (chunk != b->loop_chunk) {
        for (cudaGraphExec_t *g : {&b->g_spg, &b->g_ts[0], &b->g_ts[1]}) {
            if (*g) cudaGraphExecDestroy(*g);
            *g = nullptr;
        }
        b->loop_chunk = chunk;
    }
    b->device_loop = device_loop ? 1 : 0;
    return PASC_OK;
}

int pasc_gb300_batch_set_segment_tiles(pasc_gb300_batch *b, int tiles)
{
    if (!b) return bfail(PASC_ERR_ARG, "batch_set_segment_tiles: NULL handle");
    if (tiles > 64 || tiles == 1 || tiles < -16)
        return bfail(PASC_ERR_ARG, "batch_set_segment_tiles: tiles must be in [2, 64], 0 (automatic) or in [-16, -1]");
    BCU(cudaSetDevice(b->device));
    if (tiles > 0) {
        b->merge_per_block = 0;
        return batch_layout(b, tiles);
    }
    b->merge_per_block = tiles < 0 ? -tiles : BATCH_AUTO_ITEMS_PER_BLOCK;
    b->work_valid = false;
    return b->seg_tiles == BATCH_AUTO_SEG_TILES ? PASC_OK : batch_layout(b, BATCH_AUTO_SEG_TILES);
}

int pasc_gb300_batch_get_segment_tiles(pasc_gb300_batch *b, int *seg_tiles, int *item_tiles)
{
    if (!b || !seg_tiles) return bfail(PASC_ERR_ARG, "batch_get_segment_tiles: NULL argument");
    *seg_tiles = b->seg_tiles;
    if (item_tiles) {
        const BatchArgs a = batch_args(b);
        *item_tiles = batch_merge(b->nseg, a.merge_target, a.merge_max) * b->seg_tiles;
    }
    return PASC_OK;
}

int pasc_gb300_batch_size(pasc_gb300_batch *b, int *n)
{
    if (!b || !n) return bfail(PASC_ERR_ARG, "batch_size: NULL argument");
    *n = b->n;
    return PASC_OK;
}

int pasc_gb300_batch_set_data(pasc_gb300_batch *b, int i, const double *data)
{
    BCHK(batch_check_index(b, i));
    if (!data) return bfail(PASC_ERR_ARG, "batch_set_data: NULL data");
    BCU(cudaSetDevice(b->device));
    BCU(cudaMemcpyAsync(b->stage64, data, sizeof(double) * b->T[i], cudaMemcpyHostToDevice, b->stream));
    BCU(launch_f64_to_f32(b->stage64, b->data + b->inst_h[i].doff, b->T[i], b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return PASC_OK;
}

int pasc_gb300_batch_set_gamma(pasc_gb300_batch *b, int i, const double *gamma)
{
    BCHK(batch_check_index(b, i));
    if (!gamma) return bfail(PASC_ERR_ARG, "batch_set_gamma: NULL gamma");
    BCU(cudaSetDevice(b->device));
    const long N = b->T[i] * b->K[i];
    BCU(cudaMemcpyAsync(b->stage64, gamma, sizeof(double) * N, cudaMemcpyHostToDevice, b->stream));
    BCU(launch_f64_to_f32(b->stage64, b->xb[b->cur[i]] + b->inst_h[i].xoff, N, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return PASC_OK;
}

int pasc_gb300_batch_get_gamma(pasc_gb300_batch *b, int i, double *gamma)
{
    BCHK(batch_check_index(b, i));
    if (!gamma) return bfail(PASC_ERR_ARG, "batch_get_gamma: NULL gamma");
    BCU(cudaSetDevice(b->device));
    const long N = b->T[i] * b->K[i];
    BCU(launch_f32_to_f64(b->xb[b->cur[i]] + b->inst_h[i].xoff, b->stage64, N, b->stream));
    BCU(cudaMemcpyAsync(gamma, b->stage64, sizeof(double) * N, cudaMemcpyDeviceToHost, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return PASC_OK;
}

int pasc_gb300_batch_set_theta(pasc_gb300_batch *b, int i, const double *theta)
{
    BCHK(batch_check_index(b, i));
    if (!theta) return bfail(PASC_ERR_ARG, "batch_set_theta: NULL theta");
    BCU(cudaSetDevice(b->device));
    BatchInstDev &I = b->inst_h[i];
    for (int k = 0; k < b->K[i]; k++) I.theta[k] = (float)theta[k];
    BCU(cudaMemcpyAsync(b->theta64 + 8 * i, theta, sizeof(double) * b->K[i], cudaMemcpyHostToDevice, b->stream));
    BCU(cudaMemcpyAsync(b->inst_d + i, &I, sizeof(BatchInstDev), cudaMemcpyHostToDevice, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return PASC_OK;
}

int pasc_gb300_batch_get_theta(pasc_gb300_batch *b, int i, double *theta)
{
    BCHK(batch_check_index(b, i));
    if (!theta) return bfail(PASC_ERR_ARG, "batch_get_theta: NULL theta");
    BCU(cudaSetDevice(b->device));
    BCU(cudaMemcpyAsync(theta, b->theta64 + 8 * i, sizeof(double) * b->K[i], cudaMemcpyDeviceToHost, b->stream));
    BCU(cudaStreamSynchronize(b->stream));
    return PASC_OK;
}

}  // extern "C"

// blocked k*T+t -> interleaved t*K+k for every signal (TSSolver::gammavector_permute)
static int batch_permute(pasc_gb300_batch *b)
{
    for (int i = 0; i < b->n; i++) {
        const long off = b->inst_h[i].xoff;
        BCU(launch_permute_f32(b->xb[b->cur[i]] + off, b->xb[b->cur[i] ^ 1] + off, b->T[i], b->K[i], b->stream));
        b->cur[i] ^= 1;
    }
    return PASC_OK;
}

// Rebuilds the work list from take[i] (signal i takes part) when that set changed since the
// last upload: the items of every signal taking part, longest signals first (the list
// bl_worklist builds on the device, item for item).
template <class Pred>
static int update_worklist(pasc_gb300_batch *b, Pred take)
{
    bool same = b->work_valid;
    for (int i = 0; i < b->n && same; i++) same = (b->in_work[i] != 0) == take(i);
    if (same) return PASC_OK;
    BCU(cudaStreamSynchronize(b->stream));  // the pinned list may still be feeding an upload
    int nseg = 0;
    for (int i = 0; i < b->n; i++) {
        b->in_work[i] = take(i) ? 1 : 0;
        if (b->in_work[i]) nseg += b->inst_h[i].nseg;
    }
    const BatchArgs a = batch_args(b);
    const int m = batch_merge(nseg, a.merge_target, a.merge_max);
    int cnt = 0;
    for (int q = 0; q < b->n; q++) {
        const int i = b->order_h[q];
        if (!b->in_work[i]) continue;
        const BatchInstDev &I = b->inst_h[i];
        for (int s = 0; s < I.nseg; s += m) b->work_h[2 + cnt++] = I.seg0 + s;
    }
    b->work_h[0] = cnt;
    b->work_h[1] = m;
    b->work_valid = true;
    BCU(cudaMemcpyAsync(b->nwork_d, b->work_h, 2 * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    if (cnt) BCU(cudaMemcpyAsync(b->work_d, b->work_h + 2, sizeof(int) * cnt, cudaMemcpyHostToDevice, b->stream));
    return PASC_OK;
}

static int ensure_batch_graph(pasc_gb300_batch *b)
{
    if (b->chunk) return PASC_OK;
    BCU(cudaStreamSynchronize(b->stream));
    BatchArgs a = batch_args(b);
    cudaGraph_t g;
    BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int q = 0; q < BATCH_CHUNK; q++) {
        cudaError_t e = cudaMemsetAsync(b->next_job, 0, sizeof(unsigned int), b->stream);
        if (e == cudaSuccess) e = launch_batch_sweep(b->KB, false, b->grid, a, b->stream);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(b->stream, &g);
            return bfail(PASC_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
        }
    }
    BCU(cudaStreamEndCapture(b->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&b->chunk, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->chunk = nullptr;
        return bfail(PASC_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e));
    }
    return PASC_OK;
}

// ---------------------------------------------------------------------------------------
// graphs of the device-driven loops
// ---------------------------------------------------------------------------------------

// A conditional handle for a node of the graph stream s is capturing into.
static cudaError_t capture_handle(cudaStream_t s, unsigned int dflt, unsigned int flags, cudaGraphConditionalHandle *h)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusActive || !g) return cudaErrorStreamCaptureInvalidated;
    return cudaGraphConditionalHandleCreate(h, g, dflt, flags);
}

// Appends a WHILE node on handle h to the capture of s (after the captured work so far) and
// makes it the capture's only dependency; *body receives the node's body graph.
static cudaError_t capture_while(cudaStream_t s, cudaGraphConditionalHandle h, cudaGraph_t *body)
{
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    if (cs != cudaStreamCaptureStatusActive || !g) return cudaErrorStreamCaptureInvalidated;
    std::vector<cudaGraphNode_t> dv(deps, deps + nd);
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    e = cudaGraphAddNode(&node, g, dv.empty() ? nullptr : dv.data(), nullptr, dv.size(), &np);
    if (e != cudaSuccess) return e;
    *body = np.conditional.phGraph_out[0];
    return cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// Captures the SPG solve of the active signals on s: set-up, INIT sweep, then a WHILE loop
// of `loop_chunk` sweeps and a poll, as long as a signal runs (bounded by spg_maxit sweeps).
static cudaError_t capture_spg(pasc_gb300_batch *b, cudaStream_t s, cudaStream_t body_stream)
{
    BatchArgs a = batch_args(b);
    cudaGraphConditionalHandle hs;
    cudaError_t e = capture_handle(s, 0u, 0u, &hs);
    if (e != cudaSuccess) return e;
    bl_spg_setup_kernel<<<1, BL_NT, 0, s>>>(a, b->work_d, b->nwork_d, b->loop_d, b->coeffA_d, b->coeffB_d, hs);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = launch_batch_sweep(b->KB, true, b->grid_init, a, s)) != cudaSuccess) return e;
    cudaGraph_t body = nullptr;
    if ((e = capture_while(s, hs, &body)) != cudaSuccess) return e;
    // the loop body, captured on its own stream into the node's body graph
    if ((e = cudaStreamBeginCaptureToGraph(body_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
        return e;
    for (int q = 0; q < b->loop_chunk && e == cudaSuccess; q++) {
        e = cudaMemsetAsync(b->next_job, 0, sizeof(unsigned int), body_stream);
        if (e == cudaSuccess) e = launch_batch_sweep(b->KB, false, b->grid, a, body_stream);
    }
    if (e == cudaSuccess) {
        bl_spg_poll_kernel<<<1, BL_NT, 0, body_stream>>>(a, b->work_d, b->nwork_d, b->loop_d, hs);
        e = cudaGetLastError();
    }
    cudaGraph_t out = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(body_stream, &out);
    return e != cudaSuccess ? e : e2;
}

static int instantiate(cudaStream_t s, cudaError_t e, cudaGraphExec_t *exec, const char *what)
{
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        *exec = nullptr;
        cudaGetLastError();
        return bfail(PASC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
    return PASC_OK;
}

// The batched SPG solve as one graph.
static int ensure_spg_loop_graph(pasc_gb300_batch *b)
{
    if (b->g_spg) return PASC_OK;
    BCU(cudaStreamSynchronize(b->stream));
    BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = capture_spg(b, b->stream, b->aux[1]);
    if (e == cudaSuccess) {
        bl_spg_final_kernel<<<1, BL_NT, 0, b->stream>>>(batch_args(b), b->loop_d);
        e = cudaGetLastError();
    }
    return instantiate(b->stream, e, &b->g_spg, "batch SPG loop graph");
}

// The batched TSSolver as one graph: WHILE (a signal is in its outer loop) { theta step,
// SPG solve (its own WHILE loop), |L - L_old| test }.
static int ensure_ts_loop_graph(pasc_gb300_batch *b, int thetasolved)
{
    cudaGraphExec_t *exec = &b->g_ts[thetasolved ? 1 : 0];
    if (*exec) return PASC_OK;
    BCU(cudaStreamSynchronize(b->stream));
    BatchArgs a = batch_args(b);
    BCU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    bl_begin_kernel<<<1, BL_NT, 0, b->stream>>>(a, b->loop_d, b->outer_d, b->active_d);
    e = cudaGetLastError();
    cudaGraphConditionalHandle ho;
    cudaGraph_t body = nullptr;
    if (e == cudaSuccess) e = capture_handle(b->stream, 1u, cudaGraphCondAssignDefault, &ho);
    if (e == cudaSuccess) e = capture_while(b->stream, ho, &body);
    if (e == cudaSuccess) {
        cudaStream_t s = b->aux[0];
        e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (!thetasolved) {
                bl_theta_head_kernel<<<1, BL_NT, 0, s>>>(a, b->work_d, b->nwork_d, b->loop_d);
                e = cudaGetLastError();
                if (e == cudaSuccess) e = launch_theta_batch(b->grid_theta, a, s);
            }
            if (e == cudaSuccess) e = capture_spg(b, s, b->aux[1]);
            if (e == cudaSuccess) {
                bl_outer_tail_kernel<<<1, BL_NT, 0, s>>>(a, b->loop_d, b->outer_d, b->active_d, ho);
                e = cudaGetLastError();
            }
            cudaGraph_t out = nullptr;
            cudaError_t e2 = cudaStreamEndCapture(s, &out);
            if (e == cudaSuccess) e = e2;
        }
    }
    return instantiate(b->stream, e, exec, "batch TSSolver loop graph");
}

static void loop_settings(pasc_gb300_batch *b, const pasc_gb300_spgqp_opts *o)
{
    BatchLoop &L = *b->loop_h;
    L.eps = o->eps;
    L.gamma = o->gamma;
    L.sigma1 = o->sigma1;
    L.sigma2 = o->sigma2;
    L.alphainit = o->alphainit;
    L.maxit = o->maxit;
    L.m = o->m;
    L.stop_difff = o->stop_difff;
    L.stop_normgp = o->stop_normgp;
    L.stop_Anormgp = o->stop_Anormgp;
    L.spg_maxit = o->maxit;
    L.chunk = b->loop_chunk;
    L.outer_it = L.sweeps = L.error = L.launches = 0;
}

// Uploads the settings and each signal's current buffer index, launches `g` and reads the
// states back.
static int run_loop_graph(pasc_gb300_batch *b, cudaGraphExec_t g, double *elapsed_ms)
{
    cudaStream_t s = b->stream;
    BCU(cudaStreamSynchronize(s));
    for (int i = 0; i < b->n; i++) b->st_h[i].cur = b->cur[i];
    BCU(cudaMemcpyAsync(b->st_d, b->st_h, sizeof(SpgDevState) * b->n, cudaMemcpyHostToDevice, s));
    BCU(cudaMemcpyAsync(b->loop_d, b->loop_h, sizeof(BatchLoop), cudaMemcpyHostToDevice, s));
    BCU(cudaMemcpyAsync(b->active_d, b->active_h, sizeof(int) * b->n, cudaMemcpyHostToDevice, s));
    BCU(cudaEventRecord(b->ev0, s));
    BCU(cudaGraphLaunch(g, s));
    BCU(cudaEventRecord(b->ev1, s));
    BCU(cudaMemcpyAsync(b->st_h, b->st_d, sizeof(SpgDevState) * b->n, cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(b->loop_h, b->loop_d, sizeof(BatchLoop), cudaMemcpyDeviceToHost, s));
    BCU(cudaMemcpyAsync(b->outer_h, b->outer_d, sizeof(BatchOuter) * b->n, cudaMemcpyDeviceToHost, s));
    BCU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (elapsed_ms) *elapsed_ms += ms;
    for (int i = 0; i < b->n; i++) b->cur[i] = b->st_h[i].cur;
    b->work_valid = false;  // the device rewrote the work list
    b->launches += b->loop_h->launches;
    if (b->loop_h->error) return bfail(PASC_ERR_TIMEOUT, "batch: a bounded wait for a bulk copy gave up");
    return PASC_OK;
}

// SPG solves of the signals with active_h[i] != 0 (the others stay untouched).
static int batch_spgqp(pasc_gb300_batch *b, const pasc_gb300_spgqp_opts *o, double *elapsed_ms)
{
    if (o->stop_normgp_normb || o->stop_Anormgp_normb)
        return bfail(PASC_ERR_NOTSUPP, "batch: ||b||-scaled stopping tests are not supported");
    if (o->m < 1 || o->m > MMAX_STATE) return bfail(PASC_ERR_ARG, "batch: m must be in [1, 64]");
    if (b->device_loop) {
        BCHK(ensure_spg_loop_graph(b));
        loop_settings(b, o);
        return run_loop_graph(b, b->g_spg, elapsed_ms);
    }
    BCHK(ensure_batch_graph(b));
    cudaStream_t s = b->stream;
    BCU(cudaStreamSynchronize(s));  // the pinned state mirror may still be feeding an upload
    int nact = 0;
    for (int i = 0; i < b->n; i++) {
        SpgDevState &h = b->st_h[i];
        memset(&h, 0, sizeof h);
        h.alpha_prev = h.alpha_cur = o->alphainit;
        h.coeff = b->coeffA[i];
        h.bscale = b->coeffB[i];
        h.eps = o->eps;
        h.gamma = o->gamma;
        h.sigma1 = o->sigma1;
        h.sigma2 = o->sigma2;
        h.maxit = o->maxit;
        h.m = o->m;
        h.stop_difff = o->stop_difff;
        h.stop_normgp = o->stop_normgp;
        h.stop_Anormgp = o->stop_Anormgp;
        h.cur = b->cur[i];
        h.status = b->active_h[i] ? PASC_SPG_RUNNING : IDLE;
        nact += b->active_h[i] ? 1 : 0;
    }
    if (nact == 0) return PASC_OK;
    BatchArgs a = batch_args(b);
    BCHK(update_worklist(b, [&](int i) { return b->active_h[i] != 0; }));
    BCU(cudaEventRecord(b->ev0, s));
    BCU(cudaMemcpyAsync(b->st_d, b->st_h, sizeof(SpgDevState) * b->n, cudaMemcpyHostToDevice, s));
    BCU(cudaMemsetAsync(b->ticket, 0, sizeof(unsigned int) * b->n, s));
    BCU(cudaMemsetAsync(b->next_job, 0, sizeof(unsigned int), s));
    BCU(launch_batch_sweep(b->KB, true, b->grid_init, a, s));
    b->launches++;
    // the states are read after 2, 4, 8 and then every BATCH_CHUNK sweeps (solves that end
    // within a few iterations do not pay for a whole chunk); after each read the work list
    // drops the signals whose solve has ended
    long done = 0;
    int step = 0;
    const int sched[] = {2, 4, 8};
    while (done < o->maxit) {
        const int want = step < 3 ? sched[step] : BATCH_CHUNK;
        step++;
        if (want == BATCH_CHUNK) {
            BCU(cudaGraphLaunch(b->chunk, s));
        } else {
            for (int q = 0; q < want; q++) {
                BCU(cudaMemsetAsync(b->next_job, 0, sizeof(unsigned int), s));
                BCU(launch_batch_sweep(b->KB, false, b->grid, a, s));
            }
        }
        done += want;
        b->launches += want;
        BCU(cudaMemcpyAsync(b->st_h, b->st_d, sizeof(SpgDevState) * b->n, cudaMemcpyDeviceToHost, s));
        BCU(cudaStreamSynchronize(s));
        bool running = false, err = false;
        for (int i = 0; i < b->n; i++) {
            running = running || b->st_h[i].status == PASC_SPG_RUNNING;
            err = err || b->st_h[i].error;
        }
        if (err) return bfail(PASC_ERR_TIMEOUT, "batch: a bounded wait for a bulk copy gave up");
        if (!running) break;
        BCHK(update_worklist(b, [&](int i) { return b->st_h[i].status == PASC_SPG_RUNNING; }));
    }
    BCU(cudaEventRecord(b->ev1, s));
    BCU(cudaMemcpyAsync(b->st_h, b->st_d, sizeof(SpgDevState) * b->n, cudaMemcpyDeviceToHost, s));
    BCU(cudaEventSynchronize(b->ev1));
    BCU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (elapsed_ms) *elapsed_ms += ms;
    for (int i = 0; i < b->n; i++) {
        if (!b->active_h[i]) continue;
        b->cur[i] = b->st_h[i].cur;
        if (b->st_h[i].status == PASC_SPG_RUNNING) b->st_h[i].status = PASC_SPG_MAXIT;
    }
    return PASC_OK;
}

extern "C" {

int pasc_gb300_batch_spgqp_solve(pasc_gb300_batch *b, const pasc_gb300_spgqp_opts *o, pasc_gb300_spgqp_stats *st)
{
    if (!b || !o) return bfail(PASC_ERR_ARG, "batch_spgqp_solve: NULL argument");
    BCU(cudaSetDevice(b->device));
    for (int i = 0; i < b->n; i++) b->active_h[i] = 1;
    double ms = 0.0;
    b->launches = 0;
    BCHK(batch_spgqp(b, o, &ms));
    if (st) {
        for (int i = 0; i < b->n; i++) {
            const SpgDevState &h = b->st_h[i];
            st[i].it = h.it;
            st[i].hessmult = h.hessmult;
            st[i].status = h.status;
            st[i].kernel_launches = b->launches;
            st[i].fx = h.fx;
            st[i].gP = h.dd;
            st[i].dAd = h.dAd;
            st[i].time_s = ms * 1e-3;
        }
    }
    return PASC_OK;
}

// TSSolver::solve (include/general/solver/tssolver.h:492-715) for every signal of the batch at
// once: each signal has its own outer loop (theta step, gamma step, |L - L_old| test); a
// signal that has stopped takes no further part.  No annealing.
int pasc_gb300_batch_ts_solve(pasc_gb300_batch *b, const pasc_gb300_ts_opts *ts, const pasc_gb300_spgqp_opts *spg,
                              pasc_gb300_ts_stats *st)
{
    if (!b || !ts || !spg) return bfail(PASC_ERR_ARG, "batch_ts_solve: NULL argument");
    if (ts->annealing > 1) return bfail(PASC_ERR_NOTSUPP, "batch_ts_solve: annealing is not supported");
    BCU(cudaSetDevice(b->device));
    auto t0 = std::chrono::steady_clock::now();
    const int n = b->n;
    if (b->device_loop) {
        if (spg->stop_normgp_normb || spg->stop_Anormgp_normb)
            return bfail(PASC_ERR_NOTSUPP, "batch: ||b||-scaled stopping tests are not supported");
        if (spg->m < 1 || spg->m > MMAX_STATE) return bfail(PASC_ERR_ARG, "batch: m must be in [1, 64]");
            BCHK(ensure_ts_loop_graph(b, ts->thetasolved ? 1 : 0));
        b->launches = 0;
        if (ts->init_permute) BCHK(batch_permute(b));
        loop_settings(b, spg);
        b->loop_h->ts_maxit = ts->maxit;
        b->loop_h->ts_eps = ts->eps;
        b->loop_h->ts_relative = ts->relative;
        for (int i = 0; i < n; i++) b->active_h[i] = 1;
        if (ts->maxit > 0) BCHK(run_loop_graph(b, b->g_ts[ts->thetasolved ? 1 : 0], nullptr));
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (st) {
            for (int i = 0; i < n; i++) {
                const BatchOuter &o = b->outer_h[i];
                const bool ran = ts->maxit > 0;
                st[i].it_last = ran ? o.it_last : 0;
                st[i].it_sum = st[i].it_last;
                st[i].spg_it_sum = ran ? o.spg_it : 0;
                st[i].spg_hessmult_sum = ran ? o.spg_hm : 0;
                st[i].kernel_launches = b->launches;
                st[i].L_increased = ran ? o.incr : 0;
                st[i].L = ran ? o.L : DBL_MAX;
                st[i].deltaL = ran ? o.dL : DBL_MAX;
                st[i].aic = 2 * log(st[i].L) + b->K[i];
                st[i].time_s = secs;
            }
        }
        return PASC_OK;
    }
    std::vector<double> L(n, DBL_MAX), dL(n, DBL_MAX);
    std::vector<int> done(n, 0), it_last(n, 0), spg_it(n, 0), spg_hm(n, 0), incr(n, 0);
    b->launches = 0;
    if (ts->init_permute) BCHK(batch_permute(b));
    BatchArgs a = batch_args(b);
    for (int it = 0; it < ts->maxit; it++) {
        int nact = 0;
        for (int i = 0; i < n; i++) {
            b->active_h[i] = !done[i];
            nact += b->active_h[i];
        }
        if (nact == 0) break;
        if (!ts->thetasolved) {
            // the theta kernel reads each signal's buffer index from its state
            for (int i = 0; i < n; i++) b->st_h[i].cur = b->cur[i];
            BCU(cudaMemcpyAsync(b->st_d, b->st_h, sizeof(SpgDevState) * n, cudaMemcpyHostToDevice, b->stream));
            BCU(cudaMemcpyAsync(b->active_d, b->active_h, sizeof(int) * n, cudaMemcpyHostToDevice, b->stream));
            BCHK(update_worklist(b, [&](int i) { return b->active_h[i] != 0; }));
            BCU(cudaMemsetAsync(b->ticket, 0, sizeof(unsigned int) * n, b->stream));
            BCU(cudaMemsetAsync(b->next_job, 0, sizeof(unsigned int), b->stream));
            BCU(launch_theta_batch(b->grid_theta, a, b->stream));
            b->launches++;
        }
        BCHK(batch_spgqp(b, spg, nullptr));
        for (int i = 0; i < n; i++) {
            if (done[i]) continue;
            const SpgDevState &h = b->st_h[i];
            spg_it[i] += h.it;
            spg_hm[i] += h.hessmult;
            const double L_old = L[i];
            L[i] = h.fx;
            dL[i] = fabs(L[i] - L_old);
            if (L[i] - L_old > 0) incr[i]++;
            it_last[i] = it;
            if (ts->relative ? (dL[i] < ts->eps * fabs(L[i])) : (dL[i] < ts->eps)) done[i] = 1;
            else if (it == ts->maxit - 1) it_last[i] = ts->maxit;
        }
    }
    BCU(cudaStreamSynchronize(b->stream));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) {
        for (int i = 0; i < n; i++) {
            st[i].it_last = it_last[i];
            st[i].it_sum = it_last[i];
            st[i].spg_it_sum = spg_it[i];
            st[i].spg_hessmult_sum = spg_hm[i];
            st[i].kernel_launches = b->launches;
            st[i].L_increased = incr[i];
            st[i].L = L[i];
            st[i].deltaL = dL[i];
            st[i].aic = 2 * log(L[i]) + b->K[i];
            st[i].time_s = secs;
        }
    }
    return PASC_OK;
}

}  // extern "C"
