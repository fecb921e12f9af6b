// internal.h -- types shared by the library's translation units (not part of the ABI).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pasc_gb300.h"

namespace pasc {

constexpr int MMAX_STATE = 64;

// Device-resident state of one mixed-precision SPG solve.  The last block of every sweep
// reads the block partial sums, applies the reference's step-length rules
// (src/petscvector/solver/spgqpsolver.cpp:176-216) and writes the scalars the next sweep uses.
// All scalar arithmetic is FP64.
struct SpgDevState {
    // step lengths of the pending iterations
    double alpha_prev;  // alpha used by the direction being applied (recomputed in the sweep)
    double beta;        // beta of the direction being applied
    double alpha_cur;   // alpha of the next direction
    // objective and the dots of the last direction
    double fx, fx_old;
    double dd, dAd, gd;
    double normb;       // ||b|| (stopping variants scaled by ||b||)
    // problem and settings (copied in by the host before every solve)
    double coeff;       // A = coeff * A_hat
    double bscale;      // b = bscale * residual
    int coeffmode;      // SPGQPSolverC: coefficient factored out of the step rules (dAd, dd/dAd unscaled)
    double eps, gamma, sigma1, sigma2;
    int maxit, m;
    int stop_difff, stop_normgp, stop_normgp_normb, stop_Anormgp, stop_Anormgp_normb;
    // GLL ring (src/general/solver/spg_fs.cpp)
    double fs[MMAX_STATE];
    int fs_last;
    // progress
    int it;             // completed iterations
    int hessmult;
    int status;         // pasc_gb300_solve_status
    int cur;            // buffer (0/1) holding the current x and g
    int sweeps;         // sweeps that did work
    unsigned int counter;  // last-block-done ticket (reset by the last block)
    unsigned int counter2; // ticket of the theta kernel
    int error;             // set when a bounded device wait gave up
};

struct SweepArgs {
    const float *bmat;  // T*K: b materialised (multichannel data); null: b formed from data, theta
    const float *data;  // T (xdim == 1)
    const float *theta; // K
    float *xb0, *xb1;   // ping-pong pair holding x (gamma); buffer st->cur is current
    double *partials;   // gridDim.x * 4
    SpgDevState *st;
    long T;
    // theta in the penalty (GraphH1FEMModel with usethetainpenalty): block k of A is
    // coeff * kw[k] * A_hat with kw[k] = theta_k^2; null: every block is coeff * A_hat
    const float *kw = nullptr;
    // bulk-copy sweep with 16 values per thread (K = 4, 8): tensor maps of the two gamma
    // buffers and of the materialised b as rows of 16 floats from the start of their front
    // pads (swz != 0: the tiles come in with the 64-byte swizzle, sweep_tma.cuh), and the row
    // of timestep 0
    CUtensorMap tm_x[2], tm_b;
    int swz = 0, roff = 0;
};

// Graph (R > 1) mode, mixed path (graph.cu): x and d ping-pong, buffer st->cur current.
struct GraphSweepArgs {
    const float *data;        // T*R
    const float *theta;       // K
    float *xb0, *xb1;         // gamma
    float *db0, *db1;         // direction d of the current gamma
    double *partials;         // gridDim.x * 4
    SpgDevState *st;
    const int *ptr, *idx;     // neighbour lists (CSR over R nodes, sorted, symmetric)
    long T, R;
};

// Image mode (T = 1 on the W x H pixel grid), mixed path: the fused tile sweep (image.cu).
struct ImageSweepArgs {
    const float *data;        // W*H, row-major
    const float *theta;       // K
    float *xb0, *xb1;         // gamma, ping-pong (buffer st->cur current)
    double *partials;         // gridDim.x * 4
    SpgDevState *st;
    int W, H;
};

struct ThetaArgs {
    const float *data;
    const float *xb0, *xb1;  // gamma lives in buffer st->cur
    double *partials;         // gridDim.x * 2K
    double *theta64;
    float *theta32;
    SpgDevState *st;          // counter2 is the last-block ticket
    long T;
    int cur;                  // buffer holding gamma
    // theta in the penalty: theta_k = g'x / (sum g + g'(pen_alpha A_hat)g / 2) when tp
    double pen_alpha = 0.0;
    int tp = 0;
};

// One signal of a batch (device copy).
struct BatchInstDev {
    long xoff;       // gamma of t = 0 in the packed gamma buffers (floats)
    long doff;       // data of t = 0 in the packed data buffer
    int T, K;
    int seg0, nseg;  // its segments in the work list
    int tiles;       // bulk-copy tiles covering it
    int pad;
    float theta[8];
};

struct BatchArgs {
    BatchInstDev *inst;
    const int *seg_inst;     // segment -> signal
    const int *work;         // segments to visit in this launch (those of signals still taking part)
    const int *nwork;        // length of work and segments per item (device memory: rewritten
                             // between captured launches)
    int nseg, ninst;
    float *xb0, *xb1;        // packed gamma, ping-pong (each signal's half given by its state's cur)
    const float *data;       // packed data
    SpgDevState *st;         // one per signal
    double *partials;        // 16 per segment
    unsigned int *ticket;    // one per signal
    unsigned int *next_job;  // work-list counter (zeroed before every launch)
    const int *active;       // theta step: signals still in their outer loop
    double *theta64;         // 8 per signal
    const int *order;        // signals by decreasing T: the order of the work lists
    int seg_tiles;           // bulk-copy tiles per segment
    int merge_target;        // work items wanted per list (0: one segment per item)
    int merge_max;           // most segments in one work item
};

// Segments per work item of a list over s segments: about `target` items, between 1 and mmax
// segments each (target 0: 1).  nwork[1] holds it for the list in use; the work list names
// the first segment of every item, and an item never crosses into the next signal.
__host__ __device__ inline int batch_merge(int s, int target, int mmax)
{
    if (target <= 0) return 1;
    const int m = s / target;
    return m < 1 ? 1 : (m > mmax ? mmax : m);
}

// Multichannel data (kernels_mc.cu).
struct McArgs {
    long T;
    int n;                          // channels (xdim)
    const unsigned short *xbf;      // T*n BF16, row-major
    const float *xnorm;             // T: ||X_t||^2 of the BF16 values
    float *bmat;                    // T*K: b_tk = bscale ||X_t - theta_k||^2
    unsigned short *theta_split;    // 32*n BF16: rows k, K+k, 2K+k = three parts of theta_k
    float *theta_f32;               // K*n
    float *tnorm;                   // K: ||theta_k||^2
    double *theta64;                // K*n
    double *partials;               // theta-update partial sums
    float bscale;
    int *err;                       // set by a bounded wait that gave up
    int theta_tma_grid;             // blocks of the bulk-copy theta kernel (0: not used)
};
cudaError_t launch_mc_convert(const double *x64, unsigned short *xbf, float *xnorm, long T, int n, cudaStream_t s);
int mc_tc_supported(int n);
cudaError_t mc_make_tmap(CUtensorMap *map, const unsigned short *xbf, long T, int n);
cudaError_t prepare_mc_residual_tc(int K, int n);
cudaError_t launch_mc_residual_tc(const CUtensorMap &map, int K, int n, int grid, const McArgs &a, cudaStream_t s);
cudaError_t launch_mc_residual_simt(int K, int grid, const McArgs &a, cudaStream_t s);
// gamma != null: theta from gamma (partial kernel on `grid` blocks + per-cluster finish);
// gamma == null: only the preparation of the current theta64 (split, FP32 copy, norms)
cudaError_t launch_mc_theta(int K, int grid, const McArgs &a, const float *gamma, cudaStream_t s);
size_t mc_partials_size(int K, int n, int grid, long T);
int mc_theta_tma_blocks_per_sm(int K, int n);  // 0: the bulk-copy theta kernel does not apply

// FEM temporal coarsening (fem.cu).  launch_fem_reduce: g1 == null reduces the residual
// (data_t - theta_k)^2 instead of a stored field; the result is multiplied by scale.
long fem_T_reduced(long T, double fem_reduce);
template <typename TIn, typename TOut>
cudaError_t launch_fem_reduce(const TIn *g1, const double *data, const double *theta, TOut *g2, long T1, long T2,
                              int K, int type, double scale, cudaStream_t s);
template <typename TIn, typename TOut>
cudaError_t launch_fem_prolongate(const TIn *g2, TOut *g1, long T1, long T2, int K, int type, cudaStream_t s);

// Graph (R > 1) and image mode (graph.cu).
const char *graph_check(long R, const int *ptr, const int *idx);  // null: valid
int graph_sweep_grid(long nblocks);
cudaError_t launch_graph_sweep(int K, bool init, int grid, const GraphSweepArgs &a, cudaStream_t s);
cudaError_t launch_graph_matmult_f64(const double *x, double *y, long T, long R, int K, double coeff,
                                     const int *ptr, const int *idx, cudaStream_t s, const double *kc = nullptr);

bool graph_is_grid2d(long R, const int *ptr, const int *idx, int *W, int *H);  // host check
int image_sweep_blocks_per_sm(int K);  // also sets the kernels' shared-memory limit
int image_sweep_tiles(int W, int H);
cudaError_t launch_image_sweep(int K, bool init, int grid, const ImageSweepArgs &a, cudaStream_t s);

int batch_tile_width();
int batch_max_tile();
int batch_blocks_per_sm(int KB, bool init);
cudaError_t launch_batch_sweep(int KB, bool init, int grid, const BatchArgs &a, cudaStream_t s);
cudaError_t launch_theta_batch(int grid, const BatchArgs &a, cudaStream_t s);

// Sets the message pasc_gb300_last_error() returns on the calling thread.
void record_error(const char *msg);

// Launchers (kernels_fused.cu).  Return a cudaError_t.
int sweep_tile_width();
int sweep_blocks_per_sm(int K, bool init, bool tp = false);  // tp: the theta-in-penalty form
cudaError_t launch_sweep(int K, bool init, int grid, const SweepArgs &a, cudaStream_t s);  // a.bmat selects the b source
// Bulk-copy (TMA) form of the sweep: 4 timesteps per thread, double-buffered tiles.
bool sweep_tma_supported(int K);
int sweep_tma_tile_width();
// bmat: the materialised-b form; tp: the theta-in-penalty form (SweepArgs::kw set)
int sweep_tma_blocks_per_sm(int K, bool init, bool bmat = false, bool tp = false);
// tensor map over n floats at base (16-byte aligned, n a multiple of 16) as rows of 16 floats,
// box 16 x rows_per_box, 64-byte swizzle
cudaError_t sweep_tma_make_rowmap(CUtensorMap *map, const float *base, long n, int rows_per_box);
// threads per block of the bulk-copy sweep for K (its tile rows), and whether it reads 16
// values per thread (the swizzled form applies)
int sweep_tma_threads(int K);
bool sweep_tma_rows16(int K);
cudaError_t launch_sweep_tma(int K, bool init, int grid, const SweepArgs &a, cudaStream_t s);
cudaError_t launch_theta_f32(int K, int grid, const ThetaArgs &a, cudaStream_t s);
cudaError_t launch_project_f32(float *x, long T, int K, cudaStream_t s);
cudaError_t launch_matmult_f32(const float *x, float *y, long T, int K, float coeff, cudaStream_t s);
cudaError_t launch_f64_to_f32(const double *src, float *dst, long n, cudaStream_t s);
cudaError_t launch_f32_to_f64(const float *src, double *dst, long n, cudaStream_t s);

// Plain FP64 kernels (kernels_plain.cu).
cudaError_t launch_project_f64(double *x, long T, int K, cudaStream_t s);
// kc != null: block k scaled by kc[k] (device memory) instead of coeff
cudaError_t launch_matmult_f64(const double *x, double *y, long T, int K, double coeff, cudaStream_t s,
                               const double *kc = nullptr);
cudaError_t launch_axpy_f64(double *y, double a, const double *x, long n, cudaStream_t s);
cudaError_t launch_xmay_f64(double *d, const double *x, double a, const double *g, long n, cudaStream_t s);
cudaError_t launch_residual_f64(const double *data, const double *theta, double *b, long T, int K,
                                double bscale, cudaStream_t s);
// blocked k*R*Tt + r*Tt + t -> interleaved (t*R + r)*K + k over T = Tt*R blocks (R = 1: k*T + t)
cudaError_t launch_permute_f64(const double *src, double *dst, long T, int K, cudaStream_t s, long R = 1);
cudaError_t launch_permute_f32(const float *src, float *dst, long T, int K, cudaStream_t s, long R = 1);
// Deterministic dot products: out[q] = sum_i a_q[i] * b_q[i] for q < nq (nq <= 3); a scratch
// of dot_partials_size() doubles.  fxmode: out[0] = sum_i x_i * (g_i - b_i) (get_fx).
size_t dot_partials_size();
cudaError_t launch_dots_f64(int nq, const double *a0, const double *b0, const double *a1,
                            const double *b1, const double *a2, const double *b2, long n,
                            double *scratch, double *out, cudaStream_t s);
cudaError_t launch_fx_f64(const double *x, const double *g, const double *b, long n,
                          double *scratch, double *out, cudaStream_t s);
// tp: theta in the penalty, theta_k = g'x / (sum g + g'(pen_alpha A_hat)g / 2)
cudaError_t launch_theta_f64(const double *gamma, const double *data, double *theta, long T, int K,
                             double *scratch, cudaStream_t s, bool tp = false, double pen_alpha = 0.0);
// block coefficients of theta in the penalty from theta64: ck64[k] = (coeff theta_k) theta_k,
// kw32[k] = theta_k^2 in FP32
cudaError_t launch_tp_coeffs(const double *theta64, double coeff, int K, double *ck64, float *kw32, cudaStream_t s);
cudaError_t launch_recon_abserr(const double *gamma, const double *theta, const double *sol,
                                long T, int K, double *scratch, double *out, cudaStream_t s);
cudaError_t launch_argmax(const double *gamma, int *labels, long T, int K, cudaStream_t s);

}  // namespace pasc
