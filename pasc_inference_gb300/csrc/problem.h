// problem.h -- the problem handle behind the C ABI (shared by problem.cu and adjoint.cu; not
// part of the ABI).
#pragma once

#include <float.h>

#include "internal.h"

namespace pasc {
struct AdjointWork;  // adjoint.cu
void adjoint_free(AdjointWork *w);
}  // namespace pasc

// Host-side record of the current SPG solve (both paths; the fp64 path keeps its whole
// scalar state here, the mixed path mirrors the device state after every poll).
namespace pasc {
struct SpgRun {
    pasc_gb300_spgqp_opts o{};
    bool started = false;
    int it = 0, hessmult = 0, status = PASC_SPG_RUNNING, launches = 0;
    double fx = 0.0, fx_old = DBL_MAX, dd = 0.0, dAd = 0.0, normb = 0.0, alpha = 0.0;
    double fs[MMAX_STATE] = {0};
    int fs_last = 0;
    double time_s = 0.0;
    float last_iterate_ms = 0.f;
    int last_iterate_launches = 0;
};
}  // namespace pasc

struct pasc_gb300_problem {
    long T = 0;
    int K = 0, xdim = 1, precision = 0, device = 0;
    double epssqr = 0.0;
    int scalef = 1;
    double coeffA = 0.0, coeffB = 0.0;
    long N = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // shared
    double *data64 = nullptr;     // T (fp64 path; mixed path uses it as upload staging)
    double *theta64 = nullptr;    // K*xdim
    double *stage64 = nullptr;    // N (mixed: conversions; fp64: permutation temp)
    float *stage32 = nullptr;     // T*xdim, only where FP32 host data does not fit in stage64
    double *red = nullptr;        // reduction scratch (dot_partials_size doubles)
    double *red_out = nullptr;    // 8 doubles
    double *red_out_h = nullptr;  // pinned mirror
    int *labels_d = nullptr;      // T

    // fp64 path
    double *x = nullptr, *g = nullptr, *d = nullptr, *Ad = nullptr, *b = nullptr;

    // mixed path
    float *data32 = nullptr, *theta32 = nullptr;  // data32 points past the front pad
    float *xb[2] = {nullptr, nullptr};            // past the front pad of xb_raw
    float *xb_raw[2] = {nullptr, nullptr}, *data32_raw = nullptr;
    pasc::SpgDevState *st = nullptr, *st_h = nullptr;
    double *partials = nullptr;
    int cur = 0;
    // sweep kernels: 0 = one timestep per thread, 1 = bulk-copy tiles, 4 timesteps per thread
    int grid_sweep[2] = {0, 0}, grid_sweep_init[2] = {0, 0}, grid_theta = 0;
    int grid_sweep_max[2] = {0, 0};  // the grids the partials buffer was sized for (occupancy)
    int variant = -1;             // -1: kernel and grid chosen by timing at the first solve
    float tune_ms = 0.f;          // the chosen configuration's sweep time in the tuning runs
    cudaGraphExec_t chunk_graph = nullptr;
    int chunk_graph_len = 0, chunk_graph_variant = -1;

    // multichannel data (xdim > 1, mixed path): X in BF16, b materialised once per outer
    // iteration by the residual kernel (kernels_mc.cu)
    unsigned short *xbf = nullptr;         // T*xdim
    float *xnorm = nullptr;                // T
    float *bmat = nullptr;                 // T*K, past the front pad of bmat_raw
    float *bmat_raw = nullptr;             // zero pads as the gamma buffers (bulk-copy tiles)
    // tensor maps of xb_raw[0], xb_raw[1] and bmat_raw for the swizzled bulk-copy sweep (K = 4,
    // 8), built for the buffers in tm_base
    CUtensorMap tm_x[2], tm_b;
    const float *tm_base[3] = {nullptr, nullptr, nullptr};
    bool tm_ok = false;
    unsigned short *theta_split = nullptr; // 32*xdim
    float *theta_f32 = nullptr;            // K*xdim
    float *tnorm = nullptr;                // K
    double *mc_partials = nullptr;
    int *mc_err = nullptr;
    int mc_grid_theta = 0, mc_grid_res = 0;
    int mc_grid_theta_tma = 0;             // blocks of the bulk-copy theta kernel (0: not used)
    int mc_engine = 0;                     // residual: 0 tensor cores (when xdim allows), 1 CUDA cores
    CUtensorMap mc_tmap;

    // FEM temporal coarsening (pasc_gb300_set_fem): with fem_reduce < 1 the gamma QP runs on the
    // inner handle (T2 timesteps, b written here); this handle keeps the full data, gamma, theta
    double fem_reduce = 1.0;
    int fem_type = 0;
    pasc_gb300_problem *fem_inner = nullptr;
    bool b_external = false;               // inner handle: b is written by the owner

    // graph (R > 1) / image mode (pasc_gb300_create_graph): T above counts the T*R blocks of K;
    // graph_T is the number of timesteps (it scales A and b), graph_R the number of nodes
    bool graph = false;
    long graph_T = 0, graph_R = 1, graph_nnz = 0;
    int *gptr = nullptr, *gidx = nullptr;  // device CSR
    float *db_raw[2] = {nullptr, nullptr}; // mixed path: direction ping-pong
    double *gpartials = nullptr;
    int grid_graph = 0;
    int img_W = 0, img_H = 0, grid_image = 0;  // T = 1 on a pixel grid: the fused image sweep

    // gamma solver: 1 = SPGQPSolver, 2 = SPGQPSolverC (coefficient factored out)
    int solver_type = 1;

    // theta in the penalty (pasc_gb300_set_usethetainpenalty): block k of A is
    // coeffA * theta_k^2 * A_hat; ck64[k] = (coeffA theta_k) theta_k, kw32[k] = theta_k^2
    bool tp = false;
    double *tp_ck64 = nullptr;
    float *tp_kw32 = nullptr;
    int grid_sweep_tp[2] = {0, 0}, grid_sweep_init_tp[2] = {0, 0}, grid_sweep_tp_max[2] = {0, 0};

    pasc::SpgRun run;
    pasc::AdjointWork *adj = nullptr;  // allocated by the first adjoint call
    double fx_last = 0.0;
    bool have_fx = false;
    bool have_data = false;
};
