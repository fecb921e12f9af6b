/*
 * pasc_gb300.h -- C ABI of the GB300 (sm_103a) FEM-H1 clustering library.
 *
 * This is the drop-in boundary for PASC_inference's FEM-H1 time-series clustering hot
 * path: the gamma-step QP solved by SPGQPSolver inside the alternating TSSolver loop.  Each
 * entry point names the reference interface it replaces (paths relative to the
 * PASC_inference tree).  The C++ class surface in include/pasc/ and the ctypes binding in
 * pasc_inference_gb300/ are thin layers over these functions.
 *
 * Conventions
 *   - Every function returns an int status: PASC_OK (0) or a pasc_gb300_error code.  No C++
 *     exception crosses the ABI; pasc_gb300_last_error() gives the message of the last
 *     failure on the calling thread.  (The reference prints through TRYCXX/PetscError and
 *     continues, include/external/petscvector/algebra/vector/petscvector.h:51, or exits
 *     through gpuErrchk, include/external/petscvector/petscvector.cuh:12-20.)
 *   - Host buffers are caller-owned; device buffers behind a handle are library-owned.
 *     Entry points whose pointers are device pointers say so.  `stream` arguments are
 *     cudaStream_t values passed as void* (NULL = the legacy default stream).
 *   - Layouts follow the reference decomposition with R = 1 on one device:
 *       gamma  N = K*T values, interleaved, index t*K + k
 *              (src/petscvector/algebra/matrix/blockgraphsparse.cpp:54)
 *       data   T*xdim values, index t*xdim + j
 *       theta  K*xdim values, index k*xdim + j (src/petscvector/model/graphh1fem.cpp:94)
 *   - One handle = one problem on one device with its own CUDA stream.  Calls on one handle
 *     must not overlap; different handles may be used from different threads.
 */
#ifndef PASC_GB300_H
#define PASC_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define PASC_GB300_ABI_VERSION 1

/* ---------------------------------------------------------------------------------------
 * status codes
 * ------------------------------------------------------------------------------------- */
enum pasc_gb300_error {
    PASC_OK = 0,
    PASC_ERR_ARG = 1,       /* invalid argument (sizes, null pointers, K out of range) */
    PASC_ERR_CUDA = 2,      /* a CUDA runtime call failed */
    PASC_ERR_ALLOC = 3,     /* device or host allocation failed */
    PASC_ERR_STATE = 4,     /* call not valid in the handle's current state */
    PASC_ERR_NOTSUPP = 5,   /* configuration not supported by the library */
    PASC_ERR_TIMEOUT = 6    /* a bounded device wait gave up */
};

/* Solve outcome reported in pasc_gb300_spgqp_stats.status. */
enum pasc_gb300_solve_status {
    PASC_SPG_RUNNING = 0,
    PASC_SPG_CONVERGED = 1, /* a stopping test of spgqpsolver.cpp:260-274 was met */
    PASC_SPG_MAXIT = 2,     /* maxit iterations done */
    PASC_SPG_DAD_ZERO = 3,  /* d'Ad <= 0: the projected step vanished (the reference divides
                               by it unguarded, spgqpsolver.cpp:182-183); x is kept */
    PASC_SPG_NONFINITE = 4  /* a reduction came out NaN/Inf; x is kept at the last finite iterate */
};

/* Arithmetic of a handle. */
enum pasc_gb300_precision {
    PASC_PREC_FP64 = 0,     /* plain path: FP64 state, one kernel per reference operation,
                               host-side step-length scalars (the reference's structure) */
    PASC_PREC_MIXED = 1     /* fused path: FP32 gamma/gradient state, one HBM sweep per SPG
                               iteration, FP64 reductions and step lengths on the device */
};

/* ---------------------------------------------------------------------------------------
 * settings -- field names follow the reference's console options
 * ------------------------------------------------------------------------------------- */

/* SPGQPSolver settings: include/general/solver/spgqpsolver.h:19-36,162-202. */
typedef struct {
    int maxit;              /* spgqpsolver_maxit (1000) */
    double eps;             /* spgqpsolver_eps (1e-9) */
    int m;                  /* spgqpsolver_m: GLL memory (20), 1..64 */
    double gamma;           /* spgqpsolver_gamma (0.9) */
    double sigma1;          /* spgqpsolver_sigma1 (0) */
    double sigma2;          /* spgqpsolver_sigma2 (1) */
    double alphainit;       /* spgqpsolver_alphainit (2) */
    int stop_difff;         /* |f - f_old| < eps (on) */
    int stop_normgp;        /* ||d||^2 < eps */
    int stop_normgp_normb;  /* ||d||^2 < eps*||b|| */
    int stop_Anormgp;       /* d'Ad < eps */
    int stop_Anormgp_normb; /* d'Ad < eps*||b|| */
} pasc_gb300_spgqp_opts;

/* SPGQPSolver results (it_last, hessmult_last, fx, gP of the reference). */
typedef struct {
    int it;                 /* iterations of this solve */
    int hessmult;           /* Hessian products of this solve (1 + it, as the reference counts) */
    int status;             /* pasc_gb300_solve_status */
    int kernel_launches;    /* kernels launched by this solve */
    double fx;              /* final objective 1/2 x'Ax - b'x */
    double gP;              /* last ||d||^2 */
    double dAd;             /* last d'Ad */
    double time_s;          /* device time of the solve (CUDA events) */
} pasc_gb300_spgqp_stats;

/* TSSolver settings: include/general/solver/tssolver.h:13-15,117-162. */
typedef struct {
    int maxit;              /* tssolver_maxit (300) */
    double eps;             /* tssolver_eps (1e-6) */
    int init_permute;       /* tssolver_init_permute (1): blocked -> interleaved permutation of
                               gamma at the start of every annealing run, tssolver.h:528-530 */
    int annealing;          /* restarts (1) */
    int relative;           /* 0: stop on |L - L_old| < eps (reference, tssolver.h:642);
                               1: stop on |L - L_old| < eps*|L| */
    int thetasolved;        /* 1: theta was given (TSSolver::set_solution_theta), skip theta */
} pasc_gb300_ts_opts;

typedef struct {
    int it_last;            /* outer iterations of the kept run */
    int it_sum;             /* outer iterations over all runs */
    int spg_it_sum;         /* SPG iterations over the whole solve */
    int spg_hessmult_sum;
    int kernel_launches;
    int L_increased;        /* outer steps where L grew (the reference prints "ERROR") */
    double L;               /* final objective (gamma solver fx) */
    double deltaL;          /* last |L - L_old| */
    double aic;             /* 2 log L + K (include/general/model/graphh1fem.h:444-447) */
    double time_s;          /* wall time of the solve */
} pasc_gb300_ts_stats;

void pasc_gb300_spgqp_default_opts(pasc_gb300_spgqp_opts *o);
void pasc_gb300_ts_default_opts(pasc_gb300_ts_opts *o);

/* ---------------------------------------------------------------------------------------
 * library
 * ------------------------------------------------------------------------------------- */
int pasc_gb300_abi_version(void);
/* Message of the last failed call on this thread ("" if none). */
const char *pasc_gb300_last_error(void);
/* Number of CUDA devices visible (0 on a machine without a GPU; never fails). */
int pasc_gb300_device_count(void);

/* ---------------------------------------------------------------------------------------
 * problem handle: TSData + GraphH1FEMModel + SPGQPSolver + TSSolver state on one device.
 * Replaces the objects the driver builds in examples/test_signal1D/test_signal1D.cpp:188-249
 * (Decomposition(T,1,K,xdim,1), TSData::set_model, GraphH1FEMModel(tsdata, epssqr),
 * TSSolver(tsdata)).
 * ------------------------------------------------------------------------------------- */
typedef struct pasc_gb300_problem pasc_gb300_problem;

/* Multichannel data (xdim = n > 1, each X_t in R^n; b_tk = bscale ||X_t - theta_k||^2 and
 * theta_k = sum_t gamma_tk X_t / sum_t gamma_tk, the extension of the scalar model whose theta
 * the reference already sizes K*xdim, graphh1fem.cpp:23): mixed path only, K <= 8, n <= 256;
 * X is held on the device in BF16 (rounded to nearest) and b is formed once per update_b /
 * outer iteration. */
/* T >= 1, 1 <= K <= 32 (mixed) or <= 128 (fp64), xdim >= 1.  epssqr as in
 * GraphH1FEMModel(tsdata, epssqr) (src/petscvector/model/graphh1fem.cpp:8-65). */
int pasc_gb300_create(pasc_gb300_problem **out, long T, int K, int xdim, int precision,
                      double epssqr, int device);
int pasc_gb300_destroy(pasc_gb300_problem *p);

/* GraphH1FEMModel::set_epssqr (include/general/model/graphh1fem.h:287-306).  scalef as the
 * graphh1femmodel_scalef option (default 1: A = epssqr/T * A_hat, b = -residual/T). */
int pasc_gb300_set_epssqr(pasc_gb300_problem *p, double epssqr, int scalef);

/* TSData vectors (host buffers, FP64).  set_data replaces Signal1DData loading + permute
 * (src/petscvector/data/signal1Ddata.cpp:8-52); set_gamma replaces set_random/load_gammavector
 * (src/petscvector/data/tsdata.cpp:549-627); set_theta replaces TSSolver::set_solution_theta
 * values (include/general/solver/tssolver.h:778-790). */
int pasc_gb300_set_data(pasc_gb300_problem *p, const double *data);
int pasc_gb300_set_gamma(pasc_gb300_problem *p, const double *gamma);
int pasc_gb300_get_gamma(pasc_gb300_problem *p, double *gamma);
int pasc_gb300_set_theta(pasc_gb300_problem *p, const double *theta);
int pasc_gb300_get_theta(pasc_gb300_problem *p, double *theta);

/* The same vectors in FP32 host buffers (data T*xdim values, gamma N values, same layouts).
 * The mixed path keeps data and gamma in FP32 on the device, so these calls move half the
 * bytes of their FP64 forms and convert nothing on the way (the fp64 path widens or narrows on
 * the device).  No counterpart in the reference, whose vectors are FP64 PETSc Vecs; a caller
 * that holds FP64 arrays uses the calls above. */
int pasc_gb300_set_data_f32(pasc_gb300_problem *p, const float *data);
int pasc_gb300_set_gamma_f32(pasc_gb300_problem *p, const float *gamma);
int pasc_gb300_get_gamma_f32(pasc_gb300_problem *p, float *gamma);

/* Page-locked host memory (cudaHostAlloc, portable to every device) for the host buffers of
 * this ABI: copies from and to it run at the host link's full rate and need no staging
 * through the driver's bounce buffers.  The replacement for the host arrays PETSc's VecCreate
 * allocates (src/petscvector/common/decomposition.cpp:200-245 creates the reference's
 * vectors); free with pasc_gb300_host_free.  *ptr is NULL after a failure. */
int pasc_gb300_host_alloc(void **ptr, unsigned long bytes);
int pasc_gb300_host_free(void *ptr);

/* TSSolver::gammavector_permute (include/general/solver/tssolver.h:760-775 ->
 * src/petscvector/common/decomposition.cpp:266-356): blocked k*T+t -> interleaved t*K+k. */
int pasc_gb300_permute_gamma(pasc_gb300_problem *p);

/* GraphH1FEMModel::updatebeforesolve_thetasolver (src/petscvector/model/graphh1fem.cpp:306-396,
 * usethetainpenalty = false): theta_k = sum_t gamma_tk x_t / sum_t gamma_tk. */
int pasc_gb300_update_theta(pasc_gb300_problem *p);

/* GraphH1FEMModel::updatebeforesolve_gammasolver (graphh1fem.cpp:237-289):
 * b_tk = -(x_t - theta_k)^2 / T.  The mixed path forms b inside its sweep from data and
 * theta; this call only refreshes the theta it reads.  The fp64 path materialises b. */
int pasc_gb300_update_b(pasc_gb300_problem *p);

/* SPGQPSolver<PetscVector>::solve (src/petscvector/solver/spgqpsolver.cpp:55-312) on the
 * current gamma (warm start, spgqpsolver.cpp:110-113) and the current b. */
int pasc_gb300_spgqp_solve(pasc_gb300_problem *p, const pasc_gb300_spgqp_opts *o,
                           pasc_gb300_spgqp_stats *st);

/* The two halves of SPGQPSolver::solve, for callers that drive the iteration themselves
 * (and for timing a fixed number of iterations).  spgqp_start runs the set-up of
 * spgqpsolver.cpp:104-137 (||b||, projection of the start point, gradient, objective, GLL
 * memory); spgqp_iterate runs up to n iterations of the main loop :140-297, stopping early on
 * a stopping test or at maxit.  poll = 1 reads the device status between chunks of
 * iterations and stops launching once the solve has ended; poll = 0 (mixed path) launches n
 * iterations back to back with no host synchronisation.  st receives totals since the start.
 * spgqp_solve == spgqp_start + spgqp_iterate(maxit, poll = 1). */
int pasc_gb300_spgqp_start(pasc_gb300_problem *p, const pasc_gb300_spgqp_opts *o);
int pasc_gb300_spgqp_iterate(pasc_gb300_problem *p, long n, int poll, pasc_gb300_spgqp_stats *st);
/* Device time (CUDA events on the problem's stream) and kernel launches of the last
 * spgqp_iterate call. */
int pasc_gb300_spgqp_last_iterate(pasc_gb300_problem *p, double *ms, int *launches);

/* Sweep kernel of the mixed path (no reference counterpart: the reference has one SpMV and
 * separate vector kernels).  0 = one timestep per thread; 1 = tiles of 4 timesteps per
 * thread brought in by bulk asynchronous copies; -1 (default) = whichever is faster on the
 * first solve, measured on the solve's own first sweep. */
int pasc_gb300_set_sweep_variant(pasc_gb300_problem *p, int variant);
int pasc_gb300_get_sweep_variant(pasc_gb300_problem *p, int *variant);
/* The sweep configuration in use: kernel (-1 before the first solve), blocks of its grid,
 * and the sweep time (ms) the tuner measured for it (0 when pinned or taken from an earlier
 * problem of the same shape).  With variant -1 the first solve times both kernels at every
 * grid of 1, 2, ... blocks per SM up to their occupancy, on the solve's own start point
 * (gamma is saved and restored around the timing runs). */
int pasc_gb300_get_sweep_tuning(pasc_gb300_problem *p, int *variant, int *blocks, double *sweep_ms);

/* Measurement: device time per call (CUDA events on the handle's stream) of `reps`
 * back-to-back launches of the theta update (which = 1, as pasc_gb300_update_theta) or of the
 * residual b (which = 2, as pasc_gb300_update_b).  Changes theta / b as those calls do. */
int pasc_gb300_time_model_kernels(pasc_gb300_problem *p, int which, int reps, double *ms_per_call);

/* QPData::get_b (include/general/data/qpdata.h:23-112): the gamma problem's linear term
 * b_tk = bscale ||X_t - theta_k||^2 (N host values).  fp64 path: the stored b; multichannel:
 * the FP32 b the residual kernel wrote; 1-D mixed path (b formed inside the sweep): the same
 * formula evaluated in FP64 from the stored data and theta. */
int pasc_gb300_get_b(pasc_gb300_problem *p, double *b);

/* FEM temporal coarsening: GraphH1FEMModel(tsdata, epssqr, fem) with fem = Fem(fem_reduce)
 * (fem_type 0, FEM-SUM, src/petscvector/common/fem.cpp) or FemHat(fem_reduce) (fem_type 1,
 * FEM-HAT, src/petscvector/common/femhat.cpp); graphh1fem.cpp:48-59, 116-160, 237-303.  With
 * fem_reduce < 1 the gamma QP is solved on T2 = ceil(T*fem_reduce) timesteps: update_b reduces
 * the residual (scaled by -1/T2) and the current gamma onto the coarse grid, spgqp_solve solves
 * there and prolongates the solution to the full gamma; theta, data, gamma and the TSSolver
 * loop stay on the full grid.  fem_reduce = 1 removes the reduction.  A reduced problem solves
 * with spgqp_solve / ts_solve (not spgqp_start / spgqp_iterate) and has no adjoint. */
int pasc_gb300_set_fem(pasc_gb300_problem *p, double fem_reduce, int fem_type);
int pasc_gb300_get_fem(pasc_gb300_problem *p, double *fem_reduce, int *fem_type, long *T_reduced);

/* Graph (R > 1) and image mode: GraphH1FEMModel on Decomposition(T, graph, K, 1, 1)
 * (include/general/common/decomposition.h; graphh1fem.cpp:8-65) with the operator
 * BlockGraphSparseMatrix on a graph of R nodes (blockgraphsparse.cpp:7-103): row (t, r, k)
 * has -2 at (t+-1, r), -1 at (t, r') and (t+-1, r') for every neighbour r' of r, and the
 * diagonal that makes the row sum to zero.  The problem has T*R blocks of K: gamma index
 * (t*R + r)*K + k, data index t*R + r (T*R values), theta K values; A = epssqr/T * A_graph and
 * b = -(x - theta_k)^2 / T keep the number of timesteps T.  pasc_gb300_permute_gamma maps the
 * blocked layout k*R*T + r*T + t (Decomposition::permute_TRK, decomposition.cpp:257-340).
 * The graph: CSR neighbour lists of the R nodes (nbr_ptr: R+1 offsets, nbr_idx: nbr_ptr[R]
 * indices), each list sorted ascending, no duplicates, no self-loops, symmetric (checked;
 * PASC_ERR_ARG otherwise).  Image data (test_image): T = 1, R = width*height, the grid graph.
 * Not with FEM reduction, theta in the penalty, multichannel data or the adjoint
 * (PASC_ERR_NOTSUPP).  The mixed path runs two kernels per SPG iteration. */
int pasc_gb300_create_graph(pasc_gb300_problem **out, long T, long R, int K, int precision, double epssqr,
                            int device, const int *nbr_ptr, const int *nbr_idx);
/* T = timesteps, R = nodes (1 and 0 edges for a 1-D problem) */
int pasc_gb300_get_graph(pasc_gb300_problem *p, long *T, long *R, long *nnz);

/* Graphs the reference builds, as CSR neighbour lists sorted ascending (host functions):
 * BGMGraphGrid1D::process_grid (bgmgraphgrid1D.h:76-115; nbr_ptr: width+1, nbr_idx:
 * 2*(width-1)), BGMGraphGrid2D::process_grid (bgmgraphgrid2D.h:88-142; node i*width + j,
 * nbr_idx: 2*(height*(width-1) + width*(height-1))), and BGMGraph::process(threshold)
 * (bgmgraph.cpp:73-152): nodes i, j are neighbours when sum_d (c[i+d*n] - c[j+d*n])^2 <
 * threshold^2.  graph_threshold with nbr_idx == NULL computes nbr_ptr and *nnz only. */
int pasc_gb300_graph_grid1d(int width, int *nbr_ptr, int *nbr_idx);
int pasc_gb300_graph_grid2d(int width, int height, int *nbr_ptr, int *nbr_idx);
int pasc_gb300_graph_threshold(const double *coords, int n, int dim, double threshold, int *nbr_ptr, int *nbr_idx,
                               long idx_capacity, long *nnz);
/* y = coeff * A_graph x on device buffers (T*R*K values; nbr_* in device memory), FP64 in the
 * assembled matrix's sorted column order (MatMult of blockgraphsparse.cpp:152-160). */
int pasc_gb300_graph_matmult_f64(const double *x_dev, double *y_dev, long T, long R, int K, double coeff,
                                 const int *nbr_ptr_dev, const int *nbr_idx_dev, void *stream);

/* The gamma solver GraphH1FEMModel builds (gammasolvertype, include/general/model/
 * graphh1fem.h:42-48; console option graphh1femmodel_gammasolvertype): 0 = automatic (1),
 * 1 = SPGQPSolver, 2 = SPGQPSolverC (include/general/solver/spgqpsolver_coeff.h:611-835: the
 * coefficient eps of A = eps*A1 is factored out: d'Ad and the BB step use A1, the first step is
 * alphainit/eps, the A-condition takes 2*eps*xi and the sigma1 clamp acts on the unscaled
 * beta).  3 (PERMON) and 4 (TAO) give PASC_ERR_NOTSUPP, as does 2 with theta in the penalty. */
int pasc_gb300_set_gamma_solver_type(pasc_gb300_problem *p, int type);
int pasc_gb300_get_gamma_solver_type(pasc_gb300_problem *p, int *type);

/* Theta in the penalty: GraphH1FEMModel(tsdata, epssqr, fem, usethetainpenalty = true)
 * (graphh1fem.cpp:8-19, 154-160; include/general/model/graphh1fem.h:61, 75).  Block k of the
 * gamma QP's A is alpha*theta_k*theta_k*A_hat (BlockGraphSparseMatrix with coefficients,
 * blockgraphsparse.cpp:161-185; alpha = epssqr/T), and the theta step is
 * theta_k = gamma_k'x / (sum gamma_k + gamma_k'(alpha A_hat)gamma_k / 2)
 * (updatebeforesolve_thetasolver, graphh1fem.cpp:306-380).  xdim == 1 and fem_reduce == 1 only
 * (PASC_ERR_NOTSUPP otherwise); no adjoint. */
int pasc_gb300_set_usethetainpenalty(pasc_gb300_problem *p, int on);
int pasc_gb300_get_usethetainpenalty(pasc_gb300_problem *p, int *on);

/* Residual kernel of multichannel data (xdim > 1): 0 = tensor cores (tcgen05, BF16 X and a
 * three-part BF16 theta, FP32 accumulation; xdim in {64, 128, 256}; the default there),
 * 1 = CUDA cores (FP32; any xdim, the default otherwise).  No reference counterpart: the
 * reference's GraphH1FEM takes scalar data. */
int pasc_gb300_set_residual_engine(pasc_gb300_problem *p, int engine);
int pasc_gb300_get_residual_engine(pasc_gb300_problem *p, int *engine);

/* SPGQPSolver<PetscVector>::get_fx (spgqpsolver.cpp:316-345): 1/2 (g - b)'x of the last solve. */
int pasc_gb300_get_fx(pasc_gb300_problem *p, double *fx);

/* TSSolver<VectorBase>::solve (include/general/solver/tssolver.h:492-715) with the
 * GraphH1FEMModel hooks.  gamma_restart (nullable, N values) is what set_random() gives
 * annealing restarts (tssolver.h:700-702). */
int pasc_gb300_ts_solve(pasc_gb300_problem *p, const pasc_gb300_ts_opts *ts,
                        const pasc_gb300_spgqp_opts *spg, const double *gamma_restart,
                        pasc_gb300_ts_stats *st);

/* Signal1DData::compute_abserr_reconstructed (src/petscvector/data/signal1Ddata.cpp:134-191):
 * || sum_k theta_k gamma_k - solution ||_1, solution a host buffer of T values. */
int pasc_gb300_abserr_reconstructed(pasc_gb300_problem *p, const double *solution, double *abserr);

/* Hard labels, true argmax per t (lowest k wins ties); host buffer of T ints.  The
 * reference's TSData::cutgamma (src/petscvector/data/tsdata.cpp:196-235) seeds its running
 * maximum with gamma[t] instead of gamma[t*K]; this returns the intended argmax. */
int pasc_gb300_argmax_labels(pasc_gb300_problem *p, int *labels);

/* ---------------------------------------------------------------------------------------
 * derivatives through the converged gamma step (no counterpart in the reference, which only
 * solves).  The free set F_t = {k : z_tk > act_tol} is read from one projected-gradient step
 * z = Proj(gamma - a (A gamma - b)), a = 1/(8 coeff + |bscale|) (z = gamma at an exact solution;
 * on an FP32 end point it drops entries held at zero by their multiplier).  With F held fixed, the solution of the
 * QP moves inside S = {v : v_tk = 0 for k outside F_t, sum_k v_tk = 0}; the adjoint lambda in
 * S solves P A P lambda = P dloss/dgamma (P the orthogonal projection onto S, A = coeff *
 * A_hat) by conjugate gradients in FP64, and
 *   dloss/d epssqr  = -(d coeff/d epssqr) lambda'(A_hat gamma)
 *   dloss/d x_t     =  sum_k lambda_tk d b_tk/d x_t       (b_tk = bscale (x_t - theta_k)^2)
 *   dloss/d theta_k =  sum_t lambda_tk d b_tk/d theta_k  (+ the loss's own theta term, below)
 * theta is a given input here (the theta step is not differentiated).
 * ------------------------------------------------------------------------------------- */
typedef struct {
    double act_tol;         /* z_tk > act_tol is free (1e-7) */
    double cg_tol;          /* stop when ||r|| <= cg_tol * ||r_0|| (1e-10) */
    int cg_maxit;           /* (20000) */
} pasc_gb300_adjoint_opts;

typedef struct {
    int cg_it;              /* conjugate-gradient iterations */
    int status;             /* 1 converged, 2 cg_maxit reached */
    int kernel_launches;
    long free_dims;         /* dimension of S: sum_t max(|F_t| - 1, 0) */
    double cg_relres;       /* ||r|| / ||r_0|| at the end */
    double time_s;          /* device time (CUDA events) */
} pasc_gb300_adjoint_stats;

void pasc_gb300_adjoint_default_opts(pasc_gb300_adjoint_opts *o);
/* loss = 1/T sum_t (sum_k gamma_tk theta_k - clean_t)^2 of the current gamma and theta (clean: T
 * host values); dloss/dgamma and the loss's own dloss/dtheta are kept on the device for the
 * next pasc_gb300_adjoint call with dloss_dgamma == NULL. */
int pasc_gb300_recon_mse(pasc_gb300_problem *p, const double *clean, double *loss);
/* dloss_dgamma: N host values, or NULL for the gradient kept by pasc_gb300_recon_mse (then
 * dloss_dtheta includes that loss's direct theta term).  Outputs are nullable host buffers:
 * dloss_depssqr (1), dloss_ddata (T), dloss_dtheta (K).  K <= 8.  PASC_ERR_STATE if conjugate
 * gradients break down (the right-hand side has a part in the null space of P A P). */
int pasc_gb300_adjoint(pasc_gb300_problem *p, const double *dloss_dgamma, const pasc_gb300_adjoint_opts *o,
                       double *dloss_depssqr, double *dloss_ddata, double *dloss_dtheta,
                       pasc_gb300_adjoint_stats *st);

/* Polish (no reference counterpart): refines the problem's gamma to the optimum of its QP
 * on the face the solve ended on.  The mixed path's FP32 iteration stalls where its updates
 * drop below half an FP32 ulp of gamma, ~1e-6..1e-5 (relative 2-norm) from the optimum on
 * ill-conditioned problems, at a point that depends on the rounding of the sums; each round
 * here reads the free set F_t from one projected-gradient step (as the adjoint does), moves
 * gamma onto that face (entries outside F_t to 0, their mass spread over F_t), solves
 * P A P delta = -P (A gamma - b) on S in FP64 (FP32 conjugate gradients inside FP64 iterative
 * refinement on mixed problems, the adjoint's solver), adds delta in FP64 and projects the
 * timesteps that left their face back onto the simplex; a round that does not lower the FP64
 * objective is undone, and the rounds end when a step stays on its face or the projected
 * gradient is at the rounding level of b.  Mixed problems keep the result rounded once to FP32.  Afterwards get_fx returns
 * the FP64 objective of the polished gamma; a dloss/dgamma kept by recon_mse is dropped.  Same
 * restrictions as the adjoint (K <= 8, 1-D, no FEM reduction, theta not in the penalty). */
typedef struct {
    int rounds;             /* at most this many face-Newton rounds (4) */
    double act_tol;         /* z_tk > act_tol is free (0: every entry a projected-gradient step
                               leaves positive, so that small free entries of the optimum stay free) */
    double cg_tol;          /* relative residual of each solve (1e-6: a round gains about six
                               digits on the face; the next round starts from its end) */
    int cg_maxit;           /* conjugate-gradient iterations per solve (2000) */
} pasc_gb300_polish_opts;

typedef struct {
    int rounds;             /* rounds done */
    int cg_it;              /* conjugate-gradient iterations, all rounds */
    int kernel_launches;
    long face_changes;      /* timesteps projected back onto the simplex in the last round */
    int cg_status;          /* last solve: 1 converged, 2 cg_maxit reached, 4 stopped at the
                               rounding level (p'Ap <= 0), 0 none run */
    double cg_relres;       /* last solve: ||r|| / ||r_0|| at its end */
    double step_rel;        /* ||delta|| / ||gamma|| of the last round */
    double fx;              /* FP64 objective of the polished gamma */
    double time_s;          /* device time (CUDA events) */
} pasc_gb300_polish_stats;

void pasc_gb300_polish_default_opts(pasc_gb300_polish_opts *o);
int pasc_gb300_polish(pasc_gb300_problem *p, const pasc_gb300_polish_opts *o, pasc_gb300_polish_stats *st);

/* ---------------------------------------------------------------------------------------
 * device-pointer kernels: the reference's GPU-side operations, usable on caller buffers
 * ------------------------------------------------------------------------------------- */

/* SimplexFeasibleSet_Local<PetscVector>::project -> ExternalContent::cuda_project
 * (src/petscvector/algebra/feasibleset/simplex_local.cpp:38-65, simplex_local.cu:39-139):
 * in-place projection of T blocks of K on the device.  The fp64 form keeps the reference's
 * operation order (bit-identical to the host algorithm); K <= 128.  No scratch memory
 * (the reference allocates K*T doubles for its sort). */
int pasc_gb300_project_f64(double *x_dev, long T, int K, void *stream);
/* FP32 form: one thread per t for K <= 8, a lane group per t with shuffles for K <= 32. */
int pasc_gb300_project_f32(float *x_dev, long T, int K, void *stream);

/* BlockGraphSparseMatrix<PetscVector>::matmult (src/petscvector/algebra/matrix/
 * blockgraphsparse.cpp:152-194) for R = 1 without theta coefficients: y = coeff * A_hat x,
 * matrix-free (nothing assembled).  fp64 form sums each row like the assembled CSR MatMult. */
int pasc_gb300_fem_h1_matmult_f64(const double *x_dev, double *y_dev, long T, int K,
                                  double coeff, void *stream);
int pasc_gb300_fem_h1_matmult_f32(const float *x_dev, float *y_dev, long T, int K,
                                  float coeff, void *stream);

/* The vector level of the reference's backend interface on FP64 device buffers, for a
 * backend that keeps the reference's own generic solvers and gives them device vectors
 * (include/pasc/gb300_backend.hpp): GeneralVector<VectorBase> (include/general/algebra/
 * vector/generalvector.h:58-106) over the PETSc operations its GPU backend calls
 * (include/external/petscvector/algebra/vector/petscvector.h: VecDuplicate/VecCreate ->
 * vec_alloc, VecCopy -> vec_copy, VecAXPY -> vec_axpy, VecWAXPY -> vec_waxpy, VecScale ->
 * vec_scale, VecDot -> vec_dot; VecNorm is sqrt(vec_dot(x, x))).  FP64, each element in the
 * reference's operation order; vec_dot is a deterministic block tree (its result waits for the
 * stream); vec_alloc returns zeroed memory on `device` (which it makes current).  Operations
 * take the device of their buffers as current. */
int pasc_gb300_vec_alloc(double **v_dev, long n, int device);
int pasc_gb300_vec_free(double *v_dev);
int pasc_gb300_vec_set(double *v_dev, const double *host, long n);
int pasc_gb300_vec_get(const double *v_dev, double *host, long n);
int pasc_gb300_vec_copy(double *y_dev, const double *x_dev, long n, void *stream);                 /* y = x */
int pasc_gb300_vec_axpy(double *y_dev, double a, const double *x_dev, long n, void *stream);       /* y += a x */
int pasc_gb300_vec_waxpy(double *w_dev, double a, const double *x_dev, const double *y_dev, long n,
                         void *stream);                                                            /* w = a x + y */
int pasc_gb300_vec_scale(double *x_dev, double a, long n, void *stream);                          /* x = a x */
int pasc_gb300_vec_dot(const double *x_dev, const double *y_dev, long n, double *out, void *stream);
/* Decomposition::permute_TRK (src/petscvector/common/decomposition.cpp:266-356, R = 1):
 * blocked k*T + t -> interleaved t*K + k, out of place. */
int pasc_gb300_permute_f64(const double *src_dev, double *dst_dev, long T, int K, void *stream);
/* GraphH1FEMModel::updatebeforesolve_gammasolver (src/petscvector/model/graphh1fem.cpp:237-289)
 * on device buffers: b_tk = bscale (x_t - theta_k)^2 (theta_dev: K values on the device). */
int pasc_gb300_residual_f64(const double *data_dev, const double *theta_dev, double *b_dev, long T, int K,
                            double bscale, void *stream);
/* GraphH1FEMModel::updatebeforesolve_thetasolver (graphh1fem.cpp:347-380) on device buffers:
 * theta_k = sum_t gamma_tk x_t / sum_t gamma_tk; waits for the result. */
int pasc_gb300_theta_update_f64(const double *gamma_dev, const double *data_dev, double *theta_dev, long T, int K,
                                void *stream);

/* Fem::reduce_gamma / prolongate_gamma (src/petscvector/common/fem.cpp:32-190,
 * femhat.cpp:27-215) on device buffers: g1 T1*K fine values, g2 T2*K coarse values
 * (interleaved t*K + k), fem_type 0 FEM-SUM or 1 FEM-HAT (T2 >= 2).  The reference's CUDA
 * versions of these two operations do not link (their kernels are declared under other names,
 * fem.cu:8-9 vs :41,55); these follow its sequential code. */
int pasc_gb300_fem_reduce_f64(const double *g1_dev, double *g2_dev, long T1, long T2, int K, int fem_type,
                              void *stream);
int pasc_gb300_fem_prolongate_f64(const double *g2_dev, double *g1_dev, long T1, long T2, int K, int fem_type,
                                  void *stream);

/* Theta update for callers that cannot allocate device memory when they need it: hosts
 * whose device memory belongs to another framework's allocator, real-time loops that allow
 * no allocation (nor the device synchronisation cudaMalloc/cudaFree can imply) after
 * start-up.  No counterpart in the reference; it computes what pasc_gb300_update_theta
 * computes (theta_k = sum_t gamma_tk x_t / sum_t gamma_tk) on caller-owned device buffers:
 * gamma_dev (T*K floats, t*K + k), data_dev (T floats), theta_dev (K doubles, written).  It
 * calls no cudaMalloc, cudaFree or allocating library routine; its reduction scratch is a
 * static device array of the library (about 128 KiB, held on every GPU that loads the
 * library until the process exits), which limits K to 8.  The first call on a device looks
 * up that array's address (cudaGetSymbolAddress) and keeps it, so make that call before any
 * stream capture, and do not use the entry point on a device after cudaDeviceReset there
 * (the kept address belonged to the context the reset ended).  All calls share the array:
 * calls that overlap on the GPU (other streams, or before the previous call has finished)
 * race and must be avoided.  Asynchronous on `stream`. */
int pasc_gb300_theta_update_noalloc(const float *gamma_dev, const float *data_dev, long T, int K,
                                    double *theta_dev, void *stream);

/* ---------------------------------------------------------------------------------------
 * batch handle: n independent signals (each with its own T, K and epssqr) solved together on
 * one device, mixed precision.  The reference solves such problems one run at a time (one
 * TSSolver per signal, examples/test_signal1D/test_signal1D.cpp:188-353); here one launch
 * per SPG iteration advances every signal whose solve is still running, and each signal
 * keeps its own step lengths, GLL memory and stopping decision.
 * ------------------------------------------------------------------------------------- */
typedef struct pasc_gb300_batch pasc_gb300_batch;

/* T[i] >= 1, 1 <= K[i] <= 8, epssqr[i] as in pasc_gb300_create (xdim == 1, scalef = 1). */
int pasc_gb300_batch_create(pasc_gb300_batch **out, int n, const long *T, const int *K,
                            const double *epssqr, int device);
int pasc_gb300_batch_destroy(pasc_gb300_batch *b);
int pasc_gb300_batch_size(pasc_gb300_batch *b, int *n);
/* Host buffers of signal i, FP64, with the meaning of pasc_gb300_set_data/set_gamma/
 * get_gamma/set_theta/get_theta (T[i], T[i]*K[i] and K[i] values). */
int pasc_gb300_batch_set_data(pasc_gb300_batch *b, int i, const double *data);
int pasc_gb300_batch_set_gamma(pasc_gb300_batch *b, int i, const double *gamma);
int pasc_gb300_batch_get_gamma(pasc_gb300_batch *b, int i, double *gamma);
int pasc_gb300_batch_set_theta(pasc_gb300_batch *b, int i, const double *theta);
int pasc_gb300_batch_get_theta(pasc_gb300_batch *b, int i, double *theta);
/* How the batched solves below are driven (no reference counterpart).  device_loop = 1 (the
 * default): each solve is ONE CUDA graph launch; conditional WHILE nodes repeat the sweeps and
 * the outer iterations, and single-block control kernels decide on the device after every
 * `chunk` sweeps (1..64, default 4) which signals still run and whether to go on -- no host
 * round trip inside a solve.  The loops are bounded by the solve's maxit (sweeps) and the
 * TSSolver's maxit (outer iterations).  device_loop = 0: the host launches the sweeps in
 * chunks and reads the signals' states between chunks. */
int pasc_gb300_batch_set_loop(pasc_gb300_batch *b, int device_loop, int chunk);
/* Work items of the batched sweeps (no reference counterpart): every signal is cut into
 * segments of bulk-copy tiles of 504 timesteps, and a block takes work items (consecutive
 * segments of one signal) from a list ordered longest signals first.  tiles = 0 (the default):
 * segments of 4 tiles, merged at every rebuild of the list into items sized from the number of
 * segments still running -- about four items per resident block, 4 to 32 tiles each (long
 * items while every signal runs, short ones when few remain); -c (1 <= c <= 16): the same
 * with about c items per resident block; 2..64: every item is one segment of that many tiles.
 * get: the segment size and (nullable) the item size with every signal running, in tiles. */
int pasc_gb300_batch_set_segment_tiles(pasc_gb300_batch *b, int tiles);
int pasc_gb300_batch_get_segment_tiles(pasc_gb300_batch *b, int *seg_tiles, int *item_tiles);
/* pasc_gb300_spgqp_solve for every signal at once; st: n entries (nullable).  The
 * ||b||-scaled stopping tests are not supported (PASC_ERR_NOTSUPP). */
int pasc_gb300_batch_spgqp_solve(pasc_gb300_batch *b, const pasc_gb300_spgqp_opts *o,
                                 pasc_gb300_spgqp_stats *st);
/* pasc_gb300_ts_solve for every signal at once (annealing <= 1): every signal runs its own
 * outer loop and leaves the batch when its |L - L_old| test holds; st: n entries
 * (nullable), kernel_launches and time_s are those of the whole batch. */
int pasc_gb300_batch_ts_solve(pasc_gb300_batch *b, const pasc_gb300_ts_opts *ts,
                              const pasc_gb300_spgqp_opts *spg, pasc_gb300_ts_stats *st);

#ifdef __cplusplus
}
#endif
#endif
