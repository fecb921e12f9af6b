/*
 * pasc_oracle.h -- FP64 CPU restatement of PASC_inference's FEM-H1 clustering hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only as the checker (or as the
 * timed CPU baseline).  The GPU library never links or calls it.
 *
 * Every function restates one piece of the reference in the reference's own operation
 * order (FP64, no fused multiply-add, sequential reductions when nthreads == 1) and cites
 * the reference file:line it follows.  Paths are relative to the PASC_inference tree.
 *
 * Layout (reference decomposition with R = 1, DDT_size = 1):
 *   gamma / x / g / b : N = K*T doubles, interleaved, index t*K + k
 *                       (src/petscvector/algebra/matrix/blockgraphsparse.cpp:54,
 *                        src/petscvector/model/graphh1fem.cpp:261)
 *   data              : T*xdim doubles, index t*xdim + j
 *   theta             : K*xdim doubles, index k*xdim + j (graphh1fem.cpp:94)
 */
#ifndef PASC_ORACLE_H
#define PASC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* SPGQPSolver settings; defaults in include/general/solver/spgqpsolver.h:19-36. */
typedef struct {
    int    maxit;          /* spgqpsolver_maxit, default 1000 */
    double eps;            /* spgqpsolver_eps, default 1e-9 */
    int    m;              /* GLL memory length, default 20 */
    double gamma;          /* Armijo parameter, default 0.9 */
    double sigma1;         /* default 0 */
    double sigma2;         /* default 1 */
    double alphainit;      /* default 2 */
    int    stop_difff;     /* |f - f_old| < eps (default on) */
    int    stop_normgp;    /* dd < eps */
    int    stop_normgp_normb;  /* dd < eps*||b|| */
    int    stop_Anormgp;   /* dAd < eps */
    int    stop_Anormgp_normb; /* dAd < eps*||b|| */
} pasc_oracle_spg_opts;

typedef struct {
    int    it;             /* iterations of this solve (it_last) */
    int    hessmult;       /* Hessian products of this solve (hessmult_last) */
    double fx;             /* final objective */
    double gP;             /* last dd = ||d||^2 */
    double dAd;            /* last dAd */
    double normb;          /* ||b||_2 */
} pasc_oracle_spg_result;

/* TSSolver settings; defaults in include/general/solver/tssolver.h:13-15. */
typedef struct {
    int    maxit;          /* tssolver_maxit, default 300 */
    double eps;            /* tssolver_eps, default 1e-6 */
    int    init_permute;   /* tssolver_init_permute, default true */
    int    annealing;      /* number of annealing restarts, default 1 */
    int    relative;       /* 0: |L-L_old| < eps (reference); 1: |L-L_old| < eps*|L| */
    int    thetasolved;    /* 1: theta given (set_solution_theta), skip theta update */
} pasc_oracle_ts_opts;

typedef struct {
    int    it_last;        /* outer iterations of the kept annealing run */
    int    it_sum;         /* outer iterations over all annealing runs */
    int    spg_it_sum;     /* SPG iterations over the whole solve */
    int    spg_hessmult_sum;
    double L;              /* final objective L (gammasolver fx) */
    double deltaL;         /* final |L - L_old| */
    double aic;            /* 2 log L + K */
    int    L_increased;    /* times the reference would print "objective function increased" */
} pasc_oracle_ts_result;

void pasc_oracle_spg_default_opts(pasc_oracle_spg_opts *o);
void pasc_oracle_ts_default_opts(pasc_oracle_ts_opts *o);

/* Per-timestep Euclidean projection onto the K-simplex, in place. */
void pasc_oracle_project(double *x, long T, int K, int nthreads);

/* y = coeff * A_hat x, A_hat = the FEM-H1 block matrix for R = 1 (K tridiagonal copies). */
void pasc_oracle_fem_h1_matmult(const double *x, double *y, long T, int K, double coeff, int nthreads);

/* b_tk = bscale * ||X_t - theta_k||^2 ; bscale = -1/T with scalef. */
void pasc_oracle_residual_b(const double *data, const double *theta, double *b, long T, int K,
                            int xdim, double bscale, int nthreads);

/* K-means theta: theta_k = sum_t gamma_tk X_t / sum_t gamma_tk (0 when the sum is 0). */
void pasc_oracle_theta_update(const double *gamma, const double *data, double *theta, long T,
                              int K, int xdim, int nthreads);

/* Blocked (k*T + t) -> interleaved (t*K + k) permutation of a gamma vector. */
void pasc_oracle_permute_blocked_to_interleaved(const double *orig, double *out, long T, int K);

/* Coefficients of the QP as GraphH1FEMModel sets them (scalef = 1 is the default). */
double pasc_oracle_A_coeff(double epssqr, long T, int scalef);
double pasc_oracle_b_coeff(long T, int scalef);

/* SPG-QP solve of min 1/2 x'Ax - b'x over the simplex product, x in/out (warm start).
 * trace (nullable) receives 8 doubles per iteration 0..it:
 *   fx, dd, dAd, gd, fx_max, beta, alpha_bb, 0.  Row 0 holds the initial fx. */
int pasc_oracle_spgqp_solve(const double *b, double *x, long T, int K, double coeff,
                            const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r,
                            double *trace, int nthreads);

/* Full TSSolver::solve with the GraphH1FEMModel hooks (fem_reduce = 1, R = 1).
 * gamma (N) in/out: on entry the TSData gamma vector as the model left it (raw random values,
 * permuted here when init_permute is set); theta (K*xdim) in/out.
 * gamma_restart (nullable) is the vector set_random() would produce for annealing restarts.
 * trace_L (nullable, size ts->maxit*max(1,annealing)) receives L per outer iteration. */
int pasc_oracle_tssolver_solve(const double *data, double *gamma, double *theta, long T, int K,
                               int xdim, double epssqr, int scalef,
                               const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                               const double *gamma_restart, pasc_oracle_ts_result *r,
                               double *trace_L, int nthreads);

/* L1 error of sum_k theta_k gamma_k against a clean signal (xdim = 1). */
double pasc_oracle_abserr_reconstructed(const double *gamma, const double *theta,
                                        const double *solution, long T, int K);

/* Hard labels: true argmax per t, lowest k wins ties. */
void pasc_oracle_argmax_labels(const double *gamma, int *labels, long T, int K);

/* ------------------------------------------------------------------------------------
 * Derivatives through the converged gamma step.  The reference has no such code: this is
 * the FP64 statement of active-set implicit differentiation of the QP above, the checker of
 * the GPU adjoint.  Free set F_t = {k : z_tk > act_tol} with z = Proj(gamma - a (A gamma - b)),
 * a = 1/(8 coeff + |bscale|) (z = gamma at an exact solution); S = {v : v_tk = 0 off F_t,
 * sum_k v_tk = 0}; P = orthogonal projection onto S (per t: zero off F_t, subtract the mean
 * over F_t).  lambda in S solves P A P lambda = P dl/dgamma (conjugate gradients from 0,
 * stop at ||r|| <= cg_tol ||r_0||), A = coeff * A_hat, and
 *   dl/d epssqr  = -dcoeff * lambda'(A_hat gamma)           (dcoeff = d coeff / d epssqr)
 *   dl/d x_t     =  sum_k lambda_tk * 2 bscale (x_t - theta_k)
 *   dl/d theta_k = -sum_t lambda_tk * 2 bscale (x_t - theta_k)
 * ---------------------------------------------------------------------------------- */
typedef struct {
    double act_tol;
    double cg_tol;
    int    cg_maxit;
} pasc_oracle_adj_opts;

typedef struct {
    int    cg_it;
    int    status;         /* 1 converged, 2 maxit, 4 breakdown */
    long   free_dims;
    double cg_relres;
} pasc_oracle_adj_result;

/* loss = 1/T sum_t (sum_k gamma_tk theta_k - clean_t)^2; dgamma (N, nullable) = dl/dgamma,
 * dtheta (K, nullable) = the loss's direct dl/dtheta. */
double pasc_oracle_recon_mse(const double *gamma, const double *theta, const double *clean, long T,
                             int K, double *dgamma, double *dtheta);

/* lambda (N, nullable), dloss_ddata (T, nullable), dloss_dtheta (K, nullable). */
int pasc_oracle_adjoint(const double *gamma, const double *data, const double *theta,
                        const double *dloss_dgamma, long T, int K, double coeff, double dcoeff,
                        double bscale, const pasc_oracle_adj_opts *o, double *lambda,
                        double *dloss_depssqr, double *dloss_ddata, double *dloss_dtheta,
                        pasc_oracle_adj_result *r);

/* ------------------------------------------------------------------------------------
 * FEM temporal coarsening (GraphH1FEMModel with fem_reduce < 1): the gamma QP lives on
 * T2 = ceil(T*fem_reduce) timesteps.  One rank (Tbegin = 0, the whole range local).
 *   type 0, FEM-SUM (src/petscvector/common/fem.cpp:32-115, 124-210): diff = T1/T2; coarse
 *     t2 sums fine t in [round(t2*diff), round((t2+1)*diff)); prolongation copies it back.
 *   type 1, FEM-HAT (src/petscvector/common/femhat.cpp:27-215, include/general/common/
 *     femhat.h:154-195): diff = (T1-1)/(T2-1); reduction weights by hat functions centred at
 *     t2*diff, prolongation interpolates linearly between the two coarse neighbours (a
 *     neighbour past the last coarse point counts as 0).
 * ---------------------------------------------------------------------------------- */
long pasc_oracle_fem_T_reduced(long T, double fem_reduce);
void pasc_oracle_fem_reduce(const double *g1, double *g2, long T1, long T2, int K, int type);
void pasc_oracle_fem_prolongate(const double *g2, double *g1, long T1, long T2, int K, int type);
/* pasc_oracle_tssolver_solve with the model's gamma step on the reduced problem
 * (src/petscvector/model/graphh1fem.cpp:116-160, 237-303): b = coeffB2 * reduce((x_t -
 * theta_k)^2) with coeffB2 = -1/T2 (scalef), x = reduce(gamma) before each gamma solve,
 * A = epssqr/T * A_hat(T2) (scalef; epssqr*T2/T otherwise), gamma = prolongate(x) after it.
 * xdim == 1. */
/* A graph of R nodes for BlockGraphSparseMatrix (BGMGraph neighbour lists, src/petscvector/
 * algebra/graph/bgmgraph.cpp:73-152): node r's neighbours are idx[ptr[r] .. ptr[r+1]-1],
 * sorted ascending, no duplicates, no r itself. */
typedef struct {
    long R;
    const int *ptr;
    const int *idx;
} pasc_oracle_graph;

/* y = coeff * A_graph x over T timesteps and R nodes (x, y: T*R*K, index (t*R + r)*K + k) */
void pasc_oracle_graph_matmult(const double *x, double *y, long T, int K, double coeff, const pasc_oracle_graph *G,
                               int nthreads);
int pasc_oracle_spgqp_solve_graph(const double *b, double *x, long T, int K, double coeff, const pasc_oracle_graph *G,
                                  const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads);
void pasc_oracle_permute_TRK(const double *orig, double *out, long T, long R, int K);
void pasc_oracle_graph_grid1d(int width, int *ptr, int *idx);
void pasc_oracle_graph_grid2d(int width, int height, int *ptr, int *idx);
long pasc_oracle_graph_threshold(const double *coords, int n, int dim, double threshold, int *ptr, int *idx);

/* usethetainpenalty (graphh1fem.cpp:154-160, 306-380, blockgraphsparse.cpp:161-185): the
 * gamma QP's block k is scaled by kc[k] = coeff*theta_k*theta_k (spgqp_solve_kc), and theta is
 * updated with the penalty term (theta_update_penalty, alpha = the QP coefficient). */
void pasc_oracle_fem_h1_matmult_kc(const double *x, double *y, long T, int K, const double *kc, int nthreads);
int pasc_oracle_spgqp_solve_kc(const double *b, double *x, long T, int K, const double *kc,
                               const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads);
void pasc_oracle_theta_update_penalty(const double *gamma, const double *data, double *theta, long T, int K,
                                      double alpha);
/* the general model: FEM coarsening and/or usethetainpenalty (not both: the reference's theta
 * step multiplies the reduced operator with the full gamma) */
int pasc_oracle_tssolver_solve_model(const double *data, double *gamma, double *theta, long T, int K,
                                     double epssqr, int scalef, double fem_reduce, int fem_type,
                                     int usethetainpenalty, const pasc_oracle_ts_opts *ts,
                                     const pasc_oracle_spg_opts *spg, pasc_oracle_ts_result *r, int nthreads);
/* SPGQPSolverC (include/general/solver/spgqpsolver_coeff.h:611-835): the coefficient of
 * A = coeff * A1 factored out of the iteration; G may be NULL (1-D).  TSSolver with it. */
int pasc_oracle_spgqp_solve_coeff(const double *b, double *x, long T, int K, double coeff, const pasc_oracle_graph *G,
                                  const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads);
int pasc_oracle_tssolver_solve_coeff(const double *data, double *gamma, double *theta, long T, int K, double epssqr,
                                     int scalef, const pasc_oracle_graph *G, const pasc_oracle_ts_opts *ts,
                                     const pasc_oracle_spg_opts *spg, pasc_oracle_ts_result *r, int nthreads);
int pasc_oracle_tssolver_solve_graph(const double *data, double *gamma, double *theta, long T, int K,
                                     double epssqr, int scalef, const pasc_oracle_graph *G,
                                     const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                                     pasc_oracle_ts_result *r, int nthreads);
int pasc_oracle_tssolver_solve_fem(const double *data, double *gamma, double *theta, long T, int K,
                                   double epssqr, int scalef, double fem_reduce, int fem_type,
                                   const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                                   pasc_oracle_ts_result *r, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
