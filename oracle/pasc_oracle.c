/*
 * pasc_oracle.c -- FP64 CPU restatement of PASC_inference's FEM-H1 / SPG-QP / TSSolver path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE: the checker for the GPU library and the timed CPU
 * baseline.  Compiled with -ffp-contract=off so that no multiply-add is fused, which keeps
 * the arithmetic identical on x86-64 and aarch64 hosts.
 *
 * With nthreads == 1 every reduction runs sequentially in index order, the order of a
 * single-rank PETSc VecDot/VecSum on the host.  With nthreads > 1 the element-wise operations
 * are split over OpenMP threads and reductions are summed per static chunk, then in thread
 * order (deterministic for a fixed thread count); that mode exists for CPU-baseline timing.
 */
#include "pasc_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_KMAX_STACK 64

static int eff_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0) return omp_get_max_threads();
    return nthreads;
#else
    (void)nthreads;
    return 1;
#endif
}

void pasc_oracle_spg_default_opts(pasc_oracle_spg_opts *o)
{
    /* include/general/solver/spgqpsolver.h:19-36 */
    o->maxit = 1000;
    o->eps = 1e-9;
    o->m = 20;
    o->gamma = 0.9;
    o->sigma1 = 0.0;
    o->sigma2 = 1.0;
    o->alphainit = 2.0;
    o->stop_difff = 1;
    o->stop_normgp = 0;
    o->stop_normgp_normb = 0;
    o->stop_Anormgp = 0;
    o->stop_Anormgp_normb = 0;
}

void pasc_oracle_ts_default_opts(pasc_oracle_ts_opts *o)
{
    /* include/general/solver/tssolver.h:13-15 */
    o->maxit = 300;
    o->eps = 1e-6;
    o->init_permute = 1;
    o->annealing = 1;
    o->relative = 0;
    o->thetasolved = 0;
}

/* ------------------------------------------------------------------------------------- */
/* vector primitives in PETSc's host semantics                                            */
/* ------------------------------------------------------------------------------------- */

/* VecDot(x, y) for real vectors: sum_i x_i*y_i, sequential. */
static double vdot(const double *x, const double *y, long n, int nth)
{
    if (nth <= 1) {
        double s = 0.0;
        for (long i = 0; i < n; i++) s += x[i] * y[i];
        return s;
    }
    double part[256];
    int nt = nth > 256 ? 256 : nth;
    int used = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
        int id = 0, cnt = 1;
#ifdef _OPENMP
        id = omp_get_thread_num();
        cnt = omp_get_num_threads();
#endif
        long lo = n * id / cnt, hi = n * (id + 1) / cnt;
        double s = 0.0;
        for (long i = lo; i < hi; i++) s += x[i] * y[i];
        part[id] = s;
        if (id == 0) used = cnt;
    }
    double tot = 0.0;
    for (int j = 0; j < used; j++) tot += part[j];
    return tot;
}

/* VecAXPY(y, a, x): y_i = y_i + a*x_i */
static void vaxpy(double *y, double a, const double *x, long n, int nth)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long i = 0; i < n; i++) y[i] = y[i] + a * x[i];
}

/* VecScale(y, a): y_i = a*y_i */
static void vscale(double *y, double a, long n, int nth)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long i = 0; i < n; i++) y[i] = a * y[i];
}

static void vcopy(double *dst, const double *src, long n, int nth)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long i = 0; i < n; i++) dst[i] = src[i];
}

/* ------------------------------------------------------------------------------------- */
/* simplex projection                                                                     */
/* include/general/algebra/feasibleset/simplex_local.h:153-249 (host project_sub) and     */
/* src/petscvector/algebra/feasibleset/simplex_local.cu:48-139 (same algorithm on device) */
/* ------------------------------------------------------------------------------------- */

/* Bubble sort with last-swap bound, ascending, stable: simplex_local.h:153-173 */
static void sort_bubble(double *y, int n)
{
    int m = n;
    while (m > 0) {
        int mnew = 0;
        for (int i = 1; i < m; i++) {
            if (y[i] < y[i - 1]) {
                double sw = y[i];
                y[i] = y[i - 1];
                y[i - 1] = sw;
                mnew = i;
            }
        }
        m = mnew;
    }
}

/* One t-block of K values: simplex_local.h:176-246 */
static void project_block(double *x, int K, double *y)
{
    int inside = 1;
    double sum = 0.0;
    for (int k = 0; k < K; k++) {
        if (x[k] < 0.0) inside = 0;
        sum += x[k];
    }
    if (sum != 1) inside = 0; /* exact equality test, simplex_local.h:195 */
    if (inside) return;

    for (int k = 0; k < K; k++) y[k] = x[k];
    sort_bubble(y, K);

    double t_hat = 0.0;
    int i = K - 1;
    while (i >= 1) {
        double sum_y = 0.0;
        for (int j = i; j < K; j++) sum_y += y[j]; /* recomputed from y[i] upwards */
        double ti = (sum_y - 1.0) / (double)(K - i);
        if (ti >= y[i - 1]) {
            t_hat = ti;
            i = -1;
        } else {
            i = i - 1;
        }
    }
    if (i == 0) t_hat = (sum - 1.0) / (double)K; /* sum over the unsorted block */

    for (int k = 0; k < K; k++) {
        double ti = x[k] - t_hat;
        x[k] = ti > 0.0 ? ti : 0.0;
    }
}

void pasc_oracle_project(double *x, long T, int K, int nthreads)
{
    int nth = eff_threads(nthreads);
#ifdef _OPENMP
#pragma omp parallel num_threads(nth) if (nth > 1)
#endif
    {
        double ystack[ORACLE_KMAX_STACK];
        double *y = K <= ORACLE_KMAX_STACK ? ystack : (double *)malloc(sizeof(double) * (size_t)K);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (long t = 0; t < T; t++) project_block(x + t * (long)K, K, y);
        if (y != ystack) free(y);
    }
}

/* ------------------------------------------------------------------------------------- */
/* FEM-H1 operator                                                                        */
/* Assembly: src/petscvector/algebra/matrix/blockgraphsparse.cpp:51-109 with R = 1 and a  */
/* graph without edges (graphh1fem.cpp:35-46): diagonal Wsum = 2 at t in {0,T-1}, 4       */
/* inside, 0 when T == 1; off-diagonals -2 at column t-1 and t+1 (stride K).              */
/* Product: MatMult row by row over columns in ascending order starting from 0.0, then    */
/* VecScale by the coefficient (spgqpsolver.cpp:122-123,164-165).                          */
/* ------------------------------------------------------------------------------------- */
/* y = A x with A = coeff * A_hat, or with kc != NULL the block k scaled by kc[k] instead of coeff
 * (BlockGraphSparseMatrix with coefficients, blockgraphsparse.cpp:161-185: VecScale of the
 * MatMult's block k by alpha*theta_k*theta_k) */
static void matmult_g(const double *x, double *y, long T, int K, double coeff, const double *kc,
                      const pasc_oracle_graph *G, int nthreads);
static void matmult_kc(const double *x, double *y, long T, int K, double coeff, const double *kc, int nthreads)
{
    matmult_g(x, y, T, K, coeff, kc, NULL, nthreads);
}

void pasc_oracle_fem_h1_matmult(const double *x, double *y, long T, int K, double coeff, int nthreads)
{
    matmult_kc(x, y, T, K, coeff, NULL, nthreads);
}

void pasc_oracle_fem_h1_matmult_kc(const double *x, double *y, long T, int K, const double *kc, int nthreads)
{
    matmult_kc(x, y, T, K, 0.0, kc, nthreads);
}

/* Row (t, r, k) of the assembled BlockGraphSparseMatrix with a graph of R nodes
 * (blockgraphsparse.cpp:48-103): diagonal Wsum = 3m+4 inside, 2m+2 at t = 0 or T-1, m when
 * T = 1 (m = number of neighbours of r); -2 at (t+-1, r); -1 at (t, r') and (t+-1, r') for
 * every neighbour r'.  PETSc keeps the columns of a row sorted, and MatMult sums them in that
 * order from 0: here t' = t-1, t, t+1 and, inside each, r' ascending (neighbour lists are
 * sorted, r itself merged in).  Without neighbours (R = 1) this is the 1-D row below. */
static void graph_rows(const double *x, double *y, long T, int K, const pasc_oracle_graph *G, int nth)
{
    const long R = G->R;
    const long N = T * R * (long)K;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long i = 0; i < N; i++) {
        const long s = i / K;
        const int k = (int)(i - s * K);
        const long t = s / R, r = s - t * R;
        const int q0 = G->ptr[r], q1 = G->ptr[r + 1], m = q1 - q0;
        double wsum;
        if (t == 0 || t == T - 1) wsum = T > 1 ? (double)(2 * m + 2) : (double)m;
        else wsum = (double)(3 * m + 4);
        double sum = 0.0;
        for (long tt = t - 1; tt <= t + 1; tt++) {
            if (tt < 0 || tt >= T) continue;
            int q = q0, self = 0;
            while (q < q1 || !self) {
                long rn;
                double v;
                if (!self && (q >= q1 || G->idx[q] > r)) {
                    rn = r;
                    v = tt == t ? wsum : -2.0;
                    self = 1;
                } else {
                    rn = G->idx[q++];
                    v = -1.0;
                }
                sum += v * x[(tt * R + rn) * K + k];
            }
        }
        y[i] = sum;
    }
}

static void matmult_g(const double *x, double *y, long T, int K, double coeff, const double *kc,
                      const pasc_oracle_graph *G, int nthreads)
{
    int nth = eff_threads(nthreads);
    long N = T * (long)K * (G ? G->R : 1);
    if (G) {
        graph_rows(x, y, T, K, G, nth);
        if (!kc) vscale(y, coeff, N, nth);
        else
            for (long i = 0; i < N; i++) y[i] = kc[i % K] * y[i];
        return;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long i = 0; i < N; i++) {
        long t = i / K;
        double sum = 0.0;
        if (T == 1) {
            sum += 0.0 * x[i];
        } else {
            double wsum = (t == 0 || t == T - 1) ? 2.0 : 4.0;
            if (t > 0) sum += -2.0 * x[i - K];
            sum += wsum * x[i];
            if (t < T - 1) sum += -2.0 * x[i + K];
        }
        y[i] = sum;
    }
    if (!kc) {
        vscale(y, coeff, N, nth);
        return;
    }
    for (long i = 0; i < N; i++) y[i] = kc[i % K] * y[i];
}

double pasc_oracle_A_coeff(double epssqr, long T, int scalef)
{
    /* graphh1fem.cpp:146-151 and graphh1fem.h:293-298 (T_reduced == T) */
    double coeff = epssqr;
    if (scalef) coeff *= (1.0 / ((double)T));
    else coeff *= ((double)T / ((double)T));
    return coeff;
}

double pasc_oracle_b_coeff(long T, int scalef)
{
    /* graphh1fem.cpp:280-283 */
    double coeff = -1.0;
    if (scalef) coeff *= (1.0 / ((double)T));
    return coeff;
}

/* graphh1fem.cpp:258-264 (xdim = 1) followed by VecScale(b, bscale) at :286.
 * For xdim > 1 the residual is the squared Euclidean distance summed over j in order. */
void pasc_oracle_residual_b(const double *data, const double *theta, double *b, long T, int K,
                            int xdim, double bscale, int nthreads)
{
    int nth = eff_threads(nthreads);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nth) if (nth > 1)
#endif
    for (long t = 0; t < T; t++) {
        for (int k = 0; k < K; k++) {
            double r;
            if (xdim == 1) {
                double dv = data[t] - theta[k];
                r = dv * dv;
            } else {
                r = 0.0;
                for (int j = 0; j < xdim; j++) {
                    double dv = data[t * (long)xdim + j] - theta[k * (long)xdim + j];
                    r += dv * dv;
                }
            }
            b[t * (long)K + k] = r;
        }
    }
    vscale(b, bscale, T * (long)K, nth);
}

/* graphh1fem.cpp:347-380, usethetainpenalty = false: per k, VecDot(data, gamma_k) and
 * VecSum(gamma_k) over the stride-K sub-vector, theta_k = ratio or 0. */
void pasc_oracle_theta_update(const double *gamma, const double *data, double *theta, long T,
                              int K, int xdim, int nthreads)
{
    /* One task per (k, block of up to 16 channels): every sum runs over t in ascending order
     * on one thread, so the result does not depend on the thread count. */
    int nth = eff_threads(nthreads);
    const int JB = 16;
    const int njb = (xdim + JB - 1) / JB;
    const long ntask = (long)K * njb;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth) if (nth > 1)
#endif
    for (long task = 0; task < ntask; task++) {
        const int k = (int)(task / njb);
        const int j0 = (int)(task % njb) * JB;
        const int nj = (xdim - j0 < JB) ? xdim - j0 : JB;
        double gsum = 0.0;
        for (long t = 0; t < T; t++) gsum += gamma[t * (long)K + k];
        double gx[16];
        for (int j = 0; j < nj; j++) gx[j] = 0.0;
        for (long t = 0; t < T; t++) {
            const double gk = gamma[t * (long)K + k];
            const double *row = data + t * (long)xdim + j0;
            for (int j = 0; j < nj; j++) gx[j] += row[j] * gk;
        }
        for (int j = 0; j < nj; j++) theta[k * (long)xdim + j0 + j] = (gsum != 0) ? gx[j] / gsum : 0.0;
    }
}

/* src/petscvector/common/decomposition.cpp:280-356 with R = 1, one rank:
 * new[t*K + k] = orig[k*T + t]. */
void pasc_oracle_permute_blocked_to_interleaved(const double *orig, double *out, long T, int K)
{
    for (int k = 0; k < K; k++)
        for (long t = 0; t < T; t++) out[t * (long)K + k] = orig[k * T + t];
}

/* ------------------------------------------------------------------------------------- */
/* GLL memory: src/general/solver/spg_fs.cpp:7-63                                         */
/* ------------------------------------------------------------------------------------- */
typedef struct {
    int m;
    int last_idx;
    double *fs;
} spg_fs;

static void fs_init(spg_fs *s, double fx)
{
    for (int i = 0; i < s->m; i++) s->fs[i] = fx;
    s->last_idx = 0;
}

static double fs_get_max(const spg_fs *s)
{
    double mx = s->fs[0];
    for (int i = 0; i < s->m; i++)
        if (s->fs[i] > mx) mx = s->fs[i];
    return mx;
}

static void fs_update(spg_fs *s, double fx)
{
    s->last_idx++;
    if (s->last_idx >= s->m) s->last_idx = 0;
    s->fs[s->last_idx] = fx;
}

/* ------------------------------------------------------------------------------------- */
/* SPG-QP: src/petscvector/solver/spgqpsolver.cpp:55-312, get_fx :316-345,                */
/* compute_dots :348-367 (three separate VecDot calls).                                   */
/* ------------------------------------------------------------------------------------- */
static double get_fx(const double *g, const double *b, const double *x, double *temp, long n, int nth)
{
    vcopy(temp, g, n, nth);      /* VecCopy(g, temp)        :336 */
    vaxpy(temp, -1.0, b, n, nth); /* VecAXPY(temp, -1, b)   :337 */
    double tempt = vdot(x, temp, n, nth); /* VecDot(x, temp) :338 */
    return 0.5 * tempt;
}

static int spgqp_impl(const double *b, double *x, long T, int K, double coeff, const double *kc,
                      const pasc_oracle_graph *G, const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r,
                      double *trace, int nthreads);

int pasc_oracle_spgqp_solve_graph(const double *b, double *x, long T, int K, double coeff, const pasc_oracle_graph *G,
                                  const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads)
{
    return spgqp_impl(b, x, T, K, coeff, NULL, G, o, r, NULL, nthreads);
}

void pasc_oracle_graph_matmult(const double *x, double *y, long T, int K, double coeff, const pasc_oracle_graph *G,
                               int nthreads)
{
    matmult_g(x, y, T, K, coeff, NULL, G, nthreads);
}

int pasc_oracle_spgqp_solve(const double *b, double *x, long T, int K, double coeff,
                            const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r,
                            double *trace, int nthreads)
{
    return spgqp_impl(b, x, T, K, coeff, NULL, NULL, o, r, trace, nthreads);
}

int pasc_oracle_spgqp_solve_kc(const double *b, double *x, long T, int K, const double *kc,
                               const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads)
{
    return spgqp_impl(b, x, T, K, 0.0, kc, NULL, o, r, NULL, nthreads);
}

/* T: timesteps; with a graph the QP has T*R blocks of K (index (t*R + r)*K + k) */
static int spgqp_impl(const double *b, double *x, long T, int K, double coeff, const double *kc,
                      const pasc_oracle_graph *G, const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r,
                      double *trace, int nthreads)
{
    int nth = eff_threads(nthreads);
    const long nb = T * (G ? G->R : 1); /* blocks of K */
    long n = nb * (long)K;
    double *g = (double *)malloc(sizeof(double) * (size_t)n);
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    double *Ad = (double *)malloc(sizeof(double) * (size_t)n);
    double *temp = (double *)malloc(sizeof(double) * (size_t)n);
    spg_fs fs;
    fs.m = o->m;
    fs.last_idx = 0;
    fs.fs = (double *)malloc(sizeof(double) * (size_t)(o->m > 0 ? o->m : 1));
    if (!g || !d || !Ad || !temp || !fs.fs) {
        free(g); free(d); free(Ad); free(temp); free(fs.fs);
        return -1;
    }

    int it = 0, hessmult = 0;
    double fx, fx_old, fx_max, xi, beta_bar, beta_hat, beta = 0.0, dd = 0.0, gd = 0.0, dAd = 0.0, alpha_bb;

    double normb = sqrt(vdot(b, b, n, nth)); /* VecNorm(b, NORM_2)  :104 */
    alpha_bb = o->alphainit;                 /* :108 */

    pasc_oracle_project(x, nb, K, nth); /* :116 */

    matmult_g(x, g, T, K, coeff, kc, G, nth); /* MatMult + VecScale :122-123 */
    hessmult += 1;
    vaxpy(g, -1.0, b, n, nth); /* :128 */

    fx = get_fx(g, b, x, temp, n, nth); /* :133 */
    fx_old = DBL_MAX;
    fs_init(&fs, fx);
    if (trace) {
        trace[0] = fx;
        for (int q = 1; q < 8; q++) trace[q] = 0.0;
    }

    while (it < o->maxit) {
        it += 1;

        vcopy(d, x, n, nth);              /* :146 */
        vaxpy(d, -alpha_bb, g, n, nth);   /* :147 */
        pasc_oracle_project(d, nb, K, nth); /* :153 */
        vaxpy(d, -1.0, x, n, nth);        /* :158 */

        matmult_g(d, Ad, T, K, coeff, kc, G, nth); /* :164-165 */
        hessmult += 1;

        dd = vdot(d, d, n, nth);  /* :357 */
        dAd = vdot(d, Ad, n, nth); /* :360 */
        gd = vdot(d, g, n, nth);  /* :363 */

        fx_max = fs_get_max(&fs); /* :176 */

        /* :182-195 */
        xi = (fx_max - fx) / dAd;
        beta_bar = -gd / dAd;
        beta_hat = o->gamma * beta_bar + sqrt(o->gamma * o->gamma * beta_bar * beta_bar + 2 * xi);
        if (beta_hat < o->sigma1) beta_hat = o->sigma1;
        if (beta_hat < o->sigma2) beta = beta_hat;
        else beta = o->sigma2;

        vaxpy(x, beta, d, n, nth);  /* :200 */
        vaxpy(g, beta, Ad, n, nth); /* :201 */

        fx_old = fx;                          /* :207 */
        fx = get_fx(g, b, x, temp, n, nth);   /* :209 */
        fs_update(&fs, fx);                   /* :210 */

        alpha_bb = dd / dAd; /* :216 */

        if (trace) {
            double *row = trace + 8 * (long)it;
            row[0] = fx;
            row[1] = dd;
            row[2] = dAd;
            row[3] = gd;
            row[4] = fx_max;
            row[5] = beta;
            row[6] = alpha_bb;
            row[7] = 0.0;
        }

        /* :260-274 */
        if (o->stop_difff && fabs(fx - fx_old) < o->eps) break;
        if (o->stop_normgp && dd < o->eps) break;
        if (o->stop_normgp_normb && dd < o->eps * normb) break;
        if (o->stop_Anormgp && dAd < o->eps) break;
        if (o->stop_Anormgp_normb && dAd < o->eps * normb) break;
    }

    if (r) {
        r->it = it;
        r->hessmult = hessmult;
        r->fx = fx;
        r->gP = dd;
        r->dAd = dAd;
        r->normb = normb;
    }
    free(g); free(d); free(Ad); free(temp); free(fs.fs);
    return 0;
}

/* ------------------------------------------------------------------------------------- */
/* TSSolver::solve: include/general/solver/tssolver.h:492-715 with the GraphH1FEMModel    */
/* hooks of src/petscvector/model/graphh1fem.cpp (fem not reduced, R = 1).                */
/* ------------------------------------------------------------------------------------- */
int pasc_oracle_tssolver_solve(const double *data, double *gamma, double *theta, long T, int K,
                               int xdim, double epssqr, int scalef,
                               const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                               const double *gamma_restart, pasc_oracle_ts_result *r,
                               double *trace_L, int nthreads)
{
    int nth = eff_threads(nthreads);
    long n = T * (long)K;
    double *b = (double *)malloc(sizeof(double) * (size_t)n);
    double *perm = (double *)malloc(sizeof(double) * (size_t)n);
    double *gbest = NULL, *tbest = NULL;
    int annealing = ts->annealing > 0 ? ts->annealing : 1;
    if (annealing > 1) {
        gbest = (double *)malloc(sizeof(double) * (size_t)n);
        tbest = (double *)malloc(sizeof(double) * (size_t)K * (size_t)xdim);
    }
    if (!b || !perm || (annealing > 1 && (!gbest || !tbest))) {
        free(b); free(perm); free(gbest); free(tbest);
        return -1;
    }

    double coeffA = pasc_oracle_A_coeff(epssqr, T, scalef);
    double coeffB = pasc_oracle_b_coeff(T, scalef);
    double best_aic = DBL_MAX; /* TSData aic starts at max */
    int it_sum = 0, spg_it_sum = 0, spg_hm_sum = 0, increased = 0;
    double keepL = DBL_MAX, keepdL = DBL_MAX, keepaic = DBL_MAX;
    int keepit = 0;
    long trace_pos = 0;

    for (int a = 0; a < annealing; a++) {
        if (ts->init_permute) { /* :528-530 */
            pasc_oracle_permute_blocked_to_interleaved(gamma, perm, T, K);
            memcpy(gamma, perm, sizeof(double) * (size_t)n);
        }
        double L = DBL_MAX, L_old, deltaL = DBL_MAX;
        int it;
        for (it = 0; it < ts->maxit; it++) {
            if (!ts->thetasolved) /* :550 */
                pasc_oracle_theta_update(gamma, data, theta, T, K, xdim, nth);

            pasc_oracle_residual_b(data, theta, b, T, K, xdim, coeffB, nth); /* :586 */
            pasc_oracle_spg_result sr;
            pasc_oracle_spgqp_solve(b, gamma, T, K, coeffA, spg, &sr, NULL, nth); /* :590 */
            spg_it_sum += sr.it;
            spg_hm_sum += sr.hessmult;

            L_old = L; /* :618-620 */
            L = sr.fx;
            deltaL = fabs(L - L_old);
            if (trace_L) trace_L[trace_pos++] = L;
            if (L - L_old > 0) increased++; /* :637-639 prints ERROR and continues */
            if (ts->relative ? (deltaL < ts->eps * fabs(L)) : (deltaL < ts->eps)) break;
        }
        it_sum += it;
        double aic = 2 * log(L) + K; /* graphh1fem.h:444-447 */
        if ((annealing <= 1) || (aic < best_aic && annealing > 1)) {
            if (aic < best_aic && annealing > 1) {
                memcpy(gbest, gamma, sizeof(double) * (size_t)n);
                memcpy(tbest, theta, sizeof(double) * (size_t)K * (size_t)xdim);
            }
            best_aic = aic;
            keepL = L;
            keepdL = deltaL;
            keepaic = aic;
            keepit = it;
        }
        if (a < annealing - 1 && gamma_restart) /* :700-702 set_random */
            memcpy(gamma, gamma_restart, sizeof(double) * (size_t)n);
    }
    if (annealing > 1) {
        memcpy(gamma, gbest, sizeof(double) * (size_t)n);
        memcpy(theta, tbest, sizeof(double) * (size_t)K * (size_t)xdim);
    }
    if (r) {
        r->it_last = keepit;
        r->it_sum = it_sum;
        r->spg_it_sum = spg_it_sum;
        r->spg_hessmult_sum = spg_hm_sum;
        r->L = keepL;
        r->deltaL = keepdL;
        r->aic = keepaic;
        r->L_increased = increased;
    }
    free(b); free(perm); free(gbest); free(tbest);
    return 0;
}

/* src/petscvector/data/signal1Ddata.cpp:134-191: NORM_1 of -solution + sum_k theta_k gamma_k,
 * accumulated k by k with VecAXPY. */
double pasc_oracle_abserr_reconstructed(const double *gamma, const double *theta,
                                        const double *solution, long T, int K)
{
    double s = 0.0;
    for (long t = 0; t < T; t++) {
        double v = -solution[t];
        for (int k = 0; k < K; k++) v = v + theta[k] * gamma[t * (long)K + k];
        s += fabs(v);
    }
    return s;
}

/* True argmax (lowest k wins ties).  The reference's TSData::cutgamma
 * (src/petscvector/data/tsdata.cpp:208-221) seeds the running maximum with gamma_arr[t]
 * instead of gamma_arr[t*K]; this helper follows the intended argmax. */
void pasc_oracle_argmax_labels(const double *gamma, int *labels, long T, int K)
{
    for (long t = 0; t < T; t++) {
        int best = 0;
        double bv = gamma[t * (long)K];
        for (int k = 1; k < K; k++) {
            double v = gamma[t * (long)K + k];
            if (v > bv) {
                bv = v;
                best = k;
            }
        }
        labels[t] = best;
    }
}

/* ------------------------------------------------------------------------------------
 * adjoint (no reference counterpart; see the header)
 * ---------------------------------------------------------------------------------- */

double pasc_oracle_recon_mse(const double *gamma, const double *theta, const double *clean, long T,
                             int K, double *dgamma, double *dtheta)
{
    double loss = 0.0;
    if (dtheta)
        for (int k = 0; k < K; k++) dtheta[k] = 0.0;
    for (long t = 0; t < T; t++) {
        double rec = 0.0;
        for (int k = 0; k < K; k++) rec += gamma[t * (long)K + k] * theta[k];
        double e = rec - clean[t];
        loss += e * e;
        for (int k = 0; k < K; k++) {
            if (dgamma) dgamma[t * (long)K + k] = 2.0 / (double)T * e * theta[k];
            if (dtheta) dtheta[k] += 2.0 / (double)T * e * gamma[t * (long)K + k];
        }
    }
    return loss / (double)T;
}

/* P at one timestep, in place */
static void adj_proj(double *v, const unsigned char *fr, int K)
{
    int nf = 0;
    double s = 0.0;
    for (int k = 0; k < K; k++)
        if (fr[k]) {
            nf++;
            s += v[k];
        }
    if (nf <= 1) {
        for (int k = 0; k < K; k++) v[k] = 0.0;
        return;
    }
    double mean = s / nf;
    for (int k = 0; k < K; k++) v[k] = fr[k] ? v[k] - mean : 0.0;
}

/* y = P (coeff A_hat) v for v in S */
static void adj_apply(const double *v, double *y, const unsigned char *fr, long T, int K, double coeff)
{
    for (long t = 0; t < T; t++) {
        for (int k = 0; k < K; k++) {
            long i = t * (long)K + k;
            double a = 0.0;
            if (t > 0) a += 2.0 * (v[i] - v[i - K]);
            if (t < T - 1) a += 2.0 * (v[i] - v[i + K]);
            y[i] = coeff * a;
        }
        adj_proj(y + t * (long)K, fr + t * (long)K, K);
    }
}

int pasc_oracle_adjoint(const double *gamma, const double *data, const double *theta,
                        const double *dloss_dgamma, long T, int K, double coeff, double dcoeff,
                        double bscale, const pasc_oracle_adj_opts *o, double *lambda,
                        double *dloss_depssqr, double *dloss_ddata, double *dloss_dtheta,
                        pasc_oracle_adj_result *res)
{
    const long N = T * (long)K;
    unsigned char *fr = (unsigned char *)malloc((size_t)N);
    double *lam = (double *)calloc((size_t)N, sizeof(double));
    double *r = (double *)malloc(sizeof(double) * (size_t)N);
    double *p = (double *)malloc(sizeof(double) * (size_t)N);
    double *q = (double *)malloc(sizeof(double) * (size_t)N);
    if (!fr || !lam || !r || !p || !q) {
        free(fr); free(lam); free(r); free(p); free(q);
        return -1;
    }
    /* free sets from one projected-gradient step z = Proj(gamma - a (A gamma - b)),
     * a = 1/(8 coeff + |bscale|); z = gamma at an exact solution */
    const double a = 1.0 / (8.0 * coeff + fabs(bscale));
    double z[64], zs[64];
    long free_dims = 0;
    double rr = 0.0;
    if (K > 64) {
        free(fr); free(lam); free(r); free(p); free(q);
        return -1;
    }
    for (long t = 0; t < T; t++) {
        int nf = 0;
        for (int k = 0; k < K; k++) {
            long i = t * (long)K + k;
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gamma[i] - gamma[i - K]);
            if (t < T - 1) ag += 2.0 * (gamma[i] - gamma[i + K]);
            double res = data[t] - theta[k];
            z[k] = gamma[i] - a * (coeff * ag - bscale * res * res);
        }
        project_block(z, K, zs);
        for (int k = 0; k < K; k++) {
            long i = t * (long)K + k;
            fr[i] = z[k] > o->act_tol;
            nf += fr[i];
            r[i] = dloss_dgamma[i];
        }
        free_dims += nf > 1 ? nf - 1 : 0;
        adj_proj(r + t * (long)K, fr + t * (long)K, K);
        for (int k = 0; k < K; k++) rr += r[t * (long)K + k] * r[t * (long)K + k];
    }
    const double rr0 = rr;
    int it = 0, status = rr0 > 0.0 ? 0 : 1;
    for (long i = 0; i < N; i++) p[i] = r[i];
    while (status == 0) {
        if (it >= o->cg_maxit) {
            status = 2;
            break;
        }
        adj_apply(p, q, fr, T, K, coeff);
        double pq = 0.0;
        for (long i = 0; i < N; i++) pq += p[i] * q[i];
        if (!(pq > 0.0) || !isfinite(pq)) {
            status = 4;
            break;
        }
        double alpha = rr / pq, rrn = 0.0;
        for (long i = 0; i < N; i++) {
            lam[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            rrn += r[i] * r[i];
        }
        it++;
        double beta = rrn / rr;
        rr = rrn;
        if (rr <= o->cg_tol * o->cg_tol * rr0) {
            status = 1;
            break;
        }
        for (long i = 0; i < N; i++) p[i] = r[i] + beta * p[i];
    }
    double deps = 0.0;
    if (dloss_dtheta)
        for (int k = 0; k < K; k++) dloss_dtheta[k] = 0.0;
    for (long t = 0; t < T; t++) {
        double dx = 0.0;
        for (int k = 0; k < K; k++) {
            long i = t * (long)K + k;
            double ag = 0.0;
            if (t > 0) ag += 2.0 * (gamma[i] - gamma[i - K]);
            if (t < T - 1) ag += 2.0 * (gamma[i] - gamma[i + K]);
            deps += lam[i] * ag;
            double db = 2.0 * bscale * (data[t] - theta[k]);
            dx += lam[i] * db;
            if (dloss_dtheta) dloss_dtheta[k] -= lam[i] * db;
        }
        if (dloss_ddata) dloss_ddata[t] = dx;
    }
    if (dloss_depssqr) *dloss_depssqr = -dcoeff * deps;
    if (lambda)
        for (long i = 0; i < N; i++) lambda[i] = lam[i];
    if (res) {
        res->cg_it = it;
        res->status = status;
        res->free_dims = free_dims;
        res->cg_relres = rr0 > 0.0 ? sqrt(rr / rr0) : 0.0;
    }
    free(fr); free(lam); free(r); free(p); free(q);
    return status == 4 ? 1 : 0;
}

/* ------------------------------------------------------------------------------------
 * FEM temporal coarsening (see the header)
 * ---------------------------------------------------------------------------------- */

/* src/petscvector/common/fem.cpp:196-215 (compute_decomposition_reduced) */
long pasc_oracle_fem_T_reduced(long T, double fem_reduce)
{
    if (fem_reduce < 1.0) return (long)ceil((double)T * fem_reduce);
    return T;
}

static double fem_diff(long T1, long T2, int type)
{
    if (type == 0) return (double)T1 / (double)T2;                 /* fem.cpp:15 */
    return (double)(T1 - 1) / (double)(T2 - 1);                     /* femhat.cpp:17 */
}

void pasc_oracle_fem_reduce(const double *g1, double *g2, long T1, long T2, int K, int type)
{
    const double diff = fem_diff(T1, T2, type);
    if (type == 0) {
        /* fem.cpp:64-70 */
        for (int k = 0; k < K; k++)
            for (long t2 = 0; t2 < T2; t2++) {
                double mysum = 0.0;
                for (long i = (long)round(t2 * diff); i < (long)round((t2 + 1) * diff); i++)
                    mysum += g1[i * (long)K + k];
                g2[t2 * (long)K + k] = mysum;
            }
        return;
    }
    /* femhat.cpp:64-100 with left_t1_idx = 0 and right_t1_idx = floor(diff*(T2-1))
     * (femhat.h:170-180 on one rank) */
    const long right_t1_idx = (long)floor(diff * (double)(T2 - 1));
    for (int k = 0; k < K; k++)
        for (long t2 = 0; t2 < T2; t2++) {
            const double center_t1 = t2 * diff;
            const double left_t1 = (t2 - 1) * diff;
            const double right_t1 = (t2 + 1) * diff;
            long id_counter = (long)floor(left_t1);
            long t1 = (long)floor(left_t1);
            double mysum = 0.0;
            while (t1 <= center_t1) {
                const double phi = (t1 - left_t1) / (center_t1 - left_t1);
                if (id_counter >= 0) mysum += phi * g1[id_counter * (long)K + k];
                t1 += 1;
                id_counter += 1;
            }
            while (t1 < right_t1) {
                const double phi = (t1 - right_t1) / (center_t1 - right_t1);
                if (id_counter < right_t1_idx) mysum += phi * g1[id_counter * (long)K + k];
                t1 += 1;
                id_counter += 1;
            }
            g2[t2 * (long)K + k] = mysum;
        }
}

void pasc_oracle_fem_prolongate(const double *g2, double *g1, long T1, long T2, int K, int type)
{
    const double diff = fem_diff(T1, T2, type);
    if (type == 0) {
        /* fem.cpp:142-147 */
        for (int k = 0; k < K; k++)
            for (long t2 = 0; t2 < T2; t2++)
                for (long i = (long)round(t2 * diff); i < (long)round((t2 + 1) * diff); i++)
                    g1[i * (long)K + k] = g2[t2 * (long)K + k];
        return;
    }
    /* femhat.cpp:150-171 with Tbegin1 = left_t2_idx = 0 */
    for (int k = 0; k < K; k++)
        for (long t1 = 0; t1 < T1; t1++) {
            const long l = (long)floor(t1 / diff), r = l + 1;
            const double t1_left = l * diff, t1_right = r * diff;
            const double phi_l = (t1 - t1_left) / (t1_right - t1_left);
            const double phi_r = (t1 - t1_right) / (t1_left - t1_right);
            const double gr = r < T2 ? g2[r * (long)K + k] : 0.0;
            const double gl = l < T2 ? g2[l * (long)K + k] : 0.0;
            double v = 0.0;
            v += phi_l * gr;
            v += phi_r * gl;
            g1[t1 * (long)K + k] = v;
        }
}

/* GraphH1FEMModel::updatebeforesolve_thetasolver with usethetainpenalty
 * (src/petscvector/model/graphh1fem.cpp:306-380): theta is set to 1, Agamma = A gamma with
 * that theta (block k scaled by alpha*1*1), and theta_k = (c gamma_k'x) / (c sum gamma_k +
 * gamma_k'Agamma_k / 2) with c = 1 (0 when the denominator is 0). */
void pasc_oracle_theta_update_penalty(const double *gamma, const double *data, double *theta, long T, int K,
                                      double alpha)
{
    const long N = T * (long)K;
    double *kc = (double *)malloc(sizeof(double) * (size_t)K);
    double *Ag = (double *)malloc(sizeof(double) * (size_t)N);
    if (!kc || !Ag) {
        free(kc); free(Ag);
        return;
    }
    for (int k = 0; k < K; k++) kc[k] = alpha * 1.0 * 1.0;
    matmult_kc(gamma, Ag, T, K, 0.0, kc, 1);
    for (int k = 0; k < K; k++) {
        double gAg = 0.0, gx = 0.0, gs = 0.0;
        for (long t = 0; t < T; t++) gAg += gamma[t * (long)K + k] * Ag[t * (long)K + k];
        for (long t = 0; t < T; t++) gx += data[t] * gamma[t * (long)K + k];
        for (long t = 0; t < T; t++) gs += gamma[t * (long)K + k];
        const double c = 1.0;
        theta[k] = (c * gs + 0.5 * gAg != 0) ? (c * gx) / (c * gs + 0.5 * gAg) : 0.0;
    }
    free(kc); free(Ag);
}

int pasc_oracle_tssolver_solve_fem(const double *data, double *gamma, double *theta, long T, int K,
                                   double epssqr, int scalef, double fem_reduce, int fem_type,
                                   const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                                   pasc_oracle_ts_result *r, int nthreads)
{
    return pasc_oracle_tssolver_solve_model(data, gamma, theta, T, K, epssqr, scalef, fem_reduce, fem_type, 0, ts,
                                            spg, r, nthreads);
}

int pasc_oracle_tssolver_solve_model(const double *data, double *gamma, double *theta, long T, int K,
                                     double epssqr, int scalef, double fem_reduce, int fem_type,
                                     int usethetainpenalty, const pasc_oracle_ts_opts *ts,
                                     const pasc_oracle_spg_opts *spg, pasc_oracle_ts_result *r, int nthreads)
{
    const int nth = eff_threads(nthreads);
    const long T2 = pasc_oracle_fem_T_reduced(T, fem_reduce);
    const long n = T * (long)K, n2 = T2 * (long)K;
    double *res = (double *)malloc(sizeof(double) * (size_t)n);
    double *perm = (double *)malloc(sizeof(double) * (size_t)n);
    double *b2 = (double *)malloc(sizeof(double) * (size_t)n2);
    double *x2 = (double *)malloc(sizeof(double) * (size_t)n2);
    if (!res || !perm || !b2 || !x2) {
        free(res); free(perm); free(b2); free(x2);
        return -1;
    }
    /* graphh1fem.cpp:145-151 (A, with the original T) and :280-283 (b, with T2) */
    double coeffA = epssqr;
    if (scalef) coeffA *= (1.0 / ((double)T));
    else coeffA *= ((double)T2 / ((double)T));
    double coeffB = -1.0;
    if (scalef) coeffB *= (1.0 / ((double)T2));

    if (ts->init_permute) {
        pasc_oracle_permute_blocked_to_interleaved(gamma, perm, T, K);
        memcpy(gamma, perm, sizeof(double) * (size_t)n);
    }
    double L = DBL_MAX, L_old, deltaL = DBL_MAX;
    int it, spg_it_sum = 0, spg_hm_sum = 0, increased = 0;
    double kc[64];
    if (usethetainpenalty && (K > 64 || fem_reduce < 1.0)) {
        free(res); free(perm); free(b2); free(x2);
        return -1; /* the reference's theta step multiplies the reduced A with the full gamma */
    }
    for (it = 0; it < ts->maxit; it++) {
        if (!ts->thetasolved) {
            if (usethetainpenalty) pasc_oracle_theta_update_penalty(gamma, data, theta, T, K, coeffA);
            else pasc_oracle_theta_update(gamma, data, theta, T, K, 1, nth);
        }
        if (usethetainpenalty)
            for (int k = 0; k < K; k++) kc[k] = coeffA * theta[k] * theta[k]; /* blockgraphsparse.cpp:177 */
        pasc_oracle_residual_b(data, theta, res, T, K, 1, 1.0, nth);      /* graphh1fem.cpp:258-267 */
        pasc_oracle_fem_reduce(res, b2, T, T2, K, fem_type);               /* :275 */
        pasc_oracle_fem_reduce(gamma, x2, T, T2, K, fem_type);             /* :276 */
        for (long i = 0; i < n2; i++) b2[i] *= coeffB;                     /* :280-286 */
        pasc_oracle_spg_result sr;
        if (usethetainpenalty) pasc_oracle_spgqp_solve_kc(b2, x2, T2, K, kc, spg, &sr, nth);
        else pasc_oracle_spgqp_solve(b2, x2, T2, K, coeffA, spg, &sr, NULL, nth);
        pasc_oracle_fem_prolongate(x2, gamma, T, T2, K, fem_type);         /* :296-298 */
        spg_it_sum += sr.it;
        spg_hm_sum += sr.hessmult;
        L_old = L;
        L = sr.fx;
        deltaL = fabs(L - L_old);
        if (L - L_old > 0) increased++;
        if (ts->relative ? (deltaL < ts->eps * fabs(L)) : (deltaL < ts->eps)) break;
    }
    if (r) {
        r->it_last = it;
        r->it_sum = it;
        r->spg_it_sum = spg_it_sum;
        r->spg_hessmult_sum = spg_hm_sum;
        r->L = L;
        r->deltaL = deltaL;
        r->aic = 2 * log(L) + K;
        r->L_increased = increased;
    }
    free(res); free(perm); free(b2); free(x2);
    return 0;
}

/* ------------------------------------------------------------------------------------- */
/* Graph (R > 1) and image mode: BGMGraph / BGMGraphGrid1D / BGMGraphGrid2D neighbour      */
/* lists, Decomposition::permute_TRK, and the TSSolver of GraphH1FEMModel over T*R blocks. */
/* ------------------------------------------------------------------------------------- */

/* Decomposition<PetscVector>::permute_TRblocksize (decomposition.cpp:260-340) on one rank:
 * the blocked layout k*R*T + r*T + t becomes (t*R + r)*K + k. */
void pasc_oracle_permute_TRK(const double *orig, double *out, long T, long R, int K)
{
    for (int k = 0; k < K; k++)
        for (long r = 0; r < R; r++)
            for (long t = 0; t < T; t++) out[(t * R + r) * K + k] = orig[(long)k * R * T + r * T + t];
}

/* BGMGraphGrid1D::process_grid (include/general/algebra/graph/bgmgraphgrid1D.h:76-115):
 * node i has i-1 and i+1.  Lists sorted ascending (ptr: width+1, idx: 2*(width-1)). */
void pasc_oracle_graph_grid1d(int width, int *ptr, int *idx)
{
    int q = 0;
    for (int i = 0; i < width; i++) {
        ptr[i] = q;
        if (i > 0) idx[q++] = i - 1;
        if (i < width - 1) idx[q++] = i + 1;
    }
    ptr[width] = q;
}

/* BGMGraphGrid2D::process_grid (include/general/algebra/graph/bgmgraphgrid2D.h:88-142):
 * node idx = i*width + j has left (j > 0), right, down (i > 0, idx - width) and up; the
 * lists are stored sorted ascending: idx-width, idx-1, idx+1, idx+width. */
void pasc_oracle_graph_grid2d(int width, int height, int *ptr, int *idx)
{
    int q = 0;
    for (int id = 0; id < width * height; id++) {
        const int i = id / width, j = id - i * width;
        ptr[id] = q;
        if (i > 0) idx[q++] = id - width;
        if (j > 0) idx[q++] = id - 1;
        if (j < width - 1) idx[q++] = id + 1;
        if (i < height - 1) idx[q++] = id + width;
    }
    ptr[width * height] = q;
}

/* BGMGraph::process(threshold) (src/petscvector/algebra/graph/bgmgraph.cpp:73-152): i and j
 * are neighbours when sum_d (c_i,d - c_j,d)^2 < threshold^2, coordinates stored dimension by
 * dimension (c_i,d = coords[i + d*n], bgmgraph.h:164-171).  The pair loop (i < j) appends j
 * to i's list and i to j's, so every list comes out ascending.  idx == NULL: only ptr. */
long pasc_oracle_graph_threshold(const double *coords, int n, int dim, double threshold, int *ptr, int *idx)
{
    int *cnt = (int *)calloc((size_t)n + 1, sizeof(int));
    if (!cnt) return -1;
    const double thr2 = threshold * threshold;
    for (int i = 0; i < n; i++)
        for (int j = i + 1; j < n; j++) {
            double s = 0.0;
            for (int d = 0; d < dim; d++) {
                const double df = coords[i + (long)d * n] - coords[j + (long)d * n];
                s += df * df;
            }
            if (s < thr2) {
                cnt[i]++;
                cnt[j]++;
            }
        }
    long q = 0;
    for (int i = 0; i < n; i++) {
        ptr[i] = (int)q;
        q += cnt[i];
    }
    ptr[n] = (int)q;
    if (idx) {
        for (int i = 0; i < n; i++) cnt[i] = ptr[i];
        for (int i = 0; i < n; i++)
            for (int j = i + 1; j < n; j++) {
                double s = 0.0;
                for (int d = 0; d < dim; d++) {
                    const double df = coords[i + (long)d * n] - coords[j + (long)d * n];
                    s += df * df;
                }
                if (s < thr2) {
                    idx[cnt[i]++] = j;
                    idx[cnt[j]++] = i;
                }
            }
    }
    free(cnt);
    return q;
}

/* TSSolver::solve with GraphH1FEMModel on a graph of R nodes (fem not reduced): gamma has
 * T*R blocks of K, data T*R values (index t*R + r), theta K; A = epssqr/T * A_graph and
 * b = -(x - theta_k)^2 / T keep the number of timesteps T (graphh1fem.cpp:146-151, 280-283). */
int pasc_oracle_tssolver_solve_graph(const double *data, double *gamma, double *theta, long T, int K,
                                     double epssqr, int scalef, const pasc_oracle_graph *G,
                                     const pasc_oracle_ts_opts *ts, const pasc_oracle_spg_opts *spg,
                                     pasc_oracle_ts_result *r, int nthreads)
{
    const int nth = eff_threads(nthreads);
    const long R = G->R, nb = T * R, n = nb * (long)K;
    double *b = (double *)malloc(sizeof(double) * (size_t)n);
    double *perm = (double *)malloc(sizeof(double) * (size_t)n);
    if (!b || !perm) {
        free(b); free(perm);
        return -1;
    }
    const double coeffA = pasc_oracle_A_coeff(epssqr, T, scalef);
    const double coeffB = pasc_oracle_b_coeff(T, scalef);
    if (ts->init_permute) {
        pasc_oracle_permute_TRK(gamma, perm, T, R, K);
        memcpy(gamma, perm, sizeof(double) * (size_t)n);
    }
    double L = DBL_MAX, L_old, deltaL = DBL_MAX;
    int it, spg_it_sum = 0, spg_hm_sum = 0, increased = 0;
    for (it = 0; it < ts->maxit; it++) {
        if (!ts->thetasolved) pasc_oracle_theta_update(gamma, data, theta, nb, K, 1, nth);
        pasc_oracle_residual_b(data, theta, b, nb, K, 1, coeffB, nth);
        pasc_oracle_spg_result sr;
        spgqp_impl(b, gamma, T, K, coeffA, NULL, G, spg, &sr, NULL, nth);
        spg_it_sum += sr.it;
        spg_hm_sum += sr.hessmult;
        L_old = L;
        L = sr.fx;
        deltaL = fabs(L - L_old);
        if (L - L_old > 0) increased++;
        if (ts->relative ? (deltaL < ts->eps * fabs(L)) : (deltaL < ts->eps)) break;
    }
    if (r) {
        r->it_last = it;
        r->it_sum = it;
        r->spg_it_sum = spg_it_sum;
        r->spg_hessmult_sum = spg_hm_sum;
        r->L = L;
        r->deltaL = deltaL;
        r->aic = 2 * log(L) + K;
        r->L_increased = increased;
    }
    free(b); free(perm);
    return 0;
}

/* ------------------------------------------------------------------------------------- */
/* SPGQPSolverC: the SPG-QP with the operator's coefficient factored out                  */
/* (include/general/solver/spgqpsolver_coeff.h:611-835; GraphH1FEMModel with               */
/* graphh1femmodel_gammasolvertype = 2, src/petscvector/model/graphh1fem.cpp:185-191).     */
/* A = coeff * A1 is applied as A1 (coefficient set to 1) and the coefficient enters the   */
/* gradient, the step and the A-condition explicitly.                                       */
/* ------------------------------------------------------------------------------------- */
static int spgqp_c_impl(const double *b, double *x, long T, int K, double coeff, const pasc_oracle_graph *G,
                        const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads)
{
    int nth = eff_threads(nthreads);
    const long nb = T * (G ? G->R : 1);
    const long n = nb * (long)K;
    double *g = (double *)malloc(sizeof(double) * (size_t)n);
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    double *Ad = (double *)malloc(sizeof(double) * (size_t)n);
    double *temp = (double *)malloc(sizeof(double) * (size_t)n);
    spg_fs fs;
    fs.m = o->m;
    fs.last_idx = 0;
    fs.fs = (double *)malloc(sizeof(double) * (size_t)(o->m > 0 ? o->m : 1));
    if (!g || !d || !Ad || !temp || !fs.fs) {
        free(g); free(d); free(Ad); free(temp); free(fs.fs);
        return -1;
    }
    const double epssqr = coeff;                            /* :615 */
    const double epssqrinv = epssqr == 0 ? 1.0 : 1.0 / epssqr; /* :616-621 */
    int it = 0, hessmult = 0;
    double fx, fx_old, fx_max, xi, beta_bar, beta_hat, beta, dd = 0.0, gd = 0.0, dAd = 0.0, alpha_bb;
    const double normb = sqrt(vdot(b, b, n, nth));
    alpha_bb = o->alphainit;

    pasc_oracle_project(x, nb, K, nth);          /* :663 */
    matmult_g(x, g, T, K, 1.0, NULL, G, nth);    /* g = A*x with coefficient 1 :667 */
    vscale(g, epssqr, n, nth);                   /* g *= epssqr :668 */
    hessmult += 1;
    vaxpy(g, -1.0, b, n, nth);                   /* :671 */
    fx = get_fx(g, b, x, temp, n, nth);          /* :676 */
    fx_old = DBL_MAX;
    fs_init(&fs, fx);

    while (it < o->maxit) {
        it += 1;
        vcopy(d, x, n, nth);                      /* d = x - epssqrinv*alpha_bb*g :694 */
        vaxpy(d, -(epssqrinv * alpha_bb), g, n, nth);
        pasc_oracle_project(d, nb, K, nth);       /* :699 */
        vaxpy(d, -1.0, x, n, nth);                /* :704 */
        matmult_g(d, Ad, T, K, 1.0, NULL, G, nth); /* Ad = A*d, coefficient 1 :709 */
        hessmult += 1;
        dd = vdot(d, d, n, nth);
        dAd = vdot(d, Ad, n, nth);
        gd = vdot(d, g, n, nth);
        fx_max = fs_get_max(&fs);
        xi = (fx_max - fx) / dAd;                 /* :730-745 */
        beta_bar = -gd / dAd;
        beta_hat = o->gamma * beta_bar + sqrt(o->gamma * o->gamma * beta_bar * beta_bar + 2 * epssqr * xi);
        if (epssqrinv * beta_hat < o->sigma1) beta_hat = o->sigma1;
        if (epssqrinv * beta_hat < o->sigma2) beta = epssqrinv * beta_hat;
        else beta = o->sigma2;
        vaxpy(x, beta, d, n, nth);                /* :751 */
        vaxpy(g, epssqr * beta, Ad, n, nth);      /* :752 */
        fx_old = fx;
        fx = get_fx(g, b, x, temp, n, nth);       /* :760 */
        fs_update(&fs, fx);
        alpha_bb = dd / dAd;                      /* :768 */
        if (o->stop_difff && fabs(fx - fx_old) < o->eps) break; /* :800-814 */
        if (o->stop_normgp && dd < o->eps) break;
        if (o->stop_normgp_normb && dd < o->eps * normb) break;
        if (o->stop_Anormgp && dAd < o->eps) break;
        if (o->stop_Anormgp_normb && dAd < o->eps * normb) break;
    }
    if (r) {
        r->it = it;
        r->hessmult = hessmult;
        r->fx = fx;
        r->gP = dd;
        r->dAd = dAd;
        r->normb = normb;
    }
    free(g); free(d); free(Ad); free(temp); free(fs.fs);
    return 0;
}

int pasc_oracle_spgqp_solve_coeff(const double *b, double *x, long T, int K, double coeff, const pasc_oracle_graph *G,
                                  const pasc_oracle_spg_opts *o, pasc_oracle_spg_result *r, int nthreads)
{
    return spgqp_c_impl(b, x, T, K, coeff, G, o, r, nthreads);
}

/* TSSolver with SPGQPSolverC as the gamma solver (1-D or graph problems, fem not reduced) */
int pasc_oracle_tssolver_solve_coeff(const double *data, double *gamma, double *theta, long T, int K, double epssqr,
                                     int scalef, const pasc_oracle_graph *G, const pasc_oracle_ts_opts *ts,
                                     const pasc_oracle_spg_opts *spg, pasc_oracle_ts_result *r, int nthreads)
{
    const int nth = eff_threads(nthreads);
    const long R = G ? G->R : 1, nb = T * R, n = nb * (long)K;
    double *b = (double *)malloc(sizeof(double) * (size_t)n);
    double *perm = (double *)malloc(sizeof(double) * (size_t)n);
    if (!b || !perm) {
        free(b); free(perm);
        return -1;
    }
    const double coeffA = pasc_oracle_A_coeff(epssqr, T, scalef);
    const double coeffB = pasc_oracle_b_coeff(T, scalef);
    if (ts->init_permute) {
        pasc_oracle_permute_TRK(gamma, perm, T, R, K);
        memcpy(gamma, perm, sizeof(double) * (size_t)n);
    }
    double L = DBL_MAX, L_old, deltaL = DBL_MAX;
    int it, spg_it_sum = 0, spg_hm_sum = 0, increased = 0;
    for (it = 0; it < ts->maxit; it++) {
        if (!ts->thetasolved) pasc_oracle_theta_update(gamma, data, theta, nb, K, 1, nth);
        pasc_oracle_residual_b(data, theta, b, nb, K, 1, coeffB, nth);
        pasc_oracle_spg_result sr;
        spgqp_c_impl(b, gamma, T, K, coeffA, G, spg, &sr, nth);
        spg_it_sum += sr.it;
        spg_hm_sum += sr.hessmult;
        L_old = L;
        L = sr.fx;
        deltaL = fabs(L - L_old);
        if (L - L_old > 0) increased++;
        if (ts->relative ? (deltaL < ts->eps * fabs(L)) : (deltaL < ts->eps)) break;
    }
    if (r) {
        r->it_last = it;
        r->it_sum = it;
        r->spg_it_sum = spg_it_sum;
        r->spg_hessmult_sum = spg_hm_sum;
        r->L = L;
        r->deltaL = deltaL;
        r->aic = 2 * log(L) + K;
        r->L_increased = increased;
    }
    free(b); free(perm);
    return 0;
}
