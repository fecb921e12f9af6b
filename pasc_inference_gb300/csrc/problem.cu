// problem.cu -- the C ABI (include/pasc_gb300.h): problem handles, the SPG-QP solve loops of
// both precisions, the TSSolver outer loop and the device-pointer entry points.
#include <math.h>
#include <stdarg.h>
#include <string.h>
#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <tuple>
#include <cstdio>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "problem.h"

using namespace pasc;

// zero pads around the mixed path's gamma and data buffers (timesteps)
static constexpr long PAD_FRONT = 4;
static constexpr long PAD_BACK = 1024;

// ---------------------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------------------
static thread_local std::string g_last_error;

static int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

#define CU(call)                                                                               \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(PASC_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),        \
                        __FILE__, __LINE__);                                                   \
    } while (0)

#define CHK(call)                                                                              \
    do {                                                                                       \
        int r_ = (call);                                                                       \
        if (r_ != PASC_OK) return r_;                                                          \
    } while (0)

// ---------------------------------------------------------------------------------------
// problem
// ---------------------------------------------------------------------------------------

static void free_all(pasc_gb300_problem *p)
{
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->adj) adjoint_free(p->adj);
    if (p->fem_inner) free_all(p->fem_inner);
    if (p->chunk_graph) cudaGraphExecDestroy(p->chunk_graph);
    void *dev[] = {p->data64, p->theta64, p->stage64, p->red, p->red_out, p->labels_d, p->x, p->g,
                   p->d, p->Ad, p->b, p->data32_raw, p->theta32, p->xb_raw[0], p->xb_raw[1], p->st,
                   p->partials, p->xbf, p->xnorm, p->bmat_raw, p->theta_split, p->theta_f32, p->tnorm,
                   p->mc_partials, p->mc_err, p->tp_ck64, p->tp_kw32, p->gptr, p->gidx, p->db_raw[0],
                   p->db_raw[1], p->gpartials, p->stage32};
    for (void *q : dev)
        if (q) cudaFree(q);
    if (p->st_h) cudaFreeHost(p->st_h);
    if (p->red_out_h) cudaFreeHost(p->red_out_h);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

template <typename T>
static int dalloc(T **ptr, size_t count)
{
    cudaError_t e = cudaMalloc((void **)ptr, sizeof(T) * (count > 0 ? count : 1));
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(PASC_ERR_ALLOC, "cudaMalloc of %zu bytes failed: %s", sizeof(T) * count,
                    cudaGetErrorString(e));
    }
    return PASC_OK;
}

static void fem_set_inner_coeffs(pasc_gb300_problem *p);
static int fem_update_b_async(pasc_gb300_problem *p, int *launches);

static void set_coeffs(pasc_gb300_problem *p)
{
    // graphh1fem.cpp:146-151 and :280-283 (not reduced: T_reduced == T); T counts timesteps,
    // not the T*R blocks of a graph problem
    const long T = p->graph ? p->graph_T : p->T;
    double c = p->epssqr;
    if (p->scalef) c *= (1.0 / ((double)T));
    else c *= ((double)T / ((double)T));
    p->coeffA = c;
    double cb = -1.0;
    if (p->scalef) cb *= (1.0 / ((double)T));
    p->coeffB = cb;
}

// coeff * A_hat x in FP64 (MatMult + VecScale): the 1-D chain, or the graph operator
static cudaError_t apply_A_f64(pasc_gb300_problem *p, const double *x, double *y, cudaStream_t s, double coeff)
{
    const double *kc = p->tp ? p->tp_ck64 : nullptr;
    if (p->graph) return launch_graph_matmult_f64(x, y, p->graph_T, p->graph_R, p->K, coeff, p->gptr, p->gidx, s, kc);
    return launch_matmult_f64(x, y, p->T, p->K, coeff, s, kc);
}

extern "C" {

void pasc_gb300_spgqp_default_opts(pasc_gb300_spgqp_opts *o)
{
    if (!o) return;
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

void pasc_gb300_ts_default_opts(pasc_gb300_ts_opts *o)
{
    if (!o) return;
    o->maxit = 300;
    o->eps = 1e-6;
    o->init_permute = 1;
    o->annealing = 1;
    o->relative = 0;
    o->thetasolved = 0;
}

int pasc_gb300_abi_version(void) { return PASC_GB300_ABI_VERSION; }

const char *pasc_gb300_last_error(void) { return g_last_error.c_str(); }

int pasc_gb300_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int pasc_gb300_create(pasc_gb300_problem **out, long T, int K, int xdim, int precision,
                      double epssqr, int device)
{
    if (!out) return fail(PASC_ERR_ARG, "create: out is NULL");
    *out = nullptr;
    if (T < 1) return fail(PASC_ERR_ARG, "create: T must be >= 1 (got %ld)", T);
    if (xdim < 1) return fail(PASC_ERR_ARG, "create: xdim must be >= 1 (got %d)", xdim);
    if (xdim > 1 && precision != PASC_PREC_MIXED)
        return fail(PASC_ERR_NOTSUPP, "create: multichannel data (xdim %d) needs the mixed path", xdim);
    if (xdim > 256) return fail(PASC_ERR_NOTSUPP, "create: xdim %d > 256 not supported", xdim);
    if (precision != PASC_PREC_FP64 && precision != PASC_PREC_MIXED)
        return fail(PASC_ERR_ARG, "create: unknown precision %d", precision);
    const int kmax = precision == PASC_PREC_MIXED ? KMAX_FUSED : KMAX_PLAIN;
    if (K < 1 || K > kmax)
        return fail(PASC_ERR_ARG, "create: K must be in [1, %d] for this precision (got %d)", kmax, K);
    if ((double)T * (double)K > 2.0e9) return fail(PASC_ERR_ARG, "create: K*T too large");
    int ndev = pasc_gb300_device_count();
    if (ndev <= 0) return fail(PASC_ERR_CUDA, "create: no CUDA device available");
    if (device < 0 || device >= ndev) return fail(PASC_ERR_ARG, "create: device %d out of range", device);

    pasc_gb300_problem *p = new (std::nothrow) pasc_gb300_problem();
    if (!p) return fail(PASC_ERR_ALLOC, "create: host allocation failed");
    p->T = T;
    p->K = K;
    p->xdim = xdim;
    p->precision = precision;
    p->device = device;
    p->epssqr = epssqr;
    p->N = T * (long)K;
    set_coeffs(p);

    int rc = PASC_OK;
    auto bail = [&](int code) { free_all(p); return code; };
    if (cudaSetDevice(device) != cudaSuccess) return bail(fail(PASC_ERR_CUDA, "cudaSetDevice failed"));
    cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&p->ev0) != cudaSuccess || cudaEventCreate(&p->ev1) != cudaSuccess)
        return bail(fail(PASC_ERR_CUDA, "create: stream/event creation failed"));

    const long N = p->N;
    if ((rc = dalloc(&p->data64, (size_t)T * xdim)) || (rc = dalloc(&p->theta64, (size_t)K * xdim)) ||
        (rc = dalloc(&p->stage64, N)) || (rc = dalloc(&p->red, dot_partials_size())) ||
        (rc = dalloc(&p->red_out, 8)) || (rc = dalloc(&p->labels_d, T)))
        return bail(rc);
    if (cudaMallocHost((void **)&p->red_out_h, 8 * sizeof(double)) != cudaSuccess)
        return bail(fail(PASC_ERR_ALLOC, "create: pinned allocation failed"));
    cudaMemset(p->red, 0, dot_partials_size() * sizeof(double));
    cudaMemset(p->theta64, 0, sizeof(double) * K * xdim);
    cudaMemset(p->data64, 0, sizeof(double) * T * xdim);

    if (precision == PASC_PREC_FP64) {
        if ((rc = dalloc(&p->x, N)) || (rc = dalloc(&p->g, N)) || (rc = dalloc(&p->d, N)) ||
            (rc = dalloc(&p->Ad, N)) || (rc = dalloc(&p->b, N)))
            return bail(rc);
        cudaMemset(p->x, 0, sizeof(double) * N);
        cudaMemset(p->b, 0, sizeof(double) * N);
    } else {
        // gamma and data carry zero pads (PAD_FRONT timesteps before, PAD_BACK after) so that
        // the bulk-copy sweep can copy whole tiles at the ends of the signal; the pads stay
        // zero because every kernel writes only 0 <= t < T
        const size_t nx = (size_t)(T + PAD_FRONT + PAD_BACK) * K, nd = (size_t)(T + PAD_FRONT + PAD_BACK);
        if ((rc = dalloc(&p->data32_raw, nd)) || (rc = dalloc(&p->theta32, K)) ||
            (rc = dalloc(&p->xb_raw[0], nx)) || (rc = dalloc(&p->xb_raw[1], nx)) ||
            (rc = dalloc(&p->st, 1)))
            return bail(rc);
        cudaMemset(p->xb_raw[0], 0, sizeof(float) * nx);
        cudaMemset(p->xb_raw[1], 0, sizeof(float) * nx);
        cudaMemset(p->data32_raw, 0, sizeof(float) * nd);
        p->xb[0] = p->xb_raw[0] + (size_t)PAD_FRONT * K;
        p->xb[1] = p->xb_raw[1] + (size_t)PAD_FRONT * K;
        p->data32 = p->data32_raw + PAD_FRONT;
        if (cudaMallocHost((void **)&p->st_h, sizeof(SpgDevState)) != cudaSuccess)
            return bail(fail(PASC_ERR_ALLOC, "create: pinned allocation failed"));
        memset(p->st_h, 0, sizeof(SpgDevState));
        cudaMemset(p->st, 0, sizeof(SpgDevState));
        cudaMemset(p->theta32, 0, sizeof(float) * K);
        auto grid = [&](long per_sm, long ntiles) {
            long g = per_sm * p->sms;
            g = g < ntiles ? g : ntiles;
            return (int)(g < 1 ? 1 : g);
        };
        const long nt_thread = (T + sweep_tile_width() - 1) / sweep_tile_width();
        p->grid_sweep[0] = grid(sweep_blocks_per_sm(K, false), nt_thread);
        p->grid_sweep_init[0] = grid(sweep_blocks_per_sm(K, true), nt_thread);
        const long nt_tma = (T + sweep_tma_tile_width() - 1) / sweep_tma_tile_width();
        p->grid_sweep[1] = grid(sweep_tma_blocks_per_sm(K, false, xdim > 1), nt_tma);
        p->grid_sweep_init[1] = grid(sweep_tma_blocks_per_sm(K, true, xdim > 1), nt_tma);
        p->grid_sweep_max[0] = p->grid_sweep[0];
        p->grid_sweep_max[1] = p->grid_sweep[1];
        long gt = (long)p->sms * 4;
        long tb = (T + 255) / 256;
        p->grid_theta = (int)(gt < tb ? gt : tb);
        if (p->grid_theta < 1) p->grid_theta = 1;
        long np = 0;
        for (int v = 0; v < 2; v++) {
            np = np > p->grid_sweep[v] ? np : p->grid_sweep[v];
            np = np > p->grid_sweep_init[v] ? np : p->grid_sweep_init[v];
        }
        // (the theta kernel with theta in the penalty keeps 3K partials per block)
        np = np * 4 > (long)p->grid_theta * 3 * K ? np * 4 : (long)p->grid_theta * 3 * K;
        if ((rc = dalloc(&p->partials, np))) return bail(rc);
        if (xdim > 1) {
            long gm = (long)p->sms * 4, tb64 = (T + 63) / 64;
            p->mc_grid_theta = (int)(gm < tb64 ? gm : tb64);
            if (p->mc_grid_theta < 1) p->mc_grid_theta = 1;
            const int tb_sm = mc_theta_tma_blocks_per_sm(K, xdim);
            if (tb_sm > 0) {
                const long gt = (long)p->sms * tb_sm;
                p->mc_grid_theta_tma = (int)(gt < tb64 ? gt : tb64);
                if (p->mc_grid_theta_tma > p->mc_grid_theta) p->mc_grid_theta_tma = p->mc_grid_theta;
            }
            long nt = (T + 127) / 128;
            p->mc_grid_res = (int)((long)p->sms < nt ? p->sms : nt);
            if ((rc = dalloc(&p->xbf, (size_t)T * xdim)) || (rc = dalloc(&p->xnorm, T)) ||
                (rc = dalloc(&p->bmat_raw, nx)) || (rc = dalloc(&p->theta_split, (size_t)32 * xdim)) ||
                (rc = dalloc(&p->theta_f32, (size_t)K * xdim)) || (rc = dalloc(&p->tnorm, K)) ||
                (rc = dalloc(&p->mc_err, 1)) ||
                (rc = dalloc(&p->mc_partials, mc_partials_size(K, xdim, p->mc_grid_theta, T))))
                return bail(rc);
            cudaMemset(p->xbf, 0, sizeof(unsigned short) * T * xdim);
            cudaMemset(p->xnorm, 0, sizeof(float) * T);
            cudaMemset(p->bmat_raw, 0, sizeof(float) * nx);
            p->bmat = p->bmat_raw + (size_t)PAD_FRONT * K;
            cudaMemset(p->theta_split, 0, sizeof(unsigned short) * 32 * xdim);
            cudaMemset(p->theta_f32, 0, sizeof(float) * K * xdim);
            cudaMemset(p->tnorm, 0, sizeof(float) * K);
            cudaMemset(p->mc_err, 0, sizeof(int));
            p->mc_engine = mc_tc_supported(xdim) ? 0 : 1;
            if (p->mc_engine == 0) {
                cudaError_t e = mc_make_tmap(&p->mc_tmap, p->xbf, T, xdim);
                if (e == cudaSuccess) e = prepare_mc_residual_tc(K, xdim);
                if (e != cudaSuccess)
                    return bail(fail(PASC_ERR_CUDA, "create: tensor map / kernel set-up failed: %s", cudaGetErrorString(e)));
            }
        }
    }
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return bail(fail(PASC_ERR_CUDA, "create: initialisation failed"));
    *out = p;
    return PASC_OK;
}

int pasc_gb300_destroy(pasc_gb300_problem *p)
{
    if (!p) return PASC_OK;
    free_all(p);
    return PASC_OK;
}

int pasc_gb300_set_epssqr(pasc_gb300_problem *p, double epssqr, int scalef)
{
    if (!p) return fail(PASC_ERR_ARG, "set_epssqr: NULL problem");
    p->run.started = false;
    p->epssqr = epssqr;
    p->scalef = scalef ? 1 : 0;
    set_coeffs(p);
    if (p->fem_inner) fem_set_inner_coeffs(p);
    if (p->tp) {
        CU(cudaSetDevice(p->device));
        CU(launch_tp_coeffs(p->theta64, p->coeffA, p->K, p->tp_ck64, p->tp_kw32, p->stream));
        CU(cudaStreamSynchronize(p->stream));
    }
    return PASC_OK;
}

}  // extern "C"

// Coefficients of the reduced QP (graphh1fem.cpp:145-151 and :280-283): A keeps the original
// T (A = epssqr/T A_hat on the coarse grid; epssqr*T2/T without scalef), b the reduced one
// (b = -1/T2 * reduced residual; -1 without scalef).
static void fem_set_inner_coeffs(pasc_gb300_problem *p)
{
    pasc_gb300_problem *q = p->fem_inner;
    const double T = (double)p->T, T2 = (double)q->T;
    q->epssqr = p->epssqr;
    q->scalef = p->scalef;
    q->coeffA = p->scalef ? p->epssqr * (1.0 / T) : p->epssqr * (T2 / T);
    q->coeffB = p->scalef ? -1.0 * (1.0 / T2) : -1.0;
    q->run.started = false;
}

static McArgs mc_args(pasc_gb300_problem *p)
{
    McArgs a;
    a.T = p->T;
    a.n = p->xdim;
    a.xbf = p->xbf;
    a.xnorm = p->xnorm;
    a.bmat = p->bmat;
    a.theta_split = p->theta_split;
    a.theta_f32 = p->theta_f32;
    a.tnorm = p->tnorm;
    a.theta64 = p->theta64;
    a.partials = p->mc_partials;
    a.bscale = (float)p->coeffB;
    a.err = p->mc_err;
    a.theta_tma_grid = p->mc_grid_theta_tma;
    return a;
}

// b_tk = bscale ||X_t - theta_k||^2 into bmat (multichannel)
static int mc_residual_async(pasc_gb300_problem *p, int *launches)
{
    const McArgs a = mc_args(p);
    if (p->mc_engine == 0) CU(launch_mc_residual_tc(p->mc_tmap, p->K, p->xdim, p->mc_grid_res, a, p->stream));
    else CU(launch_mc_residual_simt(p->K, p->sms * 4, a, p->stream));
    if (launches) *launches += 1;
    return PASC_OK;
}

static int mc_check_error(pasc_gb300_problem *p)
{
    if (p->xdim == 1) return PASC_OK;
    int e = 0;
    CU(cudaMemcpyAsync(&e, p->mc_err, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    if (e) {
        cudaMemsetAsync(p->mc_err, 0, sizeof(int), p->stream);
        return fail(PASC_ERR_TIMEOUT, "residual kernel: a bounded wait for a tile copy or the tensor cores gave up (%d)", e);
    }
    return PASC_OK;
}

// GraphH1FEMModel::updatebeforesolve_gammasolver with a reduction (graphh1fem.cpp:237-289): the
// residual (x_t - theta_k)^2 on the full grid, reduced and scaled into the inner b, and the
// current gamma reduced into the inner x (the warm start, projected when the solve starts).
static int fem_update_b_async(pasc_gb300_problem *p, int *launches)
{
    pasc_gb300_problem *q = p->fem_inner;
    const long T = p->T, T2 = q->T;
    const int K = p->K, type = p->fem_type;
    cudaStream_t s = p->stream;
    if (p->precision == PASC_PREC_FP64) {
        CU((launch_fem_reduce<double, double>(nullptr, p->data64, p->theta64, q->b, T, T2, K, type, q->coeffB, s)));
        CU((launch_fem_reduce<double, double>(p->x, nullptr, nullptr, q->x, T, T2, K, type, 1.0, s)));
    } else {
        if (p->xdim > 1) {
            // the full b = bscale ||X_t - theta_k||^2 (FP32), then its reduction rescaled
            CHK(mc_residual_async(p, launches));
            CU((launch_fem_reduce<float, float>(p->bmat, nullptr, nullptr, q->bmat, T, T2, K, type,
                                               q->coeffB / p->coeffB, s)));
        } else {
            CU((launch_fem_reduce<float, float>(nullptr, p->data64, p->theta64, q->bmat, T, T2, K, type, q->coeffB, s)));
        }
        CU((launch_fem_reduce<float, float>(p->xb[p->cur], nullptr, nullptr, q->xb[q->cur], T, T2, K, type, 1.0, s)));
    }
    if (launches) *launches += 2;
    // the inner handle works on its own stream: its solve must see the reduced b and x
    CU(cudaStreamSynchronize(s));
    q->run.started = false;
    q->have_fx = false;
    return PASC_OK;
}

extern "C" {

// after data64 holds the new data (FP64 on the device): the derived device copies
static int data_uploaded(pasc_gb300_problem *p)
{
    if (p->xdim > 1) {
        // multichannel: X is kept in BF16 (rounded to nearest), with ||X_t||^2 of the rounded
        // values; b follows from the current theta
        CU(launch_mc_convert(p->data64, p->xbf, p->xnorm, p->T, p->xdim, p->stream));
        CHK(mc_residual_async(p, nullptr));
    } else if (p->precision == PASC_PREC_MIXED) {
        CU(launch_f64_to_f32(p->data64, p->data32, p->T, p->stream));
    }
    CU(cudaStreamSynchronize(p->stream));
    CHK(mc_check_error(p));
    p->have_data = true;
    return PASC_OK;
}

int pasc_gb300_set_data(pasc_gb300_problem *p, const double *data)
{
    if (!p || !data) return fail(PASC_ERR_ARG, "set_data: NULL argument");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    CU(cudaMemcpyAsync(p->data64, data, sizeof(double) * p->T * p->xdim, cudaMemcpyHostToDevice, p->stream));
    return data_uploaded(p);
}

int pasc_gb300_set_data_f32(pasc_gb300_problem *p, const float *data)
{
    if (!p || !data) return fail(PASC_ERR_ARG, "set_data_f32: NULL argument");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    const long n = p->T * p->xdim;
    if (p->xdim == 1 && p->precision == PASC_PREC_MIXED) {
        // the sweeps read FP32 data: copy it in place, widen it for the FP64 consumers
        CU(cudaMemcpyAsync(p->data32, data, sizeof(float) * n, cudaMemcpyHostToDevice, p->stream));
        CU(launch_f32_to_f64(p->data32, p->data64, n, p->stream));
        CU(cudaStreamSynchronize(p->stream));
        p->have_data = true;
        return PASC_OK;
    }
    float *stage = nullptr;
    if (n <= 2 * p->N) {
        stage = reinterpret_cast<float *>(p->stage64);
    } else {
        if (!p->stage32) CHK(dalloc(&p->stage32, (size_t)n));
        stage = p->stage32;
    }
    CU(cudaMemcpyAsync(stage, data, sizeof(float) * n, cudaMemcpyHostToDevice, p->stream));
    CU(launch_f32_to_f64(stage, p->data64, n, p->stream));
    return data_uploaded(p);
}

int pasc_gb300_set_gamma(pasc_gb300_problem *p, const double *gamma)
{
    if (!p || !gamma) return fail(PASC_ERR_ARG, "set_gamma: NULL argument");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    if (p->precision == PASC_PREC_FP64) {
        CU(cudaMemcpyAsync(p->x, gamma, sizeof(double) * p->N, cudaMemcpyHostToDevice, p->stream));
    } else {
        CU(cudaMemcpyAsync(p->stage64, gamma, sizeof(double) * p->N, cudaMemcpyHostToDevice, p->stream));
        CU(launch_f64_to_f32(p->stage64, p->xb[p->cur], p->N, p->stream));
    }
    CU(cudaStreamSynchronize(p->stream));
    p->have_fx = false;
    return PASC_OK;
}

// device FP64 view of gamma (mixed: converted into stage64)
static int gamma64(pasc_gb300_problem *p, const double **out)
{
    if (p->precision == PASC_PREC_FP64) {
        *out = p->x;
        return PASC_OK;
    }
    CU(launch_f32_to_f64(p->xb[p->cur], p->stage64, p->N, p->stream));
    *out = p->stage64;
    return PASC_OK;
}

int pasc_gb300_get_gamma(pasc_gb300_problem *p, double *gamma)
{
    if (!p || !gamma) return fail(PASC_ERR_ARG, "get_gamma: NULL argument");
    CU(cudaSetDevice(p->device));
    const double *g64 = nullptr;
    CHK(gamma64(p, &g64));
    CU(cudaMemcpyAsync(gamma, g64, sizeof(double) * p->N, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

int pasc_gb300_set_gamma_f32(pasc_gb300_problem *p, const float *gamma)
{
    if (!p || !gamma) return fail(PASC_ERR_ARG, "set_gamma_f32: NULL argument");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    if (p->precision == PASC_PREC_FP64) {
        float *stage = reinterpret_cast<float *>(p->stage64);
        CU(cudaMemcpyAsync(stage, gamma, sizeof(float) * p->N, cudaMemcpyHostToDevice, p->stream));
        CU(launch_f32_to_f64(stage, p->x, p->N, p->stream));
    } else {
        CU(cudaMemcpyAsync(p->xb[p->cur], gamma, sizeof(float) * p->N, cudaMemcpyHostToDevice, p->stream));
    }
    CU(cudaStreamSynchronize(p->stream));
    p->have_fx = false;
    return PASC_OK;
}

int pasc_gb300_get_gamma_f32(pasc_gb300_problem *p, float *gamma)
{
    if (!p || !gamma) return fail(PASC_ERR_ARG, "get_gamma_f32: NULL argument");
    CU(cudaSetDevice(p->device));
    const float *src = p->xb[p->cur];
    if (p->precision == PASC_PREC_FP64) {
        float *stage = reinterpret_cast<float *>(p->stage64);
        CU(launch_f64_to_f32(p->x, stage, p->N, p->stream));
        src = stage;
    }
    CU(cudaMemcpyAsync(gamma, src, sizeof(float) * p->N, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

int pasc_gb300_host_alloc(void **ptr, unsigned long bytes)
{
    if (!ptr) return fail(PASC_ERR_ARG, "host_alloc: NULL argument");
    *ptr = nullptr;
    cudaError_t e = cudaHostAlloc(ptr, bytes > 0 ? bytes : 1, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return fail(PASC_ERR_ALLOC, "cudaHostAlloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
    }
    return PASC_OK;
}

int pasc_gb300_host_free(void *ptr)
{
    if (!ptr) return PASC_OK;
    CU(cudaFreeHost(ptr));
    return PASC_OK;
}

int pasc_gb300_set_theta(pasc_gb300_problem *p, const double *theta)
{
    if (!p || !theta) return fail(PASC_ERR_ARG, "set_theta: NULL argument");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    CU(cudaMemcpyAsync(p->theta64, theta, sizeof(double) * p->K * p->xdim, cudaMemcpyHostToDevice, p->stream));
    if (p->xdim > 1) {
        CU(launch_mc_theta(p->K, p->mc_grid_theta, mc_args(p), nullptr, p->stream));
        if (p->have_data) CHK(mc_residual_async(p, nullptr));
    } else if (p->precision == PASC_PREC_MIXED) {
        CU(launch_f64_to_f32(p->theta64, p->theta32, p->K, p->stream));
    }
    if (p->tp) CU(launch_tp_coeffs(p->theta64, p->coeffA, p->K, p->tp_ck64, p->tp_kw32, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    CHK(mc_check_error(p));
    return PASC_OK;
}

int pasc_gb300_get_theta(pasc_gb300_problem *p, double *theta)
{
    if (!p || !theta) return fail(PASC_ERR_ARG, "get_theta: NULL argument");
    CU(cudaSetDevice(p->device));
    CU(cudaMemcpyAsync(theta, p->theta64, sizeof(double) * p->K * p->xdim, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

static int permute_gamma_async(pasc_gb300_problem *p)
{
    if (p->precision == PASC_PREC_FP64) {
        CU(launch_permute_f64(p->x, p->stage64, p->T, p->K, p->stream, p->graph_R));
        CU(cudaMemcpyAsync(p->x, p->stage64, sizeof(double) * p->N, cudaMemcpyDeviceToDevice, p->stream));
    } else {
        float *src = p->xb[p->cur], *dst = p->xb[p->cur ^ 1];
        CU(launch_permute_f32(src, dst, p->T, p->K, p->stream, p->graph_R));
        p->cur ^= 1;
    }
    return PASC_OK;
}

int pasc_gb300_permute_gamma(pasc_gb300_problem *p)
{
    if (!p) return fail(PASC_ERR_ARG, "permute_gamma: NULL problem");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    CHK(permute_gamma_async(p));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

static int update_theta_async(pasc_gb300_problem *p, int *launches)
{
    if (p->xdim > 1) {
        CU(launch_mc_theta(p->K, p->mc_grid_theta, mc_args(p), p->xb[p->cur], p->stream));
        if (launches) *launches += 2;
        return PASC_OK;
    }
    if (p->precision == PASC_PREC_FP64) {
        // theta in the penalty: Agamma with theta = 1, i.e. A = coeffA * A_hat (graphh1fem.cpp:314-325)
        CU(launch_theta_f64(p->x, p->data64, p->theta64, p->T, p->K, p->red, p->stream, p->tp, p->coeffA));
        if (launches) *launches += (p->K + 7) / 8;
    } else {
        ThetaArgs a;
        a.data = p->data32;
        a.xb0 = p->xb[0];
        a.xb1 = p->xb[1];
        a.partials = p->partials;
        a.theta64 = p->theta64;
        a.theta32 = p->theta32;
        a.st = p->st;
        a.T = p->T;
        a.cur = p->cur;
        a.tp = p->tp ? 1 : 0;
        a.pen_alpha = p->coeffA;
        CU(launch_theta_f32(p->K, p->grid_theta, a, p->stream));
        if (launches) *launches += 1;
    }
    if (p->tp) {
        CU(launch_tp_coeffs(p->theta64, p->coeffA, p->K, p->tp_ck64, p->tp_kw32, p->stream));
        if (launches) *launches += 1;
    }
    return PASC_OK;
}

int pasc_gb300_update_theta(pasc_gb300_problem *p)
{
    if (!p) return fail(PASC_ERR_ARG, "update_theta: NULL problem");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    CHK(update_theta_async(p, nullptr));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

static int update_b_async(pasc_gb300_problem *p, int *launches)
{
    if (p->fem_inner) return fem_update_b_async(p, launches);
    if (p->b_external) return PASC_OK;  // written by the owner of this (inner) handle
    if (p->xdim > 1) return mc_residual_async(p, launches);
    if (p->precision == PASC_PREC_FP64) {
        CU(launch_residual_f64(p->data64, p->theta64, p->b, p->T, p->K, p->coeffB, p->stream));
        if (launches) *launches += 1;
    }
    // mixed: b is formed inside the sweep from data32 and theta32 (kept current by
    // set_theta / update_theta)
    return PASC_OK;
}

int pasc_gb300_update_b(pasc_gb300_problem *p)
{
    if (!p) return fail(PASC_ERR_ARG, "update_b: NULL problem");
    p->run.started = false;
    CU(cudaSetDevice(p->device));
    CHK(update_b_async(p, nullptr));
    CU(cudaStreamSynchronize(p->stream));
    CHK(mc_check_error(p));
    return PASC_OK;
}

// ---------------------------------------------------------------------------------------
// SPG-QP, FP64 plain path: the reference's loop (spgqpsolver.cpp:55-312) with host scalars.
// ---------------------------------------------------------------------------------------
static int read_red(pasc_gb300_problem *p, int n, double *vals)
{
    CU(cudaMemcpyAsync(p->red_out_h, p->red_out, sizeof(double) * n, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    for (int i = 0; i < n; i++) vals[i] = p->red_out_h[i];
    return PASC_OK;
}

static void fill_stats(const SpgRun &r, pasc_gb300_spgqp_stats *st)
{
    if (!st) return;
    st->it = r.it;
    st->hessmult = r.hessmult;
    st->status = r.status;
    st->kernel_launches = r.launches;
    st->fx = r.fx;
    st->gP = r.dd;
    st->dAd = r.dAd;
    st->time_s = r.time_s;
}

// spgqpsolver.cpp:104-137
static int fp64_start(pasc_gb300_problem *p)
{
    SpgRun &r = p->run;
    const long N = p->N, T = p->T;
    const int K = p->K;
    cudaStream_t s = p->stream;
    double v[3];
    CU(cudaEventRecord(p->ev0, s));
    CU(launch_dots_f64(1, p->b, p->b, nullptr, nullptr, nullptr, nullptr, N, p->red, p->red_out, s));
    r.launches++;
    CHK(read_red(p, 1, v));
    r.normb = sqrt(v[0]);             // :104
    r.alpha = r.o.alphainit;          // :108
    CU(launch_project_f64(p->x, T, K, s));                   // :116
    // :122-123; SPGQPSolverC (spgqpsolver_coeff.h:667-668) multiplies with coefficient 1 and
    // scales by eps afterwards: 1.0 * sum is exact, so eps * sum is the same value
    CU(apply_A_f64(p, p->x, p->g, s, p->coeffA));
    CU(launch_axpy_f64(p->g, -1.0, p->b, N, s));             // :128
    CU(launch_fx_f64(p->x, p->g, p->b, N, p->red, p->red_out, s));  // :133
    r.launches += 4;
    CHK(read_red(p, 1, v));
    r.fx = 0.5 * v[0];
    r.fx_old = DBL_MAX;
    for (int q = 0; q < r.o.m; q++) r.fs[q] = r.fx;
    r.fs_last = 0;
    r.it = 0;
    r.hessmult = 1;
    r.status = r.o.maxit <= 0 ? PASC_SPG_MAXIT : (isfinite(r.fx) ? PASC_SPG_RUNNING : PASC_SPG_NONFINITE);
    CU(cudaEventRecord(p->ev1, s));
    CU(cudaEventSynchronize(p->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    r.time_s += ms * 1e-3;
    return PASC_OK;
}

// spgqpsolver.cpp:140-297, at most n iterations
static int fp64_iterate(pasc_gb300_problem *p, long n)
{
    SpgRun &r = p->run;
    const pasc_gb300_spgqp_opts *o = &r.o;
    const long N = p->N, T = p->T;
    const int K = p->K;
    cudaStream_t s = p->stream;
    double v[3];
    // SPGQPSolverC (spgqpsolver_coeff.h:611-835): d'Ad, the BB step and the A-condition without
    // the coefficient, which enters the step scalars instead
    const bool cm = p->solver_type == 2;
    const double eps = p->coeffA, einv = eps == 0 ? 1.0 : 1.0 / eps;
    CU(cudaEventRecord(p->ev0, s));
    for (long q = 0; q < n && r.status == PASC_SPG_RUNNING; q++) {
        if (r.it >= o->maxit) { r.status = PASC_SPG_MAXIT; break; }
        r.it += 1;
        CU(launch_xmay_f64(p->d, p->x, cm ? einv * r.alpha : r.alpha, p->g, N, s));  // :146-147
        CU(launch_project_f64(p->d, T, K, s));                    // :153
        CU(launch_axpy_f64(p->d, -1.0, p->x, N, s));              // :158
        CU(apply_A_f64(p, p->d, p->Ad, s, cm ? 1.0 : p->coeffA));  // :164-165
        r.hessmult += 1;
        CU(launch_dots_f64(3, p->d, p->d, p->d, p->Ad, p->d, p->g, N, p->red, p->red_out, s));  // :357-363
        r.launches += 5;
        CHK(read_red(p, 3, v));
        const double dd = v[0], dAd = v[1], gd = v[2];
        if (!(isfinite(dd) && isfinite(dAd) && isfinite(gd))) { r.status = PASC_SPG_NONFINITE; r.it -= 1; break; }
        if (!(dd > 0.0)) { r.status = PASC_SPG_DAD_ZERO; r.it -= 1; break; }
        double beta, alpha_next;
        if (dAd > 0.0) {
            double fx_max = r.fs[0];
            for (int i = 0; i < o->m; i++) fx_max = r.fs[i] > fx_max ? r.fs[i] : fx_max;  // :176
            const double xi = (fx_max - r.fx) / dAd;  // :182-195
            const double beta_bar = -gd / dAd;
            if (cm) {
                double beta_hat = o->gamma * beta_bar + sqrt(o->gamma * o->gamma * beta_bar * beta_bar + 2 * eps * xi);
                if (einv * beta_hat < o->sigma1) beta_hat = o->sigma1;
                beta = einv * beta_hat < o->sigma2 ? einv * beta_hat : o->sigma2;
            } else {
                double beta_hat = o->gamma * beta_bar + sqrt(o->gamma * o->gamma * beta_bar * beta_bar + 2 * xi);
                if (beta_hat < o->sigma1) beta_hat = o->sigma1;
                beta = beta_hat < o->sigma2 ? beta_hat : o->sigma2;
            }
            alpha_next = dd / dAd;  // :216
        } else if (gd < 0.0) {
            // linear along d (A_hat d = 0): the reference's division by zero falls through to
            // beta = sigma2; take that step and keep alpha finite
            beta = o->sigma2;
            alpha_next = r.alpha;
        } else {
            r.status = PASC_SPG_DAD_ZERO;
            r.it -= 1;
            break;
        }
        CU(launch_axpy_f64(p->x, beta, p->d, N, s));   // :200
        CU(launch_axpy_f64(p->g, cm ? eps * beta : beta, p->Ad, N, s));  // :201
        CU(launch_fx_f64(p->x, p->g, p->b, N, p->red, p->red_out, s));  // :209
        r.launches += 3;
        CHK(read_red(p, 1, v));
        r.fx_old = r.fx;
        r.fx = 0.5 * v[0];
        if (++r.fs_last >= o->m) r.fs_last = 0;  // :210
        r.fs[r.fs_last] = r.fx;
        r.alpha = alpha_next;
        r.dd = dd;
        r.dAd = dAd;
        if (!isfinite(r.fx)) { r.status = PASC_SPG_NONFINITE; break; }
        if ((o->stop_difff && fabs(r.fx - r.fx_old) < o->eps) || (o->stop_normgp && dd < o->eps) ||
            (o->stop_normgp_normb && dd < o->eps * r.normb) || (o->stop_Anormgp && dAd < o->eps) ||
            (o->stop_Anormgp_normb && dAd < o->eps * r.normb)) {
            r.status = PASC_SPG_CONVERGED;
        }
    }
    if (r.status == PASC_SPG_RUNNING && r.it >= o->maxit) r.status = PASC_SPG_MAXIT;
    CU(cudaEventRecord(p->ev1, s));
    CU(cudaEventSynchronize(p->ev1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    r.time_s += ms * 1e-3;
    p->fx_last = r.fx;
    p->have_fx = true;
    return PASC_OK;
}

// ---------------------------------------------------------------------------------------
// SPG-QP, mixed fused path: one sweep per iteration, state on the device, host polls.
// ---------------------------------------------------------------------------------------
// Tensor maps for the swizzled tiles of the bulk-copy sweep (K = 4, 8), rebuilt when the
// buffers change; tm_ok false (the plain bulk-copy form runs) where they cannot be made.
static void ensure_sweep_maps(pasc_gb300_problem *p)
{
    if (!sweep_tma_rows16(p->K) || p->precision != PASC_PREC_MIXED || !p->xb_raw[0]) {
        p->tm_ok = false;
        return;
    }
    if (p->tm_ok && p->tm_base[0] == p->xb_raw[0] && p->tm_base[1] == p->xb_raw[1] && p->tm_base[2] == p->bmat_raw)
        return;
    const long n = ((p->T + PAD_FRONT + PAD_BACK) * p->K) / 16 * 16;  // whole rows of 16 floats
    const int rows = sweep_tma_threads(p->K);
    bool ok = sweep_tma_make_rowmap(&p->tm_x[0], p->xb_raw[0], n, rows) == cudaSuccess &&
              sweep_tma_make_rowmap(&p->tm_x[1], p->xb_raw[1], n, rows) == cudaSuccess;
    if (ok && p->bmat_raw) ok = sweep_tma_make_rowmap(&p->tm_b, p->bmat_raw, n, rows) == cudaSuccess;
    p->tm_ok = ok;
    p->tm_base[0] = p->xb_raw[0];
    p->tm_base[1] = p->xb_raw[1];
    p->tm_base[2] = p->bmat_raw;
}

static int sweep_args(pasc_gb300_problem *p, SweepArgs *a)
{
    ensure_sweep_maps(p);
    if (p->tm_ok) {
        a->tm_x[0] = p->tm_x[0];
        a->tm_x[1] = p->tm_x[1];
        a->tm_b = p->tm_b;
        a->swz = 1;
        a->roff = (int)(PAD_FRONT * p->K / 16);
    }
    a->bmat = p->bmat;  // set for multichannel data and for the inner handle of a reduced problem
    a->data = p->data32;
    a->theta = p->theta32;
    a->xb0 = p->xb[0];
    a->xb1 = p->xb[1];
    a->partials = p->partials;
    a->st = p->st;
    a->T = p->T;
    a->kw = p->tp ? p->tp_kw32 : nullptr;
    return PASC_OK;
}

static constexpr int GRAPH_CHUNK = 16;

static cudaError_t launch_variant(pasc_gb300_problem *p, int v, bool init, const SweepArgs &a)
{
    if (p->graph && v == 1) {
        ImageSweepArgs g;
        g.data = p->data32;
        g.theta = p->theta32;
        g.xb0 = p->xb[0];
        g.xb1 = p->xb[1];
        g.partials = p->gpartials;
        g.st = p->st;
        g.W = p->img_W;
        g.H = p->img_H;
        return launch_image_sweep(p->K, init, p->grid_image, g, p->stream);
    }
    if (p->graph) {
        GraphSweepArgs g;
        g.data = p->data32;
        g.theta = p->theta32;
        g.xb0 = p->xb[0];
        g.xb1 = p->xb[1];
        g.db0 = p->db_raw[0];
        g.db1 = p->db_raw[1];
        g.partials = p->gpartials;
        g.st = p->st;
        g.ptr = p->gptr;
        g.idx = p->gidx;
        g.T = p->graph_T;
        g.R = p->graph_R;
        return launch_graph_sweep(p->K, init, p->grid_graph, g, p->stream);
    }
    const int *gs = a.kw ? p->grid_sweep_tp : p->grid_sweep;
    const int *gi = a.kw ? p->grid_sweep_init_tp : p->grid_sweep_init;
    if (v == 1) return launch_sweep_tma(p->K, init, init ? gi[1] : gs[1], a, p->stream);
    return launch_sweep(p->K, init, init ? gi[0] : gs[0], a, p->stream);
}

static int ensure_chunk_graph(pasc_gb300_problem *p)
{
    // (the captured kernel depends on the theta-in-penalty flag too: set_usethetainpenalty
    // destroys the graph)
    if (p->chunk_graph && p->chunk_graph_variant == p->variant) return PASC_OK;
    if (p->chunk_graph) {
        cudaGraphExecDestroy(p->chunk_graph);
        p->chunk_graph = nullptr;
    }
    CU(cudaStreamSynchronize(p->stream));
    SweepArgs a;
    sweep_args(p, &a);
    cudaGraph_t graph;
    CU(cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < GRAPH_CHUNK; i++) {
        cudaError_t e = launch_variant(p, p->variant, false, a);
        if (e != cudaSuccess) {
            cudaStreamEndCapture(p->stream, &graph);
            return fail(PASC_ERR_CUDA, "sweep capture: %s", cudaGetErrorString(e));
        }
    }
    CU(cudaStreamEndCapture(p->stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&p->chunk_graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        p->chunk_graph = nullptr;
        return fail(PASC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    p->chunk_graph_len = GRAPH_CHUNK;
    p->chunk_graph_variant = p->variant;
    return PASC_OK;
}

static int check_device_error(pasc_gb300_problem *p)
{
    if (p->st_h->error)
        return fail(PASC_ERR_TIMEOUT, "spgqp: a bounded wait for a bulk copy gave up inside the sweep");
    return PASC_OK;
}

static void sync_run_from_device(pasc_gb300_problem *p)
{
    const SpgDevState *h = p->st_h;
    SpgRun &r = p->run;
    r.it = h->it;
    r.hessmult = h->hessmult;
    r.status = h->status;
    r.fx = h->fx;
    r.dd = h->dd;
    r.dAd = h->dAd;
    p->cur = h->cur;
    p->fx_last = h->fx;
    p->have_fx = true;
}

static void fill_device_state(pasc_gb300_problem *p, SpgDevState *h)
{
    const pasc_gb300_spgqp_opts *o = &p->run.o;
    memset(h, 0, sizeof(SpgDevState));
    // alpha of the first direction (:108); SPGQPSolverC steps by alphainit / eps
    const double a0 = p->solver_type == 2 ? (p->coeffA == 0 ? 1.0 : 1.0 / p->coeffA) * o->alphainit : o->alphainit;
    h->alpha_prev = a0;
    h->alpha_cur = a0;
    h->coeffmode = p->solver_type == 2 ? 1 : 0;
    h->coeff = p->coeffA;
    h->bscale = p->coeffB;
    h->eps = o->eps;
    h->gamma = o->gamma;
    h->sigma1 = o->sigma1;
    h->sigma2 = o->sigma2;
    h->maxit = o->maxit;
    h->m = o->m;
    h->stop_difff = o->stop_difff;
    h->stop_normgp = o->stop_normgp;
    h->stop_Anormgp = o->stop_Anormgp;
    h->status = PASC_SPG_RUNNING;
    h->cur = p->cur;
}

// Choices of the sweep kernel made by timing, shared by the problems of the process: one per
// device, K, sweep form (data / materialised b / theta in the penalty) and power-of-two bucket
// of T, so that a problem of a shape already timed starts without the timing runs.
struct VariantKey {
    int device, K, form, tbucket;
    bool operator<(const VariantKey &o) const
    {
        return std::tie(device, K, form, tbucket) < std::tie(o.device, o.K, o.form, o.tbucket);
    }
};
struct VariantChoice {
    int variant, blocks_per_sm;
};
static std::mutex variant_cache_mutex;
static std::map<VariantKey, VariantChoice> variant_cache;

static VariantKey variant_key(const pasc_gb300_problem *p)
{
    int tb = 0;
    for (long t = p->T; t > 1; t >>= 1) tb++;
    return VariantKey{p->device, p->K, p->bmat ? 1 : (p->tp ? 2 : 0), tb};
}

// Chooses the sweep kernel and its grid by timing: every kernel (one timestep per thread;
// bulk-copy tiles) at every grid of 1, 2, ... blocks per SM up to its occupancy (each block
// walks the tiles grid-stride).  A candidate runs the solve's own INIT sweep and then four
// regular sweeps, of which the fastest of the last three is its time; gamma is saved first
// and put back afterwards, so the solve that follows is unchanged.  The choice is kept for
// the problem's lifetime and for later problems of the same device, K, sweep form and
// power-of-two bucket of T.  A start point that is already stationary (the sweeps stop at
// once) says nothing about speed: the bulk-copy kernel at full occupancy is taken untimed.
static int autotune_variant(pasc_gb300_problem *p)
{
    if (p->graph && p->variant < 0) p->variant = p->img_W > 0 ? 1 : 0;  // the fused image sweep where it applies
    if (p->variant >= 0) return PASC_OK;
    int *gs = p->tp ? p->grid_sweep_tp : p->grid_sweep;
    const int *gmax = p->tp ? p->grid_sweep_tp_max : p->grid_sweep_max;
    if (!sweep_tma_supported(p->K)) {
        p->variant = 0;
        return PASC_OK;
    }
    const VariantKey key = variant_key(p);
    {
        std::lock_guard<std::mutex> g(variant_cache_mutex);
        auto it = variant_cache.find(key);
        if (it != variant_cache.end()) {
            const int v = it->second.variant;
            const long g2 = (long)it->second.blocks_per_sm * p->sms;
            p->variant = v;
            gs[v] = (int)(g2 < gmax[v] ? g2 : gmax[v]);
            return PASC_OK;
        }
    }
    cudaStream_t s = p->stream;
    SweepArgs a;
    sweep_args(p, &a);
    const int cur0 = p->cur;
    float *saved = reinterpret_cast<float *>(p->stage64);  // N doubles: room for the N floats of gamma
    CU(cudaMemcpyAsync(saved, p->xb[cur0], sizeof(float) * p->N, cudaMemcpyDeviceToDevice, s));
    float best = 1e30f;
    int bestv = 0, bestm = 1;
    bool untimed = false;
    cudaEvent_t evs[5];
    for (int q = 0; q < 5; q++) CU(cudaEventCreate(&evs[q]));
    int rc = PASC_OK;
    for (int v = 0; v < 2 && rc == PASC_OK && !untimed; v++) {
        const int mmax = (gmax[v] + p->sms - 1) / p->sms;
        for (int m = 1; m <= mmax && rc == PASC_OK && !untimed; m++) {
            const long g = (long)m * p->sms;
            gs[v] = (int)(g < gmax[v] ? g : gmax[v]);
            fill_device_state(p, p->st_h);
            p->st_h->maxit = 1 << 30;
            p->st_h->stop_difff = p->st_h->stop_normgp = p->st_h->stop_Anormgp = 0;
            cudaError_t e = cudaMemcpyAsync(p->st, p->st_h, sizeof(SpgDevState), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = launch_variant(p, v, true, a);
            for (int q = 0; q < 4 && e == cudaSuccess; q++) {
                e = cudaEventRecord(evs[q], s);
                if (e == cudaSuccess) e = launch_variant(p, v, false, a);
            }
            if (e == cudaSuccess) e = cudaEventRecord(evs[4], s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(p->st_h, p->st, sizeof(SpgDevState), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                rc = fail(PASC_ERR_CUDA, "sweep tuning: %s", cudaGetErrorString(e));
                break;
            }
            if (p->st_h->error) break;
            if (p->st_h->status != PASC_SPG_RUNNING) {
                untimed = true;
                break;
            }
            float t = 1e30f;
            for (int q = 1; q < 4; q++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, evs[q], evs[q + 1]);
                t = ms < t ? ms : t;
            }
            if (t < best) {
                best = t;
                bestv = v;
                bestm = m;
            }
        }
    }
    for (int q = 0; q < 5; q++) cudaEventDestroy(evs[q]);
    CU(cudaMemcpyAsync(p->xb[cur0], saved, sizeof(float) * p->N, cudaMemcpyDeviceToDevice, s));
    CU(cudaStreamSynchronize(s));
    p->cur = cur0;
    gs[0] = gmax[0];
    gs[1] = gmax[1];
    if (rc != PASC_OK) return rc;
    CHK(check_device_error(p));
    if (untimed) {
        p->variant = 1;
        return PASC_OK;
    }
    p->variant = bestv;
    const long g = (long)bestm * p->sms;
    gs[bestv] = (int)(g < gmax[bestv] ? g : gmax[bestv]);
    p->tune_ms = best;
    std::lock_guard<std::mutex> lk(variant_cache_mutex);
    variant_cache[key] = VariantChoice{bestv, bestm};
    return PASC_OK;
}

// spgqpsolver.cpp:104-137 plus the first direction (one INIT sweep)
static int mixed_start(pasc_gb300_problem *p)
{
    const pasc_gb300_spgqp_opts *o = &p->run.o;
    if (o->stop_normgp_normb || o->stop_Anormgp_normb)
        return fail(PASC_ERR_NOTSUPP, "spgqp: ||b||-scaled stopping tests need the fp64 path");
    cudaStream_t s = p->stream;
    CHK(autotune_variant(p));
    CHK(ensure_chunk_graph(p));
    SpgDevState *h = p->st_h;
    fill_device_state(p, h);
    SweepArgs a;
    sweep_args(p, &a);
    CU(cudaEventRecord(p->ev0, s));
    CU(cudaMemcpyAsync(p->st, h, sizeof(SpgDevState), cudaMemcpyHostToDevice, s));
    CU(launch_variant(p, p->variant, true, a));
    CU(cudaEventRecord(p->ev1, s));
    CU(cudaMemcpyAsync(h, p->st, sizeof(SpgDevState), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    p->run.launches += p->graph && p->variant == 0 ? 2 : 1;
    p->run.time_s += ms * 1e-3;
    CHK(check_device_error(p));
    sync_run_from_device(p);
    return PASC_OK;
}

// Launches n regular sweeps.  With poll, the status word is read after chunks of growing
// length and launching stops once the solve has ended; without poll exactly n sweeps are
// launched back to back (sweeps after the end return at once) and timed as one region.
static int mixed_iterate(pasc_gb300_problem *p, long n, int poll)
{
    cudaStream_t s = p->stream;
    SweepArgs a;
    sweep_args(p, &a);
    SpgDevState *h = p->st_h;
    if (p->run.status != PASC_SPG_RUNNING) return PASC_OK;
    CHK(ensure_chunk_graph(p));
    const long room = p->run.o.maxit - p->run.it;
    if (n > room) n = room;
    long done = 0;
    int step = 0;
    const int sched[] = {2, 4, 8};
    CU(cudaEventRecord(p->ev0, s));
    while (done < n) {
        long want = poll ? (step < 3 ? sched[step] : GRAPH_CHUNK) : GRAPH_CHUNK;
        step++;
        if (want > n - done) want = n - done;
        if (want == GRAPH_CHUNK) {
            CU(cudaGraphLaunch(p->chunk_graph, s));
        } else {
            for (long q = 0; q < want; q++) CU(launch_variant(p, p->variant, false, a));
        }
        done += want;
        p->run.launches += (int)want * (p->graph && p->variant == 0 ? 2 : 1);
        if (poll) {
            CU(cudaMemcpyAsync(h, p->st, sizeof(SpgDevState), cudaMemcpyDeviceToHost, s));
            CU(cudaStreamSynchronize(s));
            if (h->status != PASC_SPG_RUNNING || h->error) break;
        }
    }
    CU(cudaEventRecord(p->ev1, s));
    CU(cudaMemcpyAsync(h, p->st, sizeof(SpgDevState), cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p->ev0, p->ev1);
    p->run.time_s += ms * 1e-3;
    p->run.last_iterate_ms = ms;
    p->run.last_iterate_launches = (int)done * (p->graph && p->variant == 0 ? 2 : 1);
    CHK(check_device_error(p));
    sync_run_from_device(p);
    if (p->run.status == PASC_SPG_RUNNING && p->run.it >= p->run.o.maxit) p->run.status = PASC_SPG_MAXIT;
    return PASC_OK;
}

static int check_opts(const pasc_gb300_spgqp_opts *o)
{
    if (!o) return fail(PASC_ERR_ARG, "spgqp: NULL options");
    if (o->m < 1 || o->m > MMAX_STATE) return fail(PASC_ERR_ARG, "spgqp: m must be in [1, %d]", MMAX_STATE);
    if (o->maxit < 0) return fail(PASC_ERR_ARG, "spgqp: maxit must be >= 0");
    return PASC_OK;
}

static int spgqp_start(pasc_gb300_problem *p, const pasc_gb300_spgqp_opts *o)
{
    p->run = SpgRun();
    p->run.o = *o;
    p->run.started = true;
    return p->precision == PASC_PREC_FP64 ? fp64_start(p) : mixed_start(p);
}

static int spgqp_iterate(pasc_gb300_problem *p, long n, int poll)
{
    return p->precision == PASC_PREC_FP64 ? fp64_iterate(p, n) : mixed_iterate(p, n, poll);
}

int pasc_gb300_spgqp_start(pasc_gb300_problem *p, const pasc_gb300_spgqp_opts *o)
{
    if (!p) return fail(PASC_ERR_ARG, "spgqp_start: NULL problem");
    if (p->fem_inner) return fail(PASC_ERR_NOTSUPP, "spgqp_start: a reduced (fem_reduce < 1) problem solves with spgqp_solve");
    CHK(check_opts(o));
    CU(cudaSetDevice(p->device));
    return spgqp_start(p, o);
}

int pasc_gb300_spgqp_iterate(pasc_gb300_problem *p, long n, int poll, pasc_gb300_spgqp_stats *st)
{
    if (p && p->fem_inner) return fail(PASC_ERR_NOTSUPP, "spgqp_iterate: a reduced (fem_reduce < 1) problem solves with spgqp_solve");
    if (!p) return fail(PASC_ERR_ARG, "spgqp_iterate: NULL problem");
    if (!p->run.started) return fail(PASC_ERR_STATE, "spgqp_iterate: call pasc_gb300_spgqp_start first");
    if (n < 0) return fail(PASC_ERR_ARG, "spgqp_iterate: n must be >= 0");
    CU(cudaSetDevice(p->device));
    CHK(spgqp_iterate(p, n, poll));
    fill_stats(p->run, st);
    return PASC_OK;
}

int pasc_gb300_spgqp_last_iterate(pasc_gb300_problem *p, double *ms, int *launches)
{
    if (!p) return fail(PASC_ERR_ARG, "spgqp_last_iterate: NULL problem");
    if (ms) *ms = p->run.last_iterate_ms;
    if (launches) *launches = p->run.last_iterate_launches;
    return PASC_OK;
}

int pasc_gb300_spgqp_solve(pasc_gb300_problem *p, const pasc_gb300_spgqp_opts *o, pasc_gb300_spgqp_stats *st)
{
    if (!p) return fail(PASC_ERR_ARG, "spgqp_solve: NULL problem");
    CHK(check_opts(o));
    CU(cudaSetDevice(p->device));
    if (p->fem_inner) {
        // the reduced QP (b and the warm start written by update_b), then the prolongation of
        // its solution to the full gamma (graphh1fem.cpp:292-303)
        pasc_gb300_problem *q = p->fem_inner;
        pasc_gb300_spgqp_stats ist;
        CHK(pasc_gb300_spgqp_solve(q, o, &ist));
        if (p->precision == PASC_PREC_FP64)
            CU((launch_fem_prolongate<double, double>(q->x, p->x, p->T, q->T, p->K, p->fem_type, p->stream)));
        else
            CU((launch_fem_prolongate<float, float>(q->xb[q->cur], p->xb[p->cur], p->T, q->T, p->K, p->fem_type,
                                                   p->stream)));
        CU(cudaStreamSynchronize(p->stream));
        p->fx_last = q->fx_last;
        p->have_fx = q->have_fx;
        ist.kernel_launches += 1;
        if (st) *st = ist;
        return PASC_OK;
    }
    CHK(spgqp_start(p, o));
    CHK(spgqp_iterate(p, o->maxit, 1));
    if (p->run.status == PASC_SPG_RUNNING) p->run.status = PASC_SPG_MAXIT;
    fill_stats(p->run, st);
    return PASC_OK;
}

int pasc_gb300_get_fx(pasc_gb300_problem *p, double *fx)
{
    if (!p || !fx) return fail(PASC_ERR_ARG, "get_fx: NULL argument");
    if (!p->have_fx) return fail(PASC_ERR_STATE, "get_fx: no solve since the last change of gamma");
    *fx = p->fx_last;
    return PASC_OK;
}

// ---------------------------------------------------------------------------------------
// TSSolver::solve (include/general/solver/tssolver.h:492-715)
// ---------------------------------------------------------------------------------------
int pasc_gb300_ts_solve(pasc_gb300_problem *p, const pasc_gb300_ts_opts *ts,
                        const pasc_gb300_spgqp_opts *spg, const double *gamma_restart,
                        pasc_gb300_ts_stats *out)
{
    if (!p || !ts || !spg) return fail(PASC_ERR_ARG, "ts_solve: NULL argument");
    CHK(check_opts(spg));
    CU(cudaSetDevice(p->device));
    auto t0 = std::chrono::steady_clock::now();
    const int annealing = ts->annealing > 0 ? ts->annealing : 1;
    std::vector<double> gbest, tbest;
    double best_aic = DBL_MAX, keepL = DBL_MAX, keepdL = DBL_MAX, keepaic = DBL_MAX;
    int keepit = 0, it_sum = 0, spg_it = 0, spg_hm = 0, launches = 0, increased = 0;

    for (int an = 0; an < annealing; an++) {
        if (ts->init_permute) {  // :528-530
            CHK(permute_gamma_async(p));
            launches += p->precision == PASC_PREC_FP64 ? 1 : 1;
        }
        double L = DBL_MAX, L_old, deltaL = DBL_MAX;
        int it;
        for (it = 0; it < ts->maxit; it++) {
            if (!ts->thetasolved) CHK(update_theta_async(p, &launches));  // :550
            CHK(update_b_async(p, &launches));                            // :586
            pasc_gb300_spgqp_stats ss;
            CHK(pasc_gb300_spgqp_solve(p, spg, &ss));                     // :590
            spg_it += ss.it;
            spg_hm += ss.hessmult;
            launches += ss.kernel_launches;
            L_old = L;  // :618-620
            L = ss.fx;
            deltaL = fabs(L - L_old);
            if (L - L_old > 0) increased++;  // :637-639
            if (ts->relative ? (deltaL < ts->eps * fabs(L)) : (deltaL < ts->eps)) break;  // :642
        }
        it_sum += it;
        const double aic = 2 * log(L) + p->K;  // graphh1fem.h:444-447
        if (annealing <= 1 || aic < best_aic) {
            if (annealing > 1) {
                gbest.resize(p->N);
                tbest.resize((size_t)p->K * p->xdim);
                CHK(pasc_gb300_get_gamma(p, gbest.data()));
                CHK(pasc_gb300_get_theta(p, tbest.data()));
            }
            best_aic = aic;
            keepL = L;
            keepdL = deltaL;
            keepaic = aic;
            keepit = it;
        }
        if (an < annealing - 1 && gamma_restart) CHK(pasc_gb300_set_gamma(p, gamma_restart));  // :700-702
    }
    if (annealing > 1) {
        CHK(pasc_gb300_set_gamma(p, gbest.data()));
        CHK(pasc_gb300_set_theta(p, tbest.data()));
        p->fx_last = keepL;
        p->have_fx = true;
    }
    CU(cudaStreamSynchronize(p->stream));
    CHK(mc_check_error(p));
    if (out) {
        out->it_last = keepit;
        out->it_sum = it_sum;
        out->spg_it_sum = spg_it;
        out->spg_hessmult_sum = spg_hm;
        out->kernel_launches = launches;
        out->L_increased = increased;
        out->L = keepL;
        out->deltaL = keepdL;
        out->aic = keepaic;
        out->time_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return PASC_OK;
}

int pasc_gb300_abserr_reconstructed(pasc_gb300_problem *p, const double *solution, double *abserr)
{
    if (!p || !solution || !abserr) return fail(PASC_ERR_ARG, "abserr: NULL argument");
    if (p->xdim > 1) return fail(PASC_ERR_NOTSUPP, "abserr: 1-D signals only (Signal1DData)");
    CU(cudaSetDevice(p->device));
    const double *g64 = nullptr;
    CHK(gamma64(p, &g64));
    // the solution goes through the Ad buffer (fp64) or the tail of a scratch allocation
    double *sol_d = nullptr;
    CU(cudaMallocAsync((void **)&sol_d, sizeof(double) * p->T, p->stream));
    CU(cudaMemcpyAsync(sol_d, solution, sizeof(double) * p->T, cudaMemcpyHostToDevice, p->stream));
    cudaError_t e = launch_recon_abserr(g64, p->theta64, sol_d, p->T, p->K, p->red, p->red_out, p->stream);
    cudaFreeAsync(sol_d, p->stream);
    if (e != cudaSuccess) return fail(PASC_ERR_CUDA, "abserr kernel: %s", cudaGetErrorString(e));
    double v[1];
    CHK(read_red(p, 1, v));
    *abserr = v[0];
    return PASC_OK;
}

int pasc_gb300_argmax_labels(pasc_gb300_problem *p, int *labels)
{
    if (!p || !labels) return fail(PASC_ERR_ARG, "argmax: NULL argument");
    CU(cudaSetDevice(p->device));
    const double *g64 = nullptr;
    CHK(gamma64(p, &g64));
    CU(launch_argmax(g64, p->labels_d, p->T, p->K, p->stream));
    CU(cudaMemcpyAsync(labels, p->labels_d, sizeof(int) * p->T, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

// ---------------------------------------------------------------------------------------
// device-pointer kernels
// ---------------------------------------------------------------------------------------
int pasc_gb300_project_f64(double *x_dev, long T, int K, void *stream)
{
    if (!x_dev && T > 0) return fail(PASC_ERR_ARG, "project_f64: NULL x");
    if (T < 0 || K < 1 || K > KMAX_PLAIN) return fail(PASC_ERR_ARG, "project_f64: bad T/K (%ld, %d)", T, K);
    CU(launch_project_f64(x_dev, T, K, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_project_f32(float *x_dev, long T, int K, void *stream)
{
    if (!x_dev && T > 0) return fail(PASC_ERR_ARG, "project_f32: NULL x");
    if (T < 0 || K < 1 || K > KMAX_GROUP) return fail(PASC_ERR_ARG, "project_f32: bad T/K (%ld, %d)", T, K);
    CU(launch_project_f32(x_dev, T, K, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_fem_h1_matmult_f64(const double *x_dev, double *y_dev, long T, int K, double coeff, void *stream)
{
    if ((!x_dev || !y_dev) && T > 0) return fail(PASC_ERR_ARG, "matmult_f64: NULL pointer");
    if (T < 0 || K < 1) return fail(PASC_ERR_ARG, "matmult_f64: bad T/K");
    CU(launch_matmult_f64(x_dev, y_dev, T, K, coeff, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_fem_h1_matmult_f32(const float *x_dev, float *y_dev, long T, int K, float coeff, void *stream)
{
    if ((!x_dev || !y_dev) && T > 0) return fail(PASC_ERR_ARG, "matmult_f32: NULL pointer");
    if (T < 0 || K < 1) return fail(PASC_ERR_ARG, "matmult_f32: bad T/K");
    CU(launch_matmult_f32(x_dev, y_dev, T, K, coeff, (cudaStream_t)stream));
    return PASC_OK;
}

}  // extern "C"

extern "C" {

int pasc_gb300_set_sweep_variant(pasc_gb300_problem *p, int variant)
{
    if (!p) return fail(PASC_ERR_ARG, "set_sweep_variant: NULL problem");
    if (variant < -1 || variant > 1) return fail(PASC_ERR_ARG, "set_sweep_variant: variant must be -1, 0 or 1");
    if (p->precision != PASC_PREC_MIXED) return fail(PASC_ERR_STATE, "set_sweep_variant: mixed precision only");
    if (variant == 1 && !sweep_tma_supported(p->K)) return fail(PASC_ERR_NOTSUPP, "set_sweep_variant: K not supported");
    if (variant == 1 && p->graph && p->img_W == 0)
        return fail(PASC_ERR_NOTSUPP, "set_sweep_variant: the fused image sweep needs T = 1 on a pixel grid (H >= 2)");
    p->variant = variant;
    p->run.started = false;
    // a pinned kernel runs at full occupancy; -1 tunes kernel and grid again
    for (int v = 0; v < 2; v++) {
        p->grid_sweep[v] = p->grid_sweep_max[v];
        if (p->tp) p->grid_sweep_tp[v] = p->grid_sweep_tp_max[v];
    }
    p->tune_ms = 0.f;
    return PASC_OK;
}

int pasc_gb300_get_sweep_tuning(pasc_gb300_problem *p, int *variant, int *blocks, double *sweep_ms)
{
    if (!p || !variant || !blocks || !sweep_ms) return fail(PASC_ERR_ARG, "get_sweep_tuning: NULL argument");
    *variant = p->variant;
    const int v = p->variant < 0 ? 1 : p->variant;
    *blocks = p->tp ? p->grid_sweep_tp[v] : p->grid_sweep[v];
    *sweep_ms = p->tune_ms;
    return PASC_OK;
}

int pasc_gb300_set_fem(pasc_gb300_problem *p, double fem_reduce, int fem_type)
{
    if (!p) return fail(PASC_ERR_ARG, "set_fem: NULL problem");
    if (!(fem_reduce > 0.0) || fem_reduce > 1.0) return fail(PASC_ERR_ARG, "set_fem: fem_reduce must be in (0, 1]");
    if (fem_type != 0 && fem_type != 1) return fail(PASC_ERR_ARG, "set_fem: fem_type 0 (FEM-SUM) or 1 (FEM-HAT)");
    if (p->tp && fem_reduce < 1.0)
        return fail(PASC_ERR_NOTSUPP, "set_fem: theta in the penalty with a reduced (fem_reduce < 1) problem");
    if (p->graph && fem_reduce < 1.0)
        return fail(PASC_ERR_NOTSUPP, "set_fem: FEM reduction of a graph (R > 1) problem");
    CU(cudaSetDevice(p->device));
    CU(cudaStreamSynchronize(p->stream));
    if (p->fem_inner) {
        free_all(p->fem_inner);
        p->fem_inner = nullptr;
    }
    p->fem_reduce = fem_reduce;
    p->fem_type = fem_type;
    p->run.started = false;
    p->have_fx = false;
    if (!(fem_reduce < 1.0)) return PASC_OK;  // not reduced (Fem::is_reduced, fem.h:236-246)
    const long T2 = fem_T_reduced(p->T, fem_reduce);
    if (fem_type == 1 && (T2 < 2 || p->T < 2)) return fail(PASC_ERR_ARG, "set_fem: FEM-HAT needs T and T2 >= 2");
    pasc_gb300_problem *q = nullptr;
    CHK(pasc_gb300_create(&q, T2, p->K, 1, p->precision, p->epssqr, p->device));
    q->b_external = true;
    if (p->precision == PASC_PREC_MIXED) {
        // the reduced b is materialised (the sweeps read it instead of forming it from data)
        const size_t nx = (size_t)(T2 + PAD_FRONT + PAD_BACK) * p->K;
        int rc = dalloc(&q->bmat_raw, nx);
        if (rc) {
            free_all(q);
            return rc;
        }
        cudaMemset(q->bmat_raw, 0, sizeof(float) * nx);
        q->bmat = q->bmat_raw + (size_t)PAD_FRONT * p->K;
        const long nt_tma = (T2 + sweep_tma_tile_width() - 1) / sweep_tma_tile_width();
        long g = (long)sweep_tma_blocks_per_sm(p->K, false, true) * q->sms;
        q->grid_sweep[1] = (int)(g < nt_tma ? (g < 1 ? 1 : g) : nt_tma);
        q->grid_sweep_max[1] = q->grid_sweep[1];
        g = (long)sweep_tma_blocks_per_sm(p->K, true, true) * q->sms;
        q->grid_sweep_init[1] = (int)(g < nt_tma ? (g < 1 ? 1 : g) : nt_tma);
    }
    q->solver_type = p->solver_type;
    p->fem_inner = q;
    fem_set_inner_coeffs(p);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(PASC_ERR_CUDA, "set_fem: initialisation failed");
    return PASC_OK;
}

int pasc_gb300_get_fem(pasc_gb300_problem *p, double *fem_reduce, int *fem_type, long *T_reduced)
{
    if (!p) return fail(PASC_ERR_ARG, "get_fem: NULL problem");
    if (fem_reduce) *fem_reduce = p->fem_reduce;
    if (fem_type) *fem_type = p->fem_type;
    if (T_reduced) *T_reduced = p->fem_inner ? p->fem_inner->T : p->T;
    return PASC_OK;
}

int pasc_gb300_time_model_kernels(pasc_gb300_problem *p, int which, int reps, double *ms_per_call)
{
    if (!p || !ms_per_call) return fail(PASC_ERR_ARG, "time_model_kernels: NULL argument");
    if ((which != 1 && which != 2) || reps < 1) return fail(PASC_ERR_ARG, "time_model_kernels: which 1 or 2, reps >= 1");
    CU(cudaSetDevice(p->device));
    CU(cudaStreamSynchronize(p->stream));
    CU(cudaEventRecord(p->ev0, p->stream));
    for (int r = 0; r < reps; r++) {
        if (which == 1) CHK(update_theta_async(p, nullptr));
        else CHK(update_b_async(p, nullptr));
    }
    CU(cudaEventRecord(p->ev1, p->stream));
    CU(cudaEventSynchronize(p->ev1));
    CHK(mc_check_error(p));
    float ms = 0.f;
    CU(cudaEventElapsedTime(&ms, p->ev0, p->ev1));
    *ms_per_call = (double)ms / reps;
    return PASC_OK;
}

int pasc_gb300_get_b(pasc_gb300_problem *p, double *b)
{
    if (!p || !b) return fail(PASC_ERR_ARG, "get_b: NULL argument");
    CU(cudaSetDevice(p->device));
    const double *src = nullptr;
    if (p->precision == PASC_PREC_FP64) {
        src = p->b;
    } else if (p->xdim > 1) {
        CU(launch_f32_to_f64(p->bmat, p->stage64, p->N, p->stream));
        src = p->stage64;
    } else {
        CU(launch_residual_f64(p->data64, p->theta64, p->stage64, p->T, p->K, p->coeffB, p->stream));
        src = p->stage64;
    }
    CU(cudaMemcpyAsync(b, src, sizeof(double) * p->N, cudaMemcpyDeviceToHost, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

int pasc_gb300_set_residual_engine(pasc_gb300_problem *p, int engine)
{
    if (!p) return fail(PASC_ERR_ARG, "set_residual_engine: NULL problem");
    if (p->xdim == 1) return fail(PASC_ERR_STATE, "set_residual_engine: multichannel data only");
    if (engine != 0 && engine != 1) return fail(PASC_ERR_ARG, "set_residual_engine: engine must be 0 or 1");
    if (engine == 0 && !mc_tc_supported(p->xdim))
        return fail(PASC_ERR_NOTSUPP, "set_residual_engine: tensor cores need xdim in {64, 128, 256}");
    CU(cudaSetDevice(p->device));
    p->mc_engine = engine;
    p->run.started = false;
    if (p->have_data) {
        CHK(mc_residual_async(p, nullptr));
        CU(cudaStreamSynchronize(p->stream));
        CHK(mc_check_error(p));
    }
    return PASC_OK;
}

int pasc_gb300_get_residual_engine(pasc_gb300_problem *p, int *engine)
{
    if (!p || !engine) return fail(PASC_ERR_ARG, "get_residual_engine: NULL argument");
    *engine = p->xdim > 1 ? p->mc_engine : -1;
    return PASC_OK;
}

int pasc_gb300_get_sweep_variant(pasc_gb300_problem *p, int *variant)
{
    if (!p || !variant) return fail(PASC_ERR_ARG, "get_sweep_variant: NULL argument");
    *variant = p->variant;
    return PASC_OK;
}

// GraphH1FEMModel(..., usethetainpenalty) (graphh1fem.cpp:8-19, 154-160): block k of the gamma
// QP's A is scaled by alpha*theta_k*theta_k, and the theta step includes the penalty term.
// One-dimensional data without FEM reduction only: the reference's theta step multiplies the
// reduced operator with the full gamma (PETSc refuses the sizes), and its multichannel form
// has no penalty term.
int pasc_gb300_set_usethetainpenalty(pasc_gb300_problem *p, int on)
{
    if (!p) return fail(PASC_ERR_ARG, "set_usethetainpenalty: NULL problem");
    if (on && p->xdim != 1)
        return fail(PASC_ERR_NOTSUPP, "set_usethetainpenalty: one-dimensional data (xdim == 1) only");
    if (on && p->fem_inner)
        return fail(PASC_ERR_NOTSUPP, "set_usethetainpenalty: not with a reduced (fem_reduce < 1) problem");
    if (on && p->graph) return fail(PASC_ERR_NOTSUPP, "set_usethetainpenalty: not with a graph (R > 1) problem");
    if (on && p->solver_type == 2) return fail(PASC_ERR_NOTSUPP, "set_usethetainpenalty: not with SPGQPSolverC");
    CU(cudaSetDevice(p->device));
    CU(cudaStreamSynchronize(p->stream));
    p->run.started = false;
    p->have_fx = false;
    if (p->chunk_graph) {
        cudaGraphExecDestroy(p->chunk_graph);
        p->chunk_graph = nullptr;
    }
    if (!on) {
        p->tp = false;
        return PASC_OK;
    }
    if (!p->tp_ck64 || !p->tp_kw32) {
        int rc;
        if (!p->tp_ck64 && (rc = dalloc(&p->tp_ck64, p->K))) return rc;
        if (!p->tp_kw32 && (rc = dalloc(&p->tp_kw32, p->K))) return rc;
    }
    p->tp = true;
    if (p->precision == PASC_PREC_MIXED) {
        // the theta-in-penalty sweeps may hold fewer blocks per SM; never more than the
        // partials buffer was sized for
        const long nt_thread = (p->T + sweep_tile_width() - 1) / sweep_tile_width();
        const long nt_tma = (p->T + sweep_tma_tile_width() - 1) / sweep_tma_tile_width();
        auto grid = [&](long per_sm, long ntiles, int cap) {
            long g = per_sm * p->sms;
            g = g < ntiles ? g : ntiles;
            g = g < cap ? g : cap;
            return (int)(g < 1 ? 1 : g);
        };
        p->grid_sweep_tp[0] = grid(sweep_blocks_per_sm(p->K, false, true), nt_thread, p->grid_sweep_max[0]);
        p->grid_sweep_tp_max[0] = p->grid_sweep_tp[0];
        p->grid_sweep_init_tp[0] = grid(sweep_blocks_per_sm(p->K, true, true), nt_thread, p->grid_sweep_init[0]);
        if (sweep_tma_supported(p->K)) {
            p->grid_sweep_tp[1] = grid(sweep_tma_blocks_per_sm(p->K, false, false, true), nt_tma, p->grid_sweep_max[1]);
            p->grid_sweep_tp_max[1] = p->grid_sweep_tp[1];
            p->grid_sweep_init_tp[1] =
                grid(sweep_tma_blocks_per_sm(p->K, true, false, true), nt_tma, p->grid_sweep_init[1]);
        }
    }
    CU(launch_tp_coeffs(p->theta64, p->coeffA, p->K, p->tp_ck64, p->tp_kw32, p->stream));
    CU(cudaStreamSynchronize(p->stream));
    return PASC_OK;
}

// GraphH1FEMModel on a Decomposition(T, graph, K, 1, 1) (graphh1fem.cpp:8-65 with a BGMGraph,
// blockgraphsparse.cpp:7-103): a problem of T*R blocks of K with the graph operator.
int pasc_gb300_create_graph(pasc_gb300_problem **out, long T, long R, int K, int precision, double epssqr, int device,
                            const int *nbr_ptr, const int *nbr_idx)
{
    if (!out) return fail(PASC_ERR_ARG, "create_graph: out is NULL");
    *out = nullptr;
    if (T < 1) return fail(PASC_ERR_ARG, "create_graph: T must be >= 1 (got %ld)", T);
    if (R < 1 || (double)T * (double)R > 2.0e9) return fail(PASC_ERR_ARG, "create_graph: R must be >= 1 and T*R < 2e9");
    if (const char *why = graph_check(R, nbr_ptr, nbr_idx)) return fail(PASC_ERR_ARG, "create_graph: %s", why);
    pasc_gb300_problem *p = nullptr;
    CHK(pasc_gb300_create(&p, T * R, K, 1, precision, epssqr, device));
    p->graph = true;
    p->graph_T = T;
    p->graph_R = R;
    p->graph_nnz = nbr_ptr[R];
    p->variant = -1;  // the fused image sweep where it applies, else the general graph sweep
    set_coeffs(p);
    int rc;
    auto bail = [&](int code) { free_all(p); return code; };
    if ((rc = dalloc(&p->gptr, (size_t)R + 1)) || (rc = dalloc(&p->gidx, (size_t)(p->graph_nnz > 0 ? p->graph_nnz : 1))))
        return bail(rc);
    if (cudaMemcpy(p->gptr, nbr_ptr, sizeof(int) * (R + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        (p->graph_nnz > 0 &&
         cudaMemcpy(p->gidx, nbr_idx, sizeof(int) * p->graph_nnz, cudaMemcpyHostToDevice) != cudaSuccess))
        return bail(fail(PASC_ERR_CUDA, "create_graph: upload failed"));
    if (precision == PASC_PREC_MIXED) {
        const long N = p->N;
        p->grid_graph = graph_sweep_grid(T * R);
        int W = 0, H = 0;
        if (T == 1 && graph_is_grid2d(R, nbr_ptr, nbr_idx, &W, &H)) {
            const int per_sm = image_sweep_blocks_per_sm(K);
            const int tiles = image_sweep_tiles(W, H);
            p->img_W = W;
            p->img_H = H;
            p->grid_image = std::max(1, std::min(tiles, per_sm * p->sms));
        }
        const int gp = std::max(p->grid_graph, p->grid_image);
        if ((rc = dalloc(&p->db_raw[0], N)) || (rc = dalloc(&p->db_raw[1], N)) ||
            (rc = dalloc(&p->gpartials, (size_t)gp * 4)))
            return bail(rc);
        cudaMemset(p->db_raw[0], 0, sizeof(float) * N);
        cudaMemset(p->db_raw[1], 0, sizeof(float) * N);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(PASC_ERR_CUDA, "create_graph: initialisation failed"));
    *out = p;
    return PASC_OK;
}

int pasc_gb300_get_graph(pasc_gb300_problem *p, long *T, long *R, long *nnz)
{
    if (!p) return fail(PASC_ERR_ARG, "get_graph: NULL problem");
    if (T) *T = p->graph ? p->graph_T : p->T;
    if (R) *R = p->graph ? p->graph_R : 1;
    if (nnz) *nnz = p->graph ? p->graph_nnz : 0;
    return PASC_OK;
}

// GraphH1FEMModel's gammasolvertype (include/general/model/graphh1fem.h:42-48, option
// graphh1femmodel_gammasolvertype, graphh1fem.cpp:12-16, 171-191): 0 auto (= 1), 1 SPGQPSolver,
// 2 SPGQPSolverC.  PERMON (3) and TAO (4) need libraries the reference links optionally.
int pasc_gb300_set_gamma_solver_type(pasc_gb300_problem *p, int type)
{
    if (!p) return fail(PASC_ERR_ARG, "set_gamma_solver_type: NULL problem");
    if (type < 0 || type > 4) return fail(PASC_ERR_ARG, "set_gamma_solver_type: type 0..4");
    if (type >= 3) return fail(PASC_ERR_NOTSUPP, "set_gamma_solver_type: PERMON / TAO solvers are not provided");
    if (type == 2 && p->tp)
        return fail(PASC_ERR_NOTSUPP, "set_gamma_solver_type: SPGQPSolverC with theta in the penalty");
    p->solver_type = type == 0 ? 1 : type;
    p->run.started = false;
    if (p->fem_inner) p->fem_inner->solver_type = p->solver_type;
    return PASC_OK;
}

int pasc_gb300_get_gamma_solver_type(pasc_gb300_problem *p, int *type)
{
    if (!p || !type) return fail(PASC_ERR_ARG, "get_gamma_solver_type: NULL argument");
    *type = p->solver_type;
    return PASC_OK;
}

int pasc_gb300_get_usethetainpenalty(pasc_gb300_problem *p, int *on)
{
    if (!p || !on) return fail(PASC_ERR_ARG, "get_usethetainpenalty: NULL argument");
    *on = p->tp ? 1 : 0;
    return PASC_OK;
}

}  // extern "C"

namespace pasc {
// lets other translation units report through pasc_gb300_last_error()
void record_error(const char *msg) { g_last_error = msg; }
}  // namespace pasc
