// vector.cu -- the vector level of the reference's backend interface on FP64 device buffers.
//
// The reference's solvers are templates over a vector type whose backend supplies a handful
// of operations: copy, axpy-like updates, dot products and norms, the operator product and
// the feasible-set projection (GeneralVector<VectorBase>, include/general/algebra/vector/
// generalvector.h:58-106; the PETSc backend calls VecCopy, VecAXPY, VecWAXPY, VecScale,
// VecDot and VecNorm, include/external/petscvector/algebra/vector/petscvector.h).  These entry
// points give a backend written against this library those operations on device memory, plus
// the two model steps of GraphH1FEMModel (residual b and the theta update) on device buffers,
// so that the reference's own generic SPGQPSolver and TSSolver can run with their vectors on
// the GPU (include/pasc/gb300_backend.hpp).  Arithmetic is FP64 in the reference's order for
// every element; the dot products are deterministic block trees.
#include <map>
#include <string>
#include <mutex>

#include "common.cuh"
#include "internal.h"

using namespace pasc;

namespace {

thread_local std::string g_vec_error_msg;

int vfail(int code, const char *msg)
{
    record_error(msg);
    return code;
}

#define VCU(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) {                                                                     \
            g_vec_error_msg = std::string(#call) + ": " + cudaGetErrorString(e_);                    \
            return vfail(PASC_ERR_CUDA, g_vec_error_msg.c_str());                                    \
        }                                                                                            \
    } while (0)

// Per-device reduction scratch of the dot products and the theta update (library-owned,
// allocated at the first use on a device, zeroed: its last-block counter must start at 0).
// The dot and theta entry points hold the mutex until their result is on the host, so calls
// from several threads take turns on it.
std::mutex g_scratch_mutex;
std::map<int, double *> g_scratch;

int scratch_for_current_device(double **out)
{
    int dev = 0;
    VCU(cudaGetDevice(&dev));
    auto it = g_scratch.find(dev);
    if (it == g_scratch.end()) {
        double *p = nullptr;
        const size_t n = dot_partials_size() + 16;
        if (cudaMalloc(&p, sizeof(double) * n) != cudaSuccess)
            return vfail(PASC_ERR_ALLOC, "vector: allocation of the reduction scratch failed");
        VCU(cudaMemset(p, 0, sizeof(double) * n));
        it = g_scratch.emplace(dev, p).first;
    }
    *out = it->second;
    return PASC_OK;
}

__global__ void waxpy_f64_kernel(double *w, double a, const double *x, const double *y, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) w[i] = __dadd_rn(__dmul_rn(a, x[i]), y[i]);
}

__global__ void scale_f64_kernel(double *x, double a, long n)
{
    const long stride = (long)gridDim.x * blockDim.x;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) x[i] = __dmul_rn(a, x[i]);
}

int grid_for(long n)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long g = (n + 255) / 256;
    if (g > (long)sms * 8) g = (long)sms * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

extern "C" {

int pasc_gb300_vec_alloc(double **v_dev, long n, int device)
{
    if (!v_dev || n < 0) return vfail(PASC_ERR_ARG, "vec_alloc: NULL pointer or n < 0");
    *v_dev = nullptr;
    if (pasc_gb300_device_count() <= device || device < 0) return vfail(PASC_ERR_ARG, "vec_alloc: no such device");
    VCU(cudaSetDevice(device));
    if (cudaMalloc((void **)v_dev, sizeof(double) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) {
        *v_dev = nullptr;
        return vfail(PASC_ERR_ALLOC, "vec_alloc: cudaMalloc failed");
    }
    VCU(cudaMemset(*v_dev, 0, sizeof(double) * (size_t)(n > 0 ? n : 1)));
    return PASC_OK;
}

int pasc_gb300_vec_free(double *v_dev)
{
    if (v_dev) VCU(cudaFree(v_dev));
    return PASC_OK;
}

int pasc_gb300_vec_set(double *v_dev, const double *host, long n)
{
    if (n < 0 || !v_dev || !host) return vfail(PASC_ERR_ARG, "vec_set: NULL pointer or n < 0");
    if (n) VCU(cudaMemcpy(v_dev, host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
    return PASC_OK;
}

int pasc_gb300_vec_get(const double *v_dev, double *host, long n)
{
    if (n < 0 || !v_dev || !host) return vfail(PASC_ERR_ARG, "vec_get: NULL pointer or n < 0");
    if (n) VCU(cudaMemcpy(host, v_dev, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
    return PASC_OK;
}

int pasc_gb300_vec_copy(double *y_dev, const double *x_dev, long n, void *stream)
{
    if (n < 0 || !x_dev || !y_dev) return vfail(PASC_ERR_ARG, "vec_copy: NULL pointer or n < 0");
    if (n && x_dev != y_dev)
        VCU(cudaMemcpyAsync(y_dev, x_dev, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_vec_axpy(double *y_dev, double a, const double *x_dev, long n, void *stream)
{
    if (n < 0 || !x_dev || !y_dev) return vfail(PASC_ERR_ARG, "vec_axpy: NULL pointer or n < 0");
    if (n) VCU(launch_axpy_f64(y_dev, a, x_dev, n, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_vec_waxpy(double *w_dev, double a, const double *x_dev, const double *y_dev, long n, void *stream)
{
    if (n < 0 || !w_dev || !x_dev || !y_dev) return vfail(PASC_ERR_ARG, "vec_waxpy: NULL pointer or n < 0");
    if (n) {
        waxpy_f64_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(w_dev, a, x_dev, y_dev, n);
        VCU(cudaGetLastError());
    }
    return PASC_OK;
}

int pasc_gb300_vec_scale(double *x_dev, double a, long n, void *stream)
{
    if (n < 0 || !x_dev) return vfail(PASC_ERR_ARG, "vec_scale: NULL pointer or n < 0");
    if (n) {
        scale_f64_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(x_dev, a, n);
        VCU(cudaGetLastError());
    }
    return PASC_OK;
}

int pasc_gb300_vec_dot(const double *x_dev, const double *y_dev, long n, double *out, void *stream)
{
    if (!out || n < 0 || !x_dev || !y_dev) return vfail(PASC_ERR_ARG, "vec_dot: NULL pointer or n < 0");
    *out = 0.0;
    if (n == 0) return PASC_OK;
    std::lock_guard<std::mutex> lk(g_scratch_mutex);
    double *scr = nullptr;
    int rc = scratch_for_current_device(&scr);
    if (rc != PASC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    double *res = scr + dot_partials_size();
    VCU(launch_dots_f64(1, x_dev, y_dev, nullptr, nullptr, nullptr, nullptr, n, scr, res, s));
    VCU(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, s));
    VCU(cudaStreamSynchronize(s));
    return PASC_OK;
}

int pasc_gb300_permute_f64(const double *src_dev, double *dst_dev, long T, int K, void *stream)
{
    if (T < 0 || K < 1 || (T > 0 && (!src_dev || !dst_dev || src_dev == dst_dev)))
        return vfail(PASC_ERR_ARG, "permute_f64: NULL or aliased pointers, or bad T/K");
    if (T) VCU(launch_permute_f64(src_dev, dst_dev, T, K, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_residual_f64(const double *data_dev, const double *theta_dev, double *b_dev, long T, int K,
                            double bscale, void *stream)
{
    if (T < 0 || K < 1 || (T > 0 && (!data_dev || !theta_dev || !b_dev)))
        return vfail(PASC_ERR_ARG, "residual_f64: NULL pointer or bad T/K");
    if (T) VCU(launch_residual_f64(data_dev, theta_dev, b_dev, T, K, bscale, (cudaStream_t)stream));
    return PASC_OK;
}

int pasc_gb300_theta_update_f64(const double *gamma_dev, const double *data_dev, double *theta_dev, long T, int K,
                                void *stream)
{
    if (T < 1 || K < 1 || !gamma_dev || !data_dev || !theta_dev)
        return vfail(PASC_ERR_ARG, "theta_update_f64: NULL pointer or bad T/K");
    std::lock_guard<std::mutex> lk(g_scratch_mutex);
    double *scr = nullptr;
    int rc = scratch_for_current_device(&scr);
    if (rc != PASC_OK) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    VCU(launch_theta_f64(gamma_dev, data_dev, theta_dev, T, K, scr, s));
    VCU(cudaStreamSynchronize(s));
    return PASC_OK;
}

}  // extern "C"
