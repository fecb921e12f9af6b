// noalloc.cu -- a theta update (K-means step of the FEM-H1 model) that allocates nothing.
//
// Some callers of this library cannot allocate device memory at the point where they need
// the theta step: hosts whose device memory is owned by another framework's allocator, and
// real-time loops that forbid allocation (and the implicit device synchronisation
// cudaMalloc/cudaFree may cause) after start-up.  For them this file offers pasc_gb300_theta_update_noalloc: the caller
// passes its own device buffers for the inputs and the output, and the reduction's scratch
// (per-block partial sums and the last-block ticket) lives in the file-scope array below,
// which every GPU that loads the library holds until the process exits.
//
// Limits: K <= 8 (the array holds 1024 blocks x 2*8 partial sums and a ticket, ~128 KiB).
// All calls on a device share the array and it keeps the last call's contents: each call
// clears the ticket before it launches, and calls that overlap on the GPU (different
// streams, or a second call before the first has finished) race on it.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace pasc {

constexpr int NOALLOC_THREADS = 256;
constexpr int NOALLOC_MAX_BLOCKS = 1024;
constexpr int NOALLOC_MAX_K = 8;
constexpr int NOALLOC_PARTIALS = NOALLOC_MAX_BLOCKS * 2 * NOALLOC_MAX_K;

// partial sums at [0, NOALLOC_PARTIALS), the ticket in the first word after them
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_PARTIALS + 32];

// theta_k = sum_t gamma_tk x_t / sum_t gamma_tk (src/petscvector/model/graphh1fem.cpp:347-380):
// compensated FP32 sums per thread, FP64 per block, FP64 over blocks by the last block.
template <int K>
__global__ void __launch_bounds__(NOALLOC_THREADS)
theta_noalloc_kernel(const float *gamma, const float *data, long T, double *theta, double *scratch)
{
    __shared__ double s_red[2 * K * (NOALLOC_THREADS / 32)];
    unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + NOALLOC_PARTIALS);
    KahanF sx[K], sg[K];
    const long stride = (long)gridDim.x * NOALLOC_THREADS;
    for (long t = (long)blockIdx.x * NOALLOC_THREADS + threadIdx.x; t < T; t += stride) {
        const float x = __ldg(data + t);
#pragma unroll
        for (int k = 0; k < K; k++) {
            const float gk = __ldg(gamma + t * K + k);
            sg[k].add(gk);
            sx[k].add(__fmul_rn(x, gk));
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
        for (int q = 0; q < 2 * K; q++) scratch[blockIdx.x * 2 * K + q] = v[q];
    }
    if (!last_block_done(ticket)) return;
    double w[2 * K];
#pragma unroll
    for (int q = 0; q < 2 * K; q++) w[q] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += NOALLOC_THREADS) {
#pragma unroll
        for (int q = 0; q < 2 * K; q++) w[q] += __ldcg(scratch + b * 2 * K + q);
    }
    block_sum<2 * K>(w, s_red);
    if (threadIdx.x == 0) {
        *ticket = 0;
#pragma unroll
        for (int k = 0; k < K; k++) theta[k] = (w[K + k] != 0.0) ? w[k] / w[K + k] : 0.0;
    }
}

}  // namespace pasc

using namespace pasc;

namespace {

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {nullptr};

// Device address of the scratch array on the current device.  The array's name is only a
// host-side stand-in for the symbol, so the address is looked up once per device (with that
// device current) and remembered for the life of the process: a cudaDeviceReset ends the
// context the address belongs to, and the entry point is not to be used on that device
// after one.
cudaError_t noalloc_scratch(int dev, double **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        double *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

// failures are reported through pasc_gb300_last_error(), like every other entry point
int noalloc_fail(int code, const char *msg)
{
    pasc::record_error(msg);
    return code;
}

}  // namespace

extern "C" {

int pasc_gb300_theta_update_noalloc(const float *gamma_dev, const float *data_dev, long T, int K,
                                    double *theta_dev, void *stream)
{
    if (K < 1 || K > NOALLOC_MAX_K)
        return noalloc_fail(PASC_ERR_ARG, "theta_update_noalloc: K must be in [1, 8] (the size of its static scratch)");
    if (T < 1) return noalloc_fail(PASC_ERR_ARG, "theta_update_noalloc: T must be >= 1");
    if (!gamma_dev || !data_dev || !theta_dev) return noalloc_fail(PASC_ERR_ARG, "theta_update_noalloc: NULL pointer");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return noalloc_fail(PASC_ERR_CUDA, "theta_update_noalloc: no usable current device");
    double *scratch = nullptr;
    if (noalloc_scratch(dev, &scratch) != cudaSuccess)
        return noalloc_fail(PASC_ERR_CUDA, "theta_update_noalloc: cudaGetSymbolAddress of the scratch array failed");
    cudaStream_t s = (cudaStream_t)stream;
    // the ticket must start at zero whatever the previous call left behind
    if (cudaMemsetAsync(scratch + NOALLOC_PARTIALS, 0, sizeof(unsigned int), s) != cudaSuccess)
        return noalloc_fail(PASC_ERR_CUDA, "theta_update_noalloc: clearing the ticket failed");
    int sms = 148;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long grid = (T + NOALLOC_THREADS - 1) / NOALLOC_THREADS;
    if (grid > (long)sms * 4) grid = (long)sms * 4;
    if (grid > NOALLOC_MAX_BLOCKS) grid = NOALLOC_MAX_BLOCKS;
    switch (K) {
#define PASC_CASE(KK)                                                                                    \
    case KK:                                                                                             \
        theta_noalloc_kernel<KK><<<(int)grid, NOALLOC_THREADS, 0, s>>>(gamma_dev, data_dev, T, theta_dev, scratch); \
        break;
        PASC_CASE(1) PASC_CASE(2) PASC_CASE(3) PASC_CASE(4)
        PASC_CASE(5) PASC_CASE(6) PASC_CASE(7) PASC_CASE(8)
#undef PASC_CASE
    }
    if (cudaGetLastError() != cudaSuccess) return noalloc_fail(PASC_ERR_CUDA, "theta_update_noalloc: launch failed");
    return PASC_OK;
}

}  // extern "C"
