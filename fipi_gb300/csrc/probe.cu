// Arithmetic-pipe throughput probe: the FP64 (or FP32) fused multiply-add
// rate of the device, measured with a kernel of independent FMA chains.
// The reference has no counterpart; the benchmark divides the FP64 form's
// step FLOPs by this rate to place that form on its roofline (the FP64 pipe,
// not HBM, bounds it on GB300).
#include <cuda_runtime.h>

#include "ctx.hpp"

namespace fipi {
namespace {

constexpr int kChains = 8;     // independent FMA chains per thread
constexpr int kThreadsPB = 256;

// Every thread runs kChains chains of `iters` dependent FMAs.  The values
// stay finite (|a| converges towards c / (1 - b)); the sum is stored only
// when it equals a value it cannot take, so the compiler keeps the work.
template <typename T> __global__ void __launch_bounds__(kThreadsPB) k_fma_chains(int iters, T b, T c, T* sink) {
    T a[kChains];
#pragma unroll
    for (int j = 0; j < kChains; ++j) a[j] = T(threadIdx.x + j) * T(1e-3);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int j = 0; j < kChains; ++j) a[j] = fma(a[j], b, c);
    }
    T s = T(0);
#pragma unroll
    for (int j = 0; j < kChains; ++j) s += a[j];
    if (s == T(-12345.0)) sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> fipi_status fma_peak(int device, double* tflops) {
    int nsm = 0;
    cudaError_t e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return cuda_check(nullptr, e, "cudaDeviceGetAttribute");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fma_chains<T>, kThreadsPB, 0);
    if (e != cudaSuccess) return cuda_check(nullptr, e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (per_sm < 1) per_sm = 1;
    const int blocks = nsm * per_sm;
    T* sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    fipi_status rc = FIPI_OK;
    float ms = 0.0f;
    int iters = 1 << 10;
    const T b = T(0.9999), c = T(1e-4);
    if ((e = cudaMalloc((void**)&sink, sizeof(T) * (size_t)blocks * kThreadsPB)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        rc = cuda_check(nullptr, e, "probe set-up");
        goto done;
    }
    // grow the chain length until one launch takes at least 20 ms; the
    // last launch is the one timed (the earlier ones warm the device up)
    for (int round = 0; round < 16; ++round) {
        k_fma_chains<T><<<blocks, kThreadsPB, 0, st>>>(iters, b, c, sink);
        cudaEventRecord(e0, st);
        k_fma_chains<T><<<blocks, kThreadsPB, 0, st>>>(iters, b, c, sink);
        cudaEventRecord(e1, st);
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) {
            rc = cuda_check(nullptr, e, "probe launch");
            goto done;
        }
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms >= 20.0f || iters >= (1 << 24)) break;
        iters *= 4;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) {
        rc = cuda_check(nullptr, e, "probe launch");
        goto done;
    }
    *tflops = 2.0 * (double)blocks * kThreadsPB * kChains * (double)iters / (ms * 1e-3) / 1e12;
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    return rc;
}

}  // namespace
}  // namespace fipi

extern "C" fipi_status fipi_fma_peak(int device, int fp64, double* tflops) {
    if (!tflops) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "tflops is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
        return fipi::set_error(nullptr, FIPI_ERR_NO_DEVICE, "no CUDA device visible");
    if (device < 0 || device >= n) return fipi::set_error(nullptr, FIPI_ERR_BAD_ARG, "device out of range");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fipi::cuda_check(nullptr, e, "cudaSetDevice");
    return fp64 ? fipi::fma_peak<double>(device, tflops) : fipi::fma_peak<float>(device, tflops);
}
