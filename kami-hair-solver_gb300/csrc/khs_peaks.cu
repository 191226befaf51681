// FMA-pipe throughput probe used for the FP64 roofline of the solver's
// kernels: every thread runs eight independent FMA chains, so the pipe, not
// latency, bounds the kernel.  Two flops per FMA.
#include "khs_engine.hpp"

#include <cuda_runtime.h>

namespace khs {
namespace {

template<typename T> __global__ void k_fma_probe(T *out, int iters, T a, T b)
{
    T x0 = T(threadIdx.x) * T(1e-3), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
    T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template<typename T> bool probe(int sms, int iters, double &tflops)
{
    const int blocks = sms * 4, threads = 256;
    T *out = nullptr;
    if (cudaMalloc(reinterpret_cast<void **>(&out), sizeof(T) * blocks * threads) != cudaSuccess) return false;
    cudaEvent_t s, e;
    cudaEventCreate(&s);
    cudaEventCreate(&e);
    k_fma_probe<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(s);
    k_fma_probe<T><<<blocks, threads>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e);
    cudaEventSynchronize(e);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, s, e);
    cudaEventDestroy(s);
    cudaEventDestroy(e);
    cudaFree(out);
    tflops = 2.0 * 8.0 * double(iters) * blocks * threads / (double(ms) * 1e-3) / 1e12;
    return cudaGetLastError() == cudaSuccess;
}

}  // namespace

bool measure_pipe_peaks(double &fp64_tflops, double &fp32_tflops, std::string &error)
{
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, 0) != cudaSuccess) { error = "no CUDA device"; return false; }
    if (!probe<double>(prop.multiProcessorCount, 4096, fp64_tflops) ||
        !probe<float>(prop.multiProcessorCount, 65536, fp32_tflops)) {
        error = "pipe probe failed";
        return false;
    }
    return true;
}

}  // namespace khs
