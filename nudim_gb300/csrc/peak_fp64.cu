// peak_fp64.cu -- arithmetic-peak probe of the GPU the FP64 form runs on.
//
// The FP64 form of the reconstruction loop is bound by the FP64 FMA pipe,
// whose rate on GB300 is a small fraction of the FP32 rate and is not listed
// with the measured copy bandwidth.  This program measures it (and the FP32
// FMA rate beside it) with a kernel of independent FMA chains: every thread
// runs kChains chains of `iters` dependent fused multiply-adds, enough
// independent work per warp to keep the pipe busy; the grid is a multiple of
// the SM count.  Timed with CUDA events after one untimed launch; prints one
// JSON line {"fp64_tflops": ..., "fp32_tflops": ..., "sm_count": ...}.
//
//   fp64_peak [iters]
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

template <typename T> __global__ void __launch_bounds__(kThreads) k_fma_chains(T *out, int iters, T b, T c)
{
    T a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; i++) a[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int k = 0; k < iters; k++) {
#pragma unroll
        for (int i = 0; i < kChains; i++) a[i] = fma(a[i], b, c);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < kChains; i++) s += a[i];
    // one store per thread keeps the chains live
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T> double measure(int blocks, int iters)
{
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * (size_t)blocks * kThreads) != cudaSuccess) return -1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const T b = (T)0.999999, c = (T)1e-7;
    k_fma_chains<T><<<blocks, kThreads>>>(out, iters, b, c);
    cudaEventRecord(e0);
    k_fma_chains<T><<<blocks, kThreads>>>(out, iters, b, c);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0) return -1;
    double flops = 2.0 * kChains * (double)iters * blocks * kThreads;
    return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

int main(int argc, char **argv)
{
    int iters = argc > 1 ? atoi(argv[1]) : 4096;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, 0) != cudaSuccess) {
        fprintf(stderr, "no CUDA device\n");
        return 1;
    }
    int blocks = p.multiProcessorCount * 8;
    double d = measure<double>(blocks, iters);
    double f = measure<float>(blocks, iters * 16);
    if (d <= 0 || f <= 0) {
        fprintf(stderr, "measurement failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        return 1;
    }
    printf("{\"fp64_tflops\": %.4f, \"fp32_tflops\": %.3f, \"sm_count\": %d, \"iters\": %d, "
           "\"blocks\": %d, \"threads\": %d, \"chains\": %d}\n",
           d, f, p.multiProcessorCount, iters, blocks, kThreads, kChains);
    return 0;
}
