// common.cuh -- shared types and helpers of the NUDIM GB300 engine.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/nudim.h"

namespace nudim {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
int cufft_fail(cufftResult r, const char *what, const char *file, int line);

#define NUDIM_CUDA(call)                                                        \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) return ::nudim::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)
#define NUDIM_CUFFT(call)                                                       \
    do {                                                                        \
        cufftResult r_ = (call);                                                \
        if (r_ != CUFFT_SUCCESS) return ::nudim::cufft_fail(r_, #call, __FILE__, __LINE__); \
    } while (0)
#define NUDIM_TRY(call)                                                         \
    do {                                                                        \
        int s_ = (call);                                                        \
        if (s_ != NUDIM_OK) return s_;                                          \
    } while (0)
// Every kernel launch of the library is followed by this check, which also
// counts the launch (nudim_launch_count).
extern unsigned long long g_launches;
#define NUDIM_LAUNCH_CHECK()                                                    \
    do {                                                                        \
        ++::nudim::g_launches;                                                  \
        NUDIM_CUDA(cudaGetLastError());                                         \
    } while (0)

// ---------------------------------------------------------------- constants
constexpr int kM = 6;            // NFFT cut-off (reconstruction.c:319, 393)
constexpr int kW = 2 * kM + 2;   // window taps per dimension
constexpr int kCgnrIters = 10;   // reconstruction.c:507, 593

// ---------------------------------------------------------------- types
template <typename T> struct Cplx;
template <> struct Cplx<double> { using type = double2; };
template <> struct Cplx<float> { using type = float2; };
template <typename T> using cplx_t = typename Cplx<T>::type;

template <typename T> __host__ __device__ inline cplx_t<T> mkc(T re, T im)
{
    cplx_t<T> c;
    c.x = re;
    c.y = im;
    return c;
}

// IEEE round-to-nearest arithmetic without contraction.  The stencils use
// these so that the FP64 form reproduces the reference's C arithmetic bit
// for bit (gcc -O3 on x86-64 emits no fused multiply-add).
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double rn_sqrt(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float rn_sqrt(float a) { return __fsqrt_rn(a); }

// Neumaier-compensated accumulator (used where the mixed form promises
// compensated sums: the adjoint gather and the R-factor).
template <typename T> struct Comp {
    T s, c;
    __device__ __forceinline__ void init() { s = T(0); c = T(0); }
    __device__ __forceinline__ void add(T v)
    {
        T t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v;
        else c += (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ T value() const { return s + c; }
};

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------- reductions
// Block-wide sum of a double (deterministic tree order).  blockDim.x must be
// a multiple of 32 and <= 1024.  Result valid in thread 0.
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_sum(double v, double *sh /* >= 32 */)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) v = warp_sum(v);
    return v;
}

// Block sum of per-thread values of type T.  FP32: the warps reduce in FP32
// and only the per-warp partials are summed in FP64 (FP64 arithmetic is
// slow on this GPU); FP64: block_sum.  Result valid in thread 0.
template <typename T> __device__ __forceinline__ double block_sum_t(T v, double *sh)
{
    if (sizeof(T) == 8) return block_sum((double)v, sh);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[wid] = (double)v;
    __syncthreads();
    int nw = (blockDim.x + 31) >> 5;
    double d = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) d = warp_sum(d);
    return d;
}

// Sum `nparts` per-block partials of each of `nplanes` planes, for each of
// `nsums` sums laid out back to back inside a plane's slot:
//   out[p*out_stride + k] = sum_i part[p*stride_in + k*nparts + i]
// One block per (plane, sum), fixed order, so the result is deterministic.
void launch_finish_sums(const double *part, int nparts, int nplanes, int stride_in,
                        double *out, int out_stride, int nsums, cudaStream_t st);

}  // namespace nudim
