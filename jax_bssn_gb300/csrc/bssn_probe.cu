// FMA-throughput probe: the FP64 and FP32 peaks that the roofline of the
// RHS kernels is measured against (GB300's FP64 rate is a small fraction of
// its FP32 rate, and neither is in the measured copy/GEMM peaks).
//
// Each thread runs sixteen independent FMA chains (enough to cover the FMA
// latency; the iteration loop is unrolled so loop overhead stays small),
// eight blocks of 256 threads per SM; the time of the whole launch
// (CUDA events, after one warm-up launch) gives FMAs per second, counted as
// two flops each.
#include <cuda_runtime.h>

#include "../../include/bssn_gb300.h"
#include "bssn_driver.h"
#include "bssn_fields.cuh"

namespace bssn {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 16;

template <typename T>
__global__ void __launch_bounds__(kProbeThreads) k_fma_probe(T* __restrict__ sink, int iters, T a, T b) {
    T x[kProbeChains];
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) x[j] = static_cast<T>(threadIdx.x + j) * static_cast<T>(1e-3);
#pragma unroll 4
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < kProbeChains; ++j) x[j] = fma(x[j], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int j = 0; j < kProbeChains; ++j) s += x[j];
    if (s == static_cast<T>(-1.25)) sink[0] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
int probe(double* gflops, int iters) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_status(e, "bssn_probe_fma_peak");
    T* sink = nullptr;
    e = cudaMalloc(&sink, sizeof(T));
    if (e != cudaSuccess) return cuda_status(e, "bssn_probe_fma_peak");
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    const int blocks = 8 * sms;
    // a, b close to a fixed point of x -> a x + b so values stay finite
    const T a = static_cast<T>(0.999), b = static_cast<T>(1e-3);
    k_fma_probe<T><<<blocks, kProbeThreads>>>(sink, iters / 8, a, b);
    cudaEventRecord(t0);
    k_fma_probe<T><<<blocks, kProbeThreads>>>(sink, iters, a, b);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_status(e, "bssn_probe_fma_peak");
    const double fmas = (double)blocks * kProbeThreads * kProbeChains * (double)iters;
    *gflops = 2.0 * fmas / (ms * 1e-3) / 1e9;
    return BSSN_OK;
}

__global__ void k_check_div6(const double* __restrict__ a, double* __restrict__ fast, double* __restrict__ hw,
                             long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fast[i] = div6_rn(a[i]);
    hw[i] = __ddiv_rn(a[i], 6.0);
}

}  // namespace
}  // namespace bssn

extern "C" int bssn_probe_fma_peak(int32_t precision, double* gflops) {
    if (!gflops) return bssn::fail(BSSN_ERR_INVALID, "gflops is null");
    if (precision == BSSN_PRECISION_F64) return bssn::probe<double>(gflops, 4096);
    if (precision == BSSN_PRECISION_F32) return bssn::probe<float>(gflops, 65536);
    return bssn::fail(BSSN_ERR_INVALID, "precision must be BSSN_PRECISION_F64 or BSSN_PRECISION_F32");
}

extern "C" int bssn_check_div6(const double* a, double* fast, double* hw, int64_t n, void* stream) {
    if (n < 0 || (n > 0 && (!a || !fast || !hw))) return bssn::fail(BSSN_ERR_INVALID, "bssn_check_div6: bad arguments");
    if (n == 0) return BSSN_OK;
    const long long blocks = (n + 255) / 256;
    bssn::k_check_div6<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(a, fast, hw, n);
    return bssn::cuda_status(cudaGetLastError(), "bssn_check_div6");
}
