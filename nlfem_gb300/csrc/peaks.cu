// Measured CUDA-core FMA throughput (nlfem_measure_peaks): the FP32 and FP64 pipe peaks used as
// roofline denominators for the quadrature kernels, which run on the CUDA cores (no GEMM-shaped
// work exists on this path, so the tensor-core peak does not bound it).
//
// Each thread runs CHAINS independent FMA recurrences a <- a * b + c for `iters` steps; enough
// warps per SM sub-partition hide the FMA latency, so the pipe issues every cycle. flops = 2 per
// FMA. The best of several launches, timed with CUDA events on one stream, is reported.
#include "../../include/nlfem_gpu.h"

#include <cuda_runtime.h>
#include <string>

__attribute__((visibility("hidden"))) int nlfem_fail_internal(int code, const char *msg);

namespace {

constexpr int CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T b, T c, T *out) {
    T a[CHAINS];
#pragma unroll
    for (int j = 0; j < CHAINS; j++) a[j] = (T)(threadIdx.x + j);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < CHAINS; j++) a[j] = fma(a[j], b, c);
    }
    T s = 0;
#pragma unroll
    for (int j = 0; j < CHAINS; j++) s += a[j];
    out[(long long)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int time_fma(int nsm, int iters, double *tflops) {
    const int blocks = nsm * 8, threads = 256;
    T *out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t st = nullptr;
    cudaError_t err = cudaMalloc(&out, sizeof(T) * (size_t)blocks * threads);
    if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 6 && err == cudaSuccess; rep++) {
        err = cudaEventRecord(e0, st);
        // b slightly below 1 and c small keep the recurrences finite for any iteration count
        k_fma_peak<T><<<blocks, threads, 0, st>>>(iters, (T)0.999999, (T)1e-3, out);
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaEventRecord(e1, st);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float ms = 0;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
        if (err == cudaSuccess && rep > 0 && ms < best) best = ms;   // launch 0 warms up
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (out) cudaFree(out);
    if (err != cudaSuccess) return nlfem_fail_internal(NLFEM_ERR_CUDA, cudaGetErrorString(err));
    const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return NLFEM_OK;
}

}  // namespace

extern "C" int nlfem_measure_peaks(double *fp32_tflops, double *fp64_tflops) {
    if (!fp32_tflops || !fp64_tflops) return nlfem_fail_internal(NLFEM_ERR_INVALID, "null argument");
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) {
        cudaGetLastError();
        return nlfem_fail_internal(NLFEM_ERR_CUDA, "no CUDA device available (the library has no CPU path)");
    }
    int r = time_fma<float>(nsm, 8192, fp32_tflops);
    if (!r) r = time_fma<double>(nsm, 256, fp64_tflops);
    return r;
}
