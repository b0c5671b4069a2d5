// Device diagnostics: FP64 FMA throughput probe (denominator of the FP64 roofline).
#include "fem_common.cuh"

namespace fem {
namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) k_fp64_fma(double* out, double seed) {
    double a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = seed + threadIdx.x * 1e-9 + c;
    const double m = 0.999999999, b = 1e-12;
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], m, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c];
    if (s == 12345.678) out[threadIdx.x] = s;  // keeps the chains live; never true
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" int fem_diag_fp64_tflops(double* tflops, void* stream) {
    FEM_REQUIRE(tflops != nullptr, "tflops is NULL");
    cudaStream_t st = as_stream(stream);
    int dev = 0, sms = 0;
    FEM_CUDA(cudaGetDevice(&dev));
    FEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    FEM_CUDA(cudaMallocAsync(&sink, 256 * sizeof(double), st));
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    FEM_CUDA(cudaEventCreate(&e0));
    FEM_CUDA(cudaEventCreate(&e1));
    k_fp64_fma<<<blocks, 256, 0, st>>>(sink, 1.0);  // warm-up
    FEM_CUDA(cudaEventRecord(e0, st));
    k_fp64_fma<<<blocks, 256, 0, st>>>(sink, 2.0);
    FEM_CUDA(cudaEventRecord(e1, st));
    FEM_LAUNCH_CHECK("k_fp64_fma");
    FEM_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    FEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FEM_CUDA(cudaFreeAsync(sink, st));
    const double flops = 2.0 * double(blocks) * 256.0 * kIters * kChains;
    *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return FEM_OK;
}
