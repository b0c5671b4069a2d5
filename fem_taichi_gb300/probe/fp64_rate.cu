// Arithmetic-rate probes for the benchmark's rooflines, built as their own small library
// (libfemprobe.so) so that the product library carries no measurement code.
//
// fem_probe_fma_tflops(fp64, &tflops, stream): FMA throughput of this device in TFLOP/s (an
// FMA counts 2 flops) on the FP64 pipe (fp64 = 1) or the FP32 pipe (fp64 = 0): the best rate
// of a kernel of independent FMA chains (8 per thread, 256 threads per CTA) over 1, 2, 4 and 8
// CTAs per SM (the FP64 pipe reaches its highest rate below full occupancy), each launch timed
// with CUDA events on `stream` after a warm-up launch.  Returns 0 or the CUDA error code.
#include <cuda_runtime.h>

#include <algorithm>

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;

// The multiplier and addend are computed from the thread index so that they sit in registers:
// with two compile-time constant operands the FP64 chains ran 16 % slower (1.007 against 1.196
// TFLOP/s on a GB300), which would understate the pipe's rate.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_chains(T* out, T seed) {
    T a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) a[c] = seed + T(threadIdx.x) * T(1e-6) + T(c);
    const T m = T(0.9999999) + T(threadIdx.x) * T(1e-12), b = T(1e-7) + T(threadIdx.x) * T(1e-15);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int c = 0; c < kChains; ++c) a[c] = fma(a[c], m, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += a[c];
    if (s == T(12345.678)) out[threadIdx.x] = s;  // keeps the chains live; never true
}

template <typename T>
int run(double* tflops, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return int(e);
    T* sink = nullptr;
    if ((e = cudaMallocAsync(&sink, 256 * sizeof(T), st)) != cudaSuccess) return int(e);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double best = 0.0;
    do {
        if ((e = cudaEventCreate(&e0)) != cudaSuccess) break;
        if ((e = cudaEventCreate(&e1)) != cudaSuccess) break;
        for (int per_sm = 1; per_sm <= 8 && e == cudaSuccess; per_sm *= 2) {
            const int blocks = sms * per_sm;
            float ms = 0;
            k_fma_chains<T><<<blocks, 256, 0, st>>>(sink, T(1));   // warm-up
            if ((e = cudaEventRecord(e0, st)) != cudaSuccess) break;
            k_fma_chains<T><<<blocks, 256, 0, st>>>(sink, T(2));
            if ((e = cudaGetLastError()) != cudaSuccess) break;
            if ((e = cudaEventRecord(e1, st)) != cudaSuccess) break;
            if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
            if ((e = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
            const double flops = 2.0 * double(blocks) * 256.0 * kIters * kChains;
            best = std::max(best, flops / (double(ms) * 1e-3) / 1e12);
        }
    } while (0);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFreeAsync(sink, st);
    cudaStreamSynchronize(st);
    if (e != cudaSuccess) return int(e);
    *tflops = best;
    return 0;
}

}  // namespace

extern "C" int fem_probe_fma_tflops(int fp64, double* tflops, void* stream) {
    if (!tflops) return int(cudaErrorInvalidValue);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return fp64 ? run<double>(tflops, st) : run<float>(tflops, st);
}
