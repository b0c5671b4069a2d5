// Tall-skinny FP64 products of the block-Lanczos modal solve (SOLVE_eigen.py:65-84):
// the reorthogonalisation w -= Q (Q^T M w) and the Ritz vectors X = Q V, with Q an n x m
// block of Lanczos vectors (n ~ 10^5..10^7 rows, m <= a few hundred columns) and w, M w
// n x b blocks (b <= 32).  No reference counterpart on the GPU (the reference runs these as
// numpy GEMMs on the host).
//
//  k_ts_tn_partial / k_ts_tn_reduce: C (m x b) = Q^T X, m <= 256.  Persistent CTAs step over
//    chunks of kChunk rows (a fixed assignment for a given n); a CTA stages the chunk's X rows
//    in shared memory and thread j accumulates column j of Q (coalesced loads along a row of
//    Q) against all b columns of X; the per-CTA partials are summed in CTA order by the
//    reduce kernel (deterministic).
//  k_ts_nn: W = beta W + alpha Q C (C m x b staged in shared memory): one warp per row, lanes
//    over the columns of Q's row (coalesced), per-lane partial sums for every output column,
//    then a butterfly over the warp.
// FP64 throughout and bound by the FP64 pipe, so the column count of X / W is a template
// width close to b (4, 8, 10, 12, 16, 24, 32) rather than a power of two: padded columns
// would be FMAs on zeros.
#include <algorithm>

#include "fem_common.cuh"

namespace fem {
namespace {

constexpr int kChunk = 128;    // rows per step of the transposed product
constexpr int kTsThreads = 256;
constexpr int kMaxCols = 256;  // columns of Q per launch (one per thread)

template <int B>
__global__ void __launch_bounds__(kTsThreads) k_ts_tn_partial(int64_t n, int m, int b, const double* __restrict__ Q,
                                                                int64_t ldq, const double* __restrict__ X, int64_t ldx,
                                                                double* part) {
    __shared__ double xs[kChunk][B];
    const int j = threadIdx.x;  // column of Q (m <= kMaxCols)
    double acc[B];
#pragma unroll
    for (int c = 0; c < B; ++c) acc[c] = 0.0;
    for (int64_t r0 = int64_t(blockIdx.x) * kChunk; r0 < n; r0 += int64_t(gridDim.x) * kChunk) {
        const int rows = int(std::min<int64_t>(kChunk, n - r0));
        __syncthreads();
        for (int i = threadIdx.x; i < kChunk * B; i += kTsThreads) {
            const int r = i / B, c = i % B;
            xs[r][c] = (r < rows && c < b) ? X[(r0 + r) * ldx + c] : 0.0;
        }
        __syncthreads();
        if (j < m) {
            const double* q = Q + r0 * ldq + j;
            for (int r = 0; r < rows; ++r) {
                const double qv = __ldg(q + int64_t(r) * ldq);
#pragma unroll
                for (int c = 0; c < B; ++c) acc[c] = fma(qv, xs[r][c], acc[c]);
            }
        }
    }
    if (j < m) {
        double* o = part + (int64_t(blockIdx.x) * m + j) * B;
#pragma unroll
        for (int c = 0; c < B; ++c) o[c] = acc[c];
    }
}

// C[j][c] = sum over CTAs (in order) of the partials
template <int B>
__global__ void k_ts_tn_reduce(int m, int b, int nblocks, const double* __restrict__ part, double* C, int64_t ldc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m * b) return;
    const int j = i / b, c = i % b;
    double s = 0.0;
    for (int k = 0; k < nblocks; ++k) s += part[(int64_t(k) * m + j) * B + c];
    C[int64_t(j) * ldc + c] = s;
}

template <int B>
__global__ void __launch_bounds__(kTsThreads) k_ts_nn(int64_t n, int m, int b, const double* __restrict__ Q,
                                                        int64_t ldq, const double* __restrict__ C, int64_t ldc,
                                                        double alpha, double beta, double* W, int64_t ldw) {
    extern __shared__ double cs[];  // [m][B]
    for (int i = threadIdx.x; i < m * B; i += kTsThreads) {
        const int j = i / B, c = i % B;
        cs[i] = c < b ? C[int64_t(j) * ldc + c] : 0.0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * kTsThreads + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * kTsThreads) >> 5;
    for (int64_t r = warp; r < n; r += nwarps) {
        double acc[B];
#pragma unroll
        for (int c = 0; c < B; ++c) acc[c] = 0.0;
        const double* q = Q + r * ldq;
        for (int j = lane; j < m; j += 32) {
            const double qv = __ldg(q + j);
#pragma unroll
            for (int c = 0; c < B; ++c) acc[c] = fma(qv, cs[j * B + c], acc[c]);
        }
#pragma unroll
        for (int c = 0; c < B; ++c) {
            double v = acc[c];
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
            acc[c] = v;
        }
        if (lane < b) {
            double v = acc[0];
#pragma unroll
            for (int c = 1; c < B; ++c)
                if (lane == c) v = acc[c];
            double* w = W + r * ldw + lane;
            *w = beta == 0.0 ? alpha * v : fma(alpha, v, beta * *w);
        }
    }
}

int tn_grid(int64_t n) {
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return int(std::max<int64_t>(1, std::min<int64_t>((n + kChunk - 1) / kChunk, int64_t(sms) * 4)));
}

template <int B>
int ts_tn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* X, int64_t ldx, double* C,
          int64_t ldc, double* ws, cudaStream_t st) {
    const int blocks = tn_grid(n);
    k_ts_tn_partial<B><<<unsigned(blocks), kTsThreads, 0, st>>>(n, m, b, Q, ldq, X, ldx, ws);
    FEM_LAUNCH_CHECK("k_ts_tn_partial");
    k_ts_tn_reduce<B><<<(m * b + 255) / 256, 256, 0, st>>>(m, b, blocks, ws, C, ldc);
    FEM_LAUNCH_CHECK("k_ts_tn_reduce");
    return FEM_OK;
}

template <int B>
int ts_nn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* C, int64_t ldc, double alpha,
          double beta, double* W, int64_t ldw, cudaStream_t st) {
    const size_t smem = size_t(m) * B * sizeof(double);
    FEM_CUDA(cudaFuncSetAttribute(k_ts_nn<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    int dev = 0, sms = 0;
    FEM_CUDA(cudaGetDevice(&dev));
    FEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t need = (n * 32 + kTsThreads - 1) / kTsThreads;
    const unsigned grid = unsigned(std::max<int64_t>(1, std::min<int64_t>(need, int64_t(sms) * 8)));
    k_ts_nn<B><<<grid, kTsThreads, smem, st>>>(n, m, b, Q, ldq, C, ldc, alpha, beta, W, ldw);
    FEM_LAUNCH_CHECK("k_ts_nn");
    return FEM_OK;
}

int width(int b) { return b <= 4 ? 4 : b <= 8 ? 8 : b <= 10 ? 10 : b <= 12 ? 12 : b <= 16 ? 16 : b <= 24 ? 24 : 32; }

#define FEM_TS_DISPATCH(b, CALL)  \
    switch (width(b)) {           \
        case 4: return CALL(4);   \
        case 8: return CALL(8);   \
        case 10: return CALL(10); \
        case 12: return CALL(12); \
        case 16: return CALL(16); \
        case 24: return CALL(24); \
        default: return CALL(32); \
    }

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" size_t fem_ts_gemm_tn_workspace_bytes(int64_t n, int m, int b) {
    if (n <= 0 || m <= 0 || m > kMaxCols || b <= 0 || b > 32) return 0;
    return size_t(tn_grid(n)) * size_t(m) * width(b) * sizeof(double);
}

extern "C" int fem_ts_gemm_tn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* X, int64_t ldx,
                              double* C, int64_t ldc, void* workspace, size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(n > 0 && m > 0 && m <= kMaxCols && b > 0 && b <= 32 && Q && X && C && workspace, "bad arguments");
    FEM_REQUIRE(ldq >= m && ldx >= b && ldc >= b, "leading dimensions too small");
    if (workspace_bytes < fem_ts_gemm_tn_workspace_bytes(n, m, b)) {
        set_error("workspace too small: need %zu bytes", fem_ts_gemm_tn_workspace_bytes(n, m, b));
        return FEM_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    double* ws = static_cast<double*>(workspace);
#define FEM_TS_TN(B) ts_tn<B>(n, m, b, Q, ldq, X, ldx, C, ldc, ws, st)
    FEM_TS_DISPATCH(b, FEM_TS_TN)
#undef FEM_TS_TN
}

extern "C" int fem_ts_gemm_nn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* C, int64_t ldc,
                              double alpha, double beta, double* W, int64_t ldw, void* stream) {
    FEM_REQUIRE(n > 0 && m > 0 && m <= kMaxCols && b > 0 && b <= 32 && Q && C && W, "bad arguments");
    FEM_REQUIRE(ldq >= m && ldc >= b && ldw >= b, "leading dimensions too small");
    cudaStream_t st = as_stream(stream);
#define FEM_TS_NN(B) ts_nn<B>(n, m, b, Q, ldq, C, ldc, alpha, beta, W, ldw, st)
    FEM_TS_DISPATCH(b, FEM_TS_NN)
#undef FEM_TS_NN
}
