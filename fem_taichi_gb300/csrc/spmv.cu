// BSR SpMV / SpMM entry points, precision conversion, block-Jacobi inverse and the SpMV
// launch autotuner.  The kernels are the residual product of SOLVE_static.py:36 (K * U)
// generalised to FP32 and to many right-hand sides.
#include <algorithm>
#include <mutex>
#include <vector>

#include "spmv.cuh"

namespace fem {

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return n;
}

int resident_ctas(const void* kernel, int threads, size_t smem) {
    struct Entry {
        const void* kernel;
        int threads;
        size_t smem;
        int dev;
        int ctas;
    };
    static std::mutex mu;
    static std::vector<Entry> cache;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    {
        std::lock_guard<std::mutex> lock(mu);
        for (const Entry& e : cache)
            if (e.kernel == kernel && e.threads == threads && e.smem == smem && e.dev == dev) return e.ctas;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    std::lock_guard<std::mutex> lock(mu);
    cache.push_back({kernel, threads, smem, dev, n});
    return n;
}

unsigned resident_grid(const void* kernel, int threads, int64_t need, int64_t cap) {
    const int64_t wave = int64_t(sm_count()) * resident_ctas(kernel, threads, 0);
    return unsigned(std::max<int64_t>(1, std::min<int64_t>({need, wave, cap})));
}

namespace {

template <typename T, int LPR>
__global__ void __launch_bounds__(512) k_spmv(const BsrView<T> A, const T* __restrict__ x, T* __restrict__ y) {
    spmv1_rows<T, LPR>(A, x, y, false);
}

template <typename T, int R>
__global__ void __launch_bounds__(256) k_spmm(const BsrView<T> A, const T* __restrict__ x, T* __restrict__ y) {
    spmm_rows<T, R>(A, x, y, false);
}

// BSR [nnzb][9] FP64 -> row-SoA FP32: value q of slot l of row i at 9*rs + q*L + l
__global__ void __launch_bounds__(256) k_bsr_to_rsoa_f32(int64_t n, const int32_t* __restrict__ indptr,
                                                         const double* __restrict__ src, float* __restrict__ dst) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp0; i < n; i += nw) {
        const int64_t rs = indptr[i];
        const int L = indptr[i + 1] - int(rs);
        for (int o = lane; o < 9 * L; o += 32) {
            const int q = o / L, l = o - q * L;
            dst[9 * rs + o] = float(src[9 * (rs + l) + q]);
        }
    }
}

// BSR [nnzb][9] FP64 -> padded row-SoA FP32 (rows rounded up to 4 blocks; padding: column
// = the row itself, values 0)
__global__ void __launch_bounds__(256) k_bsr_to_rsoa4_f32(int64_t n, const int32_t* __restrict__ indptr,
                                                          const int32_t* __restrict__ indices,
                                                          const double* __restrict__ src,
                                                          const int32_t* __restrict__ indptr4, int32_t* indices4,
                                                          float* __restrict__ dst) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp0; i < n; i += nw) {
        const int64_t rs = indptr[i], rs4 = indptr4[i];
        const int L = indptr[i + 1] - int(rs), Lp = indptr4[i + 1] - int(rs4);
        for (int l = lane; l < Lp; l += 32) indices4[rs4 + l] = l < L ? indices[rs + l] : int32_t(i);
        for (int o = lane; o < 9 * Lp; o += 32) {
            const int q = o / Lp, l = o - q * Lp;
            dst[9 * rs4 + o] = l < L ? float(src[9 * (rs + l) + q]) : 0.f;
        }
    }
}

__global__ void k_f64_to_f32(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        dst[i] = float(src[i]);
}

// Inverse of each block row's diagonal block (adjugate / det, FP64).  Rows whose diagonal
// block is missing or singular get the identity and are counted in *bad.
__global__ void k_block_jacobi(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                               const double* __restrict__ vals, double* inv64, float* inv32, int* bad) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t rs = indptr[i], re = indptr[i + 1];
        int64_t s = -1;
        for (int64_t k = rs; k < re; ++k)
            if (indices[k] == int(i)) {
                s = k;
                break;
            }
        double o[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (s >= 0) {
            const double* a = vals + 9 * s;
            double c[9];
            c[0] = a[4] * a[8] - a[5] * a[7];
            c[1] = a[2] * a[7] - a[1] * a[8];
            c[2] = a[1] * a[5] - a[2] * a[4];
            c[3] = a[5] * a[6] - a[3] * a[8];
            c[4] = a[0] * a[8] - a[2] * a[6];
            c[5] = a[2] * a[3] - a[0] * a[5];
            c[6] = a[3] * a[7] - a[4] * a[6];
            c[7] = a[1] * a[6] - a[0] * a[7];
            c[8] = a[0] * a[4] - a[1] * a[3];
            const double det = a[0] * c[0] + a[1] * c[3] + a[2] * c[6];
            if (det != 0.0 && isfinite(det)) {
                const double id = 1.0 / det;
#pragma unroll
                for (int k = 0; k < 9; ++k) o[k] = c[k] * id;
            } else {
                atomicAdd(bad, 1);
            }
        } else {
            atomicAdd(bad, 1);
        }
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            if (inv64) inv64[9 * i + k] = o[k];
            if (inv32) inv32[9 * i + k] = float(o[k]);
        }
    }
}

template <typename T>
int launch_spmv(const BsrView<T>& A, int nrhs, const T* x, T* y, int variant, cudaStream_t st) {
    // Grid-stride kernels: one wave of resident CTAs (a grid larger than what fits leaves a
    // second, partial wave with too few warps to keep the pipes busy)
    const int sms = sm_count();
    auto run = [&](auto kernel, int threads, int64_t rows_per_cta, int64_t cap) {
        const unsigned grid = resident_grid(reinterpret_cast<const void*>(kernel), threads,
                                            (A.n + rows_per_cta - 1) / rows_per_cta, cap);
        kernel<<<grid, threads, 0, st>>>(A, x, y);
    };
    if (nrhs == 1) {
        const SpmvVariant v = spmv_variant(variant);
        const int64_t rows_per_cta = int64_t(v.threads / 32) * (32 / v.lpr);
        const int64_t cap = int64_t(sms) * v.ctas_per_sm;
        switch (v.lpr) {
            case 32: run(k_spmv<T, 32>, v.threads, rows_per_cta, cap); break;
            case 16: run(k_spmv<T, 16>, v.threads, rows_per_cta, cap); break;
            case 8: run(k_spmv<T, 8>, v.threads, rows_per_cta, cap); break;
            case 4: run(k_spmv<T, 4>, v.threads, rows_per_cta, cap); break;
            default: run(k_spmv<T, 2>, v.threads, rows_per_cta, cap); break;
        }
    } else {
        const int64_t rows_per_cta = 8 * (32 / nrhs);
        const int64_t cap = int64_t(sms) * 8;
        switch (nrhs) {
            case 2: run(k_spmm<T, 2>, 256, rows_per_cta, cap); break;
            case 4: run(k_spmm<T, 4>, 256, rows_per_cta, cap); break;
            case 8: run(k_spmm<T, 8>, 256, rows_per_cta, cap); break;
            case 16: run(k_spmm<T, 16>, 256, rows_per_cta, cap); break;
            default: run(k_spmm<T, 32>, 256, rows_per_cta, cap); break;
        }
    }
    FEM_LAUNCH_CHECK("bsr spmv");
    return FEM_OK;
}

int check_bsr(const fem_bsr* A) {
    FEM_REQUIRE(A != nullptr, "A is NULL");
    FEM_REQUIRE(A->n_brow >= 0 && A->nnzb >= 0, "negative size");
    FEM_REQUIRE(A->dtype == FEM_F64 || A->dtype == FEM_F32, "dtype must be FEM_F64 or FEM_F32");
    FEM_REQUIRE(A->layout == FEM_LAYOUT_BSR || A->layout == FEM_LAYOUT_RSOA || A->layout == FEM_LAYOUT_RSOA4,
                "layout must be BSR, RSOA or RSOA4");
    FEM_REQUIRE(A->layout != FEM_LAYOUT_RSOA4 || A->dtype == FEM_F32, "FEM_LAYOUT_RSOA4 is FP32 only");
    FEM_REQUIRE(A->layout != FEM_LAYOUT_RSOA4 || ((reinterpret_cast<uintptr_t>(A->vals) |
                                                   reinterpret_cast<uintptr_t>(A->indices)) & 15u) == 0,
                "FEM_LAYOUT_RSOA4 arrays must be 16-byte aligned");
    if (A->n_brow) FEM_REQUIRE(A->indptr != nullptr, "indptr is NULL");
    if (A->nnzb) FEM_REQUIRE(A->indices && A->vals, "indices/vals is NULL");
    return FEM_OK;
}

bool valid_nrhs(int r) { return r == 1 || r == 2 || r == 4 || r == 8 || r == 16 || r == 32; }

}  // namespace

int bsr_spmv_any(const fem_bsr* A, int nrhs, const void* x, void* y, int variant, cudaStream_t st) {
    if (A->n_brow == 0) return FEM_OK;
    if (A->dtype == FEM_F64) {
        BsrView<double> v{A->n_brow, A->indptr, A->indices, static_cast<const double*>(A->vals),
                          rsoa_kind(A->layout)};
        return launch_spmv<double>(v, nrhs, static_cast<const double*>(x), static_cast<double*>(y), variant, st);
    }
    BsrView<float> v{A->n_brow, A->indptr, A->indices, static_cast<const float*>(A->vals),
                     rsoa_kind(A->layout)};
    return launch_spmv<float>(v, nrhs, static_cast<const float*>(x), static_cast<float*>(y), variant, st);
}

}  // namespace fem

using namespace fem;

extern "C" int fem_bsr_spmv(const fem_bsr* A, int nrhs, const void* x, void* y, int variant, void* stream) {
    int rc = check_bsr(A);
    if (rc) return rc;
    FEM_REQUIRE(valid_nrhs(nrhs), "nrhs must be 1, 2, 4, 8, 16 or 32");
    FEM_REQUIRE(A->n_brow == 0 || (x && y), "x/y is NULL");
    FEM_REQUIRE(x != y || A->n_brow == 0, "x and y must not alias");
    return bsr_spmv_any(A, nrhs, x, y, variant, as_stream(stream));
}

extern "C" int fem_convert_f64_to_f32(const double* src, float* dst, int64_t n, void* stream) {
    FEM_REQUIRE(n >= 0, "negative size");
    if (n == 0) return FEM_OK;
    FEM_REQUIRE(src && dst, "src/dst is NULL");
    const unsigned grid = unsigned(std::min<int64_t>((n + 255) / 256, int64_t(sm_count()) * 16));
    k_f64_to_f32<<<grid, 256, 0, as_stream(stream)>>>(src, dst, n);
    FEM_LAUNCH_CHECK("k_f64_to_f32");
    return FEM_OK;
}

extern "C" int fem_block_jacobi(const fem_bsr* A, double* inv64, float* inv32, int* n_bad, void* stream) {
    int rc = check_bsr(A);
    if (rc) return rc;
    FEM_REQUIRE(A->dtype == FEM_F64, "block Jacobi needs the FP64 matrix");
    FEM_REQUIRE(n_bad != nullptr, "n_bad is NULL");
    if (A->n_brow == 0) return FEM_OK;
    cudaStream_t st = as_stream(stream);
    FEM_CUDA(cudaMemsetAsync(n_bad, 0, sizeof(int), st));
    const unsigned grid = unsigned(std::min<int64_t>((A->n_brow + 255) / 256, int64_t(sm_count()) * 16));
    k_block_jacobi<<<grid, 256, 0, st>>>(A->n_brow, A->indptr, A->indices, static_cast<const double*>(A->vals),
                                         inv64, inv32, n_bad);
    FEM_LAUNCH_CHECK("k_block_jacobi");
    return FEM_OK;
}

extern "C" int fem_spmv_autotune(const fem_bsr* A, int nrhs, const void* x, void* y, int reps, int* best_variant,
                                 float* best_ms, void* stream) {
    int rc = check_bsr(A);
    if (rc) return rc;
    FEM_REQUIRE(valid_nrhs(nrhs) && best_variant, "bad nrhs or best_variant is NULL");
    FEM_REQUIRE(A->n_brow == 0 || (x && y && x != y), "x/y is NULL or aliased");
    *best_variant = 0;
    if (best_ms) *best_ms = 0.f;
    if (nrhs != 1 || A->n_brow == 0) return FEM_OK;  // SpMM has a single launch shape
    cudaStream_t st = as_stream(stream);
    cudaEvent_t e0, e1;
    FEM_CUDA(cudaEventCreate(&e0));
    FEM_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int bid = 0;
    reps = std::max(1, std::min(reps, 100));
    for (int v = 0; v < kNumSpmvVariants; ++v) {
        rc = bsr_spmv_any(A, 1, x, y, v, st);  // warm-up
        if (rc) break;
        FEM_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < reps && rc == FEM_OK; ++r) rc = bsr_spmv_any(A, 1, x, y, v, st);
        FEM_CUDA(cudaEventRecord(e1, st));
        FEM_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        FEM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= reps;
        if (ms < best) best = ms, bid = v;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *best_variant = bid;
    if (best_ms) *best_ms = best;
    return FEM_OK;
}

extern "C" int fem_bsr_to_rsoa_f32(const fem_bsr* A, float* dst, void* stream) {
    int rc = check_bsr(A);
    if (rc) return rc;
    FEM_REQUIRE(A->dtype == FEM_F64 && A->layout == FEM_LAYOUT_BSR, "source must be an FP64 BSR matrix");
    FEM_REQUIRE(A->n_brow == 0 || dst, "dst is NULL");
    if (A->n_brow == 0) return FEM_OK;
    const unsigned grid = unsigned(std::min<int64_t>((A->n_brow + 7) / 8, int64_t(sm_count()) * 16));
    k_bsr_to_rsoa_f32<<<grid, 256, 0, as_stream(stream)>>>(A->n_brow, A->indptr, static_cast<const double*>(A->vals),
                                                           dst);
    FEM_LAUNCH_CHECK("k_bsr_to_rsoa_f32");
    return FEM_OK;
}

extern "C" int fem_rsoa4_indptr(int64_t n_brow, const int32_t* indptr, int32_t* indptr4) {
    FEM_REQUIRE(n_brow >= 0, "negative size");
    FEM_REQUIRE(indptr && indptr4, "indptr/indptr4 is NULL");
    int64_t acc = 0;
    indptr4[0] = 0;
    for (int64_t i = 0; i < n_brow; ++i) {
        const int64_t L = int64_t(indptr[i + 1]) - indptr[i];
        FEM_REQUIRE(L >= 0, "indptr is not monotone");
        acc += (L + 3) / 4 * 4;
        FEM_REQUIRE(acc < (int64_t(1) << 31), "padded block count exceeds int32 range");
        indptr4[i + 1] = int32_t(acc);
    }
    return FEM_OK;
}

extern "C" int fem_bsr_to_rsoa4_f32(const fem_bsr* A, const int32_t* indptr4, int32_t* indices4, float* vals4,
                                    void* stream) {
    int rc = check_bsr(A);
    if (rc) return rc;
    FEM_REQUIRE(A->dtype == FEM_F64 && A->layout == FEM_LAYOUT_BSR, "source must be an FP64 BSR matrix");
    if (A->n_brow == 0) return FEM_OK;
    FEM_REQUIRE(indptr4 && indices4 && vals4, "indptr4/indices4/vals4 is NULL");
    const unsigned grid = unsigned(std::min<int64_t>((A->n_brow + 7) / 8, int64_t(sm_count()) * 16));
    k_bsr_to_rsoa4_f32<<<grid, 256, 0, as_stream(stream)>>>(A->n_brow, A->indptr, A->indices,
                                                            static_cast<const double*>(A->vals), indptr4, indices4,
                                                            vals4);
    FEM_LAUNCH_CHECK("k_bsr_to_rsoa4_f32");
    return FEM_OK;
}
