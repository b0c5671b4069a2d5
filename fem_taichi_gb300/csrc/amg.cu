// Smoothed-aggregation AMG on the device: FP32 copies of the hierarchy (fem_amg_upload),
// the V-cycle used as the preconditioner of the FP32 inner CG (pcg.cu), and the C entry
// points that touch device memory.  No reference counterpart (the reference factorises K
// directly, SOLVE_static.py:31-33).
//
// V-cycle on level l with right-hand side b (x starts at 0):
//   pre-smoothing: Chebyshev polynomial in D^-1 A of degree `pre` (the first step needs no
//     product: x = c D^-1 b);
//   residual r = b - A x, restriction b_c = R r, coarse cycle (dense inverse on the last
//     level), prolongation x += P x_c;
//   post-smoothing: `post` Chebyshev steps restarted from x.
// Pre- and post-smoother are the same polynomial in D^-1 A, which is self-adjoint in the A
// inner product, so the cycle is a symmetric operator and CG can use it.  Unaggregated
// (Dirichlet, in practice penalised) nodes keep x_i = D_i^-1 b_i through the whole cycle and
// contribute a zero residual, so nothing couples them to their neighbours.  Every Chebyshev
// step is one block-row product whose epilogue forms r = b - A x, z = D^-1 r,
// d = c1 d + c2 z and x' = x + d for its row (two iterate buffers, swapped per step).
// Level 0 runs on the solver's FP32 matrix with the tuned block-row products of spmv.cuh;
// coarser levels (6x6 blocks) and the transfers (3x6 / 6x3 / 6x6 blocks) use the generic
// block-row product below.  Every kernel returns at once when the solver state says done.
#include <algorithm>
#include <vector>

#include "amg.cuh"
#include "pcg.cuh"

namespace fem {
namespace amg {
namespace {

using pcgd::PcgState;
constexpr int kThreads = 256;

// Device matrices are kept twice: row-SoA (val: the values of block row i, L blocks from
// ptr[i], at val[BB * ptr[i] + q * L + l] for value q of slot l, so lanes that take
// consecutive slots read consecutive words; used with one right-hand side) and block-major
// (valb[BB * (ptr[i] + l) + q]: a block in one or two cache lines, for the many-RHS kernels
// whose lanes of a row all read the same block).
struct DevView {
    int64_t n;
    const int32_t* ptr;
    const int32_t* col;
    const float* val;
    const float* valb;
};
inline DevView view(const DevBsr& M) { return DevView{M.n, M.ptr, M.col, M.val, M.valb}; }

// value (r, q) of slot li of a row starting at block rs with L blocks
template <int BR, int BC, bool SOA>
__device__ __forceinline__ float blk(const DevView& A, int rs, int L, int li, int r, int q) {
    if constexpr (SOA)
        return __ldg(A.val + int64_t(rs) * (BR * BC) + int64_t(r * BC + q) * L + li);
    else
        return __ldg(A.valb + (int64_t(rs) + li) * (BR * BC) + r * BC + q);
}

// ---- epilogues of the generic block-row product (row, right-hand side k, BR row sums) ----
template <int BR>
struct EpiStore {
    float* y;
    int R;
    __device__ void operator()(int64_t row, int k, const float (&a)[BR]) const {
#pragma unroll
        for (int r = 0; r < BR; ++r) y[(row * BR + r) * R + k] = a[r];
    }
};
template <int BR>
struct EpiAdd {
    float* y;
    int R;
    __device__ void operator()(int64_t row, int k, const float (&a)[BR]) const {
#pragma unroll
        for (int r = 0; r < BR; ++r) y[(row * BR + r) * R + k] += a[r];
    }
};
template <int BR>
struct EpiResid {
    const float* b;
    float* res;
    const uint8_t* iso;
    int R;
    __device__ void operator()(int64_t row, int k, const float (&a)[BR]) const {
        const bool dir = iso[row] != 0;
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            const int64_t i = (row * BR + r) * R + k;
            res[i] = dir ? 0.f : b[i] - a[r];
        }
    }
};
template <int BR>
struct EpiCheb {
    const float* b;
    const float* xin;
    float* xout;
    float* d;
    const float* dinv;
    const uint8_t* iso;
    float c1, c2;
    int R;
    __device__ void operator()(int64_t row, int k, const float (&a)[BR]) const {
        if (iso[row]) {
#pragma unroll
            for (int r = 0; r < BR; ++r) {
                const int64_t i = (row * BR + r) * R + k;
                xout[i] = xin[i];
            }
            return;
        }
        float rr[BR];
#pragma unroll
        for (int r = 0; r < BR; ++r) rr[r] = b[(row * BR + r) * R + k] - a[r];
        const float* m = dinv + row * BR * BR;
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            float z = 0.f;
#pragma unroll
            for (int q = 0; q < BR; ++q) z += __ldg(m + r * BR + q) * rr[q];
            const int64_t i = (row * BR + r) * R + k;
            float dn = c2 * z;
            if (c1 != 0.f) dn += c1 * d[i];
            d[i] = dn;
            xout[i] = xin[i] + dn;
        }
    }
};

// ---- generic block-row product y = A x with BR x BC blocks ----------------------------------
// nrhs == 1: LPR lanes per block row (lane = block slot), xor-shuffle sums.
template <int BR, int BC, int LPR, typename Epi>
__global__ void __launch_bounds__(kThreads) k_bsrg1(const DevView A, const float* __restrict__ x, const Epi epi,
                                                     const PcgState* __restrict__ st) {
    if (st->done) return;
    const int lane = threadIdx.x & 31, sub = lane / LPR, sl = lane % LPR;
    constexpr int RPW = 32 / LPR;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < A.n; base += nwarps * RPW) {
        const int64_t row = base + sub;
        const bool valid = row < A.n;
        float acc[BR];
#pragma unroll
        for (int r = 0; r < BR; ++r) acc[r] = 0.f;
        if (valid) {
            const int rs = __ldg(A.ptr + row);
            const int L = __ldg(A.ptr + row + 1) - rs;
            for (int li = sl; li < L; li += LPR) {
                const float* xc = x + int64_t(__ldg(A.col + rs + li)) * BC;
                float xs[BC];
#pragma unroll
                for (int q = 0; q < BC; ++q) xs[q] = xc[q];
#pragma unroll
                for (int r = 0; r < BR; ++r)
#pragma unroll
                    for (int q = 0; q < BC; ++q) acc[r] += blk<BR, BC, true>(A, rs, L, li, r, q) * xs[q];
            }
        }
#pragma unroll
        for (int r = 0; r < BR; ++r) acc[r] = group_sum<LPR>(acc[r]);
        if (valid && sl == 0) epi(row, 0, acc);
    }
}

// nrhs R > 1: lane = right-hand side (32 / R rows per warp); the R lanes of a row read the
// same block values (broadcast).
template <int BR, int BC, int R, typename Epi>
__global__ void __launch_bounds__(kThreads) k_bsrgR(const DevView A, const float* __restrict__ x, const Epi epi,
                                                     const PcgState* __restrict__ st) {
    if (st->done) return;
    const int lane = threadIdx.x & 31, sub = lane / R, k = lane % R;
    constexpr int RPW = 32 / R;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < A.n; base += nwarps * RPW) {
        const int64_t row = base + sub;
        if (row >= A.n) continue;
        float acc[BR];
#pragma unroll
        for (int r = 0; r < BR; ++r) acc[r] = 0.f;
        const int rs = __ldg(A.ptr + row);
        const int L = __ldg(A.ptr + row + 1) - rs;
        for (int li = 0; li < L; ++li) {
            const float* xc = x + int64_t(__ldg(A.col + rs + li)) * BC * R + k;
            float xs[BC];
#pragma unroll
            for (int q = 0; q < BC; ++q) xs[q] = xc[q * R];
#pragma unroll
            for (int r = 0; r < BR; ++r)
#pragma unroll
                for (int q = 0; q < BC; ++q) acc[r] += blk<BR, BC, false>(A, rs, L, li, r, q) * xs[q];
        }
        epi(row, k, acc);
    }
}

// Long rows or few rows: W warps share one block row.  Stream s (of W * 32 / R streams; lane
// = (stream in warp, right-hand side)) takes blocks s, s + streams, ...; the partial sums are
// combined by xor shuffles inside each warp and then over the warps through shared memory,
// in a fixed order.
template <int BR, int BC, int R, int W, typename Epi>
__global__ void __launch_bounds__(W * 32) k_bsrg_split(const DevView A, const float* __restrict__ x, const Epi epi,
                                                        const PcgState* __restrict__ st) {
    if (st->done) return;
    constexpr int G = 32 / R;
    constexpr int S = W * G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / R, k = lane % R;
    const int stream = warp * G + g;
    __shared__ float red[W][BR][R];
    for (int64_t row = blockIdx.x; row < A.n; row += gridDim.x) {
        float acc[BR];
#pragma unroll
        for (int r = 0; r < BR; ++r) acc[r] = 0.f;
        const int rs = __ldg(A.ptr + row);
        const int L = __ldg(A.ptr + row + 1) - rs;
        for (int li = stream; li < L; li += S) {
            const float* xc = x + int64_t(__ldg(A.col + rs + li)) * BC * R + k;
            float xs[BC];
#pragma unroll
            for (int q = 0; q < BC; ++q) xs[q] = xc[q * R];
#pragma unroll
            for (int r = 0; r < BR; ++r)
#pragma unroll
                for (int q = 0; q < BC; ++q) acc[r] += blk<BR, BC, R == 1>(A, rs, L, li, r, q) * xs[q];
        }
#pragma unroll
        for (int off = R; off < 32; off <<= 1)
#pragma unroll
            for (int r = 0; r < BR; ++r) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], off);
        if (g == 0) {
#pragma unroll
            for (int r = 0; r < BR; ++r) red[warp][r][k] = acc[r];
        }
        __syncthreads();
        if (warp == 0 && g == 0) {
            float tot[BR];
#pragma unroll
            for (int r = 0; r < BR; ++r) {
                tot[r] = red[0][r][k];
                for (int w = 1; w < W; ++w) tot[r] += red[w][r][k];
            }
            epi(row, k, tot);
        }
        __syncthreads();
    }
}

// ---- level-0 epilogues (spmv.cuh interface: o = first component, stride = R) ----------------
struct Epi0Resid {
    const float* b;
    float* res;
    const uint8_t* iso;
    __device__ void operator()(int64_t o, int stride, int k, float a0, float a1, float a2, Dot<float>&) const {
        const bool dir = iso[(o - k) / (3 * stride)] != 0;
        res[o] = dir ? 0.f : b[o] - a0;
        res[o + stride] = dir ? 0.f : b[o + stride] - a1;
        res[o + 2 * stride] = dir ? 0.f : b[o + 2 * stride] - a2;
    }
};
struct Epi0Cheb {
    const float* b;
    const float* xin;
    float* xout;
    float* d;
    const float* dinv;
    const uint8_t* iso;
    float c1, c2;
    __device__ void operator()(int64_t o, int stride, int k, float a0, float a1, float a2, Dot<float>&) const {
        const int64_t node = (o - k) / (3 * stride);
        if (iso[node]) {
            xout[o] = xin[o];
            xout[o + stride] = xin[o + stride];
            xout[o + 2 * stride] = xin[o + 2 * stride];
            return;
        }
        const float r0 = b[o] - a0, r1 = b[o + stride] - a1, r2 = b[o + 2 * stride] - a2;
        const float* m = dinv + 9 * node;
        const float z[3] = {__ldg(m) * r0 + __ldg(m + 1) * r1 + __ldg(m + 2) * r2,
                            __ldg(m + 3) * r0 + __ldg(m + 4) * r1 + __ldg(m + 5) * r2,
                            __ldg(m + 6) * r0 + __ldg(m + 7) * r1 + __ldg(m + 8) * r2};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int64_t i = o + j * stride;
            float dn = c2 * z[j];
            if (c1 != 0.f) dn += c1 * d[i];
            d[i] = dn;
            xout[i] = xin[i] + dn;
        }
    }
};

template <int LPR, typename Epi>
__global__ void __launch_bounds__(kThreads) k_l0_1(const BsrView<float> A, const float* __restrict__ x, const Epi epi,
                                                    const PcgState* __restrict__ st) {
    if (st->done) return;
    spmv1_rows_epi<float, LPR>(A, x, epi);
}
template <int R, typename Epi>
__global__ void __launch_bounds__(kThreads) k_l0_R(const BsrView<float> A, const float* __restrict__ x, const Epi epi,
                                                    const PcgState* __restrict__ st) {
    if (st->done) return;
    spmm_rows_epi<float, R>(A, x, epi);
}

// first Chebyshev step from x = 0: d = c2 D^-1 b, x = d (Dirichlet nodes: x = D^-1 b)
template <int B>
__global__ void __launch_bounds__(kThreads) k_cheb0(int64_t n, int R, const float* __restrict__ b,
                                                     const float* __restrict__ dinv, const uint8_t* __restrict__ iso,
                                                     float c2, float* x, float* d, const PcgState* __restrict__ st) {
    if (st->done) return;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n * R; t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t node = t / R;
        const int k = int(t % R);
        float rr[B];
#pragma unroll
        for (int q = 0; q < B; ++q) rr[q] = b[(node * B + q) * R + k];
        const float* m = dinv + node * B * B;
        const float c = iso[node] ? 1.f : c2;
#pragma unroll
        for (int r = 0; r < B; ++r) {
            float z = 0.f;
#pragma unroll
            for (int q = 0; q < B; ++q) z += __ldg(m + r * B + q) * rr[q];
            const int64_t i = (node * B + r) * R + k;
            d[i] = c * z;
            x[i] = c * z;
        }
    }
}

// Dirichlet-row update, two steps so that no row reads a value another thread writes:
// tmp = x_I + D_I^-1 (b - A x)_I for the listed rows, then x_I = tmp.  One warp per (row,
// right-hand side), lanes over the row's blocks; the rows are few (the penalised nodes).
template <typename View>
__global__ void __launch_bounds__(kThreads) k_dir_fix(const View A, const int32_t* __restrict__ rows, int64_t nrows,
                                                       int R, const float* __restrict__ b, const float* __restrict__ x,
                                                       const float* __restrict__ dinv, float* tmp,
                                                       const PcgState* __restrict__ st) {
    if (st->done) return;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t t = warp; t < nrows * R; t += nwarps) {
        const int64_t row = rows[t / R];
        const int k = int(t % R);
        const int64_t rs = A.indptr[row];
        const int L = A.indptr[row + 1] - int(rs);
        float a[3] = {0.f, 0.f, 0.f};
        for (int l = lane; l < L; l += 32) {
            const int64_t c = A.indices[rs + l];
            const float* xc = x + 3 * c * R + k;
            const float x0 = xc[0], x1 = xc[R], x2 = xc[2 * R];
#pragma unroll
            for (int p = 0; p < 3; ++p)
                a[p] += *block_value(A, rs, L, l, 3 * p) * x0 + *block_value(A, rs, L, l, 3 * p + 1) * x1 +
                        *block_value(A, rs, L, l, 3 * p + 2) * x2;
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) a[p] = group_sum<32>(a[p]);
        if (lane == 0) {
            const int64_t o = 3 * row * R + k;
            const float r0 = b[o] - a[0], r1 = b[o + R] - a[1], r2 = b[o + 2 * R] - a[2];
            const float* m = dinv + 9 * row;
            float* tt = tmp + 3 * (t / R) * R + k;
            tt[0] = x[o] + m[0] * r0 + m[1] * r1 + m[2] * r2;
            tt[R] = x[o + R] + m[3] * r0 + m[4] * r1 + m[5] * r2;
            tt[2 * R] = x[o + 2 * R] + m[6] * r0 + m[7] * r1 + m[8] * r2;
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_dir_copy(const int32_t* __restrict__ rows, int64_t nrows, int R,
                                                        const float* __restrict__ tmp, float* x,
                                                        const PcgState* __restrict__ st) {
    if (st->done) return;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < nrows * R; t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t row = rows[t / R];
        const int k = int(t % R);
        const int64_t o = 3 * row * R + k;
        const float* tt = tmp + 3 * (t / R) * R + k;
        x[o] = tt[0];
        x[o + R] = tt[R];
        x[o + 2 * R] = tt[2 * R];
    }
}

// dense coarsest solve x = Ainv b: one warp per (row, right-hand side)
__global__ void __launch_bounds__(kThreads) k_dense(int64_t m, int R, const float* __restrict__ inv,
                                                     const float* __restrict__ b, float* x,
                                                     const PcgState* __restrict__ st) {
    if (st->done) return;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t w = warp; w < m * R; w += nwarps) {
        const int64_t i = w / R;
        const int k = int(w % R);
        float s = 0.f;
        for (int64_t j = lane; j < m; j += 32) s += __ldg(inv + i * m + j) * b[j * R + k];
        s = group_sum<32>(s);
        if (lane == 0) x[i * R + k] = s;
    }
}

unsigned grid_for(int64_t work_items, int per_cta) {
    const int64_t need = (work_items + per_cta - 1) / per_cta;
    return unsigned(std::max<int64_t>(1, std::min<int64_t>(need, int64_t(sm_count()) * 8)));
}

// Grid of a grid-stride block-row product: one wave of resident CTAs (a second, partial wave
// would run with too few warps to hide the gathers' latency).
unsigned product_grid(const void* kernel, int64_t rows, int rows_per_cta) {
    return resident_grid(kernel, kThreads, (rows + rows_per_cta - 1) / rows_per_cta, int64_t(sm_count()) * 8);
}

int lanes_for(const DevBsr& M) {
    const double avg = M.n > 0 ? double(M.nnzb) / double(M.n) : 1.0;
    return avg < 6 ? 4 : avg < 16 ? 8 : avg < 48 ? 16 : 32;
}

template <int BR, int BC, int R, typename Epi>
void launch_split(const DevView& v, double avg, const float* x, const Epi& epi, const PcgState* st, cudaStream_t s) {
    // about four blocks per stream: W * (32 / R) streams ~ avg / 4 (R > 1), ~ avg / 2 (R == 1)
    constexpr int G = 32 / R;
    const double want = (R == 1 ? avg / 2.0 : avg / 4.0) / G;
    const int W = want > 4 ? 8 : want > 2 ? 4 : want > 1 ? 2 : 1;
    const int64_t cap = int64_t(sm_count()) * (2048 / (W * 32)) * 4;
    const unsigned g = unsigned(std::max<int64_t>(1, std::min<int64_t>(v.n, cap)));
    switch (W) {
        case 8: k_bsrg_split<BR, BC, R, 8><<<g, 256, 0, s>>>(v, x, epi, st); break;
        case 4: k_bsrg_split<BR, BC, R, 4><<<g, 128, 0, s>>>(v, x, epi, st); break;
        case 2: k_bsrg_split<BR, BC, R, 2><<<g, 64, 0, s>>>(v, x, epi, st); break;
        default: k_bsrg_split<BR, BC, R, 1><<<g, 32, 0, s>>>(v, x, epi, st); break;
    }
}

// y (op) = M x for the generic levels; dispatch on block shape, nrhs and row length: many
// short rows take several rows per warp, long rows the split-row kernel
template <int BR, int BC, typename Epi>
int launch_gen(const DevBsr& M, const float* x, const Epi& epi, const PcgState* st, int R, cudaStream_t s) {
    const DevView v = view(M);
    const double avg = M.n > 0 ? double(M.nnzb) / double(M.n) : 1.0;
    if (avg >= (R == 1 ? 24.0 : 8.0)) {
        switch (R) {
            case 1: launch_split<BR, BC, 1>(v, avg, x, epi, st, s); break;
            case 2: launch_split<BR, BC, 2>(v, avg, x, epi, st, s); break;
            case 4: launch_split<BR, BC, 4>(v, avg, x, epi, st, s); break;
            case 8: launch_split<BR, BC, 8>(v, avg, x, epi, st, s); break;
            case 16: launch_split<BR, BC, 16>(v, avg, x, epi, st, s); break;
            default: launch_split<BR, BC, 32>(v, avg, x, epi, st, s); break;
        }
        FEM_LAUNCH_CHECK("amg block-row product (split rows)");
        return FEM_OK;
    }
    auto run = [&](auto kernel, int rows_per_cta) {
        kernel<<<product_grid(reinterpret_cast<const void*>(kernel), M.n, rows_per_cta), kThreads, 0, s>>>(v, x, epi,
                                                                                                             st);
    };
    if (R == 1) {
        const int lpr = lanes_for(M);
        const int rpc = (kThreads / 32) * (32 / lpr);
        switch (lpr) {
            case 4: run(k_bsrg1<BR, BC, 4, Epi>, rpc); break;
            case 8: run(k_bsrg1<BR, BC, 8, Epi>, rpc); break;
            case 16: run(k_bsrg1<BR, BC, 16, Epi>, rpc); break;
            default: run(k_bsrg1<BR, BC, 32, Epi>, rpc); break;
        }
    } else {
        const int rpc = (kThreads / 32) * (32 / R);
        switch (R) {
            case 2: run(k_bsrgR<BR, BC, 2, Epi>, rpc); break;
            case 4: run(k_bsrgR<BR, BC, 4, Epi>, rpc); break;
            case 8: run(k_bsrgR<BR, BC, 8, Epi>, rpc); break;
            case 16: run(k_bsrgR<BR, BC, 16, Epi>, rpc); break;
            default: run(k_bsrgR<BR, BC, 32, Epi>, rpc); break;
        }
    }
    FEM_LAUNCH_CHECK("amg block-row product");
    return FEM_OK;
}

template <typename Epi>
int launch_l0(const BsrView<float>& A, const float* x, const Epi& epi, const PcgState* st, int R, cudaStream_t s) {
    auto run = [&](auto kernel, int rows_per_cta) {
        kernel<<<product_grid(reinterpret_cast<const void*>(kernel), A.n, rows_per_cta), kThreads, 0, s>>>(A, x, epi,
                                                                                                             st);
    };
    if (R == 1) {
        run(k_l0_1<8, Epi>, (kThreads / 32) * 4);
    } else {
        const int rpc = (kThreads / 32) * (32 / R);
        switch (R) {
            case 2: run(k_l0_R<2, Epi>, rpc); break;
            case 4: run(k_l0_R<4, Epi>, rpc); break;
            case 8: run(k_l0_R<8, Epi>, rpc); break;
            case 16: run(k_l0_R<16, Epi>, rpc); break;
            default: run(k_l0_R<32, Epi>, rpc); break;
        }
    }
    FEM_LAUNCH_CHECK("amg level-0 product");
    return FEM_OK;
}

// one Chebyshev step on level l: xout = xin + d, d = c1 d + c2 D^-1 (b - A xin)
template <typename View>
int cheb_step(fem_amg* h, int l, const View& A0, const float* b, const float* xin, float* xout, float c1, float c2,
              const PcgState* st, int R, cudaStream_t s) {
    Level& L = h->lv[l];
    if (l == 0) return launch_l0(A0, xin, Epi0Cheb{b, xin, xout, L.vd, L.d_dinv, L.d_iso, c1, c2}, st, R, s);
    return launch_gen<kModes, kModes>(L.dA, xin, EpiCheb<kModes>{b, xin, xout, L.vd, L.d_dinv, L.d_iso, c1, c2, R},
                                      st, R, s);
}

template <typename View>
int cycle(fem_amg* h, int l, const View& A0, const float* b, float* out, const PcgState* st, int R, bool sym,
          cudaStream_t s) {
    const int last = int(h->lv.size()) - 1;
    if (l == last) {
        const int64_t work = h->coarse_m * R;
        k_dense<<<grid_for(work, kThreads / 32), kThreads, 0, s>>>(h->coarse_m, R, h->d_coarse_inv, b, out, st);
        FEM_LAUNCH_CHECK("amg coarse solve");
        return FEM_OK;
    }
    Level& L = h->lv[l];
    Level& C = h->lv[l + 1];
    const int pre = h->opts.pre_degree, post = h->opts.post_degree;
    float* X[2] = {out, L.vx};
    int cur = ((pre - 1) + post) & 1;  // the last step then writes `out`
    int rc;
    if (L.b == 3)
        k_cheb0<3><<<grid_for(L.n * R, kThreads), kThreads, 0, s>>>(L.n, R, b, L.d_dinv, L.d_iso, L.c2[0], X[cur],
                                                                     L.vd, st);
    else
        k_cheb0<kModes><<<grid_for(L.n * R, kThreads), kThreads, 0, s>>>(L.n, R, b, L.d_dinv, L.d_iso, L.c2[0],
                                                                          X[cur], L.vd, st);
    FEM_LAUNCH_CHECK("amg first smoothing step");
    for (int k = 1; k < pre; ++k) {
        if ((rc = cheb_step(h, l, A0, b, X[cur], X[cur ^ 1], L.c1[k], L.c2[k], st, R, s))) return rc;
        cur ^= 1;
    }
    // residual, restriction
    if (l == 0)
        rc = launch_l0(A0, X[cur], Epi0Resid{b, L.vr, L.d_iso}, st, R, s);
    else
        rc = launch_gen<kModes, kModes>(L.dA, X[cur], EpiResid<kModes>{b, L.vr, L.d_iso, R}, st, R, s);
    if (rc) return rc;
    if (L.b == 3)
        rc = launch_gen<kModes, 3>(L.dR, L.vr, EpiStore<kModes>{C.vb, R}, st, R, s);
    else
        rc = launch_gen<kModes, kModes>(L.dR, L.vr, EpiStore<kModes>{C.vb, R}, st, R, s);
    if (rc) return rc;
    if ((rc = cycle(h, l + 1, A0, C.vb, C.vo, st, R, false, s))) return rc;
    // prolongation
    if (L.b == 3)
        rc = launch_gen<3, kModes>(L.dP, C.vo, EpiAdd<3>{X[cur], R}, st, R, s);
    else
        rc = launch_gen<kModes, kModes>(L.dP, C.vo, EpiAdd<kModes>{X[cur], R}, st, R, s);
    if (rc) return rc;
    for (int k = 0; k < post; ++k) {
        if ((rc = cheb_step(h, l, A0, b, X[cur], X[cur ^ 1], k == 0 ? 0.f : L.c1[k], L.c2[k], st, R, s))) return rc;
        cur ^= 1;
    }
    if (sym && l == 0 && L.n_iso > 0) {
        k_dir_fix<<<grid_for(L.n_iso * R, kThreads / 32), kThreads, 0, s>>>(A0, L.d_iso_rows, L.n_iso, R, b, out,
                                                                             L.d_dinv, L.vfix, st);
        k_dir_copy<<<grid_for(L.n_iso * R, kThreads), kThreads, 0, s>>>(L.d_iso_rows, L.n_iso, R, L.vfix, out, st);
        FEM_LAUNCH_CHECK("amg Dirichlet rows");
    }
    return FEM_OK;
}

template <typename T>
int upload_array(const std::vector<T>& h, T** d) {
    if (h.empty()) return FEM_OK;
    FEM_CUDA(cudaMalloc(reinterpret_cast<void**>(d), sizeof(T) * h.size()));
    FEM_CUDA(cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return FEM_OK;
}

// FP32 row-SoA and block-major copies (see DevView) with 32-bit row pointers.
int upload_bsr(const HostBsr& H, DevBsr& D) {
    D.n = H.n;
    D.m = H.m;
    D.br = H.br;
    D.bc = H.bc;
    D.nnzb = H.nnzb();
    if (H.ptr.empty()) return FEM_OK;
    FEM_REQUIRE(H.nnzb() < (int64_t(1) << 31), "AMG matrix too large for 32-bit row pointers");
    std::vector<int32_t> p(H.ptr.begin(), H.ptr.end());
    const int64_t bb = int64_t(H.br) * H.bc;
    std::vector<float> v(H.val.size());
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < H.n; ++i) {
        const int64_t rs = H.ptr[i], L = H.ptr[i + 1] - rs;
        for (int64_t l = 0; l < L; ++l)
            for (int64_t q = 0; q < bb; ++q) v[bb * rs + q * L + l] = float(H.val[(rs + l) * bb + q]);
    }
    int rc;
    if ((rc = upload_array(p, &D.ptr))) return rc;
    if ((rc = upload_array(H.col, &D.col))) return rc;
    if ((rc = upload_array(v, &D.val))) return rc;
    std::vector<float> vb(H.val.size());
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < int64_t(vb.size()); ++e) vb[e] = float(H.val[e]);
    return upload_array(vb, &D.valb);
}

void free_bsr(DevBsr& D) {
    cudaFree(D.ptr);
    cudaFree(D.col);
    cudaFree(D.val);
    cudaFree(D.valb);
    D.ptr = nullptr;
    D.col = nullptr;
    D.val = nullptr;
    D.valb = nullptr;
}

void free_vectors(fem_amg* h) {
    for (Level& L : h->lv) {
        for (float** v : {&L.vb, &L.vo, &L.vx, &L.vd, &L.vr, &L.vfix}) {
            cudaFree(*v);
            *v = nullptr;
        }
    }
    cudaFree(h->r32);
    cudaFree(h->z32);
    h->r32 = h->z32 = nullptr;
    h->vec_nrhs = 0;
}

void free_dev64(Dev64& D) {
    cudaFree(D.ptr);
    cudaFree(D.col);
    cudaFree(D.val);
    D = Dev64{};
}

void free_device(fem_amg* h) {
    free_vectors(h);
    for (Level& L : h->lv) {
        free_bsr(L.dA);
        free_bsr(L.dP);
        free_bsr(L.dR);
        free_dev64(L.gA);
        free_dev64(L.gP);
        free_dev64(L.gR);
        cudaFree(L.g_dinv);
        L.g_dinv = nullptr;
        cudaFree(L.d_dinv);
        L.d_dinv = nullptr;
        cudaFree(L.d_iso);
        L.d_iso = nullptr;
        cudaFree(L.d_iso_rows);
        L.d_iso_rows = nullptr;
        L.n_iso = 0;
    }
    cudaFree(h->d_coarse_inv);
    h->d_coarse_inv = nullptr;
    cudaFree(h->d_state);
    h->d_state = nullptr;
    h->uploaded = false;
}

}  // namespace

void release_device(fem_amg* h) { free_device(h); }

int ensure_vectors(fem_amg* h, int R) {
    if (h->vec_nrhs >= R) return FEM_OK;
    free_vectors(h);
    for (size_t l = 0; l < h->lv.size(); ++l) {
        Level& L = h->lv[l];
        const size_t bytes = sizeof(float) * size_t(L.n) * L.b * R;
        if (l > 0) {
            FEM_CUDA(cudaMalloc(&L.vb, bytes));
            FEM_CUDA(cudaMalloc(&L.vo, bytes));
        }
        if (l + 1 < h->lv.size()) {
            FEM_CUDA(cudaMalloc(&L.vx, bytes));
            FEM_CUDA(cudaMalloc(&L.vd, bytes));
            FEM_CUDA(cudaMalloc(&L.vr, bytes));
        }
        if (L.n_iso > 0) FEM_CUDA(cudaMalloc(&L.vfix, sizeof(float) * size_t(L.n_iso) * L.b * R));
    }
    const size_t b0 = sizeof(float) * size_t(h->lv[0].n) * 3 * R;
    FEM_CUDA(cudaMalloc(&h->r32, b0));
    FEM_CUDA(cudaMalloc(&h->z32, b0));
    h->vec_nrhs = R;
    return FEM_OK;
}

template <typename View>
int vcycle(fem_amg* h, const View& A0, const float* r, float* z, const PcgState* st, int R, bool symmetric,
           cudaStream_t s) {
    return cycle(h, 0, A0, r, z, st, R, symmetric, s);
}
template int vcycle<BsrView<float>>(fem_amg*, const BsrView<float>&, const float*, float*, const PcgState*, int, bool,
                                     cudaStream_t);

}  // namespace amg
}  // namespace fem

using namespace fem;
using namespace fem::amg;

extern "C" int fem_amg_upload(fem_amg* h, void* stream) {
    FEM_REQUIRE(h && !h->lv.empty(), "NULL or empty AMG hierarchy");
    if (h->uploaded) return FEM_OK;
    FEM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    int rc = FEM_OK;
    for (size_t l = 0; l < h->lv.size() && !rc; ++l) {
        Level& L = h->lv[l];
        if (l > 0) rc = upload_bsr(L.A, L.dA);
        if (!rc && l + 1 < h->lv.size()) {
            rc = upload_bsr(L.P, L.dP);
            if (!rc) rc = upload_bsr(L.R, L.dR);
        }
        if (!rc) {
            std::vector<float> di(L.dinv.begin(), L.dinv.end());
            rc = upload_array(di, &L.d_dinv);
        }
        if (!rc) rc = upload_array(L.iso, &L.d_iso);
        if (!rc && l == 0) {
            std::vector<int32_t> rows;
            for (size_t i = 0; i < L.iso.size(); ++i)
                if (L.iso[i]) rows.push_back(int32_t(i));
            L.n_iso = int64_t(rows.size());
            rc = upload_array(rows, &L.d_iso_rows);
        }
    }
    if (!rc) {
        std::vector<float> ci(h->coarse_inv.begin(), h->coarse_inv.end());
        rc = upload_array(ci, &h->d_coarse_inv);
    }
    if (!rc) {
        rc = cuda_status(cudaMalloc(&h->d_state, sizeof(pcgd::PcgState)), "cudaMalloc");
        if (!rc) rc = cuda_status(cudaMemset(h->d_state, 0, sizeof(pcgd::PcgState)), "cudaMemset");
    }
    if (rc) {
        free_device(h);
        return rc;
    }
    h->uploaded = true;
    return FEM_OK;
}

extern "C" void fem_amg_destroy(fem_amg* h) {
    if (!h) return;
    free_device(h);
    delete h;
}

extern "C" int fem_amg_vcycle(fem_amg* h, const fem_bsr* A32, int nrhs, const float* r, float* z, int symmetric,
                              void* stream) {
    FEM_REQUIRE(h && A32 && r && z, "NULL argument");
    FEM_REQUIRE(h->uploaded, "call fem_amg_upload first");
    FEM_REQUIRE(A32->dtype == FEM_F32 && A32->n_brow == h->lv[0].n && A32->indptr && A32->indices && A32->vals,
                "A32 must be the FP32 copy of the level-0 matrix");
    FEM_REQUIRE(A32->layout == FEM_LAYOUT_BSR || A32->layout == FEM_LAYOUT_RSOA || A32->layout == FEM_LAYOUT_RSOA4,
                "A32: layout must be BSR, RSOA or RSOA4");
    FEM_REQUIRE(A32->layout != FEM_LAYOUT_RSOA4 || (aligned16(A32->vals) && aligned16(A32->indices)),
                "A32: FEM_LAYOUT_RSOA4 arrays must be 16-byte aligned");
    FEM_REQUIRE(nrhs == 1 || nrhs == 2 || nrhs == 4 || nrhs == 8 || nrhs == 16 || nrhs == 32,
                "nrhs must be 1, 2, 4, 8, 16 or 32");
    int rc = ensure_vectors(h, nrhs);
    if (rc) return rc;
    const BsrView<float> A{A32->n_brow, A32->indptr, A32->indices, static_cast<const float*>(A32->vals),
                           rsoa_kind(A32->layout)};
    return vcycle(h, A, r, z, static_cast<const pcgd::PcgState*>(h->d_state), nrhs, symmetric != 0, as_stream(stream));
}
