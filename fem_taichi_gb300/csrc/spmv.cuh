// BSR (3x3 block) SpMV / SpMM device code shared by spmv.cu and pcg.cu.
//
// Vectors with nrhs right-hand sides are stored [n_brow][3][nrhs] (right-hand side
// fastest), so one block row's inputs/outputs for all RHS are contiguous.
//  * nrhs == 1: LPR lanes cooperate on one block row (lane = block slot), followed by an
//    xor-shuffle reduction of the three row sums; 32/LPR rows per warp.
//  * nrhs  > 1: lanes map to right-hand sides (32/nrhs rows per warp); each block's nine
//    values are loaded once per row group (broadcast) and applied to all RHS.
// Rows are visited with a grid-stride loop so the grid can be sized in multiples of the SM
// count; a fixed grid gives a fixed row -> CTA mapping, hence deterministic partial sums.
#pragma once

#include "fem_common.cuh"

namespace fem {

template <typename T>
struct BsrView {
    int64_t n;              // block rows
    const int32_t* indptr;  // [n+1]
    const int32_t* indices; // [nnzb]
    const T* vals;          // [nnzb][3][3] (BSR) or, per block row, [9][row length] (row-SoA)
    int rsoa;               // 1: row-SoA value layout; 2: row-SoA padded to 4-block multiples (FP32)
};

// Dot-product accumulator of the solver.  FP64 vectors: plain FP64 fused multiply-adds.
// FP32 vectors: every product is formed exactly (FMA error term) and summed with a
// compensated two-sum in FP32 pairs (about 48 significant bits), and becomes a double once
// per thread, so the per-element work stays on the FP32 pipes (GB300's FP64 pipe is ~64x
// slower) while the dot products keep FP64-class accuracy.
template <typename T>
struct Dot {
    double v = 0.0;
    __device__ __forceinline__ void add(T a, T b) { v = fma(double(a), double(b), v); }
    __device__ __forceinline__ double value() const { return v; }
};
template <>
struct Dot<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float a, float b) {
        const float pr = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -pr);
        const float t = __fadd_rn(s, pr);
        const float bb = __fsub_rn(t, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(pr, bb));
        s = t;
        c = __fadd_rn(c, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return double(s) + double(c); }
};

// BsrView::rsoa for a fem_bsr layout code
inline int rsoa_kind(int layout) {
    return layout == FEM_LAYOUT_RSOA ? 1 : layout == FEM_LAYOUT_RSOA4 ? 2 : 0;
}

// address of value q (0..8) of the block in slot l of the row starting at rs with L blocks
template <typename T>
__device__ __forceinline__ const T* block_value(const BsrView<T>& A, int64_t rs, int L, int l, int q) {
    return A.rsoa ? A.vals + 9 * rs + int64_t(q) * L + l : A.vals + 9 * (rs + l) + q;
}

// (a0, a1, a2) += B x for the 3x3 block B whose values start at v (stride vs between them):
// nine chained fused multiply-adds, the product's only FP64 work (written as a sum of three
// products per row, it compiled to a multiply, two FMAs and an add: 12 instructions).
template <typename T>
__device__ __forceinline__ void block_fma3(const T* v, int64_t vs, T x0, T x1, T x2, T& a0, T& a1, T& a2) {
    a0 = fma(__ldg(v + 0 * vs), x0, a0);
    a1 = fma(__ldg(v + 3 * vs), x0, a1);
    a2 = fma(__ldg(v + 6 * vs), x0, a2);
    a0 = fma(__ldg(v + 1 * vs), x1, a0);
    a1 = fma(__ldg(v + 4 * vs), x1, a1);
    a2 = fma(__ldg(v + 7 * vs), x1, a2);
    a0 = fma(__ldg(v + 2 * vs), x2, a0);
    a1 = fma(__ldg(v + 5 * vs), x2, a1);
    a2 = fma(__ldg(v + 8 * vs), x2, a2);
}

// Sum over lanes l' with (l' / G) == (l / G) of a warp split into groups of G lanes.
template <int G, typename V>
__device__ __forceinline__ V group_sum(V v) {
#pragma unroll
    for (int off = G / 2; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Row epilogues.  The product kernels hand each finished row (and right-hand side k) to
// an epilogue: o is the index of the row's first component in the [n][3][R] vectors,
// `stride` = R, (a0, a1, a2) = (A x) of the row.

// y = A x, and dot += x_row . y_row when asked (PCG's p.q).
template <typename T>
struct StoreY {
    const T* x;
    T* y;
    bool want_dot;
    __device__ __forceinline__ void operator()(int64_t o, int stride, int, T a0, T a1, T a2, Dot<T>& dot) const {
        y[o] = a0;
        y[o + stride] = a1;
        y[o + 2 * stride] = a2;
        if (want_dot) {
            dot.add(x[o], a0);
            dot.add(x[o + stride], a1);
            dot.add(x[o + 2 * stride], a2);
        }
    }
};

// Padded row-SoA FP32 product: each lane takes 4 consecutive slots of its row per step and
// reads each of the 9 values of those 4 blocks with one 16-byte load (rows, values and
// slot groups all start on 16-byte boundaries); padding blocks hold zeros.
template <int LPR, typename Epi>
__device__ __forceinline__ double spmv4_rows_epi(const BsrView<float>& A, const float* __restrict__ x, const Epi& epi) {
    const int lane = threadIdx.x & 31;
    const int sub = lane / LPR, sl = lane % LPR;
    constexpr int RPW = 32 / LPR;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    Dot<float> dot;
    for (int64_t base = warp * RPW; base < A.n; base += nwarps * RPW) {
        const int64_t row = base + sub;
        const bool valid = row < A.n;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        if (valid) {
            const int64_t rs = __ldg(A.indptr + row);
            const int Lp = __ldg(A.indptr + row + 1) - int(rs);
            const float* v0 = A.vals + 9 * rs;
            for (int s = 4 * sl; s < Lp; s += 4 * LPR) {
                const int4 c = __ldg(reinterpret_cast<const int4*>(A.indices + rs + s));
                float4 w[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) w[q] = __ldg(reinterpret_cast<const float4*>(v0 + int64_t(q) * Lp + s));
                const int cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    // component j of each value's float4 = slot s + j
                    auto wq = [&](int q) { return j == 0 ? w[q].x : j == 1 ? w[q].y : j == 2 ? w[q].z : w[q].w; };
                    const float* xc = x + 3 * int64_t(cc[j]);
                    const float x0 = xc[0], x1 = xc[1], x2 = xc[2];
                    a0 += wq(0) * x0 + wq(1) * x1 + wq(2) * x2;
                    a1 += wq(3) * x0 + wq(4) * x1 + wq(5) * x2;
                    a2 += wq(6) * x0 + wq(7) * x1 + wq(8) * x2;
                }
            }
        }
        a0 = group_sum<LPR>(a0);
        a1 = group_sum<LPR>(a1);
        a2 = group_sum<LPR>(a2);
        if (valid && sl == 0) epi(3 * row, 1, 0, a0, a1, a2, dot);
    }
    return dot.value();
}

// One pass of A x over the rows assigned to this thread (LPR lanes per block row; one RHS);
// returns this lane's share of the epilogue's dot product.
template <typename T, int LPR, typename Epi>
__device__ __forceinline__ double spmv1_rows_epi(const BsrView<T>& A, const T* __restrict__ x, const Epi& epi) {
    if constexpr (sizeof(T) == 4) {
        if (A.rsoa == 2) return spmv4_rows_epi<(LPR > 8 ? 8 : LPR)>(A, x, epi);
    }
    const int lane = threadIdx.x & 31;
    const int sub = lane / LPR, sl = lane % LPR;
    constexpr int RPW = 32 / LPR;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    Dot<T> dot;
    for (int64_t base = warp * RPW; base < A.n; base += nwarps * RPW) {
        const int64_t row = base + sub;
        const bool valid = row < A.n;
        T a0 = 0, a1 = 0, a2 = 0;
        if (valid) {
            const int64_t rs = __ldg(A.indptr + row);
            const int L = __ldg(A.indptr + row + 1) - int(rs);
            const int64_t vs = A.rsoa ? int64_t(L) : 1;  // stride between the 9 values of a block
            for (int l = sl; l < L; l += LPR) {
                const int64_t c = __ldg(A.indices + rs + l);
                const T* v = block_value(A, rs, L, l, 0);
                const T x0 = x[3 * c], x1 = x[3 * c + 1], x2 = x[3 * c + 2];
                block_fma3(v, vs, x0, x1, x2, a0, a1, a2);
            }
        }
        a0 = group_sum<LPR>(a0);
        a1 = group_sum<LPR>(a1);
        a2 = group_sum<LPR>(a2);
        if (valid && sl == 0) epi(3 * row, 1, 0, a0, a1, a2, dot);
    }
    return dot.value();
}

// Many right-hand sides on the padded row-SoA FP32 copy: one block row per warp, lane =
// (slot group g, right-hand side k) with 32 / R slot groups; each lane takes 4 consecutive
// slots per step (one 16-byte load per value, the same address for the R lanes of a group),
// then the groups' partial sums are combined by xor-shuffles.
template <int R, typename Epi>
__device__ __forceinline__ double spmm4_rows_epi(const BsrView<float>& A, const float* __restrict__ x, const Epi& epi) {
    constexpr int G = 32 / R;
    const int lane = threadIdx.x & 31;
    const int g = lane / R, rhs = lane % R;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    Dot<float> dot;
    for (int64_t row = warp; row < A.n; row += nwarps) {
        const int64_t rs = __ldg(A.indptr + row);
        const int Lp = __ldg(A.indptr + row + 1) - int(rs);
        const float* v0 = A.vals + 9 * rs;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f;
        for (int s = 4 * g; s < Lp; s += 4 * G) {
            const int4 c = __ldg(reinterpret_cast<const int4*>(A.indices + rs + s));
            float4 w[9];
#pragma unroll
            for (int q = 0; q < 9; ++q) w[q] = __ldg(reinterpret_cast<const float4*>(v0 + int64_t(q) * Lp + s));
            const int cc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                auto wq = [&](int q) { return j == 0 ? w[q].x : j == 1 ? w[q].y : j == 2 ? w[q].z : w[q].w; };
                const float* xc = x + 3 * int64_t(cc[j]) * R + rhs;
                const float x0 = xc[0], x1 = xc[R], x2 = xc[2 * R];
                a0 += wq(0) * x0 + wq(1) * x1 + wq(2) * x2;
                a1 += wq(3) * x0 + wq(4) * x1 + wq(5) * x2;
                a2 += wq(6) * x0 + wq(7) * x1 + wq(8) * x2;
            }
        }
#pragma unroll
        for (int off = R; off < 32; off <<= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, off);
            a1 += __shfl_xor_sync(0xffffffffu, a1, off);
            a2 += __shfl_xor_sync(0xffffffffu, a2, off);
        }
        if (g == 0) epi(3 * row * R + rhs, R, rhs, a0, a1, a2, dot);
    }
    return dot.value();
}

// Many right-hand sides: lane = RHS (32 / R rows per warp), each block's values loaded once
// per row group and applied to every RHS.
template <typename T, int R, typename Epi>
__device__ __forceinline__ double spmm_rows_epi(const BsrView<T>& A, const T* __restrict__ x, const Epi& epi) {
    if constexpr (sizeof(T) == 4) {
        if (A.rsoa == 2) return spmm4_rows_epi<R>(A, x, epi);
    }
    const int lane = threadIdx.x & 31;
    const int sub = lane / R, rhs = lane % R;
    constexpr int RPW = 32 / R;
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
    Dot<T> dot;
    for (int64_t base = warp * RPW; base < A.n; base += nwarps * RPW) {
        const int64_t row = base + sub;
        if (row >= A.n) continue;
        const int64_t rs = __ldg(A.indptr + row);
        const int L = __ldg(A.indptr + row + 1) - int(rs);
        T a0 = 0, a1 = 0, a2 = 0;
        const int64_t vs = A.rsoa ? int64_t(L) : 1;
        for (int l = 0; l < L; ++l) {
            const int64_t c = __ldg(A.indices + rs + l);
            const T* v = block_value(A, rs, L, l, 0);
            const T* xc = x + 3 * c * R + rhs;
            const T x0 = xc[0], x1 = xc[R], x2 = xc[2 * R];
            block_fma3(v, vs, x0, x1, x2, a0, a1, a2);
        }
        epi(3 * row * R + rhs, R, rhs, a0, a1, a2, dot);
    }
    return dot.value();
}

// y = A x forms of the three products (dot: sum_rows x_i . y_i when want_dot).
template <typename T, int LPR>
__device__ __forceinline__ double spmv1_rows(const BsrView<T>& A, const T* __restrict__ x, T* __restrict__ y,
                                             bool want_dot) {
    return spmv1_rows_epi<T, LPR>(A, x, StoreY<T>{x, y, want_dot});
}

template <typename T, int R>
__device__ __forceinline__ double spmm_rows(const BsrView<T>& A, const T* __restrict__ x, T* __restrict__ y,
                                            bool want_dot) {
    return spmm_rows_epi<T, R>(A, x, StoreY<T>{x, y, want_dot});
}

// SpMV launch variants picked by the autotuner (nrhs == 1): lanes per block row and CTA size.
struct SpmvVariant {
    int lpr;      // 32, 16 or 8 lanes per block row
    int threads;  // CTA size
    int ctas_per_sm;
};
constexpr int kNumSpmvVariants = 8;
__host__ __device__ inline SpmvVariant spmv_variant(int id) {
    const SpmvVariant v[kNumSpmvVariants] = {{32, 256, 8}, {16, 256, 8}, {8, 256, 8},  {32, 512, 4},
                                             {16, 128, 16}, {8, 512, 4},  {4, 256, 8}, {2, 256, 8}};
    return v[(id >= 0 && id < kNumSpmvVariants) ? id : 0];
}

int sm_count();
// CTAs of `kernel` resident on one SM with `threads` threads and `smem` bytes of dynamic shared
// memory (occupancy query, cached per kernel, CTA shape and device).
int resident_ctas(const void* kernel, int threads, size_t smem);
// Grid for a grid-stride kernel: min(need, cap, one wave of resident CTAs on every SM).
unsigned resident_grid(const void* kernel, int threads, int64_t need, int64_t cap);

}  // namespace fem
