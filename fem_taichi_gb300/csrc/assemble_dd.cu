// Hex8 K / M / F assembly, double-float variant (FEM_ALGO_DD, the default).
//
// Same two-phase, atomic-free structure and the same per-element record layout as the FP64
// kernels in assemble.cu, but the element integrals and the gather sums run in double-float
// arithmetic (fem_dd.cuh) on the FP32 pipes, because FP64 throughput is the binding limit
// of these kernels on GB300.  Only the inputs are split from FP64 (node coordinates are
// first made element-local in FP64, so the ~48-bit double-float precision applies to
// element-size quantities) and only the outputs are formed in FP64 (integer assembly of
// the double nearest below hi + lo).
//
//  k_hex8_element_dd -- 8 threads per element, 16 elements per CTA, 6 CTAs per SM:
//     phase A per Gauss point (J, adjugate, det, R_a = dN_a/dxi . adj J, the scaled
//     S_a = R_a / sqrt|det|, centrifugal density), phase B per node pair (Gram
//     P_ab = sum_g sign(det_g) S_a S_b^T = sum_g R_a R_b^T / det_g -> K_ab, M_ab) and per
//     corner (F_a).  Only S lives in shared memory (29 KB per CTA); corner coordinates,
//     det and the load densities move between the 8 threads of an element by warp
//     shuffles.  Output: one 672-byte chunk per (element, corner a) -- the 8 blocks
//     K_e(a, b) with M_e(a, b) and F_e(a) -- stored at the position of (e, a) in the
//     node-to-element incidence list, so each block row's contributions are contiguous
//     and in ascending element order.
//  k_gather_dd -- one warp per 4 block rows, lane = (row, element corner): for every
//     incident element (ascending element index, the fixed order that makes the sums
//     reproducible), each of the 8 lanes of a row adds one element block into the row's
//     shared-memory accumulator at the slot given by the precomputed element-to-block map
//     (slot_map).  All lanes do useful work; a repeated corner of a degenerate element is
//     added after the first occurrence.  Rows with more than 32 blocks use a lane-per-slot
//     path.  The penalty and nodal loads are applied when the rows are written (BSR or the
//     reference CSR order, coalesced).
#include <climits>

#include "fem_common.cuh"
#include "fem_dd.cuh"

namespace fem {
namespace {

constexpr int kEpc = 16;
constexpr int kElemThreads = kEpc * 8;
constexpr int kPairStride = 10;
constexpr int kRPad = 25;
// Row-ordered contribution chunk of one (element e, corner a): the 8 blocks K_e(a, b) with
// M_e(a, b) (10 float pairs each, b = 0..7), then F_e(a) (3 pairs), padded to 84 pairs
// (672 bytes).  Chunk k of the workspace belongs to entry k of ne_list, so a block row's
// contributions are contiguous, in ascending element order.
constexpr int kChunk = 84;
constexpr int kChunkF = 80;

struct DdTables {
    float2 dnr[8][8][3];
    float2 nr[8][8];
    float2 nn[36][8];  // N_a(g) N_b(g) for pair (a <= b), Gauss point g
};

struct ElemDdParams {
    const double* xyz;
    const int4* conn4;
    const int32_t* ne_inv;
    int64_t e_begin, e_end;  // elements [e_begin, e_end) of this launch
    float2* rec;
    float2 DE, D0d, lam, mu, lm;
    float2 wc[3][3];  // f = wc . x, the centrifugal operator -w x (w x .) of UnitVectorF
    DdTables tab;
};

__device__ __forceinline__ dd ld(const float2& v) { return dd{v.x, v.y}; }
__device__ __forceinline__ float2 st(dd v) { return make_float2(v.hi, v.lo); }

// 10 float pairs (one block) as five 16-byte stores; dst is 16-byte aligned
__device__ __forceinline__ void store_block(float2* dst, const float2 (&v)[10]) {
    float4* d = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int q = 0; q < 5; ++q) d[q] = make_float4(v[2 * q].x, v[2 * q].y, v[2 * q + 1].x, v[2 * q + 1].y);
}

__device__ __forceinline__ void offdiag_pair(int q, int& a, int& b) {
    int aa = 0, rem = q;
    while (rem >= 7 - aa) {
        rem -= 7 - aa;
        ++aa;
    }
    a = aa;
    b = aa + 1 + rem;
}

struct ElemDdSmem {
    float2 dnr[8][8][3];
    float2 nr[8][8];
    float2 nn[36][8];
    float2 R[kEpc][8][kRPad];  // S_a = R_a / sqrt|det| per Gauss point
};

__device__ __forceinline__ dd shfl_dd(dd v, int src) {
    return dd{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

__global__ void __launch_bounds__(kElemThreads, 6) k_hex8_element_dd(const ElemDdParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ElemDdSmem& s = *reinterpret_cast<ElemDdSmem*>(smem_raw);
    const int tid = threadIdx.x;
    const int el = tid >> 3;
    const int t = tid & 7;
    const int base = (tid & 31) & ~7;  // lane of thread 0 of this element
    const int64_t e = p.e_begin + int64_t(blockIdx.x) * kEpc + el;
    const bool valid = e < p.e_end;

    for (int k = tid; k < 8 * 8 * 3; k += kElemThreads) (&s.dnr[0][0][0])[k] = (&p.tab.dnr[0][0][0])[k];
    for (int k = tid; k < 64; k += kElemThreads) (&s.nr[0][0])[k] = (&p.tab.nr[0][0])[k];
    for (int k = tid; k < 36 * 8; k += kElemThreads) (&s.nn[0][0])[k] = (&p.tab.nn[0][0])[k];
    dd xl[3], x0d[3];  // this thread's corner (element-local) and corner 0 (global)
    int pos = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) xl[i] = x0d[i] = dd{0.f, 0.f};
    if (valid) {
        const int* cn = reinterpret_cast<const int*>(p.conn4) + 8 * e;
        const int64_t node = __ldg(cn + t), node0 = __ldg(cn);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double x0 = __ldg(p.xyz + 3 * node0 + i);
            const double x = __ldg(p.xyz + 3 * node + i);
            xl[i] = dd_from_double(x - x0);  // element-local, exact in FP64
            x0d[i] = dd_from_double(x0);
        }
        pos = __ldg(p.ne_inv + 8 * e + t);
    }
    __syncthreads();

    // ---- phase A: Gauss point g = t (all lanes run it; lanes of absent elements see zeros) ----
    const int g = t;
    dd J[3][3];
    {
        dd_acc jacc[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) jacc[i][d] = acc_zero();
#pragma unroll 1
        for (int a = 0; a < 8; ++a) {
            dd xa[3], da[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                xa[i] = shfl_dd(xl[i], base + a);
                da[i] = ld(s.dnr[g][a][i]);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int d = 0; d < 3; ++d) acc_fma(jacc[i][d], xa[i], da[d]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) J[i][d] = acc_value(jacc[i][d]);
    }
    dd A[3][3];  // adjugate
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            dd_acc acc = acc_zero();
            acc_fma(acc, J[i1][j1], J[i2][j2]);
            acc_fma(acc, dd_neg(J[i2][j1]), J[i1][j2]);
            A[j][i] = acc_value(acc);
        }
    dd_acc da = acc_zero();
    acc_fma(da, J[0][0], A[0][0]);
    acc_fma(da, J[1][0], A[0][1]);
    acc_fma(da, J[2][0], A[0][2]);
    const dd det = acc_value(da);
    const dd isq = dd_rcp(dd_sqrt(dd_abs(det)));
#pragma unroll 1
    for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            dd_acc acc = acc_zero();
            acc_fma(acc, ld(s.dnr[g][a][0]), A[0][i]);
            acc_fma(acc, ld(s.dnr[g][a][1]), A[1][i]);
            acc_fma(acc, ld(s.dnr[g][a][2]), A[2][i]);
            s.R[el][g][3 * a + i] = st(dd_mul(acc_value(acc), isq));
        }
    dd cg[3];  // DE det f(x_g): centrifugal load density at this Gauss point
    {
        dd_acc xacc[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            xacc[i] = acc_zero();
            acc_add(xacc[i], x0d[i]);
        }
#pragma unroll 1
        for (int a = 0; a < 8; ++a) {
            const dd n = ld(s.nr[g][a]);
#pragma unroll
            for (int i = 0; i < 3; ++i) acc_fma(xacc[i], n, shfl_dd(xl[i], base + a));
        }
        dd X[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) X[i] = acc_value(xacc[i]);
        const dd jd = dd_mul(ld(p.DE), det);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            dd_acc acc = acc_zero();
#pragma unroll
            for (int j = 0; j < 3; ++j) acc_fma(acc, ld(p.wc[i][j]), X[j]);
            cg[i] = dd_mul(jd, acc_value(acc));
        }
    }
    __syncthreads();

    // ---- phase B: node pairs and corner loads -----------------------------------------------
    // block (a, b) goes to chunk pos[a] at b; its transpose (a != b) to chunk pos[b] at a
    const dd lam = ld(p.lam), mu = ld(p.mu), D0d = ld(p.D0d), DE = ld(p.DE), lm = ld(p.lm);
    {
        const int a = t, pi = pair_index(a, a);
        dd_acc P00 = acc_zero(), P11 = acc_zero(), P22 = acc_zero(), P01 = acc_zero(), P02 = acc_zero(),
               P12 = acc_zero(), m = acc_zero();
#pragma unroll 1
        for (int gg = 0; gg < 8; ++gg) {
            const dd r0 = ld(s.R[el][gg][3 * a]), r1 = ld(s.R[el][gg][3 * a + 1]), r2 = ld(s.R[el][gg][3 * a + 2]);
            const dd dg = shfl_dd(det, base + gg);
            const bool ng = dg.hi < 0.f;
            const dd q0 = ng ? dd_neg(r0) : r0, q1 = ng ? dd_neg(r1) : r1, q2 = ng ? dd_neg(r2) : r2;
            acc_fma(P00, q0, r0);
            acc_fma(P11, q1, r1);
            acc_fma(P22, q2, r2);
            acc_fma(P01, q0, r1);
            acc_fma(P02, q0, r2);
            acc_fma(P12, q1, r2);
            acc_fma(m, dg, ld(s.nn[pi][gg]));
        }
        const dd p00 = acc_value(P00), p11 = acc_value(P11), p22 = acc_value(P22);
        auto diag = [&](dd pp, dd qq, dd rr) {
            dd_acc acc = acc_zero();
            acc_fma(acc, D0d, pp);
            acc_fma(acc, mu, qq);
            acc_fma(acc, mu, rr);
            return st(acc_value(acc));
        };
        float2 o[kPairStride];
        o[0] = diag(p00, p11, p22);
        o[4] = diag(p11, p00, p22);
        o[8] = diag(p22, p00, p11);
        o[1] = o[3] = st(dd_mul(lm, acc_value(P01)));
        o[2] = o[6] = st(dd_mul(lm, acc_value(P02)));
        o[5] = o[7] = st(dd_mul(lm, acc_value(P12)));
        o[9] = st(dd_mul(DE, acc_value(m)));
        if (valid) store_block(p.rec + int64_t(pos) * kChunk + a * kPairStride, o);
    }
    // 28 off-diagonal pairs, pair t + 8 it; every lane runs 4 rounds (the shuffles need the
    // whole warp), lanes without a fourth pair compute a dummy one and store nothing
#pragma unroll 1
    for (int it = 0; it < 4; ++it) {
        const int q = t + 8 * it;
        const bool act = q < 28;
        int a, b;
        offdiag_pair(act ? q : 27, a, b);
        const int pi = pair_index(a, b);
        dd_acc P[3][3], m = acc_zero();
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) P[i][k] = acc_zero();
#pragma unroll 1
        for (int gg = 0; gg < 8; ++gg) {
            dd qa[3], rb[3];
            const dd dg = shfl_dd(det, base + gg);
            const bool ng = dg.hi < 0.f;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const dd sa = ld(s.R[el][gg][3 * a + i]);
                qa[i] = ng ? dd_neg(sa) : sa;
                rb[i] = ld(s.R[el][gg][3 * b + i]);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int k = 0; k < 3; ++k) acc_fma(P[i][k], qa[i], rb[k]);
            acc_fma(m, dg, ld(s.nn[pi][gg]));
        }
        const int pos_a = __shfl_sync(0xffffffffu, pos, base + a);
        const int pos_b = __shfl_sync(0xffffffffu, pos, base + b);
        dd Pv[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) Pv[i][k] = acc_value(P[i][k]);
        float2 kb[kPairStride];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            dd_acc acc = acc_zero();
            acc_fma(acc, D0d, Pv[i][i]);
            acc_fma(acc, mu, Pv[(i + 1) % 3][(i + 1) % 3]);
            acc_fma(acc, mu, Pv[(i + 2) % 3][(i + 2) % 3]);
            kb[4 * i] = st(acc_value(acc));
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (i == k) continue;
                dd_acc acc = acc_zero();
                acc_fma(acc, lam, Pv[i][k]);
                acc_fma(acc, mu, Pv[k][i]);
                kb[3 * i + k] = st(acc_value(acc));
            }
        kb[9] = st(dd_mul(DE, acc_value(m)));
        float2 kt[kPairStride];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) kt[3 * k + i] = kb[3 * i + k];
        kt[9] = kb[9];
        if (valid && act) {
            store_block(p.rec + int64_t(pos_a) * kChunk + b * kPairStride, kb);
            store_block(p.rec + int64_t(pos_b) * kChunk + a * kPairStride, kt);
        }
    }
    {
        dd_acc f0 = acc_zero(), f1 = acc_zero(), f2 = acc_zero();
#pragma unroll 1
        for (int gg = 0; gg < 8; ++gg) {
            const dd n = ld(s.nr[gg][t]);
            acc_fma(f0, n, shfl_dd(cg[0], base + gg));
            acc_fma(f1, n, shfl_dd(cg[1], base + gg));
            acc_fma(f2, n, shfl_dd(cg[2], base + gg));
        }
        if (valid) {
            float4* of = reinterpret_cast<float4*>(p.rec + int64_t(pos) * kChunk + kChunkF);
            const float2 v0 = st(acc_value(f0)), v1 = st(acc_value(f1)), v2 = st(acc_value(f2));
            of[0] = make_float4(v0.x, v0.y, v1.x, v1.y);
            of[1] = make_float4(v2.x, v2.y, 0.f, 0.f);
        }
    }
}

// ---- gather ---------------------------------------------------------------------------------

struct GatherDdParams {
    int64_t row_begin, row_end;  // block rows [row_begin, row_end) of this launch
    const int32_t* indptr;
    const int32_t* indices;
    const int32_t* ne_ptr;
    const uint8_t* slot_map;
    const float2* rec;  // row-ordered chunks, one per ne_list entry
    int k_layout, m_layout;
    double* K;
    double* M;
    double* F;
    const uint8_t* fixed;
    const double* loads;
};

constexpr int kGWarps = 4;
constexpr int kRowsPerWarp = 4;
constexpr int kMaxL = 32;

struct GatherDdSmem {
    float acc[kGWarps][kRowsPerWarp][kMaxL][kPairStride][2];
    int cols[kGWarps][kRowsPerWarp][kMaxL];
};

__device__ __forceinline__ int find_slot(const int* cols, int L, int node) {
    int lo = 0, hi = L - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cols[mid] < node) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// block b of chunk k as 10 raw float pairs (16-byte loads)
__device__ __forceinline__ void load_chunk_block(const float2* rec, int64_t k, int b, float4 (&v)[kPairStride / 2]) {
    const float4* blk = reinterpret_cast<const float4*>(rec + k * kChunk + b * kPairStride);
#pragma unroll
    for (int q = 0; q < kPairStride / 2; ++q) v[q] = __ldg(blk + q);
}

__device__ __forceinline__ void smem_accumulate(float (*acc)[2], const float4 (&v)[kPairStride / 2]) {
#pragma unroll
    for (int q = 0; q < kPairStride / 2; ++q) {
        const float hv[2] = {v[q].x, v[q].z}, lv[2] = {v[q].y, v[q].w};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float s, e;
            two_sum(acc[2 * q + h][0], hv[h], s, e);
            acc[2 * q + h][0] = s;
            acc[2 * q + h][1] = __fadd_rn(acc[2 * q + h][1], __fadd_rn(e, lv[h]));
        }
    }
}

__device__ __forceinline__ double smem_value(const float (*acc)[2], int k) {
    return dd_to_double(acc_value(dd_acc{acc[k][0], acc[k][1]}));
}

// Lane-per-slot path for a row of any length (rows with more than kMaxL blocks), same order
// of summation: chunk by chunk, corner by corner.
__device__ void gather_row_long(const GatherDdParams& p, int64_t row, int lane) {
    const int64_t rs = p.indptr[row];
    const int L = p.indptr[row + 1] - int(rs);
    const int ks = p.ne_ptr[row], ke = p.ne_ptr[row + 1];
    const unsigned fixed_bits = p.fixed ? p.fixed[row] : 0u;
    for (int base = 0; base < L; base += 32) {
        const int l = base + lane;
        const bool active = l < L;
        dd_acc acc[kPairStride];
#pragma unroll
        for (int q = 0; q < kPairStride; ++q) acc[q] = acc_zero();
        for (int k = ks; k < ke; ++k) {
            for (int b = 0; b < 8; ++b) {
                if (int(__ldg(p.slot_map + 8 * int64_t(k) + b)) != l) continue;
                const float2* blk = p.rec + int64_t(k) * kChunk + b * kPairStride;
#pragma unroll
                for (int q = 0; q < kPairStride; ++q) acc_add(acc[q], ld(__ldg(blk + q)));
            }
        }
        if (!active) continue;
        const bool diag = __ldg(p.indices + rs + l) == int(row);
        for (int q = 0; q < 9; ++q) {
            double val = dd_to_double(acc_value(acc[q]));
            if (diag && (q % 4 == 0) && ((fixed_bits >> (q / 4)) & 1u)) val = 1e20;
            if (p.K) {
                if (p.k_layout == FEM_LAYOUT_BSR) p.K[9 * (rs + l) + q] = val;
                else p.K[9 * rs + int64_t(3 * (q / 3)) * L + 3 * l + (q % 3)] = val;
            }
        }
        if (p.M) {
            const double mv = dd_to_double(acc_value(acc[9]));
            if (p.m_layout == FEM_LAYOUT_BSR) p.M[rs + l] = mv;
            else
                for (int pp = 0; pp < 3; ++pp) p.M[3 * rs + int64_t(pp) * L + l] = mv;
        }
    }
}

// kRanged: the launch covers rows [row_begin, row_end) (one part of a split assembly); the
// whole-mesh launch (row_begin == 0) keeps the simpler index arithmetic of kRanged == false.
template <bool kRanged>
__global__ void __launch_bounds__(kGWarps * 32) k_gather_dd(const GatherDdParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    GatherDdSmem& S = *reinterpret_cast<GatherDdSmem*>(smem_raw);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = lane >> 3, b = lane & 7;
    const int64_t row0 = (kRanged ? p.row_begin : 0) + (int64_t(blockIdx.x) * kGWarps + w) * kRowsPerWarp;
    if (row0 >= p.row_end) return;
    const int64_t row = row0 + r;
    const bool vrow = row < p.row_end;
    const int64_t rs = vrow ? p.indptr[row] : 0;
    const int L = vrow ? p.indptr[row + 1] - int(rs) : 0;
    const int ks = vrow ? p.ne_ptr[row] : 0;
    const int cnt = vrow ? p.ne_ptr[row + 1] - ks : 0;

    // ---- F for this row (lanes b < 3): corner loads in element order + nodal loads ----
    if (p.F && vrow && b < 3) {
        dd_acc f = acc_zero();
        for (int k = 0; k < cnt; ++k) acc_add(f, ld(__ldg(p.rec + int64_t(ks + k) * kChunk + kChunkF + b)));
        double fv = dd_to_double(acc_value(f));
        if (p.loads) fv += p.loads[3 * row + b];
        p.F[3 * row + b] = fv;
    }
    if (!p.K && !p.M) return;

    if (__any_sync(0xffffffffu, L > kMaxL)) {
        for (int rr = 0; rr < kRowsPerWarp; ++rr)
            if (row0 + rr < p.row_end) gather_row_long(p, row0 + rr, lane);
        return;
    }

    float* accw = &S.acc[w][0][0][0][0];
    for (int k = lane; k < kRowsPerWarp * kMaxL * kPairStride * 2; k += 32) accw[k] = 0.f;
    int* cols = S.cols[w][r];
    for (int l = b; l < kMaxL; l += 8) cols[l] = l < L ? __ldg(p.indices + rs + l) : INT_MAX;
    __syncwarp();

    int maxcnt = cnt;
#pragma unroll
    for (int off = 8; off < 32; off <<= 1) maxcnt = max(maxcnt, __shfl_xor_sync(0xffffffffu, maxcnt, off));
    // chunk k of row r: lanes (r, 0..7) read its 8 blocks (640 contiguous bytes); the next
    // chunk's blocks are in flight while the current one is added
    float4 cur[kPairStride / 2], nxt[kPairStride / 2];
    int cur_slot = 0, nxt_slot = 0;
    if (cnt > 0) {
        load_chunk_block(p.rec, ks, b, cur);
        cur_slot = __ldg(p.slot_map + 8 * int64_t(ks) + b);
    }
    for (int k = 0; k < maxcnt; ++k) {
        const bool active = k < cnt;
        if (k + 1 < cnt) {
            load_chunk_block(p.rec, ks + k + 1, b, nxt);
            nxt_slot = __ldg(p.slot_map + 8 * int64_t(ks + k + 1) + b);
        }
        // a repeated corner node (degenerate element) maps two corners to one slot:
        // the later corner is added after the earlier one
        bool dup = false;
#pragma unroll
        for (int bp = 0; bp < 7; ++bp) {
            const int other = __shfl_sync(0xffffffffu, cur_slot, (lane & ~7) | bp);
            if (bp < b && other == cur_slot) dup = true;
        }
        if (active && !dup) smem_accumulate(S.acc[w][r][cur_slot], cur);
        if (__any_sync(0xffffffffu, active && dup)) {
            for (int bb = 1; bb < 8; ++bb) {
                __syncwarp();
                if (active && dup && b == bb) smem_accumulate(S.acc[w][r][cur_slot], cur);
            }
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kPairStride / 2; ++q) cur[q] = nxt[q];
        cur_slot = nxt_slot;
    }

    // ---- write the four rows (all lanes, coalesced) ---------------------------------------------
    for (int rr = 0; rr < kRowsPerWarp; ++rr) {
        const int64_t rw = row0 + rr;
        if (rw >= p.row_end) break;
        const int64_t rrs = __shfl_sync(0xffffffffu, rs, rr * 8);
        const int LL = __shfl_sync(0xffffffffu, L, rr * 8);
        const unsigned fixed_bits = p.fixed ? p.fixed[rw] : 0u;
        const int* cc = S.cols[w][rr];
        const int sd = find_slot(cc, LL, int(rw));
        const bool has_diag = LL > 0 && cc[sd] == int(rw);
        float(*acc)[kPairStride][2] = S.acc[w][rr];
        if (p.K) {
            auto put = [&](int s_, int q9, int64_t o) {
                double val = smem_value(acc[s_], q9);
                if (has_diag && s_ == sd && (q9 % 4 == 0) && ((fixed_bits >> (q9 / 4)) & 1u)) val = 1e20;
                p.K[9 * rrs + o] = val;
            };
            if (p.k_layout == FEM_LAYOUT_BSR) {
                for (int o = lane; o < 9 * LL; o += 32) {
                    const int s_ = o / 9;
                    put(s_, o - 9 * s_, o);
                }
            } else {
                for (int pp = 0; pp < 3; ++pp)
                    for (int idx = lane; idx < 3 * LL; idx += 32) {
                        const int s_ = idx / 3;
                        put(s_, 3 * pp + (idx - 3 * s_), int64_t(3 * LL) * pp + idx);
                    }
            }
        }
        if (p.M) {
            if (p.m_layout == FEM_LAYOUT_BSR) {
                for (int o = lane; o < LL; o += 32) p.M[rrs + o] = smem_value(acc[o], 9);
            } else {
                for (int o = lane; o < LL; o += 32) {
                    const double mv = smem_value(acc[o], 9);
                    p.M[3 * rrs + o] = mv;
                    p.M[3 * rrs + LL + o] = mv;
                    p.M[3 * rrs + 2 * LL + o] = mv;
                }
            }
        }
    }
}

void split_host(double x, float2& out) {
    const float hi = float(x);
    out = make_float2(hi, float(x - double(hi)));
}

}  // namespace

int launch_hex8_element_dd(const fem_mesh* mesh, const fem_material* mat, void* workspace, cudaStream_t st,
                           int64_t e_begin, int64_t e_end) {
    if (e_end <= e_begin) return FEM_OK;
    ElemDdParams ep;
    ep.xyz = mesh->xyz;
    ep.conn4 = reinterpret_cast<const int4*>(mesh->conn);
    ep.ne_inv = mesh->ne_inv;
    ep.e_begin = e_begin;
    ep.e_end = e_end;
    ep.rec = static_cast<float2*>(workspace);
    const double EX = mat->EX, PO = mat->PO;
    const double D0d = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO);  // FEM_model_bsr.py:435-437
    const double lam = EX * PO / (1 + PO) / (1 - 2 * PO);         // :439-445
    const double mu = EX / 2 / (1 + PO);                          // :447-449
    split_host(mat->DE, ep.DE);
    split_host(D0d, ep.D0d);
    split_host(lam, ep.lam);
    split_host(mu, ep.mu);
    split_host(lam + mu, ep.lm);
    const double w0 = mat->omega[0], w1 = mat->omega[1], w2 = mat->omega[2];
    const double wc[3][3] = {{w1 * w1 + w2 * w2, -w0 * w1, -w0 * w2},   // UnitVectorF, FEM_model_bsr.py:291-300
                             {-w1 * w0, w0 * w0 + w2 * w2, -w1 * w2},
                             {-w2 * w0, -w2 * w1, w1 * w1 + w0 * w0}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) split_host(wc[i][j], ep.wc[i][j]);
    const ShapeTables& T = shape_tables();
    for (int g = 0; g < 8; ++g)
        for (int a = 0; a < 8; ++a) {
            split_host(T.nr[g][a], ep.tab.nr[g][a]);
            for (int d = 0; d < 3; ++d) split_host(T.dnr[g][a][d], ep.tab.dnr[g][a][d]);
        }
    for (int a = 0; a < 8; ++a)
        for (int b2 = a; b2 < 8; ++b2)
            for (int g = 0; g < 8; ++g) split_host(T.nr[g][a] * T.nr[g][b2], ep.tab.nn[pair_index(a, b2)][g]);
    const size_t smem = sizeof(ElemDdSmem);
    FEM_CUDA(cudaFuncSetAttribute(k_hex8_element_dd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t blocks = (e_end - e_begin + kEpc - 1) / kEpc;
    k_hex8_element_dd<<<unsigned(blocks), kElemThreads, smem, st>>>(ep);
    FEM_LAUNCH_CHECK("k_hex8_element_dd");
    return FEM_OK;
}

int launch_gather_dd(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace, cudaStream_t st,
                     int64_t row_begin, int64_t row_end) {
    if (row_end <= row_begin) return FEM_OK;
    GatherDdParams gp;
    gp.row_begin = row_begin;
    gp.row_end = row_end;
    gp.indptr = mesh->indptr;
    gp.indices = mesh->indices;
    gp.ne_ptr = mesh->ne_ptr;
    gp.slot_map = mesh->slot_map;
    gp.rec = static_cast<const float2*>(workspace);
    gp.k_layout = out->k_layout;
    gp.m_layout = out->m_layout;
    gp.K = out->K;
    gp.M = out->M;
    gp.F = out->F;
    gp.fixed = out->fixed;
    gp.loads = out->loads;
    const size_t smem = sizeof(GatherDdSmem);
    const int64_t rows_per_cta = int64_t(kGWarps) * kRowsPerWarp;
    const int64_t blocks = (row_end - row_begin + rows_per_cta - 1) / rows_per_cta;
    if (row_begin == 0) {
        FEM_CUDA(cudaFuncSetAttribute(k_gather_dd<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        k_gather_dd<false><<<unsigned(blocks), kGWarps * 32, smem, st>>>(gp);
    } else {
        FEM_CUDA(cudaFuncSetAttribute(k_gather_dd<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        k_gather_dd<true><<<unsigned(blocks), kGWarps * 32, smem, st>>>(gp);
    }
    FEM_LAUNCH_CHECK("k_gather_dd");
    return FEM_OK;
}

}  // namespace fem
