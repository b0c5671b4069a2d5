// Hex8 K / M / F assembly for sm_103a.
//
// Two kernels, both deterministic and free of floating-point atomics:
//
//  1. k_hex8_element -- 8 threads per element.  Thread t first forms coefficient t of the
//     element's trilinear map x(xi) = sum_k c_k m_k(xi) (m = 1, xi, eta, zeta, xi eta,
//     eta zeta, xi zeta, xi eta zeta; c_k = 1/8 sum_a m_k(corner a) x_a) and W x_t, where W is
//     the centrifugal operator of UnitVectorF (FEM_model_bsr.py:291-300).  Phase A: thread g
//     handles Gauss point g (Jacobian from the coefficients, 27 FMA instead of 72; adjugate,
//     determinant, the 8 scaled gradients R_a = dN_a/dxi . adj(J)); results are staged in
//     shared memory.  Phase B: the 36 node pairs (a <= b) are split across the 8 threads;
//     each accumulates the Gram matrix P_ab = sum_g R_a R_b^T / det_g and turns it into the
//     3x3 stiffness block  K_ab[p][q] = lam P[p][q] + mu P[q][p],
//     K_ab[p][p] = D0d P[p][p] + mu (tr P - P[p][p]), which equals sum_g det (B1_a^T D0 B1_b +
//     B2_a^T D1 B2_b) of the reference (FEM_model_bsr.py:262-274, 303-347) with a different
//     summation order.  The consistent mass M_ab = DE sum_g det_g N_a N_b
//     (FEM_model_bsr.py:276-287) is sum-factorised: N_a(g) is a product of one 1D factor per
//     axis, so M_ab depends only on the per-axis class of (a, b) and the 8 det_g are contracted
//     axis by axis (27 classes, 141 FP64 operations per element instead of 288).  The centrifugal
//     load (FEM_model_bsr.py:229-245) is F_a = sum_g DE det_g N_a(g) W x(g); W x is linear and
//     the isoparametric map reproduces it at the Gauss points, W x(g) = sum_b N_b(g) W x_b, so
//     F_a = sum_b M_ab W x_b: the same quantity from the mass blocks, with no per-Gauss-point
//     load density.  Each element writes one 2,944-byte record: 28 off-diagonal pairs as
//     K (3x3) + M, 8 diagonal pairs as the 6 distinct values of the symmetric K + M (8-double
//     slots), 8 x F(3).
//
//  2. k_gather -- one warp per block row i.  Lane l owns slot l of the row (column node
//     indices[indptr[i] + l]).  The warp walks the incident (element, corner) list of
//     node i in ascending element order, and each lane adds the element block whose
//     column corner matches its column node.  The fixed order makes the sums
//     reproducible bit for bit.  The penalty (FEM_model_bsr.py:248-259) and nodal loads
//     (LoadF, :220-226) are applied in the same pass, and the row is written in either
//     the BSR block order or the reference's scalar-CSR order (FEM_model_csr.py:150-173).
#include <climits>
#include <vector>

#include "fem_common.cuh"

namespace fem {
namespace {

constexpr int kEpc = 16;                 // elements per CTA in the element kernel
constexpr int kElemThreads = kEpc * 8;   // 8 threads per element
// Element record (FP64 kernels), 368 doubles = 2,944 bytes: for each corner a in turn, the
// diagonal pair (a, a) as the 6 distinct values of the symmetric K_aa (00, 11, 22, 01, 02, 12)
// + M_aa in an 8-double slot, then the pairs (a, b), b = a + 1..7, as K_ab (3x3) + M_ab; then
// F (8 x 3).  The blocks the 8 lanes of a row read for one incident entry, (a, a..7), stay
// contiguous; every block starts on a 16-byte boundary.
constexpr int kPairStride = 10;   // K (9) + M (1) of an off-diagonal pair
constexpr int kDiagStride = 8;    // K_aa (6) + M_aa + 1 unused
constexpr int kFOff = 8 * kDiagStride + 28 * kPairStride;  // 344: F block offset within a record
constexpr int kRec = kFOff + 24;  // 368 doubles per element record
constexpr int kRPad = 25;         // padded row (24 used) to spread smem banks

// record offset of pair (lo, hi), lo <= hi: 10 doubles per pair in upper-triangular order, less
// 2 for every diagonal slot before it
__host__ __device__ constexpr int pair_offset(int lo, int hi) {
    return kPairStride * (lo * 8 - (lo * (lo - 1)) / 2 + (hi - lo)) - 2 * (lo + (hi > lo ? 1 : 0));
}

struct ElemParams {
    const double* xyz;
    const int4* conn4;
    int64_t e_begin, e_end;  // elements [e_begin, e_end) of this launch
    double* rec;
    double DE, D0d, lam, mu;
    double wc[3][3];   // centrifugal operator: f = wc . x (UnitVectorF)
    DevTables tab;
    // tm[s][c]: product of the 1D shape factors of two corners along one axis at a Gauss point
    // on the negative (s = 0) or positive (s = 1) side: c = 0 both corners negative, 1 mixed,
    // 2 both positive
    double tm[2][3];
};

struct ElemSmem {
    double dnr[8][kRPad];       // dN_a/dxi_i at Gauss point g at [g][3a+i]; padded row: the 8 rows
                                // start in 8 different bank pairs (a 24-double row put every
                                // even g in one bank and every odd g in another)
    double x[kEpc][8][3];       // corner coordinates; later the first mass contraction (D1)
    double xl[kEpc][8][3];      // corner coordinates relative to corner 0; later D2
    double cf[kEpc][8][3];      // trilinear coefficients c_k of the element map (c_0 unused)
    double wx[kEpc][8][3];      // W x_a: centrifugal density per unit mass at corner a
    double R[kEpc][8][kRPad];   // R_a(g)[i] at [el][g][3a+i]
    double Rs[kEpc][8][kRPad];  // R_a(g)[i] / det_g
    double det[kEpc][8];
    double m[kEpc][36];         // mass by corner-pair class (27 used, DE included), see mass_class
};

// Class of the corner pair (a, b) for the mass: per axis 0 both corners on the negative side,
// 1 mixed, 2 both positive (corner sides as in monomial_sign); M_ab depends only on it.
__device__ __forceinline__ int mass_class(int a, int b) {
    const int nx = (0x66 >> a) & 1, ny = (0xCC >> a) & 1, nz = (0x0F >> a) & 1;
    const int mx = (0x66 >> b) & 1, my = (0xCC >> b) & 1, mz = (0x0F >> b) & 1;
    const int cx = nx != mx ? 1 : (nx ? 0 : 2), cy = ny != my ? 1 : (ny ? 0 : 2), cz = nz != mz ? 1 : (nz ? 0 : 2);
    return cx * 9 + cy * 3 + cz;
}

// m_k(corner a) for the trilinear monomials 1, xi, eta, zeta, xi eta, eta zeta, xi zeta,
// xi eta zeta; corner signs in the reference's node order (FEM_model_bsr.py:371-382):
// xi < 0 at corners 1, 2, 5, 6 (mask 0x66), eta < 0 at 2, 3, 6, 7 (0xCC), zeta < 0 at 0-3
// (0x0F); monomial k contains xi for k in {1, 4, 6, 7} (0xD2), eta for {2, 4, 5, 7} (0xB4),
// zeta for {3, 5, 6, 7} (0xE8).
__device__ __forceinline__ double monomial_sign(int k, int a) {
    const int neg = (((0xD2 >> k) & (0x66 >> a)) ^ ((0xB4 >> k) & (0xCC >> a)) ^ ((0xE8 >> k) & (0x0F >> a))) & 1;
    return neg ? -1.0 : 1.0;
}

// Off-diagonal pair list (a < b), 28 entries; thread t takes entries t, t+8, t+16, t+24.
__device__ __forceinline__ void offdiag_pair(int q, int& a, int& b) {
    // q -> (a, b) for row-major enumeration of a < b
    int aa = 0, rem = q;
    while (rem >= 7 - aa) {
        rem -= 7 - aa;
        ++aa;
    }
    a = aa;
    b = aa + 1 + rem;
}

__global__ void __launch_bounds__(kElemThreads, 3) k_hex8_element(const ElemParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ElemSmem& s = *reinterpret_cast<ElemSmem*>(smem_raw);
    const int tid = threadIdx.x;
    const int el = tid >> 3;
    const int t = tid & 7;
    const int64_t e = p.e_begin + int64_t(blockIdx.x) * kEpc + el;
    const bool valid = e < p.e_end;

    for (int k = tid; k < 8 * 8 * 3; k += kElemThreads) s.dnr[k / 24][k % 24] = (&p.tab.dnr[0][0][0])[k];
    if (valid) {
        const int* cn = reinterpret_cast<const int*>(p.conn4) + 8 * e;
        const int node = __ldg(cn + t);
        s.x[el][t][0] = __ldg(p.xyz + 3 * int64_t(node) + 0);
        s.x[el][t][1] = __ldg(p.xyz + 3 * int64_t(node) + 1);
        s.x[el][t][2] = __ldg(p.xyz + 3 * int64_t(node) + 2);
    }
    __syncthreads();

    // ---- coefficient t of the trilinear map, and W x_t ---------------------------------
    if (valid) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.wx[el][t][i] = p.wc[i][0] * s.x[el][t][0] + p.wc[i][1] * s.x[el][t][1] + p.wc[i][2] * s.x[el][t][2];
            s.xl[el][t][i] = s.x[el][t][i] - s.x[el][0][i];   // element-local: no offset to cancel
        }
    }
    __syncthreads();
    if (valid) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double acc = 0.0;
#pragma unroll
            for (int a = 1; a < 8; ++a) acc = fma(monomial_sign(t, a), s.xl[el][a][i], acc);
            s.cf[el][t][i] = 0.125 * acc;
        }
    }
    __syncthreads();

    // ---- phase A: Gauss point g = t ------------------------------------------------
    if (valid) {
        const int g = t;
        // Gauss point coordinates in the reference's order (zeta fastest, FEM_model_bsr.py:425-432)
        const double xi = (g & 4) ? kGS1 : -kGS1, et = (g & 2) ? kGS1 : -kGS1, ze = (g & 1) ? kGS1 : -kGS1;
        double J[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const double c1 = s.cf[el][1][i], c2 = s.cf[el][2][i], c3 = s.cf[el][3][i], c4 = s.cf[el][4][i];
            const double c5 = s.cf[el][5][i], c6 = s.cf[el][6][i], c7 = s.cf[el][7][i];
            J[i][0] = fma(ze, fma(et, c7, c6), fma(et, c4, c1));   // dx/dxi
            J[i][1] = fma(ze, fma(xi, c7, c5), fma(xi, c4, c2));   // dx/deta
            J[i][2] = fma(et, fma(xi, c7, c5), fma(xi, c6, c3));   // dx/dzeta
        }
        double A[3][3];  // adjugate: inverse(J) = A / det
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
                A[j][i] = J[i1][j1] * J[i2][j2] - J[i2][j1] * J[i1][j2];
            }
        const double det = J[0][0] * A[0][0] + J[1][0] * A[0][1] + J[2][0] * A[0][2];
        const double inv = 1.0 / det;
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const double r =
                    s.dnr[g][3 * a] * A[0][i] + s.dnr[g][3 * a + 1] * A[1][i] + s.dnr[g][3 * a + 2] * A[2][i];
                s.R[el][g][3 * a + i] = r;
                s.Rs[el][g][3 * a + i] = r * inv;
            }
        s.det[el][g] = det;
    }
    __syncthreads();

    // ---- mass, M_ab = DE sum_g det_g N_a(g) N_b(g), by sum factorisation ------------------
    // N_a(g) is a product of one 1D factor per axis, so M_ab depends on the class of (a, b) per
    // axis only: contract the 8 det_g along x (D1: 3 classes x 4 (y, z) points), y (D2: 9 x 2),
    // z (D3: 27 classes), 141 FP64 operations instead of 36 pairs x 8 Gauss points.
    {
        double* D1 = &s.x[el][0][0];
        double* D2 = &s.xl[el][0][0];
        double* D3 = &s.m[el][0];
        if (valid)
            for (int i = t; i < 12; i += 8) {
                const int c = i >> 2, gyz = i & 3;
                D1[i] = fma(s.det[el][4 + gyz], p.tm[1][c], s.det[el][gyz] * p.tm[0][c]);
            }
        __syncthreads();
        if (valid)
            for (int i = t; i < 18; i += 8) {
                const int cx = i / 6, r = i - 6 * cx, cy = r >> 1, gz = r & 1;
                D2[i] = fma(D1[cx * 4 + 2 + gz], p.tm[1][cy], D1[cx * 4 + gz] * p.tm[0][cy]);
            }
        __syncthreads();
        if (valid)
            for (int i = t; i < 27; i += 8) {
                const int cxy = i / 3, cz = i - 3 * cxy;
                D3[i] = p.DE * fma(D2[cxy * 2 + 1], p.tm[1][cz], D2[cxy * 2] * p.tm[0][cz]);
            }
        __syncthreads();
    }

    // ---- phase B: node pairs -----------------------------------------------------------
    double* rec = p.rec + (valid ? e : 0) * kRec;
    const double lam = p.lam, mu = p.mu, D0d = p.D0d;
    // diagonal pair (t, t): P symmetric
    if (valid) {
        const int a = t, pi = pair_index(a, a);
        double P00 = 0, P11 = 0, P22 = 0, P01 = 0, P02 = 0, P12 = 0;
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const double r0 = s.R[el][g][3 * a], r1 = s.R[el][g][3 * a + 1], r2 = s.R[el][g][3 * a + 2];
            const double q0 = s.Rs[el][g][3 * a], q1 = s.Rs[el][g][3 * a + 1], q2 = s.Rs[el][g][3 * a + 2];
            P00 = fma(q0, r0, P00);
            P11 = fma(q1, r1, P11);
            P22 = fma(q2, r2, P22);
            P01 = fma(q0, r1, P01);
            P02 = fma(q0, r2, P02);
            P12 = fma(q1, r2, P12);
        }
        const double lm = lam + mu;
        double* o = rec + kPairStride * pi - 2 * a;  // pair_offset(a, a)
        o[0] = D0d * P00 + mu * (P11 + P22);
        o[1] = D0d * P11 + mu * (P00 + P22);
        o[2] = D0d * P22 + mu * (P00 + P11);
        o[3] = lm * P01;
        o[4] = lm * P02;
        o[5] = lm * P12;
        o[6] = s.m[el][mass_class(a, a)];
        o[7] = 0.0;  // the unused slot: whole 32-byte sectors written, none read back from DRAM
    }
    // off-diagonal pairs
    for (int q = t; q < 28 && valid; q += 8) {
        int a, b;
        offdiag_pair(q, a, b);
        const int pi = pair_index(a, b);
        double P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
        for (int g = 0; g < 8; ++g) {
            const double q0 = s.Rs[el][g][3 * a], q1 = s.Rs[el][g][3 * a + 1], q2 = s.Rs[el][g][3 * a + 2];
            const double r0 = s.R[el][g][3 * b], r1 = s.R[el][g][3 * b + 1], r2 = s.R[el][g][3 * b + 2];
            P[0][0] = fma(q0, r0, P[0][0]);
            P[0][1] = fma(q0, r1, P[0][1]);
            P[0][2] = fma(q0, r2, P[0][2]);
            P[1][0] = fma(q1, r0, P[1][0]);
            P[1][1] = fma(q1, r1, P[1][1]);
            P[1][2] = fma(q1, r2, P[1][2]);
            P[2][0] = fma(q2, r0, P[2][0]);
            P[2][1] = fma(q2, r1, P[2][1]);
            P[2][2] = fma(q2, r2, P[2][2]);
        }
        double* o = rec + kPairStride * pi - 2 * (a + 1);  // pair_offset(a, b), a < b
        o[0] = D0d * P[0][0] + mu * (P[1][1] + P[2][2]);
        o[4] = D0d * P[1][1] + mu * (P[0][0] + P[2][2]);
        o[8] = D0d * P[2][2] + mu * (P[0][0] + P[1][1]);
        o[1] = lam * P[0][1] + mu * P[1][0];
        o[2] = lam * P[0][2] + mu * P[2][0];
        o[3] = lam * P[1][0] + mu * P[0][1];
        o[5] = lam * P[1][2] + mu * P[2][1];
        o[6] = lam * P[2][0] + mu * P[0][2];
        o[7] = lam * P[2][1] + mu * P[1][2];
        o[9] = s.m[el][mass_class(a, b)];
    }
    // element load for corner t: F_t = sum_b M_tb W x_b (the mass blocks of the other threads'
    // pairs come through shared memory)
    __syncthreads();
    if (valid) {
        double f0 = 0, f1 = 0, f2 = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            const double mv = s.m[el][mass_class(t, b)];
            f0 = fma(mv, s.wx[el][b][0], f0);
            f1 = fma(mv, s.wx[el][b][1], f1);
            f2 = fma(mv, s.wx[el][b][2], f2);
        }
        rec[kFOff + 3 * t + 0] = f0;
        rec[kFOff + 3 * t + 1] = f1;
        rec[kFOff + 3 * t + 2] = f2;
    }
}

// Block (a, b) of element e as 10 doubles (K row-major, then M), oriented for row corner a and
// column corner b: an off-diagonal pair is stored once (a < b) and transposed for a > b; a
// diagonal pair is stored as its 6 distinct values.  Every lane issues the same five 16-byte
// loads (a diagonal slot's last two land in the next block or in F and go unused) and picks
// its values with selects, so the lanes of a row do not diverge.
__device__ __forceinline__ void load_pair_block(const double* rec, int64_t e, int a, int b, double (&v)[kPairStride]) {
    const bool dg = a == b, tr = a > b;
    const int lo = min(a, b), hi = max(a, b);
    const double2* blk = reinterpret_cast<const double2*>(rec + e * kRec + pair_offset(lo, hi));
    double w[kPairStride];
#pragma unroll
    for (int q = 0; q < kPairStride / 2; ++q) {
        const double2 x = __ldg(blk + q);
        w[2 * q] = x.x;
        w[2 * q + 1] = x.y;
    }
    v[0] = w[0];
    v[1] = dg ? w[3] : (tr ? w[3] : w[1]);
    v[2] = dg ? w[4] : (tr ? w[6] : w[2]);
    v[3] = dg ? w[3] : (tr ? w[1] : w[3]);
    v[4] = dg ? w[1] : w[4];
    v[5] = dg ? w[5] : (tr ? w[7] : w[5]);
    v[6] = dg ? w[4] : (tr ? w[2] : w[6]);
    v[7] = dg ? w[5] : (tr ? w[5] : w[7]);
    v[8] = dg ? w[2] : w[8];
    v[9] = dg ? w[6] : w[9];
}

struct GatherParams {
    int64_t n_node;
    const int32_t* indptr;
    const int32_t* indices;
    const int32_t* ne_ptr;
    const int32_t* ne_list;
    const int4* conn4;
    const double* rec;
    int k_layout, m_layout;
    double* K;
    double* M;
    double* F;
    const uint8_t* fixed;
    const double* loads;
};

__device__ __forceinline__ unsigned corner_match(int col, const int4& c0, const int4& c1) {
    return unsigned(c0.x == col) | (unsigned(c0.y == col) << 1) | (unsigned(c0.z == col) << 2) |
           (unsigned(c0.w == col) << 3) | (unsigned(c1.x == col) << 4) | (unsigned(c1.y == col) << 5) |
           (unsigned(c1.z == col) << 6) | (unsigned(c1.w == col) << 7);
}

__global__ void __launch_bounds__(256) k_gather(const GatherParams p) {
    const int64_t row = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= p.n_node) return;
    const int64_t rs = p.indptr[row];
    const int L = p.indptr[row + 1] - int(rs);
    const int ks = p.ne_ptr[row], ke = p.ne_ptr[row + 1];
    const unsigned fixed_bits = p.fixed ? p.fixed[row] : 0u;

    for (int base = 0; base < L; base += 32) {
        const int l = base + lane;
        const bool active = l < L;
        const int col = active ? __ldg(p.indices + rs + l) : -1;
        double acc[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] = 0.0;
        double accm = 0.0;
        for (int k = ks; k < ke; ++k) {
            const int ent = __ldg(p.ne_list + k);
            const int64_t e = ent >> 3;
            const int a = ent & 7;
            const int4 c0 = __ldg(p.conn4 + 2 * e), c1 = __ldg(p.conn4 + 2 * e + 1);
            unsigned mask = corner_match(col, c0, c1);
            while (mask) {
                const int b = __ffs(mask) - 1;
                mask &= mask - 1;
                double v[kPairStride];
                load_pair_block(p.rec, e, a, b, v);
#pragma unroll
                for (int k = 0; k < 9; ++k) acc[k] += v[k];
                accm += v[9];
            }
        }
        if (col == int(row)) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if ((fixed_bits >> d) & 1u) acc[4 * d] = 1e20;
        }
        if (active) {
            if (p.K) {
                if (p.k_layout == FEM_LAYOUT_BSR) {
                    double* o = p.K + 9 * (rs + l);
#pragma unroll
                    for (int k = 0; k < 9; ++k) o[k] = acc[k];
                } else {
#pragma unroll
                    for (int pp = 0; pp < 3; ++pp) {
                        double* o = p.K + 9 * rs + int64_t(3 * pp) * L + 3 * l;
                        o[0] = acc[3 * pp];
                        o[1] = acc[3 * pp + 1];
                        o[2] = acc[3 * pp + 2];
                    }
                }
            }
            if (p.M) {
                if (p.m_layout == FEM_LAYOUT_BSR) {
                    p.M[rs + l] = accm;
                } else {
#pragma unroll
                    for (int pp = 0; pp < 3; ++pp) p.M[3 * rs + int64_t(pp) * L + l] = accm;
                }
            }
        }
    }
    if (p.F && lane < 3) {
        double f = 0.0;
        for (int k = ks; k < ke; ++k) {
            const int ent = __ldg(p.ne_list + k);
            f += __ldg(p.rec + int64_t(ent >> 3) * kRec + kFOff + 3 * (ent & 7) + lane);
        }
        if (p.loads) f += p.loads[3 * row + lane];
        p.F[3 * row + lane] = f;
    }
}

// ---- FP64 gather, lane = (row, element corner) -------------------------------------------------
//
// One warp per 4 block rows; lane (r, b) handles corner b of every element incident to row r.
// For incident entry k (ascending element index) it reads the element block of the pair
// (a, b) -- a = the row's corner in that element -- from the element record (transposed when
// a > b) and adds it into the row's shared-memory accumulator at the slot given by the
// element-to-block map (slot_map).  All 8 lanes of a row do useful FP64 work on every entry.
// The first contribution to a slot is stored instead of added (a per-row bit mask of the
// slots already holding a value), which saves the ~27 of ~64 block additions per interior
// row that would add into zero.  A repeated corner node of a degenerate element adds after
// the earlier corner.  The summation order (element by element, corners ascending) is fixed,
// so results are bitwise reproducible.  Rows with more than kG64MaxL blocks use the
// lane-per-slot path (same order).
constexpr int kG64Warps = 4;
constexpr int kG64Rows = 4;
// 27 slots: every row of a structured hex mesh (3 x 3 x 3 neighbour nodes).  A row's
// accumulator holds 29 positions of 10 doubles (2,320 bytes; 16 rows per CTA take 36 KB, so 6
// CTAs (24 warps) fit on an SM).  A row of 27 slots places slot s at kPos27(s): each element's 8
// corners hit a 2 x 2 x 2 sub-cube of the 3 x 3 x 3 neighbourhood, and the table gives the 8
// slots of every such sub-cube distinct positions mod 8, so the 16-byte accesses of a row's 8
// lanes fall in 8 different bank groups (in slot order, slots 8 apart collided).  No placement
// in 27 positions does that (the centre slot lies in all 8 sub-cubes, so its residue can hold
// nothing else); the table uses 29.  Other rows keep position = slot.  Any one-to-one placement
// gives the same sums; the table only removes bank conflicts.
constexpr int kG64MaxL = 27;
constexpr int kG64Pos = 29;
constexpr int kG64RowStride = kG64Pos * kPairStride;

// Position of slot s (0..26) in a row of 27 slots: 5 bits per slot, 12 slots per word.  The
// classes of equal position mod 8: {the 4 centres of the x edges}, 4 x {a face centre, the
// edge centre and 2 corners that complete its exact cover of the 8 sub-cubes}, 2 x {a z face
// centre, 2 edge centres}, {the centre}.
__device__ __forceinline__ int pos27(int s) {
    const unsigned long long w = s < 12 ? 0x048d9144ec575012ull : (s < 24 ? 0x0a99bc86964508e1ull : 0x671bull);
    return int((w >> (5 * (s - 12 * (s / 12)))) & 31ull);
}

struct Gather64Params {
    int64_t row_begin, row_end;  // block rows [row_begin, row_end) of this launch
    const int32_t* indptr;
    const int32_t* indices;
    const int32_t* ne_ptr;
    const int32_t* ne_list;
    const uint8_t* slot_map;
    int slot_map_aligned;  // slot_map on an 8-byte boundary: one 8-byte load per entry
    const int4* conn4;
    const double* rec;
    int k_layout, m_layout;
    double* K;
    double* M;
    double* F;
    const uint8_t* fixed;
    const double* loads;
};

struct Gather64Smem {
    double acc[kG64Warps][kG64Rows][kG64RowStride];
};

// Lane-per-slot path for one row of any length (K and M; F is summed by the caller).
__device__ void gather_row_long64(const Gather64Params& p, int64_t row, int lane) {
    const int64_t rs = p.indptr[row];
    const int L = p.indptr[row + 1] - int(rs);
    const int ks = p.ne_ptr[row], ke = p.ne_ptr[row + 1];
    const unsigned fixed_bits = p.fixed ? p.fixed[row] : 0u;
    for (int base = 0; base < L; base += 32) {
        const int l = base + lane;
        const bool active = l < L;
        double acc[kPairStride];
#pragma unroll
        for (int q = 0; q < kPairStride; ++q) acc[q] = 0.0;
        bool any = false;
        for (int k = ks; k < ke; ++k) {
            const int ent = __ldg(p.ne_list + k);
            for (int b = 0; b < 8; ++b) {
                if (int(__ldg(p.slot_map + 8 * int64_t(k) + b)) != l) continue;
                double v[kPairStride];
                load_pair_block(p.rec, ent >> 3, ent & 7, b, v);
#pragma unroll
                for (int q = 0; q < kPairStride; ++q) acc[q] = any ? acc[q] + v[q] : v[q];
                any = true;
            }
        }
        if (!active) continue;
        const bool diag = __ldg(p.indices + rs + l) == int(row);
        if (diag) {
#pragma unroll
            for (int d = 0; d < 3; ++d)
                if ((fixed_bits >> d) & 1u) acc[4 * d] = 1e20;
        }
        if (p.K) {
            if (p.k_layout == FEM_LAYOUT_BSR) {
#pragma unroll
                for (int q = 0; q < 9; ++q) p.K[9 * (rs + l) + q] = acc[q];
            } else {
#pragma unroll
                for (int q = 0; q < 9; ++q) p.K[9 * rs + int64_t(3 * (q / 3)) * L + 3 * l + (q % 3)] = acc[q];
            }
        }
        if (p.M) {
            if (p.m_layout == FEM_LAYOUT_BSR) p.M[rs + l] = acc[9];
            else
                for (int pp = 0; pp < 3; ++pp) p.M[3 * rs + int64_t(pp) * L + l] = acc[9];
        }
    }
}

__global__ void __launch_bounds__(kG64Warps * 32, 6) k_gather64(const Gather64Params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Gather64Smem& S = *reinterpret_cast<Gather64Smem*>(smem_raw);
    const unsigned full = 0xffffffffu;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = lane >> 3, b = lane & 7;
    const int64_t row0 = p.row_begin + (int64_t(blockIdx.x) * kG64Warps + w) * kG64Rows;
    if (row0 >= p.row_end) return;  // uniform per warp
    const int64_t row = row0 + r;
    const bool vrow = row < p.row_end;
    const int64_t rs = vrow ? p.indptr[row] : 0;
    const int L = vrow ? p.indptr[row + 1] - int(rs) : 0;
    const int ks = vrow ? p.ne_ptr[row] : 0;
    const int cnt = vrow ? p.ne_ptr[row + 1] - ks : 0;

    // F of this row on lanes b < 3 (corner loads in element order, then the nodal loads) for
    // the warps that leave before the main path
    auto row_F = [&]() {
        if (p.F && vrow && b < 3) {
            double f = 0.0;
            for (int k = 0; k < cnt; ++k) {
                const int ent = __ldg(p.ne_list + ks + k);
                f += __ldg(p.rec + int64_t(ent >> 3) * kRec + kFOff + 3 * (ent & 7) + b);
            }
            if (p.loads) f += p.loads[3 * row + b];
            p.F[3 * row + b] = f;
        }
    };
    if (!p.K && !p.M) {
        row_F();
        return;
    }
    if (__any_sync(full, L > kG64MaxL)) {
        row_F();
        for (int rr = 0; rr < kG64Rows; ++rr)
            if (row0 + rr < p.row_end) gather_row_long64(p, row0 + rr, lane);
        return;
    }

    // the row's diagonal slot (-1 if the node is not its own neighbour), found by the 8 lanes
    int diag = -1;
    for (int l = b; l < L; l += 8)
        if (__ldg(p.indices + rs + l) == int(row)) diag = l;
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) diag = max(diag, __shfl_xor_sync(full, diag, off));
    const bool full27 = L == kG64MaxL;
    double* accr = S.acc[w][r];

    int maxcnt = cnt;
#pragma unroll
    for (int off = 8; off < 32; off <<= 1) maxcnt = max(maxcnt, __shfl_xor_sync(full, maxcnt, off));

    // The row's incident entries, 8 at a time: lane (r, j) holds entry 8c + j of chunk c (its
    // ne_list value and its 8 slot_map bytes), and every lane of the row takes entry k from
    // lane (r, k mod 8) by a shuffle, so the element block loads of entry k + 1 issue without
    // first waiting for a load of ne_list.
    const int src = lane & ~7;
    int ent_reg = 0;
    unsigned long long sm_reg = 0ull;
    auto load_chunk = [&](int c) {
        const int j = 8 * c + b;
        ent_reg = j < cnt ? __ldg(p.ne_list + ks + j) : 0;
        if (j < cnt) {
            if (p.slot_map_aligned) {
                sm_reg = __ldg(reinterpret_cast<const unsigned long long*>(p.slot_map) + (ks + j));
            } else {
                sm_reg = 0ull;
                for (int q = 0; q < 8; ++q)
                    sm_reg |= (unsigned long long)__ldg(p.slot_map + 8 * int64_t(ks + j) + q) << (8 * q);
            }
        }
    };
    load_chunk(0);
    // F of this row on lanes b < 3: corner loads in element order, then the nodal loads
    if (p.F) {
        double f = 0.0;
        for (int k = 0; k < maxcnt; ++k) {
            if (k > 0 && (k & 7) == 0) load_chunk(k >> 3);
            const int ent = __shfl_sync(full, ent_reg, src | (k & 7));
            if (b < 3 && k < cnt) f += __ldg(p.rec + int64_t(ent >> 3) * kRec + kFOff + 3 * (ent & 7) + b);
        }
        if (maxcnt > 8) load_chunk(0);
        if (b < 3 && vrow) {
            if (p.loads) f += p.loads[3 * row + b];
            p.F[3 * row + b] = f;
        }
    }
    unsigned touched = 0;  // slots of row r holding a value (the same in the row's 8 lanes)
    double cur[kPairStride], nxt[kPairStride];
    int cur_slot = 0, nxt_slot = 0;
    if (maxcnt > 0) {
        const int ent = __shfl_sync(full, ent_reg, src);
        const unsigned long long wd = __shfl_sync(full, sm_reg, src);
        if (cnt > 0) {
            load_pair_block(p.rec, ent >> 3, ent & 7, b, cur);
            cur_slot = int((wd >> (8 * b)) & 0xffull);
        }
    }
    for (int k = 0; k < maxcnt; ++k) {
        const bool active = k < cnt;
        if (k + 1 < maxcnt) {  // uniform over the warp
            if (((k + 1) & 7) == 0) load_chunk((k + 1) >> 3);
            const int ent = __shfl_sync(full, ent_reg, src | ((k + 1) & 7));
            const unsigned long long wd = __shfl_sync(full, sm_reg, src | ((k + 1) & 7));
            if (k + 1 < cnt) {
                load_pair_block(p.rec, ent >> 3, ent & 7, b, nxt);
                nxt_slot = int((wd >> (8 * b)) & 0xffull);
            }
        }
        // a repeated corner node (degenerate element) maps two corners to one slot
        bool dup = false;
#pragma unroll
        for (int bp = 0; bp < 7; ++bp) {
            const int other = __shfl_sync(full, cur_slot, (lane & ~7) | bp);
            if (bp < b && other == cur_slot) dup = true;
        }
        const unsigned bit = 1u << cur_slot;
        double* a = accr + (full27 ? pos27(cur_slot) : cur_slot) * kPairStride;
        if (active && !dup) {
            if (touched & bit) {
#pragma unroll
                for (int q = 0; q < kPairStride; ++q) a[q] += cur[q];
            } else {
#pragma unroll
                for (int q = 0; q < kPairStride; ++q) a[q] = cur[q];
            }
        }
        if (__any_sync(full, active && dup)) {
            for (int bb = 1; bb < 8; ++bb) {
                __syncwarp();
                if (active && dup && b == bb) {
#pragma unroll
                    for (int q = 0; q < kPairStride; ++q) a[q] += cur[q];
                }
            }
        }
        unsigned nb = active ? bit : 0u;
        nb |= __shfl_xor_sync(full, nb, 1);
        nb |= __shfl_xor_sync(full, nb, 2);
        nb |= __shfl_xor_sync(full, nb, 4);
        touched |= nb;
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kPairStride; ++q) cur[q] = nxt[q];
        cur_slot = nxt_slot;
    }
    __syncwarp();

    // ---- write the four rows (all lanes, coalesced) -----------------------------------------
    for (int rr = 0; rr < kG64Rows; ++rr) {
        const int64_t rw = row0 + rr;
        if (rw >= p.row_end) break;
        const int64_t rrs = __shfl_sync(full, rs, rr * 8);
        const int LL = __shfl_sync(full, L, rr * 8);
        const unsigned tch = __shfl_sync(full, touched, rr * 8);
        const unsigned fixed_bits = p.fixed ? p.fixed[rw] : 0u;
        const int sd = __shfl_sync(full, diag, rr * 8);
        const bool has_diag = sd >= 0;
        const bool f27 = LL == kG64MaxL;
        const double* acc = S.acc[w][rr];
        auto value = [&](int s_, int q) -> double {
            if (!((tch >> s_) & 1u)) return 0.0;
            double v = acc[(f27 ? pos27(s_) : s_) * kPairStride + q];
            if (q < 9 && has_diag && s_ == sd && (q % 4 == 0) && ((fixed_bits >> (q / 4)) & 1u)) v = 1e20;
            return v;
        };
        if (p.K) {
            if (p.k_layout == FEM_LAYOUT_BSR) {
                for (int o = lane; o < 9 * LL; o += 32) {
                    const int s_ = o / 9;
                    p.K[9 * rrs + o] = value(s_, o - 9 * s_);
                }
            } else {
                for (int pp = 0; pp < 3; ++pp)
                    for (int idx = lane; idx < 3 * LL; idx += 32) {
                        const int s_ = idx / 3;
                        p.K[9 * rrs + int64_t(3 * LL) * pp + idx] = value(s_, 3 * pp + (idx - 3 * s_));
                    }
            }
        }
        if (p.M) {
            if (p.m_layout == FEM_LAYOUT_BSR) {
                for (int o = lane; o < LL; o += 32) p.M[rrs + o] = value(o, 9);
            } else {
                for (int o = lane; o < LL; o += 32) {
                    const double mv = value(o, 9);
                    p.M[3 * rrs + o] = mv;
                    p.M[3 * rrs + LL + o] = mv;
                    p.M[3 * rrs + 2 * LL + o] = mv;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_csr_index(int64_t n_node, const int32_t* __restrict__ indptr,
                                                   const int32_t* __restrict__ indices, int32_t* rowK,
                                                   int32_t* colK, int32_t* rowM, int32_t* colM) {
    const int64_t row = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n_node) return;
    const int64_t rs = indptr[row];
    const int L = indptr[row + 1] - int(rs);
    if (lane < 3) {
        // InstallIndexK / InstallIndexM: FEM_model_csr.py:167-173, 195-201
        if (rowK) rowK[3 * row + 1 + lane] = int32_t(L * 3 * (lane + 1) + rs * 9);
        if (rowM) rowM[3 * row + 1 + lane] = int32_t(L * (lane + 1) + rs * 3);
        if (row == 0) {
            if (rowK) rowK[0] = 0;
            if (rowM) rowM[0] = 0;
        }
    }
    for (int l = lane; l < L; l += 32) {
        const int col = indices[rs + l];
        for (int pp = 0; pp < 3; ++pp) {
            if (colK) {
                int32_t* o = colK + 9 * rs + int64_t(3 * pp) * L + 3 * l;
                o[0] = 3 * col;
                o[1] = 3 * col + 1;
                o[2] = 3 * col + 2;
            }
            if (colM) colM[3 * rs + int64_t(pp) * L + l] = 3 * col + pp;
        }
    }
}

int check_mesh(const fem_mesh* m) {
    FEM_REQUIRE(m != nullptr, "mesh is NULL");
    FEM_REQUIRE(m->n_node >= 0 && m->n_elem >= 0 && m->nnzb >= 0, "negative mesh size");
    FEM_REQUIRE(m->n_elem < (int64_t(1) << 28), "n_elem too large");
    FEM_REQUIRE(m->n_node < (int64_t(1) << 31) - 1, "n_node too large");
    FEM_REQUIRE(9 * m->nnzb < (int64_t(1) << 62), "nnzb too large");
    if (m->n_elem) FEM_REQUIRE(m->xyz && m->conn && aligned16(m->conn), "xyz/conn NULL or conn not 16-byte aligned");
    if (m->n_node) FEM_REQUIRE(m->indptr && m->ne_ptr && m->ne_list, "pattern/incidence arrays are NULL");
    if (m->nnzb) FEM_REQUIRE(m->indices != nullptr, "indices is NULL");
    return FEM_OK;
}

}  // namespace

}  // namespace fem

using namespace fem;

extern "C" size_t fem_assemble_workspace_bytes(int64_t n_elem) {
    // FEM_ALGO_FP64: one 2,944-byte record per element; FEM_ALGO_DD: eight 672-byte
    // row-ordered chunks per element.  The larger of the two serves both.
    return n_elem > 0 ? size_t(n_elem) * 8 * 672 : 0;
}

namespace {

int check_assembly_inputs(const fem_mesh* mesh, const fem_material* mat, void* workspace, size_t workspace_bytes) {
    int rc = check_mesh(mesh);
    if (rc) return rc;
    FEM_REQUIRE(mat != nullptr, "mat is NULL");
    FEM_REQUIRE(mat->PO > -1.0 && mat->PO < 0.5, "Poisson ratio must lie in (-1, 0.5)");
    if (workspace_bytes < fem_assemble_workspace_bytes(mesh->n_elem) || (mesh->n_elem && !workspace)) {
        set_error("workspace too small: need %zu bytes", fem_assemble_workspace_bytes(mesh->n_elem));
        return FEM_ERR_WORKSPACE;
    }
    FEM_REQUIRE(workspace == nullptr || aligned16(workspace), "workspace not 16-byte aligned");
    return FEM_OK;
}

}  // namespace

namespace fem {
int launch_hex8_element_dd(const fem_mesh* mesh, const fem_material* mat, void* workspace, cudaStream_t st,
                           int64_t e_begin, int64_t e_end);
int launch_gather_dd(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace, cudaStream_t st,
                     int64_t row_begin, int64_t row_end);
}  // namespace fem

namespace fem {
namespace {

int launch_hex8_element(const fem_mesh* mesh, const fem_material* mat, void* workspace, cudaStream_t st,
                        int64_t e_begin, int64_t e_end) {
    if (e_end <= e_begin) return FEM_OK;
    ElemParams ep;
    ep.xyz = mesh->xyz;
    ep.conn4 = reinterpret_cast<const int4*>(mesh->conn);
    ep.e_begin = e_begin;
    ep.e_end = e_end;
    ep.rec = static_cast<double*>(workspace);
    const double EX = mat->EX, PO = mat->PO;
    ep.DE = mat->DE;
    ep.D0d = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO);  // FEM_model_bsr.py:435-437
    ep.lam = EX * PO / (1 + PO) / (1 - 2 * PO);         // :439-445
    ep.mu = EX / 2 / (1 + PO);                          // :447-449
    {
        const double w0 = mat->omega[0], w1 = mat->omega[1], w2 = mat->omega[2];
        const double wc[3][3] = {{w1 * w1 + w2 * w2, -w0 * w1, -w0 * w2},   // UnitVectorF, FEM_model_bsr.py:291-300
                                 {-w1 * w0, w0 * w0 + w2 * w2, -w1 * w2},
                                 {-w2 * w0, -w2 * w1, w1 * w1 + w0 * w0}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) ep.wc[i][j] = wc[i][j];
    }
    ep.tab = make_tables();
    {
        // 1D shape factors (1 + s x) / 2 at x = +-kGS1: al for a corner on the Gauss point's
        // side, be for the other side
        const double al = 0.5 * (1.0 + kGS1), be = 0.5 * (1.0 - kGS1);
        const double tm[2][3] = {{al * al, al * be, be * be}, {be * be, al * be, al * al}};
        for (int sd = 0; sd < 2; ++sd)
            for (int c = 0; c < 3; ++c) ep.tm[sd][c] = tm[sd][c];
    }
    const size_t smem = sizeof(ElemSmem);
    FEM_CUDA(cudaFuncSetAttribute(k_hex8_element, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t blocks = (e_end - e_begin + kEpc - 1) / kEpc;
    k_hex8_element<<<unsigned(blocks), kElemThreads, smem, st>>>(ep);
    FEM_LAUNCH_CHECK("k_hex8_element");
    return FEM_OK;
}

// FP64 gather of block rows [row_begin, row_end); the lane-per-corner kernel needs the
// element-to-block map, the lane-per-slot kernel (whole mesh only) does not.
int launch_gather64(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace, cudaStream_t st,
                    int64_t row_begin, int64_t row_end) {
    if (row_end <= row_begin) return FEM_OK;
    if (!mesh->slot_map) {
        FEM_REQUIRE(row_begin == 0 && row_end == mesh->n_node, "a partial FP64 gather needs mesh->slot_map");
        GatherParams gp;
        gp.n_node = mesh->n_node;
        gp.indptr = mesh->indptr;
        gp.indices = mesh->indices;
        gp.ne_ptr = mesh->ne_ptr;
        gp.ne_list = mesh->ne_list;
        gp.conn4 = reinterpret_cast<const int4*>(mesh->conn);
        gp.rec = static_cast<const double*>(workspace);
        gp.k_layout = out->k_layout;
        gp.m_layout = out->m_layout;
        gp.K = out->K;
        gp.M = out->M;
        gp.F = out->F;
        gp.fixed = out->fixed;
        gp.loads = out->loads;
        const int64_t blocks = (mesh->n_node * 32 + 255) / 256;
        k_gather<<<unsigned(blocks), 256, 0, st>>>(gp);
        FEM_LAUNCH_CHECK("k_gather");
        return FEM_OK;
    }
    Gather64Params gp;
    gp.row_begin = row_begin;
    gp.row_end = row_end;
    gp.indptr = mesh->indptr;
    gp.indices = mesh->indices;
    gp.ne_ptr = mesh->ne_ptr;
    gp.ne_list = mesh->ne_list;
    gp.slot_map = mesh->slot_map;
    gp.slot_map_aligned = (reinterpret_cast<uintptr_t>(mesh->slot_map) & 7) == 0;
    gp.conn4 = reinterpret_cast<const int4*>(mesh->conn);
    gp.rec = static_cast<const double*>(workspace);
    gp.k_layout = out->k_layout;
    gp.m_layout = out->m_layout;
    gp.K = out->K;
    gp.M = out->M;
    gp.F = out->F;
    gp.fixed = out->fixed;
    gp.loads = out->loads;
    const size_t smem = sizeof(Gather64Smem);
    FEM_CUDA(cudaFuncSetAttribute(k_gather64, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t rows_per_cta = int64_t(kG64Warps) * kG64Rows;
    const int64_t blocks = (row_end - row_begin + rows_per_cta - 1) / rows_per_cta;
    k_gather64<<<unsigned(blocks), kG64Warps * 32, smem, st>>>(gp);
    FEM_LAUNCH_CHECK("k_gather64");
    return FEM_OK;
}

}  // namespace
}  // namespace fem

extern "C" int fem_assemble_elements(const fem_mesh* mesh, const fem_material* mat, int algo, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    int rc = check_assembly_inputs(mesh, mat, workspace, workspace_bytes);
    if (rc) return rc;
    FEM_REQUIRE(algo == FEM_ALGO_DD || algo == FEM_ALGO_FP64, "bad algo");
    if (mesh->n_elem == 0) return FEM_OK;
    FEM_REQUIRE(algo != FEM_ALGO_DD || (mesh->ne_inv && mesh->slot_map),
                "FEM_ALGO_DD needs mesh->ne_inv and mesh->slot_map (fem_gather_map)");
    if (algo == FEM_ALGO_DD) return launch_hex8_element_dd(mesh, mat, workspace, as_stream(stream), 0, mesh->n_elem);
    return launch_hex8_element(mesh, mat, workspace, as_stream(stream), 0, mesh->n_elem);
}

extern "C" int fem_assemble_gather(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace,
                                   size_t workspace_bytes, void* stream) {
    int rc = check_mesh(mesh);
    if (rc) return rc;
    FEM_REQUIRE(out != nullptr, "out is NULL");
    FEM_REQUIRE(out->k_layout == FEM_LAYOUT_BSR || out->k_layout == FEM_LAYOUT_CSR, "bad k_layout");
    FEM_REQUIRE(out->m_layout == FEM_LAYOUT_BSR || out->m_layout == FEM_LAYOUT_CSR, "bad m_layout");
    FEM_REQUIRE(out->algo == FEM_ALGO_DD || out->algo == FEM_ALGO_FP64, "bad algo");
    if (workspace_bytes < fem_assemble_workspace_bytes(mesh->n_elem) || (mesh->n_elem && !workspace)) {
        set_error("workspace too small: need %zu bytes", fem_assemble_workspace_bytes(mesh->n_elem));
        return FEM_ERR_WORKSPACE;
    }
    if (mesh->n_node == 0 || (!out->K && !out->M && !out->F)) return FEM_OK;
    if (out->algo == FEM_ALGO_DD) {
        FEM_REQUIRE(mesh->n_elem == 0 || mesh->slot_map, "FEM_ALGO_DD needs mesh->slot_map (fem_gather_map)");
        return launch_gather_dd(mesh, out, workspace, as_stream(stream), 0, mesh->n_node);
    }
    return launch_gather64(mesh, out, workspace, as_stream(stream), 0, mesh->n_node);
}

extern "C" int fem_assemble(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                            void* workspace, size_t workspace_bytes, void* stream) {
    int rc = check_assembly_inputs(mesh, mat, workspace, workspace_bytes);
    if (rc) return rc;
    FEM_REQUIRE(out != nullptr, "out is NULL");
    FEM_REQUIRE(out->k_layout == FEM_LAYOUT_BSR || out->k_layout == FEM_LAYOUT_CSR, "bad k_layout");
    FEM_REQUIRE(out->m_layout == FEM_LAYOUT_BSR || out->m_layout == FEM_LAYOUT_CSR, "bad m_layout");
    if (mesh->n_node == 0) return FEM_OK;
    rc = fem_assemble_elements(mesh, mat, out->algo, workspace, workspace_bytes, stream);
    if (rc) return rc;
    return fem_assemble_gather(mesh, out, workspace, workspace_bytes, stream);
}

namespace fem {
namespace {

// fem_assemble_host; with `on_part`, the calling thread also waits for each part's copies in
// turn and calls on_part(q) while later parts are still being copied (then returns only when
// every copy and every on_part call is done).
template <typename OnPart>
int assemble_host_impl(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                       const int64_t* row_split, const int64_t* elem_split, const int64_t* block_split, int n_parts,
                       double* K_host, double* M_host, double* F_host, void* workspace, size_t workspace_bytes,
                       void* stream, OnPart* on_part) {
    int rc = check_assembly_inputs(mesh, mat, workspace, workspace_bytes);
    if (rc) return rc;
    FEM_REQUIRE(out != nullptr, "out is NULL");
    FEM_REQUIRE(out->k_layout == FEM_LAYOUT_BSR || out->k_layout == FEM_LAYOUT_CSR, "bad k_layout");
    FEM_REQUIRE(out->m_layout == FEM_LAYOUT_BSR || out->m_layout == FEM_LAYOUT_CSR, "bad m_layout");
    FEM_REQUIRE(out->algo == FEM_ALGO_DD || out->algo == FEM_ALGO_FP64, "bad algo");
    FEM_REQUIRE((!K_host || out->K) && (!M_host || out->M) && (!F_host || out->F),
                "a host output needs the matching device output in out");
    FEM_REQUIRE(n_parts >= 1 && row_split && elem_split && block_split, "bad plan");
    FEM_REQUIRE(row_split[0] == 0 && row_split[n_parts] == mesh->n_node && elem_split[0] == 0 &&
                    elem_split[n_parts] == mesh->n_elem && block_split[0] == 0 && block_split[n_parts] == mesh->nnzb,
                "plan does not span the mesh (use fem_pipeline_plan)");
    for (int q = 0; q < n_parts; ++q)
        FEM_REQUIRE(row_split[q] <= row_split[q + 1] && elem_split[q] <= elem_split[q + 1] &&
                        block_split[q] <= block_split[q + 1],
                    "plan is not monotone");
    if (mesh->n_node == 0) return FEM_OK;
    FEM_REQUIRE(out->algo != FEM_ALGO_DD || mesh->n_elem == 0 || (mesh->ne_inv && mesh->slot_map),
                "FEM_ALGO_DD needs mesh->ne_inv and mesh->slot_map (fem_gather_map)");
    FEM_REQUIRE(out->algo == FEM_ALGO_DD || mesh->n_elem == 0 || mesh->slot_map || n_parts == 1,
                "a split FP64 assembly needs mesh->slot_map (fem_gather_map)");
    cudaStream_t st = as_stream(stream);
    const bool dd = out->algo == FEM_ALGO_DD;
    const int parts = n_parts;
    std::vector<cudaEvent_t> elems(parts, nullptr), done(parts, nullptr), copied(parts, nullptr);
    cudaStream_t cs = nullptr, gs = nullptr;
    cudaEvent_t start = nullptr, fin = nullptr;
    auto cleanup = [&] {
        for (auto* v : {&elems, &done, &copied})
            for (cudaEvent_t e : *v)
                if (e) cudaEventDestroy(e);
        if (start) cudaEventDestroy(start);
        if (fin) cudaEventDestroy(fin);
        if (cs) cudaStreamDestroy(cs);
        if (gs) cudaStreamDestroy(gs);
    };
    auto fail = [&](cudaError_t e, const char* what) {
        cleanup();
        return cuda_status(e, what);
    };
    int lo_prio = 0, hi_prio = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio);
    if (e != cudaSuccess) return fail(e, "cudaDeviceGetStreamPriorityRange");
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&gs, cudaStreamNonBlocking, hi_prio)) != cudaSuccess)
        return fail(e, "stream creation");
    if ((e = cudaEventCreateWithFlags(&start, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventRecord(start, st)) != cudaSuccess || (e = cudaStreamWaitEvent(gs, start, 0)) != cudaSuccess)
        return fail(e, "gather stream ordering");
    // All kernels first (a copy into pageable memory may block the host until it ends).  The
    // element parts run in order on the caller's stream and the gathers on a second,
    // highest-priority stream, gather q after element part q: the gather of part q fills the
    // partial last waves of element part q + 1 instead of waiting for them, and part q's copy
    // can start as soon as its gather ends.  Records of different parts never overlap, so the
    // results do not depend on how the two streams interleave.
    for (int q = 0; q < parts; ++q) {
        rc = dd ? launch_hex8_element_dd(mesh, mat, workspace, st, elem_split[q], elem_split[q + 1])
                : launch_hex8_element(mesh, mat, workspace, st, elem_split[q], elem_split[q + 1]);
        if (rc) {
            cleanup();
            return rc;
        }
        if ((e = cudaEventCreateWithFlags(&elems[q], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventRecord(elems[q], st)) != cudaSuccess || (e = cudaStreamWaitEvent(gs, elems[q], 0)) != cudaSuccess)
            return fail(e, "element part event");
        rc = dd ? launch_gather_dd(mesh, out, workspace, gs, row_split[q], row_split[q + 1])
                : launch_gather64(mesh, out, workspace, gs, row_split[q], row_split[q + 1]);
        if (rc) {
            cleanup();
            return rc;
        }
        if ((e = cudaEventCreateWithFlags(&done[q], cudaEventDisableTiming)) != cudaSuccess ||
            (e = cudaEventRecord(done[q], gs)) != cudaSuccess)
            return fail(e, "cudaEventRecord");
    }
    const int64_t kq = 9, mq = out->m_layout == FEM_LAYOUT_BSR ? 1 : 3;
    for (int q = 0; q < parts; ++q) {
        const int64_t r0 = row_split[q], r1 = row_split[q + 1];
        const int64_t b0 = block_split[q], b1 = block_split[q + 1];
        if ((e = cudaStreamWaitEvent(cs, done[q], 0)) != cudaSuccess) return fail(e, "cudaStreamWaitEvent");
        if (K_host && b1 > b0 &&
            (e = cudaMemcpyAsync(K_host + kq * b0, out->K + kq * b0, sizeof(double) * kq * (b1 - b0),
                                 cudaMemcpyDeviceToHost, cs)) != cudaSuccess)
            return fail(e, "K device->host copy");
        if (M_host && b1 > b0 &&
            (e = cudaMemcpyAsync(M_host + mq * b0, out->M + mq * b0, sizeof(double) * mq * (b1 - b0),
                                 cudaMemcpyDeviceToHost, cs)) != cudaSuccess)
            return fail(e, "M device->host copy");
        if (F_host && r1 > r0 &&
            (e = cudaMemcpyAsync(F_host + 3 * r0, out->F + 3 * r0, sizeof(double) * 3 * (r1 - r0),
                                 cudaMemcpyDeviceToHost, cs)) != cudaSuccess)
            return fail(e, "F device->host copy");
        if (on_part && ((e = cudaEventCreateWithFlags(&copied[q], cudaEventDisableTiming)) != cudaSuccess ||
                        (e = cudaEventRecord(copied[q], cs)) != cudaSuccess))
            return fail(e, "copy event");
    }
    if (on_part)
        for (int q = 0; q < parts; ++q) {
            if ((e = cudaEventSynchronize(copied[q])) != cudaSuccess) return fail(e, "copy event wait");
            (*on_part)(q);
        }
    // the caller's stream is ordered after the last copy
    if ((e = cudaEventCreateWithFlags(&fin, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventRecord(fin, cs)) != cudaSuccess || (e = cudaStreamWaitEvent(st, fin, 0)) != cudaSuccess)
        return fail(e, "copy completion event");
    cleanup();
    return FEM_OK;
}

}  // namespace
}  // namespace fem

extern "C" int fem_assemble_host(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                                 const int64_t* row_split, const int64_t* elem_split, const int64_t* block_split,
                                 int n_parts, double* K_host, double* M_host, double* F_host, void* workspace,
                                 size_t workspace_bytes, void* stream) {
    struct NoPart {
        void operator()(int) const {}
    };
    return assemble_host_impl<NoPart>(mesh, mat, out, row_split, elem_split, block_split, n_parts, K_host, M_host,
                                      F_host, workspace, workspace_bytes, stream, nullptr);
}

extern "C" int fem_assemble_host_staged(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                                        const int64_t* row_split, const int64_t* elem_split,
                                        const int64_t* block_split, int n_parts, const int32_t* indptr_host,
                                        double* K_host, double* M_host, double* F_host, double* M_stage,
                                        void* workspace, size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(out != nullptr && mesh != nullptr, "NULL argument");
    if (!M_host || !M_stage || out->m_layout != FEM_LAYOUT_CSR)
        return fem_assemble_host(mesh, mat, out, row_split, elem_split, block_split, n_parts, K_host, M_host,
                                 F_host, workspace, workspace_bytes, stream);
    FEM_REQUIRE(indptr_host != nullptr && row_split != nullptr && n_parts >= 1, "NULL argument");
    // M leaves the device as one value per block (the BSR layout) into M_stage; the reference's
    // scalar CSR (3 copies of it per block row) is written on the host, part by part, while
    // the later parts are still being copied.
    fem_assembly_out o = *out;
    o.m_layout = FEM_LAYOUT_BSR;
    auto expand = [&](int q) {
        const int64_t r0 = row_split[q], r1 = row_split[q + 1];
#pragma omp parallel for schedule(dynamic, 512)
        for (int64_t i = r0; i < r1; ++i) {
            const int64_t rs = indptr_host[i], L = indptr_host[i + 1] - rs;
            const double* src = M_stage + rs;
            double* dst = M_host + 3 * rs;
            for (int pp = 0; pp < 3; ++pp)
                for (int64_t l = 0; l < L; ++l) dst[pp * L + l] = src[l];
        }
    };
    return assemble_host_impl(mesh, mat, &o, row_split, elem_split, block_split, n_parts, K_host, M_stage, F_host,
                              workspace, workspace_bytes, stream, &expand);
}

extern "C" int fem_csr_index(const fem_mesh* mesh, int32_t* rowK, int32_t* colK, int32_t* rowM, int32_t* colM,
                             void* stream) {
    FEM_REQUIRE(mesh != nullptr, "mesh is NULL");
    FEM_REQUIRE(mesh->n_node >= 0, "negative size");
    FEM_REQUIRE(9 * mesh->nnzb < (int64_t(1) << 31), "CSR column indices exceed int32");
    if (mesh->n_node == 0) return FEM_OK;
    FEM_REQUIRE(mesh->indptr && (mesh->nnzb == 0 || mesh->indices), "pattern arrays are NULL");
    const int64_t blocks = (mesh->n_node * 32 + 255) / 256;
    k_csr_index<<<unsigned(blocks), 256, 0, as_stream(stream)>>>(mesh->n_node, mesh->indptr, mesh->indices, rowK,
                                                                 colK, rowM, colM);
    FEM_LAUNCH_CHECK("k_csr_index");
    return FEM_OK;
}
