// Large-displacement tangent and secant stiffness (Get_MatrixKN, FEM_model_bsr.py:134-145;
// UnitK :476-515, InslocalBN :544-592, MatrixS :517-525), FP64.
//
// k_hex8_tangent: 8 threads per element, 8 elements per CTA.
//   phase A (thread = Gauss point g): J, det, DN = dN/dx, T = grad u = CoordU . DN;
//   phase S (thread = corner j): c[g][j] = (D0 (B1_j + BN1_j/2) u_j, D1 (B2_j + BN2_j/2) u_j);
//   phase P (thread = Gauss point g): S_g = sum over g' <= g and all j of c[g'][j], in the
//     reference's accumulation order (S is never reset between Gauss points);
//   phase B (thread = row corner j): for every column corner k, over g,
//     KT_jk += det ((B1+BN1)_j^T D0 (B1+BN1)_k + (B2+BN2)_j^T D1 (B2+BN2)_k) + det (DN_j . S_g . DN_k) I
//     KM_jk += det ((B1+BN1)_j^T D0 (B1+BN1/2)_k + (B2+BN2)_j^T D1 (B2+BN2/2)_k)
//   and writes row j's 8 blocks of each matrix as one row-ordered chunk (the format the
//   double-float gather consumes) at the corner's incidence position.
// Both matrices are then gathered (atomic-free, fixed order) with the penalty applied.
#include "fem_common.cuh"

namespace fem {
namespace {

constexpr int kEpcT = 8;
constexpr int kThreadsT = kEpcT * 8;
constexpr int kChunkT = 84;  // float pairs per (element, corner) chunk: 8 blocks x 10 + F 3 + pad
constexpr int kChunkFT = 80;

struct TangentParams {
    const double* xyz;
    const int4* conn4;
    const double* u;
    const int32_t* ne_inv;
    int64_t n_elem;
    float2* recT;
    float2* recM;
    double D0d, lam, mu;
    double dnr[8][8][3];
};

struct TangentSmem {
    double dnr[8][8][3];
    double xl[kEpcT][8][3];
    double ue[kEpcT][8][3];
    double DN[kEpcT][8][8][3];  // [g][a][d]
    double T[kEpcT][8][3][3];   // [g][k][d]
    double det[kEpcT][8];
    double c[kEpcT][8][8][6];   // [g][j]
    double S[kEpcT][8][6];      // accumulated S after Gauss point g
};

__device__ __forceinline__ float2 split(double x) {
    const float hi = __double2float_rn(x);
    return make_float2(hi, __double2float_rn(x - double(hi)));
}

// B1 = diag(DN), B2 rows (yz, xz, xy) of corner a (installLocalB, FEM_model_bsr.py:303-347);
// BN1, BN2 of corner a (InslocalBN, :544-592); all 3x3 [row][col].
__device__ __forceinline__ void strain_ops(const double (&dn)[3], const double (&T)[3][3], double (&B1)[3][3],
                                           double (&B2)[3][3], double (&N1)[3][3], double (&N2)[3][3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) B1[r][c] = r == c ? dn[r] : 0.0;
    B2[0][0] = 0.0, B2[0][1] = dn[2], B2[0][2] = dn[1];
    B2[1][0] = dn[2], B2[1][1] = 0.0, B2[1][2] = dn[0];
    B2[2][0] = dn[1], B2[2][1] = dn[0], B2[2][2] = 0.0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        N1[0][k] = T[k][0] * dn[0];
        N1[1][k] = T[k][1] * dn[1];
        N1[2][k] = T[k][2] * dn[2];
        N2[0][k] = T[k][2] * dn[1] + T[k][1] * dn[2];
        N2[1][k] = T[k][2] * dn[0] + T[k][0] * dn[2];
        N2[2][k] = T[k][1] * dn[0] + T[k][0] * dn[1];
    }
}

__global__ void __launch_bounds__(kThreadsT) k_hex8_tangent(const TangentParams p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TangentSmem& s = *reinterpret_cast<TangentSmem*>(smem_raw);
    const int tid = threadIdx.x, el = tid >> 3, t = tid & 7;
    const int64_t e = int64_t(blockIdx.x) * kEpcT + el;
    const bool valid = e < p.n_elem;
    for (int k = tid; k < 8 * 8 * 3; k += kThreadsT) (&s.dnr[0][0][0])[k] = (&p.dnr[0][0][0])[k];
    const double D0[3][3] = {{p.D0d, p.lam, p.lam}, {p.lam, p.D0d, p.lam}, {p.lam, p.lam, p.D0d}};
    if (valid) {
        const int* cn = reinterpret_cast<const int*>(p.conn4) + 8 * e;
        const int64_t node = __ldg(cn + t), node0 = __ldg(cn);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.xl[el][t][i] = __ldg(p.xyz + 3 * node + i) - __ldg(p.xyz + 3 * node0 + i);
            s.ue[el][t][i] = __ldg(p.u + 3 * node + i);
        }
    }
    __syncthreads();
    // phase A: Gauss point g = t
    if (valid) {
        const int g = t;
        double J[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double a = 0.0;
                for (int c = 0; c < 8; ++c) a += s.xl[el][c][i] * s.dnr[g][c][d];
                J[i][d] = a;
            }
        double A[3][3];  // adjugate
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
                A[j][i] = J[i1][j1] * J[i2][j2] - J[i2][j1] * J[i1][j2];
            }
        const double det = J[0][0] * A[0][0] + J[1][0] * A[0][1] + J[2][0] * A[0][2];
        const double inv = 1.0 / det;
        s.det[el][g] = det;
        for (int a = 0; a < 8; ++a)
#pragma unroll
            for (int d = 0; d < 3; ++d)
                s.DN[el][g][a][d] = (s.dnr[g][a][0] * A[0][d] + s.dnr[g][a][1] * A[1][d] + s.dnr[g][a][2] * A[2][d]) * inv;
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                double a = 0.0;
                for (int c = 0; c < 8; ++c) a += s.ue[el][c][k] * s.DN[el][g][c][d];
                s.T[el][g][k][d] = a;
            }
    }
    __syncthreads();
    // phase S: corner j = t, every Gauss point
    if (valid) {
        const int j = t;
        const double uj[3] = {s.ue[el][j][0], s.ue[el][j][1], s.ue[el][j][2]};
        for (int g = 0; g < 8; ++g) {
            const double dn[3] = {s.DN[el][g][j][0], s.DN[el][g][j][1], s.DN[el][g][j][2]};
            const double(&T)[3][3] = s.T[el][g];
            double B1[3][3], B2[3][3], N1[3][3], N2[3][3];
            strain_ops(dn, T, B1, B2, N1, N2);
            double t1[3], t2[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                t1[r] = (B1[r][0] + 0.5 * N1[r][0]) * uj[0] + (B1[r][1] + 0.5 * N1[r][1]) * uj[1] +
                        (B1[r][2] + 0.5 * N1[r][2]) * uj[2];
                t2[r] = (B2[r][0] + 0.5 * N2[r][0]) * uj[0] + (B2[r][1] + 0.5 * N2[r][1]) * uj[1] +
                        (B2[r][2] + 0.5 * N2[r][2]) * uj[2];
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                s.c[el][g][j][r] = D0[r][0] * t1[0] + D0[r][1] * t1[1] + D0[r][2] * t1[2];
                s.c[el][g][j][3 + r] = p.mu * t2[r];
            }
        }
    }
    __syncthreads();
    // phase P: S after Gauss point g = t (accumulated in the reference's g, j order)
    if (valid) {
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int g = 0; g <= t; ++g)
            for (int j = 0; j < 8; ++j)
#pragma unroll
                for (int q = 0; q < 6; ++q) acc[q] += s.c[el][g][j][q];
#pragma unroll
        for (int q = 0; q < 6; ++q) s.S[el][t][q] = acc[q];
    }
    __syncthreads();
    if (!valid) return;
    // phase B: row corner j = t
    const int j = t;
    float2* cT = p.recT + int64_t(__ldg(p.ne_inv + 8 * e + j)) * kChunkT;
    float2* cM = p.recM + int64_t(__ldg(p.ne_inv + 8 * e + j)) * kChunkT;
    for (int k = 0; k < 8; ++k) {
        double KT[3][3] = {}, KM[3][3] = {};
        for (int g = 0; g < 8; ++g) {
            const double(&T)[3][3] = s.T[el][g];
            const double dj[3] = {s.DN[el][g][j][0], s.DN[el][g][j][1], s.DN[el][g][j][2]};
            const double dk[3] = {s.DN[el][g][k][0], s.DN[el][g][k][1], s.DN[el][g][k][2]};
            double B1j[3][3], B2j[3][3], N1j[3][3], N2j[3][3], B1k[3][3], B2k[3][3], N1k[3][3], N2k[3][3];
            strain_ops(dj, T, B1j, B2j, N1j, N2j);
            strain_ops(dk, T, B1k, B2k, N1k, N2k);
            // M1 = (B1 + BN1)_j^T D0, M2 = (B2 + BN2)_j^T D1 (= mu (B2 + BN2)_j^T)
            double M1[3][3], M2[3][3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    M1[a][b] = (B1j[0][a] + N1j[0][a]) * D0[0][b] + (B1j[1][a] + N1j[1][a]) * D0[1][b] +
                               (B1j[2][a] + N1j[2][a]) * D0[2][b];
                    M2[a][b] = p.mu * (B2j[b][a] + N2j[b][a]);
                }
            const double det = s.det[el][g];
            const double* Sg = s.S[el][g];
            // geometric term DN_j . s . DN_k with s = [[S0x, S1z, S1y], [S1z, S0y, S1x], [S1y, S1x, S0z]]
            const double sm[3][3] = {{Sg[0], Sg[5], Sg[4]}, {Sg[5], Sg[1], Sg[3]}, {Sg[4], Sg[3], Sg[2]}};
            double geo = 0.0;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) geo += dj[a] * sm[a][b] * dk[b];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    double Av = 0.0, Bv = 0.0;
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        Av += M1[a][c] * B1k[c][b] + M2[a][c] * B2k[c][b];
                        Bv += M1[a][c] * N1k[c][b] + M2[a][c] * N2k[c][b];
                    }
                    KT[a][b] += det * (Av + Bv);
                    KM[a][b] += det * (Av + 0.5 * Bv);
                }
#pragma unroll
            for (int a = 0; a < 3; ++a) KT[a][a] += det * geo;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                cT[k * 10 + 3 * a + b] = split(KT[a][b]);
                cM[k * 10 + 3 * a + b] = split(KM[a][b]);
            }
        cT[k * 10 + 9] = make_float2(0.f, 0.f);
        cM[k * 10 + 9] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < kChunkT - kChunkFT; ++q) {
        cT[kChunkFT + q] = make_float2(0.f, 0.f);
        cM[kChunkFT + q] = make_float2(0.f, 0.f);
    }
}

}  // namespace

int launch_gather_dd(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace, cudaStream_t st,
                     int64_t row_begin, int64_t row_end);

}  // namespace fem

using namespace fem;

extern "C" size_t fem_tangent_workspace_bytes(int64_t n_elem) {
    if (n_elem <= 0) return 0;
    return 2 * ((size_t(n_elem) * 8 * kChunkT * sizeof(float2) + 255) / 256 * 256);
}

extern "C" int fem_assemble_tangent(const fem_mesh* mesh, const fem_material* mat, const double* u, int k_layout,
                                    double* KT, double* KM, const uint8_t* fixed, void* workspace,
                                    size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(mesh && mat, "mesh/mat is NULL");
    FEM_REQUIRE(mesh->n_node >= 0 && mesh->n_elem >= 0 && mesh->nnzb >= 0, "negative mesh size");
    FEM_REQUIRE(mesh->n_elem < (int64_t(1) << 28), "n_elem too large");
    FEM_REQUIRE(mat->PO > -1.0 && mat->PO < 0.5, "Poisson ratio must lie in (-1, 0.5)");
    FEM_REQUIRE(k_layout == FEM_LAYOUT_BSR || k_layout == FEM_LAYOUT_CSR, "bad k_layout");
    if (mesh->n_node == 0) return FEM_OK;
    FEM_REQUIRE(KT && KM, "KT/KM is NULL");
    FEM_REQUIRE(mesh->indptr && mesh->ne_ptr && (mesh->nnzb == 0 || mesh->indices), "pattern arrays are NULL");
    const size_t need = fem_tangent_workspace_bytes(mesh->n_elem);
    if (mesh->n_elem) {
        FEM_REQUIRE(u && mesh->xyz && mesh->conn && aligned16(mesh->conn) && mesh->ne_inv && mesh->slot_map,
                    "u/xyz/conn/ne_inv/slot_map NULL or conn misaligned");
        if (workspace_bytes < need || !workspace) {
            set_error("workspace too small: need %zu bytes", need);
            return FEM_ERR_WORKSPACE;
        }
        FEM_REQUIRE(aligned16(workspace), "workspace not 16-byte aligned");
    }
    cudaStream_t st = as_stream(stream);
    float2* recT = static_cast<float2*>(workspace);
    float2* recM = reinterpret_cast<float2*>(static_cast<unsigned char*>(workspace) + need / 2);
    if (mesh->n_elem) {
        TangentParams tp;
        tp.xyz = mesh->xyz;
        tp.conn4 = reinterpret_cast<const int4*>(mesh->conn);
        tp.u = u;
        tp.ne_inv = mesh->ne_inv;
        tp.n_elem = mesh->n_elem;
        tp.recT = recT;
        tp.recM = recM;
        const double EX = mat->EX, PO = mat->PO;
        tp.D0d = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO);  // FEM_model_bsr.py:435-449
        tp.lam = EX * PO / (1 + PO) / (1 - 2 * PO);
        tp.mu = EX / 2 / (1 + PO);
        const ShapeTables& T = shape_tables();
        for (int g = 0; g < 8; ++g)
            for (int a = 0; a < 8; ++a)
                for (int d = 0; d < 3; ++d) tp.dnr[g][a][d] = T.dnr[g][a][d];
        const size_t smem = sizeof(TangentSmem);
        FEM_CUDA(cudaFuncSetAttribute(k_hex8_tangent, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        const int64_t blocks = (mesh->n_elem + kEpcT - 1) / kEpcT;
        k_hex8_tangent<<<unsigned(blocks), kThreadsT, smem, st>>>(tp);
        FEM_LAUNCH_CHECK("k_hex8_tangent");
    } else {
        // no element: zero chunks are never read; both outputs still come from the gather
        recT = recM = nullptr;
    }
    fem_assembly_out o{};
    o.k_layout = k_layout;
    o.m_layout = FEM_LAYOUT_BSR;
    o.fixed = fixed;
    o.algo = FEM_ALGO_DD;
    o.K = KT;
    int rc = launch_gather_dd(mesh, &o, recT, st, 0, mesh->n_node);
    if (rc) return rc;
    o.K = KM;
    return launch_gather_dd(mesh, &o, recM, st, 0, mesh->n_node);
}
