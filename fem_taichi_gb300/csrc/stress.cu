// Nodal stress recovery for sm_103a (POST_process.py:72-99, 172-223).
//
//  1. k_stress_element -- 8 threads per element.  Thread t first forms coefficient t of the
//     trilinear interpolants of the element-local coordinates and of the displacements
//     (c_k = 1/8 sum_a m_k(corner a) v_a for the monomials 1, xi, eta, zeta, xi eta, eta zeta,
//     xi zeta, xi eta zeta), so that J and dU/dxi at a Gauss point cost 27 FMA each instead
//     of 72.  Thread g then evaluates the displacement
//     gradient at Gauss point g as H = (sum_a u_a (x) dN_a/dxi) . adj(J) / det, and the
//     stresses  sigma_n = D0 (H00, H11, H22),  sigma_s = mu (H01+H10, H12+H21, H02+H20)
//     (components xy, yz, xz as UnitVectorS orders them, POST_process.py:190-209).
//     Corner j's extrapolated value is sum_k W[j][k] sigma(k) with the caller's 8x8 weight
//     table (get_NdSol / shapefunc_GS, POST_process.py:172-181, 212-223); the dot products of
//     the table's distinct rows are spread over the element's threads, and thread j writes
//     corner j's values to the per-element workspace.
//  2. k_stress_node -- one thread per node: sums its incident (element, corner) values in
//     ascending element order (no atomics), divides by the element count (get_NdAve,
//     :183-187; one reciprocal, six products; an isolated node stays 0 * inf = NaN), then
//     computes the principal stresses with cyclic Jacobi rotations (descending order) and the
//     reference's "VM" formula as written (:93-94).
#include <cstring>
#include <mutex>

#include "fem_common.cuh"
#include "fem_dd.cuh"

namespace fem {
namespace {

constexpr int kEpc = 16;
constexpr int kThreads = kEpc * 8;
constexpr int kSvPad = 7;

struct StressParams {
    const double* xyz;
    const int4* conn4;
    const double* u;
    int64_t n_elem;
    double* rec;  // [n_elem][8][6]
    double D0d, lam, mu;
    double W[8][8];  // the distinct rows of the caller's extrapolation table
    int nrow;        // how many
    int row_of[8];   // corner j -> its row of W
};

struct StressSmem {
    double W[8][8];
    double res[kEpc][8][6];  // extrapolated values of each distinct table row
    double x[kEpc][8][3];
    double u[kEpc][8][3];
    double cx[kEpc][8][3];  // trilinear coefficients of the element-local coordinates
    double cu[kEpc][8][3];  // and of the displacements
    double sv[kEpc][8][kSvPad];
};

// m_k(corner a) of the trilinear monomials (1, xi, eta, zeta, xi eta, eta zeta, xi zeta,
// xi eta zeta) at the reference's corner order (POST_process.py:238-273): xi < 0 at corners
// 1, 2, 5, 6 (0x66), eta < 0 at 2, 3, 6, 7 (0xCC), zeta < 0 at 0-3 (0x0F); monomial k holds
// xi for k in {1, 4, 6, 7} (0xD2), eta for {2, 4, 5, 7} (0xB4), zeta for {3, 5, 6, 7} (0xE8).
__device__ __forceinline__ double monomial_sign(int k, int a) {
    const int neg = (((0xD2 >> k) & (0x66 >> a)) ^ ((0xB4 >> k) & (0xCC >> a)) ^ ((0xE8 >> k) & (0x0F >> a))) & 1;
    return neg ? -1.0 : 1.0;
}

// d/dxi, d/deta, d/dzeta of sum_k c_k m_k at (xi, eta, zeta) for one component
__device__ __forceinline__ void trilinear_grad(const double (*c)[3], int i, double xi, double et, double ze,
                                               double& d0, double& d1, double& d2) {
    const double c1 = c[1][i], c2 = c[2][i], c3 = c[3][i], c4 = c[4][i], c5 = c[5][i], c6 = c[6][i], c7 = c[7][i];
    d0 = fma(ze, fma(et, c7, c6), fma(et, c4, c1));
    d1 = fma(ze, fma(xi, c7, c5), fma(xi, c4, c2));
    d2 = fma(et, fma(xi, c7, c5), fma(xi, c6, c3));
}

__global__ void __launch_bounds__(kThreads) k_stress_element(const StressParams p) {
    __shared__ StressSmem s;
    const int tid = threadIdx.x;
    const int el = tid >> 3;
    const int t = tid & 7;
    const int64_t e = int64_t(blockIdx.x) * kEpc + el;
    const bool valid = e < p.n_elem;
    for (int k = tid; k < 64; k += kThreads) (&s.W[0][0])[k] = (&p.W[0][0])[k];
    if (valid) {
        const int node = __ldg(reinterpret_cast<const int*>(p.conn4) + 8 * e + t);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.x[el][t][i] = __ldg(p.xyz + 3 * int64_t(node) + i);
            s.u[el][t][i] = __ldg(p.u + 3 * int64_t(node) + i);
        }
    }
    __syncthreads();
    // element-local values (corner 0 subtracted; the gradients depend on differences only)
    double x0[3] = {0, 0, 0}, u0[3] = {0, 0, 0};
    if (valid) {
#pragma unroll
        for (int i = 0; i < 3; ++i) x0[i] = s.x[el][0][i], u0[i] = s.u[el][0][i];
    }
    __syncthreads();
    if (valid) {
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.x[el][t][i] -= x0[i];
            s.u[el][t][i] -= u0[i];
        }
    }
    __syncthreads();
    if (valid) {
        // coefficient t of the interpolants (corner 0 is now zero)
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            double ax = 0.0, au = 0.0;
#pragma unroll
            for (int a = 1; a < 8; ++a) {
                const double m = monomial_sign(t, a);
                ax = fma(m, s.x[el][a][i], ax);
                au = fma(m, s.u[el][a][i], au);
            }
            s.cx[el][t][i] = 0.125 * ax;
            s.cu[el][t][i] = 0.125 * au;
        }
    }
    __syncthreads();
    if (valid) {
        const int g = t;
        const double xi = (g & 4) ? kGS1 : -kGS1, et = (g & 2) ? kGS1 : -kGS1, ze = (g & 1) ? kGS1 : -kGS1;
        double J[3][3], G[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            trilinear_grad(s.cx[el], i, xi, et, ze, J[i][0], J[i][1], J[i][2]);
            trilinear_grad(s.cu[el], i, xi, et, ze, G[i][0], G[i][1], G[i][2]);
        }
        double A[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
                A[j][i] = J[i1][j1] * J[i2][j2] - J[i2][j1] * J[i1][j2];
            }
        const double det = J[0][0] * A[0][0] + J[1][0] * A[0][1] + J[2][0] * A[0][2];
        const double inv = 1.0 / det;
        double H[3][3];  // du_i/dx_k
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) H[i][k] = (G[i][0] * A[0][k] + G[i][1] * A[1][k] + G[i][2] * A[2][k]) * inv;
        const double D0d = p.D0d, lam = p.lam, mu = p.mu;
        s.sv[el][g][0] = D0d * H[0][0] + lam * (H[1][1] + H[2][2]);
        s.sv[el][g][1] = D0d * H[1][1] + lam * (H[0][0] + H[2][2]);
        s.sv[el][g][2] = D0d * H[2][2] + lam * (H[0][0] + H[1][1]);
        s.sv[el][g][3] = mu * (H[0][1] + H[1][0]);
        s.sv[el][g][4] = mu * (H[1][2] + H[2][1]);
        s.sv[el][g][5] = mu * (H[0][2] + H[2][0]);
    }
    __syncthreads();
    // Extrapolation: the table's distinct rows only (the reference's aliased GMat gives every
    // even corner one row and every odd corner another: 12 dot products per element instead of
    // 48), spread over the element's 8 threads; corner j then takes its row's values.
    if (valid) {
        const int nout = p.nrow * 6;
        for (int o = t; o < nout; o += 8) {
            const int r = o / 6, c = o - 6 * r;
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < 8; ++k) acc = fma(s.W[r][k], s.sv[el][k][c], acc);
            s.res[el][r][c] = acc;
        }
    }
    __syncthreads();
    if (!valid) return;
    const int j = t, r = p.row_of[j];
    double* o = p.rec + (e * 8 + j) * 6;
#pragma unroll
    for (int c = 0; c < 6; ++c) o[c] = s.res[el][r][c];
}

// Eigenvalues of the symmetric 3x3 [[a00,a01,a02],[a01,a11,a12],[a02,a12,a22]] by cyclic
// Jacobi rotations in Rutishauser's form (the rotated off-diagonal set to zero, the diagonal
// updated as a_pp - t a_pq and a_qq + t a_pq, the third row rotated with tau = s / (1 + c);
// Numerical Recipes, "jacobi"); from the second sweep on, an off-diagonal below the last bit of
// both diagonals (100 |a_pq| lost in |a_pp| and |a_qq|) is dropped instead of rotated -- its
// rotation would move the diagonal by about a_pq^2 / (a_qq - a_pp) -- which ends a 3 x 3 in
// about three sweeps instead of five; c = rsqrt(1 + t^2); capped at 32 sweeps; returned
// descending.
__device__ void sym3_eig_desc(double a00, double a11, double a22, double a01, double a12, double a02,
                              double& p1, double& p2, double& p3) {
    double d[3] = {a00, a11, a22};
    double o01 = a01, o02 = a02, o12 = a12;
    for (int sweep = 0; sweep < 32; ++sweep) {
        if (fabs(o01) + fabs(o02) + fabs(o12) == 0.0) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            // (p, q, r): (0, 1, 2), (0, 2, 1), (1, 2, 0)
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            double& apq = pq == 0 ? o01 : pq == 1 ? o02 : o12;
            double& apr = pq == 0 ? o02 : pq == 1 ? o01 : o01;   // (p, r)
            double& aqr = pq == 0 ? o12 : pq == 1 ? o12 : o02;   // (q, r)
            if (apq == 0.0) continue;
            const double g = 100.0 * fabs(apq);
            if (sweep > 0 && fabs(d[p]) + g == fabs(d[p]) && fabs(d[q]) + g == fabs(d[q])) {
                apq = 0.0;
                continue;
            }
            const double h = d[q] - d[p];
            double t;
            if (fabs(h) + g == fabs(h)) {
                t = apq / h;
            } else {
                const double theta = 0.5 * h / apq;
                t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
                if (theta < 0.0) t = -t;
            }
            const double c = rsqrt(fma(t, t, 1.0)), sn = t * c, tau = sn / (1.0 + c);
            const double ht = t * apq;
            d[p] -= ht;
            d[q] += ht;
            apq = 0.0;
            const double x = apr, y = aqr;  // rotate (p, r) and (q, r)
            apr = x - sn * (y + x * tau);
            aqr = y + sn * (x - y * tau);
        }
    }
    double e0 = d[0], e1 = d[1], e2 = d[2], tmp;
    if (e0 < e1) tmp = e0, e0 = e1, e1 = tmp;
    if (e1 < e2) tmp = e1, e1 = e2, e2 = tmp;
    if (e0 < e1) tmp = e0, e0 = e1, e1 = tmp;
    p1 = e0;
    p2 = e1;
    p3 = e2;
}

__global__ void __launch_bounds__(256) k_stress_node(int64_t n_node, const int32_t* __restrict__ ne_ptr,
                                                     const int32_t* __restrict__ ne_list,
                                                     const int32_t* __restrict__ co_elem,
                                                     const double* __restrict__ rec, double* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_node) return;
    double v[6] = {0, 0, 0, 0, 0, 0};
    const int ks = ne_ptr[i], ke = ne_ptr[i + 1];
    for (int k = ks; k < ke; ++k) {
        const int ent = __ldg(ne_list + k);
        const double* r = rec + (int64_t(ent >> 3) * 8 + (ent & 7)) * 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] += __ldg(r + c);
    }
    const double rce = 1.0 / double(co_elem[i]);
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] *= rce;
    double p1, p2, p3;
    // vector order [xx, yy, zz, xy, yz, xz] (POST_process.py:79-86)
    sym3_eig_desc(v[0], v[1], v[2], v[3], v[4], v[5], p1, p2, p3);
    double* o = out + 10 * i;
#pragma unroll
    for (int c = 0; c < 6; ++c) o[c] = v[c];
    o[6] = p1;
    o[7] = p2;
    o[8] = p3;
    o[9] = sqrt((p1 - p2) * (p1 - p2) + (p2 - p3) * (p2 - p3) + (p3 - p2) * (p3 - p2));
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" size_t fem_stress_workspace_bytes(int64_t n_elem) {
    return n_elem > 0 ? size_t(n_elem) * 48 * sizeof(double) : 0;
}

namespace fem {
int launch_stress_dd(const fem_mesh* mesh, const fem_material* mat, const double* u, const int32_t* co_elem,
                     const double* extrap, double* out, void* workspace, cudaStream_t st);
}

extern "C" int fem_stress_ex(const fem_mesh* mesh, const fem_material* mat, const double* u, const int32_t* co_elem,
                             const double* extrap, double* out, void* workspace, size_t workspace_bytes, int algo,
                             void* stream) {
    FEM_REQUIRE(mesh && mat && extrap, "mesh/mat/extrap is NULL");
    FEM_REQUIRE(mesh->n_node >= 0 && mesh->n_elem >= 0, "negative mesh size");
    FEM_REQUIRE(mesh->n_elem < (int64_t(1) << 28), "n_elem too large");
    FEM_REQUIRE(mat->PO > -1.0 && mat->PO < 0.5, "Poisson ratio must lie in (-1, 0.5)");
    if (mesh->n_node == 0) return FEM_OK;
    FEM_REQUIRE(u && co_elem && out && mesh->ne_ptr && mesh->ne_list, "u/co_elem/out/incidence is NULL");
    if (mesh->n_elem) FEM_REQUIRE(mesh->xyz && mesh->conn && aligned16(mesh->conn), "xyz/conn NULL or misaligned");
    if (workspace_bytes < fem_stress_workspace_bytes(mesh->n_elem) || (mesh->n_elem && !workspace)) {
        set_error("workspace too small: need %zu bytes", fem_stress_workspace_bytes(mesh->n_elem));
        return FEM_ERR_WORKSPACE;
    }
    FEM_REQUIRE(algo == FEM_ALGO_DD || algo == FEM_ALGO_FP64, "bad algo");
    FEM_REQUIRE(workspace == nullptr || aligned16(workspace), "workspace not 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    if (algo == FEM_ALGO_DD) return launch_stress_dd(mesh, mat, u, co_elem, extrap, out, workspace, st);
    if (mesh->n_elem) {
        StressParams sp;
        sp.xyz = mesh->xyz;
        sp.conn4 = reinterpret_cast<const int4*>(mesh->conn);
        sp.u = u;
        sp.n_elem = mesh->n_elem;
        sp.rec = static_cast<double*>(workspace);
        const double EX = mat->EX, PO = mat->PO;
        sp.D0d = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO);  // POST_process.py:292-302
        sp.lam = EX * PO / (1 + PO) / (1 - 2 * PO);
        sp.mu = EX / 2 / (1 + PO);                          // :304-306
        // distinct rows of the table (exactly equal rows share one)
        std::memset(sp.W, 0, sizeof(sp.W));
        sp.nrow = 0;
        for (int j = 0; j < 8; ++j) {
            int r = 0;
            while (r < sp.nrow && std::memcmp(sp.W[r], extrap + 8 * j, sizeof(double) * 8) != 0) ++r;
            if (r == sp.nrow) {
                for (int k = 0; k < 8; ++k) sp.W[r][k] = extrap[8 * j + k];
                ++sp.nrow;
            }
            sp.row_of[j] = r;
        }
        const int64_t blocks = (mesh->n_elem + kEpc - 1) / kEpc;
        k_stress_element<<<unsigned(blocks), kThreads, 0, st>>>(sp);
        FEM_LAUNCH_CHECK("k_stress_element");
    }
    const int64_t blocks = (mesh->n_node + 255) / 256;
    k_stress_node<<<unsigned(blocks), 256, 0, st>>>(mesh->n_node, mesh->ne_ptr, mesh->ne_list, co_elem,
                                                    static_cast<const double*>(workspace), out);
    FEM_LAUNCH_CHECK("k_stress_node");
    return FEM_OK;
}

extern "C" int fem_stress(const fem_mesh* mesh, const fem_material* mat, const double* u, const int32_t* co_elem,
                          const double* extrap, double* out, void* workspace, size_t workspace_bytes, void* stream) {
    return fem_stress_ex(mesh, mat, u, co_elem, extrap, out, workspace, workspace_bytes, FEM_ALGO_FP64, stream);
}

// ---- allocation-free variant ------------------------------------------------------------------
// Some callers cannot allocate device memory at all: plug-ins living inside a host program that
// owns every device allocation and only lends them input/output buffers, or latency-critical
// loops where cudaMalloc/cudaFree are forbidden because they synchronise the device.  For them
// fem_stress_noalloc runs the same two stress kernels with their per-element scratch placed in
// this file-scope device array instead of a caller workspace.  The array is reserved on every
// GPU that loads this library and stays there until the process exits.
namespace {

static __device__ __align__(256) double g_stress_scratch[size_t(FEM_STRESS_NOALLOC_MAX_ELEMS) * 48];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_stress_scratch on the current device, looked up once per device (the
// host-side symbol is only a stand-in and must never be handed to a kernel).
int scratch_address(void** out) {
    int dev = 0;
    FEM_CUDA(cudaGetDevice(&dev));
    FEM_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        FEM_CUDA(cudaGetSymbolAddress(&p, g_stress_scratch));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return FEM_OK;
}

}  // namespace

extern "C" int fem_stress_noalloc(const fem_mesh* mesh, const fem_material* mat, const double* u,
                                  const int32_t* co_elem, const double* extrap, double* out, void* stream) {
    FEM_REQUIRE(mesh != nullptr, "mesh is NULL");
    if (mesh->n_elem > FEM_STRESS_NOALLOC_MAX_ELEMS) {
        set_error("fem_stress_noalloc: %lld elements exceed the built-in scratch limit of %d elements; "
                  "use fem_stress with a caller-allocated workspace",
                  (long long)mesh->n_elem, FEM_STRESS_NOALLOC_MAX_ELEMS);
        return FEM_ERR_WORKSPACE;
    }
    void* scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    // Every element record is fully rewritten by the element kernel before the node kernel
    // reads it, so nothing in the shared scratch has to be cleared between calls.
    return fem_stress(mesh, mat, u, co_elem, extrap, out, scratch, sizeof(g_stress_scratch), stream);
}

// ---- double-float variant (FEM_ALGO_DD; fem_stress runs FEM_ALGO_FP64) ----------------------------
// Same two kernels and record size as above, with the FP64 arithmetic moved to double-float
// on the FP32 pipes (fem_dd.cuh): node coordinates and displacements are made element-local
// in FP64 first (the gradient only depends on differences), the corner values are stored as
// float pairs, and the node kernel sums, averages and diagonalises in double-float (cyclic
// Jacobi, threshold 2^-46 of the diagonal), forming the FP64 outputs at the end.
namespace fem {
namespace {

struct StressDdParams {
    const double* xyz;
    const int4* conn4;
    const double* u;
    int64_t n_elem;
    const int32_t* ne_inv;  // NULL: record of (e, j) at e*8+j; else at ne_inv[e*8+j] (row order)
    float2* rec;            // 8 * n_elem records of 6 float pairs
    float2 D0d, lam, mu;
    float2 dnr[8][8][3];
    float2 W[8][8];  // the distinct rows of the caller's extrapolation table
    int nrow;        // how many
    int row_of[8];   // corner j -> its row of W
};

struct StressDdSmem {
    float2 dnr[8][8][3];
    float2 W[8][8];
    float2 res[kEpc][8][6];  // extrapolated values of each distinct table row
    float2 x[kEpc][8][3];
    float2 u[kEpc][8][3];
    float2 sv[kEpc][8][kSvPad];
};

__device__ __forceinline__ dd ldp(const float2& v) { return dd{v.x, v.y}; }
__device__ __forceinline__ float2 stp(dd v) { return make_float2(v.hi, v.lo); }

__global__ void __launch_bounds__(kThreads) k_stress_element_dd(const StressDdParams p) {
    __shared__ StressDdSmem s;
    const int tid = threadIdx.x;
    const int el = tid >> 3;
    const int t = tid & 7;
    const int64_t e = int64_t(blockIdx.x) * kEpc + el;
    const bool valid = e < p.n_elem;
    for (int k = tid; k < 8 * 8 * 3; k += kThreads) (&s.dnr[0][0][0])[k] = (&p.dnr[0][0][0])[k];
    for (int k = tid; k < 64; k += kThreads) (&s.W[0][0])[k] = (&p.W[0][0])[k];
    if (valid) {
        const int* cn = reinterpret_cast<const int*>(p.conn4) + 8 * e;
        const int64_t node = __ldg(cn + t), node0 = __ldg(cn);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            s.x[el][t][i] = stp(dd_from_double(__ldg(p.xyz + 3 * node + i) - __ldg(p.xyz + 3 * node0 + i)));
            s.u[el][t][i] = stp(dd_from_double(__ldg(p.u + 3 * node + i) - __ldg(p.u + 3 * node0 + i)));
        }
    }
    __syncthreads();
    if (valid) {
        const int g = t;
        dd J[3][3], G[3][3];
        {
            dd_acc aj[3][3], ag[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int d = 0; d < 3; ++d) aj[i][d] = ag[i][d] = acc_zero();
            // corner loop kept rolled: the unrolled form overflows the instruction cache
#pragma unroll 1
            for (int a = 0; a < 8; ++a) {
                dd c[3], xa[3], ua[3];
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    c[i] = ldp(s.dnr[g][a][i]);
                    xa[i] = ldp(s.x[el][a][i]);
                    ua[i] = ldp(s.u[el][a][i]);
                }
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        acc_fma(aj[i][d], xa[i], c[d]);
                        acc_fma(ag[i][d], ua[i], c[d]);
                    }
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    J[i][d] = acc_value(aj[i][d]);
                    G[i][d] = acc_value(ag[i][d]);
                }
        }
        dd A[3][3];
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
        const dd inv = dd_rcp(acc_value(da));
        dd H[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                dd_acc acc = acc_zero();
                acc_fma(acc, G[i][0], A[0][k]);
                acc_fma(acc, G[i][1], A[1][k]);
                acc_fma(acc, G[i][2], A[2][k]);
                H[i][k] = dd_mul(acc_value(acc), inv);
            }
        const dd D0d = ldp(p.D0d), lam = ldp(p.lam), mu = ldp(p.mu);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            dd_acc acc = acc_zero();
            acc_fma(acc, D0d, H[i][i]);
            acc_fma(acc, lam, H[(i + 1) % 3][(i + 1) % 3]);
            acc_fma(acc, lam, H[(i + 2) % 3][(i + 2) % 3]);
            s.sv[el][g][i] = stp(acc_value(acc));
        }
        s.sv[el][g][3] = stp(dd_mul(mu, dd_add(H[0][1], H[1][0])));
        s.sv[el][g][4] = stp(dd_mul(mu, dd_add(H[1][2], H[2][1])));
        s.sv[el][g][5] = stp(dd_mul(mu, dd_add(H[0][2], H[2][0])));
    }
    __syncthreads();
    // the table's distinct rows only, spread over the element's threads (as the FP64 kernel)
    if (valid) {
        const int nout = p.nrow * 6;
        for (int o = t; o < nout; o += 8) {
            const int r = o / 6, c = o - 6 * r;
            dd_acc acc = acc_zero();
#pragma unroll
            for (int k = 0; k < 8; ++k) acc_fma(acc, ldp(s.W[r][k]), ldp(s.sv[el][k][c]));
            s.res[el][r][c] = stp(acc_value(acc));
        }
    }
    __syncthreads();
    if (!valid) return;
    const int j = t, r = p.row_of[j];
    const int64_t slot = p.ne_inv ? int64_t(__ldg(p.ne_inv + e * 8 + j)) : e * 8 + j;
    float2* o = p.rec + slot * 6;
#pragma unroll
    for (int c = 0; c < 6; ++c) o[c] = s.res[el][r][c];
}

// Cyclic Jacobi on a symmetric 3x3 in double-float; returns the eigenvalues descending.
__device__ void sym3_eig_desc_dd(dd (&a)[3][3], dd& p1, dd& p2, dd& p3) {
    for (int sweep = 0; sweep < 16; ++sweep) {
        const float off = fabsf(a[0][1].hi) + fabsf(a[0][2].hi) + fabsf(a[1][2].hi);
        const float dia = fabsf(a[0][0].hi) + fabsf(a[1][1].hi) + fabsf(a[2][2].hi);
        if (!(off > 0.f) || off <= 1.4210855e-14f * dia) break;  // 2^-46
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int pp = pq == 2 ? 1 : 0;
            const int qq = pq == 0 ? 1 : 2;
            const dd apq = a[pp][qq];
            if (apq.hi == 0.f) continue;
            const dd theta = dd_div(dd_sub(a[qq][qq], a[pp][pp]), dd_add(apq, apq));
            dd tt;
            if (fabsf(theta.hi) > 1e18f) {
                tt = dd_rcp(dd_add(theta, theta));
            } else {
                const dd r = dd_sqrt(dd_add(dd_mul(theta, theta), dd_from_float(1.f)));
                tt = dd_rcp(dd_add(dd_abs(theta), r));
                if (theta.hi < 0.f) tt = dd_neg(tt);
            }
            const dd c = dd_rcp(dd_sqrt(dd_add(dd_mul(tt, tt), dd_from_float(1.f))));
            const dd sn = dd_mul(tt, c);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const dd akp = a[k][pp], akq = a[k][qq];
                a[k][pp] = dd_sub(dd_mul(c, akp), dd_mul(sn, akq));
                a[k][qq] = dd_add(dd_mul(sn, akp), dd_mul(c, akq));
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const dd apk = a[pp][k], aqk = a[qq][k];
                a[pp][k] = dd_sub(dd_mul(c, apk), dd_mul(sn, aqk));
                a[qq][k] = dd_add(dd_mul(sn, apk), dd_mul(c, aqk));
            }
        }
    }
    dd e0 = a[0][0], e1 = a[1][1], e2 = a[2][2], tmp;
    if (dd_lt(e0, e1)) tmp = e0, e0 = e1, e1 = tmp;
    if (dd_lt(e1, e2)) tmp = e1, e1 = e2, e2 = tmp;
    if (dd_lt(e0, e1)) tmp = e0, e0 = e1, e1 = tmp;
    p1 = e0;
    p2 = e1;
    p3 = e2;
}

__global__ void __launch_bounds__(256) k_stress_node_dd(int64_t n_node, const int32_t* __restrict__ ne_ptr,
                                                        const int32_t* __restrict__ ne_list,
                                                        const int32_t* __restrict__ co_elem,
                                                        const float2* __restrict__ rec, int row_ordered,
                                                        double* __restrict__ out) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_node) return;
    dd_acc acc[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) acc[c] = acc_zero();
    const int ks = ne_ptr[i], ke = ne_ptr[i + 1];
    for (int k = ks; k < ke; ++k) {
        int64_t slot = k;  // row order: this node's corner records are contiguous
        if (!row_ordered) {
            const int ent = __ldg(ne_list + k);
            slot = int64_t(ent >> 3) * 8 + (ent & 7);
        }
        const float4* r = reinterpret_cast<const float4*>(rec + slot * 6);  // 48 bytes, 16-byte aligned
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float4 v = __ldg(r + q);
            acc_add(acc[2 * q], dd{v.x, v.y});
            acc_add(acc[2 * q + 1], dd{v.z, v.w});
        }
    }
    double* o = out + 10 * i;
    const int ce = co_elem[i];
    if (ce == 0) {  // 0 / 0 as the reference's average (POST_process.py:186)
        const double nan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
        for (int c = 0; c < 10; ++c) o[c] = nan;
        return;
    }
    const dd inv = dd_rcp(dd_from_float(float(ce)));
    dd v[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) v[c] = dd_mul(acc_value(acc[c]), inv);
    // vector order [xx, yy, zz, xy, yz, xz] (POST_process.py:79-86)
    dd a[3][3] = {{v[0], v[3], v[5]}, {v[3], v[1], v[4]}, {v[5], v[4], v[2]}};
    dd p1, p2, p3;
    sym3_eig_desc_dd(a, p1, p2, p3);
    const dd d12 = dd_sub(p1, p2), d23 = dd_sub(p2, p3);
    // "VM" as written at POST_process.py:93-94: (p1-p2)^2 + (p2-p3)^2 + (p3-p2)^2
    const dd vm = dd_sqrt(dd_add(dd_mul(d12, d12), dd_add(dd_mul(d23, d23), dd_mul(d23, d23))));
#pragma unroll
    for (int c = 0; c < 6; ++c) o[c] = dd_to_double(v[c]);
    o[6] = dd_to_double(p1);
    o[7] = dd_to_double(p2);
    o[8] = dd_to_double(p3);
    o[9] = dd_to_double(vm);
}

void split2(double x, float2& o) {
    const float hi = float(x);
    o = make_float2(hi, float(x - double(hi)));
}

}  // namespace

int launch_stress_dd(const fem_mesh* mesh, const fem_material* mat, const double* u, const int32_t* co_elem,
                     const double* extrap, double* out, void* workspace, cudaStream_t st) {
    if (mesh->n_elem) {
        StressDdParams sp;
        sp.xyz = mesh->xyz;
        sp.conn4 = reinterpret_cast<const int4*>(mesh->conn);
        sp.u = u;
        sp.n_elem = mesh->n_elem;
        sp.ne_inv = mesh->ne_inv;
        sp.rec = static_cast<float2*>(workspace);
        const double EX = mat->EX, PO = mat->PO;
        split2(EX * (1 - PO) / (1 + PO) / (1 - 2 * PO), sp.D0d);  // POST_process.py:292-302
        split2(EX * PO / (1 + PO) / (1 - 2 * PO), sp.lam);
        split2(EX / 2 / (1 + PO), sp.mu);                          // :304-306
        const ShapeTables& T = shape_tables();
        for (int g = 0; g < 8; ++g)
            for (int a = 0; a < 8; ++a)
                for (int d = 0; d < 3; ++d) split2(T.dnr[g][a][d], sp.dnr[g][a][d]);
        // distinct rows of the table (exactly equal rows share one), split into float pairs
        std::memset(sp.W, 0, sizeof(sp.W));
        int first[8];  // the first corner of each distinct row
        sp.nrow = 0;
        for (int j = 0; j < 8; ++j) {
            int r = 0;
            while (r < sp.nrow && std::memcmp(extrap + 8 * first[r], extrap + 8 * j, sizeof(double) * 8) != 0) ++r;
            if (r == sp.nrow) {
                for (int k = 0; k < 8; ++k) split2(extrap[8 * j + k], sp.W[r][k]);
                first[r] = j;
                ++sp.nrow;
            }
            sp.row_of[j] = r;
        }
        const int64_t blocks = (mesh->n_elem + kEpc - 1) / kEpc;
        k_stress_element_dd<<<unsigned(blocks), kThreads, 0, st>>>(sp);
        FEM_LAUNCH_CHECK("k_stress_element_dd");
    }
    const int64_t blocks = (mesh->n_node + 255) / 256;
    k_stress_node_dd<<<unsigned(blocks), 256, 0, st>>>(mesh->n_node, mesh->ne_ptr, mesh->ne_list, co_elem,
                                                       static_cast<const float2*>(workspace),
                                                       mesh->ne_inv != nullptr, out);
    FEM_LAUNCH_CHECK("k_stress_node_dd");
    return FEM_OK;
}

}  // namespace fem
