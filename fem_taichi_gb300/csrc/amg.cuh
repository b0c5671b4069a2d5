// Smoothed-aggregation algebraic multigrid (SA-AMG) preconditioner: hierarchy types shared
// by the host setup (amg_setup.cpp), the device V-cycle (amg.cu) and the solver (pcg.cu).
//
// Level l holds the operator A_l as a BSR matrix with b_l x b_l blocks (b_0 = 3 DOF per
// node; every coarser "node" is an aggregate carrying 6 rigid-body DOF), the inverses of its
// diagonal blocks, the prolongator P_l (n_l x n_{l+1} block rows / columns, b_l x 6 blocks)
// and the restriction R_l = P_l^T.  The last level is solved with a dense inverse.
#pragma once

#include <stdint.h>

#include <vector>

#include "fem_common.cuh"

namespace fem {
namespace amg {

constexpr int kModes = 6;  // near-null space: 3 translations + 3 rotations

// Host BSR matrix, FP64, blocks br x bc stored row-major, 64-bit row pointers.
struct HostBsr {
    int64_t n = 0, m = 0;  // block rows, block columns
    int br = 0, bc = 0;
    std::vector<int64_t> ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    int64_t nnzb() const { return ptr.empty() ? 0 : ptr.back(); }
};

// Device BSR matrix, FP32, 32-bit row pointers, values in two layouts (amg.cu).
struct DevBsr {
    int64_t n = 0, m = 0;
    int br = 0, bc = 0;
    int64_t nnzb = 0;
    int32_t* ptr = nullptr;
    int32_t* col = nullptr;
    float* val = nullptr;   // row-SoA values
    float* valb = nullptr;  // block-major values
};

// Device BSR matrix, FP64, block-major values (block l at val[l * br * bc], row-major), 32-bit
// row pointers: the matrices of a hierarchy set up on the device (amg_device.cu), kept for
// the next level's setup and for fem_amg_export.
struct Dev64 {
    int64_t n = 0, m = 0;
    int br = 0, bc = 0;
    int64_t nnzb = 0;
    int32_t* ptr = nullptr;
    int32_t* col = nullptr;
    double* val = nullptr;
};

struct Level {
    int b = 0;       // DOF per node
    int64_t n = 0;   // nodes
    HostBsr A;       // operator (empty on level 0 after setup: the solver's matrix is used)
    std::vector<double> dinv;     // [n][b][b] inverses of the diagonal blocks
    HostBsr P, R;                 // prolongator and restriction (not on the last level)
    std::vector<int32_t> agg;     // aggregate of each node, -1 = none (not on the last level)
    std::vector<uint8_t> iso;     // 1: unaggregated (Dirichlet) node, x = D^-1 b in the cycle
    double lmax = 0.0;            // estimate of the spectral radius of D^-1 A
    double omega = 0.0;           // prolongator smoothing weight 4 / (3 lmax)
    double setup_s = 0.0;         // host seconds spent on this level
    // Chebyshev smoother coefficients: step k adds d_k = c1[k] d_{k-1} + c2[k] D^-1 r_k
    std::vector<float> c1, c2;
    // device copies
    DevBsr dA, dP, dR;
    float* d_dinv = nullptr;
    uint8_t* d_iso = nullptr;
    int32_t* d_iso_rows = nullptr;  // indices of the Dirichlet rows (level 0)
    int64_t n_iso = 0;
    float* vfix = nullptr;          // [n_iso][b][nrhs] scratch of the Dirichlet-row update
    // FP64 device copies of a hierarchy set up on the device (A on levels >= 1)
    Dev64 gA, gP, gR;
    double* g_dinv = nullptr;
    // device vectors for the current nrhs ([n][b][nrhs]): right-hand side and output of this
    // level's cycle (levels >= 1), second iterate, Chebyshev direction, residual
    float *vb = nullptr, *vo = nullptr, *vx = nullptr, *vd = nullptr, *vr = nullptr;
};

}  // namespace amg
}  // namespace fem

// The opaque handle of the C interface.
struct fem_amg {
    fem_amg_opts opts{};
    std::vector<fem::amg::Level> lv;
    int64_t coarse_m = 0;                 // size of the dense coarse problem
    std::vector<double> coarse_inv;       // [coarse_m][coarse_m]
    float* d_coarse_inv = nullptr;
    int vec_nrhs = 0;                     // nrhs the device vectors are sized for
    float* r32 = nullptr;                 // FP32 copies of the FP64 solver's r and z (level 0)
    float* z32 = nullptr;
    void* d_state = nullptr;              // solver state used by fem_amg_vcycle (done = 0)
    double setup_s[6] = {0, 0, 0, 0, 0, 0};  // strength+aggregation, tentative, eigen, smoothing, Galerkin, coarse
    bool uploaded = false;
    bool device_setup = false;            // built by fem_amg_setup_device (FP64 copies on the device)
};

namespace fem {
namespace pcgd {
struct PcgState;
}
namespace amg {

// One V-cycle z = M^-1 r on the device for nrhs right-hand sides ([n][3][nrhs] vectors),
// A0 the level-0 operator in FP32 (the solver's matrix).  symmetric: finish with one
// block-Jacobi update of the level-0 Dirichlet rows (x_I += D_I^-1 (r - A x)_I), which makes
// the cycle the symmetric I, F, I product; without it the Dirichlet rows keep
// x_I = D_I^-1 r_I (no product of a penalty row with a coupled vector, as an FP32 solver
// needs).  Every kernel returns at once when st->done is set, so the sequence can sit
// inside a captured solver iteration.
template <typename View>
int vcycle(fem_amg* h, const View& A0, const float* r, float* z, const pcgd::PcgState* st, int nrhs, bool symmetric,
           cudaStream_t s);

// Allocates the per-level vectors for nrhs right-hand sides (grow only).
int ensure_vectors(fem_amg* h, int nrhs);

// Host steps shared by both setups (amg_setup.cpp).
constexpr int64_t kMaxDense = 8192;   // largest dense coarsest level accepted
// Sums over long vectors (Lanczos dot products, the centroid of the node coordinates) are
// taken in chunks of kSumChunk consecutive elements, each summed in order, and the chunk
// sums added in order: the same sequence of roundings on the host and on the device.
constexpr int64_t kSumChunk = 2048;
constexpr double kDecoupled2 = 1e-12; // squared scaled coupling below which a row is Dirichlet
// largest eigenvalue of the symmetric tridiagonal (alpha, beta[1..m-1]) by Sturm bisection
double tridiag_lmax(const std::vector<double>& alpha, const std::vector<double>& beta);
// Chebyshev smoother coefficients for `degree` steps on [cheb_upper lmax / cheb_ratio, cheb_upper lmax]
void chebyshev_coefficients(double lmax, const fem_amg_opts& o, int degree, std::vector<float>& c1,
                            std::vector<float>& c2);
// dense inverse with partial pivoting (a is overwritten); false if singular
bool dense_inverse_host(int64_t m, std::vector<double>& a, std::vector<double>& inv);
// Releases the device memory of a hierarchy (amg.cu).
void release_device(fem_amg* h);

}  // namespace amg
}  // namespace fem
