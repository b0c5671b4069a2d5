// Smoothed-aggregation AMG setup on the device (fem_amg_setup_device).  No reference
// counterpart: the reference factorises K with Pardiso (SOLVE_static.py:31-33).
//
// The hierarchy is the one amg_setup.cpp builds on the host -- the same strength measure,
// aggregation, tentative prolongator, Lanczos estimate of lambda_max(D^-1 A), smoothed
// prolongator P = (I - omega D^-1 A) T and Galerkin operator A_c = P^T (A P) -- computed by
// FP64 kernels from the solver's FP64 matrix, which never leaves the device.  Only the two
// order-dependent greedy passes of the aggregation run on the host (steps (a) and (c): a node
// starts an aggregate only if its strong neighbours are still free, so the result depends on
// the node order); they read the strong-connection flags (one byte per block).  Step (b)
// (join the most strongly coupled aggregate) is independent per node and runs on the device.
//
// The hierarchy is bit-identical to the host setup's: every value is produced by the same
// sequence of IEEE operations on both sides (this file is compiled with -fmad=false and the
// host setup with -ffp-contract=off, so neither fuses a multiply and an add on its own; the
// sparse products use explicit fma() on both sides), and every sum runs in the host's order
// -- per-row loops in the same order, long sums in kSumChunk chunks.
//
// Kernels (FP64):
//  k_diag        per row: diagonal position, Gauss-Jordan inverse of the diagonal block,
//                inverse Cholesky factor L_i^-1 (the strength scaling)
//  k_strength    per block: |L_i^-1 A_ij L_j^-T|_F^2, strong flag
//  k_tentative   one thread per aggregate: two-pass modified Gram-Schmidt of the aggregate's
//                rows of the near-null space (columns dropped when dependent)
//  k_spmv64 ...  Lanczos: block-row product, block-diagonal products, chunked dot products
//  k_prol_*      one warp per row: the distinct aggregates of the row's neighbours (sorted),
//                then P_ia = -omega D_i^-1 sum_j A_ij T_j (+ T_i on the row's own aggregate)
//  k_tr_*        R = P^T: column counts, scan, scatter, then a per-row sort by fine row
//  k_sg_*        Z = X Y one warp per row: distinct columns in a shared-memory hash table,
//                sorted; each output block accumulates X_l Y_t over the row's X entries l in
//                ascending order (the host's Gustavson order), lanes over (t, block entry)
// The FP32 copies the V-cycle reads (amg.cu) are written directly from the FP64 results.
#include <math.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "amg.cuh"
#include "pcg.cuh"

namespace fem {
namespace amg {
namespace {

using Clock = std::chrono::steady_clock;
double since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

constexpr int kT = 256;
constexpr int kWarps = kT / 32;
constexpr int kHashCap = 4096;     // distinct columns of one Galerkin row: at most 3/4 of this
constexpr int32_t kFree = -1, kAlone = -2;

unsigned grid(int64_t work, int threads) {
    return unsigned(std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, int64_t(1) << 20)));
}

// ---- device buffers ----------------------------------------------------------------------
struct DBuf {
    void* p = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { cudaFree(p); }
    int alloc(size_t bytes) {
        cudaFree(p);
        p = nullptr;
        return cuda_status(cudaMalloc(&p, std::max<size_t>(bytes, 16)), "cudaMalloc (AMG setup)");
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
    void* release() {
        void* q = p;
        p = nullptr;
        return q;
    }
};

#define FEM_TRY(expr)                 \
    do {                              \
        int _r = (expr);              \
        if (_r != FEM_OK) return _r;  \
    } while (0)

// ---- small dense blocks --------------------------------------------------------------------
// Gauss-Jordan inverse with partial pivoting of a B x B row-major block (the host's steps).
template <int B>
__device__ bool d_invert(const double* a, double* inv) {
    double m[B][2 * B];
    for (int i = 0; i < B; ++i)
        for (int j = 0; j < B; ++j) {
            m[i][j] = a[i * B + j];
            m[i][B + j] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < B; ++c) {
        int p = c;
        for (int r = c + 1; r < B; ++r)
            if (fabs(m[r][c]) > fabs(m[p][c])) p = r;
        if (!(fabs(m[p][c]) > 0.0)) return false;
        if (p != c)
            for (int j = 0; j < 2 * B; ++j) {
                const double t = m[p][j];
                m[p][j] = m[c][j];
                m[c][j] = t;
            }
        const double s = 1.0 / m[c][c];
        for (int j = 0; j < 2 * B; ++j) m[c][j] *= s;
        for (int r = 0; r < B; ++r) {
            if (r == c) continue;
            const double f = m[r][c];
            if (f != 0.0)
                for (int j = 0; j < 2 * B; ++j) m[r][j] -= f * m[c][j];
        }
    }
    for (int i = 0; i < B; ++i)
        for (int j = 0; j < B; ++j) inv[i * B + j] = m[i][B + j];
    return true;
}

// L^-1 of the Cholesky factor of a; a block that is not numerically SPD gets 1 / sqrt|a_pp|.
template <int B>
__device__ void d_inv_cholesky(const double* a, double* g) {
    double Lm[B][B];
    for (int r = 0; r < B; ++r)
        for (int c = 0; c < B; ++c) Lm[r][c] = 0.0;
    bool ok = true;
    for (int c = 0; c < B && ok; ++c) {
        double d = a[c * B + c];
        for (int k = 0; k < c; ++k) d -= Lm[c][k] * Lm[c][k];
        if (!(d > 0.0)) {
            ok = false;
            break;
        }
        Lm[c][c] = sqrt(d);
        for (int r = c + 1; r < B; ++r) {
            double v = a[r * B + c];
            for (int k = 0; k < c; ++k) v -= Lm[r][k] * Lm[c][k];
            Lm[r][c] = v / Lm[c][c];
        }
    }
    for (int q = 0; q < B * B; ++q) g[q] = 0.0;
    if (!ok) {
        for (int p = 0; p < B; ++p) {
            const double d = fabs(a[p * B + p]);
            g[p * B + p] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
        }
        return;
    }
    for (int c = 0; c < B; ++c)
        for (int r = 0; r < B; ++r) {
            double v = r == c ? 1.0 : 0.0;
            for (int k = 0; k < r; ++k) v -= Lm[r][k] * g[k * B + c];
            g[r * B + c] = v / Lm[r][r];
        }
}

// ---- diagonal, strength, aggregation helpers -------------------------------------------------
template <int B>
__global__ void k_diag(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, int32_t* dpos, double* dinv, double* G, int* bad) {
    constexpr int BB = B * B;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        int lo = ptr[i], hi = ptr[i + 1];
        const int end = hi;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (col[mid] < int(i)) lo = mid + 1;
            else hi = mid;
        }
        const int d = (lo < end && col[lo] == int(i)) ? lo : -1;
        dpos[i] = d;
        double* gi = G + i * BB;
        double* di = dinv + i * BB;
        if (d < 0) {
            atomicAdd(bad, 1);
            for (int q = 0; q < BB; ++q) {
                gi[q] = (q % (B + 1)) == 0 ? 1.0 : 0.0;
                di[q] = 0.0;
            }
            continue;
        }
        const double* a = val + int64_t(d) * BB;
        if (!d_invert<B>(a, di)) atomicAdd(bad, 1);
        d_inv_cholesky<B>(a, gi);
    }
}

__global__ void k_rowof(int64_t n, const int32_t* __restrict__ ptr, int32_t* rowof) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int l = ptr[i]; l < ptr[i + 1]; ++l) rowof[l] = int32_t(i);
}

template <int B>
__global__ void k_strength(int64_t nnzb, const int32_t* __restrict__ rowof, const int32_t* __restrict__ col,
                           const double* __restrict__ val, const double* __restrict__ G, double t2, uint8_t* strong,
                           double* sv) {
    constexpr int BB = B * B;
    for (int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; l < nnzb; l += int64_t(gridDim.x) * blockDim.x) {
        const int i = rowof[l], j = col[l];
        if (i == j) {
            strong[l] = 0;
            sv[l] = 0.0;
            continue;
        }
        const double* gi = G + int64_t(i) * BB;
        const double* gj = G + int64_t(j) * BB;
        const double* a = val + l * BB;
        double t[BB];
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) {
                double v = 0.0;
                for (int k = 0; k <= r; ++k) v += gi[r * B + k] * a[k * B + c];
                t[r * B + c] = v;
            }
        double f = 0.0;
        for (int r = 0; r < B; ++r)
            for (int c = 0; c < B; ++c) {
                double v = 0.0;
                for (int k = 0; k <= c; ++k) v += t[r * B + k] * gj[c * B + k];
                f += v * v;
            }
        strong[l] = f > t2 ? 1 : 0;
        sv[l] = f;
    }
}

// per row: the largest scaled coupling / B over the off-diagonal blocks
template <int B>
__global__ void k_maxc(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ sv, double* maxc) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double mx = 0.0;
        for (int l = ptr[i]; l < ptr[i + 1]; ++l)
            if (col[l] != int(i)) mx = fmax(mx, sv[l] / B);
        maxc[i] = mx;
    }
}

// aggregation step (b): a node left free by step (a) joins the step-(a) aggregate of its most
// strongly coupled aggregated strong neighbour (first maximum in column order)
__global__ void k_join(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const uint8_t* __restrict__ strong, const double* __restrict__ sv,
                       const int32_t* __restrict__ first, int32_t* agg) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        if (first[i] != kFree) {
            agg[i] = first[i];
            continue;
        }
        int32_t best = -1;
        double bs = -1.0;
        for (int l = ptr[i]; l < ptr[i + 1]; ++l) {
            if (!strong[l]) continue;
            const int32_t f = first[col[l]];
            if (f < 0) continue;
            if (sv[l] > bs) {
                bs = sv[l];
                best = f;
            }
        }
        agg[i] = best >= 0 ? best : kFree;
    }
}

__global__ void k_iso(int64_t n, const int32_t* __restrict__ agg, const double* __restrict__ maxc, uint8_t* iso) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        iso[i] = (agg[i] < 0 && maxc[i] < kDecoupled2) ? 1 : 0;
}

// ---- near-null space and tentative prolongator -----------------------------------------------
__global__ void k_rigid_modes(int64_t n, const double* __restrict__ xyz, double cx, double cy, double cz, double* Bn) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double x = xyz[3 * i] - cx, y = xyz[3 * i + 1] - cy, z = xyz[3 * i + 2] - cz;
        double* b = Bn + i * 3 * kModes;
        for (int q = 0; q < 3 * kModes; ++q) b[q] = 0.0;
        b[0 * kModes + 0] = 1.0;
        b[1 * kModes + 1] = 1.0;
        b[2 * kModes + 2] = 1.0;
        b[1 * kModes + 3] = -z;
        b[2 * kModes + 3] = y;
        b[0 * kModes + 4] = z;
        b[2 * kModes + 4] = -x;
        b[0 * kModes + 5] = -y;
        b[1 * kModes + 5] = x;
    }
}

// One thread per aggregate, in the host setup's order (amg_setup.cpp:tentative): T rows of
// the members (T[node][B][6], rows in member order) = the aggregate's rows of the near-null
// space, orthonormalised column by column by two-pass modified Gram-Schmidt; Bc[a] = R.
template <int B>
__global__ void k_tentative(int64_t na, const int32_t* __restrict__ aptr, const int32_t* __restrict__ mem,
                            const double* __restrict__ Bn, double* T, double* Bc) {
    constexpr int k = kModes;
    for (int64_t a = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; a < na; a += int64_t(gridDim.x) * blockDim.x) {
        const int s0 = aptr[a], cnt = aptr[a + 1] - s0, rows = cnt * B;
        auto rowp = [&](int r) { return T + (int64_t(mem[s0 + r / B]) * B + r % B) * k; };
        for (int r = 0; r < rows; ++r) {
            const double* src = Bn + (int64_t(mem[s0 + r / B]) * B + r % B) * k;
            double* dst = rowp(r);
            for (int m = 0; m < k; ++m) dst[m] = src[m];
        }
        double R[k][k];
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) R[i][j] = 0.0;
        for (int c = 0; c < k; ++c) {
            double n0 = 0.0;
            for (int r = 0; r < rows; ++r) n0 += rowp(r)[c] * rowp(r)[c];
            n0 = sqrt(n0);
            for (int pass = 0; pass < 2; ++pass)
                for (int c2 = 0; c2 < c; ++c2) {
                    double d = 0.0;
                    for (int r = 0; r < rows; ++r) d += rowp(r)[c2] * rowp(r)[c];
                    for (int r = 0; r < rows; ++r) rowp(r)[c] -= d * rowp(r)[c2];
                    R[c2][c] += d;
                }
            double nr = 0.0;
            for (int r = 0; r < rows; ++r) nr += rowp(r)[c] * rowp(r)[c];
            nr = sqrt(nr);
            if (nr > 1e-10 * n0 && nr > 0.0) {
                for (int r = 0; r < rows; ++r) rowp(r)[c] /= nr;
                R[c][c] = nr;
            } else {
                for (int r = 0; r < rows; ++r) rowp(r)[c] = 0.0;
                R[c][c] = 0.0;
            }
        }
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) Bc[(a * k + i) * k + j] = R[i][j];
    }
}

// ---- Lanczos estimate of lambda_max(D^-1 A) ---------------------------------------------------
template <int B>
__global__ void k_spmv64(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                         const double* __restrict__ val, const double* __restrict__ x, double* y) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double acc[B];
        for (int r = 0; r < B; ++r) acc[r] = 0.0;
        for (int l = ptr[i]; l < ptr[i + 1]; ++l) {
            const double* a = val + int64_t(l) * B * B;
            const double* xc = x + int64_t(col[l]) * B;
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) acc[r] += a[r * B + c] * xc[c];
        }
        for (int r = 0; r < B; ++r) y[i * B + r] = acc[r];
    }
}

// y = blockdiag(M) x with M either [n][B][B] (dpos == nullptr) or the diagonal blocks of A
template <int B>
__global__ void k_bapply(int64_t n, const double* __restrict__ M, const int32_t* __restrict__ dpos,
                         const double* __restrict__ x, double* y) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const double* m = dpos ? M + int64_t(dpos[i]) * B * B : M + i * B * B;
        for (int r = 0; r < B; ++r) {
            double s = 0.0;
            for (int c = 0; c < B; ++c) s += m[r * B + c] * x[i * B + c];
            y[i * B + r] = s;
        }
    }
}

__global__ void k_splitmix(int64_t N, double* v) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x) {
        uint64_t z = uint64_t(i) + 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        v[i] = double(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
}

// part[c] = sum over chunk c (kSumChunk consecutive elements, in order) of a[i] * b[i], or of
// a[i * stride + off] when b is null: the host setup's order (amg_setup.cpp:dot)
__global__ void k_chunk_sums(int64_t N, const double* __restrict__ a, const double* __restrict__ b, int stride,
                             int off, double* part) {
    const int64_t nc = (N + kSumChunk - 1) / kSumChunk;
    for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < nc; c += int64_t(gridDim.x) * blockDim.x) {
        const int64_t e = std::min(N, (c + 1) * kSumChunk);
        double s = 0.0;
        if (b) {
            for (int64_t i = c * kSumChunk; i < e; ++i) s += a[i] * b[i];
        } else {
            for (int64_t i = c * kSumChunk; i < e; ++i) s += a[i * stride + off];
        }
        part[c] = s;
    }
}

__global__ void k_lanczos_w(int64_t N, double* w, double a, const double* __restrict__ v, double bj,
                            const double* __restrict__ vp) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x)
        w[i] -= a * v[i] + bj * vp[i];
}

__global__ void k_div(int64_t N, const double* __restrict__ x, double s, double* y) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x)
        y[i] = x[i] / s;
}

// ---- warp-level distinct/sorted column lists ------------------------------------------------
// keys[0..L) (negative = skip) -> flags[q] = 1 on the first occurrence of each key
__device__ void mark_first(const int32_t* keys, int L, uint8_t* flags, int lane) {
    for (int q = lane; q < L; q += 32) {
        const int32_t k = keys[q];
        bool f = k >= 0;
        for (int p = 0; p < q && f; ++p) f = keys[p] != k;
        flags[q] = f ? 1 : 0;
    }
    __syncwarp();
}
__device__ int rank_of(const int32_t* keys, const uint8_t* flags, int L, int32_t k) {
    int r = 0;
    for (int p = 0; p < L; ++p) r += (flags[p] && keys[p] < k) ? 1 : 0;
    return r;
}

// ---- smoothed prolongator ------------------------------------------------------------------------
// per row: the number of distinct aggregates among the row's neighbours (0 on Dirichlet rows;
// P = T when not smoothing)
__global__ void k_prol_count(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                             const int32_t* __restrict__ agg, const uint8_t* __restrict__ iso, int smooth, int maxL,
                             int32_t* cnt) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* keys = reinterpret_cast<int32_t*>(smem) + w * maxL;
    uint8_t* flags = reinterpret_cast<uint8_t*>(reinterpret_cast<int32_t*>(smem) + kWarps * maxL) + w * maxL;
    const int64_t nw = int64_t(gridDim.x) * kWarps;
    for (int64_t i = int64_t(blockIdx.x) * kWarps + w; i < n; i += nw) {
        if (!smooth || iso[i]) {
            if (lane == 0) cnt[i] = (!smooth && agg[i] >= 0) ? 1 : 0;
            continue;
        }
        const int rs = ptr[i], L = ptr[i + 1] - rs;
        for (int q = lane; q < L; q += 32) keys[q] = agg[col[rs + q]];
        __syncwarp();
        mark_first(keys, L, flags, lane);
        int c = 0;
        for (int q = lane; q < L; q += 32) c += flags[q];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
        if (lane == 0) cnt[i] = c;
        __syncwarp();
    }
}

// Per row: the sorted distinct aggregates u of the row's neighbours (rank order), then for
// every (u, entry (r, c)) -- lanes over these items, so all lanes do FP64 work --
// acc = sum over the row's entries l with aggregate u, ascending, of sum_q A_il[r][q] T_l[q][c]
// (the host's Gustavson order), and P_iu = -omega D_i^-1 acc (+ T_i on the row's own
// aggregate).  Shared memory per warp: keys and first-occurrence flags (maxL each), the
// distinct keys (maxU) and the accumulators (maxU blocks).
template <int B>
__global__ void k_prol_fill(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            const double* __restrict__ val, const int32_t* __restrict__ agg,
                            const uint8_t* __restrict__ iso, int smooth, double omega, const double* __restrict__ dinv,
                            const double* __restrict__ T, int maxL, int maxU, int warps,
                            const int32_t* __restrict__ pptr, int32_t* pcol, double* pval) {
    constexpr int k = kModes, BK = B * k;
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per = size_t(maxU) * BK * sizeof(double) + size_t(maxL + maxU) * sizeof(int32_t) + maxL;
    const size_t per_al = (per + 15) & ~size_t(15);
    unsigned char* base = smem + w * per_al;
    double* acc = reinterpret_cast<double*>(base);
    int32_t* keys = reinterpret_cast<int32_t*>(acc + size_t(maxU) * BK);
    int32_t* ukeys = keys + maxL;
    uint8_t* flags = reinterpret_cast<uint8_t*>(ukeys + maxU);
    const int64_t nw = int64_t(gridDim.x) * warps;
    for (int64_t i = int64_t(blockIdx.x) * warps + w; i < n; i += nw) {
        if (!smooth) {
            if (lane == 0 && agg[i] >= 0) {
                const int p = pptr[i];
                pcol[p] = agg[i];
                for (int q = 0; q < BK; ++q) pval[int64_t(p) * BK + q] = T[i * BK + q];
            }
            continue;
        }
        if (iso[i]) continue;
        const int rs = ptr[i], L = ptr[i + 1] - rs;
        const int ps = pptr[i], U = pptr[i + 1] - ps;
        for (int q = lane; q < L; q += 32) keys[q] = agg[col[rs + q]];
        __syncwarp();
        mark_first(keys, L, flags, lane);
        for (int q = lane; q < L; q += 32)
            if (flags[q]) ukeys[rank_of(keys, flags, L, keys[q])] = keys[q];
        __syncwarp();
        for (int it = lane; it < U * BK; it += 32) {
            const int u = it / BK, e = it - u * BK, r = e / k, c = e - r * k;
            const int32_t kc = ukeys[u];
            double a = 0.0;
            for (int l = 0; l < L; ++l) {
                if (keys[l] != kc) continue;
                const double* ab = val + int64_t(rs + l) * B * B + r * B;
                const double* t = T + int64_t(col[rs + l]) * BK + c;
                for (int q = 0; q < B; ++q) a = fma(ab[q], t[q * k], a);
            }
            acc[it] = a;
        }
        __syncwarp();
        const double* di = dinv + i * B * B;
        const int32_t own = agg[i];
        for (int it = lane; it < U * BK; it += 32) {
            const int u = it / BK, e = it - u * BK, r = e / k, c = e - r * k;
            double sdot = 0.0;
            for (int q = 0; q < B; ++q) sdot += di[r * B + q] * acc[u * BK + q * k + c];
            double v = -omega * sdot;
            if (ukeys[u] == own) v += T[i * BK + e];
            pval[int64_t(ps + u) * BK + e] = v;
            if (e == 0) pcol[ps + u] = ukeys[u];
        }
        __syncwarp();
    }
}

// ---- transpose R = P^T -------------------------------------------------------------------------
__global__ void k_count_cols(int64_t nnz, const int32_t* __restrict__ c, int32_t* cnt) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nnz; e += int64_t(gridDim.x) * blockDim.x)
        atomicAdd(cnt + c[e], 1);
}

__global__ void k_tr_scatter(int64_t nnz, const int32_t* __restrict__ rowof, const int32_t* __restrict__ c,
                             const int32_t* __restrict__ rptr, int32_t* cursor, int32_t* rrow, int32_t* rsrc) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nnz; e += int64_t(gridDim.x) * blockDim.x) {
        const int32_t j = c[e];
        const int32_t slot = rptr[j] + atomicAdd(cursor + j, 1);
        rrow[slot] = rowof[e];
        rsrc[slot] = int32_t(e);
    }
}

// one warp per row of R: entries sorted by fine row (distinct keys), blocks transposed
template <int BR, int BC>
__global__ void k_tr_sort(int64_t nr, const int32_t* __restrict__ rptr, const int32_t* __restrict__ rrow,
                          const int32_t* __restrict__ rsrc, const double* __restrict__ pval, int32_t* rcol,
                          double* rval) {
    constexpr int BB = BR * BC;
    const int lane = threadIdx.x & 31;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t a = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; a < nr; a += nw) {
        const int rs = rptr[a], L = rptr[a + 1] - rs;
        for (int q = lane; q < L; q += 32) {
            const int32_t key = rrow[rs + q];
            int rk = 0;
            for (int p = 0; p < L; ++p) rk += rrow[rs + p] < key ? 1 : 0;
            const int dst = rs + rk;
            rcol[dst] = key;
            const double* s = pval + int64_t(rsrc[rs + q]) * BB;
            double* d = rval + int64_t(dst) * BB;
            for (int r = 0; r < BR; ++r)
                for (int c = 0; c < BC; ++c) d[c * BR + r] = s[r * BC + c];
        }
    }
}

// ---- sparse products Z = X Y -----------------------------------------------------------------------
__device__ __forceinline__ unsigned hslot(int32_t key, int lg) { return (unsigned(key) * 0x9E3779B1u) >> (32 - lg); }

// insert key; returns the slot, sets *fresh when the key was new; -1 when the table is full
__device__ int hinsert(int32_t* hk, int cap, int lg, int32_t key, bool* fresh) {
    unsigned h = hslot(key, lg);
    for (int probe = 0; probe < cap; ++probe) {
        const int32_t prev = atomicCAS(hk + h, -1, key);
        if (prev == -1) {
            *fresh = true;
            return int(h);
        }
        if (prev == key) {
            *fresh = false;
            return int(h);
        }
        h = (h + 1) & unsigned(cap - 1);
    }
    return -1;
}

__device__ int hfind(const int32_t* hk, int cap, int lg, int32_t key) {
    unsigned h = hslot(key, lg);
    for (int probe = 0; probe < cap; ++probe) {
        const int32_t v = hk[h];
        if (v == key) return int(h);
        if (v == -1) return -1;
        h = (h + 1) & unsigned(cap - 1);
    }
    return -1;
}

// cand[i] = sum of the lengths of the Y rows that X row i touches
__global__ void k_sg_cand(int64_t n, const int32_t* __restrict__ xptr, const int32_t* __restrict__ xcol,
                          const int32_t* __restrict__ yptr, int64_t* maxcand) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        int64_t c = 0;
        for (int l = xptr[i]; l < xptr[i + 1]; ++l) c += yptr[xcol[l] + 1] - yptr[xcol[l]];
        atomicMax(reinterpret_cast<unsigned long long*>(maxcand), static_cast<unsigned long long>(c));
    }
}

__global__ void k_max_len(int64_t n, const int32_t* __restrict__ ptr, int* out) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        atomicMax(out, ptr[i + 1] - ptr[i]);
}

// per row: number of distinct columns; status bit 1: a table ran full (or > 3/4 of kHashCap)
__global__ void k_sg_count(int64_t n, const int32_t* __restrict__ xptr, const int32_t* __restrict__ xcol,
                           const int32_t* __restrict__ yptr, const int32_t* __restrict__ ycol, int cap, int lg,
                           int32_t* cnt, int* maxu, int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* hk = reinterpret_cast<int32_t*>(smem) + w * cap;
    for (int q = lane; q < cap; q += 32) hk[q] = -1;
    __syncwarp();
    const int64_t nw = int64_t(gridDim.x) * kWarps;
    for (int64_t i = int64_t(blockIdx.x) * kWarps + w; i < n; i += nw) {
        int c = 0;
        bool full = false;
        for (int l = xptr[i]; l < xptr[i + 1]; ++l) {
            const int kk = xcol[l];
            for (int t = yptr[kk] + lane; t < yptr[kk + 1]; t += 32) {
                bool fresh = false;
                if (hinsert(hk, cap, lg, ycol[t], &fresh) < 0) full = true;
                c += fresh ? 1 : 0;
            }
        }
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
        full = __any_sync(0xffffffffu, full);
        if (lane == 0) {
            cnt[i] = c;
            atomicMax(maxu, c);
            if (full || 4 * c > 3 * cap) atomicOr(status, 2);
        }
        __syncwarp();
        for (int q = lane; q < cap; q += 32) hk[q] = -1;
        __syncwarp();
    }
}

// Z row i: sorted distinct columns, then z_(i,col) = sum over X entries l ascending of
// X_l Y_t (t: the entry of Y row xcol[l] with that column).  Per warp in shared memory: the
// hash keys and positions (cap each), the distinct keys and their slots (maxu each) and the
// positions of the current Y row (maxyl).
template <int BI, int BK, int BJ>
__global__ void k_sg_fill(int64_t n, const int32_t* __restrict__ xptr, const int32_t* __restrict__ xcol,
                          const double* __restrict__ xval, const int32_t* __restrict__ yptr,
                          const int32_t* __restrict__ ycol, const double* __restrict__ yval, int cap, int lg, int maxu,
                          int maxyl, int warps, const int32_t* __restrict__ zptr, int32_t* zcol, double* zval,
                          int* status) {
    constexpr int XB = BI * BK, YB = BK * BJ, ZB = BI * BJ;
    extern __shared__ __align__(16) unsigned char smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t per = size_t(2 * cap + 2 * maxu + maxyl + 1);
    int32_t* hk = reinterpret_cast<int32_t*>(smem) + w * per;
    int32_t* hv = hk + cap;
    int32_t* ul = hv + cap;
    int32_t* us = ul + maxu;
    int32_t* pb = us + maxu;
    int32_t* nu = pb + maxyl;
    for (int q = lane; q < cap; q += 32) hk[q] = -1;
    __syncwarp();
    const int64_t nw = int64_t(gridDim.x) * warps;
    for (int64_t i = int64_t(blockIdx.x) * warps + w; i < n; i += nw) {
        if (lane == 0) *nu = 0;
        __syncwarp();
        bool bad = false;
        for (int l = xptr[i]; l < xptr[i + 1]; ++l) {
            const int kk = xcol[l];
            for (int t = yptr[kk] + lane; t < yptr[kk + 1]; t += 32) {
                bool fresh = false;
                const int h = hinsert(hk, cap, lg, ycol[t], &fresh);
                if (h < 0) {
                    bad = true;
                } else if (fresh) {
                    const int u = atomicAdd(nu, 1);
                    if (u < maxu) {
                        ul[u] = ycol[t];
                        us[u] = h;
                    } else {
                        bad = true;
                    }
                }
            }
        }
        __syncwarp();
        bad = __any_sync(0xffffffffu, bad);
        const int U = *nu;
        const int zs = zptr[i];
        if (bad || U != zptr[i + 1] - zs) {
            if (lane == 0) atomicOr(status, 4);
        } else {
            for (int u = lane; u < U; u += 32) {
                const int32_t key = ul[u];
                int rk = 0;
                for (int p = 0; p < U; ++p) rk += ul[p] < key ? 1 : 0;
                hv[us[u]] = rk;
                zcol[zs + rk] = key;
            }
            for (int64_t q = lane; q < int64_t(U) * ZB; q += 32) zval[int64_t(zs) * ZB + q] = 0.0;
            __syncwarp();
            for (int l = xptr[i]; l < xptr[i + 1]; ++l) {
                const int kk = xcol[l], ts = yptr[kk], Lk = yptr[kk + 1] - ts;
                for (int t = lane; t < Lk; t += 32) {
                    const int h = hfind(hk, cap, lg, ycol[ts + t]);
                    pb[t] = h >= 0 ? hv[h] : -1;
                    if (h < 0) atomicOr(status, 4);
                }
                __syncwarp();
                const double* xb = xval + int64_t(l) * XB;
                for (int it = lane; it < Lk * ZB; it += 32) {
                    const int t = it / ZB, e = it - t * ZB, r = e / BJ, c = e - r * BJ;
                    if (pb[t] < 0) continue;
                    const double* yb = yval + int64_t(ts + t) * YB;
                    double* z = zval + (int64_t(zs) + pb[t]) * ZB + e;
                    double acc = *z;
#pragma unroll
                    for (int q = 0; q < BK; ++q) acc = fma(xb[r * BK + q], yb[q * BJ + c], acc);
                    *z = acc;
                }
                __syncwarp();
            }
        }
        for (int q = lane; q < cap; q += 32) hk[q] = -1;
        __syncwarp();
    }
}

// coarse DOF whose prolongator column is zero have an exactly zero row and column: unit diagonal
template <int B>
__global__ void k_unit_diag(int64_t n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                            double* val) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        for (int l = ptr[i]; l < ptr[i + 1]; ++l)
            if (col[l] == int(i)) {
                double* b = val + int64_t(l) * B * B;
                for (int d = 0; d < B; ++d)
                    if (b[d * B + d] == 0.0) b[d * B + d] = 1.0;
            }
}

// ---- FP32 copies for the V-cycle ---------------------------------------------------------------
__global__ void k_f32_layouts(int64_t n, const int32_t* __restrict__ ptr, const double* __restrict__ v64, int bb,
                              float* soa, float* blk) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int64_t rs = ptr[i], L = ptr[i + 1] - rs;
        for (int64_t l = 0; l < L; ++l)
            for (int q = 0; q < bb; ++q) {
                const float f = float(v64[(rs + l) * bb + q]);
                soa[bb * rs + q * L + l] = f;
                blk[(rs + l) * bb + q] = f;
            }
    }
}

__global__ void k_to_f32(int64_t N, const double* __restrict__ x, float* y) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < N; i += int64_t(gridDim.x) * blockDim.x)
        y[i] = float(x[i]);
}

// ================================================================================================
// host driver

struct Setup {
    fem_amg* H;
    cudaStream_t st;
    DBuf parts, status, tiles;
    size_t parts_n = 0;

    int sync() { return cuda_status(cudaStreamSynchronize(st), "cudaStreamSynchronize (AMG setup)"); }
    template <typename T>
    int down(std::vector<T>& h, const T* d, size_t count) {
        h.resize(count);
        if (count) FEM_CUDA(cudaMemcpyAsync(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost, st));
        return sync();
    }
    template <typename T>
    int up(T* d, const std::vector<T>& h) {
        if (!h.empty()) FEM_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, st));
        return sync();  // h may be freed by the caller
    }
    // sum over N of a[i] * b[i], or of a[i * stride + off] when b is null, in the host
    // setup's order: chunk sums on the device, added in chunk order here
    int dot(int64_t N, const double* a, const double* b, double& out, int stride = 1, int off = 0) {
        const int64_t nc = (N + kSumChunk - 1) / kSumChunk;
        if (int64_t(parts_n) < nc) {
            FEM_TRY(parts.alloc(sizeof(double) * nc));
            parts_n = size_t(nc);
        }
        k_chunk_sums<<<grid(nc, 64), 64, 0, st>>>(N, a, b, stride, off, parts.as<double>());
        FEM_LAUNCH_CHECK("k_chunk_sums");
        std::vector<double> h;
        FEM_TRY(down(h, parts.as<const double>(), size_t(nc)));
        double s = 0.0;
        for (double v : h) s += v;
        out = s;
        return FEM_OK;
    }
    int scan(int64_t n, const int32_t* cnt, int32_t* out) {
        FEM_TRY(tiles.alloc(sizeof(int64_t) * device_scan_tiles(n)));
        FEM_CUDA(cudaMemsetAsync(status.p, 0, sizeof(int), st));
        FEM_TRY(device_exclusive_scan(n, cnt, out, tiles.as<int64_t>(), status.as<int>(), st));
        int s = 0;
        FEM_CUDA(cudaMemcpyAsync(&s, status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        FEM_TRY(sync());
        FEM_REQUIRE(!(s & 2), "AMG setup: a matrix has more than 2^31 blocks");
        return FEM_OK;
    }
    int read_int(const int32_t* d, int64_t idx, int32_t& v) {
        FEM_CUDA(cudaMemcpyAsync(&v, d + idx, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        return sync();
    }
};

// A device FP64 matrix whose arrays are owned by DBufs until handed to a Level.
struct Mat {
    int64_t n = 0, m = 0;
    int br = 0, bc = 0;
    int64_t nnzb = 0;
    DBuf ptr, col, val;
    const int32_t* P() const { return ptr.as<const int32_t>(); }
    const int32_t* C() const { return col.as<const int32_t>(); }
    const double* V() const { return val.as<const double>(); }
    Dev64 hand_over() {
        Dev64 d;
        d.n = n;
        d.m = m;
        d.br = br;
        d.bc = bc;
        d.nnzb = nnzb;
        d.ptr = static_cast<int32_t*>(ptr.release());
        d.col = static_cast<int32_t*>(col.release());
        d.val = static_cast<double*>(val.release());
        return d;
    }
};

// A view of a device FP64 matrix (borrowed arrays).
struct View {
    int64_t n, m;
    int br, bc;
    int64_t nnzb;
    const int32_t* ptr;
    const int32_t* col;
    const double* val;
};
View view_of(const Mat& M) { return View{M.n, M.m, M.br, M.bc, M.nnzb, M.P(), M.C(), M.V()}; }

int max_row_len(Setup& S, const View& A, int& out) {
    DBuf d;
    FEM_TRY(d.alloc(sizeof(int)));
    FEM_CUDA(cudaMemsetAsync(d.p, 0, sizeof(int), S.st));
    k_max_len<<<grid(A.n, kT), kT, 0, S.st>>>(A.n, A.ptr, d.as<int>());
    FEM_LAUNCH_CHECK("k_max_len");
    FEM_CUDA(cudaMemcpyAsync(&out, d.p, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    return S.sync();
}

// Z = X Y (blocks X: BI x BK, Y: BK x BJ)
template <int BI, int BK, int BJ>
int spgemm(Setup& S, const View& X, const View& Y, Mat& Z) {
    Z.n = X.n;
    Z.m = Y.m;
    Z.br = BI;
    Z.bc = BJ;
    FEM_TRY(Z.ptr.alloc(sizeof(int32_t) * (X.n + 1)));
    int64_t maxcand = 0;
    {
        DBuf d;
        FEM_TRY(d.alloc(sizeof(int64_t)));
        FEM_CUDA(cudaMemsetAsync(d.p, 0, sizeof(int64_t), S.st));
        k_sg_cand<<<grid(X.n, kT), kT, 0, S.st>>>(X.n, X.ptr, X.col, Y.ptr, d.as<int64_t>());
        FEM_LAUNCH_CHECK("k_sg_cand");
        FEM_CUDA(cudaMemcpyAsync(&maxcand, d.p, sizeof(int64_t), cudaMemcpyDeviceToHost, S.st));
        FEM_TRY(S.sync());
    }
    int lg = 5;
    while ((int64_t(1) << lg) < 2 * maxcand && (1 << lg) < kHashCap) ++lg;
    int cap = 1 << lg;
    DBuf cnt, mx;
    FEM_TRY(cnt.alloc(sizeof(int32_t) * (X.n + 1)));
    FEM_TRY(mx.alloc(sizeof(int)));
    FEM_CUDA(cudaMemsetAsync(mx.p, 0, sizeof(int), S.st));
    FEM_CUDA(cudaMemsetAsync(S.status.p, 0, sizeof(int), S.st));
    const size_t smem_c = size_t(kWarps) * cap * sizeof(int32_t);
    FEM_CUDA(cudaFuncSetAttribute(k_sg_count, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_c)));
    k_sg_count<<<grid(X.n, kWarps), kT, smem_c, S.st>>>(X.n, X.ptr, X.col, Y.ptr, Y.col, cap, lg, cnt.as<int32_t>(),
                                                        mx.as<int>(), S.status.as<int>());
    FEM_LAUNCH_CHECK("k_sg_count");
    int maxu = 0, status = 0;
    FEM_CUDA(cudaMemcpyAsync(&maxu, mx.p, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    FEM_CUDA(cudaMemcpyAsync(&status, S.status.p, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    FEM_TRY(S.sync());
    FEM_REQUIRE(!(status & 2), "AMG device setup: a Galerkin row has more than %d distinct columns (use fem_amg_setup)",
                3 * kHashCap / 4);
    FEM_TRY(S.scan(X.n, cnt.as<int32_t>(), Z.ptr.as<int32_t>()));
    int32_t nnz = 0;
    FEM_TRY(S.read_int(Z.P(), X.n, nnz));
    Z.nnzb = nnz;
    FEM_TRY(Z.col.alloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
    FEM_TRY(Z.val.alloc(sizeof(double) * std::max<int64_t>(nnz, 1) * BI * BJ));
    int maxyl = 0;
    FEM_TRY(max_row_len(S, Y, maxyl));
    lg = 5;
    while ((1 << lg) < 2 * maxu) ++lg;
    cap = 1 << lg;
    maxu = std::max(maxu, 1);
    const size_t per = sizeof(int32_t) * (2 * size_t(cap) + 2 * size_t(maxu) + size_t(maxyl) + 1);
    int warps = kWarps;
    while (warps > 1 && per * warps > 200 * 1024) warps >>= 1;
    FEM_REQUIRE(per * warps <= 220 * 1024, "AMG device setup: a product row needs %zu bytes of shared memory", per);
    auto kern = k_sg_fill<BI, BK, BJ>;
    FEM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(per * warps)));
    FEM_CUDA(cudaMemsetAsync(S.status.p, 0, sizeof(int), S.st));
    kern<<<grid(X.n, warps), 32 * warps, per * warps, S.st>>>(X.n, X.ptr, X.col, X.val, Y.ptr, Y.col, Y.val, cap, lg,
                                                               maxu, maxyl, warps, Z.P(), Z.col.as<int32_t>(),
                                                               Z.val.as<double>(), S.status.as<int>());
    FEM_LAUNCH_CHECK("k_sg_fill");
    FEM_CUDA(cudaMemcpyAsync(&status, S.status.p, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    FEM_TRY(S.sync());
    FEM_REQUIRE(!(status & 4), "AMG device setup: inconsistent product row (internal error)");
    return FEM_OK;
}

template <int BR, int BC>
int transpose(Setup& S, const View& P, Mat& R) {
    R.n = P.m;
    R.m = P.n;
    R.br = BC;
    R.bc = BR;
    R.nnzb = P.nnzb;
    DBuf cnt, cursor, rowof, rrow, rsrc;
    FEM_TRY(cnt.alloc(sizeof(int32_t) * (R.n + 1)));
    FEM_TRY(cursor.alloc(sizeof(int32_t) * (R.n + 1)));
    FEM_TRY(rowof.alloc(sizeof(int32_t) * std::max<int64_t>(P.nnzb, 1)));
    FEM_TRY(rrow.alloc(sizeof(int32_t) * std::max<int64_t>(P.nnzb, 1)));
    FEM_TRY(rsrc.alloc(sizeof(int32_t) * std::max<int64_t>(P.nnzb, 1)));
    FEM_TRY(R.ptr.alloc(sizeof(int32_t) * (R.n + 1)));
    FEM_TRY(R.col.alloc(sizeof(int32_t) * std::max<int64_t>(P.nnzb, 1)));
    FEM_TRY(R.val.alloc(sizeof(double) * std::max<int64_t>(P.nnzb, 1) * BR * BC));
    FEM_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (R.n + 1), S.st));
    FEM_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int32_t) * (R.n + 1), S.st));
    k_rowof<<<grid(P.n, kT), kT, 0, S.st>>>(P.n, P.ptr, rowof.as<int32_t>());
    k_count_cols<<<grid(P.nnzb, kT), kT, 0, S.st>>>(P.nnzb, P.col, cnt.as<int32_t>());
    FEM_LAUNCH_CHECK("k_count_cols");
    FEM_TRY(S.scan(R.n, cnt.as<int32_t>(), R.ptr.as<int32_t>()));
    k_tr_scatter<<<grid(P.nnzb, kT), kT, 0, S.st>>>(P.nnzb, rowof.as<int32_t>(), P.col, R.P(), cursor.as<int32_t>(),
                                                     rrow.as<int32_t>(), rsrc.as<int32_t>());
    FEM_LAUNCH_CHECK("k_tr_scatter");
    k_tr_sort<BR, BC><<<grid(R.n, kWarps), kT, 0, S.st>>>(R.n, R.P(), rrow.as<int32_t>(), rsrc.as<int32_t>(), P.val,
                                                          R.col.as<int32_t>(), R.val.as<double>());
    FEM_LAUNCH_CHECK("k_tr_sort");
    return S.sync();
}

// FP32 copy (row-SoA + block-major) of a device FP64 matrix for the V-cycle
int to_devbsr(Setup& S, const View& M, DevBsr& D) {
    D.n = M.n;
    D.m = M.m;
    D.br = M.br;
    D.bc = M.bc;
    D.nnzb = M.nnzb;
    const int64_t bb = int64_t(M.br) * M.bc, nv = std::max<int64_t>(M.nnzb, 1) * bb;
    FEM_CUDA(cudaMalloc(&D.ptr, sizeof(int32_t) * (M.n + 1)));
    FEM_CUDA(cudaMalloc(&D.col, sizeof(int32_t) * std::max<int64_t>(M.nnzb, 1)));
    FEM_CUDA(cudaMalloc(&D.val, sizeof(float) * nv));
    FEM_CUDA(cudaMalloc(&D.valb, sizeof(float) * nv));
    FEM_CUDA(cudaMemcpyAsync(D.ptr, M.ptr, sizeof(int32_t) * (M.n + 1), cudaMemcpyDeviceToDevice, S.st));
    if (M.nnzb)
        FEM_CUDA(cudaMemcpyAsync(D.col, M.col, sizeof(int32_t) * M.nnzb, cudaMemcpyDeviceToDevice, S.st));
    k_f32_layouts<<<grid(M.n, kT), kT, 0, S.st>>>(M.n, M.ptr, M.val, int(bb), D.val, D.valb);
    FEM_LAUNCH_CHECK("k_f32_layouts");
    return FEM_OK;
}

template <int B>
int level_kernels(Setup& S, fem_amg* H, int l, const View& A, const double* Bnull_in, DBuf& Bnext, Mat& Anext,
                  const int32_t* hptr0, const int32_t* hcol0, bool& last) {
    const fem_amg_opts& o = H->opts;
    Level& L = H->lv[l];
    const int64_t n = A.n, m = n * B;
    constexpr int BB = B * B;
    DBuf dpos, G, dinv64, bad;
    FEM_TRY(dpos.alloc(sizeof(int32_t) * n));
    FEM_TRY(G.alloc(sizeof(double) * n * BB));
    FEM_TRY(dinv64.alloc(sizeof(double) * n * BB));
    FEM_TRY(bad.alloc(sizeof(int)));
    FEM_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), S.st));
    k_diag<B><<<grid(n, kT), kT, 0, S.st>>>(n, A.ptr, A.col, A.val, dpos.as<int32_t>(), dinv64.as<double>(),
                                            G.as<double>(), bad.as<int>());
    FEM_LAUNCH_CHECK("k_diag");
    int nbad = 0;
    FEM_CUDA(cudaMemcpyAsync(&nbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, S.st));
    FEM_TRY(S.sync());
    if (nbad) {
        set_error("AMG level %d: %d missing or singular diagonal blocks", l, nbad);
        return FEM_ERR_NOT_SPD;
    }
    FEM_CUDA(cudaMalloc(&L.d_dinv, sizeof(float) * n * BB));
    k_to_f32<<<grid(n * BB, kT), kT, 0, S.st>>>(n * BB, dinv64.as<double>(), L.d_dinv);
    FEM_LAUNCH_CHECK("k_to_f32");

    const bool last_by_size = m <= o.max_coarse || l + 1 >= o.max_levels;
    int64_t na = 0;
    DBuf sv, strong, maxc, agg, iso;
    if (!last_by_size) {
        const auto ta = Clock::now();
        DBuf rowof;
        FEM_TRY(rowof.alloc(sizeof(int32_t) * std::max<int64_t>(A.nnzb, 1)));
        FEM_TRY(sv.alloc(sizeof(double) * std::max<int64_t>(A.nnzb, 1)));
        FEM_TRY(strong.alloc(std::max<int64_t>(A.nnzb, 1)));
        FEM_TRY(maxc.alloc(sizeof(double) * n));
        k_rowof<<<grid(n, kT), kT, 0, S.st>>>(n, A.ptr, rowof.as<int32_t>());
        k_strength<B><<<grid(A.nnzb, kT), kT, 0, S.st>>>(A.nnzb, rowof.as<int32_t>(), A.col, A.val, G.as<double>(),
                                                         o.theta * o.theta * B, strong.as<uint8_t>(), sv.as<double>());
        FEM_LAUNCH_CHECK("k_strength");
        k_maxc<B><<<grid(n, kT), kT, 0, S.st>>>(n, A.ptr, A.col, sv.as<double>(), maxc.as<double>());
        FEM_LAUNCH_CHECK("k_maxc");
        // host steps (a) and (c) of the aggregation on the pattern and the strong flags
        std::vector<int32_t> hp, hc;
        const int32_t *pp = hptr0, *pc = hcol0;
        if (!pp || !pc) {
            FEM_TRY(S.down(hp, A.ptr, size_t(n + 1)));
            FEM_TRY(S.down(hc, A.col, size_t(A.nnzb)));
            pp = hp.data();
            pc = hc.data();
        }
        std::vector<uint8_t> hs;
        FEM_TRY(S.down(hs, strong.as<const uint8_t>(), size_t(A.nnzb)));
        std::vector<int32_t>& ag = L.agg;
        ag.assign(n, kFree);
        for (int64_t i = 0; i < n; ++i) {
            bool any = false;
            for (int32_t q = pp[i]; q < pp[i + 1] && !any; ++q) any = hs[q] != 0;
            if (!any) ag[i] = kAlone;
        }
        int32_t nagg = 0;
        for (int64_t i = 0; i < n; ++i) {  // (a)
            if (ag[i] != kFree) continue;
            bool ok = true;
            for (int32_t q = pp[i]; q < pp[i + 1] && ok; ++q)
                if (hs[q] && ag[pc[q]] != kFree) ok = false;
            if (!ok) continue;
            ag[i] = nagg;
            for (int32_t q = pp[i]; q < pp[i + 1]; ++q)
                if (hs[q]) ag[pc[q]] = nagg;
            ++nagg;
        }
        DBuf first;
        FEM_TRY(first.alloc(sizeof(int32_t) * n));
        FEM_TRY(agg.alloc(sizeof(int32_t) * n));
        FEM_TRY(S.up(first.as<int32_t>(), ag));
        k_join<<<grid(n, kT), kT, 0, S.st>>>(n, A.ptr, A.col, strong.as<uint8_t>(), sv.as<double>(),
                                             first.as<int32_t>(), agg.as<int32_t>());  // (b)
        FEM_LAUNCH_CHECK("k_join");
        FEM_TRY(S.down(ag, agg.as<const int32_t>(), size_t(n)));
        for (int64_t i = 0; i < n; ++i) {  // (c)
            if (ag[i] != kFree) continue;
            ag[i] = nagg;
            for (int32_t q = pp[i]; q < pp[i + 1]; ++q)
                if (hs[q] && ag[pc[q]] == kFree) ag[pc[q]] = nagg;
            ++nagg;
        }
        for (auto& a : ag)
            if (a == kAlone) a = -1;
        na = nagg;
        FEM_TRY(S.up(agg.as<int32_t>(), ag));
        FEM_TRY(iso.alloc(n));
        k_iso<<<grid(n, kT), kT, 0, S.st>>>(n, agg.as<int32_t>(), maxc.as<double>(), iso.as<uint8_t>());
        FEM_LAUNCH_CHECK("k_iso");
        FEM_TRY(S.down(L.iso, iso.as<const uint8_t>(), size_t(n)));
        H->setup_s[0] += since(ta);
    }
    if (last_by_size || na == 0 || na * kModes >= m) {
        // dense coarsest level
        last = true;
        FEM_REQUIRE(m <= kMaxDense, "AMG: level %d has %lld DOF and cannot be coarsened further (raise max_levels?)",
                    l, (long long)m);
        const auto tc = Clock::now();
        L.agg.clear();
        L.iso.clear();
        std::vector<int32_t> hp, hc;
        std::vector<double> hv;
        FEM_TRY(S.down(hp, A.ptr, size_t(n + 1)));
        FEM_TRY(S.down(hc, A.col, size_t(A.nnzb)));
        FEM_TRY(S.down(hv, A.val, size_t(A.nnzb) * BB));
        std::vector<double> dense(size_t(m) * m, 0.0);
        for (int64_t i = 0; i < n; ++i)
            for (int32_t q = hp[i]; q < hp[i + 1]; ++q)
                for (int r = 0; r < B; ++r)
                    for (int c = 0; c < B; ++c)
                        dense[(i * B + r) * m + int64_t(hc[q]) * B + c] = hv[(int64_t(q) * B + r) * B + c];
        H->coarse_m = m;
        if (!dense_inverse_host(m, dense, H->coarse_inv)) {
            set_error("AMG: the coarsest operator (%lld DOF) is singular", (long long)m);
            return FEM_ERR_NOT_SPD;
        }
        std::vector<float> ci(H->coarse_inv.begin(), H->coarse_inv.end());
        FEM_CUDA(cudaMalloc(&H->d_coarse_inv, sizeof(float) * ci.size()));
        FEM_TRY(S.up(H->d_coarse_inv, ci));
        L.g_dinv = static_cast<double*>(dinv64.release());
        H->setup_s[5] += since(tc);
        return FEM_OK;
    }
    last = false;
    // ---- Lanczos estimate of lambda_max(D^-1 A) ----
    {
        const auto te = Clock::now();
        const int64_t N = m;
        DBuf v, vp, u, w, Dw;
        for (DBuf* b : {&v, &vp, &u, &w, &Dw}) FEM_TRY(b->alloc(sizeof(double) * N));
        FEM_CUDA(cudaMemsetAsync(vp.p, 0, sizeof(double) * N, S.st));
        double *pv = v.as<double>(), *pvp = vp.as<double>();
        k_splitmix<<<grid(N, kT), kT, 0, S.st>>>(N, pv);
        k_bapply<B><<<grid(n, kT), kT, 0, S.st>>>(n, A.val, dpos.as<int32_t>(), pv, Dw.as<double>());
        FEM_LAUNCH_CHECK("k_bapply");
        double nv = 0.0;
        FEM_TRY(S.dot(N, pv, Dw.as<double>(), nv));
        nv = sqrt(nv);
        double lmax = 1.0;
        if (nv > 0) {
            k_div<<<grid(N, kT), kT, 0, S.st>>>(N, pv, nv, pv);
            std::vector<double> alpha, beta(1, 0.0);
            const int steps = std::max(2, o.eig_steps);
            for (int j = 0; j < steps; ++j) {
                k_spmv64<B><<<grid(n, kT), kT, 0, S.st>>>(n, A.ptr, A.col, A.val, pv, u.as<double>());
                FEM_LAUNCH_CHECK("k_spmv64");
                double a = 0.0;
                FEM_TRY(S.dot(N, pv, u.as<double>(), a));
                alpha.push_back(a);
                k_bapply<B><<<grid(n, kT), kT, 0, S.st>>>(n, dinv64.as<double>(), nullptr, u.as<double>(),
                                                          w.as<double>());
                const double bj = beta.back();
                k_lanczos_w<<<grid(N, kT), kT, 0, S.st>>>(N, w.as<double>(), a, pv, bj, pvp);
                k_bapply<B><<<grid(n, kT), kT, 0, S.st>>>(n, A.val, dpos.as<int32_t>(), w.as<double>(),
                                                          Dw.as<double>());
                FEM_LAUNCH_CHECK("k_bapply");
                double bn = 0.0;
                FEM_TRY(S.dot(N, w.as<double>(), Dw.as<double>(), bn));
                bn = sqrt(std::max(0.0, bn));
                if (!(bn > 1e-12 * fabs(a)) || j + 1 == steps) break;
                beta.push_back(bn);
                std::swap(pv, pvp);
                k_div<<<grid(N, kT), kT, 0, S.st>>>(N, w.as<double>(), bn, pv);
            }
            beta.resize(alpha.size());
            lmax = tridiag_lmax(alpha, beta);
        }
        L.lmax = lmax;
        L.omega = 4.0 / (3.0 * lmax);
        chebyshev_coefficients(lmax, o, std::max(1, std::max(o.pre_degree, o.post_degree)), L.c1, L.c2);
        H->setup_s[2] += since(te);
    }
    // ---- tentative prolongator ----
    const auto tt = Clock::now();
    std::vector<int32_t> aptr(na + 1, 0), mem;
    for (int64_t i = 0; i < n; ++i)
        if (L.agg[i] >= 0) ++aptr[L.agg[i] + 1];
    for (int64_t a = 0; a < na; ++a) aptr[a + 1] += aptr[a];
    mem.resize(aptr[na]);
    {
        std::vector<int32_t> cur(aptr.begin(), aptr.end() - 1);
        for (int64_t i = 0; i < n; ++i)
            if (L.agg[i] >= 0) mem[cur[L.agg[i]]++] = int32_t(i);
    }
    DBuf daptr, dmem, T;
    FEM_TRY(daptr.alloc(sizeof(int32_t) * (na + 1)));
    FEM_TRY(dmem.alloc(sizeof(int32_t) * std::max<size_t>(mem.size(), 1)));
    FEM_TRY(T.alloc(sizeof(double) * n * B * kModes));
    FEM_TRY(Bnext.alloc(sizeof(double) * na * kModes * kModes));
    FEM_TRY(S.up(daptr.as<int32_t>(), aptr));
    FEM_TRY(S.up(dmem.as<int32_t>(), mem));
    k_tentative<B><<<grid(na, 64), 64, 0, S.st>>>(na, daptr.as<int32_t>(), dmem.as<int32_t>(), Bnull_in,
                                                   T.as<double>(), Bnext.as<double>());
    FEM_LAUNCH_CHECK("k_tentative");
    FEM_TRY(S.sync());
    H->setup_s[1] += since(tt);
    // ---- smoothed prolongator ----
    const auto ts = Clock::now();
    Mat P;
    P.n = n;
    P.m = na;
    P.br = B;
    P.bc = kModes;
    {
        int maxL = 1;
        FEM_TRY(max_row_len(S, A, maxL));
        maxL = std::max(maxL, 1);
        const size_t smem = size_t(kWarps) * maxL * (sizeof(int32_t) + 1) + 16;
        FEM_REQUIRE(smem <= 200 * 1024, "AMG device setup: level %d has a row of %d blocks", l, maxL);
        DBuf cnt;
        FEM_TRY(cnt.alloc(sizeof(int32_t) * (n + 1)));
        FEM_TRY(P.ptr.alloc(sizeof(int32_t) * (n + 1)));
        FEM_CUDA(cudaFuncSetAttribute(k_prol_count, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
        k_prol_count<<<grid(n, kWarps), kT, smem, S.st>>>(n, A.ptr, A.col, agg.as<int32_t>(), iso.as<uint8_t>(),
                                                          o.smooth != 0, maxL, cnt.as<int32_t>());
        FEM_LAUNCH_CHECK("k_prol_count");
        FEM_TRY(S.scan(n, cnt.as<int32_t>(), P.ptr.as<int32_t>()));
        int32_t nnz = 0;
        FEM_TRY(S.read_int(P.P(), n, nnz));
        P.nnzb = nnz;
        FEM_TRY(P.col.alloc(sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
        FEM_TRY(P.val.alloc(sizeof(double) * std::max<int64_t>(nnz, 1) * B * kModes));
        int maxU = 1;
        FEM_TRY(max_row_len(S, View{n, na, B, kModes, nnz, P.P(), nullptr, nullptr}, maxU));
        maxU = std::max(maxU, 1);
        const size_t per = size_t(maxU) * B * kModes * sizeof(double) + size_t(maxL + maxU) * sizeof(int32_t) + maxL;
        const size_t per_al = (per + 15) & ~size_t(15);
        int warps = kWarps;
        while (warps > 1 && per_al * warps > 200 * 1024) warps >>= 1;
        FEM_REQUIRE(per_al * warps <= 220 * 1024, "AMG device setup: level %d needs %zu bytes per prolongator row", l,
                    per_al);
        FEM_CUDA(cudaFuncSetAttribute(k_prol_fill<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(per_al * warps)));
        k_prol_fill<B><<<grid(n, warps), 32 * warps, per_al * warps, S.st>>>(
            n, A.ptr, A.col, A.val, agg.as<int32_t>(), iso.as<uint8_t>(), o.smooth != 0, L.omega, dinv64.as<double>(),
            T.as<double>(), maxL, maxU, warps, P.P(), P.col.as<int32_t>(), P.val.as<double>());
        FEM_LAUNCH_CHECK("k_prol_fill");
        FEM_TRY(S.sync());
    }
    H->setup_s[3] += since(ts);
    // ---- Galerkin product ----
    const auto tg = Clock::now();
    Mat R, AP;
    FEM_TRY((transpose<B, kModes>(S, view_of(P), R)));
    FEM_TRY((spgemm<B, B, kModes>(S, A, view_of(P), AP)));
    FEM_TRY((spgemm<kModes, B, kModes>(S, view_of(R), view_of(AP), Anext)));
    k_unit_diag<kModes><<<grid(Anext.n, kT), kT, 0, S.st>>>(Anext.n, Anext.P(), Anext.C(), Anext.val.as<double>());
    FEM_LAUNCH_CHECK("k_unit_diag");
    FEM_TRY(S.sync());
    H->setup_s[4] += since(tg);
    // ---- hand over: FP32 copies for the cycle, FP64 copies for export ----
    FEM_TRY(to_devbsr(S, view_of(P), L.dP));
    FEM_TRY(to_devbsr(S, view_of(R), L.dR));
    FEM_CUDA(cudaMalloc(&L.d_iso, n));
    FEM_CUDA(cudaMemcpyAsync(L.d_iso, iso.p, n, cudaMemcpyDeviceToDevice, S.st));
    FEM_TRY(S.sync());
    L.gP = P.hand_over();
    L.gR = R.hand_over();
    L.g_dinv = static_cast<double*>(dinv64.release());
    return FEM_OK;
}

int build_device(fem_amg* H, const fem_bsr* A64, const double* xyz, const int32_t* hptr, const int32_t* hcol,
                 cudaStream_t st) {
    Setup S{H, st};
    FEM_TRY(S.status.alloc(sizeof(int)));
    const int64_t n0 = A64->n_brow;
    // level-0 near-null space: rigid-body modes about the centroid
    DBuf Bnull;
    FEM_TRY(Bnull.alloc(sizeof(double) * n0 * 3 * kModes));
    {
        double c[3];  // the host setup's chunked centroid
        for (int d = 0; d < 3; ++d) {
            FEM_TRY(S.dot(n0, xyz, nullptr, c[d], 3, d));
            c[d] /= double(n0);
        }
        k_rigid_modes<<<grid(n0, kT), kT, 0, st>>>(n0, xyz, c[0], c[1], c[2], Bnull.as<double>());
        FEM_LAUNCH_CHECK("k_rigid_modes");
    }
    View A{n0, n0, 3, 3, A64->nnzb, A64->indptr, A64->indices, static_cast<const double*>(A64->vals)};
    Mat Acur;  // owns the operator of levels >= 1
    for (int l = 0;; ++l) {
        const auto t0 = Clock::now();
        H->lv.emplace_back();
        Level& L = H->lv.back();
        L.b = A.br;
        L.n = A.n;
        DBuf Bnext;
        Mat Anext;
        bool last = false;
        if (A.br == 3)
            FEM_TRY(level_kernels<3>(S, H, l, A, Bnull.as<double>(), Bnext, Anext, l == 0 ? hptr : nullptr,
                                     l == 0 ? hcol : nullptr, last));
        else
            FEM_TRY(level_kernels<kModes>(S, H, l, A, Bnull.as<double>(), Bnext, Anext, nullptr, nullptr, last));
        if (l > 0) {
            FEM_TRY(to_devbsr(S, A, H->lv[l].dA));
            FEM_TRY(S.sync());
            H->lv[l].gA = Acur.hand_over();
        }
        H->lv[l].setup_s = since(t0);
        if (last) break;
        std::swap(Bnull.p, Bnext.p);
        Acur.n = Anext.n;
        Acur.m = Anext.m;
        Acur.br = Anext.br;
        Acur.bc = Anext.bc;
        Acur.nnzb = Anext.nnzb;
        std::swap(Acur.ptr.p, Anext.ptr.p);
        std::swap(Acur.col.p, Anext.col.p);
        std::swap(Acur.val.p, Anext.val.p);
        A = view_of(Acur);
    }
    // Dirichlet rows of level 0, the solver state of the cycle
    {
        Level& L0 = H->lv[0];
        std::vector<int32_t> rows;
        for (size_t i = 0; i < L0.iso.size(); ++i)
            if (L0.iso[i]) rows.push_back(int32_t(i));
        L0.n_iso = int64_t(rows.size());
        if (!rows.empty()) {
            FEM_CUDA(cudaMalloc(&L0.d_iso_rows, sizeof(int32_t) * rows.size()));
            FEM_TRY(S.up(L0.d_iso_rows, rows));
        }
        FEM_CUDA(cudaMalloc(&H->d_state, sizeof(pcgd::PcgState)));
        FEM_CUDA(cudaMemsetAsync(H->d_state, 0, sizeof(pcgd::PcgState), st));
    }
    FEM_TRY(S.sync());
    H->device_setup = true;
    H->uploaded = true;
    return FEM_OK;
}

}  // namespace
}  // namespace amg
}  // namespace fem

using namespace fem;
using namespace fem::amg;

extern "C" int fem_amg_setup_device(const fem_bsr* A64, const double* xyz, const int32_t* indptr_host,
                                    const int32_t* indices_host, const fem_amg_opts* opts, void* stream,
                                    fem_amg** out) {
    FEM_REQUIRE(out && A64 && xyz && opts, "NULL argument");
    *out = nullptr;
    FEM_REQUIRE(A64->dtype == FEM_F64 && A64->layout == FEM_LAYOUT_BSR && A64->indptr && A64->indices && A64->vals,
                "A64 must be an FP64 BSR matrix ([nnzb][3][3] blocks)");
    FEM_REQUIRE(A64->n_brow > 0 && A64->nnzb > 0 && A64->nnzb < (int64_t(1) << 31), "bad matrix size");
    FEM_REQUIRE(opts->theta >= 0 && opts->max_levels >= 1 && opts->max_coarse >= 1 && opts->eig_steps >= 1 &&
                    opts->pre_degree >= 1 && opts->post_degree >= 1 && opts->cheb_upper >= 1.0 &&
                    opts->cheb_ratio > 1.0,
                "bad fem_amg_opts");
    fem_amg* H = nullptr;
    int rc = FEM_OK;
    try {
        H = new fem_amg();
        H->opts = *opts;
        rc = build_device(H, A64, xyz, indptr_host, indices_host, as_stream(stream));
    } catch (const std::bad_alloc&) {
        set_error("AMG device setup: out of host memory");
        rc = FEM_ERR_WORKSPACE;
    } catch (...) {
        set_error("AMG device setup: unexpected exception");
        rc = FEM_ERR_INVALID;
    }
    if (rc != FEM_OK) {
        if (H) {
            release_device(H);
            delete H;
        }
        return rc;
    }
    *out = H;
    return FEM_OK;
}
