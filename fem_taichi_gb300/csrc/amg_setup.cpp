// Smoothed-aggregation AMG: host setup of the hierarchy (fem_amg_setup) and the host-only
// C entry points.  No reference counterpart: the reference factorises K with Pardiso
// (SOLVE_static.py:31-33); this builds the preconditioner that lets CG replace it on meshes
// where block-diagonal preconditioners stall.
//
// Per level (the method of Vanek, Mandel and Brezina, "Algebraic multigrid by smoothed
// aggregation for second and fourth order elliptic problems", Computing 56 (1996)):
//  1. strength on the block-scaled matrix: with D_i = L_i L_i^T (Cholesky of the diagonal
//     block), j is a strong neighbour of i when |L_i^-1 A_ij L_j^-T|_F^2 > theta^2 b (b = DOF
//     per node, |L_i^-1 A_ii L_i^-T|_F^2 = b), which does not depend on the units of the
//     DOF.  Rows without strong neighbours join no aggregate.  Among them, rows whose every
//     scaled coupling is below 1e-6 (the penalised nodes, whose 1e20 diagonal decouples
//     them) are Dirichlet rows: their prolongator rows are zero and the cycle holds
//     x_i = D_i^-1 b_i there.  (Coupling them to their neighbours, as a plain smoother or a
//     smoothed prolongator row would, puts values of size |A_ij x_j| / 1e20 into the
//     preconditioned vector; multiplied by the penalty again in the next product they cancel
//     catastrophically in FP32.)  Other unaggregated rows are smoothed like the rest and
//     keep their smoothed prolongator rows, so the cycle stays symmetric;
//  2. aggregation, in node order: (a) a free node whose strong neighbours are all free
//     starts an aggregate with them; (b) every node still free joins the step-(a) aggregate
//     of its most strongly coupled (scaled norm) aggregated neighbour; (c) what is left
//     forms aggregates with its free strong neighbours;
//  3. tentative prolongator: per aggregate a QR factorisation (two-pass modified
//     Gram-Schmidt, numerically dependent columns dropped) of the rows of the near-null
//     space, B_a = Q_a R_a; T holds Q_a and the next level's near-null space is R_a.  On
//     level 0 B holds the six rigid-body modes of the node coordinates;
//  4. P = (I - omega D^-1 A) T (zero on the Dirichlet rows),
//     omega = 4 / (3 lambda_max(D^-1 A)), lambda_max from a few Lanczos steps in the D inner
//     product;
//  5. A_c = R (A P) with R = P^T, two row-wise sparse products.  Every output row is
//     computed by one thread in a fixed order, so the hierarchy does not depend on the
//     thread count.
// The last level (at most max_coarse DOF) is inverted densely.
#include <math.h>
#include <omp.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <new>
#include <vector>

#include "amg.cuh"

namespace fem {
namespace amg {
namespace {

using Clock = std::chrono::steady_clock;
double since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

// Gauss-Jordan inverse with partial pivoting of a b x b row-major matrix (b <= 6).
bool invert_small(int b, const double* a, double* inv) {
    double m[kModes][2 * kModes];
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) {
            m[i][j] = a[i * b + j];
            m[i][b + j] = i == j ? 1.0 : 0.0;
        }
    for (int c = 0; c < b; ++c) {
        int p = c;
        for (int r = c + 1; r < b; ++r)
            if (fabs(m[r][c]) > fabs(m[p][c])) p = r;
        if (!(fabs(m[p][c]) > 0.0)) return false;
        if (p != c)
            for (int j = 0; j < 2 * b; ++j) std::swap(m[p][j], m[c][j]);
        const double s = 1.0 / m[c][c];
        for (int j = 0; j < 2 * b; ++j) m[c][j] *= s;
        for (int r = 0; r < b; ++r) {
            if (r == c) continue;
            const double f = m[r][c];
            if (f != 0.0)
                for (int j = 0; j < 2 * b; ++j) m[r][j] -= f * m[c][j];
        }
    }
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) inv[i * b + j] = m[i][b + j];
    return true;
}

double frob2(const double* a, int len) {
    double s = 0.0;
    for (int q = 0; q < len; ++q) s += a[q] * a[q];
    return s;
}

// position of the diagonal block of every row (-1 if absent); columns ascend within a row
std::vector<int64_t> diag_positions(const HostBsr& A) {
    std::vector<int64_t> pos(A.n, -1);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        const int32_t* b = A.col.data() + A.ptr[i];
        const int32_t* e = A.col.data() + A.ptr[i + 1];
        const int32_t* f = std::lower_bound(b, e, int32_t(i));
        if (f != e && *f == i) pos[i] = A.ptr[i] + (f - b);
    }
    return pos;
}

// Inverse diagonal blocks and their Frobenius norms; returns the number of rows whose
// diagonal block is missing or singular.
int64_t diag_inverse(const HostBsr& A, const std::vector<int64_t>& dpos, std::vector<double>& dinv,
                     std::vector<double>& dnorm) {
    const int b = A.br, bb = b * b;
    dinv.assign(size_t(A.n) * bb, 0.0);
    dnorm.assign(A.n, 0.0);
    int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t i = 0; i < A.n; ++i) {
        if (dpos[i] < 0) {
            ++bad;
            continue;
        }
        const double* a = A.val.data() + dpos[i] * bb;
        dnorm[i] = sqrt(frob2(a, bb));
        if (!invert_small(b, a, dinv.data() + i * bb)) ++bad;
    }
    return bad;
}

// y = A x (square, B x B blocks)
template <int B>
void spmv_t(const HostBsr& A, const double* __restrict__ x, double* __restrict__ y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        double acc[B] = {};
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1]; ++l) {
            const double* a = A.val.data() + l * B * B;
            const double* xc = x + int64_t(A.col[l]) * B;
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) acc[r] += a[r * B + c] * xc[c];
        }
        for (int r = 0; r < B; ++r) y[i * B + r] = acc[r];
    }
}

void spmv(const HostBsr& A, const double* x, double* y) {
    if (A.br == 3) spmv_t<3>(A, x, y);
    else spmv_t<kModes>(A, x, y);
}

// y = blockdiag(M) x, M [n][B][B]
template <int B>
void block_apply_t(int64_t n, const double* __restrict__ M, const double* __restrict__ x, double* __restrict__ y) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const double* m = M + i * B * B;
        for (int r = 0; r < B; ++r) {
            double s = 0.0;
            for (int c = 0; c < B; ++c) s += m[r * B + c] * x[i * B + c];
            y[i * B + r] = s;
        }
    }
}

void block_apply(int64_t n, int b, const double* M, const double* x, double* y) {
    if (b == 3) block_apply_t<3>(n, M, x, y);
    else block_apply_t<kModes>(n, M, x, y);
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
    // fixed-shape reduction: per-chunk partial sums added in chunk order
    const int64_t n = int64_t(a.size());
    const int64_t chunk = kSumChunk;
    const int64_t nc = (n + chunk - 1) / chunk;
    std::vector<double> part(std::max<int64_t>(nc, 1), 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nc; ++c) {
        double s = 0.0;
        const int64_t e = std::min(n, (c + 1) * chunk);
        for (int64_t i = c * chunk; i < e; ++i) s += a[i] * b[i];
        part[c] = s;
    }
    double s = 0.0;
    for (double v : part) s += v;
    return s;
}

// Largest eigenvalue of the symmetric tridiagonal matrix (alpha, beta[1..m-1]) by Sturm bisection.
double tridiag_max_eig(const std::vector<double>& alpha, const std::vector<double>& beta) {
    const int m = int(alpha.size());
    double lo = 1e300, hi = -1e300;
    for (int i = 0; i < m; ++i) {
        const double r = (i > 0 ? fabs(beta[i]) : 0.0) + (i + 1 < m ? fabs(beta[i + 1]) : 0.0);
        lo = std::min(lo, alpha[i] - r);
        hi = std::max(hi, alpha[i] + r);
    }
    auto below = [&](double x) {  // number of eigenvalues < x
        int cnt = 0;
        double q = alpha[0] - x;
        if (q < 0) ++cnt;
        for (int i = 1; i < m; ++i) {
            if (q == 0.0) q = 1e-300;
            q = alpha[i] - x - beta[i] * beta[i] / q;
            if (q < 0) ++cnt;
        }
        return cnt;
    };
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (below(mid) >= m)
            hi = mid;
        else
            lo = mid;
    }
    return hi;
}

// Lanczos estimate of lambda_max(D^-1 A) in the D inner product (D = diagonal blocks of A),
// from a fixed pseudo-random start vector.
double lanczos_lmax(const HostBsr& A, const std::vector<int64_t>& dpos, const std::vector<double>& dinv,
                    int steps) {
    const int b = A.br, bb = b * b;
    const int64_t N = A.n * b;
    std::vector<double> D(size_t(A.n) * bb, 0.0);
    for (int64_t i = 0; i < A.n; ++i)
        if (dpos[i] >= 0) std::copy_n(A.val.data() + dpos[i] * bb, bb, D.data() + i * bb);
    std::vector<double> v(N), vp(N, 0.0), u(N), w(N), Dw(N);
    for (int64_t i = 0; i < N; ++i) {  // splitmix64 -> [-1, 1)
        uint64_t z = uint64_t(i) + 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        v[i] = double(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
    block_apply(A.n, b, D.data(), v.data(), Dw.data());
    double nv = sqrt(dot(v, Dw));
    if (!(nv > 0)) return 1.0;
    for (auto& x : v) x /= nv;
    std::vector<double> alpha, beta(1, 0.0);
    for (int j = 0; j < steps; ++j) {
        spmv(A, v.data(), u.data());
        const double a = dot(v, u);
        alpha.push_back(a);
        block_apply(A.n, b, dinv.data(), u.data(), w.data());
        const double bj = beta.back();
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) w[i] -= a * v[i] + bj * vp[i];
        block_apply(A.n, b, D.data(), w.data(), Dw.data());
        const double bn = sqrt(std::max(0.0, dot(w, Dw)));
        if (!(bn > 1e-12 * fabs(a)) || j + 1 == steps) break;
        beta.push_back(bn);
        vp.swap(v);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) v[i] = w[i] / bn;
    }
    beta.resize(alpha.size());
    return tridiag_max_eig(alpha, beta);
}

// Inverse Cholesky factors L_i^-1 (lower triangular) of the diagonal blocks, [n][b][b];
// a block that is not numerically SPD gets the diagonal scaling 1 / sqrt|d_pp| instead.
std::vector<double> inv_cholesky(const HostBsr& A, const std::vector<int64_t>& dpos) {
    const int b = A.br, bb = b * b;
    std::vector<double> G(size_t(A.n) * bb, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        double* g = G.data() + i * bb;
        if (dpos[i] < 0) {
            for (int p = 0; p < b; ++p) g[p * b + p] = 1.0;
            continue;
        }
        const double* a = A.val.data() + dpos[i] * bb;
        double Lm[kModes][kModes] = {};
        bool ok = true;
        for (int c = 0; c < b && ok; ++c) {
            double d = a[c * b + c];
            for (int k = 0; k < c; ++k) d -= Lm[c][k] * Lm[c][k];
            if (!(d > 0.0)) {
                ok = false;
                break;
            }
            Lm[c][c] = sqrt(d);
            for (int r = c + 1; r < b; ++r) {
                double v = a[r * b + c];
                for (int k = 0; k < c; ++k) v -= Lm[r][k] * Lm[c][k];
                Lm[r][c] = v / Lm[c][c];
            }
        }
        if (!ok) {
            for (int p = 0; p < b; ++p) {
                const double d = fabs(a[p * b + p]);
                g[p * b + p] = d > 0.0 ? 1.0 / sqrt(d) : 1.0;
            }
            continue;
        }
        for (int c = 0; c < b; ++c) {  // forward substitution on the unit vectors
            for (int r = 0; r < b; ++r) {
                double v = r == c ? 1.0 : 0.0;
                for (int k = 0; k < r; ++k) v -= Lm[r][k] * g[k * b + c];
                g[r * b + c] = v / Lm[r][r];
            }
        }
    }
    return G;
}

// Strong-connection flag per block (diagonal blocks are not strong), the scaled coupling
// sv[l] = |L_i^-1 A_ij L_j^-T|_F^2 of every block, and per row the largest sv / b over its
// off-diagonal blocks.
std::vector<uint8_t> strength(const HostBsr& A, const std::vector<double>& G, double theta,
                              std::vector<double>& sv, std::vector<double>& maxc) {
    const int b = A.br, bb = b * b;
    std::vector<uint8_t> s(A.nnzb(), 0);
    sv.assign(A.nnzb(), 0.0);
    maxc.assign(A.n, 0.0);
    const double t2 = theta * theta * b;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        const double* gi = G.data() + i * bb;
        double mx = 0.0;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1]; ++l) {
            const int64_t j = A.col[l];
            if (j == i) continue;
            const double* a = A.val.data() + l * bb;
            const double* gj = G.data() + j * bb;
            double t[kModes * kModes];  // L_i^-1 A_ij
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c) {
                    double v = 0.0;
                    for (int k = 0; k <= r; ++k) v += gi[r * b + k] * a[k * b + c];
                    t[r * b + c] = v;
                }
            double f = 0.0;  // |(L_i^-1 A_ij) L_j^-T|_F^2
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c) {
                    double v = 0.0;
                    for (int k = 0; k <= c; ++k) v += t[r * b + k] * gj[c * b + k];
                    f += v * v;
                }
            s[l] = f > t2 ? 1 : 0;
            sv[l] = f;
            mx = std::max(mx, f / b);
        }
        maxc[i] = mx;
    }
    return s;
}

// Unaggregated rows whose scaled couplings are all below 1e-6 (squared: kDecoupled2 = 1e-12)
// are Dirichlet rows.

int64_t aggregate(const HostBsr& A, const std::vector<uint8_t>& strong, const std::vector<double>& sv,
                  std::vector<int32_t>& agg) {
    const int64_t n = A.n;
    constexpr int32_t kFree = -1, kAlone = -2;
    agg.assign(n, kFree);
    for (int64_t i = 0; i < n; ++i) {
        bool any = false;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1] && !any; ++l) any = strong[l] != 0;
        if (!any) agg[i] = kAlone;
    }
    int32_t na = 0;
    for (int64_t i = 0; i < n; ++i) {  // (a) free node with all strong neighbours free
        if (agg[i] != kFree) continue;
        bool ok = true;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1] && ok; ++l)
            if (strong[l] && agg[A.col[l]] != kFree) ok = false;
        if (!ok) continue;
        agg[i] = na;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1]; ++l)
            if (strong[l]) agg[A.col[l]] = na;
        ++na;
    }
    const std::vector<int32_t> first = agg;
    for (int64_t i = 0; i < n; ++i) {  // (b) join the strongest aggregated neighbour
        if (agg[i] != kFree) continue;
        int32_t best = -1;
        double bs = -1.0;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1]; ++l) {
            if (!strong[l] || first[A.col[l]] < 0) continue;
            const double s = sv[l];
            if (s > bs) {
                bs = s;
                best = first[A.col[l]];
            }
        }
        if (best >= 0) agg[i] = best;
    }
    for (int64_t i = 0; i < n; ++i) {  // (c) the rest with their free strong neighbours
        if (agg[i] != kFree) continue;
        agg[i] = na;
        for (int64_t l = A.ptr[i]; l < A.ptr[i + 1]; ++l)
            if (strong[l] && agg[A.col[l]] == kFree) agg[A.col[l]] = na;
        ++na;
    }
    for (auto& a : agg)
        if (a == kAlone) a = -1;
    return na;
}

// T (n x na, b x k blocks, one per aggregated node) and the coarse near-null space Bc [na][k][k].
void tentative(int64_t n, int b, const std::vector<int32_t>& agg, int64_t na, const std::vector<double>& B,
               HostBsr& T, std::vector<double>& Bc) {
    const int k = kModes;
    std::vector<int64_t> aptr(na + 1, 0);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) ++aptr[agg[i] + 1];
    for (int64_t a = 0; a < na; ++a) aptr[a + 1] += aptr[a];
    std::vector<int64_t> mem(aptr[na]), cur(aptr.begin(), aptr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
        if (agg[i] >= 0) mem[cur[agg[i]]++] = i;
    T = HostBsr{};
    T.n = n;
    T.m = na;
    T.br = b;
    T.bc = k;
    T.ptr.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) T.ptr[i + 1] = T.ptr[i] + (agg[i] >= 0 ? 1 : 0);
    T.col.assign(T.ptr[n], 0);
    T.val.assign(size_t(T.ptr[n]) * b * k, 0.0);
    Bc.assign(size_t(na) * k * k, 0.0);
#pragma omp parallel
    {
        std::vector<double> Q;
#pragma omp for schedule(dynamic, 256)
        for (int64_t a = 0; a < na; ++a) {
            const int64_t s0 = aptr[a], cnt = aptr[a + 1] - s0;
            const int64_t rows = cnt * b;
            Q.assign(size_t(rows) * k, 0.0);
            for (int64_t s = 0; s < cnt; ++s)
                for (int c = 0; c < b; ++c)
                    for (int m = 0; m < k; ++m) Q[(s * b + c) * k + m] = B[(mem[s0 + s] * b + c) * k + m];
            double Rr[kModes][kModes] = {};
            for (int c = 0; c < k; ++c) {
                double n0 = 0.0;
                for (int64_t r = 0; r < rows; ++r) n0 += Q[r * k + c] * Q[r * k + c];
                n0 = sqrt(n0);
                for (int pass = 0; pass < 2; ++pass)
                    for (int c2 = 0; c2 < c; ++c2) {
                        double d = 0.0;
                        for (int64_t r = 0; r < rows; ++r) d += Q[r * k + c2] * Q[r * k + c];
                        for (int64_t r = 0; r < rows; ++r) Q[r * k + c] -= d * Q[r * k + c2];
                        Rr[c2][c] += d;
                    }
                double nr = 0.0;
                for (int64_t r = 0; r < rows; ++r) nr += Q[r * k + c] * Q[r * k + c];
                nr = sqrt(nr);
                if (nr > 1e-10 * n0 && nr > 0.0) {
                    for (int64_t r = 0; r < rows; ++r) Q[r * k + c] /= nr;
                    Rr[c][c] = nr;
                } else {
                    for (int64_t r = 0; r < rows; ++r) Q[r * k + c] = 0.0;
                    Rr[c][c] = 0.0;
                }
            }
            for (int64_t s = 0; s < cnt; ++s) {
                const int64_t i = mem[s0 + s];
                T.col[T.ptr[i]] = int32_t(a);
                for (int c = 0; c < b; ++c)
                    for (int m = 0; m < k; ++m) T.val[(T.ptr[i] * b + c) * k + m] = Q[(s * b + c) * k + m];
            }
            for (int c = 0; c < k; ++c)
                for (int m = 0; m < k; ++m) Bc[(a * k + c) * k + m] = Rr[c][m];
        }
    }
}

// z (BI x BJ) += x (BI x BK) y (BK x BJ); block shapes fixed at compile time.  Every term is
// one correctly rounded fused multiply-add, as in the device setup's products.
template <int BI, int BK, int BJ>
inline void block_fma(const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ z) {
    for (int r = 0; r < BI; ++r)
        for (int q = 0; q < BK; ++q) {
            const double xv = x[r * BK + q];
            for (int c = 0; c < BJ; ++c) z[r * BJ + c] = std::fma(xv, y[q * BJ + c], z[r * BJ + c]);
        }
}

// Z = X Y, row by row (Gustavson); columns ascending in every output row.
template <int BI, int BK, int BJ>
HostBsr spgemm_t(const HostBsr& X, const HostBsr& Y) {
    HostBsr Z;
    Z.n = X.n;
    Z.m = Y.m;
    Z.br = BI;
    Z.bc = BJ;
    Z.ptr.assign(Z.n + 1, 0);
#pragma omp parallel
    {
        std::vector<int64_t> mark(Y.m, -1);
#pragma omp for schedule(dynamic, 512)
        for (int64_t i = 0; i < X.n; ++i) {
            int64_t cnt = 0;
            for (int64_t l = X.ptr[i]; l < X.ptr[i + 1]; ++l) {
                const int64_t kk = X.col[l];
                for (int64_t t = Y.ptr[kk]; t < Y.ptr[kk + 1]; ++t)
                    if (mark[Y.col[t]] != i) {
                        mark[Y.col[t]] = i;
                        ++cnt;
                    }
            }
            Z.ptr[i + 1] = cnt;
        }
    }
    for (int64_t i = 0; i < Z.n; ++i) Z.ptr[i + 1] += Z.ptr[i];
    Z.col.assign(Z.ptr[Z.n], 0);
    Z.val.assign(size_t(Z.ptr[Z.n]) * BI * BJ, 0.0);
#pragma omp parallel
    {
        std::vector<int32_t> pos(Y.m, -1);
        std::vector<int32_t> list;
#pragma omp for schedule(dynamic, 512)
        for (int64_t i = 0; i < X.n; ++i) {
            list.clear();
            for (int64_t l = X.ptr[i]; l < X.ptr[i + 1]; ++l) {
                const int64_t kk = X.col[l];
                for (int64_t t = Y.ptr[kk]; t < Y.ptr[kk + 1]; ++t)
                    if (pos[Y.col[t]] < 0) {
                        pos[Y.col[t]] = 0;
                        list.push_back(Y.col[t]);
                    }
            }
            std::sort(list.begin(), list.end());
            const int64_t base = Z.ptr[i];
            for (size_t q = 0; q < list.size(); ++q) {
                pos[list[q]] = int32_t(q);
                Z.col[base + q] = list[q];
            }
            double* zr = Z.val.data() + base * BI * BJ;
            for (int64_t l = X.ptr[i]; l < X.ptr[i + 1]; ++l) {
                const int64_t kk = X.col[l];
                const double* xb = X.val.data() + l * BI * BK;
                for (int64_t t = Y.ptr[kk]; t < Y.ptr[kk + 1]; ++t)
                    block_fma<BI, BK, BJ>(xb, Y.val.data() + t * BK * BJ, zr + int64_t(pos[Y.col[t]]) * BI * BJ);
            }
            for (int32_t c : list) pos[c] = -1;
        }
    }
    return Z;
}

HostBsr spgemm(const HostBsr& X, const HostBsr& Y) {
    if (X.br == 3 && X.bc == 3 && Y.bc == kModes) return spgemm_t<3, 3, kModes>(X, Y);
    if (X.br == kModes && X.bc == 3 && Y.bc == kModes) return spgemm_t<kModes, 3, kModes>(X, Y);
    return spgemm_t<kModes, kModes, kModes>(X, Y);  // the only other shape the setup forms
}

// R = P^T.  Rows are cut into one chunk per thread; each thread counts its chunk's columns,
// the (column, chunk) prefix sums give every entry its place, and the threads scatter their
// chunks, so each column of P lists its rows in ascending order whatever the thread count.
HostBsr transpose(const HostBsr& P) {
    HostBsr R;
    R.n = P.m;
    R.m = P.n;
    R.br = P.bc;
    R.bc = P.br;
    const int br = P.br, bc = P.bc;
    const int nt = std::max(1, omp_get_max_threads());
    std::vector<int64_t> cut(nt + 1, 0);
    for (int t = 0; t <= nt; ++t) cut[t] = P.n * t / nt;
    std::vector<int64_t> cnt(size_t(nt) * (R.n + 1), 0);  // [chunk][column]
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        int64_t* c = cnt.data() + size_t(t) * (R.n + 1);
        for (int64_t l = P.ptr[cut[t]]; l < P.ptr[cut[t + 1]]; ++l) ++c[P.col[l]];
    }
    R.ptr.assign(R.n + 1, 0);
    std::vector<int64_t> start(size_t(nt) * (R.n + 1), 0);
    int64_t acc = 0;
    for (int64_t j = 0; j < R.n; ++j) {
        R.ptr[j] = acc;
        for (int t = 0; t < nt; ++t) {
            start[size_t(t) * (R.n + 1) + j] = acc;
            acc += cnt[size_t(t) * (R.n + 1) + j];
        }
    }
    R.ptr[R.n] = acc;
    R.col.assign(P.nnzb(), 0);
    R.val.assign(P.val.size(), 0.0);
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
        int64_t* cur = start.data() + size_t(t) * (R.n + 1);
        for (int64_t i = cut[t]; i < cut[t + 1]; ++i)
            for (int64_t l = P.ptr[i]; l < P.ptr[i + 1]; ++l) {
                const int64_t q = cur[P.col[l]]++;
                R.col[q] = int32_t(i);
                const double* s = P.val.data() + l * br * bc;
                double* d = R.val.data() + q * br * bc;
                for (int r = 0; r < br; ++r)
                    for (int c = 0; c < bc; ++c) d[c * br + r] = s[r * bc + c];
            }
    }
    return R;
}

// P = T - omega D^-1 (A T) (smooth), else P = T; rows of Dirichlet nodes stay empty.
// Row i of A T contains the aggregate of node i itself (A has every diagonal block), so T_i
// is always added.
HostBsr drop_rows(const HostBsr& X, const std::vector<uint8_t>& drop) {
    HostBsr Y;
    Y.n = X.n;
    Y.m = X.m;
    Y.br = X.br;
    Y.bc = X.bc;
    const int64_t bs = int64_t(X.br) * X.bc;
    Y.ptr.assign(X.n + 1, 0);
    for (int64_t i = 0; i < X.n; ++i) Y.ptr[i + 1] = Y.ptr[i] + (drop[i] ? 0 : X.ptr[i + 1] - X.ptr[i]);
    Y.col.resize(Y.ptr[X.n]);
    Y.val.resize(size_t(Y.ptr[X.n]) * bs);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < X.n; ++i) {
        if (Y.ptr[i + 1] == Y.ptr[i]) continue;
        std::copy(X.col.begin() + X.ptr[i], X.col.begin() + X.ptr[i + 1], Y.col.begin() + Y.ptr[i]);
        std::copy(X.val.begin() + X.ptr[i] * bs, X.val.begin() + X.ptr[i + 1] * bs, Y.val.begin() + Y.ptr[i] * bs);
    }
    return Y;
}

HostBsr smooth_prolongator(const HostBsr& A, const std::vector<double>& dinv, const HostBsr& T, double omega,
                           bool smooth, const std::vector<uint8_t>& dirichlet) {
    if (!smooth) return T;
    HostBsr AT = spgemm(A, T);
    const int b = A.br, k = T.bc, bb = b * b, bk = b * k;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        const double* di = dinv.data() + i * bb;
        const int32_t tc = T.ptr[i + 1] > T.ptr[i] ? T.col[T.ptr[i]] : -1;
        for (int64_t l = AT.ptr[i]; l < AT.ptr[i + 1]; ++l) {
            double* blk = AT.val.data() + l * bk;
            double tmp[kModes * kModes];
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < k; ++c) {
                    double s = 0.0;
                    for (int q = 0; q < b; ++q) s += di[r * b + q] * blk[q * k + c];
                    tmp[r * k + c] = -omega * s;
                }
            if (AT.col[l] == tc) {
                const double* t = T.val.data() + T.ptr[i] * bk;
                for (int q = 0; q < bk; ++q) tmp[q] += t[q];
            }
            std::copy_n(tmp, bk, blk);
        }
    }
    return drop_rows(AT, dirichlet);
}

// Chebyshev coefficients of the smoother on [upper / ratio, upper] for `degree` steps:
// step 0: d = (1/theta) D^-1 r;  step k: d = c1 d + c2 D^-1 r.
void chebyshev(double lmax, const fem_amg_opts& o, int degree, std::vector<float>& c1, std::vector<float>& c2) {
    const double up = o.cheb_upper * lmax, lo = up / o.cheb_ratio;
    const double theta = 0.5 * (up + lo), delta = 0.5 * (up - lo), sigma = theta / delta;
    c1.assign(degree, 0.f);
    c2.assign(degree, 0.f);
    c2[0] = float(1.0 / theta);
    double rho = 1.0 / sigma;
    for (int k = 1; k < degree; ++k) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        c1[k] = float(rn * rho);
        c2[k] = float(2.0 * rn / delta);
        rho = rn;
    }
}

bool dense_inverse(int64_t m, std::vector<double>& a, std::vector<double>& inv) {
    inv.assign(size_t(m) * m, 0.0);
    for (int64_t i = 0; i < m; ++i) inv[i * m + i] = 1.0;
    for (int64_t c = 0; c < m; ++c) {
        int64_t p = c;
        for (int64_t r = c + 1; r < m; ++r)
            if (fabs(a[r * m + c]) > fabs(a[p * m + c])) p = r;
        if (!(fabs(a[p * m + c]) > 0.0)) return false;
        if (p != c)
            for (int64_t j = 0; j < m; ++j) {
                std::swap(a[p * m + j], a[c * m + j]);
                std::swap(inv[p * m + j], inv[c * m + j]);
            }
        const double s = 1.0 / a[c * m + c];
        for (int64_t j = 0; j < m; ++j) {
            a[c * m + j] *= s;
            inv[c * m + j] *= s;
        }
#pragma omp parallel for schedule(static)
        for (int64_t r = 0; r < m; ++r) {
            if (r == c) continue;
            const double f = a[r * m + c];
            if (f == 0.0) continue;
            for (int64_t j = 0; j < m; ++j) {
                a[r * m + j] -= f * a[c * m + j];
                inv[r * m + j] -= f * inv[c * m + j];
            }
        }
    }
    return true;
}

int build(fem_amg* H, HostBsr&& A0, const double* xyz) {
    const fem_amg_opts& o = H->opts;
    HostBsr A = std::move(A0);
    std::vector<double> B;  // near-null space [n][b][k]
    {
        const int64_t n = A.n;
        double c[3] = {0, 0, 0};
        for (int d = 0; d < 3; ++d) {  // chunked like dot()
            for (int64_t c0 = 0; c0 < n; c0 += kSumChunk) {
                double s = 0.0;
                for (int64_t i = c0; i < std::min(n, c0 + kSumChunk); ++i) s += xyz[3 * i + d];
                c[d] += s;
            }
            c[d] /= double(n);
        }
        B.assign(size_t(n) * 3 * kModes, 0.0);
        for (int64_t i = 0; i < n; ++i) {
            const double x = xyz[3 * i] - c[0], y = xyz[3 * i + 1] - c[1], z = xyz[3 * i + 2] - c[2];
            double* b = B.data() + i * 3 * kModes;
            b[0 * kModes + 0] = 1.0;
            b[1 * kModes + 1] = 1.0;
            b[2 * kModes + 2] = 1.0;
            // rotations e_d x (x, y, z)
            b[1 * kModes + 3] = -z;
            b[2 * kModes + 3] = y;
            b[0 * kModes + 4] = z;
            b[2 * kModes + 4] = -x;
            b[0 * kModes + 5] = -y;
            b[1 * kModes + 5] = x;
        }
    }
    for (int l = 0;; ++l) {
        const auto t0 = Clock::now();
        H->lv.emplace_back();
        Level& L = H->lv.back();
        L.b = A.br;
        L.n = A.n;
        const std::vector<int64_t> dpos = diag_positions(A);
        std::vector<double> dnorm;
        if (const int64_t bad = diag_inverse(A, dpos, L.dinv, dnorm)) {
            set_error("AMG level %d: %lld missing or singular diagonal blocks", l, (long long)bad);
            return FEM_ERR_NOT_SPD;
        }
        const int64_t m = A.n * A.br;
        const bool last_by_size = m <= o.max_coarse || l + 1 >= o.max_levels;
        int64_t na = 0;
        if (!last_by_size) {
            auto ta = Clock::now();
            std::vector<double> sv, maxc;
            const std::vector<uint8_t> strong = strength(A, inv_cholesky(A, dpos), o.theta, sv, maxc);
            na = aggregate(A, strong, sv, L.agg);
            L.iso.resize(L.agg.size());
            for (size_t i = 0; i < L.agg.size(); ++i) L.iso[i] = (L.agg[i] < 0 && maxc[i] < kDecoupled2) ? 1 : 0;
            H->setup_s[0] += since(ta);
        }
        if (last_by_size || na == 0 || na * kModes >= m) {
            // dense coarsest level
            if (m > kMaxDense) {
                set_error("AMG: level %d has %lld DOF and cannot be coarsened further (raise max_levels?)", l,
                          (long long)m);
                return FEM_ERR_INVALID;
            }
            auto tc = Clock::now();
            L.agg.clear();
            L.iso.clear();
            std::vector<double> dense(size_t(m) * m, 0.0);
            const int b = A.br;
            for (int64_t i = 0; i < A.n; ++i)
                for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
                    for (int r = 0; r < b; ++r)
                        for (int c = 0; c < b; ++c)
                            dense[(i * b + r) * m + int64_t(A.col[q]) * b + c] = A.val[(q * b + r) * b + c];
            H->coarse_m = m;
            if (!dense_inverse(m, dense, H->coarse_inv)) {
                set_error("AMG: the coarsest operator (%lld DOF) is singular", (long long)m);
                return FEM_ERR_NOT_SPD;
            }
            if (l > 0) L.A = std::move(A);
            H->setup_s[5] += since(tc);
            L.setup_s = since(t0);
            return FEM_OK;
        }
        auto te = Clock::now();
        L.lmax = lanczos_lmax(A, dpos, L.dinv, std::max(2, o.eig_steps));
        L.omega = 4.0 / (3.0 * L.lmax);
        chebyshev(L.lmax, o, std::max(1, std::max(o.pre_degree, o.post_degree)), L.c1, L.c2);
        H->setup_s[2] += since(te);
        auto tt = Clock::now();
        HostBsr T;
        std::vector<double> Bc;
        tentative(A.n, A.br, L.agg, na, B, T, Bc);
        H->setup_s[1] += since(tt);
        auto ts = Clock::now();
        L.P = smooth_prolongator(A, L.dinv, T, L.omega, o.smooth != 0, L.iso);
        H->setup_s[3] += since(ts);
        auto tg = Clock::now();
        L.R = transpose(L.P);
        HostBsr Ac;
        {
            HostBsr AP = spgemm(A, L.P);
            Ac = spgemm(L.R, AP);
        }
        // coarse DOF whose prolongator column is zero (dropped dependent modes) have an
        // exactly zero row and column: give them a unit diagonal
        {
            const std::vector<int64_t> cd = diag_positions(Ac);
            const int bc = Ac.br;
            for (int64_t a = 0; a < Ac.n; ++a) {
                if (cd[a] < 0) continue;
                double* blk = Ac.val.data() + cd[a] * bc * bc;
                for (int d = 0; d < bc; ++d)
                    if (blk[d * bc + d] == 0.0) blk[d * bc + d] = 1.0;
            }
        }
        H->setup_s[4] += since(tg);
        if (l > 0) L.A = std::move(A);
        A = std::move(Ac);
        B = std::move(Bc);
        L.setup_s = since(t0);
    }
}

}  // namespace

double tridiag_lmax(const std::vector<double>& alpha, const std::vector<double>& beta) {
    return tridiag_max_eig(alpha, beta);
}
void chebyshev_coefficients(double lmax, const fem_amg_opts& o, int degree, std::vector<float>& c1,
                            std::vector<float>& c2) {
    chebyshev(lmax, o, degree, c1, c2);
}
bool dense_inverse_host(int64_t m, std::vector<double>& a, std::vector<double>& inv) {
    return dense_inverse(m, a, inv);
}

}  // namespace amg
}  // namespace fem

using namespace fem;
using namespace fem::amg;

extern "C" void fem_amg_default_opts(fem_amg_opts* o) {
    if (!o) return;
    o->theta = 0.08;
    o->max_levels = 10;
    o->max_coarse = 512;
    o->smooth = 1;
    o->eig_steps = 12;
    o->pre_degree = 2;
    o->post_degree = 2;
    o->cheb_upper = 1.1;
    o->cheb_ratio = 30.0;
}

extern "C" int fem_amg_setup(int64_t n_brow, const int32_t* indptr, const int32_t* indices, const double* vals,
                             const double* xyz, const fem_amg_opts* opts, fem_amg** out) {
    FEM_REQUIRE(out && indptr && indices && vals && xyz && opts, "NULL argument");
    *out = nullptr;
    FEM_REQUIRE(n_brow > 0 && indptr[0] == 0, "bad matrix size / row pointers");
    FEM_REQUIRE(opts->theta >= 0 && opts->max_levels >= 1 && opts->max_coarse >= 1 && opts->eig_steps >= 1 &&
                    opts->pre_degree >= 1 && opts->post_degree >= 1 && opts->cheb_upper >= 1.0 &&
                    opts->cheb_ratio > 1.0,
                "bad fem_amg_opts");
    for (int64_t i = 0; i < n_brow; ++i)
        FEM_REQUIRE(indptr[i + 1] >= indptr[i], "row pointers must not decrease (row %lld)", (long long)i);
    const int64_t nnzb = indptr[n_brow];
    int64_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (int64_t i = 0; i < n_brow; ++i)
        for (int64_t l = indptr[i]; l < indptr[i + 1]; ++l)
            if (indices[l] < 0 || indices[l] >= n_brow || (l > indptr[i] && indices[l] <= indices[l - 1])) ++bad;
    FEM_REQUIRE(bad == 0, "column indices must lie in [0, n) and ascend within each row");
    fem_amg* H = nullptr;
    try {
        H = new fem_amg();
        H->opts = *opts;
        HostBsr A;
        A.n = A.m = n_brow;
        A.br = A.bc = 3;
        A.ptr.assign(indptr, indptr + n_brow + 1);
        A.col.assign(indices, indices + nnzb);
        A.val.assign(vals, vals + 9 * nnzb);
        const int rc = build(H, std::move(A), xyz);
        if (rc) {
            delete H;
            return rc;
        }
    } catch (const std::bad_alloc&) {
        delete H;
        set_error("AMG setup: out of host memory");
        return FEM_ERR_WORKSPACE;
    } catch (...) {
        delete H;
        set_error("AMG setup: unexpected exception");
        return FEM_ERR_INVALID;
    }
    *out = H;
    return FEM_OK;
}

extern "C" int fem_amg_num_levels(const fem_amg* h) { return h ? int(h->lv.size()) : 0; }

extern "C" int fem_amg_set_smoother(fem_amg* h, int level, double upper, double ratio) {
    FEM_REQUIRE(h, "NULL argument");
    FEM_REQUIRE(level >= 0 && level + 1 < int(h->lv.size()), "level out of range (the last level is solved densely)");
    FEM_REQUIRE(upper >= 1.0 && upper <= 4.0 && ratio > 1.0 && ratio <= 1e4,
                "smoother interval: need 1 <= upper <= 4 and 1 < ratio <= 1e4");
    Level& L = h->lv[level];
    fem_amg_opts o = h->opts;
    o.cheb_upper = upper;
    o.cheb_ratio = ratio;
    chebyshev(L.lmax, o, std::max(1, std::max(o.pre_degree, o.post_degree)), L.c1, L.c2);
    return FEM_OK;
}

extern "C" int fem_amg_setup_phases(const fem_amg* h, double* seconds6) {
    FEM_REQUIRE(h && seconds6, "NULL argument");
    for (int i = 0; i < 6; ++i) seconds6[i] = h->setup_s[i];
    return FEM_OK;
}

extern "C" int fem_amg_get_level(const fem_amg* h, int level, fem_amg_level_info* info) {
    FEM_REQUIRE(h && info, "NULL argument");
    FEM_REQUIRE(level >= 0 && level < int(h->lv.size()), "level out of range");
    const Level& L = h->lv[level];
    info->n = L.n;
    info->b = L.b;
    info->nnzb_A = h->device_setup ? L.gA.nnzb : L.A.nnzb();
    info->nnzb_P = h->device_setup ? L.gP.nnzb : L.P.nnzb();
    info->lmax = L.lmax;
    info->omega = L.omega;
    info->setup_s = L.setup_s;
    return FEM_OK;
}

extern "C" int fem_amg_export(const fem_amg* h, int level, int what, int64_t* dims, int64_t* indptr,
                              int32_t* indices, double* vals) {
    FEM_REQUIRE(h && dims, "NULL argument");
    FEM_REQUIRE(level >= 0 && level < int(h->lv.size()), "level out of range");
    const Level& L = h->lv[level];
    if (h->device_setup && (what <= 3)) {  // FP64 copies on the device
        if (what == 3) {
            dims[0] = L.n;
            dims[1] = L.g_dinv ? L.n * L.b * L.b : 0;
            dims[2] = dims[3] = L.b;
            if (vals && L.g_dinv)
                FEM_CUDA(cudaMemcpy(vals, L.g_dinv, sizeof(double) * dims[1], cudaMemcpyDeviceToHost));
            return FEM_OK;
        }
        FEM_REQUIRE(what >= 0, "what must be 0..6");
        const Dev64& D = what == 0 ? L.gA : what == 1 ? L.gP : L.gR;
        dims[0] = D.n;
        dims[1] = D.nnzb;
        dims[2] = D.br;
        dims[3] = D.bc;
        if (D.ptr) {
            if (indptr) {
                std::vector<int32_t> p(D.n + 1);
                FEM_CUDA(cudaMemcpy(p.data(), D.ptr, sizeof(int32_t) * (D.n + 1), cudaMemcpyDeviceToHost));
                std::copy(p.begin(), p.end(), indptr);
            }
            if (indices) FEM_CUDA(cudaMemcpy(indices, D.col, sizeof(int32_t) * D.nnzb, cudaMemcpyDeviceToHost));
            if (vals)
                FEM_CUDA(cudaMemcpy(vals, D.val, sizeof(double) * D.nnzb * D.br * D.bc, cudaMemcpyDeviceToHost));
        }
        return FEM_OK;
    }
    const HostBsr* M = nullptr;
    switch (what) {
        case 0: M = &L.A; break;
        case 1: M = &L.P; break;
        case 2: M = &L.R; break;
        case 3:
            dims[0] = L.n;
            dims[1] = int64_t(L.dinv.size());
            dims[2] = dims[3] = L.b;
            if (vals) std::copy(L.dinv.begin(), L.dinv.end(), vals);
            return FEM_OK;
        case 4:
            dims[0] = L.n;
            dims[1] = int64_t(L.agg.size());
            dims[2] = dims[3] = 1;
            if (indices) std::copy(L.agg.begin(), L.agg.end(), indices);
            return FEM_OK;
        case 6:
            dims[0] = L.n;
            dims[1] = int64_t(L.iso.size());
            dims[2] = dims[3] = 1;
            if (indices)
                for (size_t i = 0; i < L.iso.size(); ++i) indices[i] = L.iso[i];
            return FEM_OK;
        case 5:
            FEM_REQUIRE(level + 1 == int(h->lv.size()), "the dense inverse belongs to the last level");
            dims[0] = h->coarse_m;
            dims[1] = h->coarse_m * h->coarse_m;
            dims[2] = dims[3] = 1;
            if (vals) std::copy(h->coarse_inv.begin(), h->coarse_inv.end(), vals);
            return FEM_OK;
        default: FEM_REQUIRE(false, "what must be 0..6");
    }
    dims[0] = M->n;
    dims[1] = M->nnzb();
    dims[2] = M->br;
    dims[3] = M->bc;
    if (indptr) std::copy(M->ptr.begin(), M->ptr.end(), indptr);
    if (indices) std::copy(M->col.begin(), M->col.end(), indices);
    if (vals) std::copy(M->val.begin(), M->val.end(), vals);
    return FEM_OK;
}
