// Device-resident block-preconditioned conjugate gradients on the 3x3-block BSR matrix.
// Replaces pardisoSolver(KL, mtype=2).factor()/solve(F) of SOLVE_static.py:31-33.
//
// One PCG iteration is three kernels (p = z + beta p;  q = A p with p.q;  x += alpha p,
// r -= alpha q, z = M r with r.z and r.r).  All scalars live in a device state block:
// every reduction writes per-CTA partials and the last CTA to finish (atomic ticket) sums
// them in CTA order, so results are bitwise reproducible, and computes alpha / beta /
// convergence on the device.  Each kernel returns immediately once the state says the
// solve is done, so a CUDA graph holding `unroll` iterations can be replayed without a
// host round trip per iteration; the host reads the state once per replay and stops at
// convergence or at the iteration cap.  Up to 32 right-hand sides run in lockstep with
// per-RHS alpha / beta and a per-RHS convergence mask (converged systems freeze).
//
// Mixed precision: the inner PCG runs with an FP32 matrix, FP32 vectors and FP32
// preconditioner blocks (dot products accumulated in FP64); an FP64 iterative-refinement
// loop forms the true residual r = F - K u with the FP64 matrix, scales it to unit norm,
// solves K d = r approximately in FP32, and updates u += |r| d in FP64.
#include <algorithm>
#include <vector>

#include "amg.cuh"
#include "pcg.cuh"

namespace fem {

int bsr_spmv_any(const fem_bsr* A, int nrhs, const void* x, void* y, int variant, cudaStream_t st);

namespace {

using namespace pcgd;

// x = 0, r = b, z = M r; rz, rr -> state (bb = rr, tol2 = rtol^2 bb).
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_init(int64_t n, const T* __restrict__ M, const T* __restrict__ b,
                                                    T* x, T* r, T* z, double* part, PcgState* st, double rtol,
                                                    int maxit) {
    double v[2] = {0.0, 0.0};
    Dot<T> d_rz, d_rr;
    const int64_t total_t = n * R;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < ((total_t + 31) / 32) * 32;
         t += int64_t(gridDim.x) * blockDim.x) {
        if (t < total_t) {
            const int64_t node = t / R;
            const int k = int(t % R);
            const int64_t o = 3 * node * R + k;
            const T r0 = b[o], r1 = b[o + R], r2 = b[o + 2 * R];
            T z0, z1, z2;
            apply_block(M + 9 * node, r0, r1, r2, z0, z1, z2);
            x[o] = 0;
            x[o + R] = 0;
            x[o + 2 * R] = 0;
            r[o] = r0;
            r[o + R] = r1;
            r[o + 2 * R] = r2;
            z[o] = z0;
            z[o + R] = z1;
            z[o + 2 * R] = z2;
            d_rz.add(r0, z0);
            d_rz.add(r1, z1);
            d_rz.add(r2, z2);
            d_rr.add(r0, r0);
            d_rr.add(r1, r1);
            d_rr.add(r2, r2);
        }
    }
    v[0] = d_rz.value();
    v[1] = d_rr.value();
    if (!block_partials<R, 2>(v, part, &st->ticket)) return;
    __shared__ double tot[2][kMaxR];
    last_block_totals<R, 2>(part, gridDim.x, tot);
    if (threadIdx.x == 0) {
        int any = 0, status = FEM_OK;
        for (int k = 0; k < kMaxR; ++k) {
            double rz = 0.0, rr = 0.0;
            if (k < R) {
                rz = tot[0][k];
                rr = tot[1][k];
            }
            const bool finite = isfinite(rz) && isfinite(rr);
            if (!finite) status = FEM_ERR_BREAKDOWN;
            st->rz[k] = rz;
            st->bb[k] = rr;
            st->rr[k] = rr;
            st->tol2[k] = rtol * rtol * rr;
            st->active[k] = (k < R && finite && rr > 0.0) ? 1 : 0;
            st->beta[k] = 0.0;
            st->alpha[k] = 0.0;
            st->iters[k] = 0;
            any |= st->active[k];
        }
        st->it = 0;
        st->done = !any;
        st->status = status;
        st->maxit = maxit;
        st->ticket = 0;
    }
}

// p = z + beta p  (p = z on the first iteration)
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_p_update(int64_t nv, const T* __restrict__ z, T* p,
                                                        const PcgState* __restrict__ st) {
    if (st->done) return;
    const bool first = st->it == 0;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nv; e += int64_t(gridDim.x) * blockDim.x) {
        const int k = int(e % R);
        p[e] = first ? z[e] : T(z[e] + T(st->beta[k]) * p[e]);
    }
}

// q = A p and p.q -> alpha = rz / pq on the device.  (Folding p = z + beta p into this
// kernel as q = A z + beta q was measured slower: the row epilogue's extra loads sit on the
// product's critical path, and the recurrence drifts from A p in FP32.)
template <typename T, int LPR_OR_R>
__global__ void __launch_bounds__(kThreads) k_spmv_pq(const BsrView<T> A, const T* __restrict__ p, T* __restrict__ q,
                                                       double* part, PcgState* st, int R) {
    if (st->done) return;
    double v[1];
    if (R == 1)
        v[0] = spmv1_rows<T, LPR_OR_R>(A, p, q, true);
    else
        v[0] = spmm_rows<T, LPR_OR_R>(A, p, q, true);
    constexpr int RR = LPR_OR_R;
    __shared__ double tot[1][kMaxR];
    bool last;
    if (R == 1) {
        last = block_partials<1, 1>(v, part, &st->ticket);
        if (last) last_block_totals<1, 1>(part, gridDim.x, tot);
    } else {
        last = block_partials<RR, 1>(v, part, &st->ticket);
        if (last) last_block_totals<RR, 1>(part, gridDim.x, tot);
    }
    if (last) {
        const int k = threadIdx.x;
        if (k < R) {
            if (st->active[k]) {
                const double pq = tot[0][k];
                st->pq[k] = pq;
                if (pq > 0.0 && isfinite(pq)) {
                    st->alpha[k] = st->rz[k] / pq;
                } else {
                    st->alpha[k] = 0.0;
                    st->active[k] = 0;
                    st->status = isfinite(pq) ? FEM_ERR_NOT_SPD : FEM_ERR_BREAKDOWN;
                }
            } else {
                st->alpha[k] = 0.0;  // converged systems stay frozen
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) st->ticket = 0;
    }
}

// x += alpha p; r -= alpha q; z = M r; rz, rr -> beta, convergence, iteration count.
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_update(int64_t n, const T* __restrict__ M, const T* __restrict__ p,
                                                      const T* __restrict__ q, T* x, T* r, T* z, double* part,
                                                      PcgState* st) {
    if (st->done) return;
    double v[2] = {0.0, 0.0};
    Dot<T> d_rz, d_rr;
    const int64_t total_t = n * R;
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < ((total_t + 31) / 32) * 32;
         t += int64_t(gridDim.x) * blockDim.x) {
        if (t < total_t) {
            const int64_t node = t / R;
            const int k = int(t % R);
            const int64_t o = 3 * node * R + k;
            const T a = T(st->alpha[k]);
            x[o] += a * p[o];
            x[o + R] += a * p[o + R];
            x[o + 2 * R] += a * p[o + 2 * R];
            const T r0 = r[o] - a * q[o], r1 = r[o + R] - a * q[o + R], r2 = r[o + 2 * R] - a * q[o + 2 * R];
            r[o] = r0;
            r[o + R] = r1;
            r[o + 2 * R] = r2;
            T z0, z1, z2;
            apply_block(M + 9 * node, r0, r1, r2, z0, z1, z2);
            z[o] = z0;
            z[o + R] = z1;
            z[o + 2 * R] = z2;
            d_rz.add(r0, z0);
            d_rz.add(r1, z1);
            d_rz.add(r2, z2);
            d_rr.add(r0, r0);
            d_rr.add(r1, r1);
            d_rr.add(r2, r2);
        }
    }
    v[0] = d_rz.value();
    v[1] = d_rr.value();
    if (block_partials<R, 2>(v, part, &st->ticket)) {
        __shared__ double tot[2][kMaxR];
        last_block_totals<R, 2>(part, gridDim.x, tot);
        const int k = threadIdx.x;
        if (k < R && st->active[k]) {
            const double rz = tot[0][k], rr = tot[1][k];
            st->beta[k] = rz / st->rz[k];
            st->rz[k] = rz;
            st->rr[k] = rr;
            st->iters[k] += 1;
            if (!(rr > st->tol2[k])) st->active[k] = 0;
            if (!isfinite(rr)) {
                st->active[k] = 0;
                st->status = FEM_ERR_BREAKDOWN;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int any = 0;
            for (int kk = 0; kk < R; ++kk) any |= st->active[kk];
            st->it += 1;
            if (any && st->it >= st->maxit) {
                st->status = st->status ? st->status : FEM_ERR_MAXITER;
                any = 0;
            }
            st->done = !any;
            st->ticket = 0;
        }
    }
}

// ---- multigrid-preconditioned iteration: the preconditioner is a V-cycle launched between
// k_update_r and k_rz, so r.z and beta move to a kernel of their own.  In the FP64 iteration
// the (FP32) cycle reads an FP32 copy of r written by k_update_r and k_rz widens its output;
// beta then takes the flexible (Polak-Ribiere) form beta = z_new.(r_new - r_old) / rz_old =
// -alpha q.z_new / rz_old, which tolerates the cycle's FP32 rounding. ----------------------
// x = 0, r = b (r32 = b when given); rr -> state (bb, tol2, active).
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_init_r(int64_t nv, const T* __restrict__ b, T* x, T* r, float* r32,
                                                      double* part, PcgState* st, double rtol, int maxit) {
    double v[1];
    Dot<T> d_rr;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ((nv + 31) / 32) * 32;
         e += int64_t(gridDim.x) * blockDim.x) {
        if (e < nv) {
            const T b0 = b[e];
            x[e] = T(0);
            r[e] = b0;
            if (r32) r32[e] = float(b0);
            d_rr.add(b0, b0);
        }
    }
    v[0] = d_rr.value();
    if (!block_partials<R, 1>(v, part, &st->ticket)) return;
    __shared__ double tot[1][kMaxR];
    last_block_totals<R, 1>(part, gridDim.x, tot);
    if (threadIdx.x == 0) {
        int any = 0, status = FEM_OK;
        for (int k = 0; k < kMaxR; ++k) {
            const double rr = k < R ? tot[0][k] : 0.0;
            if (!isfinite(rr)) status = FEM_ERR_BREAKDOWN;
            st->rz[k] = 0.0;
            st->bb[k] = rr;
            st->rr[k] = rr;
            st->tol2[k] = rtol * rtol * rr;
            st->active[k] = (k < R && isfinite(rr) && rr > 0.0) ? 1 : 0;
            st->beta[k] = 0.0;
            st->alpha[k] = 0.0;
            st->iters[k] = 0;
            any |= st->active[k];
        }
        st->it = 0;
        st->done = !any;
        st->status = status;
        st->maxit = maxit;
        st->ticket = 0;
    }
}

// x += alpha p; r -= alpha q (r32 = r when given); rr -> convergence and iteration count.
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_update_r(int64_t nv, const T* __restrict__ p, const T* __restrict__ q,
                                                        T* x, T* r, float* r32, double* part, PcgState* st) {
    if (st->done) return;
    double v[1];
    Dot<T> d_rr;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ((nv + 31) / 32) * 32;
         e += int64_t(gridDim.x) * blockDim.x) {
        if (e < nv) {
            const T a = T(st->alpha[e % R]);
            x[e] += a * p[e];
            const T r0 = r[e] - a * q[e];
            r[e] = r0;
            if (r32) r32[e] = float(r0);
            d_rr.add(r0, r0);
        }
    }
    v[0] = d_rr.value();
    if (block_partials<R, 1>(v, part, &st->ticket)) {
        __shared__ double tot[1][kMaxR];
        last_block_totals<R, 1>(part, gridDim.x, tot);
        const int k = threadIdx.x;
        if (k < R && st->active[k]) {
            const double rr = tot[0][k];
            st->rr[k] = rr;
            st->iters[k] += 1;
            if (!(rr > st->tol2[k])) st->active[k] = 0;
            if (!isfinite(rr)) {
                st->active[k] = 0;
                st->status = FEM_ERR_BREAKDOWN;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int any = 0;
            for (int kk = 0; kk < R; ++kk) any |= st->active[kk];
            st->it += 1;
            if (any && st->it >= st->maxit) {
                st->status = st->status ? st->status : FEM_ERR_MAXITER;
                any = 0;
            }
            st->done = !any;
            st->ticket = 0;
        }
    }
}

// z = z32 when given (FP64 iteration); r.z (and q.z when q is given) -> beta, rz.
template <typename T, int R>
__global__ void __launch_bounds__(kThreads) k_rz(int64_t nv, const T* __restrict__ r, T* z, const float* z32,
                                                  const T* __restrict__ q, double* part, PcgState* st) {
    if (st->done) return;
    double v[2];
    Dot<T> d_rz, d_qz;
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ((nv + 31) / 32) * 32;
         e += int64_t(gridDim.x) * blockDim.x) {
        if (e < nv) {
            T ze;
            if (z32) {
                ze = T(z32[e]);
                z[e] = ze;
            } else {
                ze = z[e];
            }
            d_rz.add(r[e], ze);
            if (q) d_qz.add(q[e], ze);
        }
    }
    v[0] = d_rz.value();
    v[1] = d_qz.value();
    if (block_partials<R, 2>(v, part, &st->ticket)) {
        __shared__ double tot[2][kMaxR];
        last_block_totals<R, 2>(part, gridDim.x, tot);
        const int k = threadIdx.x;
        if (k < R && st->active[k]) {
            const double rz = tot[0][k];
            if (rz > 0.0 && isfinite(rz)) {
                if (st->it > 0) st->beta[k] = q ? -st->alpha[k] * tot[1][k] / st->rz[k] : rz / st->rz[k];
                st->rz[k] = rz;
            } else {
                st->active[k] = 0;
                st->status = isfinite(rz) ? FEM_ERR_NOT_SPD : FEM_ERR_BREAKDOWN;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int any = 0;
            for (int kk = 0; kk < R; ++kk) any |= st->active[kk];
            st->done = !any;
            st->ticket = 0;
        }
    }
}

// ---- FP64 refinement helpers --------------------------------------------------------------
// r = b - y (y = A u computed by the SpMV), norms of r per RHS -> st->norm2.
template <int R>
__global__ void __launch_bounds__(kThreads) k_residual(int64_t nv, const double* __restrict__ b,
                                                        const double* __restrict__ y, double* r, double* part,
                                                        PcgState* st) {
    double v[1] = {0.0};
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ((nv + 31) / 32) * 32;
         e += int64_t(gridDim.x) * blockDim.x) {
        if (e < nv) {
            const double d = b[e] - y[e];
            r[e] = d;
            v[0] += d * d;
        }
    }
    if (block_partials<R, 1>(v, part, &st->ticket)) {
        __shared__ double tot[1][kMaxR];
        last_block_totals<R, 1>(part, gridDim.x, tot);
        if (threadIdx.x < R) st->norm2[threadIdx.x] = tot[0][threadIdx.x];
        __syncthreads();
        if (threadIdx.x == 0) st->ticket = 0;
    }
}

// True residual r = F - A u per scalar row with its rounding scale |F| + |A||u|; per RHS
// ||r||^2 -> st->norm2 and || |F| + |A||u| ||^2 -> st->anorm2.  kExtra: each row sum is the
// compensated dot product "Dot2" of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26 (2005)
// 1955-1988): every product is split exactly into its rounded value and error by an FMA,
// every addition by Knuth's two-sum, and the errors are summed alongside, so r is as
// accurate as if formed in twice the FP64 precision and then rounded.  Without kExtra the
// row sums are plain FP64 FMAs (rounding error up to ~(row length) x 2^-53 x the scale).
template <int R, bool kExtra>
__global__ void __launch_bounds__(kThreads) k_residual_ex(const BsrView<double> A, const double* __restrict__ F,
                                                          const double* __restrict__ u, double* r, double* part,
                                                          PcgState* st) {
    const int64_t nv = 3 * A.n * R;
    double v[2] = {0.0, 0.0};
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < ((nv + 31) / 32) * 32;
         e += int64_t(gridDim.x) * blockDim.x) {
        if (e < nv) {
            const int64_t rowc = e / R;  // scalar row 3 node + c
            const int k = int(e % R);
            const int64_t node = rowc / 3;
            const int c = int(rowc - 3 * node);
            const int64_t rs = __ldg(A.indptr + node);
            const int L = __ldg(A.indptr + node + 1) - int(rs);
            const double f = F[e];
            double s = f, comp = 0.0, sc = fabs(f);
            for (int l = 0; l < L; ++l) {
                const int64_t col = __ldg(A.indices + rs + l);
                const double* ub = u + 3 * col * R + k;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const double m = __ldg(block_value(A, rs, L, l, 3 * c + q));
                    const double x = ub[q * R];
                    sc = fma(fabs(m), fabs(x), sc);
                    if (kExtra) {
                        const double pr = __dmul_rn(m, x);
                        const double pe = fma(m, x, -pr);  // m x = pr + pe exactly
                        const double t = __dsub_rn(s, pr);
                        const double bb = __dsub_rn(t, s);
                        const double err = __dadd_rn(__dsub_rn(s, __dsub_rn(t, bb)), __dsub_rn(-pr, bb));
                        s = t;
                        comp = __dsub_rn(__dadd_rn(comp, err), pe);
                    } else {
                        s = fma(-m, x, s);
                    }
                }
            }
            const double rv = kExtra ? __dadd_rn(s, comp) : s;
            r[e] = rv;
            v[0] = fma(rv, rv, v[0]);
            v[1] = fma(sc, sc, v[1]);
        }
    }
    if (block_partials<R, 2>(v, part, &st->ticket)) {
        __shared__ double tot[2][kMaxR];
        last_block_totals<R, 2>(part, gridDim.x, tot);
        if (threadIdx.x < R) {
            st->norm2[threadIdx.x] = tot[0][threadIdx.x];
            st->anorm2[threadIdx.x] = tot[1][threadIdx.x];
        }
        __syncthreads();
        if (threadIdx.x == 0) st->ticket = 0;
    }
}

// r_k = 0 for the right-hand sides whose scale s_k is 0 (already converged)
template <int R>
__global__ void k_mask_rhs(int64_t nv, const double* __restrict__ s, double* r) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nv; e += int64_t(gridDim.x) * blockDim.x)
        if (!(s[e % R] > 0.0)) r[e] = 0.0;
}

// u += d
__global__ void k_add(int64_t n, const double* __restrict__ d, double* u) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x)
        u[e] += d[e];
}

// b32 = r / s_k (s_k = 0 -> zero right-hand side)
template <int R>
__global__ void k_scale_cast(int64_t nv, const double* __restrict__ r, const double* __restrict__ s, float* b32) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nv; e += int64_t(gridDim.x) * blockDim.x) {
        const double sk = s[e % R];
        b32[e] = sk > 0.0 ? float(r[e] / sk) : 0.0f;
    }
}

// u += s_k d
template <int R>
__global__ void k_axpy_cast(int64_t nv, const double* __restrict__ s, const float* __restrict__ d, double* u) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < nv; e += int64_t(gridDim.x) * blockDim.x)
        u[e] += s[e % R] * double(d[e]);
}

__global__ void k_zero(int64_t n, double* u) {
    for (int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; e < n; e += int64_t(gridDim.x) * blockDim.x)
        u[e] = 0.0;
}

// ---- host side ------------------------------------------------------------------------------
struct Layout {
    size_t state, part, v64[6], v32[6], m32, scale, total;
};

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

Layout layout(int64_t n, int R, int mixed) {
    Layout L{};
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes);
        return o;
    };
    const size_t nv = size_t(3) * n * R;
    L.state = take(sizeof(PcgState));
    L.part = take(sizeof(double) * kMaxCtas * kSlots * kMaxR);
    for (int i = 0; i < 6; ++i) L.v64[i] = take(mixed ? (i < 2 ? sizeof(double) * nv : 0) : sizeof(double) * nv);
    for (int i = 0; i < 6; ++i) L.v32[i] = take(mixed ? sizeof(float) * nv : 0);
    L.m32 = take(mixed ? sizeof(float) * 9 * n : 0);
    L.scale = take(sizeof(double) * kMaxR);
    L.total = off;
    return L;
}

// Grid of a grid-stride vector kernel over `work` items: one wave of resident CTAs (these
// kernels stream HBM and need every warp slot to keep enough loads in flight), at most
// kMaxCtas (the partial-sum buffer of their dot products).
template <typename Kernel>
unsigned vec_grid(Kernel kernel, int64_t work) {
    return resident_grid(reinterpret_cast<const void*>(kernel), kThreads, (work + kThreads - 1) / kThreads, kMaxCtas);
}

// Grid of the product kernel: one wave of resident CTAs (grid-stride rows), at most kMaxCtas
// (the size of the partial-sum buffer).  The grid fixes each row's CTA, hence the order of the
// dot-product partial sums.
template <typename T, int R>
void launch_spmv_pq(const BsrView<T>& A, const T* p, T* q, double* part, PcgState* st, int variant, cudaStream_t s) {
    auto run = [&](auto kernel, int64_t rows_per_cta, int64_t cap, int r) {
        const unsigned g = resident_grid(reinterpret_cast<const void*>(kernel), kThreads,
                                         (A.n + rows_per_cta - 1) / rows_per_cta, std::min<int64_t>(cap, kMaxCtas));
        kernel<<<g, kThreads, 0, s>>>(A, p, q, part, st, r);
    };
    if (R > 1) {
        run(k_spmv_pq<T, R>, int64_t(kThreads / 32) * (32 / R), int64_t(sm_count()) * 8, R);
        return;
    }
    const SpmvVariant v = spmv_variant(variant);
    const int64_t rows_per_cta = int64_t(kThreads / 32) * (32 / v.lpr);
    const int64_t cap = int64_t(sm_count()) * (v.ctas_per_sm * v.threads / kThreads);
    switch (v.lpr) {
        case 32: run(k_spmv_pq<T, 32>, rows_per_cta, cap, 1); break;
        case 16: run(k_spmv_pq<T, 16>, rows_per_cta, cap, 1); break;
        case 8: run(k_spmv_pq<T, 8>, rows_per_cta, cap, 1); break;
        case 4: run(k_spmv_pq<T, 4>, rows_per_cta, cap, 1); break;
        default: run(k_spmv_pq<T, 2>, rows_per_cta, cap, 1); break;
    }
}

template <typename T, int R>
int launch_iterations(const BsrView<T>& A, const T* M, T* x, T* r, T* z, T* p, T* q, double* part, PcgState* st,
                      int variant, int count, cudaStream_t s) {
    const int64_t nv = 3 * A.n * R;
    for (int i = 0; i < count; ++i) {
        k_p_update<T, R><<<vec_grid(k_p_update<T, R>, nv), kThreads, 0, s>>>(nv, z, p, st);
        launch_spmv_pq<T, R>(A, p, q, part, st, variant, s);
        k_update<T, R><<<vec_grid(k_update<T, R>, A.n * R), kThreads, 0, s>>>(A.n, M, p, q, x, r, z, part, st);
    }
    FEM_LAUNCH_CHECK("pcg iteration");
    return FEM_OK;
}

struct InnerResult {
    int iters, status;
};

// Initialises the solver state (init(s)), then runs `unroll` iterations at a time
// (iters(count, s), replayed as one CUDA graph when use_graph) until the state says done.
// stall > 0: the solve also ends, with FEM_ERR_NOT_CONVERGED, once the largest relative
// recursive residual over the active right-hand sides has not halved within `stall`
// iterations (checked at every host check, i.e. every `unroll` iterations).
template <typename Init, typename Iters>
int pcg_drive(const Init& init, const Iters& iters, PcgState* st, int maxit, int use_graph, int unroll,
              cudaStream_t s, InnerResult* res, int stall = 0) {
    int rc0 = init(s);
    if (rc0) return rc0;
    unroll = std::max(1, std::min(unroll, 256));
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        cudaGraph_t g = nullptr;
        FEM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        int rc = iters(unroll, s);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc) return rc;
        FEM_CUDA(ce);
        ce = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        FEM_CUDA(ce);
    }
    PcgState h;
    int launched = 0, rc = FEM_OK;
    bool stalled = false;
    double ref = -1.0;  // residual at the last halving
    int ref_it = 0;
    // the device caps iterations at maxit; the host loop is bounded by the same count
    while (launched < maxit + unroll) {
        if (exec) {
            rc = cuda_status(cudaGraphLaunch(exec, s), "cudaGraphLaunch");
        } else {
            rc = iters(unroll, s);
        }
        if (rc) break;
        launched += unroll;
        rc = cuda_status(cudaMemcpyAsync(&h, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s), "state copy");
        if (rc) break;
        rc = cuda_status(cudaStreamSynchronize(s), "state sync");
        if (rc || h.done) break;
        if (stall > 0) {
            double w = 0.0;
            for (int k = 0; k < kMaxR; ++k)
                if (h.active[k] && h.bb[k] > 0.0) w = std::max(w, sqrt(h.rr[k] / h.bb[k]));
            if (ref < 0.0 || w <= 0.5 * ref) {
                ref = w;
                ref_it = h.it;
            } else if (h.it - ref_it >= stall) {
                stalled = true;
                break;
            }
        }
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (rc) return rc;
    res->iters = h.it;
    res->status = h.done ? h.status : (stalled ? FEM_ERR_NOT_CONVERGED : FEM_ERR_MAXITER);
    return FEM_OK;
}

// Runs PCG on (A, M) with right-hand side b into x; vectors r z p q are workspace.
template <typename T, int R>
int pcg_core(const BsrView<T>& A, const T* M, const T* b, T* x, T* r, T* z, T* p, T* q, double* part, PcgState* st,
             double rtol, int maxit, int variant, int use_graph, int unroll, cudaStream_t s, InnerResult* res,
             int stall = 0) {
    auto init = [&](cudaStream_t ss) -> int {
        k_init<T, R><<<vec_grid(k_init<T, R>, A.n * R), kThreads, 0, ss>>>(A.n, M, b, x, r, z, part, st, rtol, maxit);
        FEM_LAUNCH_CHECK("k_init");
        return FEM_OK;
    };
    auto iters = [&](int count, cudaStream_t ss) -> int {
        return launch_iterations<T, R>(A, M, x, r, z, p, q, part, st, variant, count, ss);
    };
    return pcg_drive(init, iters, st, maxit, use_graph, unroll, s, res, stall);
}

// The same with the multigrid V-cycle as the preconditioner.  T = float: the FP32 inner
// solve (A the FP32 matrix, which the cycle also uses).  T = double: FP64 vectors and
// products with A, the cycle in FP32 on A32 through the handle's FP32 copies of r and z.
template <typename T, int R>
int pcg_core_amg(const BsrView<T>& A, const BsrView<float>& A32, fem_amg* amg, const T* b, T* x, T* r, T* z, T* p,
                 T* q, double* part, PcgState* st, double rtol, int maxit, int variant, int use_graph, int unroll,
                 cudaStream_t s, InnerResult* res, int stall = 0) {
    const int64_t nv = 3 * A.n * R;
    constexpr bool f64 = sizeof(T) == 8;
    float* r32 = f64 ? amg->r32 : nullptr;
    float* z32 = f64 ? amg->z32 : nullptr;
    const float* rin = f64 ? r32 : reinterpret_cast<const float*>(r);
    float* zout = f64 ? z32 : reinterpret_cast<float*>(z);
    const T* qflex = f64 ? q : nullptr;
    auto init = [&](cudaStream_t ss) -> int {
        k_init_r<T, R><<<vec_grid(k_init_r<T, R>, nv), kThreads, 0, ss>>>(nv, b, x, r, r32, part, st, rtol, maxit);
        FEM_LAUNCH_CHECK("k_init_r");
        int rc = amg::vcycle(amg, A32, rin, zout, st, R, f64, ss);
        if (rc) return rc;
        k_rz<T, R><<<vec_grid(k_rz<T, R>, nv), kThreads, 0, ss>>>(nv, r, z, z32, nullptr, part, st);
        FEM_LAUNCH_CHECK("k_rz");
        return FEM_OK;
    };
    auto iters = [&](int count, cudaStream_t ss) -> int {
        for (int i = 0; i < count; ++i) {
            k_p_update<T, R><<<vec_grid(k_p_update<T, R>, nv), kThreads, 0, ss>>>(nv, z, p, st);
            launch_spmv_pq<T, R>(A, p, q, part, st, variant, ss);
            k_update_r<T, R><<<vec_grid(k_update_r<T, R>, nv), kThreads, 0, ss>>>(nv, p, q, x, r, r32, part, st);
            int rc = amg::vcycle(amg, A32, rin, zout, st, R, f64, ss);
            if (rc) return rc;
            k_rz<T, R><<<vec_grid(k_rz<T, R>, nv), kThreads, 0, ss>>>(nv, r, z, z32, qflex, part, st);
        }
        FEM_LAUNCH_CHECK("pcg iteration (amg)");
        return FEM_OK;
    };
    return pcg_drive(init, iters, st, maxit, use_graph, unroll, s, res, stall);
}

template <int R>
int solve_r(const fem_bsr* A64, const fem_bsr* A32, const double* M64, fem_amg* amg, const double* F, double* U,
            const fem_pcg_opts* o, fem_pcg_stats* out, unsigned char* ws, cudaStream_t s) {
    const int64_t n = A64->n_brow;
    const int64_t nv = 3 * n * R;
    const Layout L = layout(n, R, o->mixed);
    PcgState* st = reinterpret_cast<PcgState*>(ws + L.state);
    double* part = reinterpret_cast<double*>(ws + L.part);
    double* scale = reinterpret_cast<double*>(ws + L.scale);
    BsrView<double> K64{n, A64->indptr, A64->indices, static_cast<const double*>(A64->vals),
                        rsoa_kind(A64->layout)};
    const int maxit = std::max(1, o->maxit);
    const bool extra = o->residual == FEM_RESIDUAL_EXTRA;
    InnerResult ir{0, FEM_OK};
    PcgState h;
    // r = F - K u (FP64 or compensated), its norms and rounding scales -> h
    auto true_residual = [&](const double* u, double* r) -> int {
        if (extra)
            k_residual_ex<R, true><<<vec_grid(k_residual_ex<R, true>, nv), kThreads, 0, s>>>(K64, F, u, r, part, st);
        else
            k_residual_ex<R, false><<<vec_grid(k_residual_ex<R, false>, nv), kThreads, 0, s>>>(K64, F, u, r, part, st);
        FEM_LAUNCH_CHECK("k_residual_ex");
        FEM_CUDA(cudaMemcpyAsync(&h, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
        FEM_CUDA(cudaStreamSynchronize(s));
        return FEM_OK;
    };
    // the reduction ticket and all scalars start from zero (the workspace is uninitialised)
    FEM_CUDA(cudaMemsetAsync(st, 0, sizeof(PcgState), s));
    double bnorm[kMaxR];
    {
        // ||F_k||: the residual of u = 0
        double* z0 = reinterpret_cast<double*>(ws + L.v64[0]);
        double* r0 = reinterpret_cast<double*>(ws + L.v64[1]);
        k_zero<<<vec_grid(k_zero, nv), kThreads, 0, s>>>(nv, z0);
        FEM_LAUNCH_CHECK("k_zero");
        k_residual_ex<R, false><<<vec_grid(k_residual_ex<R, false>, nv), kThreads, 0, s>>>(K64, F, z0, r0, part, st);
        FEM_LAUNCH_CHECK("k_residual_ex");
        FEM_CUDA(cudaMemcpyAsync(&h, st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
        FEM_CUDA(cudaStreamSynchronize(s));
        for (int k = 0; k < R; ++k) bnorm[k] = sqrt(h.norm2[k]);
    }
    // relative true residual per RHS from h, worst over the RHS
    auto rel = [&](int k) { return bnorm[k] > 0 ? sqrt(h.norm2[k]) / bnorm[k] : 0.0; };
    auto worst_rel = [&]() {
        double w = 0.0;
        for (int k = 0; k < R; ++k) w = std::max(w, rel(k));
        return w;
    };
    // scale[k] = ||r_k|| for the RHS still above rtol, 0 for the others; returns how many
    auto set_active = [&](double* sc) {
        int any = 0;
        for (int k = 0; k < R; ++k) {
            const bool act = bnorm[k] > 0 && rel(k) > o->rtol;
            sc[k] = act ? sqrt(h.norm2[k]) : 0.0;
            any += act;
        }
        return any;
    };
    int total_iters = 0, outer = 0, status = FEM_OK;
    const int max_outer = std::max(1, o->max_outer);
    if (!o->mixed) {
        // FP64 PCG on K U = F, then residual replacement: while the true residual is above
        // rtol (the recursive residual drifts from it on ill-conditioned systems), solve
        // K d = r for the correction and add it (at most max_outer solves in all; stop when
        // a step does not halve the worst residual).
        double* r = reinterpret_cast<double*>(ws + L.v64[0]);
        double* z = reinterpret_cast<double*>(ws + L.v64[1]);
        double* p = reinterpret_cast<double*>(ws + L.v64[2]);
        double* q = reinterpret_cast<double*>(ws + L.v64[3]);
        double* rt = reinterpret_cast<double*>(ws + L.v64[4]);
        double* d = reinterpret_cast<double*>(ws + L.v64[5]);
        auto core = [&](const double* b, double* x, double tol, int cap) -> int {
            if (amg) {
                const BsrView<float> K32{n, A32->indptr, A32->indices, static_cast<const float*>(A32->vals),
                                         rsoa_kind(A32->layout)};
                return pcg_core_amg<double, R>(K64, K32, amg, b, x, r, z, p, q, part, st, tol, cap, o->spmv_variant,
                                               o->use_graph, o->unroll, s, &ir, o->stall_window);
            }
            return pcg_core<double, R>(K64, M64, b, x, r, z, p, q, part, st, tol, cap, o->spmv_variant,
                                       o->use_graph, o->unroll, s, &ir, o->stall_window);
        };
        int rc = core(F, U, o->rtol, maxit);
        if (rc) return rc;
        total_iters = ir.iters;
        status = ir.status;
        outer = 1;
        if ((rc = true_residual(U, rt))) return rc;
        double prev = worst_rel();
        while (status == FEM_OK && outer < max_outer && total_iters < maxit) {
            double sc[kMaxR];
            if (!set_active(sc)) break;
            // the correction must bring ||r_k|| down to rtol ||F_k|| for every active RHS
            double tol = 0.5;
            for (int k = 0; k < R; ++k)
                if (sc[k] > 0) tol = std::min(tol, o->rtol * bnorm[k] / sc[k]);
            tol = std::max(tol, 1e-15);
            FEM_CUDA(cudaMemcpyAsync(scale, sc, sizeof(double) * R, cudaMemcpyHostToDevice, s));
            k_mask_rhs<R><<<vec_grid(k_mask_rhs<R>, nv), kThreads, 0, s>>>(nv, scale, rt);
            FEM_LAUNCH_CHECK("k_mask_rhs");
            if ((rc = core(rt, d, tol, maxit - total_iters))) return rc;
            total_iters += ir.iters;
            ++outer;
            if (ir.status == FEM_ERR_BREAKDOWN || ir.status == FEM_ERR_NOT_SPD) {
                status = ir.status;
                break;
            }
            k_add<<<vec_grid(k_add, nv), kThreads, 0, s>>>(nv, d, U);
            FEM_LAUNCH_CHECK("k_add");
            if ((rc = true_residual(U, rt))) return rc;
            const double w = worst_rel();
            if (!(w < 0.5 * prev)) break;  // no further progress: the FP64 floor is reached
            prev = w;
        }
    } else {
        BsrView<float> K32{n, A32->indptr, A32->indices, static_cast<const float*>(A32->vals),
                           rsoa_kind(A32->layout)};
        double* r64 = reinterpret_cast<double*>(ws + L.v64[1]);
        float* b32 = reinterpret_cast<float*>(ws + L.v32[0]);
        float* d32 = reinterpret_cast<float*>(ws + L.v32[1]);
        float* rr = reinterpret_cast<float*>(ws + L.v32[2]);
        float* zz = reinterpret_cast<float*>(ws + L.v32[3]);
        float* pp = reinterpret_cast<float*>(ws + L.v32[4]);
        float* qq = reinterpret_cast<float*>(ws + L.v32[5]);
        float* M32 = reinterpret_cast<float*>(ws + L.m32);
        int rc = amg ? FEM_OK : fem_convert_f64_to_f32(M64, M32, 9 * n, s);
        if (rc) return rc;
        k_zero<<<vec_grid(k_zero, nv), kThreads, 0, s>>>(nv, U);
        FEM_LAUNCH_CHECK("k_zero");
        rc = true_residual(U, r64);
        if (rc) return rc;
        double prev = 1e300;
        for (outer = 0; outer < max_outer; ++outer) {
            double sc[kMaxR];
            if (!set_active(sc)) break;
            const double worst = worst_rel();
            if (outer > 0 && !(worst < 0.5 * prev)) break;  // refinement stalled
            prev = worst;
            FEM_CUDA(cudaMemcpyAsync(scale, sc, sizeof(double) * R, cudaMemcpyHostToDevice, s));
            k_scale_cast<R><<<vec_grid(k_scale_cast<R>, nv), kThreads, 0, s>>>(nv, r64, scale, b32);
            FEM_LAUNCH_CHECK("k_scale_cast");
            if (amg)
                rc = pcg_core_amg<float, R>(K32, K32, amg, b32, d32, rr, zz, pp, qq, part, st, o->inner_rtol,
                                            std::max(1, o->inner_maxit), o->spmv_variant32, o->use_graph, o->unroll,
                                            s, &ir, o->stall_window);
            else
                rc = pcg_core<float, R>(K32, M32, b32, d32, rr, zz, pp, qq, part, st, o->inner_rtol,
                                        std::max(1, o->inner_maxit), o->spmv_variant32, o->use_graph, o->unroll, s,
                                        &ir, o->stall_window);
            if (rc) return rc;
            total_iters += ir.iters;
            if (o->stall_window > 0 && ir.status == FEM_ERR_NOT_CONVERGED) {
                status = FEM_ERR_NOT_CONVERGED;  // the inner solve stalled
                break;
            }
            if (ir.status == FEM_ERR_BREAKDOWN || ir.status == FEM_ERR_NOT_SPD) {
                status = ir.status;
                break;
            }
            k_axpy_cast<R><<<vec_grid(k_axpy_cast<R>, nv), kThreads, 0, s>>>(nv, scale, d32, U);
            FEM_LAUNCH_CHECK("k_axpy_cast");
            rc = true_residual(U, r64);
            if (rc) return rc;
            if (total_iters >= maxit) {
                status = FEM_ERR_MAXITER;
                break;
            }
        }
    }
    // The status is judged on the true residual of the returned U, whatever the mode: a solve
    // that stopped above rtol (iteration cap, stall, recursive residual drifting from the true
    // one) does not report success.
    const double worst = worst_rel();
    double floor_rel = 0.0;
    for (int k = 0; k < R; ++k)
        if (bnorm[k] > 0) floor_rel = std::max(floor_rel, 0x1p-53 * sqrt(h.anorm2[k]) / bnorm[k]);
    if (status == FEM_OK && worst > o->rtol) status = total_iters >= maxit ? FEM_ERR_MAXITER : FEM_ERR_NOT_CONVERGED;
    out->status = status;
    out->iterations = total_iters;
    out->outer = outer;
    out->relres = worst;
    out->floor = floor_rel;
    return FEM_OK;
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" size_t fem_pcg_workspace_bytes(int64_t n_brow, int nrhs, int mixed) {
    if (n_brow < 0 || nrhs < 1 || nrhs > kMaxR) return 0;
    return layout(n_brow, nrhs, mixed ? 1 : 0).total;
}

namespace fem {
namespace {

int run_solve(const fem_bsr* A64, const fem_bsr* A32, const double* precond, fem_amg* amg, const double* F,
              double* U, const fem_pcg_opts* opts, fem_pcg_stats* stats, void* workspace, size_t workspace_bytes,
              void* stream) {
    FEM_REQUIRE(A64 && opts && stats && (precond || amg) && F && U, "NULL argument");
    FEM_REQUIRE(A64->dtype == FEM_F64 && A64->n_brow > 0 && A64->indptr && A64->indices && A64->vals,
                "A64 must be a non-empty FP64 BSR matrix");
    FEM_REQUIRE(A64->layout == FEM_LAYOUT_BSR || A64->layout == FEM_LAYOUT_RSOA, "A64: layout must be BSR or RSOA");
    const int R = opts->nrhs;
    FEM_REQUIRE(R == 1 || R == 2 || R == 4 || R == 8 || R == 16 || R == 32, "nrhs must be 1, 2, 4, 8, 16 or 32");
    FEM_REQUIRE(opts->rtol > 0 && opts->maxit > 0, "rtol and maxit must be positive");
    if (opts->mixed || amg) {
        FEM_REQUIRE(A32 && A32->dtype == FEM_F32 && A32->n_brow == A64->n_brow && A32->vals && A32->indptr &&
                        A32->indices,
                    "mixed precision needs the FP32 copy of the matrix (A32)");
        FEM_REQUIRE(A32->layout == FEM_LAYOUT_BSR || A32->layout == FEM_LAYOUT_RSOA || A32->layout == FEM_LAYOUT_RSOA4,
                    "A32: layout must be BSR, RSOA or RSOA4");
        FEM_REQUIRE(A32->layout != FEM_LAYOUT_RSOA4 ||
                        ((reinterpret_cast<uintptr_t>(A32->vals) | reinterpret_cast<uintptr_t>(A32->indices)) & 15u) == 0,
                    "A32: FEM_LAYOUT_RSOA4 arrays must be 16-byte aligned");
        FEM_REQUIRE(!opts->mixed || (opts->inner_rtol > 0 && opts->inner_rtol < 1), "inner_rtol must lie in (0, 1)");
    }
    if (amg) {
        FEM_REQUIRE(amg->uploaded, "call fem_amg_upload first");
        FEM_REQUIRE(amg->lv[0].n == A64->n_brow, "the AMG hierarchy belongs to a matrix of another size");
    }
    const Layout L = layout(A64->n_brow, R, opts->mixed);
    if (!workspace || workspace_bytes < L.total) {
        set_error("workspace too small: need %zu bytes", L.total);
        return FEM_ERR_WORKSPACE;
    }
    FEM_REQUIRE(aligned16(workspace), "workspace must be 16-byte aligned");
    if (amg) {
        // per-level vectors are allocated before any capture
        int rc = amg::ensure_vectors(amg, R);
        if (rc) return rc;
    }
    // Work on a private stream ordered after / before the caller's stream (graph capture
    // is not allowed on the legacy default stream).
    cudaStream_t caller = as_stream(stream), s = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, t0 = nullptr, t1 = nullptr;
    FEM_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    int rc = FEM_OK;
    auto cleanup = [&]() {
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (t0) cudaEventDestroy(t0);
        if (t1) cudaEventDestroy(t1);
        if (s) cudaStreamDestroy(s);
    };
    do {
        if ((rc = cuda_status(cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming), "event"))) break;
        if ((rc = cuda_status(cudaEventCreateWithFlags(&ev1, cudaEventDisableTiming), "event"))) break;
        if ((rc = cuda_status(cudaEventCreate(&t0), "event"))) break;
        if ((rc = cuda_status(cudaEventCreate(&t1), "event"))) break;
        if ((rc = cuda_status(cudaEventRecord(ev0, caller), "record"))) break;
        if ((rc = cuda_status(cudaStreamWaitEvent(s, ev0, 0), "wait"))) break;
        if ((rc = cuda_status(cudaEventRecord(t0, s), "record"))) break;
        unsigned char* ws = static_cast<unsigned char*>(workspace);
        switch (R) {
            case 1: rc = solve_r<1>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
            case 2: rc = solve_r<2>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
            case 4: rc = solve_r<4>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
            case 8: rc = solve_r<8>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
            case 16: rc = solve_r<16>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
            default: rc = solve_r<32>(A64, A32, precond, amg, F, U, opts, stats, ws, s); break;
        }
        if (rc) break;
        if ((rc = cuda_status(cudaEventRecord(t1, s), "record"))) break;
        if ((rc = cuda_status(cudaEventSynchronize(t1), "sync"))) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, t0, t1);
        stats->time_ms = ms;
        if ((rc = cuda_status(cudaEventRecord(ev1, s), "record"))) break;
        if ((rc = cuda_status(cudaStreamWaitEvent(caller, ev1, 0), "wait"))) break;
    } while (0);
    if (rc) cudaStreamSynchronize(s);
    cleanup();
    return rc;
}

}  // namespace
}  // namespace fem

extern "C" int fem_pcg_solve(const fem_bsr* A64, const fem_bsr* A32, const double* precond, const double* F,
                             double* U, const fem_pcg_opts* opts, fem_pcg_stats* stats, void* workspace,
                             size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(precond, "NULL argument");
    return run_solve(A64, A32, precond, nullptr, F, U, opts, stats, workspace, workspace_bytes, stream);
}

extern "C" int fem_pcg_solve_amg(const fem_bsr* A64, const fem_bsr* A32, fem_amg* amg, const double* F, double* U,
                                 const fem_pcg_opts* opts, fem_pcg_stats* stats, void* workspace,
                                 size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(amg, "NULL argument");
    return run_solve(A64, A32, nullptr, amg, F, U, opts, stats, workspace, workspace_bytes, stream);
}
