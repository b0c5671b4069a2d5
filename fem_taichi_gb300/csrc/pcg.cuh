// Pieces of the block-preconditioned CG solver (pcg.cu): solver state, per-CTA partial
// sums and their fixed-order reduction, block-Jacobi application.
#pragma once

#include "spmv.cuh"

namespace fem {
namespace pcgd {

constexpr int kMaxR = 32;
constexpr int kThreads = 256;
constexpr int kMaxCtas = 4096;
constexpr int kSlots = 3;

struct PcgState {
    double rz[kMaxR], pq[kMaxR], alpha[kMaxR], beta[kMaxR], bb[kMaxR], rr[kMaxR], tol2[kMaxR];
    double norm2[kMaxR];
    double anorm2[kMaxR];  // || |F| + |A||u| ||^2 of the last true residual (its rounding scale)
    int active[kMaxR];
    int iters[kMaxR];
    int it, done, status, maxit;
    unsigned ticket;
};

// Sum of v over the lanes of this warp that hold the same right-hand side (lane % R).
template <int R>
__device__ __forceinline__ double warp_rhs_sum(double v) {
#pragma unroll
    for (int off = 16; off >= R; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// This CTA's sums of v[s] (per RHS) into part[blockIdx.x] slots slot0 .. slot0 + NS - 1.
template <int R, int NS>
__device__ void write_partials(const double (&v)[NS], double* part, int slot0) {
    __shared__ double sm[kThreads / 32][NS][kMaxR];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        const double w = warp_rhs_sum<R>(v[s]);
        if (lane < R) sm[warp][s][lane] = w;
    }
    __syncthreads();
    if (threadIdx.x < R) {
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            double acc = 0.0;
            for (int w = 0; w < int(blockDim.x / 32); ++w) acc += sm[w][s][threadIdx.x];
            part[(int64_t(blockIdx.x) * kSlots + slot0 + s) * kMaxR + threadIdx.x] = acc;
        }
    }
}

// Block-level reduction of up to kSlots values per RHS into part[blockIdx.x]; returns true
// in every thread of the CTA that finished last (after which part[] is complete).
template <int R, int NS>
__device__ bool block_partials(const double (&v)[NS], double* part, unsigned* ticket) {
    __shared__ bool last;
    write_partials<R, NS>(v, part, 0);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (last) __threadfence();
    return last;
}

// In the last CTA (all threads call it): tot[s][k] = sum over CTAs of slot s, RHS k.  The
// kThreads / R threads of each RHS stride over the CTAs, then a fixed-shape tree in shared
// memory combines them, so the result does not depend on timing.
template <int R, int NS>
__device__ void last_block_totals(const double* part, int nblocks, double (&tot)[NS][kMaxR], int slot0 = 0) {
    constexpr int G = kThreads / R;
    __shared__ double red[NS][kThreads];
    const int t = threadIdx.x, k = t % R, g = t / R;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        double acc = 0.0;
        for (int b = g; b < nblocks; b += G) acc += __ldcg(part + (int64_t(b) * kSlots + slot0 + s) * kMaxR + k);
        red[s][t] = acc;
    }
    __syncthreads();
#pragma unroll
    for (int off = G / 2; off >= 1; off >>= 1) {
        if (g < off) {
#pragma unroll
            for (int s = 0; s < NS; ++s) red[s][t] += red[s][t + off * R];
        }
        __syncthreads();
    }
    if (t < R) {
#pragma unroll
        for (int s = 0; s < NS; ++s) tot[s][t] = red[s][t];
    }
    __syncthreads();
}

// z = M r for one node / RHS, M the node's 3x3 preconditioner block.
template <typename T>
__device__ __forceinline__ void apply_block(const T* __restrict__ Mi, T r0, T r1, T r2, T& z0, T& z1, T& z2) {
    z0 = Mi[0] * r0 + Mi[1] * r1 + Mi[2] * r2;
    z1 = Mi[3] * r0 + Mi[4] * r1 + Mi[5] * r2;
    z2 = Mi[6] * r0 + Mi[7] * r1 + Mi[8] * r2;
}

}  // namespace pcgd
}  // namespace fem
