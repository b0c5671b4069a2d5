// Learned correction of the block-Jacobi preconditioner (no reference counterpart).
//
// For node i with diagonal block D_i = G_i G_i^T (Cholesky), a 3-layer per-node MLP
// (16 -> 64 -> 64 -> 6, SiLU, BF16 weights and activations, FP32 accumulation) emits the
// Cholesky factor L_i of an SPD 3x3 matrix C_i = L_i L_i^T, and the preconditioner block is
// P_i = G_i^{-T} C_i G_i^{-1}  (C_i = I gives block Jacobi exactly).
//
//  * k_features   node features from the assembled FP64 BSR matrix (normalised diagonal
//                 block, penalty flag, normalised coupling strengths of G^{-1} K G^{-T},
//                 normalised coordinates, local stiffness contrast) and G_i^{-1}.
//  * k_mlp_fwd    fused forward pass on the 5th-generation tensor cores: one CTA of 128
//                 threads per 128-node tile; weights and activations live in shared memory
//                 in the no-swizzle K-major core-matrix layout, one elected thread issues
//                 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128) into TMEM, tcgen05.commit
//                 arrives on an mbarrier, and each warp reads its 32 TMEM lanes back with
//                 tcgen05.ld for the bias + SiLU epilogue, which writes the next layer's
//                 BF16 operand to shared memory.  Every mbarrier wait is bounded (~1 s of
//                 clock) and sets an error flag on timeout; TMEM is always freed.
//  * k_loss       per-node loss sum_r |C_i yhat_r - zhat_r|^2 over probe pairs (zhat ~ N(0,I),
//                 yhat = G^{-1} K G^{-T} zhat) and its gradient w.r.t. the 6 outputs.
//  * k_mlp_bwd_tc backward pass on the tensor cores (the training default): dz1 = dz2 W2 and
//                 the weight / bias gradients as tcgen05 products with BF16 operands and FP32
//                 accumulation in TMEM (see the kernel's comment); one partial per CTA.
//  * k_mlp_bwd    backward pass on CUDA cores in FP32 (no BF16 rounding of the gradients), kept
//                 as the full-precision reference: per 64-node tile, register-tiled weight
//                 gradients, one partial per CTA.  k_sum_partials reduces the partials of
//                 either kernel in CTA order (deterministic).
//  * k_adam       Adam on FP32 master weights + BF16 copies for the forward kernel.
//  * k_learned_blocks  P_i = G_i^{-T} C_i G_i^{-1} in FP64 for the PCG.
#include <cuda_bf16.h>

#include "spmv.cuh"

namespace fem {
namespace {

constexpr int kIn = 16, kHid = 64, kOut = 16, kOutUsed = 6;
constexpr int kTile = 128;
constexpr int kNParams = kHid * kIn + kHid + kHid * kHid + kHid + kOut * kHid + kOut;  // 6288
// offsets of the flat FP32 parameter vector
constexpr int oW1 = 0, ob1 = oW1 + kHid * kIn, oW2 = ob1 + kHid, ob2 = oW2 + kHid * kHid, oW3 = ob2 + kHid,
              ob3 = oW3 + kOut * kHid;

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ---- tcgen05 / mbarrier helpers -------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices of 8 rows x 16 bytes;
// lbo = byte distance between core matrices adjacent in K, sbo = between 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= uint64_t((saddr & 0x3FFFFu) >> 4);
    d |= uint64_t((lbo & 0x3FFFFu) >> 4) << 16;
    d |= uint64_t((sbo & 0x3FFFFu) >> 4) << 32;
    d |= uint64_t(1) << 46;  // descriptor version for sm_100-family tensor cores
    return d;                // base offset 0, relative LBO, layout type 0 = no swizzle
}

// Instruction descriptor, kind::f16: D = F32, A = B = BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* mbar, uint32_t parity) {
    const long long deadline = clock64() + 2000000000LL;  // about one second at 2 GHz
    uint32_t ok = 0;
    while (!ok) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (!ok && clock64() > deadline) return false;
    }
    return true;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) of a K-major bf16 tile with K columns (core-matrix layout).
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, int K) {
    return uint32_t((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

struct MlpParams {
    const uint16_t* W1;
    const float* b1;
    const uint16_t* W2;
    const float* b2;
    const uint16_t* W3;
    const float* b3;
    const uint16_t* X;  // [n][16] bf16
    int64_t n;
    float* out;         // [n][16]
    float* z1;          // [n][64] pre-activations (optional)
    float* z2;          // [n][64] (optional)
    int* err;           // device flag, set on a bounded-wait timeout
};

// shared memory plan (bytes); W3 first so that every descriptor-addressed byte stays inside
struct MlpSmem {
    alignas(1024) unsigned char W3s[kOut * kHid * 2];    // 2 KB   B operand, layer 3 (N=16, K=64)
    alignas(1024) unsigned char W1s[kHid * kIn * 2];     // 2 KB   B operand, layer 1 (N=64, K=16)
    alignas(1024) unsigned char W2s[kHid * kHid * 2];    // 8 KB   B operand, layer 2 (N=64, K=64)
    alignas(1024) unsigned char Xs[kTile * kIn * 2];     // 4 KB   A operand, layer 1
    alignas(1024) unsigned char H1s[kTile * kHid * 2];   // 16 KB  A operand, layer 2
    alignas(1024) unsigned char H2s[kTile * kHid * 2];   // 16 KB  A operand, layer 3
    float b1[kHid], b2[kHid], b3[kOut];
    alignas(8) uint64_t mbar;
    uint32_t tmem_base;
};

__device__ __forceinline__ void store_row_bf16(unsigned char* tile, int row, int k0, int K, const float (&v)[16]) {
    // 16 consecutive k values = two 16-byte core rows
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        __nv_bfloat162 p[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) p[j] = __floats2bfloat162_rn(v[8 * h + 2 * j], v[8 * h + 2 * j + 1]);
        *reinterpret_cast<uint4*>(tile + core_off(row, k0 + 8 * h, K)) = *reinterpret_cast<uint4*>(p);
    }
}

__global__ void __launch_bounds__(kTile, 1) k_mlp_fwd(const MlpParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;

    // stage weights (generic proxy) in the core-matrix layout
    for (int i = tid; i < kHid * kIn; i += kTile)
        *reinterpret_cast<uint16_t*>(s.W1s + core_off(i / kIn, i % kIn, kIn)) = p.W1[i];
    for (int i = tid; i < kHid * kHid; i += kTile)
        *reinterpret_cast<uint16_t*>(s.W2s + core_off(i / kHid, i % kHid, kHid)) = p.W2[i];
    for (int i = tid; i < kOut * kHid; i += kTile)
        *reinterpret_cast<uint16_t*>(s.W3s + core_off(i / kHid, i % kHid, kHid)) = p.W3[i];
    for (int i = tid; i < kHid; i += kTile) {
        s.b1[i] = p.b1[i];
        s.b2[i] = p.b2[i];
    }
    for (int i = tid; i < kOut; i += kTile) s.b3[i] = p.b3[i];
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem_base)),
                     "r"(128u));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&s.mbar)), "r"(1u));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s.tmem_base;
    const uint32_t lane_base = uint32_t(32 * warp) << 16;
    const uint32_t id64 = idesc_bf16(kTile, kHid), id16 = idesc_bf16(kTile, kOut);
    const uint32_t aX = smem_u32(s.Xs), aH1 = smem_u32(s.H1s), aH2 = smem_u32(s.H2s);
    const uint32_t aW1 = smem_u32(s.W1s), aW2 = smem_u32(s.W2s), aW3 = smem_u32(s.W3s);
    uint32_t phase = 0;
    bool ok = true;

    for (int64_t tile = blockIdx.x; tile * kTile < p.n && ok; tile += gridDim.x) {
        const int64_t node = tile * kTile + tid;
        const bool valid = node < p.n;
        {
            uint4 a = make_uint4(0, 0, 0, 0), b = make_uint4(0, 0, 0, 0);
            if (valid) {
                const uint4* src = reinterpret_cast<const uint4*>(p.X + node * kIn);
                a = src[0];
                b = src[1];
            }
            *reinterpret_cast<uint4*>(s.Xs + core_off(tid, 0, kIn)) = a;
            *reinterpret_cast<uint4*>(s.Xs + core_off(tid, 8, kIn)) = b;
        }
        fence_proxy_async();
        __syncthreads();
        // ---- layer 1: D[0:64) = X W1^T -------------------------------------------------
        if (tid == 0) {
            fence_after();
            mma_bf16(tmem, sdesc(aX, 128, 256), sdesc(aW1, 128, 256), id64, 0u);
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(&s.mbar, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_base + uint32_t(c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float z = v[j] + s.b1[c0 + j];
                if (p.z1 && valid) p.z1[node * kHid + c0 + j] = z;
                v[j] = silu(z);
            }
            store_row_bf16(s.H1s, tid, c0, kHid, v);
        }
        fence_before();
        fence_proxy_async();
        __syncthreads();
        // ---- layer 2: D[64:128) = H1 W2^T (four K=16 slices) -----------------------------
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem + 64, sdesc(aH1 + 256 * ks, 128, 1024), sdesc(aW2 + 256 * ks, 128, 1024), id64,
                         ks > 0 ? 1u : 0u);
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(&s.mbar, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_base + uint32_t(64 + c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float z = v[j] + s.b2[c0 + j];
                if (p.z2 && valid) p.z2[node * kHid + c0 + j] = z;
                v[j] = silu(z);
            }
            store_row_bf16(s.H2s, tid, c0, kHid, v);
        }
        fence_before();
        fence_proxy_async();
        __syncthreads();
        // ---- layer 3: D[0:16) = H2 W3^T ---------------------------------------------------
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem, sdesc(aH2 + 256 * ks, 128, 1024), sdesc(aW3 + 256 * ks, 128, 1024), id16,
                         ks > 0 ? 1u : 0u);
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(&s.mbar, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        {
            float v[16];
            tmem_ld16(tmem + lane_base, v);
            if (valid) {
                float4* o = reinterpret_cast<float4*>(p.out + node * kOut);
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    o[j] = make_float4(v[4 * j] + s.b3[4 * j], v[4 * j + 1] + s.b3[4 * j + 1],
                                       v[4 * j + 2] + s.b3[4 * j + 2], v[4 * j + 3] + s.b3[4 * j + 3]);
            }
        }
        fence_before();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicExch(p.err, 1);
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u));
}

// ---- features ---------------------------------------------------------------------------------
// G^{-1} for the Cholesky factor G of the SPD 3x3 block a (row-major); returns false if not SPD.
__device__ bool chol_inv3(const double* a, double (&gi)[9]) {
    const double g00 = a[0];
    if (!(g00 > 0)) return false;
    const double l00 = sqrt(g00);
    const double l10 = a[3] / l00, l20 = a[6] / l00;
    const double d11 = a[4] - l10 * l10;
    if (!(d11 > 0)) return false;
    const double l11 = sqrt(d11);
    const double l21 = (a[7] - l20 * l10) / l11;
    const double d22 = a[8] - l20 * l20 - l21 * l21;
    if (!(d22 > 0)) return false;
    const double l22 = sqrt(d22);
    // inverse of lower-triangular L
    const double i00 = 1.0 / l00, i11 = 1.0 / l11, i22 = 1.0 / l22;
    const double i10 = -l10 * i00 * i11;
    const double i21 = -l21 * i11 * i22;
    const double i20 = -(l20 * i00 + l21 * i10) * i22;
    gi[0] = i00; gi[1] = 0; gi[2] = 0;
    gi[3] = i10; gi[4] = i11; gi[5] = 0;
    gi[6] = i20; gi[7] = i21; gi[8] = i22;
    return true;
}

__device__ __forceinline__ int64_t diag_slot(const int32_t* indptr, const int32_t* indices, int64_t i) {
    for (int64_t k = indptr[i]; k < indptr[i + 1]; ++k)
        if (indices[k] == int(i)) return k;
    return -1;
}

__global__ void k_chol_inv(int64_t n, const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices,
                           const double* __restrict__ K, double* ginv, int* bad) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        double gi[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        const int64_t s = diag_slot(indptr, indices, i);
        if (s < 0 || !chol_inv3(K + 9 * s, gi)) atomicAdd(bad, 1);
#pragma unroll
        for (int k = 0; k < 9; ++k) ginv[9 * i + k] = gi[k];
    }
}

// Frobenius norm^2 of Gi Kb Gj^T (3x3 each; Gi, Gj lower triangular)
__device__ double scaled_block_norm2(const double* gi, const double* kb, const double* gj) {
    double t[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) t[3 * r + c] = gi[3 * r] * kb[c] + gi[3 * r + 1] * kb[3 + c] + gi[3 * r + 2] * kb[6 + c];
    double s = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double v = t[3 * r] * gj[3 * c] + t[3 * r + 1] * gj[3 * c + 1] + t[3 * r + 2] * gj[3 * c + 2];
            s += v * v;
        }
    return s;
}

struct FeatParams {
    int64_t n;
    const int32_t* indptr;
    const int32_t* indices;
    const double* K;
    const double* ginv;
    const double* xyz;
    const uint8_t* fixed;
    double lo[3], inv_ext[3];
    uint16_t* X;  // [n][16] bf16
    float* Xf;    // optional [n][16] FP32 copy
};

__global__ void k_features(const FeatParams p) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < p.n; i += int64_t(gridDim.x) * blockDim.x) {
        float f[kIn];
        const int64_t rs = p.indptr[i], re = p.indptr[i + 1];
        const int64_t sd = diag_slot(p.indptr, p.indices, i);
        const double* D = sd >= 0 ? p.K + 9 * sd : nullptr;
        const double tr = D ? D[0] + D[4] + D[8] : 1.0;
        const double sc = tr > 0 ? 3.0 / tr : 1.0;
        f[0] = D ? float(D[0] * sc) : 1.f;
        f[1] = D ? float(D[4] * sc) : 1.f;
        f[2] = D ? float(D[8] * sc) : 1.f;
        f[3] = D ? float(D[1] * sc) : 0.f;
        f[4] = D ? float(D[2] * sc) : 0.f;
        f[5] = D ? float(D[5] * sc) : 0.f;
        f[6] = (p.fixed && p.fixed[i]) ? 1.f : 0.f;
        double ssum = 0, smax = 0, s2 = 0, trn = 0;
        const double* gi = p.ginv + 9 * i;
        for (int64_t k = rs; k < re; ++k) {
            const int64_t j = p.indices[k];
            const double* Dj = nullptr;
            if (j != i) {
                const double q2 = scaled_block_norm2(gi, p.K + 9 * k, p.ginv + 9 * j);
                const double q = sqrt(q2);
                ssum += q;
                s2 += q2;
                smax = fmax(smax, q);
                const int64_t sj = diag_slot(p.indptr, p.indices, j);
                Dj = sj >= 0 ? p.K + 9 * sj : nullptr;
                if (Dj) trn += Dj[0] + Dj[4] + Dj[8];
            }
        }
        const int nn = int(re - rs) - 1;
        f[7] = float(ssum);
        f[8] = float(smax);
        f[9] = float(s2);
        f[10] = float(nn) / 26.f;
#pragma unroll
        for (int d = 0; d < 3; ++d) f[11 + d] = float((p.xyz[3 * i + d] - p.lo[d]) * p.inv_ext[d]);
        f[14] = (nn > 0 && trn > 0 && tr > 0) ? float(log(tr * nn / trn)) : 0.f;
        f[15] = 1.f;
#pragma unroll
        for (int k = 0; k < kIn; ++k) {
            p.X[i * kIn + k] = __bfloat16_as_ushort(__float2bfloat16_rn(f[k]));
            if (p.Xf) p.Xf[i * kIn + k] = f[k];
        }
    }
}

// ---- probes -------------------------------------------------------------------------------------
// w = G^{-T} z (blockwise, per RHS);  layout [n][3][R]
__global__ void k_apply_ginv_t(int64_t n, int R, const double* __restrict__ ginv, const double* __restrict__ z,
                               double* w) {
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n * R; t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = t / R;
        const int k = int(t % R);
        const double* g = ginv + 9 * i;
        const double* zi = z + 3 * i * R + k;
        const double z0 = zi[0], z1 = zi[R], z2 = zi[2 * R];
        double* wi = w + 3 * i * R + k;
        wi[0] = g[0] * z0 + g[3] * z1 + g[6] * z2;
        wi[R] = g[4] * z1 + g[7] * z2;
        wi[2 * R] = g[8] * z2;
    }
}

// yhat = G^{-1} y (blockwise), FP32 output
__global__ void k_apply_ginv(int64_t n, int R, const double* __restrict__ ginv, const double* __restrict__ y,
                             float* yh) {
    for (int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n * R; t += int64_t(gridDim.x) * blockDim.x) {
        const int64_t i = t / R;
        const int k = int(t % R);
        const double* g = ginv + 9 * i;
        const double* yi = y + 3 * i * R + k;
        const double y0 = yi[0], y1 = yi[R], y2 = yi[2 * R];
        float* o = yh + 3 * i * R + k;
        o[0] = float(g[0] * y0);
        o[R] = float(g[3] * y0 + g[4] * y1);
        o[2 * R] = float(g[6] * y0 + g[7] * y1 + g[8] * y2);
    }
}

// ---- loss -----------------------------------------------------------------------------------------
__device__ __forceinline__ void lower_from_out(const float* o, float (&L)[9]) {
    L[0] = __expf(o[0]); L[1] = 0.f; L[2] = 0.f;
    L[3] = o[3]; L[4] = __expf(o[1]); L[5] = 0.f;
    L[6] = o[4]; L[7] = o[5]; L[8] = __expf(o[2]);
}

__global__ void __launch_bounds__(256) k_loss(int64_t n, int R, const float* __restrict__ out,
                                              const float* __restrict__ yh, const float* __restrict__ zh,
                                              float* dout, double* part, double scale) {
    double acc = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const float* o = out + i * kOut;
        float L[9];
        lower_from_out(o, L);
        float C[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) C[3 * r + c] = L[3 * r] * L[3 * c] + L[3 * r + 1] * L[3 * c + 1] + L[3 * r + 2] * L[3 * c + 2];
        float G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // dloss/dC
        for (int k = 0; k < R; ++k) {
            const float y0 = yh[3 * i * R + k], y1 = yh[3 * i * R + R + k], y2 = yh[3 * i * R + 2 * R + k];
            const float z0 = zh[3 * i * R + k], z1 = zh[3 * i * R + R + k], z2 = zh[3 * i * R + 2 * R + k];
            const float e0 = C[0] * y0 + C[1] * y1 + C[2] * y2 - z0;
            const float e1 = C[3] * y0 + C[4] * y1 + C[5] * y2 - z1;
            const float e2 = C[6] * y0 + C[7] * y1 + C[8] * y2 - z2;
            acc += double(e0) * e0 + double(e1) * e1 + double(e2) * e2;
            const float e[3] = {e0, e1, e2}, y[3] = {y0, y1, y2};
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) G[3 * r + c] += 2.f * e[r] * y[c];
        }
        // dC -> dL = (G + G^T) L ; outputs: diagonal through exp
        float S[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) S[3 * r + c] = G[3 * r + c] + G[3 * c + r];
        float dL[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) dL[3 * r + c] = S[3 * r] * L[c] + S[3 * r + 1] * L[3 + c] + S[3 * r + 2] * L[6 + c];
        const float sc = float(scale);
        float* d = dout + i * kOut;
        d[0] = sc * dL[0] * L[0];
        d[1] = sc * dL[4] * L[4];
        d[2] = sc * dL[8] * L[8];
        d[3] = sc * dL[3];
        d[4] = sc * dL[6];
        d[5] = sc * dL[7];
#pragma unroll
        for (int k = 6; k < kOut; ++k) d[k] = 0.f;
    }
    // deterministic block partial
    __shared__ double sm[8];
    for (int off = 16; off >= 1; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) t += sm[w];
        part[blockIdx.x] = t;
    }
}

// ---- backward (CUDA cores) -------------------------------------------------------------------------
constexpr int kBT = 64;  // nodes per backward tile

struct BwdParams {
    const float* W;      // FP32 master parameters (flat)
    const uint16_t* X;   // [n][16]
    const float* z1;     // [n][64]
    const float* z2;     // [n][64]
    const float* dout;   // [n][16]
    int64_t n;
    float* part;         // [gridDim][kNParams]
};

struct BwdSmem {
    float W2[kHid][kHid + 1];
    float W3[kOutUsed][kHid];
    float x[kBT][kIn];
    float h1[kBT][kHid + 1];
    float h2[kBT][kHid + 1];
    float dz1[kBT][kHid + 1];
    float dz2[kBT][kHid + 1];
    float dz3[kBT][kOutUsed];
};

__global__ void __launch_bounds__(256) k_mlp_bwd(const BwdParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    BwdSmem& s = *reinterpret_cast<BwdSmem*>(smem_raw);
    const int tid = threadIdx.x;
    // weights as the forward pass used them (BF16-rounded)
    for (int i = tid; i < kHid * kHid; i += 256) s.W2[i / kHid][i % kHid] = bf16r(p.W[oW2 + i]);
    for (int i = tid; i < kOutUsed * kHid; i += 256) s.W3[i / kHid][i % kHid] = bf16r(p.W[oW3 + i]);
    // gradient accumulators: thread owns W2 entries (o = 4*(tid/16)+a, k = 4*(tid%16)+b)
    float gW2[4][4] = {}, gW1[4] = {}, gW3[2] = {}, gb = 0.f;
    const int o2 = 4 * (tid / 16), k2 = 4 * (tid % 16);
    const int o1 = tid / 4, k1 = 4 * (tid % 4);           // W1: 64 x 16
    const int w3i = tid * 2;                               // W3 used rows: 6 x 64 = 384 = 256*1.5
    __syncthreads();
    for (int64_t base = int64_t(blockIdx.x) * kBT; base < p.n; base += int64_t(gridDim.x) * kBT) {
        // stage activations of the tile: 4 threads per node
        {
            const int ln = tid / 4, q = tid % 4;
            const int64_t node = base + ln;
            const bool valid = node < p.n;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int c = q * 16 + j;
                const float a1 = valid ? p.z1[node * kHid + c] : 0.f;
                const float a2 = valid ? p.z2[node * kHid + c] : 0.f;
                s.h1[ln][c] = valid ? bf16r(silu(a1)) : 0.f;
                s.h2[ln][c] = valid ? bf16r(silu(a2)) : 0.f;
                s.dz1[ln][c] = valid ? silu_grad(a1) : 0.f;  // holds s1' until dz1 is formed
                s.dz2[ln][c] = valid ? silu_grad(a2) : 0.f;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = q * 4 + j;
                s.x[ln][c] = valid ? __bfloat162float(__ushort_as_bfloat16(p.X[node * kIn + c])) : 0.f;
            }
            if (q == 0) {
#pragma unroll
                for (int j = 0; j < kOutUsed; ++j) s.dz3[ln][j] = valid ? p.dout[node * kOut + j] : 0.f;
            }
        }
        __syncthreads();
        // dz2 = (W3^T dz3) * s2'
        {
            const int ln = tid / 4, q = tid % 4;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int c = q * 16 + j;
                float d = 0.f;
#pragma unroll
                for (int o = 0; o < kOutUsed; ++o) d += s.W3[o][c] * s.dz3[ln][o];
                s.dz2[ln][c] *= d;
            }
        }
        __syncthreads();
        // dz1 = (W2^T dz2) * s1'
        {
            const int ln = tid / 4, q = tid % 4;
            float d[16] = {};
            for (int o = 0; o < kHid; ++o) {
                const float g = s.dz2[ln][o];
#pragma unroll
                for (int j = 0; j < 16; ++j) d[j] += s.W2[o][q * 16 + j] * g;
            }
#pragma unroll
            for (int j = 0; j < 16; ++j) s.dz1[ln][q * 16 + j] *= d[j];
        }
        __syncthreads();
        // weight gradients over the tile's nodes
        for (int ln = 0; ln < kBT; ++ln) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = s.dz2[ln][o2 + i], b[i] = s.h1[ln][k2 + i];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) gW2[i][j] += a[i] * b[j];
            const float g1 = s.dz1[ln][o1];
#pragma unroll
            for (int j = 0; j < 4; ++j) gW1[j] += g1 * s.x[ln][k1 + j];
            if (w3i < kOutUsed * kHid) {
                gW3[0] += s.dz3[ln][w3i / kHid] * s.h2[ln][w3i % kHid];
                gW3[1] += s.dz3[ln][(w3i + 1) / kHid] * s.h2[ln][(w3i + 1) % kHid];
            }
            if (tid < kHid) gb += s.dz1[ln][tid];
            else if (tid < 2 * kHid) gb += s.dz2[ln][tid - kHid];
            else if (tid < 2 * kHid + kOutUsed) gb += s.dz3[ln][tid - 2 * kHid];
        }
        __syncthreads();
    }
    float* out = p.part + int64_t(blockIdx.x) * kNParams;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) out[oW2 + (o2 + i) * kHid + k2 + j] = gW2[i][j];
#pragma unroll
    for (int j = 0; j < 4; ++j) out[oW1 + o1 * kIn + k1 + j] = gW1[j];
    if (w3i < kOutUsed * kHid) {
        out[oW3 + w3i] = gW3[0];
        out[oW3 + w3i + 1] = gW3[1];
    }
    for (int i = kOutUsed * kHid + tid; i < kOut * kHid; i += 256) out[oW3 + i] = 0.f;
    if (tid < kHid) out[ob1 + tid] = gb;
    else if (tid < 2 * kHid) out[ob2 + tid - kHid] = gb;
    else if (tid < 2 * kHid + kOutUsed) out[ob3 + tid - 2 * kHid] = gb;
    if (tid < kOut - kOutUsed) out[ob3 + kOutUsed + tid] = 0.f;
}

// ---- backward on the tensor cores -------------------------------------------------------------
//
// k_mlp_bwd_tc: one persistent CTA of 128 threads per SM, 128 nodes per tile (thread = node).
//  1. CUDA cores: h1 = bf16(silu(z1)), h2 = bf16(silu(z2)), s' = silu'(z), dz3 = dout[:6],
//     dz2 = (dz3 W3[:6]) * s2' (K = 6 is too short for an MMA).
//  2. tcgen05 (M = 128 nodes, N = 64, K = 64): D1 = bf16(dz2) W2 in TMEM columns [0, 64);
//     the epilogue forms dz1 = D1 * s1'.
//  3. tcgen05 gradient products, accumulated in TMEM across all tiles of the CTA:
//       D_g  = [bf16(dz2)^T ; bf16(dz1)^T] (128 x K=nodes) . [h1 | X | valid]  (N = 96)
//            -> rows 0-63: gW2 (cols 0-63) and gb2 (col 80); rows 64-127: gW1 (cols 64-79)
//               and gb1 (col 80)                                      TMEM columns [64, 160)
//       D_3  = [h2^T ; valid ; 0] (128 x K=nodes) . bf16(dz3)  (N = 16)
//            -> rows 0-63: gW3^T (cols 0-5); row 64: gb3                TMEM columns [160, 176)
//     The node dimension is K; each operand is written transposed into the no-swizzle
//     K-major core-matrix layout by the thread that owns the node.
//  4. After the last tile the accumulators are read back (tcgen05.ld) into this CTA's partial
//     gradient, reduced in CTA order by k_sum_partials (deterministic).
// BF16 operands, FP32 accumulation: the rounding points are dz3, dz2 and dz1 (as
// mlp_oracle.backward_bf16 states them).  Every mbarrier wait is bounded and TMEM is freed on
// every exit.
constexpr int kBwdCols = 256;  // TMEM columns allocated (176 used)

struct BwdTcParams {
    const float* W;      // FP32 master parameters (flat)
    const uint16_t* X;   // [n][16] bf16
    const float* z1;     // [n][64]
    const float* z2;     // [n][64]
    const float* dout;   // [n][16]
    int64_t n;
    float* part;         // [gridDim][kNParams]
    int* err;
};

struct BwdTcSmem {
    alignas(1024) unsigned char Ag[kTile * kTile * 2];     // 32 KB [dz2^T ; dz1^T], K = 128 nodes
    alignas(1024) unsigned char Bg[96 * kTile * 2];        // 24 KB [h1^T ; X^T ; valid ; 0]
    alignas(1024) unsigned char A3[kTile * kTile * 2];     // 32 KB [h2^T ; valid ; 0]
    alignas(1024) unsigned char B3[16 * kTile * 2];        // 4 KB  [dz3^T ; 0]
    alignas(1024) unsigned char Dz2[kTile * kHid * 2];     // 16 KB dz2, node-major (A of D1)
    alignas(1024) unsigned char W2T[kHid * kHid * 2];      // 8 KB  W2^T as B of D1 (row k, K = o)
    float W3[kOutUsed][kHid];
    alignas(8) uint64_t mbar;
    uint32_t tmem_base;
};

__device__ __forceinline__ void put_bf16(unsigned char* tile, int row, int k, int K, float v) {
    *reinterpret_cast<__nv_bfloat16*>(tile + core_off(row, k, K)) = __float2bfloat16_rn(v);
}

__global__ void __launch_bounds__(kTile, 1) k_mlp_bwd_tc(const BwdTcParams p) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    BwdTcSmem& s = *reinterpret_cast<BwdTcSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5;

    // W2^T in the core-matrix layout: element (row k, col o) = W2[o][k], BF16 as the forward used it
    for (int i = tid; i < kHid * kHid; i += kTile) {
        const int o = i / kHid, k = i % kHid;
        put_bf16(s.W2T, k, o, kHid, p.W[oW2 + i]);
    }
    for (int i = tid; i < kOutUsed * kHid; i += kTile) s.W3[i / kHid][i % kHid] = bf16r(p.W[oW3 + i]);
    // constant zero rows of the operands (rows 81-95 of Bg, 65-127 of A3, 6-15 of B3)
    for (int i = tid; i < 15 * kTile; i += kTile) put_bf16(s.Bg, 81 + i / kTile, i % kTile, kTile, 0.f);
    for (int i = tid; i < 63 * kTile; i += kTile) put_bf16(s.A3, 65 + i / kTile, i % kTile, kTile, 0.f);
    for (int i = tid; i < 10 * kTile; i += kTile) put_bf16(s.B3, 6 + i / kTile, i % kTile, kTile, 0.f);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&s.tmem_base)),
                     "r"(uint32_t(kBwdCols)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&s.mbar)), "r"(1u));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = s.tmem_base;
    const uint32_t lane_base = uint32_t(32 * warp) << 16;
    const uint32_t id_d1 = idesc_bf16(kTile, kHid), id_g = idesc_bf16(kTile, 96), id_3 = idesc_bf16(kTile, 16);
    const uint32_t aDz2 = smem_u32(s.Dz2), aW2T = smem_u32(s.W2T);
    const uint32_t aAg = smem_u32(s.Ag), aBg = smem_u32(s.Bg), aA3 = smem_u32(s.A3), aB3 = smem_u32(s.B3);
    uint32_t phase = 0;
    bool ok = true;
    bool first = true;

    for (int64_t tile = blockIdx.x; tile * kTile < p.n && ok; tile += gridDim.x) {
        const int64_t node = tile * kTile + tid;
        const bool valid = node < p.n;
        const int t = tid;  // column (K index) of this node in the transposed operands
        float s1g[kHid];
        {
            // dz3 and dz2 = (dz3 W3) s2'; h2^T, X^T, valid; dz3^T
            float d3[kOutUsed];
#pragma unroll
            for (int o = 0; o < kOutUsed; ++o) d3[o] = valid ? p.dout[node * kOut + o] : 0.f;
#pragma unroll
            for (int o = 0; o < kOutUsed; ++o) put_bf16(s.B3, o, t, kTile, d3[o]);
#pragma unroll
            for (int c0 = 0; c0 < kHid; c0 += 16) {
                float a1v[16], a2v[16], v[16];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    float4 u1 = make_float4(0.f, 0.f, 0.f, 0.f), u2 = u1;
                    if (valid) {
                        u1 = *reinterpret_cast<const float4*>(p.z1 + node * kHid + c0 + 4 * q);
                        u2 = *reinterpret_cast<const float4*>(p.z2 + node * kHid + c0 + 4 * q);
                    }
                    a1v[4 * q] = u1.x, a1v[4 * q + 1] = u1.y, a1v[4 * q + 2] = u1.z, a1v[4 * q + 3] = u1.w;
                    a2v[4 * q] = u2.x, a2v[4 * q + 1] = u2.y, a2v[4 * q + 2] = u2.z, a2v[4 * q + 3] = u2.w;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = c0 + j;
                    float d = 0.f;
#pragma unroll
                    for (int o = 0; o < kOutUsed; ++o) d = fmaf(s.W3[o][c], d3[o], d);
                    d = valid ? d * silu_grad(a2v[j]) : 0.f;
                    v[j] = d;
                    put_bf16(s.Ag, c, t, kTile, d);                            // dz2^T (rows 0-63)
                    put_bf16(s.A3, c, t, kTile, valid ? silu(a2v[j]) : 0.f);  // h2^T
                    put_bf16(s.Bg, c, t, kTile, valid ? silu(a1v[j]) : 0.f);  // h1^T
                    s1g[c] = valid ? silu_grad(a1v[j]) : 0.f;
                }
                store_row_bf16(s.Dz2, tid, c0, kHid, v);                       // dz2, node-major
            }
            uint4 xa = make_uint4(0, 0, 0, 0), xb = make_uint4(0, 0, 0, 0);
            if (valid) {
                const uint4* src = reinterpret_cast<const uint4*>(p.X + node * kIn);
                xa = src[0];
                xb = src[1];
            }
            const uint16_t* xs = reinterpret_cast<const uint16_t*>(&xa);
            const uint16_t* xt = reinterpret_cast<const uint16_t*>(&xb);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                *reinterpret_cast<uint16_t*>(s.Bg + core_off(64 + k, t, kTile)) = xs[k];
                *reinterpret_cast<uint16_t*>(s.Bg + core_off(72 + k, t, kTile)) = xt[k];
            }
            put_bf16(s.Bg, 80, t, kTile, valid ? 1.f : 0.f);
            put_bf16(s.A3, 64, t, kTile, valid ? 1.f : 0.f);
        }
        fence_proxy_async();
        __syncthreads();
        // ---- D1 = dz2 W2 (M = 128 nodes, N = 64, K = 64 in four K = 16 slices) ---------------
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int ks = 0; ks < kHid / 16; ++ks)
                mma_bf16(tmem, sdesc(aDz2 + 256 * ks, 128, 1024), sdesc(aW2T + 256 * ks, 128, 1024), id_d1,
                         ks > 0 ? 1u : 0u);
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(&s.mbar, phase));
        phase ^= 1;
        if (!ok) break;
        fence_after();
        // dz1 = D1 s1'  -> rows 64-127 of Ag (transposed)
#pragma unroll
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + lane_base + uint32_t(c0), v);
#pragma unroll
            for (int j = 0; j < 16; ++j) put_bf16(s.Ag, 64 + c0 + j, t, kTile, v[j] * s1g[c0 + j]);
        }
        fence_before();
        fence_proxy_async();
        __syncthreads();
        // ---- gradient products, accumulated over the tiles (K = 128 nodes, eight K = 16 slices)
        if (tid == 0) {
            fence_after();
#pragma unroll
            for (int ks = 0; ks < kTile / 16; ++ks) {
                const uint32_t acc = (first && ks == 0) ? 0u : 1u;
                mma_bf16(tmem + 64, sdesc(aAg + 256 * ks, 128, 2048), sdesc(aBg + 256 * ks, 128, 2048), id_g, acc);
                mma_bf16(tmem + 160, sdesc(aA3 + 256 * ks, 128, 2048), sdesc(aB3 + 256 * ks, 128, 2048), id_3, acc);
            }
            mma_commit(&s.mbar);
        }
        ok = __syncthreads_and(mbar_wait_bounded(&s.mbar, phase));
        phase ^= 1;
        first = false;
        if (!ok) break;
        fence_after();
    }

    // ---- this CTA's partial gradient --------------------------------------------------------------
    float* out = p.part + int64_t(blockIdx.x) * kNParams;
    if (ok) {
        const int r = tid;  // TMEM lane = row of the accumulators
        if (first) {
            // no tile: zero partial
            for (int i = tid; i < kNParams; i += kTile) out[i] = 0.f;
        } else {
#pragma unroll
            for (int c0 = 0; c0 < 96; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + lane_base + uint32_t(64 + c0), v);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = c0 + j;
                    if (r < 64) {
                        if (c < 64) out[oW2 + r * kHid + c] = v[j];
                        else if (c == 80) out[ob2 + r] = v[j];
                    } else {
                        if (c >= 64 && c < 80) out[oW1 + (r - 64) * kIn + (c - 64)] = v[j];
                        else if (c == 80) out[ob1 + (r - 64)] = v[j];
                    }
                }
            }
            {
                float v[16];
                tmem_ld16(tmem + lane_base + 160u, v);
                if (r < 64) {
#pragma unroll
                    for (int o = 0; o < kOutUsed; ++o) out[oW3 + o * kHid + r] = v[o];
                } else if (r == 64) {
#pragma unroll
                    for (int o = 0; o < kOutUsed; ++o) out[ob3 + o] = v[o];
                }
            }
            for (int i = kOutUsed * kHid + tid; i < kOut * kHid; i += kTile) out[oW3 + i] = 0.f;
            if (tid < kOut - kOutUsed) out[ob3 + kOutUsed + tid] = 0.f;
        }
    } else if (tid == 0) {
        atomicExch(p.err, 1);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(uint32_t(kBwdCols)));
}

__global__ void k_sum_partials(const float* __restrict__ part, int nblocks, int count, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += part[int64_t(b) * count + i];
    out[i] = s;
}

__global__ void k_adam(float* w, const float* __restrict__ g, float* m, float* v, int count, float lr, float b1,
                       float b2, float eps, float c1, float c2, uint16_t* W1b, uint16_t* W2b, uint16_t* W3b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float gi = g[i];
    if (!isfinite(gi)) gi = 0.f;
    const float mi = b1 * m[i] + (1 - b1) * gi, vi = b2 * v[i] + (1 - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    if (i >= oW3 && i < ob3 && (i - oW3) >= kOutUsed * kHid) wi = 0.f;  // unused output rows
    if (i >= ob3 + kOutUsed) wi = 0.f;
    w[i] = wi;
    const uint16_t b = __bfloat16_as_ushort(__float2bfloat16_rn(wi));
    if (i < ob1) W1b[i - oW1] = b;
    else if (i >= oW2 && i < ob2) W2b[i - oW2] = b;
    else if (i >= oW3 && i < ob3) W3b[i - oW3] = b;
}

// P_i = G_i^{-T} C_i G_i^{-1}, C = L L^T from the MLP outputs
__global__ void k_learned_blocks(int64_t n, const float* __restrict__ out, const double* __restrict__ ginv,
                                 double* P) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        float Lf[9];
        lower_from_out(out + i * kOut, Lf);
        double C[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                C[3 * r + c] = double(Lf[3 * r]) * Lf[3 * c] + double(Lf[3 * r + 1]) * Lf[3 * c + 1] +
                               double(Lf[3 * r + 2]) * Lf[3 * c + 2];
        const double* g = ginv + 9 * i;
        double T[9];  // C G^{-1}
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) T[3 * r + c] = C[3 * r] * g[c] + C[3 * r + 1] * g[3 + c] + C[3 * r + 2] * g[6 + c];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                P[9 * i + 3 * r + c] = g[r] * T[c] + g[3 + r] * T[3 + c] + g[6 + r] * T[6 + c];
    }
}

unsigned grid_for(int64_t n, int threads) {
    return unsigned(std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, int64_t(sm_count()) * 16)));
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" int fem_mlp_nparams(void) { return kNParams; }

extern "C" int fem_precond_cholesky(const fem_bsr* A, double* ginv, int* n_bad, void* stream) {
    FEM_REQUIRE(A && A->dtype == FEM_F64 && ginv && n_bad, "bad arguments");
    if (A->n_brow == 0) return FEM_OK;
    cudaStream_t st = as_stream(stream);
    FEM_CUDA(cudaMemsetAsync(n_bad, 0, sizeof(int), st));
    k_chol_inv<<<grid_for(A->n_brow, 256), 256, 0, st>>>(A->n_brow, A->indptr, A->indices,
                                                         static_cast<const double*>(A->vals), ginv, n_bad);
    FEM_LAUNCH_CHECK("k_chol_inv");
    return FEM_OK;
}

extern "C" int fem_precond_features(const fem_bsr* A, const double* ginv, const double* xyz, const uint8_t* fixed,
                                    const double* lo, const double* hi, uint16_t* X, float* Xf, void* stream) {
    FEM_REQUIRE(A && A->dtype == FEM_F64 && ginv && xyz && lo && hi && X, "bad arguments");
    if (A->n_brow == 0) return FEM_OK;
    FeatParams p;
    p.n = A->n_brow;
    p.indptr = A->indptr;
    p.indices = A->indices;
    p.K = static_cast<const double*>(A->vals);
    p.ginv = ginv;
    p.xyz = xyz;
    p.fixed = fixed;
    for (int d = 0; d < 3; ++d) {
        p.lo[d] = lo[d];
        p.inv_ext[d] = hi[d] > lo[d] ? 1.0 / (hi[d] - lo[d]) : 0.0;
    }
    p.X = X;
    p.Xf = Xf;
    k_features<<<grid_for(A->n_brow, 128), 128, 0, as_stream(stream)>>>(p);
    FEM_LAUNCH_CHECK("k_features");
    return FEM_OK;
}

extern "C" int fem_probe_products(const fem_bsr* A, int nrhs, const double* ginv, const double* z, double* w,
                                  double* y, float* yhat, void* stream) {
    FEM_REQUIRE(A && A->dtype == FEM_F64 && ginv && z && w && y && yhat, "bad arguments");
    FEM_REQUIRE(nrhs == 1 || nrhs == 2 || nrhs == 4 || nrhs == 8 || nrhs == 16 || nrhs == 32, "bad nrhs");
    if (A->n_brow == 0) return FEM_OK;
    cudaStream_t st = as_stream(stream);
    const unsigned g = grid_for(A->n_brow * nrhs, 256);
    k_apply_ginv_t<<<g, 256, 0, st>>>(A->n_brow, nrhs, ginv, z, w);
    FEM_LAUNCH_CHECK("k_apply_ginv_t");
    int rc = fem_bsr_spmv(A, nrhs, w, y, 0, stream);
    if (rc) return rc;
    k_apply_ginv<<<g, 256, 0, st>>>(A->n_brow, nrhs, ginv, y, yhat);
    FEM_LAUNCH_CHECK("k_apply_ginv");
    return FEM_OK;
}

extern "C" int fem_mlp_forward(const fem_mlp* net, const uint16_t* X, int64_t n, float* out, float* z1, float* z2,
                               int* err, void* stream) {
    FEM_REQUIRE(net && net->W1 && net->b1 && net->W2 && net->b2 && net->W3 && net->b3, "net has NULL members");
    FEM_REQUIRE(n >= 0 && err && (n == 0 || (X && out)), "bad arguments");
    FEM_REQUIRE(n == 0 || aligned16(X), "X must be 16-byte aligned");
    if (n == 0) return FEM_OK;
    MlpParams p{net->W1, net->b1, net->W2, net->b2, net->W3, net->b3, X, n, out, z1, z2, err};
    const size_t smem = sizeof(MlpSmem) + 1024;
    FEM_CUDA(cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t tiles = (n + kTile - 1) / kTile;
    const unsigned grid = unsigned(std::max<int64_t>(1, std::min<int64_t>(tiles, int64_t(sm_count()) * 3)));
    k_mlp_fwd<<<grid, kTile, smem, as_stream(stream)>>>(p);
    FEM_LAUNCH_CHECK("k_mlp_fwd");
    return FEM_OK;
}

extern "C" int fem_mlp_loss_grad(const float* out, const float* yhat, const float* zhat, int nprobe, int64_t n,
                                 float* dout, double* loss_partials, int* n_partials, void* stream) {
    FEM_REQUIRE(out && yhat && zhat && dout && loss_partials && n_partials && nprobe >= 1 && n > 0, "bad arguments");
    const unsigned grid = std::min<unsigned>(grid_for(n, 256), 1024u);
    k_loss<<<grid, 256, 0, as_stream(stream)>>>(n, nprobe, out, yhat, zhat, dout, loss_partials,
                                                1.0 / (double(n) * nprobe));
    FEM_LAUNCH_CHECK("k_loss");
    *n_partials = int(grid);
    return FEM_OK;
}

extern "C" size_t fem_mlp_backward_workspace_bytes(int64_t n) {
    const int64_t tiles = (n + kBT - 1) / kBT;
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>(tiles, 152 * 4));
    return size_t(g) * kNParams * sizeof(float) + 1024;
}

extern "C" int fem_mlp_backward(const float* params, const uint16_t* X, const float* z1, const float* z2,
                                const float* dout, int64_t n, float* grad, void* workspace, size_t workspace_bytes,
                                void* stream) {
    FEM_REQUIRE(params && X && z1 && z2 && dout && grad && workspace && n > 0, "bad arguments");
    const int64_t tiles = (n + kBT - 1) / kBT;
    const int g = int(std::max<int64_t>(1, std::min<int64_t>(tiles, 152 * 4)));
    if (workspace_bytes < size_t(g) * kNParams * sizeof(float)) {
        set_error("workspace too small");
        return FEM_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    BwdParams p{params, X, z1, z2, dout, n, static_cast<float*>(workspace)};
    const size_t smem = sizeof(BwdSmem);
    FEM_CUDA(cudaFuncSetAttribute(k_mlp_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    k_mlp_bwd<<<g, 256, smem, st>>>(p);
    FEM_LAUNCH_CHECK("k_mlp_bwd");
    k_sum_partials<<<(kNParams + 255) / 256, 256, 0, st>>>(static_cast<const float*>(workspace), g, kNParams, grad);
    FEM_LAUNCH_CHECK("k_sum_partials");
    return FEM_OK;
}

extern "C" size_t fem_mlp_backward_tc_workspace_bytes(int64_t n) {
    int dev = 0, sms = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (n + kTile - 1) / kTile;
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>(tiles, sms));
    return size_t(g) * kNParams * sizeof(float);
}

extern "C" int fem_mlp_backward_tc(const float* params, const uint16_t* X, const float* z1, const float* z2,
                                   const float* dout, int64_t n, float* grad, void* workspace, size_t workspace_bytes,
                                   int* err, void* stream) {
    FEM_REQUIRE(params && X && z1 && z2 && dout && grad && workspace && err && n > 0, "bad arguments");
    FEM_REQUIRE(aligned16(X) && aligned16(z1) && aligned16(z2), "X, z1 and z2 must be 16-byte aligned");
    int dev = 0, sms = 0;
    FEM_CUDA(cudaGetDevice(&dev));
    FEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t tiles = (n + kTile - 1) / kTile;
    const int g = int(std::max<int64_t>(1, std::min<int64_t>(tiles, sms)));
    if (workspace_bytes < size_t(g) * kNParams * sizeof(float)) {
        set_error("workspace too small: need %zu bytes", size_t(g) * kNParams * sizeof(float));
        return FEM_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    BwdTcParams p{params, X, z1, z2, dout, n, static_cast<float*>(workspace), err};
    const size_t smem = sizeof(BwdTcSmem) + 1024;
    FEM_CUDA(cudaFuncSetAttribute(k_mlp_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    k_mlp_bwd_tc<<<g, kTile, smem, st>>>(p);
    FEM_LAUNCH_CHECK("k_mlp_bwd_tc");
    k_sum_partials<<<(kNParams + 255) / 256, 256, 0, st>>>(static_cast<const float*>(workspace), g, kNParams, grad);
    FEM_LAUNCH_CHECK("k_sum_partials");
    return FEM_OK;
}

extern "C" int fem_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                            float beta2, float eps, uint16_t* W1, uint16_t* W2, uint16_t* W3, void* stream) {
    FEM_REQUIRE(params && grad && m && v && W1 && W2 && W3 && step >= 1, "bad arguments");
    const float c1 = 1.f - powf(beta1, float(step)), c2 = 1.f - powf(beta2, float(step));
    k_adam<<<(kNParams + 255) / 256, 256, 0, as_stream(stream)>>>(params, grad, m, v, kNParams, lr, beta1, beta2, eps,
                                                                 c1, c2, W1, W2, W3);
    FEM_LAUNCH_CHECK("k_adam");
    return FEM_OK;
}

extern "C" int fem_learned_blocks(int64_t n, const float* out, const double* ginv, double* P, void* stream) {
    FEM_REQUIRE(n >= 0 && (n == 0 || (out && ginv && P)), "bad arguments");
    if (n == 0) return FEM_OK;
    k_learned_blocks<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(n, out, ginv, P);
    FEM_LAUNCH_CHECK("k_learned_blocks");
    return FEM_OK;
}
