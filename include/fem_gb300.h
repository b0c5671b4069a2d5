/*
 * fem_gb300.h -- C ABI of the GB300 (sm_103a) hex8 finite-element hot path.
 *
 * Plain C types only: sizes are int64_t, index arrays int32_t, values double/float.
 * Unless stated otherwise a pointer argument is a DEVICE pointer on the current CUDA
 * device, and `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * Every entry point returns an int status (FEM_OK == 0, negative on error) and never
 * throws; fem_last_error() returns a thread-local message for the last failure.
 * No entry point keeps global mutable state: callers own every buffer (outputs and
 * workspaces are caller-allocated; *_workspace_bytes() tells how much to allocate).  The
 * one object that owns device memory is the multigrid hierarchy (fem_amg), which the
 * caller creates and destroys explicitly.
 *
 * Reference interfaces replaced (tianshao1992/FEM_taichi):
 *   fem_pattern_*          READ_physics.py:42-61       Read.pre_process (SmNode/ReNode/CoNode)
 *   fem_topology_*_gpu     READ_physics.py:42-61       the same, built on the device
 *   fem_incidence_build    READ_physics.py:51-60       Elem_Node incidence, CoElem
 *   fem_assemble           FEM_model_csr.py:150-242    InstallIndexK, InstallMatrixK, InstallMatrixM,
 *                          FEM_model_bsr.py:163-259    InstallIndexM, InstallVectorF, LoadF, ModifyK,
 *                                                      UnitMatrixK/M, UnitVectorF, installLocalB/N
 *   fem_csr_index          FEM_model_csr.py:163,167-173,191,195-201   RowK/ColK/RowM/ColM
 *   fem_assemble_tangent   FEM_model_bsr.py:134-145,178-191,476-592   Get_MatrixKN (large displacement)
 *   fem_stress             POST_process.py:172-209,72-99  get_NdSol, get_NdAve, UnitVectorS,
 *                                                      shapefunc_GS, Get_Stress (eigh, "VM")
 *   fem_bsr_spmv*          SOLVE_static.py:36          KL * U (residual product)
 *   fem_pcg_solve          SOLVE_static.py:31-33       pardisoSolver(KL, mtype=2).factor/solve
 *   fem_amg_*, fem_pcg_solve_amg  SOLVE_static.py:31-33  the same solve, multigrid-preconditioned
 *                                                      (setup on the host or on the device)
 *   fem_ts_gemm_*          SOLVE_eigen.py:65-84        Lanczos reorthogonalisation w -= Q (Q^T M w)
 *                                                      and the Ritz vectors X = Q V (numpy GEMMs)
 */
#ifndef FEM_GB300_H
#define FEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
#define FEM_OK 0
#define FEM_ERR_INVALID (-1)       /* bad argument: null pointer, size, index out of range */
#define FEM_ERR_CUDA (-2)          /* CUDA runtime error (see fem_last_error) */
#define FEM_ERR_PATTERN (-3)       /* an element node pair is absent from the block pattern */
#define FEM_ERR_NOT_CONVERGED (-4) /* solver stalled before reaching the tolerance */
#define FEM_ERR_MAXITER (-5)       /* solver hit its iteration cap */
#define FEM_ERR_NOT_SPD (-6)       /* non-positive curvature / preconditioner detected */
#define FEM_ERR_WORKSPACE (-7)     /* workspace too small */
#define FEM_ERR_BREAKDOWN (-8)     /* NaN/Inf encountered */

#define FEM_LAYOUT_BSR 0 /* K: [nnzb][3][3] block-major;  M: [nnzb] one scalar per block      */
#define FEM_LAYOUT_CSR 1 /* K: reference scalar CSR value order (row 3i+p: blocks m, cols q);
                            M: reference scalar CSR with 3 entries per block, [3*nnzb]        */

const char* fem_last_error(void);
int fem_abi_version(void);

/* ---- topology (HOST pointers) -------------------------------------------------- */
/* Block-row pattern of K: row i lists, ascending, every node sharing an element with node
 * i (itself included).  Same arrays as READ_physics.py:55-61 (SmNode = indptr,
 * ReNode = indices).  conn: [n_elem][8] node indices in [0, n_node).
 * fem_pattern_count fills indptr[n_node+1] and *nnzb; fem_pattern_fill fills indices. */
int fem_pattern_count(int64_t n_node, int64_t n_elem, const int32_t* conn, int32_t* indptr,
                      int64_t* nnzb);
int fem_pattern_fill(int64_t n_node, int64_t n_elem, const int32_t* conn, const int32_t* indptr,
                     int32_t* indices);
/* Node -> element incidence: for node i, ne_list[ne_ptr[i] .. ne_ptr[i+1]) holds e*8+a for
 * every (element e, local corner a) with conn[e][a] == i, ascending in (e, a).
 * co_elem[i] = number of distinct elements touching node i (READ_physics.py:60). */
int fem_incidence_build(int64_t n_node, int64_t n_elem, const int32_t* conn, int32_t* ne_ptr,
                        int32_t* ne_list, int32_t* co_elem);
/* Element-to-block map of the gather (the precomputed form of the reference's linear slot
 * search, FEM_model_bsr.py:171-175): ne_inv[e*8+a] = position k of (e, a) in ne_list, and
 * slot_map[8*k+b] = slot of node conn[e][b] in block row conn[e][a] (0..255).
 * FEM_ERR_PATTERN if a pair is absent from the pattern or a row has more than 256 blocks. */
int fem_gather_map(int64_t n_node, int64_t n_elem, const int32_t* conn, const int32_t* indptr,
                   const int32_t* indices, const int32_t* ne_ptr, const int32_t* ne_list, int32_t* ne_inv,
                   uint8_t* slot_map);

/* ---- topology on the device (DEVICE pointers) ----------------------------------- */
/* Device build of the same arrays as fem_incidence_build + fem_pattern_count/fill +
 * fem_gather_map (READ_physics.py:42-61, FEM_model_bsr.py:171-175), bit for bit.  Two calls
 * with the same workspace (fem_topology_workspace_bytes, left unchanged between them):
 *   fem_topology_count_gpu: ne_ptr [N+1], ne_list [8E], co_elem [N] (may be NULL),
 *     indptr [N+1]; returns nnzb in *nnzb (HOST; the call synchronises the stream);
 *   fem_topology_fill_gpu: indices [nnzb] and, if both are non-NULL, ne_inv [8E] and
 *     slot_map [8E][8].
 * Limits: at most 128 elements per node; otherwise FEM_ERR_INVALID (use the host build). */
size_t fem_topology_workspace_bytes(int64_t n_node, int64_t n_elem);
int fem_topology_count_gpu(int64_t n_node, int64_t n_elem, const int32_t* conn, int32_t* ne_ptr, int32_t* ne_list,
                           int32_t* co_elem, int32_t* indptr, int64_t* nnzb, void* workspace,
                           size_t workspace_bytes, void* stream);
int fem_topology_fill_gpu(int64_t n_node, int64_t n_elem, const int32_t* conn, const int32_t* ne_ptr,
                          const int32_t* ne_list, const int32_t* indptr, int32_t* indices, int32_t* ne_inv,
                          uint8_t* slot_map, void* workspace, size_t workspace_bytes, void* stream);

/* ---- device mesh descriptor ---------------------------------------------------- */
typedef struct fem_mesh {
    int64_t n_node, n_elem, nnzb;
    const double* xyz;      /* [n_node][3] */
    const int32_t* conn;    /* [n_elem][8], 16-byte aligned */
    const int32_t* indptr;  /* [n_node+1] */
    const int32_t* indices; /* [nnzb] */
    const int32_t* ne_ptr;  /* [n_node+1] */
    const int32_t* ne_list; /* [8*n_elem] */
    const int32_t* ne_inv;  /* [8*n_elem] (fem_gather_map), needed by FEM_ALGO_DD assembly */
    const uint8_t* slot_map; /* [8*n_elem][8] (fem_gather_map), needed by FEM_ALGO_DD assembly and by
                                the FP64 lane-per-corner gather (without it the FP64 gather runs one
                                lane per block slot, and fem_assemble_host cannot split it) */
} fem_mesh;

typedef struct fem_material {
    double DE, EX, PO;  /* density, Young's modulus, Poisson ratio (FEM_model_bsr.py:10) */
    double omega[3];    /* global angular velocity about an axis through the origin      */
} fem_material;

#define FEM_ALGO_DD 0   /* element integrals and gather sums in double-float on the FP32 pipes
                           (inputs split from FP64, outputs formed in FP64; ~48-bit significands,
                           not FP64 arithmetic) */
#define FEM_ALGO_FP64 1 /* the same two stages in native FP64 arithmetic, as the reference computes
                           (ti.f64); the Python drop-in's default                                 */

typedef struct fem_assembly_out {
    int k_layout;          /* FEM_LAYOUT_BSR or FEM_LAYOUT_CSR                            */
    int m_layout;          /* FEM_LAYOUT_BSR or FEM_LAYOUT_CSR                            */
    double* K;             /* 9*nnzb values, or NULL to skip K                           */
    double* M;             /* nnzb (BSR) or 3*nnzb (CSR) values, or NULL to skip M        */
    double* F;             /* [n_node][3], or NULL to skip F                             */
    const uint8_t* fixed;  /* [n_node] bit p => DOF p of the node is penalised (K diagonal
                              entry set to 1e20, FEM_model_bsr.py:248-259), or NULL       */
    const double* loads;   /* [n_node][3] nodal loads added to F after the element terms
                              (LoadF, FEM_model_bsr.py:220-226), or NULL                   */
    int algo;              /* FEM_ALGO_DD or FEM_ALGO_FP64                                */
} fem_assembly_out;

/* Assemble K, M and F for one mesh: element integrals (2x2x2 Gauss) into a workspace,
 * then a deterministic, atomic-free gather that sums every block's element contributions
 * in ascending element order.  FEM_ALGO_DD writes the contributions row-ordered (chunk k =
 * entry k of ne_list) and gathers them through mesh->slot_map. */
size_t fem_assemble_workspace_bytes(int64_t n_elem);
int fem_assemble(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                 void* workspace, size_t workspace_bytes, void* stream);
/* The two phases of fem_assemble, callable separately (same workspace): element records
 * (UnitMatrixK/M + UnitVectorF, FEM_model_bsr.py:262-300), then the gather into K/M/F
 * (InstallMatrixK/M, InstallVectorF scatter, LoadF, ModifyK; FEM_model_csr.py:150-242). */
int fem_assemble_elements(const fem_mesh* mesh, const fem_material* mat, int algo, void* workspace,
                          size_t workspace_bytes, void* stream);
int fem_assemble_gather(const fem_mesh* mesh, const fem_assembly_out* out, const void* workspace,
                        size_t workspace_bytes, void* stream);

/* Assembly delivered to host memory: replaces the reference getters' "run the kernels, then
 * to_numpy()" (Get_MatrixKL / Get_MatrixM / Get_VectorF, FEM_model_csr.py:118-146).  The
 * mesh is assembled in n_parts parts of consecutive block rows: element parts run on `stream`,
 * the gathers on an internal high-priority stream (gather q after element part q, beside
 * element part q + 1), and part q's rows are copied from the device outputs in `out` to
 * K_host / M_host / F_host (same layouts as out; NULL skips one) on an internal copy stream
 * while later parts still compute, so the copies overlap the kernels.  The plan comes from fem_pipeline_plan.  Host buffers may be
 * page-locked (copies asynchronous) or pageable (copies then finish before the call
 * returns).  `stream` is ordered after the last copy: synchronise it before reading the host
 * buffers.  Not capturable into a CUDA graph.  FEM_ALGO_FP64 without mesh->slot_map runs as
 * a single part. */
int fem_assemble_host(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                      const int64_t* row_split, const int64_t* elem_split, const int64_t* block_split,
                      int n_parts, double* K_host, double* M_host, double* F_host, void* workspace,
                      size_t workspace_bytes, void* stream);
/* fem_assemble_host for getters that return M in the reference's scalar CSR (out->m_layout =
 * FEM_LAYOUT_CSR): M leaves the device as one value per block into M_stage (HOST, nnzb
 * doubles, page-locked) instead of three, and the calling thread writes M_host in the CSR
 * order from it, part by part, while the later parts are still being copied; indptr_host is
 * the host copy of the block row pointers.  Returns when K_host, M_host and F_host are complete.
 * With M_stage or M_host NULL, or a BSR M, it is fem_assemble_host. */
int fem_assemble_host_staged(const fem_mesh* mesh, const fem_material* mat, const fem_assembly_out* out,
                             const int64_t* row_split, const int64_t* elem_split, const int64_t* block_split,
                             int n_parts, const int32_t* indptr_host, double* K_host, double* M_host,
                             double* F_host, double* M_stage, void* workspace, size_t workspace_bytes,
                             void* stream);
/* Plan of fem_assemble_host (host arrays, no reference counterpart): row_split[0..n_parts]
 * splits the block rows into parts of about nnzb / n_parts blocks; block_split[q] =
 * indptr[row_split[q]]; elem_split[q + 1] = 1 + the largest element incident to a row below
 * row_split[q + 1] (prefix maximum), so part q computes elements [elem_split[q],
 * elem_split[q+1]) and then gathers its rows.  indptr, ne_ptr, ne_list: host copies. */
int fem_pipeline_plan(int64_t n_node, int64_t n_elem, const int32_t* indptr, const int32_t* ne_ptr,
                      const int32_t* ne_list, int n_parts, int64_t* row_split, int64_t* elem_split,
                      int64_t* block_split);

/* Large-displacement tangent KT and secant KM at nodal displacements u ([n_node][3]):
 * Get_MatrixKN / InstallMatrixKN / UnitK (FEM_model_bsr.py:134-145,178-191,476-592), with the
 * penalty of ModifyMatrixK on both (:248-259).  FP64 element integrals, gathered like K
 * (atomic-free, fixed order).  KT, KM: 9*nnzb values each in k_layout (BSR or the reference
 * CSR order); fixed: per-node DOF bit mask as in fem_assembly_out, or NULL.  Needs
 * mesh->ne_inv and mesh->slot_map. */
size_t fem_tangent_workspace_bytes(int64_t n_elem);
int fem_assemble_tangent(const fem_mesh* mesh, const fem_material* mat, const double* u, int k_layout,
                         double* KT, double* KM, const uint8_t* fixed, void* workspace, size_t workspace_bytes,
                         void* stream);

/* Reference CSR index arrays (depend on the pattern only): rowK [3N+1], colK [9 nnzb],
 * rowM [3N+1], colM [3 nnzb]; any may be NULL. */
int fem_csr_index(const fem_mesh* mesh, int32_t* rowK, int32_t* colK, int32_t* rowM,
                  int32_t* colM, void* stream);

/* ---- stress recovery ------------------------------------------------------------- */
/* u: [n_node][3] displacement; co_elem: [n_node]; extrap: HOST [8][8] weights W[j][k]
 * (node j <- Gauss point k; POST_process.py:176-181); out: [n_node][10] =
 * [xx,yy,zz,xy,yz,xz, p1>=p2>=p3, "VM" as written at POST_process.py:93-94].
 * fem_stress computes in FP64 (FEM_ALGO_FP64); fem_stress_ex takes the algo. */
size_t fem_stress_workspace_bytes(int64_t n_elem);
int fem_stress(const fem_mesh* mesh, const fem_material* mat, const double* u,
               const int32_t* co_elem, const double* extrap, double* out, void* workspace,
               size_t workspace_bytes, void* stream);
/* fem_stress with the arithmetic chosen: FEM_ALGO_DD (double-float on the FP32 pipes, what
 * fem_stress uses) or FEM_ALGO_FP64 (native FP64).  With mesh->ne_inv set, FEM_ALGO_DD keeps
 * each node's corner records contiguous in the workspace (faster node pass); without it the
 * records stay in element order.  Same results either way.  workspace: 16-byte aligned. */
int fem_stress_ex(const fem_mesh* mesh, const fem_material* mat, const double* u,
                  const int32_t* co_elem, const double* extrap, double* out, void* workspace,
                  size_t workspace_bytes, int algo, void* stream);

/* Same as fem_stress, but for callers that cannot allocate device memory (a plug-in whose
 * host program owns every device buffer, or a loop where cudaMalloc/cudaFree are banned
 * because they synchronise the device).  No counterpart in the reference.  The per-element
 * scratch is a 24 MiB array built into the library, reserved on each GPU that loads it until
 * the process exits, so meshes are limited to FEM_STRESS_NOALLOC_MAX_ELEMS elements (larger
 * ones return FEM_ERR_WORKSPACE).  The first call on a device looks up the array's device
 * address and keeps it for the life of the process; make that first call before any stream
 * capture.  The kept address belongs to the device's context at that time: after
 * cudaDeviceReset (a new primary context) it is stale, so a program that resets a device does
 * not call this entry point on it again without reloading the library.  All calls share the one array:
 * calls that can overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  Nothing in the array needs clearing between calls.  It calls no
 * allocator. */
#define FEM_STRESS_NOALLOC_MAX_ELEMS 65536
int fem_stress_noalloc(const fem_mesh* mesh, const fem_material* mat, const double* u,
                       const int32_t* co_elem, const double* extrap, double* out, void* stream);

/* ---- BSR operators and the static solve ------------------------------------------- */
#define FEM_F64 0
#define FEM_F32 1

#define FEM_LAYOUT_RSOA 2 /* values of block row i stored [9][L_i] from 9*indptr[i] (value q of slot l
                             at 9*indptr[i] + q*L_i + l): lanes of a row read consecutive words */
#define FEM_LAYOUT_RSOA4 3 /* FP32 row-SoA with every row padded to a multiple of 4 blocks (its own
                              indptr/indices; padding blocks: column = the row, values 0), so a lane
                              reads 4 slots of one value with one 16-byte load */

typedef struct fem_bsr {
    int64_t n_brow, nnzb;   /* block rows (= nodes), 3x3 blocks                         */
    const int32_t* indptr;  /* [n_brow+1]                                               */
    const int32_t* indices; /* [nnzb]                                                   */
    const void* vals;       /* 9*nnzb values, double (FEM_F64) or float (FEM_F32)       */
    int dtype;
    int layout;             /* FEM_LAYOUT_BSR ([nnzb][3][3]), _RSOA or _RSOA4 (FP32)    */
} fem_bsr;

/* y = A x (SOLVE_static.py:36, KL * U).  nrhs in {1,2,4,8,16,32}; x, y: [n_brow][3][nrhs]
 * in A's precision.  variant: launch shape from fem_spmv_autotune (0 = default). */
int fem_bsr_spmv(const fem_bsr* A, int nrhs, const void* x, void* y, int variant, void* stream);
/* Times every nrhs == 1 launch variant on A (reps launches each) and returns the fastest.
 * No reference counterpart (tuning of the block-row tile shape). */
int fem_spmv_autotune(const fem_bsr* A, int nrhs, const void* x, void* y, int reps, int* best_variant,
                      float* best_ms, void* stream);
/* dst[i] = (float)src[i]: the FP32 copy of K / of preconditioner blocks for the mixed solve. */
int fem_convert_f64_to_f32(const double* src, float* dst, int64_t n, void* stream);
/* FP32 row-SoA copy (FEM_LAYOUT_RSOA) of an FP64 BSR matrix. */
int fem_bsr_to_rsoa_f32(const fem_bsr* A, float* dst, void* stream);
/* Padded FP32 row-SoA copy (FEM_LAYOUT_RSOA4), the inner-solve operator.  fem_rsoa4_indptr
 * (HOST arrays) gives its row pointers indptr4[n_brow+1] (rows rounded up to multiples of 4
 * blocks; nnzb4 = indptr4[n_brow]); fem_bsr_to_rsoa4_f32 fills indices4[nnzb4] and
 * vals4[9*nnzb4] from the FP64 BSR matrix A (indptr4 on the device). */
int fem_rsoa4_indptr(int64_t n_brow, const int32_t* indptr, int32_t* indptr4);
int fem_bsr_to_rsoa4_f32(const fem_bsr* A, const int32_t* indptr4, int32_t* indices4, float* vals4, void* stream);
/* Inverses of the 3x3 diagonal blocks (block-Jacobi preconditioner), FP64 and/or FP32
 * outputs [n_brow][9] (either may be NULL); *n_bad (device int) counts rows whose diagonal
 * block is missing or singular (identity used). */
int fem_block_jacobi(const fem_bsr* A, double* inv64, float* inv32, int* n_bad, void* stream);

typedef struct fem_pcg_opts {
    int nrhs;           /* 1, 2, 4, 8, 16 or 32 right-hand sides solved in lockstep          */
    int mixed;          /* 0: FP64 PCG; 1: FP32 inner PCG + FP64 iterative refinement       */
    double rtol;        /* stop when ||F - K U|| / ||F|| <= rtol for every RHS              */
    int maxit;          /* cap on PCG iterations (total inner iterations when mixed)         */
    double inner_rtol;  /* mixed: relative residual reduction asked of each inner FP32 solve */
    int inner_maxit;    /* mixed: cap per inner solve                                        */
    int max_outer;      /* mixed: cap on refinement steps                                    */
    int use_graph;      /* replay `unroll` iterations as one CUDA graph                      */
    int unroll;         /* iterations per graph / per host convergence check                 */
    int spmv_variant;   /* launch variant of the FP64 SpMV (fem_spmv_autotune)               */
    int spmv_variant32; /* launch variant of the FP32 SpMV                                   */
    int residual;       /* true residual F - K U: FEM_RESIDUAL_FP64 (0) or FEM_RESIDUAL_EXTRA */
    int stall_window;   /* > 0: stop with FEM_ERR_NOT_CONVERGED when the worst relative
                           (recursive) residual has not halved in this many iterations    */
} fem_pcg_opts;

/* How the solver forms the true residual r = F - K U that decides convergence and drives
 * the refinement / residual-replacement steps.  FEM_RESIDUAL_EXTRA evaluates each row as a
 * compensated dot product (as accurate as twice-FP64 arithmetic), so the refinement can drive
 * the forward error of U to the FP64 rounding level even where ||F - K U|| / ||F|| itself
 * cannot fall below the floor reported in fem_pcg_stats.floor. */
#define FEM_RESIDUAL_FP64 0
#define FEM_RESIDUAL_EXTRA 1

typedef struct fem_pcg_stats {
    int status;        /* FEM_OK, FEM_ERR_MAXITER, FEM_ERR_NOT_CONVERGED, FEM_ERR_NOT_SPD, ... */
    int iterations;    /* PCG iterations executed (sum of inner iterations when mixed)        */
    int outer;         /* refinement steps (1 for FP64 PCG)                                   */
    double relres;     /* max over RHS of the true residual ||F - K U|| / ||F||               */
    double time_ms;    /* device time of the solve (CUDA events)                              */
    double floor;      /* max over RHS of 2^-53 || |F| + |K||U| || / ||F||: the residual that
                          rounding U to FP64 alone leaves; an rtol below it cannot be met    */
} fem_pcg_stats;

/* Solve K U = F (SOLVE_static.py:31-33; Pardiso replaced by PCG).  precond: [n_brow][9]
 * FP64 preconditioner blocks applied as z_i = P_i r_i (block Jacobi from fem_block_jacobi,
 * or a learned SPD correction).  F, U: [n_brow][3][nrhs] FP64.  A32 (FP32 copy of A64) is
 * required when opts->mixed.  The call returns FEM_OK when it ran; stats->status tells
 * whether the tolerance was met: FEM_OK only when the true residual of the returned U
 * (formed as opts->residual says) is at most rtol for every right-hand side.  FP64 mode
 * (mixed = 0) runs PCG, then residual-replacement steps (K d = F - K U, U += d) while the
 * true residual is above rtol, at most max_outer solves in all. */
size_t fem_pcg_workspace_bytes(int64_t n_brow, int nrhs, int mixed);
int fem_pcg_solve(const fem_bsr* A64, const fem_bsr* A32, const double* precond, const double* F, double* U,
                  const fem_pcg_opts* opts, fem_pcg_stats* stats, void* workspace, size_t workspace_bytes,
                  void* stream);

/* ---- tall-skinny FP64 products of the block-Lanczos modal solve -------------------- */
/* Row-major FP64, DEVICE pointers, 1 <= m <= 256 columns of Q, 1 <= b <= 32.
 * fem_ts_gemm_tn: C (m x b, leading dimension ldc) = Q^T X for Q n x m (ldq) and X n x b
 * (ldx); deterministic (per-CTA partials summed in a fixed order).  workspace: at least
 * fem_ts_gemm_tn_workspace_bytes(n, m, b) bytes of device memory.
 * fem_ts_gemm_nn: W (n x b, ldw) = beta W + alpha Q C (beta = 0 does not read W). */
size_t fem_ts_gemm_tn_workspace_bytes(int64_t n, int m, int b);
int fem_ts_gemm_tn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* X, int64_t ldx, double* C,
                   int64_t ldc, void* workspace, size_t workspace_bytes, void* stream);
int fem_ts_gemm_nn(int64_t n, int m, int b, const double* Q, int64_t ldq, const double* C, int64_t ldc,
                   double alpha, double beta, double* W, int64_t ldw, void* stream);

/* ---- smoothed-aggregation AMG preconditioner (no reference counterpart) ----------- */
/* The reference factorises K directly (Pardiso, SOLVE_static.py:31-33).  Block-diagonal
 * preconditioners stall on slender or stretched meshes (condition numbers of 1e9 and more);
 * a smoothed-aggregation multigrid V-cycle built on the rigid-body modes does not.
 * fem_amg is a hierarchy object: fem_amg_setup builds it on the host (HOST arrays: K as FP64
 * BSR and the node coordinates), fem_amg_upload copies it to the device, fem_amg_destroy
 * frees it.  Unlike the rest of this interface the object allocates device memory itself
 * (the FP32 hierarchy, and per-level vectors on first use with a given nrhs).  One host
 * thread at a time per object. */
typedef struct fem_amg fem_amg;
typedef struct fem_amg_opts {
    double theta;     /* strength of connection: |A_ij|_F > theta sqrt(|A_ii|_F |A_jj|_F)    */
    int max_levels;   /* levels including the dense coarsest one                             */
    int max_coarse;   /* the coarsest level is solved densely once it has <= max_coarse DOF */
    int smooth;       /* 1: Jacobi-smoothed prolongator P = (I - w D^-1 A) T; 0: P = T       */
    int eig_steps;    /* Lanczos steps estimating lambda_max(D^-1 A) per level              */
    int pre_degree;   /* Chebyshev pre-smoothing degree (>= 1)                               */
    int post_degree;  /* Chebyshev post-smoothing degree (>= 1)                              */
    double cheb_upper; /* smoother interval [upper / cheb_ratio, upper], upper = cheb_upper * lambda_max */
    double cheb_ratio;
} fem_amg_opts;
void fem_amg_default_opts(fem_amg_opts* opts);
int fem_amg_setup(int64_t n_brow, const int32_t* indptr, const int32_t* indices, const double* vals,
                  const double* xyz, const fem_amg_opts* opts, fem_amg** out);
int fem_amg_upload(fem_amg* amg, void* stream);
/* The same hierarchy set up on the device: A64 the solver's FP64 matrix (FEM_LAYOUT_BSR,
 * DEVICE arrays), xyz [n_brow][3] node coordinates (DEVICE).  indptr_host / indices_host: an
 * optional HOST copy of A64's pattern (NULL: it is downloaded).  Every step runs in FP64
 * kernels except the two order-dependent greedy passes of the aggregation, which run on the
 * host from the strong-connection flags (one byte per block).  The result is ready for
 * fem_pcg_solve_amg (no fem_amg_upload); fem_amg_export reads its FP64 device copies.  Fails
 * with FEM_ERR_INVALID when a row of a Galerkin product has more than 3072 distinct block
 * columns (fem_amg_setup has no such limit).  Synchronises the stream. */
int fem_amg_setup_device(const fem_bsr* A64, const double* xyz, const int32_t* indptr_host,
                         const int32_t* indices_host, const fem_amg_opts* opts, void* stream, fem_amg** out);
void fem_amg_destroy(fem_amg* amg);
typedef struct fem_amg_level_info {
    int64_t n;        /* nodes (block rows) of the level                                    */
    int b;            /* DOF per node (3 on level 0, 6 on coarser levels)                    */
    int64_t nnzb_A;   /* blocks of the level operator (level 0: 0, the caller's matrix)     */
    int64_t nnzb_P;   /* blocks of the prolongator (0 on the last level)                     */
    double lmax;      /* Lanczos estimate of lambda_max(D^-1 A)                              */
    double omega;     /* prolongator smoothing weight                                        */
    double setup_s;   /* host seconds spent building this level's transfer and coarse operator */
} fem_amg_level_info;
int fem_amg_num_levels(const fem_amg* amg);
/* Replaces the Chebyshev smoother of one level (0 <= level < levels - 1) by the polynomial of
 * the same degree on [upper lmax / ratio, upper lmax] (1 <= upper <= 4, 1 < ratio <= 1e4):
 * per-level smoother weights, e.g. the learned ones of learned.py:LearnedSmoother.  Takes
 * effect from the next solve. */
int fem_amg_set_smoother(fem_amg* amg, int level, double upper, double ratio);
/* Host seconds of the setup phases summed over the levels: [0] strength + aggregation,
 * [1] tentative prolongator, [2] Lanczos, [3] prolongator smoothing, [4] Galerkin products,
 * [5] dense coarsest inverse. */
int fem_amg_setup_phases(const fem_amg* amg, double* seconds6);
int fem_amg_get_level(const fem_amg* amg, int level, fem_amg_level_info* info);
/* Host copies of one level's arrays.  what: 0 A (levels >= 1), 1 P, 2 R = P^T, 3 the inverse
 * diagonal blocks (vals [n][b][b]), 4 the aggregate of each node (indices [n], -1 = none),
 * 5 the dense inverse of the last level (vals [m][m]), 6 the Dirichlet flag of each node
 * (indices [n]: 1 = decoupled row held at x = D^-1 b in the cycle).  dims[4] receives (rows, nnzb or
 * entries, block rows, block cols); call with NULL arrays to size them. */
int fem_amg_export(const fem_amg* amg, int level, int what, int64_t* dims, int64_t* indptr, int32_t* indices,
                   double* vals);
/* One V-cycle z = M^-1 r on the device: FP32 vectors [n][3][nrhs]; A32 the FP32 copy of the
 * level-0 matrix (FEM_LAYOUT_BSR, _RSOA or _RSOA4).  symmetric = 1 ends the cycle with one
 * block-Jacobi update of the Dirichlet rows (the form the FP64 solve uses); 0 holds them at
 * D^-1 r (the form of the FP32 inner solve, which avoids FP32 products of penalty rows with
 * coupled vectors). */
int fem_amg_vcycle(fem_amg* amg, const fem_bsr* A32, int nrhs, const float* r, float* z, int symmetric, void* stream);
/* fem_pcg_solve with the V-cycle as the preconditioner.  opts->mixed = 1: the cycle
 * preconditions the FP32 inner solve of the refinement loop.  opts->mixed = 0: FP64 CG with
 * FP64 products with A64 around the FP32 cycle, with the flexible (Polak-Ribiere) beta; it
 * converges where FP32 refinement stalls (condition numbers beyond ~1e7).  A32 (the FP32
 * copy of A64) is required either way; workspace from fem_pcg_workspace_bytes(n, nrhs,
 * opts->mixed). */
int fem_pcg_solve_amg(const fem_bsr* A64, const fem_bsr* A32, fem_amg* amg, const double* F, double* U,
                      const fem_pcg_opts* opts, fem_pcg_stats* stats, void* workspace, size_t workspace_bytes,
                      void* stream);

/* ---- learned block-Jacobi correction (no reference counterpart) ------------------ */
/* Per-node MLP 16 -> 64 -> 64 -> 6 (SiLU), BF16 weights in PyTorch [out][in] layout, FP32
 * biases.  Output o (6 used of 16) gives L = [[e^o0,0,0],[o3,e^o1,0],[o4,o5,e^o2]] and the
 * preconditioner block P_i = G_i^{-T} L L^T G_i^{-1}, D_i = G_i G_i^T the diagonal block. */
typedef struct fem_mlp {
    const uint16_t* W1; /* [64][16] bf16 */
    const float* b1;    /* [64] */
    const uint16_t* W2; /* [64][64] bf16 */
    const float* b2;    /* [64] */
    const uint16_t* W3; /* [16][64] bf16, rows 6..15 zero */
    const float* b3;    /* [16] */
} fem_mlp;

int fem_mlp_nparams(void); /* flat FP32 parameter vector: W1, b1, W2, b2, W3, b3 */
/* ginv[n][9] = inverse Cholesky factors of the diagonal blocks of A (FP64 BSR). */
int fem_precond_cholesky(const fem_bsr* A, double* ginv, int* n_bad, void* stream);
/* Node features X[n][16] (bf16; Xf optional FP32 copy); lo/hi: HOST bounding box. */
int fem_precond_features(const fem_bsr* A, const double* ginv, const double* xyz, const uint8_t* fixed,
                         const double* lo, const double* hi, uint16_t* X, float* Xf, void* stream);
/* Probe products yhat = G^{-1} K G^{-T} z for nrhs probes ([n][3][nrhs]); w, y: FP64 scratch. */
int fem_probe_products(const fem_bsr* A, int nrhs, const double* ginv, const double* z, double* w, double* y,
                       float* yhat, void* stream);
/* Fused forward pass on the tensor cores (tcgen05); out[n][16]; z1, z2 ([n][64]
 * pre-activations, optional) for training; *err (device int) set if a wait timed out. */
int fem_mlp_forward(const fem_mlp* net, const uint16_t* X, int64_t n, float* out, float* z1, float* z2, int* err,
                    void* stream);
/* Loss mean_{i,r} |C_i yhat_ir - zhat_ir|^2 (as per-CTA partials, *n_partials of them, to be
 * summed and scaled by 1/(n nprobe)) and its gradient dout[n][16]. */
int fem_mlp_loss_grad(const float* out, const float* yhat, const float* zhat, int nprobe, int64_t n, float* dout,
                      double* loss_partials, int* n_partials, void* stream);
size_t fem_mlp_backward_workspace_bytes(int64_t n);
/* Parameter gradient grad[nparams] (deterministic CTA-ordered reduction). */
int fem_mlp_backward(const float* params, const uint16_t* X, const float* z1, const float* z2, const float* dout,
                     int64_t n, float* grad, void* workspace, size_t workspace_bytes, void* stream);
/* The same gradient on the tensor cores (tcgen05, BF16 operands, FP32 accumulation in TMEM):
 * dz3, dz2 and dz1 are rounded to BF16 where they enter a matrix product.  workspace: one
 * partial gradient per SM (fem_mlp_backward_tc_workspace_bytes); *err (device int) is set if a
 * bounded wait on the tensor cores timed out.  X, z1, z2 16-byte aligned. */
size_t fem_mlp_backward_tc_workspace_bytes(int64_t n);
int fem_mlp_backward_tc(const float* params, const uint16_t* X, const float* z1, const float* z2,
                        const float* dout, int64_t n, float* grad, void* workspace, size_t workspace_bytes,
                        int* err, void* stream);
/* Adam step on the FP32 parameters (step >= 1); refreshes the BF16 weight copies. */
int fem_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
                 float eps, uint16_t* W1, uint16_t* W2, uint16_t* W3, void* stream);
/* P[n][9] = G^{-T} C G^{-1} (FP64) from the MLP outputs. */
int fem_learned_blocks(int64_t n, const float* out, const double* ginv, double* P, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FEM_GB300_H */
