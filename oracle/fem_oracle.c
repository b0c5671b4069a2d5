/*
 * CPU restatement of the FEM_taichi hex8 hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Follows the reference algorithm step for step so that it can serve both as an
 * independent cross-check of the numpy oracle (oracle/fem_oracle.py) and as the timed
 * CPU baseline ("port") on the host cores:
 *   - element loop, parallel over elements           FEM_model_bsr.py:163-175
 *   - per-element 8x8 block scratch (KTmat / MMat)   FEM_model_bsr.py:60-62, 262-287
 *   - B^T D B for all 64 node pairs at 8 Gauss pts   FEM_model_bsr.py:262-274, 303-347
 *   - linear search of the slot in ReNode            FEM_model_bsr.py:171-175
 *   - atomic += scatter into the block values        (Taichi parallel-for +=)
 *   - 1e20 diagonal penalty                          FEM_model_bsr.py:248-259
 *   - centrifugal F + int-cast nodal loads           FEM_model_bsr.py:220-245, 291-300
 *   - stress: GP stress, extrapolation, average      POST_process.py:172-209
 * With nthreads == 1 the scatter order is element-major (e, j, k), i.e. the order a
 * serial run of the reference kernels would use.
 *
 * Parity: agrees with the numpy restatement (oracle/fem_oracle.py), which is pinned to
 * outputs of the reference's own code (tests/golden/refexec_*.npz, tests/test_refexec.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define GS1 0.57735026918962

static double RM[8][3];      /* Gauss points, zeta fastest: FEM_model_bsr.py:425-432 */
static double NRg[8][8];     /* N_a(g)          FEM_model_bsr.py:371-382 */
static double DNRg[8][8][3]; /* dN_a/dxi_d (g)  FEM_model_bsr.py:384-419 */
static int inited = 0;

static void shape_func(const double r[3], double N[8]) {
    N[0] = 0.125 * (1 + r[0]) * (1 + r[1]) * (1 - r[2]);
    N[1] = 0.125 * (1 - r[0]) * (1 + r[1]) * (1 - r[2]);
    N[2] = 0.125 * (1 - r[0]) * (1 - r[1]) * (1 - r[2]);
    N[3] = 0.125 * (1 + r[0]) * (1 - r[1]) * (1 - r[2]);
    N[4] = 0.125 * (1 + r[0]) * (1 + r[1]) * (1 + r[2]);
    N[5] = 0.125 * (1 - r[0]) * (1 + r[1]) * (1 + r[2]);
    N[6] = 0.125 * (1 - r[0]) * (1 - r[1]) * (1 + r[2]);
    N[7] = 0.125 * (1 + r[0]) * (1 - r[1]) * (1 + r[2]);
}

static void shape_derv(const double r[3], double d[8][3]) {
    d[2][0] = 0.125 * (-1) * (1 - r[1]) * (1 - r[2]);
    d[2][1] = 0.125 * (1 - r[0]) * (-1) * (1 - r[2]);
    d[2][2] = 0.125 * (1 - r[0]) * (1 - r[1]) * (-1);
    d[6][0] = 0.125 * (-1) * (1 - r[1]) * (1 + r[2]);
    d[6][1] = 0.125 * (1 - r[0]) * (-1) * (1 + r[2]);
    d[6][2] = 0.125 * (1 - r[0]) * (1 - r[1]) * (+1);
    d[7][0] = 0.125 * (+1) * (1 - r[1]) * (1 + r[2]);
    d[7][1] = 0.125 * (1 + r[0]) * (-1) * (1 + r[2]);
    d[7][2] = 0.125 * (1 + r[0]) * (1 - r[1]) * (+1);
    d[3][0] = 0.125 * (+1) * (1 - r[1]) * (1 - r[2]);
    d[3][1] = 0.125 * (1 + r[0]) * (-1) * (1 - r[2]);
    d[3][2] = 0.125 * (1 + r[0]) * (1 - r[1]) * (-1);
    d[1][0] = 0.125 * (-1) * (1 + r[1]) * (1 - r[2]);
    d[1][1] = 0.125 * (1 - r[0]) * (+1) * (1 - r[2]);
    d[1][2] = 0.125 * (1 - r[0]) * (1 + r[1]) * (-1);
    d[5][0] = 0.125 * (-1) * (1 + r[1]) * (1 + r[2]);
    d[5][1] = 0.125 * (1 - r[0]) * (+1) * (1 + r[2]);
    d[5][2] = 0.125 * (1 - r[0]) * (1 + r[1]) * (+1);
    d[4][0] = 0.125 * (+1) * (1 + r[1]) * (1 + r[2]);
    d[4][1] = 0.125 * (1 + r[0]) * (+1) * (1 + r[2]);
    d[4][2] = 0.125 * (1 + r[0]) * (1 + r[1]) * (+1);
    d[0][0] = 0.125 * (+1) * (1 + r[1]) * (1 - r[2]);
    d[0][1] = 0.125 * (1 + r[0]) * (+1) * (1 - r[2]);
    d[0][2] = 0.125 * (1 + r[0]) * (1 + r[1]) * (-1);
}

static void init_tables(void) {
    if (inited) return;
    const double gs[2] = {-GS1, GS1};
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
                int g = 4 * i + 2 * j + k;
                RM[g][0] = gs[i]; RM[g][1] = gs[j]; RM[g][2] = gs[k];
            }
    for (int g = 0; g < 8; ++g) {
        shape_func(RM[g], NRg[g]);
        shape_derv(RM[g], DNRg[g]);
    }
    inited = 1;
}

static double det3(const double a[3][3]) {
    return a[0][0] * (a[1][1] * a[2][2] - a[2][1] * a[1][2])
         - a[1][0] * (a[0][1] * a[2][2] - a[2][1] * a[0][2])
         + a[2][0] * (a[0][1] * a[1][2] - a[1][1] * a[0][2]);
}

static void inv3(const double a[3][3], double out[3][3]) {
    double inv_det = 1.0 / det3(a);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
            out[j][i] = inv_det * (a[i1][j1] * a[i2][j2] - a[i2][j1] * a[i1][j2]);
        }
}

/* J = Coord(3x8) @ DNr(8x3) ; Coord[k][a] = xyz of node a */
static void jacobian(const double C[3][8], const double D[8][3], double J[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 3; ++d) {
            double s = 0;
            for (int a = 0; a < 8; ++a) s += C[i][a] * D[a][d];
            J[i][d] = s;
        }
}

static inline void atomic_add(double* p, double v, int nthreads) {
    if (nthreads > 1) {
#pragma omp atomic
        *p += v;
    } else {
        *p += v;
    }
}

static inline int64_t find_slot(const int32_t* indptr, const int32_t* indices, int row, int col) {
    int64_t s0 = indptr[row], n = (int64_t)indptr[row + 1] - s0;
    for (int64_t m = 0; m < n; ++m)
        if (indices[s0 + m] == col) return s0 + m;
    return -1;
}

/*
 * Assemble K (BSR [nnzb][3][3]), per-block scalar M [nnzb] and F [n_node][3].
 * conn: [n_elem][8] node indices (Nind already applied).
 * bounds: n_bound entries of (node index, 3 dof codes; code != -1 => fixed).
 * forces: n_force entries of (node index, 3 values already int-cast by the caller).
 * Returns 0 on success, -1 if an element node pair is missing from the pattern.
 */
int oracle_assemble(int64_t n_node, int64_t n_elem, const double* xyz, const int32_t* conn,
                    const int32_t* indptr, const int32_t* indices,
                    double DE, double EX, double PO, const double* omega,
                    int64_t n_bound, const int32_t* bound_node, const double* bound_code,
                    int64_t n_force, const int32_t* force_node, const double* force_val,
                    double* K, double* M, double* F, int nthreads) {
    init_tables();
    const int64_t nnzb = indptr[n_node];
    memset(K, 0, sizeof(double) * 9 * nnzb);
    memset(M, 0, sizeof(double) * nnzb);
    memset(F, 0, sizeof(double) * 3 * n_node);
    double D0[3][3], mu = EX / 2 / (1 + PO);
    double dd = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO), dof = EX * PO / (1 + PO) / (1 - 2 * PO);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D0[i][j] = (i == j) ? dd : dof;
    const double w0 = omega[0], w1 = omega[1], w2 = omega[2];
    int bad = 0;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads) reduction(| : bad)
#endif
    for (int64_t e = 0; e < n_elem; ++e) {
        double C[3][8];
        int nd[8];
        for (int a = 0; a < 8; ++a) {
            nd[a] = conn[8 * e + a];
            for (int k = 0; k < 3; ++k) C[k][a] = xyz[3 * (int64_t)nd[a] + k];
        }
        double Ke[8][8][3][3];
        double Me[8][8];
        double Fe[8][3];
        memset(Ke, 0, sizeof Ke);
        memset(Me, 0, sizeof Me);
        memset(Fe, 0, sizeof Fe);
        for (int g = 0; g < 8; ++g) {
            double J[3][3], Ji[3][3], DN[8][3];
            jacobian(C, DNRg[g], J);
            inv3(J, Ji);
            double det = det3(J);
            for (int a = 0; a < 8; ++a)
                for (int i = 0; i < 3; ++i) {
                    double s = 0;
                    for (int d = 0; d < 3; ++d) s += DNRg[g][a][d] * Ji[d][i];
                    DN[a][i] = s;
                }
            /* B1 = diag(DN_j); B2 rows (yz, xz, xy):  FEM_model_bsr.py:303-347 */
            for (int j = 0; j < 8; ++j) {
                double B2j[3][3] = {{0, DN[j][2], DN[j][1]}, {DN[j][2], 0, DN[j][0]}, {DN[j][1], DN[j][0], 0}};
                for (int k = 0; k < 8; ++k) {
                    double B2k[3][3] = {{0, DN[k][2], DN[k][1]}, {DN[k][2], 0, DN[k][0]}, {DN[k][1], DN[k][0], 0}};
                    for (int p = 0; p < 3; ++p)
                        for (int q = 0; q < 3; ++q) {
                            double t1 = DN[j][p] * D0[p][q] * DN[k][q];
                            double t2 = 0;
                            for (int r = 0; r < 3; ++r) t2 += B2j[r][p] * mu * B2k[r][q];
                            Ke[j][k][p][q] += det * (t1 + t2);
                        }
                }
            }
            /* M: FEM_model_bsr.py:276-287 */
            double jdm = DE * det;
            for (int j = 0; j < 8; ++j)
                for (int k = 0; k < 8; ++k) Me[j][k] += jdm * NRg[g][j] * NRg[g][k];
            /* F: FEM_model_bsr.py:229-245, 291-300 */
            double R[3];
            for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int a = 0; a < 8; ++a) s += C[i][a] * NRg[g][a];
                R[i] = s;
            }
            double f0 = w1 * w1 * R[0] + w2 * w2 * R[0] - w0 * w1 * R[1] - w0 * w2 * R[2];
            double f1 = w0 * w0 * R[1] + w2 * w2 * R[1] - w1 * w2 * R[2] - w1 * w0 * R[0];
            double f2 = w1 * w1 * R[2] + w0 * w0 * R[2] - w2 * w0 * R[0] - w2 * w1 * R[1];
            for (int k = 0; k < 8; ++k) {
                Fe[k][0] += jdm * NRg[g][k] * f0;
                Fe[k][1] += jdm * NRg[g][k] * f1;
                Fe[k][2] += jdm * NRg[g][k] * f2;
            }
        }
        /* scatter: linear search over the row, then += (atomic when threaded) */
        for (int j = 0; j < 8; ++j)
            for (int k = 0; k < 8; ++k) {
                int64_t s = find_slot(indptr, indices, nd[j], nd[k]);
                if (s < 0) { bad = 1; continue; }
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) atomic_add(&K[9 * s + 3 * p + q], Ke[j][k][p][q], nthreads);
                atomic_add(&M[s], Me[j][k], nthreads);
            }
        for (int k = 0; k < 8; ++k)
            for (int c = 0; c < 3; ++c) atomic_add(&F[3 * (int64_t)nd[k] + c], Fe[k][c], nthreads);
    }
    if (bad) return -1;
    /* LoadF: FEM_model_bsr.py:220-226 */
    for (int64_t i = 0; i < n_force; ++i)
        for (int c = 0; c < 3; ++c) F[3 * (int64_t)force_node[i] + c] += force_val[3 * i + c];
    /* ModifyMatrixK: FEM_model_bsr.py:248-259 */
    for (int64_t i = 0; i < n_bound; ++i) {
        int idx = bound_node[i];
        int64_t s = find_slot(indptr, indices, idx, idx);
        if (s < 0) continue;
        for (int j = 0; j < 3; ++j)
            if (bound_code[3 * i + j] != -1) K[9 * s + 3 * j + j] = 1e20;
    }
    return 0;
}

/* Cyclic Jacobi eigenvalues of a symmetric 3x3 (ascending). */
static void sym3_eig(const double A[3][3], double ev[3]) {
    double a[3][3];
    memcpy(a, A, sizeof a);
    for (int sweep = 0; sweep < 50; ++sweep) {
        double off = fabs(a[0][1]) + fabs(a[0][2]) + fabs(a[1][2]);
        if (off == 0.0) break;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                if (a[p][q] == 0.0) continue;
                double theta = (a[q][q] - a[p][p]) / (2 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < 3; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
            }
    }
    double e[3] = {a[0][0], a[1][1], a[2][2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (e[j] < e[i]) { double t = e[i]; e[i] = e[j]; e[j] = t; }
    ev[0] = e[0]; ev[1] = e[1]; ev[2] = e[2];
}

/*
 * Nodal stress table [n_node][10]; POST_process.py:72-99,172-209.
 * W: [8][8] extrapolation weights W[j][k] (node j <- GP k).
 */
int oracle_stress(int64_t n_node, int64_t n_elem, const double* xyz, const int32_t* conn,
                  const int32_t* co_elem, double EX, double PO, const double* u,
                  const double* W, double* out, int nthreads) {
    init_tables();
    double* S = (double*)calloc((size_t)n_node * 6, sizeof(double));
    if (!S) return -1;
    double D0[3][3], mu = EX / 2 / (1 + PO);
    double dd = EX * (1 - PO) / (1 + PO) / (1 - 2 * PO), dof = EX * PO / (1 + PO) / (1 - 2 * PO);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) D0[i][j] = (i == j) ? dd : dof;
#ifdef _OPENMP
    if (nthreads < 1) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#endif
    for (int64_t e = 0; e < n_elem; ++e) {
        double C[3][8], U[8][3];
        int nd[8];
        for (int a = 0; a < 8; ++a) {
            nd[a] = conn[8 * e + a];
            for (int k = 0; k < 3; ++k) {
                C[k][a] = xyz[3 * (int64_t)nd[a] + k];
                U[a][k] = u[3 * (int64_t)nd[a] + k];
            }
        }
        double SV[8][6];
        memset(SV, 0, sizeof SV);
        for (int g = 0; g < 8; ++g) {
            double J[3][3], Ji[3][3];
            jacobian(C, DNRg[g], J);
            inv3(J, Ji);
            for (int k = 0; k < 8; ++k) {
                double d[3];
                for (int i = 0; i < 3; ++i) {
                    double s = 0;
                    for (int m = 0; m < 3; ++m) s += DNRg[g][k][m] * Ji[m][i];
                    d[i] = s;
                }
                double en[3] = {d[0] * U[k][0], d[1] * U[k][1], d[2] * U[k][2]};
                double es[3] = {d[1] * U[k][0] + d[0] * U[k][1], d[2] * U[k][1] + d[1] * U[k][2],
                                d[2] * U[k][0] + d[0] * U[k][2]};
                for (int i = 0; i < 3; ++i) {
                    SV[g][i] += D0[i][0] * en[0] + D0[i][1] * en[1] + D0[i][2] * en[2];
                    SV[g][3 + i] += mu * es[i];
                }
            }
        }
        for (int j = 0; j < 8; ++j)
            for (int c = 0; c < 6; ++c) {
                double s = 0;
                for (int k = 0; k < 8; ++k) s += W[8 * j + k] * SV[k][c];
                atomic_add(&S[6 * (int64_t)nd[j] + c], s, nthreads);
            }
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n_node; ++i) {
        double v[6];
        for (int c = 0; c < 6; ++c) v[c] = S[6 * i + c] / co_elem[i];
        double A[3][3] = {{v[0], v[3], v[5]}, {v[3], v[1], v[4]}, {v[5], v[4], v[2]}};
        double ev[3];
        sym3_eig(A, ev);
        double p1 = ev[2], p2 = ev[1], p3 = ev[0];
        double* o = out + 10 * i;
        for (int c = 0; c < 6; ++c) o[c] = v[c];
        o[6] = p1; o[7] = p2; o[8] = p3;
        o[9] = sqrt((p1 - p2) * (p1 - p2) + (p2 - p3) * (p2 - p3) + (p3 - p2) * (p3 - p2));
    }
    free(S);
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
