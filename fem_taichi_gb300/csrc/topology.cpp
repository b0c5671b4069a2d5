// Host-side topology: block pattern (READ_physics.py:42-61) and node->element incidence.
//
// The reference builds Node_Node = Elem_Node^T * Elem_Node with a scipy SpGEMM and sorts
// each row; the pattern is the set of node pairs that share an element, columns ascending.
// Here the same set is built directly: counting-sort incidence, then per row a sort/unique
// of the corner lists of the incident elements.  Rows are independent (OpenMP).
#include <stdarg.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "fem_common.cuh"

namespace fem {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const ShapeTables& shape_tables() {
    static ShapeTables t = [] {
        ShapeTables s{};
        const double gs[2] = {-kGS1, kGS1};
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const int g = 4 * i + 2 * j + k;  // zeta fastest (FEM_model_bsr.py:425-432)
                    const double r0 = gs[i], r1 = gs[j], r2 = gs[k];
                    double* n = s.nr[g];
                    n[0] = 0.125 * (1 + r0) * (1 + r1) * (1 - r2);
                    n[1] = 0.125 * (1 - r0) * (1 + r1) * (1 - r2);
                    n[2] = 0.125 * (1 - r0) * (1 - r1) * (1 - r2);
                    n[3] = 0.125 * (1 + r0) * (1 - r1) * (1 - r2);
                    n[4] = 0.125 * (1 + r0) * (1 + r1) * (1 + r2);
                    n[5] = 0.125 * (1 - r0) * (1 + r1) * (1 + r2);
                    n[6] = 0.125 * (1 - r0) * (1 - r1) * (1 + r2);
                    n[7] = 0.125 * (1 + r0) * (1 - r1) * (1 + r2);
                    double(*d)[3] = s.dnr[g];
                    d[2][0] = 0.125 * (-1) * (1 - r1) * (1 - r2);
                    d[2][1] = 0.125 * (1 - r0) * (-1) * (1 - r2);
                    d[2][2] = 0.125 * (1 - r0) * (1 - r1) * (-1);
                    d[6][0] = 0.125 * (-1) * (1 - r1) * (1 + r2);
                    d[6][1] = 0.125 * (1 - r0) * (-1) * (1 + r2);
                    d[6][2] = 0.125 * (1 - r0) * (1 - r1) * (+1);
                    d[7][0] = 0.125 * (+1) * (1 - r1) * (1 + r2);
                    d[7][1] = 0.125 * (1 + r0) * (-1) * (1 + r2);
                    d[7][2] = 0.125 * (1 + r0) * (1 - r1) * (+1);
                    d[3][0] = 0.125 * (+1) * (1 - r1) * (1 - r2);
                    d[3][1] = 0.125 * (1 + r0) * (-1) * (1 - r2);
                    d[3][2] = 0.125 * (1 + r0) * (1 - r1) * (-1);
                    d[1][0] = 0.125 * (-1) * (1 + r1) * (1 - r2);
                    d[1][1] = 0.125 * (1 - r0) * (+1) * (1 - r2);
                    d[1][2] = 0.125 * (1 - r0) * (1 + r1) * (-1);
                    d[5][0] = 0.125 * (-1) * (1 + r1) * (1 + r2);
                    d[5][1] = 0.125 * (1 - r0) * (+1) * (1 + r2);
                    d[5][2] = 0.125 * (1 - r0) * (1 + r1) * (+1);
                    d[4][0] = 0.125 * (+1) * (1 + r1) * (1 + r2);
                    d[4][1] = 0.125 * (1 + r0) * (+1) * (1 + r2);
                    d[4][2] = 0.125 * (1 + r0) * (1 + r1) * (+1);
                    d[0][0] = 0.125 * (+1) * (1 + r1) * (1 - r2);
                    d[0][1] = 0.125 * (1 + r0) * (+1) * (1 - r2);
                    d[0][2] = 0.125 * (1 + r0) * (1 + r1) * (-1);
                }
        return s;
    }();
    return t;
}

namespace {

int check_conn(int64_t n_node, int64_t n_elem, const int32_t* conn) {
    FEM_REQUIRE(n_node >= 0 && n_elem >= 0, "negative size");
    FEM_REQUIRE(n_elem == 0 || conn != nullptr, "conn is NULL");
    FEM_REQUIRE(n_node < (int64_t(1) << 31) - 1, "n_node too large for int32 indices");
    FEM_REQUIRE(n_elem < (int64_t(1) << 28), "n_elem too large for e*8+a int32 encoding");
    for (int64_t i = 0; i < 8 * n_elem; ++i)
        FEM_REQUIRE(conn[i] >= 0 && conn[i] < n_node, "conn[%lld] = %d out of range [0, %lld)",
                    (long long)i, conn[i], (long long)n_node);
    return FEM_OK;
}

// Counting sort of (e, a) by node; stable, so each node's list is ascending in (e, a).
void incidence(int64_t n_node, int64_t n_elem, const int32_t* conn, std::vector<int32_t>& ptr,
               std::vector<int32_t>& list) {
    ptr.assign(n_node + 1, 0);
    for (int64_t i = 0; i < 8 * n_elem; ++i) ptr[conn[i] + 1]++;
    for (int64_t i = 0; i < n_node; ++i) ptr[i + 1] += ptr[i];
    list.resize(8 * n_elem);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int64_t i = 0; i < 8 * n_elem; ++i) list[fill[conn[i]]++] = int32_t(i);
}

// Sorted unique neighbours of node i into out (cleared first).
inline void row_nodes(int64_t i, const int32_t* conn, const std::vector<int32_t>& ptr,
                      const std::vector<int32_t>& list, std::vector<int32_t>& out) {
    out.clear();
    for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
        const int64_t e = list[k] >> 3;
        for (int a = 0; a < 8; ++a) out.push_back(conn[8 * e + a]);
    }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
}

}  // namespace
}  // namespace fem

using namespace fem;

extern "C" const char* fem_last_error(void) { return g_err; }

extern "C" int fem_abi_version(void) { return 1; }

extern "C" int fem_pattern_count(int64_t n_node, int64_t n_elem, const int32_t* conn,
                                 int32_t* indptr, int64_t* nnzb) {
    int rc = check_conn(n_node, n_elem, conn);
    if (rc) return rc;
    FEM_REQUIRE(indptr && nnzb, "indptr/nnzb is NULL");
    std::vector<int32_t> ptr, list;
    incidence(n_node, n_elem, conn, ptr, list);
    std::vector<int64_t> cnt(n_node, 0);
#pragma omp parallel
    {
        std::vector<int32_t> row;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t i = 0; i < n_node; ++i) {
            row_nodes(i, conn, ptr, list, row);
            cnt[i] = int64_t(row.size());
        }
    }
    int64_t acc = 0;
    indptr[0] = 0;
    for (int64_t i = 0; i < n_node; ++i) {
        acc += cnt[i];
        FEM_REQUIRE(acc < (int64_t(1) << 31), "nnzb exceeds int32 range");
        indptr[i + 1] = int32_t(acc);
    }
    *nnzb = acc;
    return FEM_OK;
}

extern "C" int fem_pattern_fill(int64_t n_node, int64_t n_elem, const int32_t* conn,
                                const int32_t* indptr, int32_t* indices) {
    int rc = check_conn(n_node, n_elem, conn);
    if (rc) return rc;
    FEM_REQUIRE(indptr && indices, "indptr/indices is NULL");
    std::vector<int32_t> ptr, list;
    incidence(n_node, n_elem, conn, ptr, list);
    int bad = 0;
#pragma omp parallel
    {
        std::vector<int32_t> row;
#pragma omp for schedule(dynamic, 1024) reduction(| : bad)
        for (int64_t i = 0; i < n_node; ++i) {
            row_nodes(i, conn, ptr, list, row);
            if (int64_t(row.size()) != int64_t(indptr[i + 1]) - indptr[i]) {
                bad = 1;
                continue;
            }
            std::copy(row.begin(), row.end(), indices + indptr[i]);
        }
    }
    FEM_REQUIRE(!bad, "indptr does not match this connectivity");
    return FEM_OK;
}

extern "C" int fem_incidence_build(int64_t n_node, int64_t n_elem, const int32_t* conn,
                                   int32_t* ne_ptr, int32_t* ne_list, int32_t* co_elem) {
    int rc = check_conn(n_node, n_elem, conn);
    if (rc) return rc;
    FEM_REQUIRE(ne_ptr && ne_list, "ne_ptr/ne_list is NULL");
    std::vector<int32_t> ptr, list;
    incidence(n_node, n_elem, conn, ptr, list);
    memcpy(ne_ptr, ptr.data(), sizeof(int32_t) * (n_node + 1));
    if (n_elem) memcpy(ne_list, list.data(), sizeof(int32_t) * 8 * n_elem);
    if (co_elem) {
        // Distinct elements per node: the reference's COO->CSC conversion sums duplicate
        // (element, node) entries, so a repeated corner counts once.
        for (int64_t i = 0; i < n_node; ++i) {
            int32_t c = 0, last = -1;
            for (int32_t k = ptr[i]; k < ptr[i + 1]; ++k) {
                const int32_t e = list[k] >> 3;
                if (e != last) ++c, last = e;
            }
            co_elem[i] = c;
        }
    }
    return FEM_OK;
}

extern "C" int fem_gather_map(int64_t n_node, int64_t n_elem, const int32_t* conn, const int32_t* indptr,
                              const int32_t* indices, const int32_t* ne_ptr, const int32_t* ne_list, int32_t* ne_inv,
                              uint8_t* slot_map) {
    int rc = check_conn(n_node, n_elem, conn);
    if (rc) return rc;
    FEM_REQUIRE(indptr && ne_ptr && ne_list && ne_inv && slot_map, "NULL argument");
    FEM_REQUIRE(n_elem == 0 || indices, "indices is NULL");
    // ne_inv[e*8+a] = position of (e, a) in the incidence list of node conn[e][a]
    for (int64_t k = 0; k < 8 * n_elem; ++k) ne_inv[k] = -1;
    for (int64_t i = 0; i < n_node; ++i)
        for (int32_t k = ne_ptr[i]; k < ne_ptr[i + 1]; ++k) {
            const int32_t ent = ne_list[k];
            FEM_REQUIRE(ent >= 0 && ent < 8 * n_elem && conn[ent] == i, "incidence does not match conn");
            ne_inv[ent] = k;
        }
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t e = 0; e < n_elem; ++e) {
        for (int a = 0; a < 8; ++a) {
            const int32_t row = conn[8 * e + a];
            const int32_t* b0 = indices + indptr[row];
            const int32_t* b1 = indices + indptr[row + 1];
            const int64_t pos = ne_inv[8 * e + a];
            if (pos < 0) {
                bad = 1;
                continue;
            }
            for (int b = 0; b < 8; ++b) {
                const int32_t col = conn[8 * e + b];
                const int32_t* it = std::lower_bound(b0, b1, col);
                if (it == b1 || *it != col || it - b0 > 255) {
                    bad = 1;
                    slot_map[8 * pos + b] = 0;
                    continue;
                }
                slot_map[8 * pos + b] = uint8_t(it - b0);
            }
        }
    }
    if (bad) {
        set_error("an element node pair is missing from the pattern, or a block row has more than 256 blocks");
        return FEM_ERR_PATTERN;
    }
    return FEM_OK;
}

extern "C" int fem_pipeline_plan(int64_t n_node, int64_t n_elem, const int32_t* indptr, const int32_t* ne_ptr,
                                 const int32_t* ne_list, int n_parts, int64_t* row_split, int64_t* elem_split,
                                 int64_t* block_split) {
    FEM_REQUIRE(n_node >= 0 && n_elem >= 0, "negative size");
    FEM_REQUIRE(n_parts >= 1 && n_parts <= 4096, "n_parts must lie in [1, 4096]");
    FEM_REQUIRE(row_split && elem_split && block_split, "NULL output");
    FEM_REQUIRE(n_node == 0 || (indptr && ne_ptr && (n_elem == 0 || ne_list)), "NULL pattern/incidence array");
    const int64_t nnzb = n_node ? indptr[n_node] : 0;
    // rows split so that every part holds about the same number of blocks (copy volume)
    row_split[0] = 0;
    for (int q = 1; q < n_parts; ++q) {
        const int64_t target = nnzb * q / n_parts;
        const int32_t* it = std::lower_bound(indptr, indptr + n_node + 1, int32_t(target));
        row_split[q] = std::max(row_split[q - 1], int64_t(it - indptr));
        row_split[q] = std::min<int64_t>(row_split[q], n_node);
    }
    row_split[n_parts] = n_node;
    // elements a part needs: every element incident to one of its rows or an earlier row
    int64_t emax = 0;
    int64_t r = 0;
    elem_split[0] = 0;
    for (int q = 1; q <= n_parts; ++q) {
        for (; r < row_split[q]; ++r)
            if (ne_ptr[r + 1] > ne_ptr[r]) emax = std::max<int64_t>(emax, (ne_list[ne_ptr[r + 1] - 1] >> 3) + 1);
        elem_split[q] = q == n_parts ? n_elem : std::min(emax, n_elem);
    }
    for (int q = 0; q <= n_parts; ++q) block_split[q] = n_node ? indptr[row_split[q]] : 0;
    return FEM_OK;
}
