// Device build of the mesh topology: node -> element incidence, the block pattern of K
// (READ_physics.py:42-61: Node_Node = Elem_Node^T Elem_Node, columns sorted) and the
// element-to-block map of the gather.  Same arrays, bit for bit, as the host build in
// topology.cpp (fem_incidence_build, fem_pattern_count/fill, fem_gather_map).
//
//  1. incidence: per-node counts (integer atomics), exclusive scan -> ne_ptr, scatter of the
//     entries e*8+a, then each node's short list sorted ascending (so the order does not
//     depend on the atomics); co_elem = distinct elements per node.
//  2. pattern: one warp per block row gathers the corner nodes of the row's incident
//     elements (8 per element) into shared memory, sorts them (bitonic, padded to a power of
//     two) and keeps the distinct ones -> row length; scan -> indptr; the sorted rows are then
//     compacted into indices.
//  3. gather map: ne_inv by scatter; slot_map by binary search of each corner's node in the
//     row of the entry's node.
#include <climits>

#include "fem_common.cuh"

namespace fem {
namespace {

constexpr int kMaxCand = 1024;  // corner candidates per block row (128 incident elements)
constexpr int kRowWarps = 4;

__global__ void k_count_corners(int64_t n8, const int32_t* __restrict__ conn, int32_t* cnt) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n8; i += int64_t(gridDim.x) * blockDim.x)
        atomicAdd(cnt + conn[i], 1);
}

__global__ void k_scatter_corners(int64_t n8, const int32_t* __restrict__ conn, const int32_t* __restrict__ ne_ptr,
                                  int32_t* fill, int32_t* ne_list) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n8; i += int64_t(gridDim.x) * blockDim.x) {
        const int32_t node = conn[i];
        ne_list[ne_ptr[node] + atomicAdd(fill + node, 1)] = int32_t(i);
    }
}

// Insertion sort of each node's incidence list; co_elem = distinct elements.
__global__ void k_sort_incidence(int64_t n, const int32_t* __restrict__ ne_ptr, int32_t* ne_list, int32_t* co_elem) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int32_t b = ne_ptr[i], e = ne_ptr[i + 1];
        for (int32_t k = b + 1; k < e; ++k) {
            const int32_t v = ne_list[k];
            int32_t j = k - 1;
            while (j >= b && ne_list[j] > v) {
                ne_list[j + 1] = ne_list[j];
                --j;
            }
            ne_list[j + 1] = v;
        }
        int32_t c = 0, last = -1;
        for (int32_t k = b; k < e; ++k) {
            const int32_t el = ne_list[k] >> 3;
            if (el != last) ++c, last = el;
        }
        if (co_elem) co_elem[i] = c;
    }
}

// Exclusive scan of cnt[0..n) into out[0..n] (out[n] = total), three passes.  status bit 1:
// the total exceeds the int32 range.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int64_t kScanTile = int64_t(kScanThreads) * kScanPer;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t* sh, int64_t& total) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    int64_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int64_t s = lane < int(blockDim.x / 32) ? sh[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, s, off);
            if (lane >= off) s += y;
        }
        sh[lane] = s;  // inclusive warp totals
    }
    __syncthreads();
    total = sh[blockDim.x / 32 - 1];
    const int64_t before = w > 0 ? sh[w - 1] : 0;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(int64_t n, const int32_t* __restrict__ cnt, int32_t* out,
                                                             int64_t* tile_sum) {
    __shared__ int64_t sh[32];
    const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanPer;
    int64_t v[kScanPer], s = 0;
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        v[j] = base + j < n ? cnt[base + j] : 0;
        s += v[j];
    }
    int64_t total;
    int64_t run = block_exclusive_scan(s, sh, total);
#pragma unroll
    for (int j = 0; j < kScanPer; ++j) {
        if (base + j < n) out[base + j] = int32_t(run);  // tile-local; offsets added later
        run += v[j];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int64_t ntiles, int64_t* tile_sum, int32_t* out_total,
                                                            int64_t n, int* status) {
    __shared__ int64_t sh[32];
    int64_t carry = 0;
    for (int64_t b = 0; b < ntiles; b += kScanThreads) {
        const int64_t i = b + threadIdx.x;
        const int64_t v = i < ntiles ? tile_sum[i] : 0;
        int64_t total;
        const int64_t ex = block_exclusive_scan(v, sh, total);
        if (i < ntiles) tile_sum[i] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) {
        if (carry >= (int64_t(1) << 31)) atomicOr(status, 2);
        out_total[n] = int32_t(carry);
    }
}

__global__ void k_scan_add(int64_t n, const int64_t* __restrict__ tile_sum, int32_t* out) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        out[i] = int32_t(out[i] + tile_sum[i / kScanTile]);
}

// Sorted distinct corner nodes of row i's incident elements -> rows[8 * ne_ptr[i] ...],
// count -> len[i].  One warp per row.  status bit 1: a row has more than kMaxCand candidates.
__global__ void __launch_bounds__(kRowWarps * 32) k_row_nodes(int64_t n, const int32_t* __restrict__ conn,
                                                              const int32_t* __restrict__ ne_ptr,
                                                              const int32_t* __restrict__ ne_list, int32_t* rows,
                                                              int32_t* len, int* status) {
    __shared__ int32_t buf[kRowWarps][kMaxCand];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int32_t* b = buf[w];
    const int64_t nwarps = int64_t(gridDim.x) * kRowWarps;
    for (int64_t i = int64_t(blockIdx.x) * kRowWarps + w; i < n; i += nwarps) {
        const int32_t k0 = ne_ptr[i], k1 = ne_ptr[i + 1];
        const int m = 8 * (k1 - k0);
        if (m > kMaxCand) {
            if (lane == 0) {
                atomicOr(status, 1);
                len[i] = 0;
            }
            continue;
        }
        int p2 = 32;
        while (p2 < m) p2 <<= 1;
        for (int j = lane; j < p2; j += 32)
            b[j] = j < m ? __ldg(conn + 8 * int64_t(ne_list[k0 + (j >> 3)] >> 3) + (j & 7)) : INT_MAX;
        __syncwarp();
        // bitonic sort of b[0 .. p2)
        for (int size = 2; size <= p2; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int j = lane; j < p2; j += 32) {
                    const int partner = j ^ stride;
                    if (partner > j) {
                        const bool up = (j & size) == 0;
                        const int32_t x = b[j], y = b[partner];
                        if ((x > y) == up) {
                            b[j] = y;
                            b[partner] = x;
                        }
                    }
                }
                __syncwarp();
            }
        }
        // keep the distinct values, in order
        int32_t* out = rows + 8 * int64_t(k0);
        int written = 0;
        for (int base = 0; base < m; base += 32) {
            const int j = base + lane;
            const bool keep = j < m && (j == 0 || b[j] != b[j - 1]);
            const unsigned mask = __ballot_sync(0xffffffffu, keep);
            if (keep) out[written + __popc(mask & ((1u << lane) - 1u))] = b[j];
            written += __popc(mask);
        }
        if (lane == 0) len[i] = written;
        __syncwarp();
    }
}

__global__ void k_compact_rows(int64_t n, const int32_t* __restrict__ ne_ptr, const int32_t* __restrict__ rows,
                               const int32_t* __restrict__ indptr, int32_t* indices) {
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = (int64_t(gridDim.x) * blockDim.x) >> 5;
    for (int64_t i = warp0; i < n; i += nw) {
        const int32_t* src = rows + 8 * int64_t(ne_ptr[i]);
        const int32_t s = indptr[i], L = indptr[i + 1] - s;
        for (int l = lane; l < L; l += 32) indices[s + l] = src[l];
    }
}

// ne_inv[e*8+a] = k; slot_map[8k+b] = slot of conn[e][b] in row conn[e][a].  status bit 4:
// a pair is missing from the pattern or a row has more than 256 blocks.
__global__ void k_gather_map(int64_t n8, const int32_t* __restrict__ conn, const int32_t* __restrict__ ne_list,
                             const int32_t* __restrict__ indptr, const int32_t* __restrict__ indices, int32_t* ne_inv,
                             uint8_t* slot_map, int* status) {
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n8; k += int64_t(gridDim.x) * blockDim.x) {
        const int32_t ent = ne_list[k];
        ne_inv[ent] = int32_t(k);
        const int64_t e = ent >> 3;
        const int32_t row = conn[ent];
        const int32_t s = indptr[row], L = indptr[row + 1] - s;
        for (int b = 0; b < 8; ++b) {
            const int32_t col = conn[8 * e + b];
            int lo = 0, hi = L;  // first position with indices >= col
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (indices[s + mid] < col) lo = mid + 1;
                else hi = mid;
            }
            const bool ok = lo < L && indices[s + lo] == col && lo <= 255;
            if (!ok) atomicOr(status, 4);
            slot_map[8 * k + b] = ok ? uint8_t(lo) : uint8_t(0);
        }
    }
}

__global__ void k_check_conn(int64_t n8, int64_t n_node, const int32_t* __restrict__ conn, int* status) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n8; i += int64_t(gridDim.x) * blockDim.x)
        if (conn[i] < 0 || conn[i] >= n_node) atomicOr(status, 8);
}

struct TopoWs {
    size_t status, cnt, tiles, rows, len, total;
};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

TopoWs topo_layout(int64_t n_node, int64_t n_elem) {
    TopoWs L{};
    size_t off = 0;
    auto take = [&](size_t b) {
        const size_t o = off;
        off += align256(b);
        return o;
    };
    L.status = take(sizeof(int) * 4);
    L.cnt = take(sizeof(int32_t) * size_t(n_node + 1));
    L.tiles = take(sizeof(int64_t) * size_t((n_node + kScanTile) / kScanTile + 1));
    L.rows = take(sizeof(int32_t) * size_t(64) * size_t(n_elem));
    L.len = take(sizeof(int32_t) * size_t(n_node + 1));
    L.total = off;
    return L;
}

unsigned grid_for(int64_t work, int threads) {
    return unsigned(std::max<int64_t>(1, std::min<int64_t>((work + threads - 1) / threads, int64_t(1) << 20)));
}

int exclusive_scan(int64_t n, const int32_t* cnt, int32_t* out, int64_t* tiles, int* status, cudaStream_t st) {
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    if (ntiles > 0) {
        k_scan_tiles<<<unsigned(ntiles), kScanThreads, 0, st>>>(n, cnt, out, tiles);
        FEM_LAUNCH_CHECK("k_scan_tiles");
    }
    k_scan_sums<<<1, kScanThreads, 0, st>>>(ntiles, tiles, out, n, status);
    FEM_LAUNCH_CHECK("k_scan_sums");
    if (n > 0) {
        k_scan_add<<<grid_for(n, 256), 256, 0, st>>>(n, tiles, out);
        FEM_LAUNCH_CHECK("k_scan_add");
    }
    return FEM_OK;
}

int read_status(const int* d_status, cudaStream_t st, int& h) {
    FEM_CUDA(cudaMemcpyAsync(&h, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    FEM_CUDA(cudaStreamSynchronize(st));
    return FEM_OK;
}

}  // namespace

int device_exclusive_scan(int64_t n, const int32_t* cnt, int32_t* out, int64_t* tiles, int* status, cudaStream_t st) {
    return exclusive_scan(n, cnt, out, tiles, status, st);
}
int64_t device_scan_tiles(int64_t n) { return std::max<int64_t>(1, (n + kScanTile - 1) / kScanTile); }

}  // namespace fem

using namespace fem;

extern "C" size_t fem_topology_workspace_bytes(int64_t n_node, int64_t n_elem) {
    if (n_node < 0 || n_elem < 0) return 0;
    return topo_layout(n_node, n_elem).total;
}

extern "C" int fem_topology_count_gpu(int64_t n_node, int64_t n_elem, const int32_t* conn, int32_t* ne_ptr,
                                      int32_t* ne_list, int32_t* co_elem, int32_t* indptr, int64_t* nnzb,
                                      void* workspace, size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(n_node >= 0 && n_elem >= 0, "negative size");
    FEM_REQUIRE(n_node < (int64_t(1) << 31) - 1 && n_elem < (int64_t(1) << 28), "mesh too large for int32 indices");
    FEM_REQUIRE(nnzb != nullptr, "nnzb is NULL");
    FEM_REQUIRE(ne_ptr && indptr && (n_elem == 0 || (conn && ne_list)), "NULL argument");
    const TopoWs L = topo_layout(n_node, n_elem);
    if (!workspace || workspace_bytes < L.total) {
        set_error("workspace too small: need %zu bytes", L.total);
        return FEM_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    int* status = reinterpret_cast<int*>(ws + L.status);
    int32_t* cnt = reinterpret_cast<int32_t*>(ws + L.cnt);
    int64_t* tiles = reinterpret_cast<int64_t*>(ws + L.tiles);
    int32_t* rows = reinterpret_cast<int32_t*>(ws + L.rows);
    int32_t* len = reinterpret_cast<int32_t*>(ws + L.len);
    const int64_t n8 = 8 * n_elem;
    FEM_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * 4, st));
    FEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * size_t(n_node + 1), st));
    if (n8) {
        k_check_conn<<<grid_for(n8, 256), 256, 0, st>>>(n8, n_node, conn, status);
        FEM_LAUNCH_CHECK("k_check_conn");
        int h = 0;
        int rc = read_status(status, st, h);
        if (rc) return rc;
        FEM_REQUIRE(!(h & 8), "conn holds a node index outside [0, n_node)");
        k_count_corners<<<grid_for(n8, 256), 256, 0, st>>>(n8, conn, cnt);
        FEM_LAUNCH_CHECK("k_count_corners");
    }
    int rc = exclusive_scan(n_node, cnt, ne_ptr, tiles, status, st);
    if (rc) return rc;
    FEM_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * size_t(n_node + 1), st));
    if (n8) {
        k_scatter_corners<<<grid_for(n8, 256), 256, 0, st>>>(n8, conn, ne_ptr, cnt, ne_list);
        FEM_LAUNCH_CHECK("k_scatter_corners");
    }
    if (n_node) {
        k_sort_incidence<<<grid_for(n_node, 128), 128, 0, st>>>(n_node, ne_ptr, ne_list, co_elem);
        FEM_LAUNCH_CHECK("k_sort_incidence");
        k_row_nodes<<<grid_for(n_node, kRowWarps), kRowWarps * 32, 0, st>>>(n_node, conn, ne_ptr, ne_list, rows, len,
                                                                             status);
        FEM_LAUNCH_CHECK("k_row_nodes");
    }
    rc = exclusive_scan(n_node, len, indptr, tiles, status, st);
    if (rc) return rc;
    int h = 0;
    rc = read_status(status, st, h);
    if (rc) return rc;
    FEM_REQUIRE(!(h & 1), "a node touches more than %d elements (use the host pattern build)", kMaxCand / 8);
    FEM_REQUIRE(!(h & 2), "nnzb exceeds int32 range");
    int32_t total = 0;
    FEM_CUDA(cudaMemcpyAsync(&total, indptr + n_node, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    FEM_CUDA(cudaStreamSynchronize(st));
    *nnzb = total;
    return FEM_OK;
}

extern "C" int fem_topology_fill_gpu(int64_t n_node, int64_t n_elem, const int32_t* conn, const int32_t* ne_ptr,
                                     const int32_t* ne_list, const int32_t* indptr, int32_t* indices, int32_t* ne_inv,
                                     uint8_t* slot_map, void* workspace, size_t workspace_bytes, void* stream) {
    FEM_REQUIRE(n_node >= 0 && n_elem >= 0, "negative size");
    FEM_REQUIRE(ne_ptr && indptr && (n_elem == 0 || (conn && ne_list && indices)), "NULL argument");
    const TopoWs L = topo_layout(n_node, n_elem);
    if (!workspace || workspace_bytes < L.total) {
        set_error("workspace too small: need %zu bytes", L.total);
        return FEM_ERR_WORKSPACE;
    }
    cudaStream_t st = as_stream(stream);
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    int* status = reinterpret_cast<int*>(ws + L.status);
    const int32_t* rows = reinterpret_cast<const int32_t*>(ws + L.rows);
    if (n_node) {
        k_compact_rows<<<grid_for(n_node * 32, 256), 256, 0, st>>>(n_node, ne_ptr, rows, indptr, indices);
        FEM_LAUNCH_CHECK("k_compact_rows");
    }
    const int64_t n8 = 8 * n_elem;
    if (n8 && ne_inv && slot_map) {
        FEM_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
        k_gather_map<<<grid_for(n8, 256), 256, 0, st>>>(n8, conn, ne_list, indptr, indices, ne_inv, slot_map, status);
        FEM_LAUNCH_CHECK("k_gather_map");
        int h = 0;
        int rc = read_status(status, st, h);
        if (rc) return rc;
        if (h & 4) {
            set_error("an element node pair is missing from the pattern, or a block row has more than 256 blocks");
            return FEM_ERR_PATTERN;
        }
    }
    return FEM_OK;
}
