// Shared helpers for the sm_103a hex8 kernels: status/error plumbing and constants.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>

#include "../../include/fem_gb300.h"

namespace fem {

// Thread-local message behind fem_last_error().
void set_error(const char* fmt, ...);

inline int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return FEM_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return FEM_ERR_CUDA;
}

#define FEM_CUDA(call)                                              \
    do {                                                            \
        int _rc = ::fem::cuda_status((call), #call);                \
        if (_rc != FEM_OK) return _rc;                              \
    } while (0)

#define FEM_LAUNCH_CHECK(name)                                      \
    do {                                                            \
        int _rc = ::fem::cuda_status(cudaGetLastError(), name);     \
        if (_rc != FEM_OK) return _rc;                              \
    } while (0)

#define FEM_REQUIRE(cond, ...)                                      \
    do {                                                            \
        if (!(cond)) {                                              \
            ::fem::set_error(__VA_ARGS__);                          \
            return FEM_ERR_INVALID;                                 \
        }                                                           \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Exclusive scan of cnt[0..n) into out[0..n] (out[n] = total) on stream st (topology_gpu.cu).
// tiles: device scratch of device_scan_tiles(n) int64 values; bit 1 of *status (device) is
// set when the total exceeds the int32 range.
int device_exclusive_scan(int64_t n, const int32_t* cnt, int32_t* out, int64_t* tiles, int* status, cudaStream_t st);
int64_t device_scan_tiles(int64_t n);

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Gauss abscissa exactly as the reference literal (FEM_model_bsr.py:97).
constexpr double kGS1 = 0.57735026918962;

// Host-side reference constant tables (same literal expressions as the reference's
// shape_func / shape_derv, FEM_model_bsr.py:371-419), filled once per process.
struct ShapeTables {
    double dnr[8][8][3];  // [gp][node][d]
    double nr[8][8];      // [gp][node]
};
const ShapeTables& shape_tables();

// Kernel-parameter copy of the tables (passed by value, staged into shared memory).
struct DevTables {
    double dnr[8][8][3];
    double nr[8][8];
};
inline DevTables make_tables() {
    const ShapeTables& t = shape_tables();
    DevTables d;
    for (int g = 0; g < 8; ++g)
        for (int a = 0; a < 8; ++a) {
            d.nr[g][a] = t.nr[g][a];
            for (int k = 0; k < 3; ++k) d.dnr[g][a][k] = t.dnr[g][a][k];
        }
    return d;
}

// Upper-triangular node-pair numbering (a <= b), row-major: 36 pairs per element.
__host__ __device__ constexpr int pair_index(int a, int b) {
    return a * 8 - (a * (a - 1)) / 2 + (b - a);
}

}  // namespace fem
