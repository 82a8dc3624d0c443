// Shared internals of the sm_103a hot-path library (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ssp_gb300.h"

namespace ssp {

// Device-side error word: kernels that detect an out-of-range index or a non-finite input
// OR a code into it and skip the access instead of trapping.  Read (and cleared) by
// ssp_device_status().
extern __device__ int g_device_status;

__device__ __forceinline__ void flag(int code) { atomicOr(&g_device_status, code); }

// Fire-and-forget FP64 add into global memory (a reduction, not an atomic that returns the old
// value), so a scattering warp does not wait for each add to complete.
__device__ __forceinline__ void red_add(double *p, double v) {
    asm volatile("red.relaxed.gpu.global.add.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int launch_status() {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SSP_OK : SSP_ERR_CUDA;
}

inline unsigned grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return static_cast<unsigned>(g);
}

// Voigt bookkeeping.  Strains are engineering ([11,22,33,12,23,13] in 3D, [11,22,12] in 2D);
// tangents are stored column-major per point, entry (i, j) at i + n_strain * j.
//
// B^T rows: for a local dof alpha = dim*node + comp, the strain rows it touches and which
// gradient component multiplies each.  3D comp 0 -> rows {0, 3, 5} with (dx, dy, dz);
// comp 1 -> rows {3, 1, 4} with (dx, dy, dz); comp 2 -> rows {5, 4, 2} with (dx, dy, dz).
// 2D comp 0 -> rows {0, 2} with (dx, dy); comp 1 -> rows {2, 1} with (dx, dy).
// The tables are packed one entry per 4-bit nibble into a constant, so a runtime index costs a
// shift and a mask (an indexed local array would live in local memory).
__host__ __device__ __forceinline__ int bt_row3(int comp, int grad) {
    // grad 0 = d/dx, 1 = d/dy, 2 = d/dz; entries {0,3,5, 3,1,4, 5,4,2}
    return static_cast<int>((0x245413530ull >> (4 * (comp * 3 + grad))) & 0xFull);
}
__host__ __device__ __forceinline__ int bt_row2(int comp, int grad) {
    // entries {0,2, 2,1}
    return static_cast<int>((0x1220u >> (4 * (comp * 2 + grad))) & 0xFu);
}

// Mixed-precision plastic-correction tangent of 3D P4 elements on the tensor cores (tangent_tc.cu).
int correction_tc_p4(const double *d1, const double *d2, const double *d3, const double *DS, const double *w,
                     const int8_t *branch, const double *shear, const double *lame, const int32_t *emap, int n_elem,
                     long long nnz, double scale, double *values, cudaStream_t st);

}  // namespace ssp
