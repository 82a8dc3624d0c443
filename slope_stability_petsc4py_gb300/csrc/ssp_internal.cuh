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

// The binned 3D return mapping (constitutive.cu).  scratch: counters at scratch[0..3] (listed,
// smooth, left edge, right edge), the listed points from scratch + 4, the smooth list from
// scratch + 4 + n_int, the edge lists from scratch + 4 + 2 n_int.
// Pass A: zero the counters, screen every point, finish the screened ones, list the others
// (write_elastic_ds = false: the DS rows of the screened points are left unwritten).
int binned_screen(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                  const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                  cudaStream_t st, bool write_elastic_ds = true);
// Passes B and C: decide the points of n_lists lists (list k: counts[k] entries from
// lists + k list_stride), finish elastic and apex points, record and list the others by branch,
// finish those (compensated_ds: the plastic DS in double-float arithmetic).
int binned_decide_finish(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                         const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                         int32_t *scratch, const int32_t *lists, const int32_t *counts, int n_lists,
                         long long list_stride, bool compensated_ds, cudaStream_t st);

// Mixed-precision plastic-correction tangent of 3D P4 elements on the tensor cores (tangent_tc.cu).
int correction_tc_p4(const double *d1, const double *d2, const double *d3, const double *DS, const double *w,
                     const int8_t *branch, const double *shear, const double *lame, const int32_t *emap, int n_elem,
                     long long nnz, double scale, double *values, const int32_t *elist, const int32_t *elist_count,
                     cudaStream_t st);

}  // namespace ssp

namespace ssp {

// ---------------------------------------------------------------------------------------------
// Double-float arithmetic on the FP32 pipe (a value is an unevaluated sum hi + lo of two floats,
// about 48 significant bits).  GB300 issues FP64 at a small fraction of the FP32 rate, so the
// mixed-precision kernels form their compensated products this way.  Error-free transformations
// after Knuth (TwoSum) and Dekker (TwoProduct, here with a fused multiply-add), in the form of
// Hida, Li and Bailey's double-double library.  Conversions to and from FP64 use integer bit
// operations only, so they take no FP64 issue slots.

struct df32 {
    float hi, lo;
};

__device__ __forceinline__ df32 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ df32 df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
    df32 s = df_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df32 df_add_f(df32 a, float b) {
    df32 s = df_two_sum(a.hi, b);
    s.lo = __fadd_rn(s.lo, a.lo);
    return df_fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_fast_two_sum(p, e);
}
// a + b * c
__device__ __forceinline__ df32 df_fma(df32 a, df32 b, df32 c) { return df_add(a, df_mul(b, c)); }
// a0 b0 + a1 b1 + a2 b2 as a compensated dot product (Ogita, Rump and Oishi's Dot2 on the hi
// parts, with the hi*lo cross terms and the rounding errors gathered in one float).
__device__ __forceinline__ df32 df_dot3(df32 a0, df32 b0, df32 a1, df32 b1, df32 a2, df32 b2) {
    const float p0 = __fmul_rn(a0.hi, b0.hi), p1 = __fmul_rn(a1.hi, b1.hi), p2 = __fmul_rn(a2.hi, b2.hi);
    float e = __fmaf_rn(a0.hi, b0.hi, -p0);
    e = __fadd_rn(e, __fmaf_rn(a1.hi, b1.hi, -p1));
    e = __fadd_rn(e, __fmaf_rn(a2.hi, b2.hi, -p2));
    const df32 s1 = df_two_sum(p0, p1);
    const df32 s2 = df_two_sum(s1.hi, p2);
    e = __fadd_rn(e, __fadd_rn(s1.lo, s2.lo));
    e = __fmaf_rn(a0.hi, b0.lo, __fmaf_rn(a0.lo, b0.hi, e));
    e = __fmaf_rn(a1.hi, b1.lo, __fmaf_rn(a1.lo, b1.hi, e));
    e = __fmaf_rn(a2.hi, b2.lo, __fmaf_rn(a2.lo, b2.hi, e));
    return df_fast_two_sum(s2.hi, e);
}

// FP64 -> hi + lo: hi = x truncated to 24 significant bits, lo = the remaining 29 bits rounded to
// a float.  Integer operations and one integer->float conversion only.  Zero, FP64 values below
// the FP32 normal range and non-finite values give (0, 0), (0, 0) and (+-inf or nan, 0); lo is
// flushed to 0 when it would be subnormal (|x| < 2^-73), where hi alone keeps 2^-24.
__device__ __forceinline__ df32 df_from_f64(double x) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned sign = static_cast<unsigned>(u >> 32) & 0x80000000u;
    const int e = static_cast<int>((u >> 52) & 0x7FFull);
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return {__uint_as_float(sign | 0x7F800000u | (m ? 0x400000u : 0u)), 0.0f};
    const int ef = e - 1023 + 127;  // biased FP32 exponent
    if (ef <= 0) return {__uint_as_float(sign), 0.0f};
    if (ef >= 255) return {__uint_as_float(sign | 0x7F800000u), 0.0f};
    const float hi = __uint_as_float(sign | (static_cast<unsigned>(ef) << 23) | static_cast<unsigned>(m >> 29));
    const unsigned r = static_cast<unsigned>(m & 0x1FFFFFFFull);  // 29 bits below hi
    // lo = r * 2^(e - 1023 - 52); the power of two as a float when it is normal
    const int es = e - 1023 - 52 + 127;
    float lo = 0.0f;
    if (r != 0u && es > 0) lo = __uint2float_rn(r) * __uint_as_float(static_cast<unsigned>(es) << 23);
    return {hi, sign ? -lo : lo};
}
// Exact float -> double by bit operations (subnormal floats flush to a signed zero).
__device__ __forceinline__ double f32_widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
    if (e == 0u) return __longlong_as_double(static_cast<long long>(sign));
    const unsigned long long ed = e == 0xFFu ? 0x7FFull : static_cast<unsigned long long>(e + 896u);
    return __longlong_as_double(
        static_cast<long long>(sign | (ed << 52) | (static_cast<unsigned long long>(u & 0x7FFFFFu) << 29)));
}
// hi + lo as one double (one FP64 add).
__device__ __forceinline__ double df_to_f64(df32 a) { return f32_widen(a.hi) + f32_widen(a.lo); }

// Compensated accumulator: value = s + c, s accumulates the leading parts with TwoSum, c the
// rounding errors and the low-order product terms (about 2^-48 of the sum of |terms|).
struct CSum {
    float s = 0.0f, c = 0.0f;
    __device__ __forceinline__ void add_prod(df32 x, df32 y) {
        const float p = __fmul_rn(x.hi, y.hi);
        float e = __fmaf_rn(x.hi, y.hi, -p);
        e = __fmaf_rn(x.hi, y.lo, __fmaf_rn(x.lo, y.hi, e));
        const df32 t = df_two_sum(s, p);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, e));
    }
    __device__ __forceinline__ void add(df32 x) {
        const df32 t = df_two_sum(s, x.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, x.lo));
    }
    __device__ __forceinline__ double value() const { return df_to_f64(df_fast_two_sum(s, c)); }
    __device__ __forceinline__ df32 df() const { return df_fast_two_sum(s, c); }
};

}  // namespace ssp
