// Mohr–Coulomb potential energy density at every quadrature point and its weighted sum over the
// points: the scalar J(U) = ∫Ψ(ε(U)) that the direct SSR continuation differences in λ
// (src/slope_stability/continuation/omega.py:61,83 through ConstitutiveOperator.potential_energy,
// src/slope_stability/constitutive/problem.py:2148-2157).
//
// Per point the formulas are the reference's potential_3D (problem.py:1111-1190) and
// potential_2D (problem.py:1029-1108), with what their NumPy code computes kept as computed:
//   * 3D: the invariants read E's rows 3, 4, 5 as the tensor entries (12), (13), (23) with the
//     engineering shears unhalved (E is ordered [11,22,33,12,23,13]);
//   * 2D: the sorted eigenvalue arrays alias the unsorted ones, so where the in-plane eigenvalues
//     straddle the out-of-plane zero (e_a >= 0 > e_b) the sorted triple is (e_a, 0, 0) and where
//     both are negative it is (0, 0, 0).
// Comparisons are written as the NumPy masks are (a NaN fails every test and lands on the apex).
//
// The sum is deterministic: a fixed grid of at most SSP_POTENTIAL_PARTIALS blocks writes one
// partial each (in-block tree), and one block adds the partials in a fixed tree.

#include "ssp_internal.cuh"

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ double np_maximum(double floor_value, double x) {
    // np.maximum(floor, x): NaN propagates
    return isnan(x) ? x : (x > floor_value ? x : floor_value);
}

__device__ __forceinline__ double safe_denominator(double d) {
    // np.where(|d| < 1e-15, sign(d + 1e-15) * 1e-15, d)
    if (fabs(d) < 1.0e-15) {
        const double t = d + 1.0e-15;
        return (t > 0.0 ? 1.0e-15 : (t < 0.0 ? -1.0e-15 : 0.0));
    }
    return d;
}

// Branch selection and energy of one point from its sorted principal strains (e1 >= e2 >= e3 in
// the regular case), trace, reduced strength and moduli, and the three dimension-specific
// denominators.  Returns the branch code (0 elastic, 1 smooth, 2 left edge, 3 right edge, 4 apex).
__device__ __forceinline__ int mc_potential(double e1, double e2, double e3, double tr, double c, double s, double G,
                                            double K, double L, double d_s, double d_l, double d_r, double &psi) {
    const double f_tr = 2.0 * G * ((1.0 + s) * e1 - (1.0 - s) * e3) + 2.0 * (L * s) * tr - c;
    const double g_sl = (e1 - e2) / np_maximum(1.0e-15, 1.0 + s);
    const double g_sr = (e2 - e3) / np_maximum(1.0e-15, 1.0 - s);
    const double g_la = (e1 + e2 - 2.0 * e3) / np_maximum(1.0e-15, 3.0 - s);
    const double g_ra = (2.0 * e1 - e2 - e3) / np_maximum(1.0e-15, 3.0 + s);
    const double vol = 0.5 * L * tr * tr;
    if (f_tr <= 0.0) {
        psi = vol + G * (e1 * e1 + e2 * e2 + e3 * e3);
        return 0;
    }
    const double l_s = f_tr / safe_denominator(d_s);
    if (l_s <= g_sl && l_s <= g_sr) {  // lambda_s <= np.minimum(g_sl, g_sr), NaN-failing
        psi = vol + G * (e1 * e1 + e2 * e2 + e3 * e3) - 0.5 * d_s * (l_s * l_s);
        return 1;
    }
    const double lin = 2.0 * L * s * tr - c;
    if (g_sl < g_sr) {
        const double l_l = (G * ((1.0 + s) * (e1 + e2) - 2.0 * (1.0 - s) * e3) + lin) / safe_denominator(d_l);
        if (l_l >= g_sl && l_l <= g_la) {
            const double h = e1 + e2;
            psi = vol + G * (e3 * e3 + 0.5 * (h * h)) - 0.5 * d_l * (l_l * l_l);
            return 2;
        }
    }
    if (g_sl > g_sr) {
        const double l_r = (G * (2.0 * (1.0 + s) * e1 - (1.0 - s) * (e2 + e3)) + lin) / safe_denominator(d_r);
        if (l_r >= g_sr && l_r <= g_ra) {
            const double h = e2 + e3;
            psi = vol + G * (e1 * e1 + 0.5 * (h * h)) - 0.5 * d_r * (l_r * l_r);
            return 3;
        }
    }
    const double d_a = 4.0 * K * (s * s);
    const double l_a = (2.0 * K * s * tr - c) / safe_denominator(d_a);
    psi = 0.5 * K * tr * tr - 0.5 * d_a * (l_a * l_a);
    return 4;
}

template <int DIM>
__device__ __forceinline__ int point_potential(const double *__restrict__ E, double c, double s, double G, double K,
                                               double L, double &psi) {
    const double s2 = s * s;
    if (DIM == 3) {
        const double e11 = E[0], e22 = E[1], e33 = E[2], r3 = E[3], r4 = E[4], r5 = E[5];
        const double I1 = e11 + e22 + e33;
        const double I2 = e11 * e22 + e11 * e33 + e22 * e33 - r3 * r3 - r4 * r4 - r5 * r5;
        const double I3 = e11 * e22 * e33 - e33 * r3 * r3 - e22 * r4 * r4 - e11 * r5 * r5 + 2.0 * r3 * r4 * r5;
        const double Q = np_maximum(0.0, (I1 * I1 - 3.0 * I2) / 9.0);
        const double R = (-2.0 * (I1 * I1 * I1) + 9.0 * I1 * I2 - 27.0 * I3) / 54.0;
        double theta = 0.0;
        if (Q > 0.0) {
            double t = R / np_maximum(1.0e-15, sqrt(Q * Q * Q));
            t = t < -1.0 ? -1.0 : (t > 1.0 ? 1.0 : t);
            theta = acos(t) / 3.0;
        }
        const double rq = sqrt(Q);
        const double third = I1 / 3.0;
        const double two_pi_3 = 2.0 * 3.14159265358979323846 / 3.0;
        const double e1 = -2.0 * rq * cos(theta + two_pi_3) + third;
        const double e2 = -2.0 * rq * cos(theta - two_pi_3) + third;
        const double e3 = -2.0 * rq * cos(theta) + third;
        const double d_s = 4.0 * L * s2 + 4.0 * G * (1.0 + s2);
        const double d_l = 4.0 * L * s2 + G * (1.0 + s) * (1.0 + s) + 2.0 * G * (1.0 - s) * (1.0 - s);
        const double d_r = 4.0 * L * s2 + 2.0 * G * (1.0 + s) * (1.0 + s) + G * (1.0 - s) * (1.0 - s);
        return mc_potential(e1, e2, e3, I1, c, s, G, K, L, d_s, d_l, d_r, psi);
    } else {
        const double e11 = E[0], e22 = E[1], g12 = E[2];
        const double tr2 = e11 + e22;
        const double dd = e11 - e22;
        const double rad = sqrt(dd * dd + g12 * g12);
        const double ea = (tr2 + rad) / 2.0, eb = (tr2 - rad) / 2.0;
        const bool straddle = (ea >= 0.0) && (0.0 > eb);
        const bool negative = 0.0 > ea;
        const double e1 = negative ? 0.0 : ea;
        const double e2 = (straddle || negative) ? 0.0 : eb;
        const double e3 = 0.0;
        const double tr = e1 + e2 + e3;
        const double ps = (1.0 + s) * (1.0 + s), ms = (1.0 - s) * (1.0 - s);
        const double d_s = 4.0 * L * s2 + 2.0 * G * ps + 2.0 * G * ms;
        const double d_l = 4.0 * L * s2 + G * ps + 2.0 * G * ms;
        const double d_r = 4.0 * L * s2 + 2.0 * G * ps + G * ms;
        return mc_potential(e1, e2, e3, tr, c, s, G, K, L, d_s, d_l, d_r, psi);
    }
}

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    v = 0.0;
    if (warp == 0) {
        v = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;  // valid in thread 0
}

template <int DIM>
__global__ void __launch_bounds__(kBlock) potential_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                           const double *__restrict__ sin_phi,
                                                           const double *__restrict__ shear,
                                                           const double *__restrict__ bulk,
                                                           const double *__restrict__ lame,
                                                           const double *__restrict__ weight, int n, double *psi_out,
                                                           int8_t *branch_out, double *partial) {
    __shared__ double red[kBlock / 32];
    constexpr int NS = DIM == 3 ? 6 : 3;
    double acc = 0.0;
    for (long long p = (long long)blockIdx.x * kBlock + threadIdx.x; p < n; p += (long long)gridDim.x * kBlock) {
        double e[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) e[k] = E[p * NS + k];
        double psi;
        const int b = point_potential<DIM>(e, c_bar[p], sin_phi[p], shear[p], bulk[p], lame[p], psi);
        if (psi_out) psi_out[p] = psi;
        if (branch_out) branch_out[p] = (int8_t)b;
        if (weight) acc += weight[p] * psi;
    }
    if (!partial) return;
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(1024) potential_total_kernel(const double *__restrict__ partial, int count,
                                                               double *total) {
    __shared__ double red[32];
    double v = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) v += partial[i];
    v = block_sum(v, red);
    if (threadIdx.x == 0) *total = v;
}

}  // namespace

using namespace ssp;

extern "C" {

int ssp_potential_energy(int dim, const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                         const double *bulk, const double *lame, const double *weight, int n_int, double *psi_out,
                         int8_t *branch_out, double *partial, double *total_out, void *stream) {
    if (dim != 2 && dim != 3) return SSP_ERR_INVALID;
    if (n_int < 0) return SSP_ERR_INVALID;
    if (total_out && (!weight || !partial)) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    const int blocks = n_int == 0 ? 0 : (int)((n_int + kBlock - 1) / kBlock < SSP_POTENTIAL_PARTIALS
                                                  ? (n_int + kBlock - 1) / kBlock
                                                  : SSP_POTENTIAL_PARTIALS);
    if (blocks > 0) {
        if (!E || !c_bar || !sin_phi || !shear || !bulk || !lame) return SSP_ERR_INVALID;
        const double *w = total_out ? weight : nullptr;
        double *part = total_out ? partial : nullptr;
        if (dim == 3)
            potential_kernel<3><<<blocks, kBlock, 0, st>>>(E, c_bar, sin_phi, shear, bulk, lame, w, n_int, psi_out,
                                                           branch_out, part);
        else
            potential_kernel<2><<<blocks, kBlock, 0, st>>>(E, c_bar, sin_phi, shear, bulk, lame, w, n_int, psi_out,
                                                           branch_out, part);
    }
    if (total_out) potential_total_kernel<<<1, 1024, 0, st>>>(partial, blocks, total_out);
    return launch_status();
}

}  // extern "C"
