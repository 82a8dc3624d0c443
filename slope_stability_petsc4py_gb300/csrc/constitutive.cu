// Mohr-Coulomb return mapping with consistent tangent, one thread per integration point.
//
// 3D follows src/slope_stability/cython/constitutive_3D_kernel.h:68-351 (the production C
// kernel, batched by constitutive_3d_batch.c:9-50); 2D follows the NumPy plane-strain operator
// src/slope_stability/constitutive/problem.py:143-475.  Strength reduction follows
// src/slope_stability/constitutive/reduction.py:14-78.
//
// GB300 notes.  FP64 on this part issues at a small fraction of the FP32 rate, so the
// kernels minimise double-precision work: the tangent is evaluated on its upper triangle
// only and mirrored (the return mapping is associated, sin(psi) = sin(phi), so DS is
// symmetric; the mirrored entries are bitwise equal to what the full evaluation gives
// because every term is a commutative product/sum of the same operands), and the branch is
// decided before any tangent work starts.
#include <math.h>

#include "ssp_internal.cuh"

namespace ssp {

__device__ int g_device_status = 0;

namespace {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ double vol_iota(int i) { return i < 3 ? 1.0 : 0.0; }
__device__ __forceinline__ double half_ident(int i) { return i < 3 ? 1.0 : 0.5; }

// Branch codes shared with the learned branch proposal (ssp_branch_*).
enum Branch : int { kElastic = 0, kSmooth = 1, kLeft = 2, kRight = 3, kApex = 4 };

struct Principal3 {
    double t[6], sq[6];
    double I1, e1, e2, e3;
};

__device__ __forceinline__ void principal3(const double *E, Principal3 &p) {
#pragma unroll
    for (int i = 0; i < 6; ++i) p.t[i] = half_ident(i) * E[i];
    const double *t = p.t;
    p.sq[0] = t[0] * t[0] + t[3] * t[3] + t[5] * t[5];
    p.sq[1] = t[1] * t[1] + t[3] * t[3] + t[4] * t[4];
    p.sq[2] = t[2] * t[2] + t[4] * t[4] + t[5] * t[5];
    p.sq[3] = t[0] * t[3] + t[1] * t[3] + t[4] * t[5];
    p.sq[4] = t[3] * t[5] + t[1] * t[4] + t[2] * t[4];
    p.sq[5] = t[0] * t[5] + t[3] * t[4] + t[2] * t[5];
    const double I1 = t[0] + t[1] + t[2];
    const double I2 = t[0] * t[1] + t[0] * t[2] + t[1] * t[2] - t[3] * t[3] - t[4] * t[4] - t[5] * t[5];
    const double I3 = t[0] * t[1] * t[2] - t[2] * t[3] * t[3] - t[1] * t[5] * t[5] - t[0] * t[4] * t[4] +
                      2.0 * t[3] * t[4] * t[5];
    double Q = (I1 * I1 - 3.0 * I2) / 9.0;
    if (Q < 0.0) Q = 0.0;
    const double R = (-2.0 * I1 * I1 * I1 + 9.0 * I1 * I2 - 27.0 * I3) / 54.0;
    const double rq = sqrt(Q);
    double theta = 0.0;
    if (!(Q < 1e-30)) {
        double c = R / (rq * Q);
        c = fmin(1.0, fmax(-1.0, c));
        theta = acos(c) / 3.0;
    }
    const double third = I1 / 3.0;
    p.I1 = I1;
    p.e1 = -2.0 * rq * cos(theta + 2.0 * kPi / 3.0) + third;
    p.e2 = -2.0 * rq * cos(theta - 2.0 * kPi / 3.0) + third;
    p.e3 = -2.0 * rq * cos(theta) + third;
}

// d(t*t)_i / dE_j (symmetric), entry for i <= j only.
__device__ __forceinline__ double square_jac(const double *t, int i, int j) {
    // i <= j
    switch (i * 6 + j) {
        case 0: return 2.0 * t[0];
        case 3: return t[3];
        case 5: return t[5];
        case 7: return 2.0 * t[1];
        case 9: return t[3];
        case 10: return t[4];
        case 14: return 2.0 * t[2];
        case 16: return t[4];
        case 17: return t[5];
        case 21: return 0.5 * (t[0] + t[1]);
        case 22: return 0.5 * t[5];
        case 23: return 0.5 * t[4];
        case 28: return 0.5 * (t[1] + t[2]);
        case 29: return 0.5 * t[3];
        case 35: return 0.5 * (t[0] + t[2]);
        default: return 0.0;
    }
}

__device__ __forceinline__ void projection(const Principal3 &p, double sum_o, double prod_o, double inv, double *P) {
#pragma unroll
    for (int i = 0; i < 6; ++i) P[i] = inv * (p.sq[i] - sum_o * p.t[i] + prod_o * vol_iota(i));
}

__device__ __forceinline__ void store_sym(double *DS, int i, int j, double v) {
    DS[i + 6 * j] = v;
    DS[j + 6 * i] = v;
}

// Returns the branch code.  DS may be null (stress only).
__device__ int mc3d_point(const double *E, double c_bar, double sin_phi, double shear, double lame, double *S,
                          double *DS) {
    const double sp = sin_phi;
    Principal3 p;
    principal3(E, p);
    const double e1 = p.e1, e2 = p.e2, e3 = p.e3, I1 = p.I1;
    const double f_tr = 2.0 * shear * ((1.0 + sin_phi) * e1 - (1.0 - sin_phi) * e3) + 2.0 * lame * sin_phi * I1 - c_bar;

    if (f_tr <= 0.0) {
        const double lI1 = lame * I1, s2 = 2.0 * shear;
#pragma unroll
        for (int i = 0; i < 3; ++i) S[i] = lI1 + s2 * p.t[i];
#pragma unroll
        for (int i = 3; i < 6; ++i) S[i] = s2 * p.t[i];
        if (DS) {
#pragma unroll
            for (int k = 0; k < 36; ++k) DS[k] = 0.0;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                DS[i * 7] = s2 + lame;
                DS[(i + 3) * 7] = shear;
            }
            store_sym(DS, 0, 1, lame);
            store_sym(DS, 0, 2, lame);
            store_sym(DS, 1, 2, lame);
        }
        return kElastic;
    }

    const double g_sl = (e1 - e2) / (1.0 + sp);
    const double g_sr = (e2 - e3) / (1.0 - sp);
    const double den_s = 4.0 * lame * sin_phi * sp + 4.0 * shear * (1.0 + sin_phi * sp);
    const double lam_s = f_tr / den_s;

    if (lam_s <= g_sl && lam_s <= g_sr) {
        const double inv1 = 1.0 / ((e1 - e2) * (e1 - e3));
        const double inv2 = 1.0 / ((e2 - e1) * (e2 - e3));
        const double inv3 = 1.0 / ((e3 - e1) * (e3 - e2));
        double P1[6], P2[6], P3[6];
        projection(p, e2 + e3, e2 * e3, inv1, P1);
        projection(p, e1 + e3, e1 * e3, inv2, P2);
        projection(p, e1 + e2, e1 * e2, inv3, P3);
        const double s1 = lame * I1 + 2.0 * shear * e1 - lam_s * (2.0 * lame * sp + 2.0 * shear * (1.0 + sp));
        const double s2 = lame * I1 + 2.0 * shear * e2 - lam_s * 2.0 * lame * sp;
        const double s3 = lame * I1 + 2.0 * shear * e3 - lam_s * (2.0 * lame * sp - 2.0 * shear * (1.0 - sp));
#pragma unroll
        for (int i = 0; i < 6; ++i) S[i] = s1 * P1[i] + s2 * P2[i] + s3 * P3[i];
        if (DS) {
            double Dp[6];
#pragma unroll
            for (int i = 0; i < 6; ++i)
                Dp[i] = 2.0 * shear * ((1.0 + sin_phi) * P1[i] - (1.0 - sin_phi) * P3[i]) + 2.0 * lame * sin_phi * vol_iota(i);
            const double em23 = e2 + e3, em13 = e1 + e3, em12 = e1 + e2;
            const double c1a = 2.0 * e1 - e2 - e3, c1b = e2 - e3;
            const double c2a = 2.0 * e2 - e1 - e3, c2b = e1 - e3;
            const double c3a = 2.0 * e3 - e1 - e2, c3b = e1 - e2;
            const double inv_den = 1.0 / den_s;
#pragma unroll
            for (int j = 0; j < 6; ++j) {
#pragma unroll
                for (int i = 0; i <= j; ++i) {
                    const double idk = (i == j) ? half_ident(i) : 0.0;
                    const double jq = square_jac(p.t, i, j);
                    const double o11 = P1[i] * P1[j], o22 = P2[i] * P2[j], o33 = P3[i] * P3[j];
                    const double d1 = inv1 * (jq - idk * em23 - c1a * o11 - c1b * (o22 - o33));
                    const double d2 = inv2 * (jq - idk * em13 - c2a * o22 - c2b * (o11 - o33));
                    const double d3 = inv3 * (jq - idk * em12 - c3a * o33 - c3b * (o11 - o22));
                    const double v = s1 * d1 + s2 * d2 + s3 * d3 + lame * vol_iota(i) * vol_iota(j) +
                                     2.0 * shear * (o11 + o22 + o33) - Dp[i] * Dp[j] * inv_den;
                    store_sym(DS, i, j, v);
                }
            }
        }
        return kSmooth;
    }

    if (g_sl < g_sr) {
        const double den_l = 4.0 * lame * sin_phi * sp + shear * (1.0 + sin_phi) * (1.0 + sp) +
                             2.0 * shear * (1.0 - sin_phi) * (1.0 - sp);
        const double lam_l =
            (shear * ((1.0 + sin_phi) * (e1 + e2) - 2.0 * (1.0 - sin_phi) * e3) + 2.0 * lame * sin_phi * I1 - c_bar) / den_l;
        const double g_la = (e1 + e2 - 2.0 * e3) / (3.0 - sp);
        if (lam_l >= g_sl && lam_l <= g_la) {
            const double inv3 = 1.0 / ((e3 - e1) * (e3 - e2));
            double P3[6], P12[6];
            projection(p, e1 + e2, e1 * e2, inv3, P3);
#pragma unroll
            for (int i = 0; i < 6; ++i) P12[i] = vol_iota(i) - P3[i];
            const double s1 = lame * I1 + shear * (e1 + e2) - lam_l * (2.0 * lame * sp + shear * (1.0 + sp));
            const double s3 = lame * I1 + 2.0 * shear * e3 - lam_l * (2.0 * lame * sp - 2.0 * shear * (1.0 - sp));
#pragma unroll
            for (int i = 0; i < 6; ++i) S[i] = s1 * P12[i] + s3 * P3[i];
            if (DS) {
                double Dp[6];
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    Dp[i] = shear * ((1.0 + sin_phi) * P12[i] - 2.0 * (1.0 - sin_phi) * P3[i]) + 2.0 * lame * sin_phi * vol_iota(i);
                const double em12 = e1 + e2;
                const double inv_den = 1.0 / den_l;
#pragma unroll
                for (int j = 0; j < 6; ++j) {
#pragma unroll
                    for (int i = 0; i <= j; ++i) {
                        const double idk = (i == j) ? half_ident(i) : 0.0;
                        const double o33 = P3[i] * P3[j], oAA = P12[i] * P12[j];
                        const double d3 = inv3 * (square_jac(p.t, i, j) - idk * em12 - (P12[i] * p.t[j] + p.t[i] * P12[j]) +
                                                  em12 * oAA + (em12 - 2.0 * e3) * o33 + e3 * (P12[i] * P3[j] + P3[i] * P12[j]));
                        const double v = (s3 - s1) * d3 + lame * vol_iota(i) * vol_iota(j) + shear * (oAA + 2.0 * o33) -
                                         Dp[i] * Dp[j] * inv_den;
                        store_sym(DS, i, j, v);
                    }
                }
            }
            return kLeft;
        }
    }

    if (g_sl > g_sr) {
        const double den_r = 4.0 * lame * sin_phi * sp + 2.0 * shear * (1.0 + sin_phi) * (1.0 + sp) +
                             shear * (1.0 - sin_phi) * (1.0 - sp);
        const double lam_r =
            (shear * (2.0 * (1.0 + sin_phi) * e1 - (1.0 - sin_phi) * (e2 + e3)) + 2.0 * lame * sin_phi * I1 - c_bar) / den_r;
        const double g_ra = (2.0 * e1 - e2 - e3) / (3.0 + sp);
        if (lam_r >= g_sr && lam_r <= g_ra) {
            const double inv1 = 1.0 / ((e1 - e2) * (e1 - e3));
            double P1[6], P23[6];
            projection(p, e2 + e3, e2 * e3, inv1, P1);
#pragma unroll
            for (int i = 0; i < 6; ++i) P23[i] = vol_iota(i) - P1[i];
            const double s1 = lame * I1 + 2.0 * shear * e1 - lam_r * (2.0 * lame * sp + 2.0 * shear * (1.0 + sp));
            const double s3 = lame * I1 + shear * (e2 + e3) - lam_r * (2.0 * lame * sp - shear * (1.0 - sp));
#pragma unroll
            for (int i = 0; i < 6; ++i) S[i] = s1 * P1[i] + s3 * P23[i];
            if (DS) {
                double Dp[6];
#pragma unroll
                for (int i = 0; i < 6; ++i)
                    Dp[i] = shear * (2.0 * (1.0 + sin_phi) * P1[i] - (1.0 - sin_phi) * P23[i]) + 2.0 * lame * sin_phi * vol_iota(i);
                const double em23 = e2 + e3;
                const double inv_den = 1.0 / den_r;
#pragma unroll
                for (int j = 0; j < 6; ++j) {
#pragma unroll
                    for (int i = 0; i <= j; ++i) {
                        const double idk = (i == j) ? half_ident(i) : 0.0;
                        const double o11 = P1[i] * P1[j], oBB = P23[i] * P23[j];
                        const double d1 = inv1 * (square_jac(p.t, i, j) - idk * em23 - (P23[i] * p.t[j] + p.t[i] * P23[j]) +
                                                  em23 * oBB + (em23 - 2.0 * e1) * o11 + e1 * (P23[i] * P1[j] + P1[i] * P23[j]));
                        const double v = (s1 - s3) * d1 + lame * vol_iota(i) * vol_iota(j) + shear * (2.0 * o11 + oBB) -
                                         Dp[i] * Dp[j] * inv_den;
                        store_sym(DS, i, j, v);
                    }
                }
            }
            return kRight;
        }
    }

    const double sa = c_bar / (2.0 * sin_phi);
#pragma unroll
    for (int i = 0; i < 3; ++i) S[i] = sa;
#pragma unroll
    for (int i = 3; i < 6; ++i) S[i] = 0.0;
    if (DS) {
#pragma unroll
        for (int k = 0; k < 36; ++k) DS[k] = 0.0;
    }
    return kApex;
}

template <bool TANGENT>
__global__ void __launch_bounds__(128) mc3d_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                   const double *__restrict__ sin_phi, const double *__restrict__ shear,
                                                   const double *__restrict__ lame, int n, double *__restrict__ S,
                                                   double *__restrict__ DS, int8_t *__restrict__ branch) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    double e[6];
    const double2 *E2 = reinterpret_cast<const double2 *>(E + 6ll * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        double2 v = E2[k];
        e[2 * k] = v.x;
        e[2 * k + 1] = v.y;
    }
    double s[6];
    int b;
    if (TANGENT) {
        double ds[36];
        b = mc3d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, ds);
        double2 *D2 = reinterpret_cast<double2 *>(DS + 36ll * p);
#pragma unroll
        for (int k = 0; k < 18; ++k) D2[k] = make_double2(ds[2 * k], ds[2 * k + 1]);
    } else {
        b = mc3d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, nullptr);
    }
    double2 *S2 = reinterpret_cast<double2 *>(S + 6ll * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) S2[k] = make_double2(s[2 * k], s[2 * k + 1]);
    if (branch) branch[p] = static_cast<int8_t>(b);
}

// ---------------------------------------------------------------------------- 2D

// Plane strain, E = [e11, e22, g12] -> S = [s11, s22, s12, s33], DS 3x3 column-major.
__device__ int mc2d_point(const double *E, double c, double s, double G, double lam, double *S, double *DS) {
    const double e11 = E[0], e22 = E[1], g12 = E[2];
    const double tr2 = e11 + e22;
    const double rad = sqrt((e11 - e22) * (e11 - e22) + g12 * g12);
    const double ev0[3] = {0.5 * (tr2 + rad), 0.5 * (tr2 - rad), 0.0};
    // projections in [11, 22, 12, 33] representation and their derivatives (3x3 in-plane)
    double P0[4], P1[4];
    double dP0[9];
    if (rad != 0.0) {
        P0[0] = (e11 - ev0[1]) / rad;
        P0[1] = (e22 - ev0[1]) / rad;
        P0[2] = (g12 / 2.0) / rad;
    } else {
        P0[0] = 1.0;
        P0[1] = 1.0;
        P0[2] = 0.0;
    }
    P0[3] = 0.0;
    P1[0] = 1.0 - P0[0];
    P1[1] = 1.0 - P0[1];
    P1[2] = 0.0 - P0[2];
    P1[3] = 0.0;
    const double hI[3] = {1.0, 1.0, 0.5};
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i)
            dP0[i + 3 * j] = rad != 0.0 ? (((i == j) ? hI[i] : 0.0) - P0[i] * P0[j] - P1[i] * P1[j]) / rad : 0.0;
    // sort: (0,2,1) when ev0[0] >= 0 > ev0[1]; (2,0,1) when 0 > ev0[0]
    int ord[3] = {0, 1, 2};
    if (ev0[0] >= ev0[2] && ev0[2] > ev0[1]) {
        ord[1] = 2;
        ord[2] = 1;
    } else if (ev0[2] > ev0[0]) {
        ord[0] = 2;
        ord[1] = 0;
        ord[2] = 1;
    }
    double ev[3], P[3][4], dP[3][9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int o = ord[k];
        ev[k] = ev0[o];
#pragma unroll
        for (int i = 0; i < 4; ++i) P[k][i] = o == 0 ? P0[i] : (o == 1 ? P1[i] : (i == 3 ? 1.0 : 0.0));
#pragma unroll
        for (int i = 0; i < 9; ++i) dP[k][i] = o == 0 ? dP0[i] : (o == 1 ? -dP0[i] : 0.0);
    }
    const double e1 = ev[0], e2 = ev[1], e3 = ev[2];
    const double tr = e1 + e2 + e3;
    const double f_tr = 2.0 * G * ((1.0 + s) * e1 - (1.0 - s) * e3) + 2.0 * lam * s * tr - c;
    const double io[3] = {1.0, 1.0, 0.0};
    if (f_tr <= 0.0) {
        const double vt = e11 + e22;  // iota4 . [e11, e22, g12, 0]
        S[0] = lam * vt + 2.0 * G * e11;
        S[1] = lam * vt + 2.0 * G * e22;
        S[2] = 2.0 * G * (0.5 * g12);
        S[3] = lam * vt;
        if (DS) {
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i) DS[i + 3 * j] = io[i] * io[j] * lam + 2.0 * ((i == j) ? hI[i] : 0.0) * G;
        }
        return kElastic;
    }
    const double g_sl = (e1 - e2) / (1.0 + s);
    const double g_sr = (e2 - e3) / (1.0 - s);
    const double g_la = (e1 + e2 - 2.0 * e3) / (3.0 - s);
    const double g_ra = (2.0 * e1 - e2 - e3) / (3.0 + s);
    const double d_s = 4.0 * lam * s * s + 2.0 * G * (1.0 + s) * (1.0 + s) + 2.0 * G * (1.0 - s) * (1.0 - s);
    const double l_s = f_tr / d_s;
    if (l_s <= fmin(g_sl, g_sr)) {
        const double s1 = lam * tr + 2.0 * G * e1 - l_s * (2.0 * lam * s + 2.0 * G * (1.0 + s));
        const double s2 = lam * tr + 2.0 * G * e2 - l_s * (2.0 * lam * s);
        const double s3 = lam * tr + 2.0 * G * e3 - l_s * (2.0 * lam * s - 2.0 * G * (1.0 - s));
#pragma unroll
        for (int i = 0; i < 4; ++i) S[i] = s1 * P[0][i] + s2 * P[1][i] + s3 * P[2][i];
        if (DS) {
            double q6[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) q6[i] = 2.0 * G * (1.0 + s) * P[0][i] - 2.0 * G * (1.0 - s) * P[2][i] + io[i] * (2.0 * lam * s);
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    DS[i + 3 * j] = s1 * dP[0][i + 3 * j] + s2 * dP[1][i + 3 * j] + s3 * dP[2][i + 3 * j] + io[i] * io[j] * lam +
                                    2.0 * G * (P[0][i] * P[0][j] + P[1][i] * P[1][j] + P[2][i] * P[2][j]) - q6[i] * q6[j] / d_s;
        }
        return kSmooth;
    }
    const double d_l = 4.0 * lam * s * s + G * (1.0 + s) * (1.0 + s) + 2.0 * G * (1.0 - s) * (1.0 - s);
    const double l_l = (G * ((1.0 + s) * (e1 + e2) - 2.0 * (1.0 - s) * e3) + 2.0 * lam * s * tr - c) / d_l;
    if (g_sl < g_sr && l_l >= g_sl && l_l <= g_la) {
        const double s1 = lam * tr + G * (e1 + e2) - l_l * (2.0 * lam * s + G * (1.0 + s));
        const double s3 = lam * tr + 2.0 * G * e3 - l_l * (2.0 * lam * s - 2.0 * G * (1.0 - s));
        double P12[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            P12[i] = P[0][i] + P[1][i];
            S[i] = s1 * P12[i] + s3 * P[2][i];
        }
        if (DS) {
            double q6[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) q6[i] = G * (1.0 + s) * P12[i] - 2.0 * G * (1.0 - s) * P[2][i] + io[i] * (2.0 * lam * s);
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    DS[i + 3 * j] = s1 * (dP[0][i + 3 * j] + dP[1][i + 3 * j]) + s3 * dP[2][i + 3 * j] + io[i] * io[j] * lam +
                                    G * (P12[i] * P12[j]) + 2.0 * G * (P[2][i] * P[2][j]) - q6[i] * q6[j] / d_l;
        }
        return kLeft;
    }
    const double d_r = 4.0 * lam * s * s + 2.0 * G * (1.0 + s) * (1.0 + s) + G * (1.0 - s) * (1.0 - s);
    const double l_r = (G * (2.0 * (1.0 + s) * e1 - (1.0 - s) * (e2 + e3)) + 2.0 * lam * s * tr - c) / d_r;
    if (g_sl > g_sr && l_r >= g_sr && l_r <= g_ra) {
        const double s1 = lam * tr + 2.0 * G * e1 - l_r * (2.0 * lam * s + 2.0 * G * (1.0 + s));
        const double s3 = lam * tr + G * (e2 + e3) - l_r * (2.0 * lam * s - G * (1.0 - s));
        double P23[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            P23[i] = P[1][i] + P[2][i];
            S[i] = s1 * P[0][i] + s3 * P23[i];
        }
        if (DS) {
            double q6[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) q6[i] = 2.0 * G * (1.0 + s) * P[0][i] - G * (1.0 - s) * P23[i] + io[i] * (2.0 * lam * s);
#pragma unroll
            for (int j = 0; j < 3; ++j)
#pragma unroll
                for (int i = 0; i < 3; ++i)
                    DS[i + 3 * j] = s1 * dP[0][i + 3 * j] + s3 * (dP[1][i + 3 * j] + dP[2][i + 3 * j]) + io[i] * io[j] * lam +
                                    2.0 * G * (P[0][i] * P[0][j]) + G * (P23[i] * P23[j]) - q6[i] * q6[j] / d_r;
        }
        return kRight;
    }
    const double sa = c / (2.0 * s);
    S[0] = sa;
    S[1] = sa;
    S[2] = 0.0;
    S[3] = sa;
    if (DS) {
#pragma unroll
        for (int k = 0; k < 9; ++k) DS[k] = 0.0;
    }
    return kApex;
}

template <bool TANGENT>
__global__ void __launch_bounds__(128) mc2d_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                   const double *__restrict__ sin_phi, const double *__restrict__ shear,
                                                   const double *__restrict__ lame, int n, double *__restrict__ S,
                                                   double *__restrict__ DS, int8_t *__restrict__ branch) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double e[3] = {E[3ll * p], E[3ll * p + 1], E[3ll * p + 2]};
    double s[4], ds[9];
    const int b = mc2d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, TANGENT ? ds : nullptr);
    if (branch) branch[p] = static_cast<int8_t>(b);
#pragma unroll
    for (int k = 0; k < 4; ++k) S[4ll * p + k] = s[k];
    if (TANGENT) {
#pragma unroll
        for (int k = 0; k < 9; ++k) DS[9ll * p + k] = ds[k];
    }
}

// ---------------------------------------------------------------------------- reduction

__global__ void reduction_kernel(const double *__restrict__ c0, const double *__restrict__ phi,
                                 const double *__restrict__ psi, int n, double lam, int davis, double *__restrict__ c_bar,
                                 double *__restrict__ sin_phi) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double f = phi[p], y = psi[p], c = c0[p];
    double c_l, phi_l;
    if (davis == 0) {  // A
        const double beta = cos(f) * cos(y) / (1.0 - sin(f) * sin(y));
        c_l = beta * c / lam;
        phi_l = atan(beta * tan(f) / lam);
    } else if (davis == 1) {  // B
        const double c1 = c / lam;
        const double f1 = atan(tan(f) / lam);
        const double y1 = atan(tan(y) / lam);
        const double beta = cos(f1) * cos(y1) / (1.0 - sin(f1) * sin(y1));
        c_l = beta * c1;
        phi_l = atan(beta * tan(f1));
    } else {  // C
        const double c1 = c / lam;
        const double f1 = atan(tan(f) / lam);
        const double beta = f1 > y ? cos(f1) * cos(y) / (1.0 - sin(f1) * sin(y)) : 1.0;
        c_l = beta * c1;
        phi_l = atan(beta * tan(f1));
    }
    c_bar[p] = 2.0 * c_l * cos(phi_l);
    sin_phi[p] = sin(phi_l);
}

}  // namespace
}  // namespace ssp

using namespace ssp;

extern "C" {

int ssp_constitutive_3d_s(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                          const double *bulk, const double *lame, int n_int, double *S_out, void *stream) {
    (void)bulk;
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out) return SSP_ERR_INVALID;
    mc3d_kernel<false><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                             nullptr, nullptr);
    return launch_status();
}

int ssp_constitutive_3d_sds(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                            const double *bulk, const double *lame, int n_int, double *S_out, double *DS_out,
                            void *stream) {
    (void)bulk;
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out) return SSP_ERR_INVALID;
    mc3d_kernel<true><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                            DS_out, nullptr);
    return launch_status();
}

int ssp_constitutive_3d_branch(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                               const double *lame, int n_int, double *S_out, int8_t *branch_out, void *stream) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !branch_out) return SSP_ERR_INVALID;
    mc3d_kernel<false><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                             nullptr, branch_out);
    return launch_status();
}

int ssp_constitutive_2d(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                        const double *bulk, const double *lame, int n_int, double *S_out, double *DS_out, void *stream) {
    (void)bulk;
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out) return SSP_ERR_INVALID;
    if (DS_out)
        mc2d_kernel<true><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                                DS_out, nullptr);
    else
        mc2d_kernel<false><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                                 nullptr, nullptr);
    return launch_status();
}

int ssp_constitutive_sds_branch(int dim, const double *E, const double *c_bar, const double *sin_phi,
                                const double *shear, const double *lame, int n_int, double *S_out, double *DS_out,
                                int8_t *branch_out, void *stream) {
    if ((dim != 2 && dim != 3) || n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out) return SSP_ERR_INVALID;
    if (dim == 3)
        mc3d_kernel<true><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                                DS_out, branch_out);
    else
        mc2d_kernel<true><<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                                DS_out, branch_out);
    return launch_status();
}

int ssp_reduction(const double *c0, const double *phi, const double *psi, int n_int, double lam, char davis_type,
                  double *c_bar_out, double *sin_phi_out, void *stream) {
    if (n_int < 0 || !(lam > 0.0)) return SSP_ERR_INVALID;
    int d;
    switch (davis_type) {
        case 'A': case 'a': d = 0; break;
        case 'B': case 'b': d = 1; break;
        case 'C': case 'c': d = 2; break;
        default: return SSP_ERR_INVALID;
    }
    if (n_int == 0) return SSP_OK;
    if (!c0 || !phi || !psi || !c_bar_out || !sin_phi_out) return SSP_ERR_INVALID;
    reduction_kernel<<<grid_for(n_int, 256), 256, 0, as_stream(stream)>>>(c0, phi, psi, n_int, lam, d, c_bar_out,
                                                                          sin_phi_out);
    return launch_status();
}

int ssp_device_status(int *status_out, int clear) {
    if (!status_out) return SSP_ERR_INVALID;
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_status, sizeof(int)) != cudaSuccess) return SSP_ERR_CUDA;
    *status_out = v;
    if (clear) {
        int z = 0;
        if (cudaMemcpyToSymbol(g_device_status, &z, sizeof(int)) != cudaSuccess) return SSP_ERR_CUDA;
    }
    return SSP_OK;
}

}  // extern "C"
