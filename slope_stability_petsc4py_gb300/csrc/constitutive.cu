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

#include <mutex>

#include "ssp_internal.cuh"

namespace ssp {

__device__ int g_device_status = 0;

namespace {

__device__ __forceinline__ double vol_iota(int i) { return i < 3 ? 1.0 : 0.0; }
__device__ __forceinline__ double half_ident(int i) { return i < 3 ? 1.0 : 0.5; }

// Branch codes shared with the learned branch proposal (ssp_branch_*).
enum Branch : int { kElastic = 0, kSmooth = 1, kLeft = 2, kRight = 3, kApex = 4 };

struct Principal3 {
    double t[6], sq[6];
    double I1, e1, e2, e3;
};

// sin and cos of a Lode angle theta in [0, pi/3] from their Taylor series, Horner in theta^2: the
// first omitted terms, theta^19 / 19! and theta^20 / 20!, are below 2e-17 there, and without a
// branch every lane of a warp runs the same instructions (a general sincos reduces its argument by
// quadrants, and pi/4 < pi/3).  Within one ulp of the correctly rounded values on [0, pi/3].
__device__ __forceinline__ void sincos_lode(double theta, double &s, double &c) {
    const double z = theta * theta;
    double ps = 1.0 / 355687428096000.0;  // 1/17!
    ps = fma(ps, z, -1.0 / 1307674368000.0);
    ps = fma(ps, z, 1.0 / 6227020800.0);
    ps = fma(ps, z, -1.0 / 39916800.0);
    ps = fma(ps, z, 1.0 / 362880.0);
    ps = fma(ps, z, -1.0 / 5040.0);
    ps = fma(ps, z, 1.0 / 120.0);
    ps = fma(ps, z, -1.0 / 6.0);
    s = fma(theta * z, ps, theta);
    double pc = -1.0 / 6402373705728000.0;  // -1/18!
    pc = fma(pc, z, 1.0 / 20922789888000.0);
    pc = fma(pc, z, -1.0 / 87178291200.0);
    pc = fma(pc, z, 1.0 / 479001600.0);
    pc = fma(pc, z, -1.0 / 3628800.0);
    pc = fma(pc, z, 1.0 / 40320.0);
    pc = fma(pc, z, -1.0 / 720.0);
    pc = fma(pc, z, 1.0 / 24.0);
    pc = fma(pc, z, -0.5);
    c = fma(z, pc, 1.0);
}

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
    // divisions by constants as products with the rounded reciprocals (an ulp from the quotients)
    double Q = (I1 * I1 - 3.0 * I2) * (1.0 / 9.0);
    if (Q < 0.0) Q = 0.0;
    const double R = (-2.0 * I1 * I1 * I1 + 9.0 * I1 * I2 - 27.0 * I3) * (1.0 / 54.0);
    const double rq = sqrt(Q);
    double theta = 0.0;
    if (!(Q < 1e-30)) {
        double c = R / (rq * Q);
        c = fmin(1.0, fmax(-1.0, c));
        theta = acos(c) * (1.0 / 3.0);
    }
    const double third = I1 * (1.0 / 3.0);
    p.I1 = I1;
    // cos(theta -+ 2 pi/3) = -cos(theta)/2 +- (sqrt(3)/2) sin(theta): one sine and cosine instead of
    // three cosines
    double st, ct;
    sincos_lode(theta, st, ct);
    const double r3 = 1.7320508075688772 * st;
    p.e1 = rq * (ct + r3) + third;
    p.e2 = rq * (ct - r3) + third;
    p.e3 = -2.0 * rq * ct + third;
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

struct Decision3 {
    int branch;
    double lam;  // plastic multiplier of the selected branch (elastic / apex: unused)
    double den;  // its denominator
};

struct Mat3 {
    double c_bar, sin_phi, shear, lame;
};

// Plastic multipliers of the three return branches (constitutive_3D_kernel.h:144-147, 213-215, 277-279).
__device__ __forceinline__ void smooth_lam(const Principal3 &p, const Mat3 &m, double f_tr, double &lam, double &den) {
    const double sp = m.sin_phi;
    den = 4.0 * m.lame * m.sin_phi * sp + 4.0 * m.shear * (1.0 + m.sin_phi * sp);
    lam = f_tr / den;
}
__device__ __forceinline__ void left_lam(const Principal3 &p, const Mat3 &m, double &lam, double &den) {
    const double sp = m.sin_phi, sf = m.sin_phi, G = m.shear, L = m.lame;
    den = 4.0 * L * sf * sp + G * (1.0 + sf) * (1.0 + sp) + 2.0 * G * (1.0 - sf) * (1.0 - sp);
    lam = (G * ((1.0 + sf) * (p.e1 + p.e2) - 2.0 * (1.0 - sf) * p.e3) + 2.0 * L * sf * p.I1 - m.c_bar) / den;
}
__device__ __forceinline__ void right_lam(const Principal3 &p, const Mat3 &m, double &lam, double &den) {
    const double sp = m.sin_phi, sf = m.sin_phi, G = m.shear, L = m.lame;
    den = 4.0 * L * sf * sp + 2.0 * G * (1.0 + sf) * (1.0 + sp) + G * (1.0 - sf) * (1.0 - sp);
    lam = (G * (2.0 * (1.0 + sf) * p.e1 - (1.0 - sf) * (p.e2 + p.e3)) + 2.0 * L * sf * p.I1 - m.c_bar) / den;
}
__device__ __forceinline__ double trial_yield(const Principal3 &p, const Mat3 &m) {
    return 2.0 * m.shear * ((1.0 + m.sin_phi) * p.e1 - (1.0 - m.sin_phi) * p.e3) + 2.0 * m.lame * m.sin_phi * p.I1 -
           m.c_bar;
}

// Branch selection (constitutive_3D_kernel.h:114-338).
__device__ __forceinline__ Decision3 decide3(const Principal3 &p, const Mat3 &m) {
    const double sp = m.sin_phi;
    const double f_tr = trial_yield(p, m);
    if (f_tr <= 0.0) return {kElastic, 0.0, 1.0};
    // the reference's bounds g = x / d (d = 1 +- sin phi, 3 -+ sin phi, all positive) compared as
    // lam d against x, and g_sl against g_sr cross-multiplied: no division for the tests
    const double a_sl = p.e1 - p.e2, d_sl = 1.0 + sp;  // g_sl = a_sl / d_sl
    const double a_sr = p.e2 - p.e3, d_sr = 1.0 - sp;  // g_sr = a_sr / d_sr
    double lam, den;
    smooth_lam(p, m, f_tr, lam, den);
    if (lam * d_sl <= a_sl && lam * d_sr <= a_sr) return {kSmooth, lam, den};
    const double l_sl = a_sl * d_sr, l_sr = a_sr * d_sl;  // g_sl < g_sr <=> l_sl < l_sr
    if (l_sl < l_sr) {
        left_lam(p, m, lam, den);
        if (lam * d_sl >= a_sl && lam * (3.0 - sp) <= p.e1 + p.e2 - 2.0 * p.e3) return {kLeft, lam, den};
    }
    if (l_sl > l_sr) {
        right_lam(p, m, lam, den);
        if (lam * d_sr >= a_sr && lam * (3.0 + sp) <= 2.0 * p.e1 - p.e2 - p.e3) return {kRight, lam, den};
    }
    return {kApex, 0.0, 1.0};
}

// Elastic branch: S = lambda tr(E) I + 2 G t (t = E with halved shears), DS = the elastic matrix.
__device__ __forceinline__ void finish_elastic(const double *t, double I1, const Mat3 &m, double *S, double *DS) {
    const double shear = m.shear, lame = m.lame;
    const double lI1 = lame * I1, s2 = 2.0 * shear;
#pragma unroll
    for (int i = 0; i < 3; ++i) S[i] = lI1 + s2 * t[i];
#pragma unroll
    for (int i = 3; i < 6; ++i) S[i] = s2 * t[i];
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
}

// Elastic screen from invariants, before any eigen-decomposition, in FP32.  With principal trial
// strains e1 >= e2 >= e3, Q = J2/3 and Lode angle a, the trial yield function is
//   f = 2G[(e1 - e3) + s(e1 + e3)] + 2 lambda s I1 - c_bar,
//   (e1 - e3) + s(e1 + e3) = 2 sqrt(Q) (sqrt(3) sin a + s cos a) + 2 s I1 / 3,
// and sqrt(3) sin a + s cos a <= sqrt(3 + s^2) for every a (Cauchy-Schwarz), so
//   f <= bound = 2G[2 sqrt(Q) sqrt(3 + s^2) + 2 s I1 / 3] + 2 lambda s I1 - c_bar.
// The bound is evaluated in FP32 from inputs truncated to 24 bits (J2 from differences of the
// normal components, so no cancellation against I1): its absolute error stays below ~4e-6 of
//   size = 2|G| (2 sqrt(Q) sqrt(3 + s^2) + 3 max|t_i|) + 2|lambda s I1| + |c_bar|.
// A point with bound <= -1e-4 size is therefore elastic however the FP64 eigenvalues of the full
// path round (their error is at most ~1e-8 sqrt(Q), near repeated roots): the full path's branch
// test would say elastic too.  Such a point is finished from t and I1 in FP64 with the elastic
// branch's own arithmetic, so S and DS are bitwise those of the full path, and it costs about a
// dozen FP64 instructions instead of an eigen-decomposition.
__device__ __forceinline__ bool screen_elastic(const double *E, const Mat3 &m) {
    float t[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = df_from_f64(E[i]).hi * (i < 3 ? 1.0f : 0.5f);
    const float G = df_from_f64(m.shear).hi, L = df_from_f64(m.lame).hi;
    const float s = df_from_f64(m.sin_phi).hi, c = df_from_f64(m.c_bar).hi;
    const float d01 = t[0] - t[1], d12 = t[1] - t[2], d20 = t[2] - t[0];
    const float J2 = (d01 * d01 + d12 * d12 + d20 * d20) * (1.0f / 6.0f) + t[3] * t[3] + t[4] * t[4] + t[5] * t[5];
    const float I1 = t[0] + t[1] + t[2];
    const float dev = 2.0f * sqrtf(J2 * (1.0f / 3.0f)) * sqrtf(3.0f + s * s);
    const float bound = 2.0f * G * (dev + (2.0f / 3.0f) * s * I1) + 2.0f * L * s * I1 - c;
    const float tmax = fmaxf(fmaxf(fabsf(t[0]), fabsf(t[1])), fmaxf(fabsf(t[2]), fmaxf(fabsf(t[3]), fmaxf(fabsf(t[4]), fabsf(t[5])))));
    const float size = 2.0f * fabsf(G) * (dev + 3.0f * tmax) + 2.0f * fabsf(L * s * I1) + fabsf(c);
    return bound <= -1e-4f * size;
}
// t (shears halved) and I1 of the trial strain, in FP64, as principal3 forms them.
__device__ __forceinline__ void elastic_trial(const double *E, double *t, double &I1) {
#pragma unroll
    for (int i = 0; i < 6; ++i) t[i] = half_ident(i) * E[i];
    I1 = t[0] + t[1] + t[2];
}

// ---- consistent tangent of the plastic branches in double-float arithmetic (the mixed form)
//
// The FP64 formulas below (finish3) are regrouped per point into FP64 coefficients, and each DS
// entry becomes a short sum of products of per-point vectors, accumulated compensated on the FP32
// pipe (CSum, about 2^-48 of the sum of |terms|) and widened once.  Smooth face, with
// a_k = s_k inv_k, A = sum_k a_k, B = sum_k a_k em_k:
//   DS_ij = A J_ij - I_ij B + sum_k (K_k P_k,i) P_k,j + lambda iota_i iota_j - (Dp_i / den) Dp_j,
//   K_1 = 2G - (a1 c1a + a2 c2b + a3 c3b), K_2 = 2G - (a1 c1b + a2 c2a - a3 c3b),
//   K_3 = 2G + (a1 c1b + a2 c2b - a3 c3a);
// edges (left: Q = P12, R = P3, e = e3, em = e1 + e2, a = (s3 - s1) inv3; right: Q = P23, R = P1,
// e = e1, em = e2 + e3, a = (s1 - s3) inv1):
//   DS_ij = a J_ij - I_ij a em - a (Q_i t_j + t_i Q_j) + (a em + G) Q_i Q_j
//           + (a (em - 2e) + 2G) R_i R_j + a e (Q_i R_j + R_i Q_j) + lambda iota_i iota_j - (Dp_i / den) Dp_j,
// with J = d(t t)/dE (square_jac) and I_ij = half_ident(i) on the diagonal.  The inverse gaps make
// the terms larger than the result by about (|e| / gap)^2, so a point whose smallest eigenvalue
// gap is below 1e-3 of max|e|, or whose coefficients leave the float range, keeps the FP64 loop.
__device__ __forceinline__ df32 df_pow2(df32 a, float f) { return {a.hi * f, a.lo * f}; }  // f a power of two

// acc += A * d(t t)_ij / dE_j (square_jac's entries)
__device__ __forceinline__ void add_square_jac(CSum &acc, df32 A, const df32 *t, int i, int j) {
    const df32 A2 = df_pow2(A, 2.0f), Ah = df_pow2(A, 0.5f);
    switch (i * 6 + j) {
        case 0: acc.add_prod(A2, t[0]); break;
        case 3: case 9: acc.add_prod(A, t[3]); break;
        case 5: case 17: acc.add_prod(A, t[5]); break;
        case 7: acc.add_prod(A2, t[1]); break;
        case 10: case 16: acc.add_prod(A, t[4]); break;
        case 14: acc.add_prod(A2, t[2]); break;
        case 21: acc.add_prod(Ah, t[0]); acc.add_prod(Ah, t[1]); break;
        case 22: acc.add_prod(Ah, t[5]); break;
        case 23: acc.add_prod(Ah, t[4]); break;
        case 28: acc.add_prod(Ah, t[1]); acc.add_prod(Ah, t[2]); break;
        case 29: acc.add_prod(Ah, t[3]); break;
        case 35: acc.add_prod(Ah, t[0]); acc.add_prod(Ah, t[2]); break;
        default: break;
    }
}
__device__ __forceinline__ bool in_float_range(double x) { return fabs(x) <= 1e30; }  // false for nan

__device__ __forceinline__ bool smooth_ds_compensated(const Principal3 &p, const Mat3 &m, const double *P1,
                                                      const double *P2, const double *P3, double inv1, double inv2,
                                                      double inv3, double s1, double s2, double s3, const double *Dp,
                                                      double inv_den, double *DS) {
    const double e1 = p.e1, e2 = p.e2, e3 = p.e3;
    if (!(fmin(e1 - e2, e2 - e3) >= 1e-3 * fmax(fabs(e1), fabs(e3)))) return false;
    const double a1 = s1 * inv1, a2 = s2 * inv2, a3 = s3 * inv3;
    const double c1a = 2.0 * e1 - e2 - e3, c1b = e2 - e3;
    const double c2a = 2.0 * e2 - e1 - e3, c2b = e1 - e3;
    const double c3a = 2.0 * e3 - e1 - e2, c3b = e1 - e2;
    const double A = a1 + a2 + a3, B = a1 * (e2 + e3) + a2 * (e1 + e3) + a3 * (e1 + e2);
    const double G2 = 2.0 * m.shear;
    const double K1 = G2 - (a1 * c1a + a2 * c2b + a3 * c3b);
    const double K2 = G2 - (a1 * c1b + a2 * c2a - a3 * c3b);
    const double K3 = G2 + (a1 * c1b + a2 * c2b - a3 * c3a);
    if (!(in_float_range(A) && in_float_range(B) && in_float_range(K1) && in_float_range(K2) && in_float_range(K3)))
        return false;
    df32 t[6], r1[6], r2[6], r3[6], q1[6], q2[6], q3[6], dp[6], dq[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = df_from_f64(p.t[i]);
        r1[i] = df_from_f64(P1[i]);
        r2[i] = df_from_f64(P2[i]);
        r3[i] = df_from_f64(P3[i]);
        q1[i] = df_from_f64(K1 * P1[i]);
        q2[i] = df_from_f64(K2 * P2[i]);
        q3[i] = df_from_f64(K3 * P3[i]);
        dp[i] = df_from_f64(Dp[i]);
        dq[i] = df_from_f64(-Dp[i] * inv_den);
    }
    const df32 Ad = df_from_f64(A), Bd = df_from_f64(B), Ld = df_from_f64(m.lame);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) {
            CSum acc;
            add_square_jac(acc, Ad, t, i, j);
            if (i == j) acc.add(df_pow2(Bd, i < 3 ? -1.0f : -0.5f));
            acc.add_prod(q1[i], r1[j]);
            acc.add_prod(q2[i], r2[j]);
            acc.add_prod(q3[i], r3[j]);
            if (j < 3) acc.add(Ld);
            acc.add_prod(dq[i], dp[j]);
            store_sym(DS, i, j, acc.value());
        }
    }
    return true;
}

__device__ __forceinline__ bool edge_ds_compensated(const Principal3 &p, const Mat3 &m, const double *Q,
                                                    const double *R, double a, double em, double e, double gap,
                                                    const double *Dp, double inv_den, double *DS) {
    if (!(gap >= 1e-3 * fmax(fabs(p.e1), fabs(p.e3)))) return false;
    const double kQ = a * em + m.shear, kR = a * (em - 2.0 * e) + 2.0 * m.shear, ae = a * e, aem = a * em;
    if (!(in_float_range(a) && in_float_range(kQ) && in_float_range(kR) && in_float_range(ae) && in_float_range(aem)))
        return false;
    df32 t[6], qd[6], rd[6], aq[6], kqq[6], krr[6], aeq[6], dp[6], dq[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        t[i] = df_from_f64(p.t[i]);
        qd[i] = df_from_f64(Q[i]);
        rd[i] = df_from_f64(R[i]);
        aq[i] = df_from_f64(-a * Q[i]);
        kqq[i] = df_from_f64(kQ * Q[i]);
        krr[i] = df_from_f64(kR * R[i]);
        aeq[i] = df_from_f64(ae * Q[i]);
        dp[i] = df_from_f64(Dp[i]);
        dq[i] = df_from_f64(-Dp[i] * inv_den);
    }
    const df32 ad = df_from_f64(a), aemd = df_from_f64(aem), Ld = df_from_f64(m.lame);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) {
            CSum acc;
            add_square_jac(acc, ad, t, i, j);
            if (i == j) acc.add(df_pow2(aemd, i < 3 ? -1.0f : -0.5f));
            acc.add_prod(aq[i], t[j]);
            acc.add_prod(t[i], aq[j]);
            acc.add_prod(kqq[i], qd[j]);
            acc.add_prod(krr[i], rd[j]);
            acc.add_prod(aeq[i], rd[j]);
            acc.add_prod(rd[i], aeq[j]);
            if (j < 3) acc.add(Ld);
            acc.add_prod(dq[i], dp[j]);
            store_sym(DS, i, j, acc.value());
        }
    }
    return true;
}

// ---- consistent tangent of the plastic branches, FP64, regrouped per point
//
// The same regrouping as the double-float form above, in FP64: per point the coefficients A, B, K_k
// (smooth) or a, kQ, kR (edges) and the vectors K_k P_k, -Dp / den are formed once, and each of the
// 21 upper entries is a short sum of products (about 300 FP64 operations per smooth point against
// about 700 for the entry-by-entry form of constitutive_3D_kernel.h:242-262, whose inverse gaps
// multiply each entry's own combination).  Its terms are larger than the result by about
// (max|e| / gap)^2, which multiplies the rounding errors: it is used only where every gap is at
// least kRegroupGap of max|e| (amplification <= 400, errors ~1e-14 of the tangent's scale); other
// points keep the entry-by-entry form.
constexpr double kRegroupGap = 0.05;

__device__ __forceinline__ bool smooth_ds_regrouped(const Principal3 &p, const Mat3 &m, const double *P1,
                                                    const double *P2, const double *P3, double inv1, double inv2,
                                                    double inv3, double s1, double s2, double s3, const double *Dp,
                                                    double inv_den, double *DS) {
    const double e1 = p.e1, e2 = p.e2, e3 = p.e3;
    if (!(fmin(e1 - e2, e2 - e3) >= kRegroupGap * fmax(fabs(e1), fabs(e3)))) return false;
    const double a1 = s1 * inv1, a2 = s2 * inv2, a3 = s3 * inv3;
    const double c1a = 2.0 * e1 - e2 - e3, c1b = e2 - e3;
    const double c2a = 2.0 * e2 - e1 - e3, c2b = e1 - e3;
    const double c3a = 2.0 * e3 - e1 - e2, c3b = e1 - e2;
    const double A = a1 + a2 + a3, B = a1 * (e2 + e3) + a2 * (e1 + e3) + a3 * (e1 + e2);
    const double G2 = 2.0 * m.shear;
    const double K1 = G2 - (a1 * c1a + a2 * c2b + a3 * c3b);
    const double K2 = G2 - (a1 * c1b + a2 * c2a - a3 * c3b);
    const double K3 = G2 + (a1 * c1b + a2 * c2b - a3 * c3a);
    double q1[6], q2[6], q3[6], dq[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        q1[i] = K1 * P1[i];
        q2[i] = K2 * P2[i];
        q3[i] = K3 * P3[i];
        dq[i] = -Dp[i] * inv_den;
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) {
            double v = A * square_jac(p.t, i, j) + q1[i] * P1[j] + q2[i] * P2[j] + q3[i] * P3[j] + dq[i] * Dp[j];
            if (i == j) v -= half_ident(i) * B;
            if (j < 3) v += m.lame;
            store_sym(DS, i, j, v);
        }
    }
    return true;
}

// Edges: left Q = P12, R = P3, e = e3, em = e1 + e2; right Q = P23, R = P1, e = e1, em = e2 + e3;
// a the branch's (s_R - s_Q) inv and gap its eigenvalue gap.
__device__ __forceinline__ bool edge_ds_regrouped(const Principal3 &p, const Mat3 &m, const double *Q, const double *R,
                                                  double a, double em, double e, double gap, const double *Dp,
                                                  double inv_den, double *DS) {
    if (!(gap >= kRegroupGap * fmax(fabs(p.e1), fabs(p.e3)))) return false;
    const double kQ = a * em + m.shear, kR = a * (em - 2.0 * e) + 2.0 * m.shear, ae = a * e, aem = a * em;
    double aq[6], kqq[6], krr[6], aeq[6], dq[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        aq[i] = -a * Q[i];
        kqq[i] = kQ * Q[i];
        krr[i] = kR * R[i];
        aeq[i] = ae * Q[i];
        dq[i] = -Dp[i] * inv_den;
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) {
#pragma unroll
        for (int i = 0; i <= j; ++i) {
            double v = a * square_jac(p.t, i, j) + aq[i] * p.t[j] + p.t[i] * aq[j] + kqq[i] * Q[j] + krr[i] * R[j] +
                       aeq[i] * R[j] + R[i] * aeq[j] + dq[i] * Dp[j];
            if (i == j) v -= half_ident(i) * aem;
            if (j < 3) v += m.lame;
            store_sym(DS, i, j, v);
        }
    }
    return true;
}

// Stress and (when DS != null) consistent tangent of the decided branch.  COMP: the plastic
// branches' DS in double-float arithmetic where the point allows it (S is always FP64 and the
// same as without COMP); otherwise the regrouped FP64 form where the gaps allow it.
template <bool COMP>
__device__ void finish3(const Principal3 &p, const Decision3 &d, const Mat3 &m, double *S, double *DS) {
    const double sp = m.sin_phi, sin_phi = m.sin_phi, shear = m.shear, lame = m.lame;
    const double e1 = p.e1, e2 = p.e2, e3 = p.e3, I1 = p.I1;
    if (d.branch == kElastic) {
        finish_elastic(p.t, I1, m, S, DS);
        return;
    }
    if (d.branch == kSmooth) {
        const double lam_s = d.lam;
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
            const double inv_den = 1.0 / d.den;
            if constexpr (COMP) {
                if (smooth_ds_compensated(p, m, P1, P2, P3, inv1, inv2, inv3, s1, s2, s3, Dp, inv_den, DS)) return;
            } else {
                if (smooth_ds_regrouped(p, m, P1, P2, P3, inv1, inv2, inv3, s1, s2, s3, Dp, inv_den, DS)) return;
            }
            const double em23 = e2 + e3, em13 = e1 + e3, em12 = e1 + e2;
            const double c1a = 2.0 * e1 - e2 - e3, c1b = e2 - e3;
            const double c2a = 2.0 * e2 - e1 - e3, c2b = e1 - e3;
            const double c3a = 2.0 * e3 - e1 - e2, c3b = e1 - e2;
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
        return;
    }
    if (d.branch == kLeft) {
        const double lam_l = d.lam;
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
            const double inv_den = 1.0 / d.den;
            if constexpr (COMP) {
                if (edge_ds_compensated(p, m, P12, P3, (s3 - s1) * inv3, em12, e3, e2 - e3, Dp, inv_den, DS)) return;
            } else {
                if (edge_ds_regrouped(p, m, P12, P3, (s3 - s1) * inv3, em12, e3, e2 - e3, Dp, inv_den, DS)) return;
            }
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
        return;
    }
    if (d.branch == kRight) {
        const double lam_r = d.lam;
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
            const double inv_den = 1.0 / d.den;
            if constexpr (COMP) {
                if (edge_ds_compensated(p, m, P23, P1, (s1 - s3) * inv1, em23, e1, e1 - e2, Dp, inv_den, DS)) return;
            } else {
                if (edge_ds_regrouped(p, m, P23, P1, (s1 - s3) * inv1, em23, e1, e1 - e2, Dp, inv_den, DS)) return;
            }
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
        return;
    }
    const double sa = m.c_bar / (2.0 * sin_phi);
#pragma unroll
    for (int i = 0; i < 3; ++i) S[i] = sa;
#pragma unroll
    for (int i = 3; i < 6; ++i) S[i] = 0.0;
    if (DS) {
#pragma unroll
        for (int k = 0; k < 36; ++k) DS[k] = 0.0;
    }
}

// Returns the branch code.  DS may be null (stress only).
__device__ int mc3d_point(const double *E, double c_bar, double sin_phi, double shear, double lame, double *S,
                          double *DS) {
    const Mat3 m{c_bar, sin_phi, shear, lame};
    if (screen_elastic(E, m)) {
        double t[6], I1;
        elastic_trial(E, t, I1);
        finish_elastic(t, I1, m, S, DS);
        return kElastic;
    }
    Principal3 p;
    principal3(E, p);
    const Decision3 d = decide3(p, m);
    finish3<false>(p, d, m, S, DS);
    return d.branch;
}

__device__ __forceinline__ void load6(const double *A, long long p, double *e) {
    const double2 *A2 = reinterpret_cast<const double2 *>(A + 6 * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double2 v = A2[k];
        e[2 * k] = v.x;
        e[2 * k + 1] = v.y;
    }
}
__device__ __forceinline__ void store6(double *A, long long p, const double *s) {
    double2 *A2 = reinterpret_cast<double2 *>(A + 6 * p);
#pragma unroll
    for (int k = 0; k < 3; ++k) A2[k] = make_double2(s[2 * k], s[2 * k + 1]);
}
__device__ __forceinline__ void store36(double *A, long long p, const double *s) {
    double2 *A2 = reinterpret_cast<double2 *>(A + 36 * p);
#pragma unroll
    for (int k = 0; k < 18; ++k) A2[k] = make_double2(s[2 * k], s[2 * k + 1]);
}

// Single pass, one thread per point.  With the tangent, a warp's 32 consecutive DS rows are staged
// in shared memory (row stride 37 doubles) and written as one contiguous block with full-line
// stores.
template <bool TANGENT>
__global__ void __launch_bounds__(128) mc3d_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                   const double *__restrict__ sin_phi, const double *__restrict__ shear,
                                                   const double *__restrict__ lame, int n, double *__restrict__ S,
                                                   double *__restrict__ DS, int8_t *__restrict__ branch) {
    constexpr int kStride = 37;
    __shared__ double stage[TANGENT ? 4 : 1][TANGENT ? 32 * kStride : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) {
        double e[6], s[6];
        load6(E, p, e);
        int b;
        if (TANGENT) {
            double ds[36];
            b = mc3d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, ds);
#pragma unroll
            for (int k = 0; k < 36; ++k) stage[warp][lane * kStride + k] = ds[k];
        } else {
            b = mc3d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, nullptr);
        }
        store6(S, p, s);
        if (branch) branch[p] = static_cast<int8_t>(b);
    }
    if (TANGENT) {
        __syncwarp();
        const int p0 = blockIdx.x * blockDim.x + warp * 32;
        if (p0 < n) {
            const int nw = n - p0 < 32 ? n - p0 : 32;
            double *dst = DS + 36ll * p0;
            for (int idx = lane; idx < nw * 36; idx += 32) {
                const int pt = idx / 36;
                dst[idx] = stage[warp][pt * kStride + (idx - pt * 36)];
            }
        }
    }
}

// Binned return mapping in three passes.  scratch = 4 counters, then three regions of n int32.
//   A: every point is screened (screen_elastic, FP32); screened points are finished as elastic
//      (a dozen FP64 instructions), the others are appended to list L (counter 0, region 0).
//   B: over L, the FP64 eigen-decomposition and branch decision (dense warps); elastic and apex
//      points are finished here; a smooth / left-edge / right-edge point leaves its decision record
//      (principal values, t, t*t, I1, multiplier, denominator: 18 doubles) in the first entries of
//      its own DS row, which pass C overwrites, and is appended to its branch's list (smooth:
//      region 1 from the front; left: region 2 from the front; right: region 2 from the back;
//      counters 1, 2, 3).
//   C: one branch per blockIdx.y: the stress and consistent tangent from the record, so every
//      warp runs one branch's code and nothing is computed twice.
// Every result equals the single-pass kernel's (the same operations on the same values).
constexpr int kRecord = 18;
__device__ __forceinline__ void store_record(double *DS, long long p, const Principal3 &pr, const Decision3 &d) {
    double r[kRecord];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        r[i] = pr.t[i];
        r[6 + i] = pr.sq[i];
    }
    r[12] = pr.I1;
    r[13] = pr.e1;
    r[14] = pr.e2;
    r[15] = pr.e3;
    r[16] = d.lam;
    r[17] = d.den;
    double2 *D2 = reinterpret_cast<double2 *>(DS + 36 * p);
#pragma unroll
    for (int k = 0; k < kRecord / 2; ++k) D2[k] = make_double2(r[2 * k], r[2 * k + 1]);
}
__device__ __forceinline__ void load_record(const double *DS, long long p, Principal3 &pr, Decision3 &d) {
    double r[kRecord];
    const double2 *D2 = reinterpret_cast<const double2 *>(DS + 36 * p);
#pragma unroll
    for (int k = 0; k < kRecord / 2; ++k) {
        const double2 v = D2[k];
        r[2 * k] = v.x;
        r[2 * k + 1] = v.y;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        pr.t[i] = r[i];
        pr.sq[i] = r[6 + i];
    }
    pr.I1 = r[12];
    pr.e1 = r[13];
    pr.e2 = r[14];
    pr.e3 = r[15];
    d.lam = r[16];
    d.den = r[17];
}

// warp-aggregated append of the lanes with want == true to list[...] through counter *ctr;
// returns this lane's slot
__device__ __forceinline__ int warp_append(bool want, int32_t *ctr) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(__activemask(), want);
    if (mask == 0u) return -1;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if ((int)lane == leader) base = atomicAdd(ctr, __popc(mask));
    base = __shfl_sync(__activemask(), base, leader);
    return want ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

// The DS rows of a warp's 32 points are one contiguous 9 KiB block: pass A stages them in shared
// memory (row stride 37 doubles, so the per-lane row writes are at most 2-way bank conflicts) and
// the warp writes the block with consecutive 8-byte stores (full cache lines) instead of 32
// strided rows.  Rows of listed points are written with whatever the stage holds; passes B and C
// overwrite them.  WRITE_EL = false: the rows of the points the screen finishes are not written at
// all (they hold the elastic matrix, which the tangent's plastic corrections never read; a
// caller that needs them fills them from the branch codes, ssp_fill_elastic_ds).
constexpr int kDsStride = 37;
template <bool WRITE_EL>
__global__ void __launch_bounds__(128) mc3d_bin_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                       const double *__restrict__ sin_phi,
                                                       const double *__restrict__ shear, const double *__restrict__ lame,
                                                       int n, double *__restrict__ S, double *__restrict__ DS,
                                                       int8_t *__restrict__ branch, int32_t *__restrict__ scratch) {
    __shared__ double stage[WRITE_EL ? 4 : 1][WRITE_EL ? 32 * kDsStride : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int p0 = blockIdx.x * blockDim.x + warp * 32;
    double *w = stage[WRITE_EL ? warp : 0];
    bool listed = false;
    if (p < n) {
        double e[6];
        load6(E, p, e);
        const Mat3 m{c_bar[p], sin_phi[p], shear[p], lame[p]};
        if (screen_elastic(e, m)) {
            double t[6], I1, s[6], ds[36];
            elastic_trial(e, t, I1);
            finish_elastic(t, I1, m, s, WRITE_EL ? ds : nullptr);
            store6(S, p, s);
            if (WRITE_EL) {
#pragma unroll
                for (int k = 0; k < 36; ++k) w[lane * kDsStride + k] = ds[k];
            }
            branch[p] = static_cast<int8_t>(kElastic);
        } else {
            listed = true;
        }
    }
    if (WRITE_EL) {
        __syncwarp();
        if (p0 < n) {
            const int nw = n - p0 < 32 ? n - p0 : 32;
            double *dst = DS + 36ll * p0;
            for (int idx = lane; idx < nw * 36; idx += 32) {
                const int pt = idx / 36;
                dst[idx] = w[pt * kDsStride + (idx - pt * 36)];
            }
        }
    }
    const int slot = warp_append(listed, scratch);
    if (listed) scratch[4 + slot] = p;
}

// five CTAs per SM (at most 102 registers; 96 used without spills): the pass is FP64-bound with long
// dependent chains per point, and more resident warps hide more of their latency
__global__ void __launch_bounds__(128, 5) mc3d_decide_kernel(const double *__restrict__ E,
                                                          const double *__restrict__ c_bar,
                                                          const double *__restrict__ sin_phi,
                                                          const double *__restrict__ shear,
                                                          const double *__restrict__ lame, int n,
                                                          double *__restrict__ S, double *__restrict__ DS,
                                                          int8_t *__restrict__ branch, int32_t *__restrict__ scratch,
                                                          const int32_t *__restrict__ lists,
                                                          const int32_t *__restrict__ counts, long long list_stride) {
    const int cnt = counts[blockIdx.y];
    const int32_t *L = lists + blockIdx.y * list_stride;
    int32_t *smooth = scratch + 4 + n, *edges = scratch + 4 + 2ll * n;
    const int stride = gridDim.x * blockDim.x;
    // whole warps iterate together (the appends are warp-collective)
    const int iters = (cnt + stride - 1) / stride;
    for (int it = 0; it < iters; ++it) {
        const int i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        int p = -1, b = -1;
        if (i < cnt) {
            p = L[i];
            if (p < 0 || p >= n) {
                flag(SSP_DEV_BAD_INDEX);
                p = -1;
            }
        }
        if (p >= 0) {
            double e[6];
            load6(E, p, e);
            const Mat3 m{c_bar[p], sin_phi[p], shear[p], lame[p]};
            Principal3 pr;
            principal3(e, pr);
            const Decision3 d = decide3(pr, m);
            b = d.branch;
            branch[p] = static_cast<int8_t>(b);
            if (b == kElastic || b == kApex) {
                double s[6], ds[36];
                finish3<false>(pr, d, m, s, ds);
                store6(S, p, s);
                store36(DS, p, ds);
            } else {
                store_record(DS, p, pr, d);
            }
        }
        const int js = warp_append(b == kSmooth, scratch + 1);
        if (b == kSmooth) smooth[js] = p;
        const int jl = warp_append(b == kLeft, scratch + 2);
        if (b == kLeft) edges[jl] = p;
        const int jr = warp_append(b == kRight, scratch + 3);
        if (b == kRight) edges[n - 1 - jr] = p;
    }
}

// three CTAs per SM (168 registers): the lists are short and each point a long dependent chain
template <bool COMP>
__global__ void __launch_bounds__(128, 3) mc3d_finish_kernel(const double *__restrict__ c_bar,
                                                          const double *__restrict__ sin_phi,
                                                          const double *__restrict__ shear,
                                                          const double *__restrict__ lame, int n,
                                                          double *__restrict__ S, double *__restrict__ DS,
                                                          const int32_t *__restrict__ scratch) {
    const int k = blockIdx.y;  // 0 smooth, 1 left edge, 2 right edge
    const int cnt = scratch[1 + k];
    const int32_t *smooth = scratch + 4 + n, *edges = scratch + 4 + 2ll * n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int p = k == 0 ? smooth[i] : (k == 1 ? edges[i] : edges[n - 1 - i]);
        if (p < 0 || p >= n) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        Principal3 pr;
        Decision3 d{k + 1, 0.0, 1.0};
        load_record(DS, p, pr, d);
        const Mat3 m{c_bar[p], sin_phi[p], shear[p], lame[p]};
        double s[6], ds[36];
        finish3<COMP>(pr, d, m, s, ds);
        store6(S, p, s);
        store36(DS, p, ds);
    }
}

}  // namespace

// Pass A on one stream (counters zeroed first).  scratch: 4 + 3 n int32.  write_elastic_ds = false
// leaves the DS rows of the points it finishes unwritten (mc3d_bin_kernel).
int binned_screen(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                  const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                  cudaStream_t st, bool write_elastic_ds) {
    if (cudaMemsetAsync(scratch, 0, 4 * sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    if (write_elastic_ds)
        mc3d_bin_kernel<true><<<grid_for(n_int, 128), 128, 0, st>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                    DS_out, branch_out, scratch);
    else
        mc3d_bin_kernel<false><<<grid_for(n_int, 128), 128, 0, st>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out,
                                                                     DS_out, branch_out, scratch);
    return launch_status();
}

// Passes B (over n_lists point lists, blockIdx.y = list) and C.
int binned_decide_finish(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                         const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                         int32_t *scratch, const int32_t *lists, const int32_t *counts, int n_lists,
                         long long list_stride, bool compensated_ds, cudaStream_t st) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long gx = (long long)sms * 8;
    const long long need = (n_int + 127) / 128;
    if (gx > need) gx = need;
    mc3d_decide_kernel<<<dim3(static_cast<unsigned>(gx), n_lists), 128, 0, st>>>(
        E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, lists, counts, list_stride);
    const dim3 grid(static_cast<unsigned>(gx), 3);
    if (compensated_ds)
        mc3d_finish_kernel<true><<<grid, 128, 0, st>>>(c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, scratch);
    else
        mc3d_finish_kernel<false><<<grid, 128, 0, st>>>(c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, scratch);
    return launch_status();
}

namespace {

int launch_binned(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                  const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                  bool compensated_ds, cudaStream_t st, bool write_elastic_ds = true) {
    const int rc = binned_screen(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, st,
                                 write_elastic_ds);
    if (rc != SSP_OK) return rc;
    return binned_decide_finish(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch,
                                scratch + 4, scratch, 1, 0, compensated_ds, st);
}

// ---------------------------------------------------------------------------- 2D

// Plane strain, E = [e11, e22, g12] -> S = [s11, s22, s12, s33], DS 3x3 column-major.

// The trial state of a point: in-plane principal values ev0 (with the out-of-plane 0), their
// order (0,2,1) when ev0[0] >= 0 > ev0[1] and (2,0,1) when 0 > ev0[0], the ordered principal
// values e1 >= e2 >= e3 and the trial yield function.
struct Trial2 {
    double ev0[3], rad, e1, e2, e3, tr, f_tr;
    int ord[3];
};

__device__ __forceinline__ Trial2 mc2d_trial(const double *E, double c, double s, double G, double lam) {
    Trial2 t;
    const double e11 = E[0], e22 = E[1], g12 = E[2];
    const double tr2 = e11 + e22;
    t.rad = sqrt((e11 - e22) * (e11 - e22) + g12 * g12);
    t.ev0[0] = 0.5 * (tr2 + t.rad);
    t.ev0[1] = 0.5 * (tr2 - t.rad);
    t.ev0[2] = 0.0;
    t.ord[0] = 0;
    t.ord[1] = 1;
    t.ord[2] = 2;
    if (t.ev0[0] >= t.ev0[2] && t.ev0[2] > t.ev0[1]) {
        t.ord[1] = 2;
        t.ord[2] = 1;
    } else if (t.ev0[2] > t.ev0[0]) {
        t.ord[0] = 2;
        t.ord[1] = 0;
        t.ord[2] = 1;
    }
    t.e1 = t.ev0[t.ord[0]];
    t.e2 = t.ev0[t.ord[1]];
    t.e3 = t.ev0[t.ord[2]];
    t.tr = t.e1 + t.e2 + t.e3;
    t.f_tr = 2.0 * G * ((1.0 + s) * t.e1 - (1.0 - s) * t.e3) + 2.0 * lam * s * t.tr - c;
    return t;
}

__device__ __forceinline__ void mc2d_elastic(const double *E, double G, double lam, double *S, double *DS) {
    const double e11 = E[0], e22 = E[1], g12 = E[2];
    const double vt = e11 + e22;  // iota4 . [e11, e22, g12, 0]
    S[0] = lam * vt + 2.0 * G * e11;
    S[1] = lam * vt + 2.0 * G * e22;
    S[2] = 2.0 * G * (0.5 * g12);
    S[3] = lam * vt;
    if (DS) {
        const double io[3] = {1.0, 1.0, 0.0}, hI[3] = {1.0, 1.0, 0.5};
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) DS[i + 3 * j] = io[i] * io[j] * lam + 2.0 * ((i == j) ? hI[i] : 0.0) * G;
    }
}

__device__ int mc2d_point(const double *E, double c, double s, double G, double lam, double *S, double *DS) {
    const Trial2 t = mc2d_trial(E, c, s, G, lam);
    if (t.f_tr <= 0.0) {
        mc2d_elastic(E, G, lam, S, DS);
        return kElastic;
    }
    // projections in [11, 22, 12, 33] representation and their derivatives (3x3 in-plane): the
    // plastic branches only
    const double e11 = E[0], e22 = E[1], g12 = E[2];
    const double rad = t.rad;
    double P0[4], P1[4];
    double dP0[9];
    if (rad != 0.0) {
        P0[0] = (e11 - t.ev0[1]) / rad;
        P0[1] = (e22 - t.ev0[1]) / rad;
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
    double P[3][4], dP[3][9];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int o = t.ord[k];
#pragma unroll
        for (int i = 0; i < 4; ++i) P[k][i] = o == 0 ? P0[i] : (o == 1 ? P1[i] : (i == 3 ? 1.0 : 0.0));
#pragma unroll
        for (int i = 0; i < 9; ++i) dP[k][i] = o == 0 ? dP0[i] : (o == 1 ? -dP0[i] : 0.0);
    }
    const double e1 = t.e1, e2 = t.e2, e3 = t.e3;
    const double tr = t.tr;
    const double f_tr = t.f_tr;
    const double io[3] = {1.0, 1.0, 0.0};
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

// Binned 2D return mapping.  Pass A decides every point's trial state (the closed-form in-plane
// eigenvalues, exactly mc2d_point's arithmetic), finishes the elastic points and lists the others
// (scratch[0] = count, scratch[1..] = points); pass B runs mc2d_point on the listed points only, so
// no warp pays for the projections and the plastic branches of another point.  Same arithmetic as
// mc2d_kernel (same branch codes; values within a few ulps, where the compiler contracts a
// multiply-add into an FMA differently in the two kernels).
__global__ void __launch_bounds__(128) mc2d_screen_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                          const double *__restrict__ sin_phi,
                                                          const double *__restrict__ shear,
                                                          const double *__restrict__ lame, int n,
                                                          double *__restrict__ S, double *__restrict__ DS,
                                                          int8_t *__restrict__ branch, int32_t *__restrict__ scratch) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    bool listed = false;
    if (p < n) {
        const double e[3] = {E[3ll * p], E[3ll * p + 1], E[3ll * p + 2]};
        const double G = shear[p], lam = lame[p];
        const Trial2 t = mc2d_trial(e, c_bar[p], sin_phi[p], G, lam);
        if (t.f_tr <= 0.0) {
            double s[4], ds[9];
            mc2d_elastic(e, G, lam, s, ds);
#pragma unroll
            for (int k = 0; k < 4; ++k) S[4ll * p + k] = s[k];
#pragma unroll
            for (int k = 0; k < 9; ++k) DS[9ll * p + k] = ds[k];
            branch[p] = static_cast<int8_t>(kElastic);
        } else {
            listed = true;
        }
    }
    const int slot = warp_append(listed, scratch);
    if (listed) scratch[1 + slot] = p;
}

__global__ void __launch_bounds__(128) mc2d_list_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                                        const double *__restrict__ sin_phi,
                                                        const double *__restrict__ shear,
                                                        const double *__restrict__ lame, int n,
                                                        double *__restrict__ S, double *__restrict__ DS,
                                                        int8_t *__restrict__ branch,
                                                        const int32_t *__restrict__ scratch) {
    const int cnt = scratch[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int p = scratch[1 + i];
        if (p < 0 || p >= n) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const double e[3] = {E[3ll * p], E[3ll * p + 1], E[3ll * p + 2]};
        double s[4], ds[9];
        branch[p] = static_cast<int8_t>(mc2d_point(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, ds));
#pragma unroll
        for (int k = 0; k < 4; ++k) S[4ll * p + k] = s[k];
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
    // The reference evaluates atan/cos/sin chains; the same quantities follow from tangents
    // alone: for a = atan(t), cos a = 1/sqrt(1+t^2) and sin a = t/sqrt(1+t^2) (|a| < pi/2).  This
    // needs two sincos per point instead of seven transcendental calls.
    const double c = c0[p];
    double sf, cf, sy, cy;
    sincos(phi[p], &sf, &cf);
    sincos(psi[p], &sy, &cy);
    double c_l, T;  // c_lambda and tan(phi_lambda)
    if (davis == 0) {  // A
        const double beta = cf * cy / (1.0 - sf * sy);
        c_l = beta * c / lam;
        T = beta * (sf / cf) / lam;
    } else {
        const double t1 = (sf / cf) / lam;  // tan(phi1)
        const double rf = rsqrt(1.0 + t1 * t1);
        const double c1f = rf, s1f = t1 * rf;  // cos, sin of phi1
        double beta;
        if (davis == 1) {  // B
            const double u1 = (sy / cy) / lam;  // tan(psi1)
            const double ry = rsqrt(1.0 + u1 * u1);
            beta = c1f * ry / (1.0 - s1f * (u1 * ry));
        } else {  // C: phi1 > psi  <=>  tan(phi1) > tan(psi) on (-pi/2, pi/2)
            beta = t1 > sy / cy ? c1f * cy / (1.0 - s1f * sy) : 1.0;
        }
        c_l = beta * (c / lam);
        T = beta * t1;
    }
    const double rT = rsqrt(1.0 + T * T);
    c_bar[p] = 2.0 * c_l * rT;
    sin_phi[p] = T * rT;
}

// Fixed scratch of ssp_constitutive_3d_sds_binned_noalloc: four counters, then three point lists
// of SSP_NOALLOC_MAX_POINTS entries (24 MiB + 16 B per GPU, for the life of the process).
static __device__ __align__(256) int32_t g_fixed_scratch[4 + 3 * SSP_NOALLOC_MAX_POINTS];

constexpr int kMaxDevices = 128;
std::mutex g_fixed_mutex;
int32_t *g_fixed_ptr[kMaxDevices] = {};

// Device address of g_fixed_scratch on the current device.  In host code the symbol's name is a
// host-side stand-in, not a device address, so it is looked up once per device (with that device
// current) and cached; nullptr on failure.  The cache assumes the device's context lives as long as
// the process: after a device reset the address would be stale (documented in the header).
int32_t *fixed_scratch_for_current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_fixed_mutex);
    if (!g_fixed_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_fixed_scratch) != cudaSuccess || !p) return nullptr;
        g_fixed_ptr[dev] = static_cast<int32_t *>(p);
    }
    return g_fixed_ptr[dev];
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

int ssp_constitutive_3d_sds_binned(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                                   const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                                   int32_t *scratch, void *stream) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    return launch_binned(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, false,
                         as_stream(stream));
}

// The binned return mapping of the mixed-precision form: branches, multipliers and S in FP64 as
// above, the plastic points' DS in double-float arithmetic.
int ssp_constitutive_3d_sds_binned_mixed(const double *E, const double *c_bar, const double *sin_phi,
                                         const double *shear, const double *lame, int n_int, double *S_out,
                                         double *DS_out, int8_t *branch_out, int32_t *scratch, void *stream) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    return launch_binned(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, true,
                         as_stream(stream));
}

// Same two-pass return mapping for callers that have no way to allocate device memory: a
// constitutive hook called from inside another solver's assembly loop that is handed device
// pointers to its inputs and outputs only, with all device memory owned and budgeted by the
// host framework (an allocation there would also synchronise the device in the middle of the
// loop).  Its point lists live in the fixed array below, which every GPU that loads this
// library holds until the process exits.
int ssp_constitutive_3d_sds_binned_noalloc(const double *E, const double *c_bar, const double *sin_phi,
                                           const double *shear, const double *lame, int n_int, double *S_out,
                                           double *DS_out, int8_t *branch_out, void *stream) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int > SSP_NOALLOC_MAX_POINTS) return SSP_ERR_TOO_LARGE;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out) return SSP_ERR_INVALID;
    int32_t *scratch = fixed_scratch_for_current_device();
    if (!scratch) return SSP_ERR_CUDA;
    return launch_binned(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, false,
                         as_stream(stream));
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

int ssp_constitutive_2d_sds_binned(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                                   const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                                   int32_t *scratch, void *stream) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(scratch, 0, sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    mc2d_screen_kernel<<<grid_for(n_int, 128), 128, 0, st>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out,
                                                             branch_out, scratch);
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long gx = (long long)sms * 8;  // grid-stride over the listed points (count on the device)
    const long long need = ((long long)n_int + 127) / 128;
    if (gx > need) gx = need;
    mc2d_list_kernel<<<static_cast<unsigned>(gx), 128, 0, st>>>(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out,
                                                                branch_out, scratch);
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
