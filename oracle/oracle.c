/*
 * oracle.c -- CPU restatement of the reference's Newton hot-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product package links or calls
 * this file.  It is used by the tests (the oracle for the CUDA kernels),
 * by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.
 *
 * Every function restates one reference routine (paths relative to the
 * reference project root):
 *
 *   orc_mc3d_point          src/slope_stability/cython/constitutive_3D_kernel.h:68-351
 *   orc_constitutive_3d     src/slope_stability/cython/constitutive_3d_batch.c:9-50
 *   orc_strain_3d           src/slope_stability/cython/assemble_tangent_values_3d.c:216-273
 *   orc_force_rows_3d       src/slope_stability/cython/assemble_tangent_values_3d.c:275-327
 *   orc_tangent_rows_3d     src/slope_stability/cython/assemble_tangent_values_3d.c:111-214
 *   orc_tangent_scatter     src/slope_stability/cython/assemble_tangent_values_3d.c:13-109
 *                           and src/slope_stability/fem/distributed_tangent.py:1437-1484 (2D)
 *   orc_strain_2d           src/slope_stability/fem/assembly.py:96-123 (B rows of the 2D operator)
 *   orc_overlap_force_2d    src/slope_stability/fem/distributed_tangent.py:845-852
 *   orc_geometry_3d         src/slope_stability/fem/assembly.py:139-245 (dphi, weights)
 *   orc_pattern_build       src/slope_stability/fem/distributed_tangent.py:297-478 (owned-row
 *                           CSR, constrained diagonals, row-slot metadata) and
 *                           src/slope_stability/fem/distributed_elastic.py:36-52 (overlap)
 *
 * Parity of this restatement is pinned against the reference's own outputs
 * (golden fixtures generated by tests/golden/make_golden.py).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PI 3.14159265358979323846

/* ------------------------------------------------------------------------ */
/* 3D Mohr-Coulomb return mapping (strain in engineering shear, Voigt order  */
/* [11,22,33,12,23,13]; tangent stored column-major, entry (i,j) at i+6j).   */
/* ------------------------------------------------------------------------ */

static const double VOL_IOTA[6] = {1.0, 1.0, 1.0, 0.0, 0.0, 0.0};
static const double HALF_IDENT[6] = {1.0, 1.0, 1.0, 0.5, 0.5, 0.5};

/* t*t for a symmetric tensor t stored as [11,22,33,12,23,13]. */
static void orc_tensor_square(const double t[6], double sq[6])
{
    sq[0] = t[0] * t[0] + t[3] * t[3] + t[5] * t[5];
    sq[1] = t[1] * t[1] + t[3] * t[3] + t[4] * t[4];
    sq[2] = t[2] * t[2] + t[4] * t[4] + t[5] * t[5];
    sq[3] = t[0] * t[3] + t[1] * t[3] + t[4] * t[5];
    sq[4] = t[3] * t[5] + t[1] * t[4] + t[2] * t[4];
    sq[5] = t[0] * t[5] + t[3] * t[4] + t[2] * t[5];
}

/* Jacobian d(t*t)_i / dE_j where t = HALF_IDENT .* E (constitutive_3D_kernel.h:30-57). */
static void orc_square_jacobian(const double t[6], double J[36])
{
    memset(J, 0, 36 * sizeof(double));
#define JS(i, j, v) do { J[(i) + 6 * (j)] = (v); } while (0)
    JS(0, 0, 2.0 * t[0]); JS(0, 3, t[3]); JS(0, 5, t[5]);
    JS(1, 1, 2.0 * t[1]); JS(1, 3, t[3]); JS(1, 4, t[4]);
    JS(2, 2, 2.0 * t[2]); JS(2, 4, t[4]); JS(2, 5, t[5]);
    JS(3, 0, t[3]); JS(3, 1, t[3]);
    JS(3, 3, 0.5 * (t[0] + t[1])); JS(3, 4, 0.5 * t[5]); JS(3, 5, 0.5 * t[4]);
    JS(4, 1, t[4]); JS(4, 2, t[4]);
    JS(4, 3, 0.5 * t[5]); JS(4, 4, 0.5 * (t[1] + t[2])); JS(4, 5, 0.5 * t[3]);
    JS(5, 0, t[5]); JS(5, 2, t[5]);
    JS(5, 3, 0.5 * t[4]); JS(5, 4, 0.5 * t[3]); JS(5, 5, 0.5 * (t[0] + t[2]));
#undef JS
}

/* Eigenprojection P = (t^2 - (ea+eb) t + ea*eb I) * inv, with ea, eb the other eigenvalues. */
static void orc_projection(const double sq[6], const double t[6], double sum_other,
                           double prod_other, double inv, double P[6])
{
    for (int i = 0; i < 6; ++i)
        P[i] = inv * (sq[i] - sum_other * t[i] + prod_other * VOL_IOTA[i]);
}

void orc_mc3d_point(const double *E, double c_bar, double sin_phi, double shear,
                    double lame, double *S, double *DS)
{
    const double sp = sin_phi; /* associated flow: sin(psi) := sin(phi) (kernel.h:73) */
    double t[6], sq[6];
    for (int i = 0; i < 6; ++i)
        t[i] = HALF_IDENT[i] * E[i];
    orc_tensor_square(t, sq);

    /* invariants and trigonometric principal values (kernel.h:86-112) */
    const double I1 = t[0] + t[1] + t[2];
    const double I2 = t[0] * t[1] + t[0] * t[2] + t[1] * t[2] - t[3] * t[3] - t[4] * t[4] - t[5] * t[5];
    const double I3 = t[0] * t[1] * t[2] - t[2] * t[3] * t[3] - t[1] * t[5] * t[5] - t[0] * t[4] * t[4]
                      + 2.0 * t[3] * t[4] * t[5];
    double Q = (I1 * I1 - 3.0 * I2) / 9.0;
    if (Q < 0.0)
        Q = 0.0;
    const double R = (-2.0 * I1 * I1 * I1 + 9.0 * I1 * I2 - 27.0 * I3) / 54.0;
    const double rq = sqrt(Q);
    double theta = 0.0;
    if (!(Q < 1e-30)) {
        double c = R / (rq * Q);
        c = c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
        theta = acos(c) / 3.0;
    }
    const double e1 = -2.0 * rq * cos(theta + 2.0 * ORC_PI / 3.0) + I1 / 3.0;
    const double e2 = -2.0 * rq * cos(theta - 2.0 * ORC_PI / 3.0) + I1 / 3.0;
    const double e3 = -2.0 * rq * cos(theta) + I1 / 3.0;

    const double f_tr = 2.0 * shear * ((1.0 + sin_phi) * e1 - (1.0 - sin_phi) * e3)
                        + 2.0 * lame * sin_phi * I1 - c_bar;

    if (f_tr <= 0.0) { /* elastic (kernel.h:116-142) */
        for (int i = 0; i < 6; ++i)
            S[i] = lame * I1 * VOL_IOTA[i] + 2.0 * shear * t[i];
        if (DS) {
            for (int j = 0; j < 6; ++j)
                for (int i = 0; i < 6; ++i)
                    DS[i + 6 * j] = lame * VOL_IOTA[i] * VOL_IOTA[j]
                                    + (i == j ? 2.0 * shear * HALF_IDENT[i] : 0.0);
        }
        return;
    }

    const double g_sl = (e1 - e2) / (1.0 + sp);
    const double g_sr = (e2 - e3) / (1.0 - sp);
    const double den_s = 4.0 * lame * sin_phi * sp + 4.0 * shear * (1.0 + sin_phi * sp);
    const double lam_s = f_tr / den_s;

    if (lam_s <= g_sl && lam_s <= g_sr) { /* smooth face (kernel.h:149-209) */
        const double ev[3] = {e1, e2, e3};
        double inv[3], P[3][6], sig[3];
        for (int k = 0; k < 3; ++k) {
            const double ea = ev[(k + 1) % 3], eb = ev[(k + 2) % 3];
            inv[k] = 1.0 / ((ev[k] - ea) * (ev[k] - eb));
            orc_projection(sq, t, ea + eb, ea * eb, inv[k], P[k]);
        }
        sig[0] = lame * I1 + 2.0 * shear * e1 - lam_s * (2.0 * lame * sp + 2.0 * shear * (1.0 + sp));
        sig[1] = lame * I1 + 2.0 * shear * e2 - lam_s * 2.0 * lame * sp;
        sig[2] = lame * I1 + 2.0 * shear * e3 - lam_s * (2.0 * lame * sp - 2.0 * shear * (1.0 - sp));
        for (int i = 0; i < 6; ++i)
            S[i] = sig[0] * P[0][i] + sig[1] * P[1][i] + sig[2] * P[2][i];
        if (DS) {
            double Jsq[36], Dp[6], Dq[6];
            orc_square_jacobian(t, Jsq);
            for (int i = 0; i < 6; ++i) {
                Dp[i] = 2.0 * shear * ((1.0 + sin_phi) * P[0][i] - (1.0 - sin_phi) * P[2][i]) + 2.0 * lame * sin_phi * VOL_IOTA[i];
                Dq[i] = 2.0 * shear * ((1.0 + sp) * P[0][i] - (1.0 - sp) * P[2][i]) + 2.0 * lame * sp * VOL_IOTA[i];
            }
            /* coefficients of the derivative of each projection */
            const double sum_o[3] = {e2 + e3, e1 + e3, e1 + e2};
            const double ca[3] = {2.0 * e1 - e2 - e3, 2.0 * e2 - e1 - e3, 2.0 * e3 - e1 - e2};
            const double cb[3] = {e2 - e3, e1 - e3, e1 - e2};
            for (int j = 0; j < 6; ++j) {
                for (int i = 0; i < 6; ++i) {
                    const int k = i + 6 * j;
                    const double id = (i == j) ? HALF_IDENT[i] : 0.0;
                    const double o[3] = {P[0][i] * P[0][j], P[1][i] * P[1][j], P[2][i] * P[2][j]};
                    const double d1 = inv[0] * (Jsq[k] - id * sum_o[0] - ca[0] * o[0] - cb[0] * (o[1] - o[2]));
                    const double d2 = inv[1] * (Jsq[k] - id * sum_o[1] - ca[1] * o[1] - cb[1] * (o[0] - o[2]));
                    const double d3 = inv[2] * (Jsq[k] - id * sum_o[2] - ca[2] * o[2] - cb[2] * (o[0] - o[1]));
                    DS[k] = sig[0] * d1 + sig[1] * d2 + sig[2] * d3 + lame * VOL_IOTA[i] * VOL_IOTA[j]
                            + 2.0 * shear * (o[0] + o[1] + o[2]) - Dq[i] * Dp[j] * (1.0 / den_s);
                }
            }
        }
        return;
    }

    if (g_sl < g_sr) { /* left edge (kernel.h:211-273) */
        const double den_l = 4.0 * lame * sin_phi * sp + shear * (1.0 + sin_phi) * (1.0 + sp)
                             + 2.0 * shear * (1.0 - sin_phi) * (1.0 - sp);
        const double lam_l = (shear * ((1.0 + sin_phi) * (e1 + e2) - 2.0 * (1.0 - sin_phi) * e3)
                              + 2.0 * lame * sin_phi * I1 - c_bar) / den_l;
        const double g_la = (e1 + e2 - 2.0 * e3) / (3.0 - sp);
        if (lam_l >= g_sl && lam_l <= g_la) {
            const double inv3 = 1.0 / ((e3 - e1) * (e3 - e2));
            double P3[6], P12[6];
            orc_projection(sq, t, e1 + e2, e1 * e2, inv3, P3);
            for (int i = 0; i < 6; ++i)
                P12[i] = VOL_IOTA[i] - P3[i];
            const double s1 = lame * I1 + shear * (e1 + e2) - lam_l * (2.0 * lame * sp + shear * (1.0 + sp));
            const double s3 = lame * I1 + 2.0 * shear * e3 - lam_l * (2.0 * lame * sp - 2.0 * shear * (1.0 - sp));
            for (int i = 0; i < 6; ++i)
                S[i] = s1 * P12[i] + s3 * P3[i];
            if (DS) {
                double Jsq[36], Dp[6], Dq[6];
                orc_square_jacobian(t, Jsq);
                const double e12 = e1 + e2;
                for (int i = 0; i < 6; ++i) {
                    Dp[i] = shear * ((1.0 + sin_phi) * P12[i] - 2.0 * (1.0 - sin_phi) * P3[i]) + 2.0 * lame * sin_phi * VOL_IOTA[i];
                    Dq[i] = shear * ((1.0 + sp) * P12[i] - 2.0 * (1.0 - sp) * P3[i]) + 2.0 * lame * sp * VOL_IOTA[i];
                }
                for (int j = 0; j < 6; ++j) {
                    for (int i = 0; i < 6; ++i) {
                        const int k = i + 6 * j;
                        const double id = (i == j) ? HALF_IDENT[i] : 0.0;
                        const double o33 = P3[i] * P3[j];
                        const double oAA = P12[i] * P12[j];
                        const double d3 = inv3 * (Jsq[k] - id * e12 - (P12[i] * t[j] + t[i] * P12[j]) + e12 * oAA
                                                  + (e12 - 2.0 * e3) * o33 + e3 * (P12[i] * P3[j] + P3[i] * P12[j]));
                        DS[k] = (s3 - s1) * d3 + lame * VOL_IOTA[i] * VOL_IOTA[j] + shear * (oAA + 2.0 * o33)
                                - Dq[i] * Dp[j] * (1.0 / den_l);
                    }
                }
            }
            return;
        }
    }

    if (g_sl > g_sr) { /* right edge (kernel.h:275-338) */
        const double den_r = 4.0 * lame * sin_phi * sp + 2.0 * shear * (1.0 + sin_phi) * (1.0 + sp)
                             + shear * (1.0 - sin_phi) * (1.0 - sp);
        const double lam_r = (shear * (2.0 * (1.0 + sin_phi) * e1 - (1.0 - sin_phi) * (e2 + e3))
                              + 2.0 * lame * sin_phi * I1 - c_bar) / den_r;
        const double g_ra = (2.0 * e1 - e2 - e3) / (3.0 + sp);
        if (lam_r >= g_sr && lam_r <= g_ra) {
            const double inv1 = 1.0 / ((e1 - e2) * (e1 - e3));
            double P1[6], P23[6];
            orc_projection(sq, t, e2 + e3, e2 * e3, inv1, P1);
            for (int i = 0; i < 6; ++i)
                P23[i] = VOL_IOTA[i] - P1[i];
            const double s1 = lame * I1 + 2.0 * shear * e1 - lam_r * (2.0 * lame * sp + 2.0 * shear * (1.0 + sp));
            const double s3 = lame * I1 + shear * (e2 + e3) - lam_r * (2.0 * lame * sp - shear * (1.0 - sp));
            for (int i = 0; i < 6; ++i)
                S[i] = s1 * P1[i] + s3 * P23[i];
            if (DS) {
                double Jsq[36], Dp[6], Dq[6];
                orc_square_jacobian(t, Jsq);
                const double e23 = e2 + e3;
                for (int i = 0; i < 6; ++i) {
                    Dp[i] = shear * (2.0 * (1.0 + sin_phi) * P1[i] - (1.0 - sin_phi) * P23[i]) + 2.0 * lame * sin_phi * VOL_IOTA[i];
                    Dq[i] = shear * (2.0 * (1.0 + sp) * P1[i] - (1.0 - sp) * P23[i]) + 2.0 * lame * sp * VOL_IOTA[i];
                }
                for (int j = 0; j < 6; ++j) {
                    for (int i = 0; i < 6; ++i) {
                        const int k = i + 6 * j;
                        const double id = (i == j) ? HALF_IDENT[i] : 0.0;
                        const double o11 = P1[i] * P1[j];
                        const double oBB = P23[i] * P23[j];
                        const double d1 = inv1 * (Jsq[k] - id * e23 - (P23[i] * t[j] + t[i] * P23[j]) + e23 * oBB
                                                  + (e23 - 2.0 * e1) * o11 + e1 * (P23[i] * P1[j] + P1[i] * P23[j]));
                        DS[k] = (s1 - s3) * d1 + lame * VOL_IOTA[i] * VOL_IOTA[j] + shear * (2.0 * o11 + oBB)
                                - Dq[i] * Dp[j] * (1.0 / den_r);
                    }
                }
            }
            return;
        }
    }

    /* apex (kernel.h:340-350) */
    {
        const double sa = c_bar / (2.0 * sin_phi);
        for (int i = 0; i < 6; ++i)
            S[i] = sa * VOL_IOTA[i];
        if (DS)
            memset(DS, 0, 36 * sizeof(double));
    }
}

/* Batch driver over AoS arrays E[n][6] -> S[n][6], DS[n][36] (DS may be NULL).
 * `bulk` is accepted for signature parity and unused, as in the reference. */
void orc_constitutive_3d(const double *E, const double *c_bar, const double *sin_phi,
                         const double *shear, const double *bulk, const double *lame,
                         int n_int, double *S, double *DS)
{
    (void)bulk;
#pragma omp parallel for schedule(static)
    for (int p = 0; p < n_int; ++p)
        orc_mc3d_point(E + (size_t)6 * p, c_bar[p], sin_phi[p], shear[p], lame[p],
                       S + (size_t)6 * p, DS ? DS + (size_t)36 * p : NULL);
}

/* ------------------------------------------------------------------------ */
/* 3D assembly restatements.                                                */
/* ------------------------------------------------------------------------ */

/* E[g][6] = B_g u for every point of every element (assemble_tangent_values_3d.c:216-273). */
void orc_strain_3d(const double *dphi1, const double *dphi2, const double *dphi3,
                   const double *u, const int32_t *dof, int n_elem, int n_p, int n_q, double *E)
{
#pragma omp parallel for schedule(static)
    for (int e = 0; e < n_elem; ++e) {
        const int32_t *d = dof + (size_t)e * 3 * n_p;
        for (int q = 0; q < n_q; ++q) {
            const size_t g = (size_t)e * n_q + q;
            double acc[6] = {0, 0, 0, 0, 0, 0};
            for (int a = 0; a < n_p; ++a) {
                const double gx = dphi1[g * n_p + a], gy = dphi2[g * n_p + a], gz = dphi3[g * n_p + a];
                const double ux = u[d[3 * a]], uy = u[d[3 * a + 1]], uz = u[d[3 * a + 2]];
                acc[0] += gx * ux;
                acc[1] += gy * uy;
                acc[2] += gz * uz;
                acc[3] += gy * ux + gx * uy;
                acc[4] += gz * uy + gy * uz;
                acc[5] += gz * ux + gx * uz;
            }
            memcpy(E + 6 * g, acc, sizeof(acc));
        }
    }
}

/* Row r of B_g^T s for a local dof alpha = 3*node + comp. */
static inline double orc_bt_row(int comp, double gx, double gy, double gz, const double *s)
{
    if (comp == 0)
        return gx * s[0] + gy * s[3] + gz * s[5];
    if (comp == 1)
        return gx * s[3] + gy * s[1] + gz * s[4];
    return gx * s[5] + gy * s[4] + gz * s[2];
}

/* Owned force F[row] = sum over the row's slots of B^T (w S) (assemble_tangent_values_3d.c:275-327).
 * Rows without slots (constrained) come out as 0. */
void orc_force_rows_3d(const double *dphi1, const double *dphi2, const double *dphi3,
                       const double *S, const double *w, const int32_t *row_slot_ptr,
                       const int32_t *slot_elem, const uint8_t *slot_lrow,
                       int n_rows, int n_p, int n_q, double *F)
{
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n_rows; ++r) {
        double acc = 0.0;
        for (int s = row_slot_ptr[r]; s < row_slot_ptr[r + 1]; ++s) {
            const int e = slot_elem[s], node = slot_lrow[s] / 3, comp = slot_lrow[s] % 3;
            for (int q = 0; q < n_q; ++q) {
                const size_t g = (size_t)e * n_q + q;
                acc += w[g] * orc_bt_row(comp, dphi1[g * n_p + node], dphi2[g * n_p + node],
                                         dphi3[g * n_p + node], S + 6 * g);
            }
        }
        F[r] = acc;
    }
}

/* t_m = w * (B^T DS)[alpha][m] for one point (assemble_tangent_values_3d.c:162-190). */
static void orc_bt_d(int comp, double gx, double gy, double gz, double w, const double *ds, double t[6])
{
    /* column m of DS is ds[6m .. 6m+5]; B^T row alpha picks Voigt rows by component */
    for (int m = 0; m < 6; ++m)
        t[m] = w * orc_bt_row(comp, gx, gy, gz, ds + 6 * m);
}

/* CSR values of owned rows via row slots (assemble_tangent_values_3d.c:111-214).
 * `values` must be zeroed by the caller; constrained diagonals are not touched. */
void orc_tangent_rows_3d(const double *dphi1, const double *dphi2, const double *dphi3,
                         const double *DS, const double *w, const int32_t *row_slot_ptr,
                         const int32_t *slot_elem, const uint8_t *slot_lrow, const int32_t *slot_pos,
                         int n_rows, int n_p, int n_q, double *values)
{
    const int nld = 3 * n_p;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n_rows; ++r) {
        for (int s = row_slot_ptr[r]; s < row_slot_ptr[r + 1]; ++s) {
            const int e = slot_elem[s], node = slot_lrow[s] / 3, comp = slot_lrow[s] % 3;
            const int32_t *pos = slot_pos + (size_t)s * nld;
            for (int q = 0; q < n_q; ++q) {
                const size_t g = (size_t)e * n_q + q;
                const double *d1 = dphi1 + g * n_p, *d2 = dphi2 + g * n_p, *d3 = dphi3 + g * n_p;
                double t[6];
                orc_bt_d(comp, d1[node], d2[node], d3[node], w[g], DS + 36 * g, t);
                for (int b = 0; b < n_p; ++b) {
                    const double bx = d1[b], by = d2[b], bz = d3[b];
                    if (pos[3 * b] >= 0)
                        values[pos[3 * b]] += t[0] * bx + t[3] * by + t[5] * bz;
                    if (pos[3 * b + 1] >= 0)
                        values[pos[3 * b + 1]] += t[3] * bx + t[1] * by + t[4] * bz;
                    if (pos[3 * b + 2] >= 0)
                        values[pos[3 * b + 2]] += t[5] * bx + t[4] * by + t[2] * bz;
                }
            }
        }
    }
}

/* Strain-displacement matrix of one point: B[k][c] for k < n_strain, c < dim*n_p. */
static void orc_point_B(int dim, int n_p, const double *d1, const double *d2, const double *d3, double *B)
{
    const int nld = dim * n_p;
    const int ns = dim == 3 ? 6 : 3;
    memset(B, 0, (size_t)ns * nld * sizeof(double));
    for (int a = 0; a < n_p; ++a) {
        const int c = dim * a;
        if (dim == 3) {
            B[0 * nld + c] = d1[a];
            B[1 * nld + c + 1] = d2[a];
            B[2 * nld + c + 2] = d3[a];
            B[3 * nld + c] = d2[a];
            B[3 * nld + c + 1] = d1[a];
            B[4 * nld + c + 1] = d3[a];
            B[4 * nld + c + 2] = d2[a];
            B[5 * nld + c] = d3[a];
            B[5 * nld + c + 2] = d1[a];
        } else {
            B[0 * nld + c] = d1[a];
            B[1 * nld + c + 1] = d2[a];
            B[2 * nld + c] = d2[a];
            B[2 * nld + c + 1] = d1[a];
        }
    }
}

/* Element-dense k_e = sum_q B^T (w D) B scattered through scatter_map[e][(dim n_p)^2]
 * (assemble_tangent_values_3d.c:13-109; 2D: distributed_tangent.py:1437-1484).
 * DS is AoS [n_int][ns*ns], column-major per point.  Serial (deterministic). */
void orc_tangent_scatter(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                         const double *DS, const double *w, const int32_t *scatter_map,
                         int n_elem, int n_p, int n_q, double *values, double *work)
{
    const int nld = dim * n_p, ns = dim == 3 ? 6 : 3;
    double *ke = work;                       /* nld*nld */
    double *B = ke + (size_t)nld * nld;      /* ns*nld  */
    double *DB = B + (size_t)ns * nld;       /* ns*nld  */
    for (int e = 0; e < n_elem; ++e) {
        memset(ke, 0, (size_t)nld * nld * sizeof(double));
        for (int q = 0; q < n_q; ++q) {
            const size_t g = (size_t)e * n_q + q;
            orc_point_B(dim, n_p, dphi1 + g * n_p, dphi2 + g * n_p, dim == 3 ? dphi3 + g * n_p : NULL, B);
            const double *D = DS + (size_t)ns * ns * g;
            for (int i = 0; i < ns; ++i)
                for (int c = 0; c < nld; ++c) {
                    double acc = 0.0;
                    for (int k = 0; k < ns; ++k)
                        acc += (w[g] * D[i + ns * k]) * B[k * nld + c];
                    DB[i * nld + c] = acc;
                }
            for (int a = 0; a < nld; ++a)
                for (int c = 0; c < nld; ++c) {
                    double acc = 0.0;
                    for (int k = 0; k < ns; ++k)
                        acc += B[k * nld + a] * DB[k * nld + c];
                    ke[a * nld + c] += acc;
                }
        }
        const int32_t *sm = scatter_map + (size_t)e * nld * nld;
        for (int k = 0; k < nld * nld; ++k)
            if (sm[k] >= 0)
                values[sm[k]] += ke[k];
    }
}

/* 2D strain [e11, e22, gamma12] per point from element dofs (assembly.py:96-123). */
void orc_strain_2d(const double *dphi1, const double *dphi2, const double *u, const int32_t *dof,
                   int n_elem, int n_p, int n_q, double *E)
{
    for (int e = 0; e < n_elem; ++e) {
        const int32_t *d = dof + (size_t)e * 2 * n_p;
        for (int q = 0; q < n_q; ++q) {
            const size_t g = (size_t)e * n_q + q;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0;
            for (int a = 0; a < n_p; ++a) {
                const double gx = dphi1[g * n_p + a], gy = dphi2[g * n_p + a];
                const double ux = u[d[2 * a]], uy = u[d[2 * a + 1]];
                a0 += gx * ux;
                a1 += gy * uy;
                a2 += gy * ux + gx * uy;
            }
            E[3 * g] = a0;
            E[3 * g + 1] = a1;
            E[3 * g + 2] = a2;
        }
    }
}

/* Overlap force B^T (w S) in 2D accumulated on overlap dofs (distributed_tangent.py:845-852).
 * S is AoS [n_int][3]; out has n_overlap_dofs entries and must be zeroed by the caller. */
void orc_overlap_force_2d(const double *dphi1, const double *dphi2, const double *S, const double *w,
                          const int32_t *dof, int n_elem, int n_p, int n_q, double *out)
{
    for (int e = 0; e < n_elem; ++e) {
        const int32_t *d = dof + (size_t)e * 2 * n_p;
        for (int q = 0; q < n_q; ++q) {
            const size_t g = (size_t)e * n_q + q;
            const double *s = S + 3 * g;
            for (int a = 0; a < n_p; ++a) {
                const double gx = dphi1[g * n_p + a], gy = dphi2[g * n_p + a];
                out[d[2 * a]] += w[g] * (gx * s[0] + gy * s[2]);
                out[d[2 * a + 1]] += w[g] * (gy * s[1] + gx * s[2]);
            }
        }
    }
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* 3D geometry: per-point gradients dphi = J^{-T} dhat and weights          */
/* w = wf |det J| (assembly.py:167-197, 232), J[r][c] = sum_a x_c(a) dhat_r. */
/* coord [3][n_nodes]; elem [n_el][n_p] (node ids); dhat [3][n_p][n_q];     */
/* outputs dphi_k [n_el*n_q][n_p], w [n_el*n_q].                            */
/* ------------------------------------------------------------------------ */

void orc_geometry_3d(const double *coord, int64_t n_nodes, const int64_t *elem, int64_t n_el, int n_p,
                     int n_q, const double *dhat, const double *wf, double *dphi1, double *dphi2,
                     double *dphi3, double *w)
{
    const double *X = coord, *Y = coord + n_nodes, *Z = coord + 2 * n_nodes;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < n_el; ++e) {
        const int64_t *nd = elem + e * n_p;
        for (int q = 0; q < n_q; ++q) {
            double j11 = 0, j12 = 0, j13 = 0, j21 = 0, j22 = 0, j23 = 0, j31 = 0, j32 = 0, j33 = 0;
            for (int a = 0; a < n_p; ++a) {
                const double x = X[nd[a]], y = Y[nd[a]], z = Z[nd[a]];
                const double h1 = dhat[(0 * n_p + a) * n_q + q], h2 = dhat[(1 * n_p + a) * n_q + q],
                             h3 = dhat[(2 * n_p + a) * n_q + q];
                j11 += x * h1; j12 += y * h1; j13 += z * h1;
                j21 += x * h2; j22 += y * h2; j23 += z * h2;
                j31 += x * h3; j32 += y * h3; j33 += z * h3;
            }
            const double det = j11 * (j22 * j33 - j23 * j32) - j12 * (j21 * j33 - j23 * j31) +
                               j13 * (j21 * j32 - j22 * j31);
            const double inv = 1.0 / det;
            const int64_t g = e * n_q + q;
            for (int a = 0; a < n_p; ++a) {
                const double h1 = dhat[(0 * n_p + a) * n_q + q], h2 = dhat[(1 * n_p + a) * n_q + q],
                             h3 = dhat[(2 * n_p + a) * n_q + q];
                dphi1[g * n_p + a] = ((j22 * j33 - j23 * j32) * h1 - (j12 * j33 - j13 * j32) * h2 +
                                      (j12 * j23 - j13 * j22) * h3) * inv;
                dphi2[g * n_p + a] = (-(j21 * j33 - j23 * j31) * h1 + (j11 * j33 - j13 * j31) * h2 -
                                      (j11 * j23 - j13 * j21) * h3) * inv;
                dphi3[g * n_p + a] = ((j21 * j32 - j22 * j31) * h1 - (j11 * j32 - j12 * j31) * h2 +
                                      (j11 * j22 - j12 * j21) * h3) * inv;
            }
            w[g] = wf[q] * fabs(det);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Owned-row pattern.  The reference builds it with Python sets and dicts:   */
/*  - overlap elements: every element with a node in [n0, n1), ascending;    */
/*  - a free owned row holds the free dofs of every overlap element that     */
/*    has the row's dof, sorted; a constrained owned row only its diagonal;  */
/*  - constrained_diag_positions: the diagonal's position per constrained    */
/*    owned row, in row order;                                               */
/*  - row slots: per free owned row, one slot per overlap element with the   */
/*    row's dof, in element order: (element, local dof a, positions of the   */
/*    element's free dofs in the row, -1 for constrained ones).              */
/* A free row's dof belongs to one node, and the elements with that dof are  */
/* the elements of that node, so the columns are the free dofs of the nodes  */
/* of the node's elements: the same sets, gathered per node.                 */
/* ------------------------------------------------------------------------ */

typedef struct {
    int dim, n_p;
    int64_t n_ov, n_ovn, n_rows, nnz, n_slots, n_cd;
    int64_t *overlap_elements, *overlap_nodes;
    int32_t *dof_lids, *indptr, *indices, *row_slot_ptr, *slot_elem, *slot_pos, *cdiag;
    uint8_t *slot_lrow;
} orc_pattern;

static int orc_cmp_i64(const void *a, const void *b)
{
    const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* sorted distinct nodes of the elements of owned node v (adjacency adj[ap[v]..ap[v+1]]) into buf */
static int64_t orc_node_set(const int64_t *elem, int n_p, const int64_t *ov, const int32_t *adj,
                            const int64_t *ap, int64_t v, int64_t *buf)
{
    int64_t m = 0;
    for (int64_t k = ap[v]; k < ap[v + 1]; ++k) {
        const int64_t *nd = elem + ov[adj[k]] * n_p;
        for (int a = 0; a < n_p; ++a)
            buf[m++] = nd[a];
    }
    qsort(buf, (size_t)m, sizeof(int64_t), orc_cmp_i64);
    int64_t u = 0;
    for (int64_t i = 0; i < m; ++i)
        if (u == 0 || buf[i] != buf[u - 1])
            buf[u++] = buf[i];
    return u;
}

static int32_t orc_find(const int32_t *a, int32_t lo, int32_t hi, int32_t key)
{
    while (lo < hi) {
        const int32_t mid = lo + (hi - lo) / 2;
        if (a[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

void orc_pattern_free(void *h)
{
    orc_pattern *p = (orc_pattern *)h;
    if (!p)
        return;
    free(p->overlap_elements); free(p->overlap_nodes); free(p->dof_lids); free(p->indptr);
    free(p->indices); free(p->row_slot_ptr); free(p->slot_elem); free(p->slot_pos); free(p->cdiag);
    free(p->slot_lrow);
    free(p);
}

/* elem: [n_elem][n_p] node ids (element-major); free_dof: [dim * n_nodes], dof = dim*node + comp.
 * Returns a handle (NULL on allocation failure or an index beyond int32). */
void *orc_pattern_build(int dim, int64_t n_nodes, int n_p, int64_t n_elem, const int64_t *elem,
                        const uint8_t *free_dof, int64_t n0, int64_t n1)
{
    orc_pattern *p = (orc_pattern *)calloc(1, sizeof(orc_pattern));
    if (!p)
        return NULL;
    p->dim = dim;
    p->n_p = n_p;
    const int nld = dim * n_p;
    const int64_t n_own = n1 - n0;
    /* overlap elements and nodes */
    int64_t n_ov = 0;
    for (int64_t e = 0; e < n_elem; ++e)
        for (int a = 0; a < n_p; ++a)
            if (elem[e * n_p + a] >= n0 && elem[e * n_p + a] < n1) { ++n_ov; break; }
    p->n_ov = n_ov;
    p->overlap_elements = (int64_t *)malloc((size_t)(n_ov ? n_ov : 1) * sizeof(int64_t));
    int64_t *lid = (int64_t *)malloc((size_t)(n_nodes ? n_nodes : 1) * sizeof(int64_t));
    if (!p->overlap_elements || !lid) { free(lid); orc_pattern_free(p); return NULL; }
    n_ov = 0;
    for (int64_t e = 0; e < n_elem; ++e)
        for (int a = 0; a < n_p; ++a)
            if (elem[e * n_p + a] >= n0 && elem[e * n_p + a] < n1) { p->overlap_elements[n_ov++] = e; break; }
    for (int64_t v = 0; v < n_nodes; ++v)
        lid[v] = -1;
    for (int64_t k = 0; k < n_ov; ++k)
        for (int a = 0; a < n_p; ++a)
            lid[elem[p->overlap_elements[k] * n_p + a]] = 0;
    int64_t n_ovn = 0;
    for (int64_t v = 0; v < n_nodes; ++v)
        if (lid[v] == 0)
            lid[v] = n_ovn++;
    p->n_ovn = n_ovn;
    p->overlap_nodes = (int64_t *)malloc((size_t)(n_ovn ? n_ovn : 1) * sizeof(int64_t));
    p->dof_lids = (int32_t *)malloc((size_t)(n_ov ? n_ov : 1) * nld * sizeof(int32_t));
    if (!p->overlap_nodes || !p->dof_lids) { free(lid); orc_pattern_free(p); return NULL; }
    for (int64_t v = 0; v < n_nodes; ++v)
        if (lid[v] >= 0)
            p->overlap_nodes[lid[v]] = v;
    for (int64_t k = 0; k < n_ov; ++k)
        for (int a = 0; a < n_p; ++a)
            for (int c = 0; c < dim; ++c)
                p->dof_lids[k * nld + dim * a + c] = (int32_t)(dim * lid[elem[p->overlap_elements[k] * n_p + a]] + c);
    free(lid);

    /* owned node -> overlap elements (ascending) */
    int64_t *ap = (int64_t *)calloc((size_t)n_own + 1, sizeof(int64_t));
    if (!ap) { orc_pattern_free(p); return NULL; }
    for (int64_t k = 0; k < n_ov; ++k)
        for (int a = 0; a < n_p; ++a) {
            const int64_t v = elem[p->overlap_elements[k] * n_p + a];
            if (v >= n0 && v < n1)
                ap[v - n0 + 1]++;
        }
    for (int64_t v = 0; v < n_own; ++v)
        ap[v + 1] += ap[v];
    int32_t *adj = (int32_t *)malloc((size_t)(ap[n_own] ? ap[n_own] : 1) * sizeof(int32_t));
    int64_t *fill = (int64_t *)malloc((size_t)(n_own ? n_own : 1) * sizeof(int64_t));
    if (!adj || !fill) { free(ap); free(adj); free(fill); orc_pattern_free(p); return NULL; }
    memcpy(fill, ap, (size_t)n_own * sizeof(int64_t));
    for (int64_t k = 0; k < n_ov; ++k)
        for (int a = 0; a < n_p; ++a) {
            const int64_t v = elem[p->overlap_elements[k] * n_p + a];
            if (v >= n0 && v < n1)
                adj[fill[v - n0]++] = (int32_t)k;
        }
    free(fill);
    int64_t max_deg = 0;
    for (int64_t v = 0; v < n_own; ++v)
        if (ap[v + 1] - ap[v] > max_deg)
            max_deg = ap[v + 1] - ap[v];

    /* row lengths */
    const int64_t n_rows = dim * n_own;
    p->n_rows = n_rows;
    int64_t *rlen = (int64_t *)calloc((size_t)n_rows + 1, sizeof(int64_t));
    if (!rlen) { free(ap); free(adj); orc_pattern_free(p); return NULL; }
    int failed = 0;
#pragma omp parallel
    {
        int64_t *buf = (int64_t *)malloc((size_t)(max_deg * n_p + 1) * sizeof(int64_t));
        if (!buf) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 1024)
        for (int64_t v = 0; v < n_own; ++v) {
            if (!buf)
                continue;
            const int64_t m = orc_node_set(elem, n_p, p->overlap_elements, adj, ap, v, buf);
            int64_t nfree = 0;
            for (int64_t i = 0; i < m; ++i)
                for (int c = 0; c < dim; ++c)
                    nfree += free_dof[dim * buf[i] + c] != 0;
            for (int c = 0; c < dim; ++c)
                rlen[dim * v + c + 1] = free_dof[dim * (n0 + v) + c] ? nfree : 1;
        }
        free(buf);
    }
    for (int64_t r = 0; r < n_rows; ++r)
        rlen[r + 1] += rlen[r];
    p->nnz = rlen[n_rows];
    if (failed || p->nnz > INT32_MAX) { free(rlen); free(ap); free(adj); orc_pattern_free(p); return NULL; }
    p->indptr = (int32_t *)malloc((size_t)(n_rows + 1) * sizeof(int32_t));
    p->indices = (int32_t *)malloc((size_t)(p->nnz ? p->nnz : 1) * sizeof(int32_t));
    if (!p->indptr || !p->indices) { free(rlen); free(ap); free(adj); orc_pattern_free(p); return NULL; }
    for (int64_t r = 0; r <= n_rows; ++r)
        p->indptr[r] = (int32_t)rlen[r];
    free(rlen);
#pragma omp parallel
    {
        int64_t *buf = (int64_t *)malloc((size_t)(max_deg * n_p + 1) * sizeof(int64_t));
        if (!buf) {
#pragma omp atomic write
            failed = 1;
        }
#pragma omp for schedule(dynamic, 1024)
        for (int64_t v = 0; v < n_own; ++v) {
            if (!buf)
                continue;
            const int64_t m = orc_node_set(elem, n_p, p->overlap_elements, adj, ap, v, buf);
            for (int c = 0; c < dim; ++c) {
                const int64_t r = dim * v + c, gr = dim * (n0 + v) + c;
                int32_t *out = p->indices + p->indptr[r];
                if (!free_dof[gr]) {
                    out[0] = (int32_t)gr;
                    continue;
                }
                int64_t o = 0;
                for (int64_t i = 0; i < m; ++i)
                    for (int c2 = 0; c2 < dim; ++c2)
                        if (free_dof[dim * buf[i] + c2])
                            out[o++] = (int32_t)(dim * buf[i] + c2);
            }
        }
        free(buf);
    }
    if (failed) { free(ap); free(adj); orc_pattern_free(p); return NULL; }

    /* constrained diagonals, in row order */
    int64_t n_cd = 0;
    for (int64_t r = 0; r < n_rows; ++r)
        n_cd += !free_dof[dim * n0 + r];
    p->n_cd = n_cd;
    p->cdiag = (int32_t *)malloc((size_t)(n_cd ? n_cd : 1) * sizeof(int32_t));
    p->row_slot_ptr = (int32_t *)malloc((size_t)(n_rows + 1) * sizeof(int32_t));
    if (!p->cdiag || !p->row_slot_ptr) { free(ap); free(adj); orc_pattern_free(p); return NULL; }
    n_cd = 0;
    for (int64_t r = 0; r < n_rows; ++r)
        if (!free_dof[dim * n0 + r])
            p->cdiag[n_cd++] = p->indptr[r];

    /* row slots: a free row gets one slot per element of its node, in element order */
    int64_t ns = 0;
    p->row_slot_ptr[0] = 0;
    for (int64_t r = 0; r < n_rows; ++r) {
        if (free_dof[dim * n0 + r])
            ns += ap[r / dim + 1] - ap[r / dim];
        if (ns > INT32_MAX) { free(ap); free(adj); orc_pattern_free(p); return NULL; }
        p->row_slot_ptr[r + 1] = (int32_t)ns;
    }
    p->n_slots = ns;
    p->slot_elem = (int32_t *)malloc((size_t)(ns ? ns : 1) * sizeof(int32_t));
    p->slot_lrow = (uint8_t *)malloc((size_t)(ns ? ns : 1));
    p->slot_pos = (int32_t *)malloc((size_t)(ns ? ns : 1) * nld * sizeof(int32_t));
    if (!p->slot_elem || !p->slot_lrow || !p->slot_pos) { free(ap); free(adj); orc_pattern_free(p); return NULL; }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t r = 0; r < n_rows; ++r) {
        const int64_t v = r / dim, c = r % dim, gv = n0 + v;
        if (!free_dof[dim * gv + c])
            continue;
        int64_t s = p->row_slot_ptr[r];
        for (int64_t k = ap[v]; k < ap[v + 1]; ++k, ++s) {
            const int64_t *nd = elem + p->overlap_elements[adj[k]] * n_p;
            int a_loc = 0;
            while (nd[a_loc] != gv)
                ++a_loc;
            p->slot_elem[s] = adj[k];
            p->slot_lrow[s] = (uint8_t)(dim * a_loc + c);
            int32_t *pos = p->slot_pos + s * nld;
            for (int b = 0; b < n_p; ++b)
                for (int c2 = 0; c2 < dim; ++c2) {
                    const int64_t col = dim * nd[b] + c2;
                    pos[dim * b + c2] = free_dof[col]
                        ? orc_find(p->indices, p->indptr[r], p->indptr[r + 1], (int32_t)col) : -1;
                }
        }
    }
    free(ap);
    free(adj);
    return p;
}

/* sizes: n_ov, n_ovn, n_rows, nnz, n_slots, n_cd */
void orc_pattern_sizes(const void *h, int64_t *out)
{
    const orc_pattern *p = (const orc_pattern *)h;
    out[0] = p->n_ov; out[1] = p->n_ovn; out[2] = p->n_rows; out[3] = p->nnz; out[4] = p->n_slots;
    out[5] = p->n_cd;
}

/* copy one array out: 0 overlap_elements, 1 overlap_nodes, 2 dof_lids, 3 indptr, 4 indices,
 * 5 constrained_diag_positions, 6 row_slot_ptr, 7 slot_elem, 8 slot_lrow, 9 slot_pos */
void orc_pattern_copy(const void *h, int which, void *dst)
{
    const orc_pattern *p = (const orc_pattern *)h;
    const int nld = p->dim * p->n_p;
    switch (which) {
    case 0: memcpy(dst, p->overlap_elements, (size_t)p->n_ov * sizeof(int64_t)); break;
    case 1: memcpy(dst, p->overlap_nodes, (size_t)p->n_ovn * sizeof(int64_t)); break;
    case 2: memcpy(dst, p->dof_lids, (size_t)p->n_ov * nld * sizeof(int32_t)); break;
    case 3: memcpy(dst, p->indptr, (size_t)(p->n_rows + 1) * sizeof(int32_t)); break;
    case 4: memcpy(dst, p->indices, (size_t)p->nnz * sizeof(int32_t)); break;
    case 5: memcpy(dst, p->cdiag, (size_t)p->n_cd * sizeof(int32_t)); break;
    case 6: memcpy(dst, p->row_slot_ptr, (size_t)(p->n_rows + 1) * sizeof(int32_t)); break;
    case 7: memcpy(dst, p->slot_elem, (size_t)p->n_slots * sizeof(int32_t)); break;
    case 8: memcpy(dst, p->slot_lrow, (size_t)p->n_slots); break;
    case 9: memcpy(dst, p->slot_pos, (size_t)p->n_slots * nld * sizeof(int32_t)); break;
    default: break;
    }
}
