// Strain and internal force of the mixed-precision form in compensated FP32 arithmetic.
//
// GB300 issues FP64 at a small fraction of its FP32 rate, and the FP64 strain E = B u and force
// F = B^T (w S) kernels (assembly.cu) run at 82-86 % of the FP64 pipe.  Here the same sums are
// formed in double-float arithmetic on the FP32 pipe (inputs split into hi + lo float pairs by bit
// operations; every product's rounding error recovered with an FMA, the sums kept as an unevaluated
// hi + lo pair), about 46 significant bits, and widened to FP64 once per output.
//
// The FP64 inputs are split once where they are constant (the gradients dphi and w * dphi, once per
// pattern, ssp_split_f64), once per call otherwise (the overlap displacements), and the stresses
// by the force kernel's blocks into shared memory.
//
// Strain: with sum_a grad N_a = 0, E = sum_a dphi_a (x) (u_a - u_0), node 0 of the element as the
// reference displacement.  The differences remove the rigid translation of the element, so the
// products are of the size of the strain itself and the compensated sum keeps its relative
// accuracy (a plain FP32 sum of dphi_a u_a would cancel three or more digits).
//
// Force: one thread per (element, local dof) as force_element_kernel; the element sum over the
// quadrature points is compensated and added to the FP64 force vector with one FP64 reduction.
#include "ssp_internal.cuh"

namespace ssp {
namespace {

__device__ __forceinline__ df32 df_neg(df32 a) { return {-a.hi, -a.lo}; }

// out[i] = hi + lo split of x[i] * (scale ? scale[i / group] : 1), the product in FP64.
__global__ void split_kernel(const double *__restrict__ x, const double *__restrict__ scale, long long n, int group,
                             float2 *__restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = scale ? x[i] * scale[i / group] : x[i];
    const df32 d = df_from_f64(v);
    out[i] = make_float2(d.hi, d.lo);
}

__device__ __forceinline__ df32 ld(const float2 *p) {
    const float2 v = *p;
    return {v.x, v.y};
}

// Strain from hi + lo pairs of the gradients (split once per pattern) and of the overlap
// displacements (split once per call).
__global__ void __launch_bounds__(128) strain3_mixed_kernel(const float2 *__restrict__ g1, const float2 *__restrict__ g2,
                                                            const float2 *__restrict__ g3,
                                                            const float2 *__restrict__ u,
                                                            const int32_t *__restrict__ dof, long long n_u, int n_elem,
                                                            int n_p, int n_q, double *__restrict__ E) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)n_elem * n_q) return;
    const long long e = g / n_q;
    const int32_t *dl = dof + e * 3 * n_p;
    const int32_t r0 = dl[0], r1 = dl[1], r2 = dl[2];
    if (r0 < 0 || r1 < 0 || r2 < 0 || r0 >= n_u || r1 >= n_u || r2 >= n_u) {
        flag(SSP_DEV_BAD_INDEX);
        return;
    }
    const df32 u0x = df_neg(ld(u + r0)), u0y = df_neg(ld(u + r1)), u0z = df_neg(ld(u + r2));
    CSum a0, a1, a2, a3, a4, a5;
    for (int a = 1; a < n_p; ++a) {
        const int32_t i0 = dl[3 * a], i1 = dl[3 * a + 1], i2 = dl[3 * a + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= n_u || i1 >= n_u || i2 >= n_u) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const df32 gx = ld(g1 + g * n_p + a), gy = ld(g2 + g * n_p + a), gz = ld(g3 + g * n_p + a);
        const df32 ux = df_add(ld(u + i0), u0x), uy = df_add(ld(u + i1), u0y), uz = df_add(ld(u + i2), u0z);
        a0.add_prod(gx, ux);
        a1.add_prod(gy, uy);
        a2.add_prod(gz, uz);
        a3.add_prod(gy, ux);
        a3.add_prod(gx, uy);
        a4.add_prod(gz, uy);
        a4.add_prod(gy, uz);
        a5.add_prod(gz, ux);
        a5.add_prod(gx, uz);
    }
    double2 *o = reinterpret_cast<double2 *>(E + 6 * g);
    o[0] = make_double2(a0.value(), a1.value());
    o[1] = make_double2(a2.value(), a3.value());
    o[2] = make_double2(a4.value(), a5.value());
}

// Force from hi + lo pairs of w * dphi (split once per pattern) and of the stresses, which the block
// splits itself into shared memory for the elements its threads cover (each stress value once).
// One thread per (element, node) accumulates the node's three displacement components, so each
// w * dphi value is loaded once.
constexpr int kForceThreads = 128, kForceMaxStress = 6 * 24 * 8;  // up to 8 elements of 24 points
__global__ void __launch_bounds__(kForceThreads) force3_mixed_kernel(const float2 *__restrict__ wg1,
                                                                     const float2 *__restrict__ wg2,
                                                                     const float2 *__restrict__ wg3,
                                                                     const double *__restrict__ S,
                                                                     const int32_t *__restrict__ elem_row, int n_rows,
                                                                     int n_elem, int n_p, int n_q,
                                                                     double *__restrict__ F) {
    __shared__ float2 s_hl[kForceMaxStress];
    const long long t0 = (long long)blockIdx.x * kForceThreads;
    const long long e_first = t0 / n_p;
    long long e_last = (t0 + kForceThreads - 1) / n_p;
    if (e_last >= n_elem) e_last = n_elem - 1;
    const int n_vals = static_cast<int>(e_last - e_first + 1) * n_q * 6;  // <= kForceMaxStress (host check)
    const double *Sb = S + e_first * n_q * 6;
    for (int i = threadIdx.x; i < n_vals; i += kForceThreads) {
        const df32 d = df_from_f64(Sb[i]);
        s_hl[i] = make_float2(d.hi, d.lo);
    }
    __syncthreads();
    const long long t = t0 + threadIdx.x;
    if (t >= (long long)n_elem * n_p) return;
    const long long e = t / n_p;
    const int node = static_cast<int>(t % n_p);
    const int32_t *er = elem_row + (e * n_p + node) * 3;
    const int r0 = er[0], r1 = er[1], r2 = er[2];
    if (r0 < 0 && r1 < 0 && r2 < 0) return;
    if (r0 >= n_rows || r1 >= n_rows || r2 >= n_rows) {
        flag(SSP_DEV_BAD_INDEX);
        return;
    }
    const float2 *sl = s_hl + (e - e_first) * n_q * 6;
    // component c sums d/dx, d/dy, d/dz times the stresses bt_row3(c, 0..2): {0,3,5}, {3,1,4}, {5,4,2}
    CSum a0, a1, a2;
    for (int q = 0; q < n_q; ++q) {
        const long long g = (e * n_q + q) * n_p + node;
        const df32 x = ld(wg1 + g), y = ld(wg2 + g), z = ld(wg3 + g);
        const float2 *sq = sl + 6 * q;
        a0.add_prod(x, ld(sq + 0));
        a0.add_prod(y, ld(sq + 3));
        a0.add_prod(z, ld(sq + 5));
        a1.add_prod(x, ld(sq + 3));
        a1.add_prod(y, ld(sq + 1));
        a1.add_prod(z, ld(sq + 4));
        a2.add_prod(x, ld(sq + 5));
        a2.add_prod(y, ld(sq + 4));
        a2.add_prod(z, ld(sq + 2));
    }
    if (r0 >= 0) red_add(F + r0, a0.value());
    if (r1 >= 0) red_add(F + r1, a1.value());
    if (r2 >= 0) red_add(F + r2, a2.value());
}

// Affine elements (straight-sided tetrahedra, every point with the same Jacobian J): the gradients
// are dphi_a(q) = J^{-T} ghat_a(q) with ghat the reference-element table, the same for every
// element.  The kernels below read J^{-1} once per element (9 hi + lo pairs) and the table from
// shared memory instead of the per-point gradients (3 n_p hi + lo pairs per point), at the cost
// of the product with J^{-1}.  ghat: [n_q][n_p][3] hi + lo pairs; jinv: [n_elem][3][3] row-major.

// Strain: grad u = G J^{-1} with G_ik = sum_{a>=1} (u_a - u_0)_i ghat_a,k(q) (rigid translation
// removed as in strain3_mixed_kernel); E = the engineering strains of grad u, each a compensated
// sum of its 3 or 6 products G_ik J^{-1}_kj.
__global__ void __launch_bounds__(128) strain3_affine_mixed_kernel(const float2 *__restrict__ jinv,
                                                                   const float2 *__restrict__ ghat,
                                                                   const float2 *__restrict__ u,
                                                                   const int32_t *__restrict__ dof, long long n_u,
                                                                   int n_elem, int n_p, int n_q,
                                                                   double *__restrict__ E) {
    // shared: the reference table, then the displacements of the elements the block's points
    // belong to (gathered once per element instead of once per point)
    extern __shared__ float2 s_dyn[];
    float2 *s_ghat = s_dyn;                // n_q * n_p * 3
    float2 *s_u = s_dyn + n_q * n_p * 3;   // (elements of the block) * 3 n_p
    for (int i = threadIdx.x; i < n_q * n_p * 3; i += blockDim.x) s_ghat[i] = ghat[i];
    const int nld = 3 * n_p;
    const long long g0 = (long long)blockIdx.x * blockDim.x;
    const long long e_first = g0 / n_q;
    long long e_last = (g0 + blockDim.x - 1) / n_q;
    if (e_last >= n_elem) e_last = n_elem - 1;
    const int n_vals = static_cast<int>(e_last - e_first + 1) * nld;
    bool bad = false;
    for (int i = threadIdx.x; i < n_vals; i += blockDim.x) {
        const int32_t lid = dof[e_first * nld + i];
        if (lid < 0 || lid >= n_u) {
            bad = true;
            s_u[i] = make_float2(0.0f, 0.0f);
        } else {
            s_u[i] = u[lid];
        }
    }
    if (bad) flag(SSP_DEV_BAD_INDEX);
    __syncthreads();
    const long long g = g0 + threadIdx.x;
    if (g >= (long long)n_elem * n_q) return;
    const long long e = g / n_q;
    const int q = static_cast<int>(g - e * n_q);
    const float2 *ue = s_u + (e - e_first) * nld;
    const df32 u0x = df_neg(ld(ue)), u0y = df_neg(ld(ue + 1)), u0z = df_neg(ld(ue + 2));
    CSum G[3][3];
    const float2 *gq = s_ghat + q * n_p * 3;
    for (int a = 1; a < n_p; ++a) {
        const df32 du[3] = {df_add(ld(ue + 3 * a), u0x), df_add(ld(ue + 3 * a + 1), u0y),
                            df_add(ld(ue + 3 * a + 2), u0z)};
        const df32 gh[3] = {ld(gq + 3 * a), ld(gq + 3 * a + 1), ld(gq + 3 * a + 2)};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) G[i][k].add_prod(du[i], gh[k]);
    }
    df32 Gd[3][3], J[3][3];
    const float2 *je = jinv + e * 9;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            Gd[i][k] = G[i][k].df();
            J[i][k] = ld(je + 3 * i + k);
        }
    // E_11, E_22, E_33: (G J^{-1})_ii; E_12, E_23, E_13: (G J^{-1})_ij + (G J^{-1})_ji
    CSum s[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s[0].add_prod(Gd[0][k], J[k][0]);
        s[1].add_prod(Gd[1][k], J[k][1]);
        s[2].add_prod(Gd[2][k], J[k][2]);
        s[3].add_prod(Gd[0][k], J[k][1]);
        s[3].add_prod(Gd[1][k], J[k][0]);
        s[4].add_prod(Gd[1][k], J[k][2]);
        s[4].add_prod(Gd[2][k], J[k][1]);
        s[5].add_prod(Gd[0][k], J[k][2]);
        s[5].add_prod(Gd[2][k], J[k][0]);
    }
    double2 *o = reinterpret_cast<double2 *>(E + 6 * g);
    o[0] = make_double2(s[0].value(), s[1].value());
    o[1] = make_double2(s[2].value(), s[3].value());
    o[2] = make_double2(s[4].value(), s[5].value());
}

// Force: F_(a,i) = sum_q sum_k T_ik(q) ghat_a,k(q) with T(q) = w_q sigma_q J^{-T}, i.e.
// T_ik = w sum_j sigma_ij J^{-1}_kj.  The block forms T of every point of the elements its
// threads cover in shared memory (each once); one thread per (element, node) then sums its
// three components over the points.
__global__ void __launch_bounds__(kForceThreads) force3_affine_mixed_kernel(const float2 *__restrict__ jinv,
                                                                            const float2 *__restrict__ ghat,
                                                                            const float2 *__restrict__ w,
                                                                            const double *__restrict__ S,
                                                                            const int32_t *__restrict__ elem_row,
                                                                            int n_rows, int n_elem, int n_p, int n_q,
                                                                            double *__restrict__ F) {
    extern __shared__ float2 s_dyn[];
    float2 *s_ghat = s_dyn;                   // n_q * n_p * 3
    float2 *s_T = s_dyn + n_q * n_p * 3;      // (elements of the block) * n_q * 9
    for (int i = threadIdx.x; i < n_q * n_p * 3; i += kForceThreads) s_ghat[i] = ghat[i];
    const long long t0 = (long long)blockIdx.x * kForceThreads;
    const long long e_first = t0 / n_p;
    long long e_last = (t0 + kForceThreads - 1) / n_p;
    if (e_last >= n_elem) e_last = n_elem - 1;
    const int n_pts = static_cast<int>(e_last - e_first + 1) * n_q;
    for (int i = threadIdx.x; i < n_pts; i += kForceThreads) {
        const long long g = e_first * n_q + i;
        const long long e = g / n_q;
        const df32 wq = ld(w + g);
        const double *sg = S + 6 * g;
        // w sigma, symmetric: sigma_00..22 = s0, s1, s2; sigma_01 = s3, sigma_12 = s4, sigma_02 = s5
        const df32 s0 = df_mul(wq, df_from_f64(sg[0])), s1 = df_mul(wq, df_from_f64(sg[1])),
                   s2 = df_mul(wq, df_from_f64(sg[2])), s3 = df_mul(wq, df_from_f64(sg[3])),
                   s4 = df_mul(wq, df_from_f64(sg[4])), s5 = df_mul(wq, df_from_f64(sg[5]));
        const df32 ws[3][3] = {{s0, s3, s5}, {s3, s1, s4}, {s5, s4, s2}};
        const float2 *je = jinv + e * 9;
        float2 *T = s_T + i * 9;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                CSum acc;
#pragma unroll
                for (int j = 0; j < 3; ++j) acc.add_prod(ws[a][j], ld(je + 3 * k + j));
                const df32 v = acc.df();
                T[3 * a + k] = make_float2(v.hi, v.lo);
            }
    }
    __syncthreads();
    const long long t = t0 + threadIdx.x;
    if (t >= (long long)n_elem * n_p) return;
    const long long e = t / n_p;
    const int node = static_cast<int>(t - e * n_p);
    const int32_t *er = elem_row + (e * n_p + node) * 3;
    const int r0 = er[0], r1 = er[1], r2 = er[2];
    if (r0 < 0 && r1 < 0 && r2 < 0) return;
    if (r0 >= n_rows || r1 >= n_rows || r2 >= n_rows) {
        flag(SSP_DEV_BAD_INDEX);
        return;
    }
    const float2 *Te = s_T + (e - e_first) * n_q * 9;
    CSum a0, a1, a2;
    for (int q = 0; q < n_q; ++q) {
        const float2 *gh = s_ghat + (q * n_p + node) * 3;
        const df32 g0 = ld(gh), g1 = ld(gh + 1), g2 = ld(gh + 2);
        const float2 *T = Te + q * 9;
        a0.add_prod(ld(T + 0), g0);
        a0.add_prod(ld(T + 1), g1);
        a0.add_prod(ld(T + 2), g2);
        a1.add_prod(ld(T + 3), g0);
        a1.add_prod(ld(T + 4), g1);
        a1.add_prod(ld(T + 5), g2);
        a2.add_prod(ld(T + 6), g0);
        a2.add_prod(ld(T + 7), g1);
        a2.add_prod(ld(T + 8), g2);
    }
    if (r0 >= 0) red_add(F + r0, a0.value());
    if (r1 >= 0) red_add(F + r1, a1.value());
    if (r2 >= 0) red_add(F + r2, a2.value());
}

// ---------------------------------------------------------------------------- P2, barycentric form

// Straight-sided P2 tetrahedra in double-float arithmetic: the barycentric regrouping of the FP64
// strain3_p2_affine_kernel / force3_p2_affine_kernel.  ∇φ_i = (4λ_i − 1)∇λ_i at vertex i,
// ∇φ_ij = 4(λ_i∇λ_j + λ_j∇λ_i) at the node of edge ij, ∇λ_1..3 the rows of J⁻¹, ∇λ_0 = −Σ; the
// strain is Σ_m λ_m S_m with four strain vectors per element, the force needs the four moments
// M_m = Σ_q λ_qm w_q σ_q.  One thread per element; local nodes: vertices 0-3, then the edges
// 01, 12, 02, 13, 23, 03 (simplex_lagrange.py:15-83).
__device__ __forceinline__ constexpr int p2_edge(int i, int j) {
    return (i < j ? i : j) == 0 ? ((i > j ? i : j) == 1 ? 4 : ((i > j ? i : j) == 2 ? 6 : 9))
                                : ((i < j ? i : j) == 1 ? ((i > j ? i : j) == 2 ? 5 : 7) : 8);
}
__device__ __forceinline__ df32 df_times4(df32 a) { return {4.0f * a.hi, 4.0f * a.lo}; }  // exact
__device__ __forceinline__ df32 df_times3(df32 a) { return df_mul(a, df32{3.0f, 0.0f}); }

// Four lanes per element (lane m = 0..3 of an aligned group of 4): the double-float chains are
// latency-bound, so the element's work is spread over the group.  Lane m forms S_m, the group
// swaps the four S through shuffles, and lane m evaluates the points q = m, m + 4, m + 8.
constexpr int kBaryThreads = 128;

__device__ __forceinline__ df32 shfl_df(df32 v, int src) {
    return {__shfl_sync(0xffffffffu, v.hi, src, 4), __shfl_sync(0xffffffffu, v.lo, src, 4)};
}

__global__ void __launch_bounds__(kBaryThreads) strain3_p2_bary_mixed_kernel(const float2 *__restrict__ jinv,
                                                                             const float2 *__restrict__ bary,
                                                                             const float2 *__restrict__ u,
                                                                             const int32_t *__restrict__ dof,
                                                                             long long n_u, int n_elem, int n_q,
                                                                             double *__restrict__ E) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int m = static_cast<int>(t & 3);
    const bool valid = (t >> 2) < n_elem;
    const long long e = valid ? (t >> 2) : (long long)n_elem - 1;  // every lane of a group shuffles
    const int32_t *dl = dof + e * 30;
    auto load_u = [&](int node, int c) -> df32 {
        const int32_t i = dl[3 * node + c];
        if (i < 0 || i >= n_u) {
            flag(SSP_DEV_BAD_INDEX);
            return df32{0.0f, 0.0f};
        }
        return ld(u + i);
    };
    // A_im = 3 u_i when i == m, else 4 u_(edge im) - u_i; as a u_i + 4 u_x with (a, x) selected per lane
    df32 A[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const bool own = i == m;
        const int x = own ? i : p2_edge(i, m);
#pragma unroll
        for (int c = 0; c < 3; ++c) {  // both forms computed, one selected: no divergence in the group
            const df32 ui = load_u(i, c);
            const df32 ux = load_u(x, c);
            const df32 vertex = df_times3(ui), edge = df_add(df_times4(ux), df_neg(ui));
            A[i][c] = own ? vertex : edge;
        }
    }
    df32 gl[3][3];
#pragma unroll
    for (int k = 0; k < 9; ++k) gl[k / 3][k % 3] = ld(jinv + e * 9 + k);
    CSum G[3][3];
#pragma unroll
    for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const df32 b = df_add(A[i][c], df_neg(A[0][c]));
#pragma unroll
            for (int k = 0; k < 3; ++k) G[c][k].add_prod(b, gl[i - 1][k]);
        }
    df32 Sm[6];
    Sm[0] = G[0][0].df();
    Sm[1] = G[1][1].df();
    Sm[2] = G[2][2].df();
    Sm[3] = df_add(G[0][1].df(), G[1][0].df());
    Sm[4] = df_add(G[1][2].df(), G[2][1].df());
    Sm[5] = df_add(G[0][2].df(), G[2][0].df());
    df32 S[4][6];
#pragma unroll
    for (int src = 0; src < 4; ++src)
#pragma unroll
        for (int c = 0; c < 6; ++c) S[src][c] = shfl_df(Sm[c], src);
    if (!valid) return;
    for (int q = m; q < n_q; q += 4) {
        const df32 l[4] = {ld(bary + 4 * q), ld(bary + 4 * q + 1), ld(bary + 4 * q + 2), ld(bary + 4 * q + 3)};
        double v[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            CSum acc;
#pragma unroll
            for (int k = 0; k < 4; ++k) acc.add_prod(l[k], S[k][c]);
            v[c] = acc.value();
        }
        double2 *o = reinterpret_cast<double2 *>(E + 6 * (e * n_q + q));
        o[0] = make_double2(v[0], v[1]);
        o[1] = make_double2(v[2], v[3]);
        o[2] = make_double2(v[4], v[5]);
    }
}

// (M v) for M symmetric as [11,22,33,12,23,13], accumulated into three compensated sums
__device__ __forceinline__ void df_sym_matvec_add(const df32 *M, const df32 *v, CSum *out) {
    out[0].add_prod(M[0], v[0]);
    out[0].add_prod(M[3], v[1]);
    out[0].add_prod(M[5], v[2]);
    out[1].add_prod(M[3], v[0]);
    out[1].add_prod(M[1], v[1]);
    out[1].add_prod(M[4], v[2]);
    out[2].add_prod(M[5], v[0]);
    out[2].add_prod(M[4], v[1]);
    out[2].add_prod(M[2], v[2]);
}

// One thread per element (spreading the points over four lanes measured slower: 81 µs against
// 70 µs on 3d_p2_homo; the FP64 -> double-float conversions of the stresses dominate and are
// not shared).
__global__ void __launch_bounds__(64) force3_p2_bary_mixed_kernel(const float2 *__restrict__ jinv,
                                                                  const float2 *__restrict__ bary,
                                                                  const float2 *__restrict__ w,
                                                                  const double *__restrict__ S,
                                                                  const int32_t *__restrict__ elem_row, int n_rows,
                                                                  int n_elem, int n_q, double *__restrict__ F) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    CSum Ms[4][6];
    for (int q = 0; q < n_q; ++q) {
        const long long g = e * n_q + q;
        const double2 *s2 = reinterpret_cast<const double2 *>(S + 6 * g);
        const double2 a = s2[0], b = s2[1], c2 = s2[2];
        const double sv[6] = {a.x, a.y, b.x, b.y, c2.x, c2.y};
        const df32 wq = ld(w + g);
        const df32 l[4] = {ld(bary + 4 * q), ld(bary + 4 * q + 1), ld(bary + 4 * q + 2), ld(bary + 4 * q + 3)};
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            const df32 T = df_mul(wq, df_from_f64(sv[c]));
#pragma unroll
            for (int m = 0; m < 4; ++m) Ms[m][c].add_prod(l[m], T);
        }
    }
    df32 M[4][6], Mt[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
        CSum t;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            M[m][c] = Ms[m][c].df();
            t.add(M[m][c]);
        }
        Mt[c] = t.df();
    }
    df32 gl[4][3];
#pragma unroll
    for (int k = 0; k < 9; ++k) gl[1 + k / 3][k % 3] = ld(jinv + e * 9 + k);
#pragma unroll
    for (int k = 0; k < 3; ++k) gl[0][k] = df_neg(df_add(df_add(gl[1][k], gl[2][k]), gl[3][k]));
    const int32_t *er = elem_row + e * 30;
    auto emit = [&](int a, int c, double v) {
        const int row = er[3 * a + c];
        if (row < 0) return;
        if (row >= n_rows) {
            flag(SSP_DEV_BAD_INDEX);
            return;
        }
        red_add(F + row, v);
    };
#pragma unroll
    for (int i = 0; i < 4; ++i) {  // vertices: (4 M_i − Σ_m M_m) ∇λ_i
        df32 V[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) V[c] = df_add(df_times4(M[i][c]), df_neg(Mt[c]));
        CSum o[3];
        df_sym_matvec_add(V, gl[i], o);
#pragma unroll
        for (int c = 0; c < 3; ++c) emit(i, c, o[c].value());
    }
    constexpr int kEi[6] = {0, 1, 0, 1, 2, 0}, kEj[6] = {1, 2, 2, 3, 3, 3};
#pragma unroll
    for (int k = 0; k < 6; ++k) {  // edges: 4 (M_i ∇λ_j + M_j ∇λ_i)
        const int i = kEi[k], j = kEj[k];
        CSum o[3];
        df_sym_matvec_add(M[i], gl[j], o);
        df_sym_matvec_add(M[j], gl[i], o);
#pragma unroll
        for (int c = 0; c < 3; ++c) emit(p2_edge(i, j), c, 4.0 * o[c].value());
    }
}

}  // namespace
}  // namespace ssp

using namespace ssp;

extern "C" {

int ssp_split_f64(const double *x, const double *scale, long long n, int group, float *out_pairs, void *stream) {
    if (n < 0 || (scale && group <= 0)) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!x || !out_pairs) return SSP_ERR_INVALID;
    split_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(x, scale, n, group, reinterpret_cast<float2 *>(out_pairs));
    return launch_status();
}

int ssp_assemble_overlap_strain_3d_mixed(const float *dphi1_hl, const float *dphi2_hl, const float *dphi3_hl,
                                         const float *u_hl, int n_u, const int32_t *elem_dof_lids, int n_int,
                                         int n_elem, int n_p, int n_q, double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1_hl || !dphi2_hl || !dphi3_hl || !u_hl || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    const float2 *g1 = reinterpret_cast<const float2 *>(dphi1_hl), *g2 = reinterpret_cast<const float2 *>(dphi2_hl),
                 *g3 = reinterpret_cast<const float2 *>(dphi3_hl);
    strain3_mixed_kernel<<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(
        g1, g2, g3, reinterpret_cast<const float2 *>(u_hl), elem_dof_lids, n_u, n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element_mixed(const float *wdphi1_hl, const float *wdphi2_hl, const float *wdphi3_hl,
                                     const double *stress, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                     int n_rows, double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    // a block's threads cover at most 128 / n_p + 2 elements, whose stresses it stages
    if ((kForceThreads / n_p + 2) * n_q * 6 > kForceMaxStress) return SSP_ERR_UNSUPPORTED;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!wdphi1_hl || !wdphi2_hl || !wdphi3_hl || !stress || !elem_row) return SSP_ERR_INVALID;
    const long long n = (long long)n_elem * n_p;
    force3_mixed_kernel<<<grid_for(n, kForceThreads), kForceThreads, 0, st>>>(
        reinterpret_cast<const float2 *>(wdphi1_hl), reinterpret_cast<const float2 *>(wdphi2_hl),
        reinterpret_cast<const float2 *>(wdphi3_hl), stress, elem_row, n_rows, n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_overlap_strain_3d_p2_affine_mixed(const float *jinv_hl, const float *bary_hl, const float *u_hl,
                                                   int n_u, const int32_t *elem_dof_lids, int n_int, int n_elem, int n_q,
                                                   double *out_values, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv_hl || !bary_hl || !u_hl || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    strain3_p2_bary_mixed_kernel<<<grid_for(4LL * n_elem, kBaryThreads), kBaryThreads, 0, as_stream(stream)>>>(
        reinterpret_cast<const float2 *>(jinv_hl), reinterpret_cast<const float2 *>(bary_hl),
        reinterpret_cast<const float2 *>(u_hl), elem_dof_lids, n_u, n_elem, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element_p2_affine_mixed(const float *jinv_hl, const float *bary_hl, const float *w_hl,
                                               const double *stress, const int32_t *elem_row, int n_elem, int n_q,
                                               int n_rows, double *out_values, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!jinv_hl || !bary_hl || !w_hl || !stress || !elem_row) return SSP_ERR_INVALID;
    force3_p2_bary_mixed_kernel<<<grid_for(n_elem, 64), 64, 0, st>>>(
        reinterpret_cast<const float2 *>(jinv_hl), reinterpret_cast<const float2 *>(bary_hl),
        reinterpret_cast<const float2 *>(w_hl), stress, elem_row, n_rows, n_elem, n_q, out_values);
    return launch_status();
}

int ssp_assemble_overlap_strain_3d_affine_mixed(const float *jinv_hl, const float *ghat_hl, const float *u_hl, int n_u,
                                                const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                                double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv_hl || !ghat_hl || !u_hl || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    // the table plus the displacements of the at most 128 / n_q + 2 elements a block's points cover
    const size_t smem = sizeof(float2) * (3 * (size_t)n_p * n_q + 3 * (size_t)n_p * (128 / n_q + 2));
    if (smem > 48 * 1024) return SSP_ERR_UNSUPPORTED;
    strain3_affine_mixed_kernel<<<grid_for(n_int, 128), 128, smem, as_stream(stream)>>>(
        reinterpret_cast<const float2 *>(jinv_hl), reinterpret_cast<const float2 *>(ghat_hl),
        reinterpret_cast<const float2 *>(u_hl), elem_dof_lids, n_u, n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element_affine_mixed(const float *jinv_hl, const float *ghat_hl, const float *w_hl,
                                            const double *stress, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                            int n_rows, double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    // a block's threads cover at most 128 / n_p + 2 elements, whose points' T it stages
    const size_t smem = sizeof(float2) * (3 * (size_t)n_p * n_q + 9 * (size_t)(kForceThreads / n_p + 2) * n_q);
    if (smem > 48 * 1024) return SSP_ERR_UNSUPPORTED;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!jinv_hl || !ghat_hl || !w_hl || !stress || !elem_row) return SSP_ERR_INVALID;
    const long long n = (long long)n_elem * n_p;
    force3_affine_mixed_kernel<<<grid_for(n, kForceThreads), kForceThreads, smem, st>>>(
        reinterpret_cast<const float2 *>(jinv_hl), reinterpret_cast<const float2 *>(ghat_hl),
        reinterpret_cast<const float2 *>(w_hl), stress, elem_row, n_rows, n_elem, n_p, n_q, out_values);
    return launch_status();
}

}  // extern "C"
