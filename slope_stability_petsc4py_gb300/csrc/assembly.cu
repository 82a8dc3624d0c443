// Strain, internal force and tangent CSR-value assembly on the fixed owned-row pattern.
//
// Reference routines (src/slope_stability/...):
//   ssp_assemble_overlap_strain_3d   cython/assemble_tangent_values_3d.c:216-273
//   ssp_assemble_force_3d_rows       cython/assemble_tangent_values_3d.c:275-327
//   ssp_assemble_tangent_values_3d_rows  cython/assemble_tangent_values_3d.c:111-214
//   ssp_assemble_tangent_values_3d_p2    cython/assemble_tangent_values_3d.c:13-109
//   ssp_tangent_element_*            the same sum K = sum_q B^T (w D) B, scattered through the
//                                    element->CSR map (fem/distributed_tangent.py:328-366)
//   2D variants                      fem/distributed_tangent.py:845-907, 1437-1484
//   ssp_geometry_*                   fem/assembly.py:50-136 (2D), 139-245 (3D)
//   ssp_finish_values                fem/distributed_tangent.py:1606-1607 and
//                                    constitutive/problem.py:1614-1615
//
// Layout (all FP64 unless stated): points are element-major (g = e*n_q + q); dphi arrays are
// [n_int][n_p]; strains/stresses/tangents are per-point AoS ([n_int][6], [n_int][36]), which is
// the reference's C layout and makes each element's data one contiguous block.
#include <type_traits>

#include "ssp_internal.cuh"

namespace ssp {
namespace {

// ---------------------------------------------------------------------------- geometry

template <int DIM>
__global__ void geometry_kernel(const double *__restrict__ coord, const int64_t *__restrict__ elem,
                                const double *__restrict__ dhat, const double *__restrict__ wf, int n_nodes,
                                int n_elem, int n_p, int n_q, double *__restrict__ d1, double *__restrict__ d2,
                                double *__restrict__ d3, double *__restrict__ weight) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)n_elem * n_q) return;
    const int e = static_cast<int>(g / n_q), q = static_cast<int>(g % n_q);
    // dhat is [DIM][n_p][n_q]; elem is [n_p][n_elem]; coord is [DIM][n_nodes]
    double J[DIM][DIM];
#pragma unroll
    for (int r = 0; r < DIM; ++r)
#pragma unroll
        for (int c = 0; c < DIM; ++c) J[r][c] = 0.0;
    for (int a = 0; a < n_p; ++a) {
        const long long node = elem[(long long)a * n_elem + e];
#pragma unroll
        for (int r = 0; r < DIM; ++r) {
            const double h = dhat[((long long)r * n_p + a) * n_q + q];
#pragma unroll
            for (int c = 0; c < DIM; ++c) J[r][c] += coord[(long long)c * n_nodes + node] * h;
        }
    }
    if (DIM == 3) {
        const double c11 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c12 = J[1][0] * J[2][2] - J[1][2] * J[2][0];
        const double c13 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c11 - J[0][1] * c12 + J[0][2] * c13;
        const double inv = 1.0 / det;
        const double r12 = J[0][1] * J[2][2] - J[0][2] * J[2][1];
        const double r13 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
        const double r22 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
        const double r23 = J[0][0] * J[1][2] - J[0][2] * J[1][0];
        const double r32 = J[0][0] * J[2][1] - J[0][1] * J[2][0];
        const double r33 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        for (int a = 0; a < n_p; ++a) {
            const double h1 = dhat[(0ll * n_p + a) * n_q + q];
            const double h2 = dhat[(1ll * n_p + a) * n_q + q];
            const double h3 = dhat[(2ll * n_p + a) * n_q + q];
            d1[g * n_p + a] = (c11 * h1 - r12 * h2 + r13 * h3) * inv;
            d2[g * n_p + a] = (-c12 * h1 + r22 * h2 - r23 * h3) * inv;
            d3[g * n_p + a] = (c13 * h1 - r32 * h2 + r33 * h3) * inv;
        }
        weight[g] = wf[q] * fabs(det);
    } else {
        const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const double i11 = J[1][1] / det, i12 = -J[0][1] / det, i21 = -J[1][0] / det, i22 = J[0][0] / det;
        for (int a = 0; a < n_p; ++a) {
            const double h1 = dhat[(0ll * n_p + a) * n_q + q];
            const double h2 = dhat[(1ll * n_p + a) * n_q + q];
            d1[g * n_p + a] = i11 * h1 + i12 * h2;
            d2[g * n_p + a] = i21 * h1 + i22 * h2;
        }
        weight[g] = fabs(det) * wf[q];
    }
}

// ---------------------------------------------------------------------------- strain

__global__ void strain3_kernel(const double *__restrict__ d1, const double *__restrict__ d2,
                               const double *__restrict__ d3, const double *__restrict__ u,
                               const int32_t *__restrict__ dof, long long n_u, int n_elem, int n_p, int n_q,
                               double *__restrict__ E) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)n_elem * n_q) return;
    const long long e = g / n_q;
    const int32_t *dl = dof + e * 3 * n_p;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0, a4 = 0.0, a5 = 0.0;
    for (int a = 0; a < n_p; ++a) {
        const int32_t i0 = dl[3 * a], i1 = dl[3 * a + 1], i2 = dl[3 * a + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= n_u || i1 >= n_u || i2 >= n_u) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const double gx = d1[g * n_p + a], gy = d2[g * n_p + a], gz = d3[g * n_p + a];
        const double ux = u[i0], uy = u[i1], uz = u[i2];
        a0 += gx * ux;
        a1 += gy * uy;
        a2 += gz * uz;
        a3 += gy * ux + gx * uy;
        a4 += gz * uy + gy * uz;
        a5 += gz * ux + gx * uz;
    }
    double2 *o = reinterpret_cast<double2 *>(E + 6 * g);
    o[0] = make_double2(a0, a1);
    o[1] = make_double2(a2, a3);
    o[2] = make_double2(a4, a5);
}

__global__ void strain2_kernel(const double *__restrict__ d1, const double *__restrict__ d2,
                               const double *__restrict__ u, const int32_t *__restrict__ dof, long long n_u, int n_elem,
                               int n_p, int n_q, double *__restrict__ E) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g >= (long long)n_elem * n_q) return;
    const long long e = g / n_q;
    const int32_t *dl = dof + e * 2 * n_p;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int a = 0; a < n_p; ++a) {
        const int32_t i0 = dl[2 * a], i1 = dl[2 * a + 1];
        if (i0 < 0 || i1 < 0 || i0 >= n_u || i1 >= n_u) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const double gx = d1[g * n_p + a], gy = d2[g * n_p + a];
        const double ux = u[i0], uy = u[i1];
        a0 += gx * ux;
        a1 += gy * uy;
        a2 += gy * ux + gx * uy;
    }
    E[3 * g] = a0;
    E[3 * g + 1] = a1;
    E[3 * g + 2] = a2;
}

// ---------------------------------------------------------------------------- force

__device__ __forceinline__ double bt3(int comp, double gx, double gy, double gz, const double *s) {
    return comp == 0 ? gx * s[0] + gy * s[3] + gz * s[5]
                     : (comp == 1 ? gx * s[3] + gy * s[1] + gz * s[4] : gx * s[5] + gy * s[4] + gz * s[2]);
}

// Owned force by row gather: deterministic, one thread per owned row.
__global__ void force_rows3_kernel(const double *__restrict__ d1, const double *__restrict__ d2,
                                   const double *__restrict__ d3, const double *__restrict__ S,
                                   const double *__restrict__ w, const int32_t *__restrict__ rsp,
                                   const int32_t *__restrict__ slot_elem, const uint8_t *__restrict__ slot_lrow,
                                   int n_rows, int n_elem, int n_p, int n_q, double *__restrict__ F) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    double acc = 0.0;
    for (int s = rsp[r]; s < rsp[r + 1]; ++s) {
        const int e = slot_elem[s];
        const int alpha = slot_lrow[s];
        const int node = alpha / 3, comp = alpha % 3;
        if (e < 0 || e >= n_elem || node >= n_p) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        for (int q = 0; q < n_q; ++q) {
            const long long g = (long long)e * n_q + q;
            acc += w[g] * bt3(comp, d1[g * n_p + node], d2[g * n_p + node], d3[g * n_p + node], S + 6 * g);
        }
    }
    F[r] = acc;
}

// Owned force by element scatter (2D and 3D): elem_row[e][alpha] is the owned free row of
// local dof alpha or -1.  One thread per (element, local dof); atomics into F.
template <int DIM>
__global__ void force_element_kernel(const double *__restrict__ d1, const double *__restrict__ d2,
                                     const double *__restrict__ d3, const double *__restrict__ S,
                                     const double *__restrict__ w, const int32_t *__restrict__ elem_row, int n_rows,
                                     int n_elem, int n_p, int n_q, double *__restrict__ F) {
    constexpr int NS = DIM == 3 ? 6 : 3;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int nld = DIM * n_p;
    if (t >= (long long)n_elem * nld) return;
    const long long e = t / nld;
    const int alpha = static_cast<int>(t % nld);
    const int row = elem_row[t];
    if (row < 0) return;
    if (row >= n_rows) {
        flag(SSP_DEV_BAD_INDEX);
        return;
    }
    const int node = alpha / DIM, comp = alpha % DIM;
    double acc = 0.0;
    for (int q = 0; q < n_q; ++q) {
        const long long g = e * n_q + q;
        const double *s = S + NS * g;
        const double gx = d1[g * n_p + node], gy = d2[g * n_p + node];
        if (DIM == 3) {
            acc += w[g] * bt3(comp, gx, gy, d3[g * n_p + node], s);
        } else {
            acc += w[g] * (comp == 0 ? gx * s[0] + gy * s[2] : gy * s[1] + gx * s[2]);
        }
    }
    red_add(F + row, acc);
}

// ---------------------------------------------------------------------------- P2 tetrahedra, affine map

// Straight-sided P2 tetrahedra (x(ξ) affine, J constant per element).  In barycentric form the
// quadratic basis has ∇φ_i = (4λ_i − 1)∇λ_i at vertex i and ∇φ_ij = 4(λ_i∇λ_j + λ_j∇λ_i) at the
// node of edge ij, with ∇λ_1..3 the rows of J⁻¹ and ∇λ_0 = −(∇λ_1 + ∇λ_2 + ∇λ_3); the gradients
// are then linear in λ, so the strain is Σ_m λ_m S_m with four strain vectors S_m per element and
// the force needs only the four moments Σ_q λ_qm w_q σ_q.  This is the reference's dphi-based
// arithmetic (assemble_tangent_values_3d.c:216-273, 275-327) regrouped: ≈470 and ≈530 FP64
// operations per 11-point element instead of ≈990 and ≈1,320, and no per-point gradients read.
// Local nodes: vertices 0-3, then edges 01, 12, 02, 13, 23, 03 (simplex_lagrange.py:15-83).
__host__ __device__ __forceinline__ constexpr int p2_edge_node(int i, int j) {
    return (i < j ? i : j) == 0 ? ((i > j ? i : j) == 1 ? 4 : ((i > j ? i : j) == 2 ? 6 : 9))
                                : ((i < j ? i : j) == 1 ? ((i > j ? i : j) == 2 ? 5 : 7) : 8);
}

__device__ __forceinline__ void sym_matvec(const double *M, const double *v, double *out) {  // M as [11,22,33,12,23,13]
    out[0] = M[0] * v[0] + M[3] * v[1] + M[5] * v[2];
    out[1] = M[3] * v[0] + M[1] * v[1] + M[4] * v[2];
    out[2] = M[5] * v[0] + M[4] * v[1] + M[2] * v[2];
}

// One thread per element: bary is [n_q][4] (λ0..λ3 of each point).
__global__ void __launch_bounds__(64) strain3_p2_affine_kernel(const double *__restrict__ jinv,
                                                               const double *__restrict__ bary,
                                                               const double *__restrict__ u,
                                                               const int32_t *__restrict__ dof, long long n_u,
                                                               int n_elem, int n_q, double *__restrict__ E) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    double un[10][3];
    const int32_t *dl = dof + e * 30;
#pragma unroll
    for (int a = 0; a < 10; ++a) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int32_t i = dl[3 * a + c];
            if (i < 0 || i >= n_u) {
                flag(SSP_DEV_BAD_INDEX);
                un[a][c] = 0.0;
            } else {
                un[a][c] = u[i];
            }
        }
    }
    double gl[3][3];  // ∇λ_1..3
#pragma unroll
    for (int k = 0; k < 9; ++k) gl[k / 3][k % 3] = jinv[e * 9 + k];
    // ∇u = Σ_m λ_m G_m, G_m = Σ_{i=1..3} (A_im − A_0m) ⊗ ∇λ_i, A_ii = 3u_i, A_im = 4u_(edge im) − u_i
    double S[4][6];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        double A0[3], G[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c) A0[c] = m == 0 ? 3.0 * un[0][c] : 4.0 * un[p2_edge_node(0, m)][c] - un[0][c];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
            for (int k = 0; k < 3; ++k) G[c][k] = 0.0;
#pragma unroll
        for (int i = 1; i < 4; ++i) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double Ai = i == m ? 3.0 * un[i][c] : 4.0 * un[p2_edge_node(i, m)][c] - un[i][c];
                const double b = Ai - A0[c];
#pragma unroll
                for (int k = 0; k < 3; ++k) G[c][k] += b * gl[i - 1][k];
            }
        }
        S[m][0] = G[0][0];
        S[m][1] = G[1][1];
        S[m][2] = G[2][2];
        S[m][3] = G[0][1] + G[1][0];
        S[m][4] = G[1][2] + G[2][1];
        S[m][5] = G[0][2] + G[2][0];
    }
    // the coordinates sum to one: E(q) = S_0 + sum_{m>=1} lambda_qm (S_m - S_0), 18 FMA per point
#pragma unroll
    for (int m = 1; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 6; ++c) S[m][c] -= S[0][c];
    for (int q = 0; q < n_q; ++q) {
        const double l1 = bary[4 * q + 1], l2 = bary[4 * q + 2], l3 = bary[4 * q + 3];
        double v[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) v[c] = fma(l3, S[3][c], fma(l2, S[2][c], fma(l1, S[1][c], S[0][c])));
        double2 *o = reinterpret_cast<double2 *>(E + 6 * (e * n_q + q));
        o[0] = make_double2(v[0], v[1]);
        o[1] = make_double2(v[2], v[3]);
        o[2] = make_double2(v[4], v[5]);
    }
}

// ---------------------------------------------------------------------------- affine tetrahedra, FP64
//
// Straight-sided tetrahedra (every point of an element has the same Jacobian): dphi_a(q) =
// J^{-T} ghat_a(q), ghat the reference element's gradient table [n_q][n_p][3], the same for every
// element.  Instead of the per-point gradients (24 n_p bytes per point: 840 for P4) the kernels
// read J^{-1} once per element (72 bytes) and the table from shared memory.  Used for P1 and P4
// (P2 has the barycentric form above).

// Strain: grad u = G J^{-1}, G_ik = sum_{a>=1} (u_a - u_0)_i ghat_a,k(q) (the element's rigid
// translation removed first, as the mixed form does); E the engineering strains of grad u.
constexpr int kAffineThreads = 128;
__global__ void __launch_bounds__(kAffineThreads) strain3_affine_kernel(const double *__restrict__ jinv,
                                                                        const double *__restrict__ ghat,
                                                                        const double *__restrict__ u,
                                                                        const int32_t *__restrict__ dof, long long n_u,
                                                                        int n_elem, int n_p, int n_q,
                                                                        double *__restrict__ E) {
    // shared: the reference table, then the displacements of the elements the block's points
    // belong to (gathered once per element instead of once per point)
    extern __shared__ double s_aff[];
    double *s_ghat = s_aff;                // n_q * n_p * 3
    double *s_u = s_aff + n_q * n_p * 3;   // (elements of the block) * 3 n_p
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
            s_u[i] = 0.0;
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
    const double *ue = s_u + (e - e_first) * nld;
    const double u0x = ue[0], u0y = ue[1], u0z = ue[2];
    double G[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    const double *gq = s_ghat + q * n_p * 3;
    for (int a = 1; a < n_p; ++a) {
        const double du[3] = {ue[3 * a] - u0x, ue[3 * a + 1] - u0y, ue[3 * a + 2] - u0z};
        const double gh[3] = {gq[3 * a], gq[3 * a + 1], gq[3 * a + 2]};
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int k = 0; k < 3; ++k) G[i][k] = fma(du[i], gh[k], G[i][k]);
    }
    double J[3][3];
    const double *je = jinv + e * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) J[k / 3][k % 3] = je[k];
    // E_11, E_22, E_33: (G J^{-1})_ii; E_12, E_23, E_13: (G J^{-1})_ij + (G J^{-1})_ji
    double s[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s[0] = fma(G[0][k], J[k][0], s[0]);
        s[1] = fma(G[1][k], J[k][1], s[1]);
        s[2] = fma(G[2][k], J[k][2], s[2]);
        s[3] = fma(G[0][k], J[k][1], fma(G[1][k], J[k][0], s[3]));
        s[4] = fma(G[1][k], J[k][2], fma(G[2][k], J[k][1], s[4]));
        s[5] = fma(G[0][k], J[k][2], fma(G[2][k], J[k][0], s[5]));
    }
    double2 *o = reinterpret_cast<double2 *>(E + 6 * g);
    o[0] = make_double2(s[0], s[1]);
    o[1] = make_double2(s[2], s[3]);
    o[2] = make_double2(s[4], s[5]);
}

// Force: F_(a,i) = sum_q sum_k T_ik(q) ghat_a,k(q), T(q) = w_q sigma_q J^{-T} (T_ik = w sum_j
// sigma_ij J^{-1}_kj).  The block forms T of every point of the elements its threads cover in
// shared memory, once each; one thread per (element, node) then sums its three components over the
// points and adds them to the owned rows with FP64 reductions.
__global__ void __launch_bounds__(kAffineThreads) force3_affine_kernel(const double *__restrict__ jinv,
                                                                       const double *__restrict__ ghat,
                                                                       const double *__restrict__ w,
                                                                       const double *__restrict__ S,
                                                                       const int32_t *__restrict__ elem_row, int n_rows,
                                                                       int n_elem, int n_p, int n_q,
                                                                       double *__restrict__ F) {
    extern __shared__ double s_aff[];
    double *s_ghat = s_aff;                  // n_q * n_p * 3
    double *s_T = s_aff + n_q * n_p * 3;     // (elements of the block) * n_q * 9
    for (int i = threadIdx.x; i < n_q * n_p * 3; i += kAffineThreads) s_ghat[i] = ghat[i];
    const long long t0 = (long long)blockIdx.x * kAffineThreads;
    const long long e_first = t0 / n_p;
    long long e_last = (t0 + kAffineThreads - 1) / n_p;
    if (e_last >= n_elem) e_last = n_elem - 1;
    const int n_pts = static_cast<int>(e_last - e_first + 1) * n_q;
    for (int i = threadIdx.x; i < n_pts; i += kAffineThreads) {
        const long long g = e_first * n_q + i;
        const long long e = g / n_q;
        const double wq = w[g];
        const double *sg = S + 6 * g;
        // w sigma, symmetric: sigma_00..22 = s0, s1, s2; sigma_01 = s3, sigma_12 = s4, sigma_02 = s5
        const double s0 = wq * sg[0], s1 = wq * sg[1], s2 = wq * sg[2], s3 = wq * sg[3], s4 = wq * sg[4],
                     s5 = wq * sg[5];
        const double ws[3][3] = {{s0, s3, s5}, {s3, s1, s4}, {s5, s4, s2}};
        const double *je = jinv + e * 9;
        double *T = s_T + i * 9;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                T[3 * a + k] = fma(ws[a][0], je[3 * k], fma(ws[a][1], je[3 * k + 1], ws[a][2] * je[3 * k + 2]));
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
    const double *Te = s_T + (e - e_first) * n_q * 9;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int q = 0; q < n_q; ++q) {
        const double *gh = s_ghat + (q * n_p + node) * 3;
        const double g0 = gh[0], g1 = gh[1], g2 = gh[2];
        const double *T = Te + q * 9;
        a0 = fma(T[0], g0, fma(T[1], g1, fma(T[2], g2, a0)));
        a1 = fma(T[3], g0, fma(T[4], g1, fma(T[5], g2, a1)));
        a2 = fma(T[6], g0, fma(T[7], g1, fma(T[8], g2, a2)));
    }
    if (r0 >= 0) red_add(F + r0, a0);
    if (r1 >= 0) red_add(F + r1, a1);
    if (r2 >= 0) red_add(F + r2, a2);
}

// One thread per element; elem_row as in force_element_kernel; atomics into F.
__global__ void __launch_bounds__(64) force3_p2_affine_kernel(const double *__restrict__ jinv,
                                                              const double *__restrict__ bary,
                                                              const double *__restrict__ S,
                                                              const double *__restrict__ w,
                                                              const int32_t *__restrict__ elem_row, int n_rows,
                                                              int n_elem, int n_q, double *__restrict__ F) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    double M[4][6];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int c = 0; c < 6; ++c) M[m][c] = 0.0;
    for (int q = 0; q < n_q; ++q) {
        const long long g = e * n_q + q;
        const double2 *s2 = reinterpret_cast<const double2 *>(S + 6 * g);
        const double2 a = s2[0], b = s2[1], c2 = s2[2];
        const double wq = w[g];
        const double T[6] = {wq * a.x, wq * a.y, wq * b.x, wq * b.y, wq * c2.x, wq * c2.y};
        const double l[4] = {bary[4 * q], bary[4 * q + 1], bary[4 * q + 2], bary[4 * q + 3]};
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int c = 0; c < 6; ++c) M[m][c] += l[m] * T[c];
    }
    double gl[4][3];
#pragma unroll
    for (int k = 0; k < 9; ++k) gl[1 + k / 3][k % 3] = jinv[e * 9 + k];
#pragma unroll
    for (int k = 0; k < 3; ++k) gl[0][k] = -(gl[1][k] + gl[2][k] + gl[3][k]);
    double f[10][3];
#pragma unroll
    for (int i = 0; i < 4; ++i) {  // vertices: (4 M_i − Σ_m M_m) ∇λ_i
        double V[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) V[c] = 4.0 * M[i][c] - (M[0][c] + M[1][c] + M[2][c] + M[3][c]);
        sym_matvec(V, gl[i], f[i]);
    }
    constexpr int kEi[6] = {0, 1, 0, 1, 2, 0}, kEj[6] = {1, 2, 2, 3, 3, 3};
#pragma unroll
    for (int k = 0; k < 6; ++k) {  // edges: 4 (M_i ∇λ_j + M_j ∇λ_i)
        const int i = kEi[k], j = kEj[k];
        double x[3], y[3];
        sym_matvec(M[i], gl[j], x);
        sym_matvec(M[j], gl[i], y);
        const int a = p2_edge_node(i, j);
#pragma unroll
        for (int c = 0; c < 3; ++c) f[a][c] = 4.0 * (x[c] + y[c]);
    }
    const int32_t *er = elem_row + e * 30;
#pragma unroll
    for (int a = 0; a < 10; ++a) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int row = er[3 * a + c];
            if (row < 0) continue;
            if (row >= n_rows) {
                flag(SSP_DEV_BAD_INDEX);
                continue;
            }
            red_add(F + row, f[a][c]);
        }
    }
}

// ---------------------------------------------------------------------------- tangent (rows)

// Direct counterpart of the reference "rows" kernel: one thread per owned row, walking the
// row's slots; deterministic.  out must be zeroed by the caller.
__global__ void tangent_rows3_kernel(const double *__restrict__ d1, const double *__restrict__ d2,
                                     const double *__restrict__ d3, const double *__restrict__ DS,
                                     const double *__restrict__ w, const int32_t *__restrict__ rsp,
                                     const int32_t *__restrict__ slot_elem, const uint8_t *__restrict__ slot_lrow,
                                     const int32_t *__restrict__ slot_pos, int n_rows, int n_elem, int n_p, int n_q,
                                     long long nnz, double *__restrict__ out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    const int nld = 3 * n_p;
    for (int s = rsp[r]; s < rsp[r + 1]; ++s) {
        const int e = slot_elem[s];
        const int alpha = slot_lrow[s];
        const int node = alpha / 3, comp = alpha % 3;
        if (e < 0 || e >= n_elem || node >= n_p) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const int32_t *pos = slot_pos + (long long)s * nld;
        for (int q = 0; q < n_q; ++q) {
            const long long g = (long long)e * n_q + q;
            const double *D = DS + 36 * g;
            const double wg = w[g];
            const double gx = d1[g * n_p + node], gy = d2[g * n_p + node], gz = d3[g * n_p + node];
            double t[6];
#pragma unroll
            for (int m = 0; m < 6; ++m) t[m] = wg * bt3(comp, gx, gy, gz, D + 6 * m);
            for (int b = 0; b < n_p; ++b) {
                const double bx = d1[g * n_p + b], by = d2[g * n_p + b], bz = d3[g * n_p + b];
                const int32_t p0 = pos[3 * b], p1 = pos[3 * b + 1], p2 = pos[3 * b + 2];
                if (p0 >= nnz || p1 >= nnz || p2 >= nnz) {
                    flag(SSP_DEV_BAD_INDEX);
                    continue;
                }
                if (p0 >= 0) out[p0] += t[0] * bx + t[3] * by + t[5] * bz;
                if (p1 >= 0) out[p1] += t[3] * bx + t[1] * by + t[4] * bz;
                if (p2 >= 0) out[p2] += t[5] * bx + t[4] * by + t[2] * bz;
            }
        }
    }
}

// ---------------------------------------------------------------------------- tangent (element)

struct ElemArgs {
    const double *d1, *d2, *d3, *DS, *w;
    const int32_t *emap;
    int n_elem;
    long long nnz;
    double *values;
    // correction mode only
    const int8_t *branch;
    const double *shear, *lame;
    double scale;
    // optional list of the elements to visit (elist[0 .. *elist_count)), else every element
    const int32_t *elist = nullptr;
    const int32_t *elist_count = nullptr;
};

// Element of iteration it: from the list when one is given (bounds-checked), else it itself;
// -1 for an out-of-range list entry.
__device__ __forceinline__ long long element_of(const ElemArgs &A, long long it) {
    if (!A.elist) return it;
    const int32_t e = A.elist[it];
    if (e < 0 || e >= A.n_elem) {
        flag(SSP_DEV_BAD_INDEX);
        return -1;
    }
    return e;
}
__device__ __forceinline__ long long element_iterations(const ElemArgs &A) {
    return A.elist ? static_cast<long long>(*A.elist_count) : static_cast<long long>(A.n_elem);
}

// Entry (i, j) of the elastic tangent the return mapping emits for an elastic point
// (constitutive.cu, mc3d_point / mc2d_point elastic branches), with the same arithmetic.
template <int DIM>
__device__ __forceinline__ double elastic_d(int i, int j, double G, double lam) {
    constexpr int NN = DIM == 3 ? 3 : 2;  // normal components
    if (i < NN && j < NN) return i == j ? 2.0 * G + lam : lam;
    if (i == j) return G;
    return 0.0;
}

// One CTA per element (grid-stride).  K_e = sum_q B_q^T (w_q D_q) B_q is formed in two
// stages per quadrature point through shared memory:
//   H[alpha][m] = (B^T (w D))[alpha][m]      (n_ld x n_s, split over the CTA)
//   K[alpha][beta] += sum_m H[alpha][m] B[m][beta]   (each thread owns fixed entries in registers)
// and scattered with FP64 atomics through the element->CSR map (the reference's legacy
// scatter_map).  SYM evaluates only alpha <= beta and writes both mirror positions; it is
// valid when every D_q is symmetric (tangents produced by ssp_constitutive_*).
//
// CORR (correction mode): only points whose branch is not elastic contribute, with
// D_q := scale * (DS_q - D_el,q).  Added to the elastic tangent assembled once, this gives the
// full tangent with the FP64 work of the plastic points only: for an elastic point DS_q equals
// D_el,q exactly, so its term vanishes.
template <int DIM, int NP, int NQ, int THREADS, bool SYM, bool CORR>
__global__ void __launch_bounds__(THREADS, SYM ? 2 : 1) tangent_element_kernel(ElemArgs A) {
    constexpr int NS = DIM == 3 ? 6 : 3;
    constexpr int NLD = DIM * NP;
    constexpr int NENT = SYM ? NLD * (NLD + 1) / 2 : NLD * NLD;
    constexpr int PER = (NENT + THREADS - 1) / THREADS;
    static_assert(NLD < 256, "entry codes hold alpha and beta in 8 bits each");
    __shared__ double sg[NQ][DIM][NP];
    __shared__ double sD[NQ][NS * NS];
    __shared__ double sH[NLD * NS];
    // SYM: entry id -> alpha | beta << 8 of the row-major upper triangle, 0xFFFF past the last entry
    // (in shared memory rather than registers, so two CTAs fit an SM); the full matrix decodes
    // id = alpha NLD + beta directly
    __shared__ uint16_t scode[SYM ? PER * THREADS : 1];
    __shared__ int sq[NQ];
    __shared__ int snq;

    const int tid = threadIdx.x;
    if (SYM) {
        for (int id = tid; id < PER * THREADS; id += THREADS) {
            uint16_t c = 0xFFFFu;
            if (id < NENT) {
                int rem = id, a = 0;  // row a holds NLD - a entries
                while (rem >= NLD - a) {
                    rem -= NLD - a;
                    ++a;
                }
                c = static_cast<uint16_t>(a | ((a + rem) << 8));
            }
            scode[id] = c;
        }
    }
    auto entry_code = [&](int i) -> int {
        const int id = tid + i * THREADS;
        if (SYM) return scode[id];
        return id < NENT ? ((id / NLD) | ((id % NLD) << 8)) : 0xFFFF;
    };

    const long long n_iter = element_iterations(A);
    for (long long it = blockIdx.x; it < n_iter; it += gridDim.x) {
        const long long e = element_of(A, it);
        if (e < 0) continue;  // uniform across the CTA
        const long long g0 = e * NQ;
        __syncthreads();  // the previous element is done with the shared buffers
        if (tid == 0) {
            int k = 0;
            for (int q = 0; q < NQ; ++q)
                if (!CORR || A.branch[g0 + q] != 0) sq[k++] = q;
            snq = k;
        }
        __syncthreads();
        const int nq = snq;
        if (nq == 0) continue;  // uniform across the CTA
        for (int i = tid; i < nq * NP; i += THREADS) {
            const int k = i / NP, a = i % NP;
            const long long src = (g0 + sq[k]) * NP + a;
            sg[k][0][a] = A.d1[src];
            sg[k][1][a] = A.d2[src];
            if (DIM == 3) sg[k][DIM - 1][a] = A.d3[src];
        }
        for (int i = tid; i < nq * NS * NS; i += THREADS) {
            const int k = i / (NS * NS), kk = i % (NS * NS);
            const long long g = g0 + sq[k];
            double v = A.DS[g * (NS * NS) + kk];
            if (CORR) v = A.scale * (v - elastic_d<DIM>(kk % NS, kk / NS, A.shear[g], A.lame[g]));
            sD[k][kk] = A.w[g] * v;
        }
        double acc[PER];
#pragma unroll
        for (int i = 0; i < PER; ++i) acc[i] = 0.0;
        __syncthreads();

        for (int q = 0; q < nq; ++q) {
            for (int it = tid; it < NLD * NS; it += THREADS) {
                const int alpha = it / NS, m = it % NS;
                const int a = alpha / DIM, c = alpha % DIM;
                double h = 0.0;
#pragma unroll
                for (int r = 0; r < DIM; ++r) {
                    const int k = DIM == 3 ? bt_row3(c, r) : bt_row2(c, r);
                    h += sg[q][r][a] * sD[q][k + NS * m];
                }
                sH[it] = h;
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int c = entry_code(i);
                if (c != 0xFFFF) {
                    const int alpha = c & 0xff, beta = c >> 8;
                    const int b = beta / DIM, cp = beta % DIM;
                    double v = acc[i];
#pragma unroll
                    for (int r = 0; r < DIM; ++r) {
                        const int m = DIM == 3 ? bt_row3(cp, r) : bt_row2(cp, r);
                        v += sH[alpha * NS + m] * sg[q][r][b];
                    }
                    acc[i] = v;
                }
            }
            __syncthreads();
        }

        const int32_t *em = A.emap + (long long)e * NLD * NLD;
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int c = entry_code(i);
            if (c == 0xFFFF) continue;
            const int alpha = c & 0xff, beta = c >> 8;
            const int32_t p = em[alpha * NLD + beta];
            if (p >= 0) {
                if (p < A.nnz) red_add(A.values + p, acc[i]);
                else flag(SSP_DEV_BAD_INDEX);
            }
            if (SYM && alpha != beta) {
                const int32_t p2 = em[beta * NLD + alpha];
                if (p2 >= 0) {
                    if (p2 < A.nnz) red_add(A.values + p2, acc[i]);
                    else flag(SSP_DEV_BAD_INDEX);
                }
            }
        }
    }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Warp-per-element variant for small elements (n_q <= 32): WARPS independent warps per CTA, each
// with its own shared-memory slice, grid-striding over elements.  In correction mode a warp reads
// the element's branch codes with one coalesced load and a ballot, so an all-elastic element
// costs a few instructions and no shared-memory traffic.  The element's row of the element->CSR
// map is fetched into shared memory asynchronously (cp.async) while the products are formed.
//
// MIXED (mixed-precision form; correction mode only): the gradients and w s (DS - D_el) are split
// into hi + lo float pairs by bit operations, H = B^T (w D) is formed in compensated double-float
// arithmetic on the FP32 pipe (about 48 significant bits; the only FP64 instructions left are the
// D_el subtractions and w s), the products B^T H are taken as Hh gh + Hl gh + Hh gl and
// accumulated in FP32, and the per-element sums are widened exactly and added to the FP64 CSR
// values with FP64 reductions.  Otherwise the arithmetic and scatter are those of
// tangent_element_kernel.
// Per-warp shared-memory slice of tangent_element_warp_kernel (dynamic shared memory).
template <int DIM, int NP, int NQ, bool MIXED>
struct WarpSlice {
    static constexpr int NS = DIM == 3 ? 6 : 3;
    static constexpr int NLD = DIM * NP;
    struct WorkF64 {
        double sg[NQ][DIM][NP];  // gradients of the contributing points
        double sD[NQ][NS * NS];  // w * D of the contributing points
        double sH[NLD * NS];     // B^T (w D) of one point
    };
    struct WorkMixed {
        df32 sgm[NQ][DIM][NP];  // gradients as hi + lo
        df32 sDm[NQ][NS * NS];  // w * D as hi + lo
        float2 sHhl[NLD * NS];  // B^T (w D) of one point as hi + lo
    };
    union {
        typename std::conditional<MIXED, WorkMixed, WorkF64>::type w;  // while the products are formed
        double sK[NLD * NLD];              // then the element's sums, staged for the row-wise scatter
    } u;
    alignas(16) int32_t smap[NLD * NLD];   // the element's row of the element->CSR map
    double spt[3][NQ];                     // w, shear, lame of the contributing points
    int sq[NQ];                            // contributing point indices
};

template <int DIM, int NP, int NQ, int WARPS, bool SYM, bool CORR, bool MIXED>
__global__ void __launch_bounds__(32 * WARPS, MIXED ? 5 : 4) tangent_element_warp_kernel(ElemArgs A) {
    constexpr int NS = DIM == 3 ? 6 : 3;
    constexpr int NLD = DIM * NP;
    // FP64 form (bound by the FP64 pipe): each lane owns PER scattered entries of K_e, which keeps
    // 97 % of the lanes' FP64 slots busy.  Mixed form (bound by issue): each lane owns whole
    // node-pair blocks (a, b) of DIM x DIM entries (a <= b when SYM), so it reads one row of H per
    // block row and one gradient per direction and reuses them across the block's entries.
    constexpr int NENT = SYM ? NLD * (NLD + 1) / 2 : NLD * NLD;
    constexpr int PER = (NENT + 31) / 32;  // entries per lane (FP64 form)
    constexpr int NBLK = SYM ? NP * (NP + 1) / 2 : NP * NP;
    constexpr int BPL = MIXED ? (NBLK + 31) / 32 : 1;  // blocks per lane (mixed form)
    constexpr int MAPV = NLD * NLD / 4;  // 16-byte chunks of one element's map row
    static_assert(NQ <= 32, "one branch code per lane");
    static_assert((NLD * NLD) % 4 == 0, "map rows are whole 16-byte chunks");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Slice = WarpSlice<DIM, NP, NQ, MIXED>;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    Slice &S = reinterpret_cast<Slice *>(smem_raw)[wid];
    double(*sg)[DIM][NP] = nullptr;  // FP64 form
    double(*sD)[NS * NS] = nullptr;
    double *sH = nullptr;
    df32(*sgm)[DIM][NP] = nullptr;  // mixed form
    df32(*sDm)[NS * NS] = nullptr;
    float2 *sHhl = nullptr;
    if constexpr (MIXED) {
        sgm = S.u.w.sgm;
        sDm = S.u.w.sDm;
        sHhl = S.u.w.sHhl;
    } else {
        sg = S.u.w.sg;
        sD = S.u.w.sD;
        sH = S.u.w.sH;
    }
    double *sK = S.u.sK;
    int32_t *smap = S.smap;
    double(*spt)[NQ] = S.spt;
    int *sq = S.sq;
    const bool map_aligned = (reinterpret_cast<uintptr_t>(A.emap) & 15u) == 0;

    int code[MIXED ? 1 : PER];  // FP64 form: entry alpha | beta << 8 of each of the lane's entries, or -1
    if constexpr (!MIXED) {
#pragma unroll
        for (int i = 0; i < PER; ++i) {
            const int id = lane + i * 32;
            int c = -1;
            if (id < NENT) {
                int a, b;
                if (SYM) {  // row-major upper triangle: row a holds NLD - a entries
                    int rem = id;
                    a = 0;
                    while (rem >= NLD - a) {
                        rem -= NLD - a;
                        ++a;
                    }
                    b = a + rem;
                } else {
                    a = id / NLD;
                    b = id % NLD;
                }
                c = a | (b << 8);
            }
            code[i] = c;
        }
    }
    int blk[BPL];  // mixed form: node pair a | b << 8 of each of the lane's blocks, or -1
#pragma unroll
    for (int j = 0; j < BPL; ++j) {
        const int id = lane + j * 32;
        int c = -1;
        if (MIXED && id < NBLK) {
            int a, b;
            if (SYM) {  // row-major upper triangle of node pairs: row a holds NP - a pairs
                int rem = id;
                a = 0;
                while (rem >= NP - a) {
                    rem -= NP - a;
                    ++a;
                }
                b = a + rem;
            } else {
                a = id / NP;
                b = id % NP;
            }
            c = a | (b << 8);
        }
        blk[j] = c;
    }

    const long long warp_global = (long long)blockIdx.x * WARPS + wid;
    const long long warp_count = (long long)gridDim.x * WARPS;
    const long long n_iter = element_iterations(A);
    for (long long it = warp_global; it < n_iter; it += warp_count) {
        const long long e = element_of(A, it);
        if (e < 0) continue;  // warp-uniform
        const long long g0 = e * NQ;
        bool mine = lane < NQ;
        if (CORR && mine) mine = A.branch[g0 + lane] != 0;
        const unsigned qmask = __ballot_sync(0xffffffffu, mine);
        if (qmask == 0u) continue;  // warp-uniform
        const int nq = __popc(qmask);
        __syncwarp();  // the previous element of this warp is done with the shared slice
        const int32_t *em = A.emap + e * NLD * NLD;
        if (map_aligned) {
            for (int i = lane; i < MAPV; i += 32) cp_async16(smap + 4 * i, em + 4 * i);
        } else {
            for (int i = lane; i < NLD * NLD; i += 32) smap[i] = em[i];
        }
        if (mine) {
            const int k = __popc(qmask & ((1u << lane) - 1u));  // compact list of contributing points
            sq[k] = lane;
            spt[0][k] = A.w[g0 + lane];
            if (CORR) {
                spt[1][k] = A.shear[g0 + lane];
                spt[2][k] = A.lame[g0 + lane];
            }
        }
        __syncwarp();
        for (int i = lane; i < nq * NP; i += 32) {
            const int k = i / NP, a = i % NP;
            const long long src = (g0 + sq[k]) * NP + a;
            const double x = A.d1[src], y = A.d2[src];
            const double z = DIM == 3 ? A.d3[src] : 0.0;
            if (MIXED) {
                sgm[k][0][a] = df_from_f64(x);
                sgm[k][1][a] = df_from_f64(y);
                if (DIM == 3) sgm[k][DIM - 1][a] = df_from_f64(z);
            } else {
                sg[k][0][a] = x;
                sg[k][1][a] = y;
                if (DIM == 3) sg[k][DIM - 1][a] = z;
            }
        }
        for (int i = lane; i < nq * NS * NS; i += 32) {
            const int k = i / (NS * NS), kk = i % (NS * NS);
            const long long g = g0 + sq[k];
            double v = A.DS[g * (NS * NS) + kk];
            if (MIXED) {
                // w s (DS - D_el): the FP64 subtraction only where D_el is nonzero, the scaling by
                // w s as a double-float product
                const double de = elastic_d<DIM>(kk % NS, kk / NS, spt[1][k], spt[2][k]);
                if (de != 0.0) v -= de;
                sDm[k][kk] = df_mul(df_from_f64(v), df_from_f64(A.scale * spt[0][k]));
            } else {
                if (CORR) v = A.scale * (v - elastic_d<DIM>(kk % NS, kk / NS, spt[1][k], spt[2][k]));
                sD[k][kk] = spt[0][k] * v;
            }
        }
        float acc[MIXED ? BPL : 1][DIM][DIM];  // mixed form
        double dacc[MIXED ? 1 : PER];           // FP64 form
#pragma unroll
        for (int j = 0; j < (MIXED ? BPL : 1); ++j)
#pragma unroll
            for (int c = 0; c < DIM; ++c)
#pragma unroll
                for (int c2 = 0; c2 < DIM; ++c2) acc[j][c][c2] = 0.0f;
#pragma unroll
        for (int i = 0; i < (MIXED ? 1 : PER); ++i) dacc[i] = 0.0;
        __syncwarp();
        for (int q = 0; q < nq; ++q) {
            for (int it = lane; it < NLD * NS; it += 32) {
                const int alpha = it / NS, m = it % NS;
                const int a = alpha / DIM, c = alpha % DIM;
                if (MIXED) {  // H = B^T (w D) in double-float arithmetic on the FP32 pipe
                    df32 h = df_mul(sgm[q][0][a], sDm[q][(DIM == 3 ? bt_row3(c, 0) : bt_row2(c, 0)) + NS * m]);
#pragma unroll
                    for (int r = 1; r < DIM; ++r) {
                        const int k = DIM == 3 ? bt_row3(c, r) : bt_row2(c, r);
                        h = df_fma(h, sgm[q][r][a], sDm[q][k + NS * m]);
                    }
                    sHhl[it] = make_float2(h.hi, h.lo);
                } else {
                    double h = 0.0;
#pragma unroll
                    for (int r = 0; r < DIM; ++r) {
                        const int k = DIM == 3 ? bt_row3(c, r) : bt_row2(c, r);
                        h += sg[q][r][a] * sD[q][k + NS * m];
                    }
                    sH[it] = h;
                }
            }
            __syncwarp();
            if constexpr (MIXED) {
                // K[(a,c)][(b,c2)] += sum_r H[(a,c)][m(c2,r)] g[r][b]: per block the DIM gradients of
                // node b and, per block row, the NS entries of H's row are read once;
                // (Hh + Hl)(gh + gl) without the Hl gl term, FP32 accumulation
#pragma unroll
                for (int j = 0; j < BPL; ++j) {
                    const int bc = blk[j];
                    if (bc < 0) continue;
                    const int a = bc & 0xff, b = bc >> 8;
                    df32 gb[DIM];
#pragma unroll
                    for (int r = 0; r < DIM; ++r) gb[r] = sgm[q][r][b];
#pragma unroll
                    for (int c = 0; c < DIM; ++c) {
                        float2 h[NS];
#pragma unroll
                        for (int m = 0; m < NS; ++m) h[m] = sHhl[(a * DIM + c) * NS + m];
#pragma unroll
                        for (int c2 = 0; c2 < DIM; ++c2) {
                            float v = acc[j][c][c2];
#pragma unroll
                            for (int r = 0; r < DIM; ++r) {
                                const float2 hl = h[DIM == 3 ? bt_row3(c2, r) : bt_row2(c2, r)];
                                v = fmaf(hl.x, gb[r].hi, v);
                                v = fmaf(hl.y, gb[r].hi, v);
                                v = fmaf(hl.x, gb[r].lo, v);
                            }
                            acc[j][c][c2] = v;
                        }
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < PER; ++i) {
                    const int c = code[i];
                    if (c >= 0) {
                        const int alpha = c & 0xff, beta = c >> 8;
                        const int b = beta / DIM, cp = beta % DIM;
                        double v = dacc[i];
#pragma unroll
                        for (int r = 0; r < DIM; ++r) v += sH[alpha * NS + (DIM == 3 ? bt_row3(cp, r) : bt_row2(cp, r))] * sg[q][r][b];
                        dacc[i] = v;
                    }
                }
            }
            __syncwarp();
        }
        if (map_aligned) cp_async_wait_all();
        // stage the sums (the products are done with the work buffers), then scatter every entry
        // row by row: consecutive lanes take consecutive columns of one CSR row, so a warp's
        // reductions share cache lines; SYM reads alpha > beta from the mirrored entry
        if constexpr (MIXED) {
#pragma unroll
            for (int j = 0; j < BPL; ++j) {
                const int bc = blk[j];
                if (bc < 0) continue;
                const int a = bc & 0xff, b = bc >> 8;
#pragma unroll
                for (int c = 0; c < DIM; ++c)
#pragma unroll
                    for (int c2 = 0; c2 < DIM; ++c2) {
                        if (SYM && a == b && c2 < c) continue;  // below the diagonal: mirrored in the scatter
                        sK[(a * DIM + c) * NLD + b * DIM + c2] = f32_widen(acc[j][c][c2]);  // exact, integer pipe
                    }
            }
        } else {
#pragma unroll
            for (int i = 0; i < PER; ++i) {
                const int c = code[i];
                if (c >= 0) sK[(c & 0xff) * NLD + (c >> 8)] = dacc[i];
            }
        }
        __syncwarp();
        for (int idx = lane; idx < NLD * NLD; idx += 32) {
            const int alpha = idx / NLD, beta = idx - alpha * NLD;
            const double val = (!SYM || beta >= alpha) ? sK[idx] : sK[beta * NLD + alpha];
            const int32_t p = smap[idx];
            if (p >= 0) {
                if (p < A.nnz) red_add(A.values + p, val);
                else flag(SSP_DEV_BAD_INDEX);
            }
        }
    }
}

// Elements with at least one plastic point (branch != 0), appended to list with warp-aggregated
// atomics (count[0]); the order is unspecified.
__global__ void plastic_elements_kernel(const int8_t *__restrict__ branch, int n_elem, int n_q, int32_t *__restrict__ list,
                                        int32_t *__restrict__ count) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    bool pl = false;
    if (e < n_elem) {
        const int8_t *b = branch + (long long)e * n_q;
        for (int q = 0; q < n_q && !pl; ++q) pl = b[q] != 0;
    }
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, pl);
    if (mask == 0u) return;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if ((int)lane == leader) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (pl) list[base + __popc(mask & ((1u << lane) - 1u))] = e;
}

// Per-point elastic tangent of the return mapping (for assembling the elastic tangent once).
template <int DIM>
__global__ void elastic_blocks_kernel(const double *__restrict__ shear, const double *__restrict__ lame, int n,
                                      double *__restrict__ DS) {
    constexpr int NS = DIM == 3 ? 6 : 3;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * NS * NS) return;
    const long long g = t / (NS * NS);
    const int kk = static_cast<int>(t % (NS * NS));
    DS[t] = elastic_d<DIM>(kk % NS, kk / NS, shear[g], lame[g]);
}

// The elastic rows of a DS whose return mapping left them unwritten: rows of points with branch 0.
template <int DIM>
__global__ void fill_elastic_ds_kernel(const int8_t *__restrict__ branch, const double *__restrict__ shear,
                                       const double *__restrict__ lame, int n, double *__restrict__ DS) {
    constexpr int NS = DIM == 3 ? 6 : 3;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * NS * NS) return;
    const long long g = t / (NS * NS);
    if (branch[g] != 0) return;
    const int kk = static_cast<int>(t % (NS * NS));
    DS[t] = elastic_d<DIM>(kk % NS, kk / NS, shear[g], lame[g]);
}

// ---------------------------------------------------------------------------- P2 correction, moment form
//
// The plastic correction K_e = sum_q B_q^T dD_q B_q of a straight-sided P2 tetrahedron, regrouped.
// Every shape-function gradient is linear in the barycentric coordinates.  With the constant
// lambda_4 = 1 as a fifth coordinate, every node's gradient has exactly two terms
// c lambda_m grad lambda_k:
//   vertex i:     (4 lambda_i - 1) grad lambda_i = 4 lambda_i grad lambda_i - lambda_4 grad lambda_i,
//   edge (i, j):  4 lambda_i grad lambda_j + 4 lambda_j grad lambda_i.
// Hence, with the moments M_mn = sum_q w_q s lambda_qm lambda_qn dD_q (m, n in 0..4) and
// beta_(k,c) the strain of grad lambda_k (x) e_c (three nonzeros),
//   K_e[(a,c),(b,d)] = sum_{x,y = 1,2} c_ax c_by R_(m_ax m_by)[(k_ax, c), (k_by, d)],   R_mn = beta^T M_mn beta,
// four terms per entry for every node pair, so the lanes of a warp do equal work.  Only the ten
// pairs m <= n < 4 are formed from the points; since the coordinates sum to one,
// R_m4 = sum_n R_mn and R_44 = sum_m R_m4.  FP64 operations per element: 21 n_pl (DS - D_el),
// 30 n_pl (weighted coordinate products), 210 n_pl (moments), 2,160 (beta^T M), 2,340 (R),
// 1,170 (the sums), 1,860 (K): about 7,500 + 260 n_pl against about 1,935 n_pl point by point,
// fewer from five plastic points up.  Elements with fewer plastic points keep the point-by-point
// kernel (the element lists are split by ssp_plastic_elements_split).  The result is the
// reference's contraction (assemble_tangent_values_3d.c:135-214) regrouped: equal to rounding.
constexpr int kMaxQ = 11;
constexpr int kMomWarps = 4;  // warps per CTA (one element per warp)
constexpr int kMomEntries = 465;  // alpha <= beta of the 30 x 30 element matrix

struct MomentWarp {
    union {
        struct {
            double M[10][21];  // moments of the pairs m <= n < 4, packed upper triangle of 6 x 6
            double v[4][3];    // grad lambda_0..3
            union {
                struct {
                    double dD[kMaxQ][21];  // DS - D_el of the plastic points, packed upper triangle
                    double ll[kMaxQ][10];  // w s lambda_m lambda_n of the plastic points, pair order
                } in;
                double T[10][12][6];  // (beta_(k,c)^T M_p)[t]
            } t;
        } a;
        double ke[30][31];  // the element's correction, padded rows
    } x;
    double R[15][78];  // R over the pairs m <= n of five coordinates, packed upper triangle of 12 x 12
    int8_t qidx[16];   // the plastic points of the element, in order
};

struct MomentTables {
    unsigned long long k_terms[kMomEntries];  // four (R offset | coefficient code << 11) fields of 16 bits
    uint16_t k_pos[kMomEntries];              // alpha << 5 | beta
    uint16_t r_pos[78];                       // (k,c) << 8 | (l,d), packed upper triangle of 12 x 12
    uint8_t s_pos[21];                        // r << 4 | c, packed upper triangle of 6 x 6
};

// packed upper-triangle index of (i, j) in an n x n symmetric matrix (row-major upper)
__device__ __forceinline__ int sym_index(int i, int j, int n) {
    if (i > j) {
        const int t = i;
        i = j;
        j = t;
    }
    return i * n - (i * (i - 1)) / 2 + (j - i);
}
// (i, j), i <= j, of the packed upper-triangle index p of an n x n matrix
__device__ __forceinline__ void sym_pair(int p, int n, int &i, int &j) {
    i = 0;
    while (p >= n - i) {
        p -= n - i;
        ++i;
    }
    j = i + p;
}

// the (strain row, gradient component) pairs of beta_(k,c)'s three nonzeros (B^T's row of component c)
__device__ __forceinline__ void beta_rows(int c, int *srow, int *gcomp) {
    if (c == 0) { srow[0] = 0; gcomp[0] = 0; srow[1] = 3; gcomp[1] = 1; srow[2] = 5; gcomp[2] = 2; }
    else if (c == 1) { srow[0] = 3; gcomp[0] = 0; srow[1] = 1; gcomp[1] = 1; srow[2] = 4; gcomp[2] = 2; }
    else { srow[0] = 5; gcomp[0] = 0; srow[1] = 4; gcomp[1] = 1; srow[2] = 2; gcomp[2] = 2; }
}

// term t (0, 1) of node a's gradient: coordinate m (0..4), coefficient 4 or -1, gradient k (0..3).
// Nodes 4..9 are the mid-edge nodes of edges 01, 12, 02, 13, 23, 03.
__device__ __forceinline__ void node_term(int a, int t, int &m, int &coef, int &k) {
    if (a < 4) {
        m = t == 0 ? a : 4;
        coef = t == 0 ? 4 : -1;
        k = a;
        return;
    }
    const int i = (a == 5 || a == 7) ? 1 : (a == 8 ? 2 : 0);
    const int j = a == 4 ? 1 : (a == 5 || a == 6) ? 2 : 3;
    m = t == 0 ? i : j;
    k = t == 0 ? j : i;
    coef = 4;
}

__device__ void build_moment_tables(MomentTables &tb) {
    for (int i = threadIdx.x; i < kMomEntries; i += blockDim.x) {
        int al, be;
        sym_pair(i, 30, al, be);
        const int a = al / 3, c = al - 3 * a, b = be / 3, d = be - 3 * b;
        unsigned long long packed = 0;
        for (int x = 0; x < 2; ++x)
            for (int y = 0; y < 2; ++y) {
                int mx, cx, kx, my, cy, ky;
                node_term(a, x, mx, cx, kx);
                node_term(b, y, my, cy, ky);
                const int cc = cx * cy;  // 16, -4 or 1
                const unsigned code = cc == 16 ? 0u : (cc == -4 ? 1u : 2u);
                const unsigned off = static_cast<unsigned>(sym_index(mx, my, 5) * 78 + sym_index(3 * kx + c, 3 * ky + d, 12));
                packed |= static_cast<unsigned long long>(off | (code << 11)) << (16 * (2 * x + y));
            }
        tb.k_terms[i] = packed;
        tb.k_pos[i] = static_cast<uint16_t>(al << 5 | be);
    }
    for (int i = threadIdx.x; i < 78; i += blockDim.x) {
        int kc, ld;
        sym_pair(i, 12, kc, ld);
        tb.r_pos[i] = static_cast<uint16_t>(kc << 8 | ld);
    }
    for (int i = threadIdx.x; i < 21; i += blockDim.x) {
        int r, c;
        sym_pair(i, 6, r, c);
        tb.s_pos[i] = static_cast<uint8_t>(r << 4 | c);
    }
}

__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ double moment_coef(unsigned code) { return code == 0u ? 16.0 : (code == 1u ? -4.0 : 1.0); }

__global__ void __launch_bounds__(32 * kMomWarps) correction_p2_moment_kernel(
    const double *__restrict__ jinv, const double *__restrict__ bary, const double *__restrict__ DS,
    const double *__restrict__ w, const int8_t *__restrict__ branch, const double *__restrict__ shear,
    const double *__restrict__ lame, const int32_t *__restrict__ emap, int n_elem, int n_q, long long nnz,
    double scale, double *__restrict__ values, const int32_t *__restrict__ elist, const int32_t *__restrict__ elist_count) {
    constexpr int kWarps = kMomWarps;
    extern __shared__ __align__(16) unsigned char mom_raw[];
    MomentTables &tb = *reinterpret_cast<MomentTables *>(mom_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    MomentWarp &W = reinterpret_cast<MomentWarp *>(mom_raw + sizeof(MomentTables))[wid];
    build_moment_tables(tb);
    __syncthreads();
    const long long n_iter = *elist_count;
    const long long stride = (long long)gridDim.x * kWarps;
    constexpr int kInBatch = (kMaxQ * 21 + 31) / 32;  // DS entries a lane loads at a time
    constexpr int kMapBatch = 8;                        // map entries a lane loads at a time
    for (long long it = (long long)blockIdx.x * kWarps + wid; it < n_iter; it += stride) {
        const int32_t e32 = elist[it];
        if (e32 < 0 || e32 >= n_elem) {  // warp-uniform
            if (lane == 0) flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const long long e = e32, g0 = e * n_q;
        if (it + stride < n_iter) {  // the next element's DS rows and map row towards L2
            const int32_t en = elist[it + stride];
            if (en >= 0 && en < n_elem) {
                const char *ds_next = reinterpret_cast<const char *>(DS + (long long)en * n_q * 36);
                const char *em_next = reinterpret_cast<const char *>(emap + (long long)en * 900);
                if (lane * 128 < n_q * 288) prefetch_l2(ds_next + lane * 128);
                if (lane * 128 < 3600) prefetch_l2(em_next + lane * 128);
            }
        }
        const bool pl = lane < n_q && branch[g0 + lane] != 0;
        const unsigned qmask = __ballot_sync(0xffffffffu, pl);
        const int nq = __popc(qmask);
        __syncwarp();  // the previous element of this warp is done with its shared slice
        if (pl) W.qidx[__popc(qmask & ((1u << lane) - 1u))] = static_cast<int8_t>(lane);
        if (lane < 9) W.x.a.v[1 + lane / 3][lane % 3] = jinv[e * 9 + lane];
        __syncwarp();
        if (lane < 3) W.x.a.v[0][lane] = -(W.x.a.v[1][lane] + W.x.a.v[2][lane] + W.x.a.v[3][lane]);
        // inputs: DS - D_el of the plastic points (every load of a lane issued before its first use)
        // and their weighted coordinate products
        const int n_in = nq * 21;
        for (int base = 0; base < n_in; base += 32 * kInBatch) {
            double dsv[kInBatch], gv[kInBatch], lv[kInBatch];
#pragma unroll
            for (int u = 0; u < kInBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (i < n_in) {
                    const int kk = i / 21, ee = i - 21 * kk, rc = tb.s_pos[ee];
                    const long long g = g0 + W.qidx[kk];
                    dsv[u] = DS[g * 36 + (rc >> 4) + 6 * (rc & 15)];
                    gv[u] = shear[g];
                    lv[u] = lame[g];
                }
            }
#pragma unroll
            for (int u = 0; u < kInBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (i < n_in) {
                    const int kk = i / 21, ee = i - 21 * kk, rc = tb.s_pos[ee];
                    W.x.a.t.in.dD[kk][ee] = dsv[u] - elastic_d<3>(rc >> 4, rc & 15, gv[u], lv[u]);
                }
            }
        }
        for (int i = lane; i < nq * 10; i += 32) {
            const int kk = i / 10, pp = i - 10 * kk, q = W.qidx[kk];
            int m, n;
            sym_pair(pp, 4, m, n);
            W.x.a.t.in.ll[kk][pp] = (scale * w[g0 + q]) * (bary[q * 4 + m] * bary[q * 4 + n]);
        }
        __syncwarp();
        // moments M_p = sum_q (w s lambda_qm lambda_qn) dD_q, two entries per lane at a time
        for (int i0 = lane; i0 < 210; i0 += 64) {
            const int i1 = i0 + 32 < 210 ? i0 + 32 : i0;
            const int p0 = i0 / 21, e0 = i0 - 21 * p0, p1 = i1 / 21, e1 = i1 - 21 * p1;
            double a0 = 0.0, a1 = 0.0;
            for (int kk = 0; kk < nq; ++kk) {
                a0 = fma(W.x.a.t.in.ll[kk][p0], W.x.a.t.in.dD[kk][e0], a0);
                a1 = fma(W.x.a.t.in.ll[kk][p1], W.x.a.t.in.dD[kk][e1], a1);
            }
            W.x.a.M[p0][e0] = a0;
            W.x.a.M[p1][e1] = a1;
        }
        __syncwarp();
        // T_p[(k,c)][t] = sum over beta_(k,c)'s nonzeros of grad lambda_k[comp] M_p[s][t]
        for (int i0 = lane; i0 < 720; i0 += 64) {
            double acc[2];
            int idx[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = i0 + 32 * h < 720 ? i0 + 32 * h : i0;
                const int pp = i / 72, rr = i - 72 * pp, kc = rr / 6, t = rr - 6 * kc, k = kc / 3, c = kc - 3 * k;
                int sr[3], gc[3];
                beta_rows(c, sr, gc);
                double a = 0.0;
#pragma unroll
                for (int z = 0; z < 3; ++z) a = fma(W.x.a.v[k][gc[z]], W.x.a.M[pp][sym_index(sr[z], t, 6)], a);
                acc[h] = a;
                idx[h] = i;
            }
            (&W.x.a.t.T[0][0][0])[idx[0]] = acc[0];
            (&W.x.a.t.T[0][0][0])[idx[1]] = acc[1];
        }
        __syncwarp();
        // R_p[(k,c),(l,d)] = sum over beta_(l,d)'s nonzeros of T_p[(k,c)][s] grad lambda_l[comp]
        for (int i0 = lane; i0 < 780; i0 += 64) {
            double acc[2];
            int dst[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = i0 + 32 * h < 780 ? i0 + 32 * h : i0;
                const int pp = i / 78, ee = i - 78 * pp;
                const int kc = tb.r_pos[ee] >> 8, ld = tb.r_pos[ee] & 0xff, l = ld / 3, d = ld - 3 * l;
                int m, n;
                sym_pair(pp, 4, m, n);
                int sr[3], gc[3];
                beta_rows(d, sr, gc);
                double a = 0.0;
#pragma unroll
                for (int z = 0; z < 3; ++z) a = fma(W.x.a.t.T[pp][kc][sr[z]], W.x.a.v[l][gc[z]], a);
                acc[h] = a;
                dst[h] = sym_index(m, n, 5) * 78 + ee;
            }
            (&W.R[0][0])[dst[0]] = acc[0];
            (&W.R[0][0])[dst[1]] = acc[1];
        }
        __syncwarp();
        // R_m4 = sum_n R_mn, then R_44 = sum_m R_m4
        for (int i = lane; i < 4 * 78; i += 32) {
            const int m = i / 78, ee = i - 78 * m;
            W.R[sym_index(m, 4, 5)][ee] = (W.R[sym_index(m, 0, 5)][ee] + W.R[sym_index(m, 1, 5)][ee]) +
                                         (W.R[sym_index(m, 2, 5)][ee] + W.R[sym_index(m, 3, 5)][ee]);
        }
        __syncwarp();
        for (int ee = lane; ee < 78; ee += 32)
            W.R[14][ee] = (W.R[4][ee] + W.R[8][ee]) + (W.R[11][ee] + W.R[13][ee]);
        // the first batch of the element -> CSR map, in flight during K
        const int32_t *em = emap + e * 900;
        int32_t pos[kMapBatch];
#pragma unroll
        for (int u = 0; u < kMapBatch; ++u) {
            const int i = lane + 32 * u;
            pos[u] = i < 900 ? em[i] : -1;
        }
        __syncwarp();  // M, T and grad lambda are dead: their storage becomes the element matrix
        const double *Rf = &W.R[0][0];
        for (int i0 = lane; i0 < kMomEntries; i0 += 96) {
            double acc[3];
            int at[3];
#pragma unroll
            for (int h = 0; h < 3; ++h) {
                const int i = i0 + 32 * h < kMomEntries ? i0 + 32 * h : i0;
                const unsigned long long tm = tb.k_terms[i];
                double a = 0.0;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const unsigned f = static_cast<unsigned>(tm >> (16 * t)) & 0xffffu;
                    a = fma(moment_coef(f >> 11), Rf[f & 0x7ffu], a);
                }
                acc[h] = a;
                at[h] = tb.k_pos[i];
            }
#pragma unroll
            for (int h = 0; h < 3; ++h) {
                const int al = at[h] >> 5, be = at[h] & 31;
                W.x.ke[al][be] = acc[h];
                W.x.ke[be][al] = acc[h];
            }
        }
        __syncwarp();
        // scatter through the element -> CSR map (both mirror positions were written)
        for (int base = 0; base < 900; base += 32 * kMapBatch) {
            if (base > 0) {
#pragma unroll
                for (int u = 0; u < kMapBatch; ++u) {
                    const int i = base + lane + 32 * u;
                    pos[u] = i < 900 ? em[i] : -1;
                }
            }
#pragma unroll
            for (int u = 0; u < kMapBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (pos[u] < 0) continue;
                if (pos[u] >= nnz) {
                    flag(SSP_DEV_BAD_INDEX);
                    continue;
                }
                red_add(values + pos[u], W.x.ke[i / 30][i % 30]);
            }
        }
    }
}

// ---------------------------------------------------------------------------- P2 correction, moment form, FP32
//
// The mixed form of the kernel above: DS - D_el and w s in FP64, rounded to FP32; the moments,
// beta^T M beta, the lambda_4 sums and the element matrix in FP32; the element's 900 sums widened
// exactly and reduced into the FP64 CSR values.  With the FP32 pipe far faster than the FP64 one,
// the layout is chosen for few instructions rather than few operations: full 6 x 6 moments (their
// shared-memory addresses a lane base plus constants), beta^T M beta formed in registers by one
// lane per (pair, component) and stored by rows of the packed 12 x 12 upper triangle, the K entries
// grouped by node-pair type so each group's four coefficients are constants, the element matrix
// unpadded.  8.4 KB of shared memory per warp: three 8-warp CTAs per SM.
constexpr int kF32Warps = 8;
constexpr int kF32KEntries = 512;        // vertex-vertex 78 -> 96, vertex-edge 216 -> 224, edge-edge 171 -> 192
constexpr int kF32VertexVertexIters = 3, kF32VertexEdgeIters = 7;

struct MomentF32Tables {
    unsigned long long k_terms[kF32KEntries];  // four packed R offsets (16-bit fields), term order (x, y)
    uint16_t k_pos[kF32KEntries];             // alpha << 5 | beta; 0xFFFF pads a type group
    float lam[kMaxQ][4];                      // the points' barycentric coordinates, rounded to FP32
    uint8_t s_pos[21];                        // r << 4 | c of the packed upper triangle of 6 x 6
    uint8_t pair_mn[10];                      // m << 4 | n of the pairs m <= n < 4
};

struct MomentF32Warp {
    union {
        struct {
            float dD[kMaxQ][21];  // DS - D_el of the plastic points, packed upper triangle
            float ws[12];         // w s of the plastic points
            float ll[kMaxQ][10];  // w s lambda_m lambda_n, pair order
            float M[10][36];      // moments, full 6 x 6
        } a;
        float ke[900];  // the element's correction, 30 x 30 row-major
    } x;
    float v[4][3];      // grad lambda_0..3
    float R[15][78];    // R over the pairs m <= n of five coordinates, packed upper triangle of 12 x 12
    int8_t qidx[16];
};

// FP64 -> FP32 rounded to nearest even by integer operations (values below the FP32 normal range
// flush to a signed zero; overflow gives +-inf, nan stays nan).
__device__ __forceinline__ float f64_to_f32_bits(double x) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned sign = static_cast<unsigned>(u >> 32) & 0x80000000u;
    const int e = static_cast<int>((u >> 52) & 0x7FFull);
    const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
    if (e == 0x7FF) return __uint_as_float(sign | 0x7F800000u | (m ? 0x400000u : 0u));
    const int ef = e - 1023 + 127;
    if (ef <= 0) return __uint_as_float(sign);
    if (ef >= 255) return __uint_as_float(sign | 0x7F800000u);
    unsigned f = (static_cast<unsigned>(ef) << 23) | static_cast<unsigned>(m >> 29);
    const unsigned r = static_cast<unsigned>(m & 0x1FFFFFFFull);
    f += (r > 0x10000000u || (r == 0x10000000u && (f & 1u))) ? 1u : 0u;  // a carry into the exponent rounds up
    return __uint_as_float(sign | f);
}

__device__ void build_moment_f32_tables(MomentF32Tables &tb, const double *bary, int n_q) {
    for (int i = threadIdx.x; i < kF32KEntries; i += blockDim.x) {
        int al = -1, be = -1;
        if (i < 32 * kF32VertexVertexIters) {
            if (i < 78) sym_pair(i, 12, al, be);
        } else if (i < 32 * (kF32VertexVertexIters + kF32VertexEdgeIters)) {
            const int j = i - 32 * kF32VertexVertexIters;
            if (j < 216) {
                al = j / 18;
                be = 12 + j % 18;
            }
        } else {
            const int j = i - 32 * (kF32VertexVertexIters + kF32VertexEdgeIters);
            if (j < 171) {
                sym_pair(j, 18, al, be);
                al += 12;
                be += 12;
            }
        }
        unsigned long long packed = 0;
        if (al >= 0) {
            const int a = al / 3, c = al - 3 * a, b = be / 3, d = be - 3 * b;
            for (int x = 0; x < 2; ++x)
                for (int y = 0; y < 2; ++y) {
                    int mx, cx, kx, my, cy, ky;
                    node_term(a, x, mx, cx, kx);
                    node_term(b, y, my, cy, ky);
                    const unsigned off = static_cast<unsigned>(sym_index(mx, my, 5) * 78 + sym_index(3 * kx + c, 3 * ky + d, 12));
                    packed |= static_cast<unsigned long long>(off) << (16 * (2 * x + y));
                }
        }
        tb.k_terms[i] = packed;
        tb.k_pos[i] = al >= 0 ? static_cast<uint16_t>(al << 5 | be) : static_cast<uint16_t>(0xFFFFu);
    }
    for (int i = threadIdx.x; i < n_q * 4; i += blockDim.x) tb.lam[i >> 2][i & 3] = f64_to_f32_bits(bary[i]);
    for (int i = threadIdx.x; i < 21; i += blockDim.x) {
        int r, c;
        sym_pair(i, 6, r, c);
        tb.s_pos[i] = static_cast<uint8_t>(r << 4 | c);
    }
    for (int i = threadIdx.x; i < 10; i += blockDim.x) {
        int m, n;
        sym_pair(i, 4, m, n);
        tb.pair_mn[i] = static_cast<uint8_t>(m << 4 | n);
    }
}

__global__ void __launch_bounds__(32 * kF32Warps, 3) correction_p2_moment_f32_kernel(
    const double *__restrict__ jinv, const double *__restrict__ bary, const double *__restrict__ DS,
    const double *__restrict__ w, const int8_t *__restrict__ branch, const double *__restrict__ shear,
    const double *__restrict__ lame, const int32_t *__restrict__ emap, int n_elem, int n_q, long long nnz,
    double scale, double *__restrict__ values, const int32_t *__restrict__ elist, const int32_t *__restrict__ elist_count) {
    extern __shared__ __align__(16) unsigned char mom_raw[];
    MomentF32Tables &tb = *reinterpret_cast<MomentF32Tables *>(mom_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    MomentF32Warp &W = reinterpret_cast<MomentF32Warp *>(mom_raw + sizeof(MomentF32Tables))[wid];
    build_moment_f32_tables(tb, bary, n_q);
    __syncthreads();
    const long long n_iter = *elist_count;
    const long long stride = (long long)gridDim.x * kF32Warps;
    constexpr int kInBatch = 4;   // DS entries a lane loads at a time
    constexpr int kMapBatch = 8;  // map entries a lane loads at a time
    for (long long it = (long long)blockIdx.x * kF32Warps + wid; it < n_iter; it += stride) {
        const int32_t e32 = elist[it];
        if (e32 < 0 || e32 >= n_elem) {  // warp-uniform
            if (lane == 0) flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const long long e = e32, g0 = e * n_q;
        if (it + stride < n_iter) {  // the next element's DS rows and map row towards L2
            const int32_t en = elist[it + stride];
            if (en >= 0 && en < n_elem) {
                const char *ds_next = reinterpret_cast<const char *>(DS + (long long)en * n_q * 36);
                const char *em_next = reinterpret_cast<const char *>(emap + (long long)en * 900);
                if (lane * 128 < n_q * 288) prefetch_l2(ds_next + lane * 128);
                if (lane * 128 < 3600) prefetch_l2(em_next + lane * 128);
            }
        }
        const bool pl = lane < n_q && branch[g0 + lane] != 0;
        const unsigned qmask = __ballot_sync(0xffffffffu, pl);
        const int nq = __popc(qmask);
        __syncwarp();  // the previous element of this warp is done with its shared slice
        if (pl) {
            const int kk = __popc(qmask & ((1u << lane) - 1u));
            W.qidx[kk] = static_cast<int8_t>(lane);
            W.x.a.ws[kk] = f64_to_f32_bits(scale * w[g0 + lane]);
        }
        if (lane < 9) W.v[1 + lane / 3][lane % 3] = f64_to_f32_bits(jinv[e * 9 + lane]);
        __syncwarp();
        if (lane < 3) W.v[0][lane] = -(W.v[1][lane] + W.v[2][lane] + W.v[3][lane]);
        // DS - D_el in FP64, rounded to FP32 (every load of a batch issued before its first use)
        const int n_in = nq * 21;
        for (int base = 0; base < n_in; base += 32 * kInBatch) {
            double dsv[kInBatch], gv[kInBatch], lv[kInBatch];
#pragma unroll
            for (int u = 0; u < kInBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (i < n_in) {
                    const int kk = i / 21, ee = i - 21 * kk, rc = tb.s_pos[ee];
                    const long long g = g0 + W.qidx[kk];
                    dsv[u] = DS[g * 36 + (rc >> 4) + 6 * (rc & 15)];
                    gv[u] = shear[g];
                    lv[u] = lame[g];
                }
            }
#pragma unroll
            for (int u = 0; u < kInBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (i < n_in) {
                    const int kk = i / 21, ee = i - 21 * kk, rc = tb.s_pos[ee];
                    W.x.a.dD[kk][ee] = f64_to_f32_bits(dsv[u] - elastic_d<3>(rc >> 4, rc & 15, gv[u], lv[u]));
                }
            }
        }
        for (int i = lane; i < nq * 10; i += 32) {
            const int kk = i / 10, pp = i - 10 * kk, q = W.qidx[kk], mn = tb.pair_mn[pp];
            W.x.a.ll[kk][pp] = W.x.a.ws[kk] * (tb.lam[q][mn >> 4] * tb.lam[q][mn & 15]);
        }
        __syncwarp();
        // moments, both mirror positions of the full 6 x 6
        for (int i0 = lane; i0 < 210; i0 += 64) {
            const int i1 = i0 + 32 < 210 ? i0 + 32 : i0;
            const int p0 = i0 / 21, e0 = i0 - 21 * p0, p1 = i1 / 21, e1 = i1 - 21 * p1;
            float a0 = 0.0f, a1 = 0.0f;
            for (int kk = 0; kk < nq; ++kk) {
                a0 = __fmaf_rn(W.x.a.ll[kk][p0], W.x.a.dD[kk][e0], a0);
                a1 = __fmaf_rn(W.x.a.ll[kk][p1], W.x.a.dD[kk][e1], a1);
            }
            const int rc0 = tb.s_pos[e0], rc1 = tb.s_pos[e1];
            W.x.a.M[p0][(rc0 >> 4) * 6 + (rc0 & 15)] = a0;
            W.x.a.M[p0][(rc0 & 15) * 6 + (rc0 >> 4)] = a0;
            W.x.a.M[p1][(rc1 >> 4) * 6 + (rc1 & 15)] = a1;
            W.x.a.M[p1][(rc1 & 15) * 6 + (rc1 >> 4)] = a1;
        }
        __syncwarp();
        // R_p = beta^T M_p beta: lane (p, c) forms T[k][t] = sum_z grad lambda_k[z] M_p[s_z(c)][t] and
        // the rows (k, c) of R_p, R[(k,c),(l,d)] = sum_z T[k][s_z(d)] grad lambda_l[z]
        if (lane < 30) {
            const int p = lane / 3, c = lane - 3 * p, mn = tb.pair_mn[p];
            float vk[4][3];
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int z = 0; z < 3; ++z) vk[k][z] = W.v[k][z];
            int sr[3], gc[3];
            beta_rows(c, sr, gc);  // gc = (0, 1, 2) for every c
            const float *m0 = &W.x.a.M[p][sr[0] * 6], *m1 = &W.x.a.M[p][sr[1] * 6], *m2 = &W.x.a.M[p][sr[2] * 6];
            float T[4][6];
#pragma unroll
            for (int t = 0; t < 6; ++t) {
                const float x0 = m0[t], x1 = m1[t], x2 = m2[t];
#pragma unroll
                for (int k = 0; k < 4; ++k) T[k][t] = __fmaf_rn(vk[k][2], x2, __fmaf_rn(vk[k][1], x1, vk[k][0] * x0));
            }
            // row i = 3k + c of the packed upper triangle starts at i * 12 - i (i - 1) / 2 - i; the
            // entries j = 3l + d >= i are stored (l > k always, l == k when d >= c)
            float *Rp = &W.R[sym_index(mn >> 4, mn & 15, 5)][0];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = 3 * k + c;
                float *row = Rp + (i * 11 - (i * (i - 1)) / 2);
#pragma unroll
                for (int l = k; l < 4; ++l)
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        int sd[3], gd[3];
                        beta_rows(d, sd, gd);
                        if (l > k || d >= c)
                            row[3 * l + d] = __fmaf_rn(T[k][sd[2]], vk[l][2],
                                                       __fmaf_rn(T[k][sd[1]], vk[l][1], T[k][sd[0]] * vk[l][0]));
                    }
            }
        }
        __syncwarp();
        // R_m4 = sum_n R_mn, R_44 = sum_m R_m4 (pair indices over five coordinates)
        for (int ee = lane; ee < 78; ee += 32) {
            const float r00 = W.R[0][ee], r01 = W.R[1][ee], r02 = W.R[2][ee], r03 = W.R[3][ee];
            const float r11 = W.R[5][ee], r12 = W.R[6][ee], r13 = W.R[7][ee];
            const float r22 = W.R[9][ee], r23 = W.R[10][ee], r33 = W.R[12][ee];
            const float s0 = (r00 + r01) + (r02 + r03), s1 = (r01 + r11) + (r12 + r13);
            const float s2 = (r02 + r12) + (r22 + r23), s3 = (r03 + r13) + (r23 + r33);
            W.R[4][ee] = s0;
            W.R[8][ee] = s1;
            W.R[11][ee] = s2;
            W.R[13][ee] = s3;
            W.R[14][ee] = (s0 + s1) + (s2 + s3);
        }
        // the first batch of the element -> CSR map, in flight during K
        const int32_t *em = emap + e * 900;
        int32_t pos[kMapBatch];
#pragma unroll
        for (int u = 0; u < kMapBatch; ++u) {
            const int i = lane + 32 * u;
            pos[u] = i < 900 ? em[i] : -1;
        }
        __syncwarp();  // the moments and inputs are dead: their storage becomes the element matrix
        const float *Rf = &W.R[0][0];
#pragma unroll 1
        for (int k0 = 0; k0 < kF32KEntries / 32; ++k0) {
            const int i = 32 * k0 + lane;
            const unsigned long long tm = tb.k_terms[i];
            const float r0 = Rf[tm & 0xFFFu], r1 = Rf[(tm >> 16) & 0xFFFu], r2 = Rf[(tm >> 32) & 0xFFFu],
                        r3 = Rf[(tm >> 48) & 0xFFFu];
            float kv;
            if (k0 < kF32VertexVertexIters)  // (4, -1) x (4, -1)
                kv = __fmaf_rn(16.0f, r0, __fmaf_rn(-4.0f, r1 + r2, r3));
            else if (k0 < kF32VertexVertexIters + kF32VertexEdgeIters)  // (4, -1) x (4, 4)
                kv = __fmaf_rn(16.0f, r0 + r1, -4.0f * (r2 + r3));
            else  // (4, 4) x (4, 4)
                kv = 16.0f * ((r0 + r1) + (r2 + r3));
            const unsigned pk = tb.k_pos[i];
            if (pk != 0xFFFFu) {
                const int al = pk >> 5, be = pk & 31;
                W.x.ke[al * 30 + be] = kv;
                W.x.ke[be * 30 + al] = kv;
            }
        }
        __syncwarp();
        // scatter through the element -> CSR map (both mirror positions were written)
        for (int base = 0; base < 900; base += 32 * kMapBatch) {
            if (base > 0) {
#pragma unroll
                for (int u = 0; u < kMapBatch; ++u) {
                    const int i = base + lane + 32 * u;
                    pos[u] = i < 900 ? em[i] : -1;
                }
            }
#pragma unroll
            for (int u = 0; u < kMapBatch; ++u) {
                const int i = base + lane + 32 * u;
                if (pos[u] < 0) continue;
                if (pos[u] >= nnz) {
                    flag(SSP_DEV_BAD_INDEX);
                    continue;
                }
                red_add(values + pos[u], f32_widen(W.x.ke[i]));
            }
        }
    }
}

// Plastic elements split by their number of plastic points: fewer than min_points to list_few,
// at least min_points to list_many (warp-aggregated appends).
__global__ void plastic_elements_split_kernel(const int8_t *__restrict__ branch, int n_elem, int n_q, int min_points,
                                              int32_t *__restrict__ list_few, int32_t *__restrict__ count_few,
                                              int32_t *__restrict__ list_many, int32_t *__restrict__ count_many) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    int np = 0;
    if (e < n_elem) {
        const int8_t *b = branch + (long long)e * n_q;
        for (int q = 0; q < n_q; ++q) np += b[q] != 0;
    }
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int which = 0; which < 2; ++which) {
        const bool want = which == 0 ? (np > 0 && np < min_points) : np >= min_points;
        int32_t *list = which == 0 ? list_few : list_many;
        int32_t *count = which == 0 ? count_few : count_many;
        const unsigned mask = __ballot_sync(0xffffffffu, want);
        if (mask == 0u) continue;
        const int leader = __ffs(mask) - 1;
        int base = 0;
        if ((int)lane == leader) base = atomicAdd(count, __popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (want) list[base + __popc(mask & ((1u << lane) - 1u))] = e;
    }
}

// ---------------------------------------------------------------------------- epilogue

__global__ void set_positions_kernel(double *__restrict__ values, const int32_t *__restrict__ pos, int n, long long nnz,
                                     double v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t p = pos[i];
    if (p < 0 || p >= nnz) {
        flag(SSP_DEV_BAD_INDEX);
        return;
    }
    values[p] = v;
}

__global__ void blend_kernel(double *__restrict__ values, const double *__restrict__ elastic, long long nnz, double r) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    values[i] = values[i] * (1.0 - r) + r * elastic[i];
}

__global__ void blend_base_kernel(double *__restrict__ out, const double *__restrict__ base,
                                  const double *__restrict__ elastic, long long nnz, double r) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nnz) return;
    out[i] = base[i] * (1.0 - r) + r * elastic[i];
}

// Device -> host copy by the SMs (16-byte stores when both ends are 16-byte aligned) into pinned,
// device-mapped host memory: on a part whose host link is coherent the stores stream straight over
// it, and several SMs keep more of it busy than one copy engine.
__global__ void copy_out_kernel(const double *__restrict__ src, long long n, double *__restrict__ dst, int vec) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (vec) {
        const long long n2 = n / 2;
        const double2 *s2 = reinterpret_cast<const double2 *>(src);
        double2 *d2 = reinterpret_cast<double2 *>(dst);
        for (long long k = i; k < n2; k += stride) d2[k] = s2[k];
        if (i == 0 && (n & 1)) dst[n - 1] = src[n - 1];
    } else {
        for (long long k = i; k < n; k += stride) dst[k] = src[k];
    }
}

// row_mark[r] = 1 for every owned row r = elem_row[e][a] of the listed elements e.
__global__ void mark_rows_kernel(const int32_t *__restrict__ elem_row, int n_elem, int n_ld,
                                 const int32_t *__restrict__ list, const int32_t *__restrict__ count, int n_rows,
                                 uint8_t *__restrict__ mark) {
    const long long total = (long long)count[0] * n_ld;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long k = i / n_ld;
        const int e = list[k];
        if (e < 0 || e >= n_elem) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const int r = elem_row[(long long)e * n_ld + (i - k * n_ld)];
        if (r < 0) continue;
        if (r < n_rows) mark[r] = 1;
        else flag(SSP_DEV_BAD_INDEX);
    }
}

// The marked CSR rows of src stored to dst (device-mapped host memory), a warp per row.  With both
// arrays 16-byte aligned (vec) the row's body goes as 16-byte stores, 512 contiguous bytes per warp
// instruction over the host link, an odd first or last value as one 8-byte store; unmarked rows
// cost one byte read.
__global__ void copy_rows_out_kernel(const double *__restrict__ src, const int32_t *__restrict__ indptr,
                                     const uint8_t *__restrict__ mark, int n_rows, long long nnz,
                                     double *__restrict__ dst, int vec) {
    const int lane = threadIdx.x & 31;
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; row < n_rows; row += warps) {
        if (!mark[row]) continue;
        const long long b = indptr[row], e = indptr[row + 1];
        if (b < 0 || e < b || e > nnz) {
            if (lane == 0) flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        if (!vec) {
            for (long long k = b + lane; k < e; k += 32) dst[k] = src[k];
            continue;
        }
        const long long b2 = (b + 1) & ~1ll, e2 = e & ~1ll;  // [b2, e2): whole 16-byte pairs
        if (b2 >= e2) {  // fewer than two values past an odd start
            for (long long k = b + lane; k < e; k += 32) dst[k] = src[k];
            continue;
        }
        if (lane == 0 && b < b2) dst[b] = src[b];
        if (lane == 1 && e2 < e) dst[e2] = src[e2];
        const double2 *s2 = reinterpret_cast<const double2 *>(src + b2);
        double2 *d2 = reinterpret_cast<double2 *>(dst + b2);
        for (long long k = lane; k < (e2 - b2) / 2; k += 32) d2[k] = s2[k];
    }
}

__global__ void gather_rows_kernel(const double *__restrict__ src, const int32_t *__restrict__ idx, int n,
                                   double *__restrict__ dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

// ---------------------------------------------------------------------------- dispatch

template <int DIM, int NP, int NQ, int THREADS, bool SYM, bool CORR>
int launch_element(const ElemArgs &a, cudaStream_t st) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tangent_element_kernel<DIM, NP, NQ, THREADS, SYM, CORR>,
                                                  THREADS, 0);
    if (per_sm < 1) per_sm = 1;
    long long grid = (long long)sms * per_sm;
    if (grid > a.n_elem) grid = a.n_elem;
    tangent_element_kernel<DIM, NP, NQ, THREADS, SYM, CORR><<<static_cast<unsigned>(grid), THREADS, 0, st>>>(a);
    return launch_status();
}

template <int DIM, int NP, int NQ, bool SYM, bool CORR, bool MIXED = false>
int launch_element_warp(const ElemArgs &a, cudaStream_t st) {
    constexpr int WARPS = 4;
    constexpr size_t smem = WARPS * sizeof(WarpSlice<DIM, NP, NQ, MIXED>);
    auto kernel = tangent_element_warp_kernel<DIM, NP, NQ, WARPS, SYM, CORR, MIXED>;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
        cudaSuccess)
        return SSP_ERR_CUDA;
    // the mixed form fits five CTAs per SM when the unified L1 / shared memory is mostly shared
    if (MIXED && cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return SSP_ERR_CUDA;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * WARPS, smem);
    if (per_sm < 1) per_sm = 1;
    long long grid = (long long)sms * per_sm;
    const long long need = (a.n_elem + WARPS - 1) / WARPS;
    if (grid > need) grid = need;
    kernel<<<static_cast<unsigned>(grid), 32 * WARPS, smem, st>>>(a);
    return launch_status();
}

template <bool SYM, bool CORR>
int dispatch_element(int dim, int n_p, int n_q, const ElemArgs &a, cudaStream_t st) {
    if (dim == 3 && n_p == 10 && n_q == 11) return launch_element_warp<3, 10, 11, SYM, CORR>(a, st);
    if (dim == 3 && n_p == 35 && n_q == 24) return launch_element<3, 35, 24, 256, SYM, CORR>(a, st);
    if (dim == 3 && n_p == 4 && n_q == 1) return launch_element<3, 4, 1, 32, SYM, CORR>(a, st);
    if (dim == 2 && n_p == 6 && n_q == 7) return launch_element<2, 6, 7, 32, SYM, CORR>(a, st);
    if (dim == 2 && n_p == 3 && n_q == 1) return launch_element<2, 3, 1, 32, SYM, CORR>(a, st);
    if (dim == 2 && n_p == 15 && n_q == 12) return launch_element_warp<2, 15, 12, SYM, CORR>(a, st);
    return SSP_ERR_UNSUPPORTED;
}

// persistent grid: as many CTAs as fit on the device, one element per warp at a time
template <typename Kernel>
int launch_p2_moments(Kernel kernel, int warps, size_t smem, const double *jinv, const double *bary, const double *ds,
                      const double *weight, const int8_t *branch, const double *shear, const double *lame,
                      const int32_t *scatter_map, int n_elem, int n_q, long long nnz_out, double scale,
                      double *out_values, const int32_t *elem_list, const int32_t *elem_count, cudaStream_t st) {
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
        return SSP_ERR_CUDA;
    int dev = 0, sms = 148, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * warps, smem);
    if (per_sm < 1) per_sm = 1;
    long long grid = (long long)sms * per_sm;
    const long long need = (n_elem + warps - 1) / warps;
    if (grid > need) grid = need;
    kernel<<<static_cast<unsigned>(grid), 32 * warps, smem, st>>>(jinv, bary, ds, weight, branch, shear, lame,
                                                                 scatter_map, n_elem, n_q, nnz_out, scale, out_values,
                                                                 elem_list, elem_count);
    return launch_status();
}

}  // namespace
}  // namespace ssp

using namespace ssp;

extern "C" {

int ssp_geometry(int dim, const double *coord, const int64_t *elem, const double *dhat, const double *wf, int n_nodes,
                 int n_elem, int n_p, int n_q, double *dphi1, double *dphi2, double *dphi3, double *weight,
                 void *stream) {
    if ((dim != 2 && dim != 3) || n_elem < 0 || n_p <= 0 || n_q <= 0 || n_nodes < 0) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!coord || !elem || !dhat || !wf || !dphi1 || !dphi2 || !weight || (dim == 3 && !dphi3)) return SSP_ERR_INVALID;
    const long long n = (long long)n_elem * n_q;
    if (dim == 3)
        geometry_kernel<3><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(coord, elem, dhat, wf, n_nodes, n_elem, n_p,
                                                                            n_q, dphi1, dphi2, dphi3, weight);
    else
        geometry_kernel<2><<<grid_for(n, 128), 128, 0, as_stream(stream)>>>(coord, elem, dhat, wf, n_nodes, n_elem, n_p,
                                                                            n_q, dphi1, dphi2, nullptr, weight);
    return launch_status();
}

int ssp_assemble_overlap_strain_3d(const double *dphi1, const double *dphi2, const double *dphi3,
                                   const double *u_overlap, int n_u, const int32_t *elem_dof_lids, int n_int,
                                   int n_elem, int n_p, int n_q, double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || !dphi3 || !u_overlap || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    strain3_kernel<<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(dphi1, dphi2, dphi3, u_overlap, elem_dof_lids, n_u,
                                                                        n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_overlap_strain_2d(const double *dphi1, const double *dphi2, const double *u_overlap, int n_u,
                                   const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                   double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || !u_overlap || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    strain2_kernel<<<grid_for(n_int, 128), 128, 0, as_stream(stream)>>>(dphi1, dphi2, u_overlap, elem_dof_lids, n_u,
                                                                        n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_3d_rows(const double *dphi1, const double *dphi2, const double *dphi3, const double *stress,
                               const double *weight, const int32_t *row_slot_ptr, const int32_t *slot_elem,
                               const uint8_t *slot_lrow, int n_int, int n_rows, int n_slots, int n_p, int n_q,
                               double *out_values, void *stream) {
    (void)n_slots;
    if (n_rows < 0 || n_p <= 0 || n_q <= 0 || n_int < 0 || n_int % n_q) return SSP_ERR_INVALID;
    if (n_rows == 0) return SSP_OK;
    if (!row_slot_ptr || !out_values) return SSP_ERR_INVALID;
    force_rows3_kernel<<<grid_for(n_rows, 128), 128, 0, as_stream(stream)>>>(
        dphi1, dphi2, dphi3, stress, weight, row_slot_ptr, slot_elem, slot_lrow, n_rows, n_int / n_q, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                               const double *stress, const double *weight, const int32_t *elem_row, int n_elem,
                               int n_p, int n_q, int n_rows, double *out_values, void *stream) {
    if ((dim != 2 && dim != 3) || n_elem < 0 || n_p <= 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || (dim == 3 && !dphi3) || !stress || !weight || !elem_row) return SSP_ERR_INVALID;
    const long long n = (long long)n_elem * dim * n_p;
    if (dim == 3)
        force_element_kernel<3><<<grid_for(n, 128), 128, 0, st>>>(dphi1, dphi2, dphi3, stress, weight, elem_row, n_rows,
                                                                  n_elem, n_p, n_q, out_values);
    else
        force_element_kernel<2><<<grid_for(n, 128), 128, 0, st>>>(dphi1, dphi2, nullptr, stress, weight, elem_row, n_rows,
                                                                  n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_overlap_strain_3d_p2_affine(const double *jinv, const double *bary, const double *u_overlap, int n_u,
                                             const int32_t *elem_dof_lids, int n_int, int n_elem, int n_q,
                                             double *out_values, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !bary || !u_overlap || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    strain3_p2_affine_kernel<<<grid_for(n_elem, 64), 64, 0, as_stream(stream)>>>(jinv, bary, u_overlap, elem_dof_lids,
                                                                                 n_u, n_elem, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element_p2_affine(const double *jinv, const double *bary, const double *stress,
                                         const double *weight, const int32_t *elem_row, int n_elem, int n_q,
                                         int n_rows, double *out_values, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !bary || !stress || !weight || !elem_row) return SSP_ERR_INVALID;
    force3_p2_affine_kernel<<<grid_for(n_elem, 64), 64, 0, st>>>(jinv, bary, stress, weight, elem_row, n_rows, n_elem,
                                                                 n_q, out_values);
    return launch_status();
}

int ssp_assemble_overlap_strain_3d_affine(const double *jinv, const double *ghat, const double *u_overlap, int n_u,
                                          const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                          double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_u < 0) return SSP_ERR_INVALID;
    if ((long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !ghat || !u_overlap || !elem_dof_lids || !out_values) return SSP_ERR_INVALID;
    // the table plus the displacements of the at most 128 / n_q + 2 elements a block's points cover
    const size_t smem = sizeof(double) * (3 * (size_t)n_p * n_q + 3 * (size_t)n_p * (kAffineThreads / n_q + 2));
    if (smem > 48 * 1024) return SSP_ERR_UNSUPPORTED;
    strain3_affine_kernel<<<grid_for(n_int, kAffineThreads), kAffineThreads, smem, as_stream(stream)>>>(
        jinv, ghat, u_overlap, elem_dof_lids, n_u, n_elem, n_p, n_q, out_values);
    return launch_status();
}

int ssp_assemble_force_element_affine(const double *jinv, const double *ghat, const double *stress,
                                      const double *weight, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                      int n_rows, double *out_values, void *stream) {
    if (n_elem < 0 || n_p <= 0 || n_q <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    // a block's threads cover at most 128 / n_p + 2 elements, whose points' T it stages
    const size_t smem = sizeof(double) * (3 * (size_t)n_p * n_q + 9 * (size_t)(kAffineThreads / n_p + 2) * n_q);
    if (smem > 48 * 1024) return SSP_ERR_UNSUPPORTED;
    if (!out_values && n_rows > 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_rows > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * n_rows, st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !ghat || !stress || !weight || !elem_row) return SSP_ERR_INVALID;
    const long long n = (long long)n_elem * n_p;
    force3_affine_kernel<<<grid_for(n, kAffineThreads), kAffineThreads, smem, st>>>(jinv, ghat, weight, stress,
                                                                                    elem_row, n_rows, n_elem, n_p, n_q,
                                                                                    out_values);
    return launch_status();
}

int ssp_assemble_tangent_values_3d_rows(const double *dphi1, const double *dphi2, const double *dphi3, const double *ds,
                                        const double *weight, const int32_t *row_slot_ptr, const int32_t *slot_elem,
                                        const uint8_t *slot_lrow, const int32_t *slot_pos, int n_int, int n_rows,
                                        int n_slots, int n_p, int n_q, int nnz_out, double *out_values, void *stream) {
    (void)n_slots;
    if (n_rows < 0 || n_p <= 0 || n_q <= 0 || nnz_out < 0 || n_int < 0 || n_int % n_q) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (nnz_out > 0) {
        if (!out_values) return SSP_ERR_INVALID;
        if (cudaMemsetAsync(out_values, 0, sizeof(double) * nnz_out, st) != cudaSuccess) return SSP_ERR_CUDA;
    }
    if (n_rows == 0) return SSP_OK;
    if (!row_slot_ptr) return SSP_ERR_INVALID;
    tangent_rows3_kernel<<<grid_for(n_rows, 64), 64, 0, st>>>(dphi1, dphi2, dphi3, ds, weight, row_slot_ptr, slot_elem,
                                                              slot_lrow, slot_pos, n_rows, n_int / n_q, n_p, n_q, nnz_out,
                                                              out_values);
    return launch_status();
}

int ssp_tangent_element(int dim, int symmetric, const double *dphi1, const double *dphi2, const double *dphi3,
                        const double *ds, const double *weight, const int32_t *scatter_map, int n_elem, int n_p, int n_q,
                        long long nnz_out, double *out_values, int accumulate, void *stream) {
    if ((dim != 2 && dim != 3) || n_elem < 0 || n_p <= 0 || n_q <= 0 || nnz_out < 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (nnz_out > 0 && !out_values) return SSP_ERR_INVALID;
    if (!accumulate && nnz_out > 0 && cudaMemsetAsync(out_values, 0, sizeof(double) * nnz_out, st) != cudaSuccess)
        return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || (dim == 3 && !dphi3) || !ds || !weight || !scatter_map) return SSP_ERR_INVALID;
    ElemArgs a{dphi1, dphi2, dphi3, ds, weight, scatter_map, n_elem, nnz_out, out_values, nullptr, nullptr, nullptr, 1.0};
    return symmetric ? dispatch_element<true, false>(dim, n_p, n_q, a, st) : dispatch_element<false, false>(dim, n_p, n_q, a, st);
}

int ssp_tangent_plastic_correction(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                                   const double *ds, const double *weight, const int8_t *branch, const double *shear,
                                   const double *lame, const int32_t *scatter_map, int n_elem, int n_p, int n_q,
                                   long long nnz_out, double scale, double *out_values, const int32_t *elem_list,
                                   const int32_t *elem_count, void *stream) {
    if ((dim != 2 && dim != 3) || n_elem < 0 || n_p <= 0 || n_q <= 0 || nnz_out < 0) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || (dim == 3 && !dphi3) || !ds || !weight || !branch || !shear || !lame || !scatter_map ||
        (nnz_out > 0 && !out_values))
        return SSP_ERR_INVALID;
    if ((elem_list == nullptr) != (elem_count == nullptr)) return SSP_ERR_INVALID;
    ElemArgs a{dphi1, dphi2, dphi3, ds, weight, scatter_map, n_elem, nnz_out, out_values, branch, shear, lame, scale,
               elem_list, elem_count};
    return dispatch_element<true, true>(dim, n_p, n_q, a, as_stream(stream));
}

int ssp_tangent_plastic_correction_mixed(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                                         const double *ds, const double *weight, const int8_t *branch,
                                         const double *shear, const double *lame, const int32_t *scatter_map,
                                         int n_elem, int n_p, int n_q, long long nnz_out, double scale,
                                         double *out_values, const int32_t *elem_list, const int32_t *elem_count,
                                         void *stream) {
    if ((dim != 2 && dim != 3) || n_elem < 0 || n_p <= 0 || n_q <= 0 || nnz_out < 0) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!dphi1 || !dphi2 || (dim == 3 && !dphi3) || !ds || !weight || !branch || !shear || !lame || !scatter_map ||
        (nnz_out > 0 && !out_values))
        return SSP_ERR_INVALID;
    if ((elem_list == nullptr) != (elem_count == nullptr)) return SSP_ERR_INVALID;
    ElemArgs a{dphi1, dphi2, dphi3, ds, weight, scatter_map, n_elem, nnz_out, out_values, branch, shear, lame, scale,
               elem_list, elem_count};
    cudaStream_t st = as_stream(stream);
    if (dim == 3 && n_p == 10 && n_q == 11) return launch_element_warp<3, 10, 11, true, true, true>(a, st);
    if (dim == 3 && n_p == 4 && n_q == 1) return launch_element_warp<3, 4, 1, true, true, true>(a, st);
    if (dim == 2 && n_p == 6 && n_q == 7) return launch_element_warp<2, 6, 7, true, true, true>(a, st);
    if (dim == 2 && n_p == 3 && n_q == 1) return launch_element_warp<2, 3, 1, true, true, true>(a, st);
    if (dim == 2 && n_p == 15 && n_q == 12) return launch_element_warp<2, 15, 12, true, true, true>(a, st);
    if (dim == 3 && n_p == 35 && n_q == 24)
        return correction_tc_p4(dphi1, dphi2, dphi3, ds, weight, branch, shear, lame, scatter_map, n_elem, nnz_out, scale,
                                out_values, elem_list, elem_count, st);
    return SSP_ERR_UNSUPPORTED;
}

int ssp_plastic_elements(const int8_t *branch, int n_elem, int n_q, int32_t *list_out, int32_t *count_out,
                         void *stream) {
    if (n_elem < 0 || n_q <= 0 || !count_out) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(count_out, 0, sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!branch || !list_out) return SSP_ERR_INVALID;
    plastic_elements_kernel<<<grid_for(n_elem, 256), 256, 0, st>>>(branch, n_elem, n_q, list_out, count_out);
    return launch_status();
}

int ssp_plastic_elements_split(const int8_t *branch, int n_elem, int n_q, int min_points, int32_t *list_few,
                               int32_t *count_few, int32_t *list_many, int32_t *count_many, void *stream) {
    if (n_elem < 0 || n_q <= 0 || min_points < 1) return SSP_ERR_INVALID;
    if (!count_few || !count_many) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(count_few, 0, sizeof(int32_t), st) != cudaSuccess ||
        cudaMemsetAsync(count_many, 0, sizeof(int32_t), st) != cudaSuccess)
        return SSP_ERR_CUDA;
    if (n_elem == 0) return SSP_OK;
    if (!branch || !list_few || !list_many) return SSP_ERR_INVALID;
    plastic_elements_split_kernel<<<grid_for(n_elem, 256), 256, 0, st>>>(branch, n_elem, n_q, min_points, list_few,
                                                                         count_few, list_many, count_many);
    return launch_status();
}

int ssp_tangent_plastic_correction_p2_moments(const double *jinv, const double *bary, const double *ds,
                                              const double *weight, const int8_t *branch, const double *shear,
                                              const double *lame, const int32_t *scatter_map, int n_elem, int n_q,
                                              long long nnz_out, double scale, double *out_values,
                                              const int32_t *elem_list, const int32_t *elem_count, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_q > kMaxQ || nnz_out < 0) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !bary || !ds || !weight || !branch || !shear || !lame || !scatter_map || !elem_list || !elem_count ||
        (nnz_out > 0 && !out_values))
        return SSP_ERR_INVALID;
    return launch_p2_moments(correction_p2_moment_kernel, kMomWarps, sizeof(MomentTables) + sizeof(MomentWarp) * kMomWarps,
                             jinv, bary, ds, weight, branch, shear, lame, scatter_map, n_elem, n_q, nnz_out, scale,
                             out_values, elem_list, elem_count, as_stream(stream));
}

int ssp_tangent_plastic_correction_p2_moments_mixed(const double *jinv, const double *bary, const double *ds,
                                                    const double *weight, const int8_t *branch, const double *shear,
                                                    const double *lame, const int32_t *scatter_map, int n_elem, int n_q,
                                                    long long nnz_out, double scale, double *out_values,
                                                    const int32_t *elem_list, const int32_t *elem_count, void *stream) {
    if (n_elem < 0 || n_q <= 0 || n_q > kMaxQ || nnz_out < 0) return SSP_ERR_INVALID;
    if (n_elem == 0) return SSP_OK;
    if (!jinv || !bary || !ds || !weight || !branch || !shear || !lame || !scatter_map || !elem_list || !elem_count ||
        (nnz_out > 0 && !out_values))
        return SSP_ERR_INVALID;
    return launch_p2_moments(correction_p2_moment_f32_kernel, kF32Warps,
                             sizeof(MomentF32Tables) + sizeof(MomentF32Warp) * kF32Warps, jinv, bary, ds, weight,
                             branch, shear, lame, scatter_map, n_elem, n_q, nnz_out, scale, out_values, elem_list,
                             elem_count, as_stream(stream));
}

int ssp_fill_elastic_ds(int dim, const int8_t *branch, const double *shear, const double *lame, int n_int,
                        double *ds_inout, void *stream) {
    if (n_int < 0 || (dim != 2 && dim != 3)) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!branch || !shear || !lame || !ds_inout) return SSP_ERR_INVALID;
    const long long n = (long long)n_int * (dim == 3 ? 36 : 9);
    if (dim == 3)
        fill_elastic_ds_kernel<3><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(branch, shear, lame, n_int, ds_inout);
    else
        fill_elastic_ds_kernel<2><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(branch, shear, lame, n_int, ds_inout);
    return launch_status();
}

int ssp_elastic_tangent_blocks(int dim, const double *shear, const double *lame, int n_int, double *ds_out,
                               void *stream) {
    if ((dim != 2 && dim != 3) || n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!shear || !lame || !ds_out) return SSP_ERR_INVALID;
    const long long n = (long long)n_int * (dim == 3 ? 36 : 9);
    if (dim == 3)
        elastic_blocks_kernel<3><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(shear, lame, n_int, ds_out);
    else
        elastic_blocks_kernel<2><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(shear, lame, n_int, ds_out);
    return launch_status();
}

int ssp_blend_values(double *out_values, const double *base, const double *elastic_values, double r, long long nnz,
                     void *stream) {
    if (nnz < 0) return SSP_ERR_INVALID;
    if (nnz == 0) return SSP_OK;
    if (!out_values || !base || !elastic_values) return SSP_ERR_INVALID;
    blend_base_kernel<<<grid_for(nnz, 256), 256, 0, as_stream(stream)>>>(out_values, base, elastic_values, nnz, r);
    return launch_status();
}

int ssp_assemble_tangent_values_3d_p2(const double *dphi1, const double *dphi2, const double *dphi3, const double *ds,
                                      const double *weight, const int32_t *scatter_map, int n_int, int n_elem, int n_p,
                                      int n_q, int nnz_out, double *out_values, void *stream) {
    if (n_elem < 0 || n_q <= 0 || (long long)n_elem * n_q != n_int) return SSP_ERR_INVALID;
    return ssp_tangent_element(3, 0, dphi1, dphi2, dphi3, ds, weight, scatter_map, n_elem, n_p, n_q, nnz_out, out_values, 0,
                               stream);
}

int ssp_finish_values(double *values, long long nnz, const int32_t *constrained_diag_positions, int n_diag,
                      const double *elastic_values, double r, void *stream) {
    if (nnz < 0 || n_diag < 0) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (n_diag > 0) {
        if (!values || !constrained_diag_positions) return SSP_ERR_INVALID;
        set_positions_kernel<<<grid_for(n_diag, 128), 128, 0, st>>>(values, constrained_diag_positions, n_diag, nnz, 1.0);
    }
    if (elastic_values && nnz > 0) {
        if (!values) return SSP_ERR_INVALID;
        blend_kernel<<<grid_for(nnz, 256), 256, 0, st>>>(values, elastic_values, nnz, r);
    }
    return launch_status();
}

int ssp_gather(const double *src, const int32_t *idx, int n, double *dst, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!src || !idx || !dst) return SSP_ERR_INVALID;
    gather_rows_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(src, idx, n, dst);
    return launch_status();
}

}  // extern "C"

// The device address of pinned, device-mapped host memory (nullptr if the pointer is not such memory).
static void *mapped_device_pointer(const void *host_ptr) {
    if (!host_ptr) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, host_ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

extern "C" {

int ssp_host_writable(const void *host_ptr) { return mapped_device_pointer(host_ptr) != nullptr ? 1 : 0; }

int ssp_mark_element_rows(const int32_t *elem_row, int n_elem, int n_ld, const int32_t *elem_list,
                          const int32_t *elem_count, int n_rows, uint8_t *row_mark, void *stream) {
    if (n_elem < 0 || n_ld <= 0 || n_rows < 0) return SSP_ERR_INVALID;
    if (n_elem == 0 || n_rows == 0) return SSP_OK;
    if (!elem_row || !elem_list || !elem_count || !row_mark) return SSP_ERR_INVALID;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    mark_rows_kernel<<<static_cast<unsigned>(sms * 4), 256, 0, as_stream(stream)>>>(elem_row, n_elem, n_ld, elem_list,
                                                                                   elem_count, n_rows, row_mark);
    return launch_status();
}

int ssp_copy_rows_out_share(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows,
                            long long nnz, double *dst_host, int blocks_per_sm, void *stream) {
    if (n_rows < 0 || nnz < 0 || blocks_per_sm < 1 || blocks_per_sm > 8) return SSP_ERR_INVALID;
    if (n_rows == 0 || nnz == 0) return SSP_OK;
    double *dst = static_cast<double *>(mapped_device_pointer(dst_host));
    if (!src || !indptr || !row_mark || !dst) return SSP_ERR_INVALID;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0 ? 1 : 0;
    copy_rows_out_kernel<<<static_cast<unsigned>(sms * blocks_per_sm), 256, 0, as_stream(stream)>>>(
        src, indptr, row_mark, n_rows, nnz, dst, vec);
    return launch_status();
}

// four 256-thread blocks per SM keep the host link busy and leave half of each SM's threads to the
// kernels that run beside the copy (the internal force of the same Newton iteration); C5 end to end
// measured 19.0 ms with four, 19.3-19.5 ms with two, 19.2 ms with six, 21.0 ms with eight
int ssp_copy_rows_out(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows, long long nnz,
                      double *dst_host, void *stream) {
    return ssp_copy_rows_out_share(src, indptr, row_mark, n_rows, nnz, dst_host, 4, stream);
}

namespace {
int copy_rows_device(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows, long long nnz,
                     double *dst, int blocks_per_sm, void *stream) {
    if (n_rows < 0 || nnz < 0) return SSP_ERR_INVALID;
    if (n_rows == 0 || nnz == 0) return SSP_OK;
    if (!src || !indptr || !row_mark || !dst) return SSP_ERR_INVALID;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0 ? 1 : 0;
    copy_rows_out_kernel<<<static_cast<unsigned>(sms * blocks_per_sm), 256, 0, as_stream(stream)>>>(
        src, indptr, row_mark, n_rows, nnz, dst, vec);
    return launch_status();
}
}  // namespace

int ssp_copy_rows_device(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows, long long nnz,
                         double *dst, void *stream) {
    return copy_rows_device(src, indptr, row_mark, n_rows, nnz, dst, 8, stream);
}

// A grid of blocks_per_sm 256-thread blocks per SM (1..8): on a second stream beside long kernels a
// small share of each SM's threads and registers leaves the rest to them (a grid that fills every
// SM would run before them instead of beside them).
int ssp_copy_rows_device_share(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows,
                               long long nnz, double *dst, int blocks_per_sm, void *stream) {
    if (blocks_per_sm < 1 || blocks_per_sm > 8) return SSP_ERR_INVALID;
    return copy_rows_device(src, indptr, row_mark, n_rows, nnz, dst, blocks_per_sm, stream);
}

int ssp_copy_device(const double *src, long long n, double *dst, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!src || !dst) return SSP_ERR_INVALID;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
    copy_out_kernel<<<static_cast<unsigned>(sms * 8), 256, 0, as_stream(stream)>>>(src, n, dst, vec ? 1 : 0);
    return launch_status();
}

int ssp_copy_out(const double *src, long long n, double *dst_host, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    double *dst = static_cast<double *>(mapped_device_pointer(dst_host));
    if (!src || !dst) return SSP_ERR_INVALID;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0;
    copy_out_kernel<<<static_cast<unsigned>(sms * 8), 256, 0, as_stream(stream)>>>(src, n, dst, vec ? 1 : 0);
    return launch_status();
}

}  // extern "C"
