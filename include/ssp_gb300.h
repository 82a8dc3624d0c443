/*
 * ssp_gb300.h -- C ABI of the GB300 (sm_103a) Newton hot path of the slope-stability solver.
 *
 * Conventions shared by every entry point:
 *   - plain pointers and sizes only; no framework types cross this boundary;
 *   - array arguments are DEVICE pointers (caller-allocated, e.g. cudaMalloc or a torch
 *     CUDA tensor) unless the comment says "host";
 *   - layouts are the reference's C layouts: per-point AoS strains/stresses [n_int][6]
 *     (2D: [n_int][3] in, [n_int][4] out), tangents [n_int][36] (2D [n_int][9]) column-major
 *     per point (entry (i,j) at i + n_strain*j), dphi arrays [n_int][n_p], points
 *     element-major (g = e*n_q + q);
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream); all work is
 *     enqueued asynchronously on it;
 *   - the return value is an ssp_status; the reference's C functions return void and its
 *     Cython wrappers raise ValueError on bad shapes -- here a bad argument returns
 *     SSP_ERR_INVALID before anything is launched;
 *   - kernels that meet an out-of-range index skip the access and set a bit in a device
 *     status word instead of faulting; ssp_device_status() reads it.
 *
 * Reference paths below are relative to the reference project root
 * (Beremi/slope_stability_petsc4py).
 */
#ifndef SSP_GB300_H
#define SSP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum ssp_status {
    SSP_OK = 0,
    SSP_ERR_INVALID = 1,     /* bad argument (shape, size, null pointer) */
    SSP_ERR_CUDA = 2,        /* a CUDA call or launch failed */
    SSP_ERR_UNSUPPORTED = 3, /* element type / quadrature combination without a kernel */
    SSP_ERR_OVERFLOW = 4,    /* an index does not fit int32 (distributed_tangent.py:122-124) */
    SSP_ERR_PATTERN = 5,     /* structural entry missing from the pattern (distributed_tangent.py:431-432) */
    SSP_ERR_TOO_LARGE = 6    /* more points than the fixed scratch of the no-allocation entry point holds */
};

/* bits of the device status word */
#define SSP_DEV_BAD_INDEX 1
#define SSP_DEV_NONFINITE 2
#define SSP_DEV_TIMEOUT 4 /* a bounded wait on the tensor cores expired; the kernel stopped */

/* ------------------------------------------------------------------ constitutive */

/* Replaces constitutive_problem_3d_s_batch_c (src/slope_stability/cython/constitutive_3d_batch.h:4-13).
 * S only (line search / residual-only Newton steps).  `bulk` is unused, as in the reference. */
int ssp_constitutive_3d_s(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                          const double *bulk, const double *lame, int n_int, double *S_out, void *stream);

/* Replaces constitutive_problem_3d_sds_batch_c (src/slope_stability/cython/constitutive_3d_batch.h:15-25).
 * S and the consistent tangent DS; DS is symmetric (associated flow, sin(psi) = sin(phi)). */
int ssp_constitutive_3d_sds(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                            const double *bulk, const double *lame, int n_int, double *S_out, double *DS_out,
                            void *stream);

/* S plus the return branch of every point (0 elastic, 1 smooth face, 2 left edge, 3 right edge,
 * 4 apex); the branch decision of constitutive_3D_kernel.h:116-350.  Used to label training data
 * of the learned branch proposal. */
int ssp_constitutive_3d_branch(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                               const double *lame, int n_int, double *S_out, int8_t *branch_out, void *stream);

/* Binned plane-strain return mapping: the same branch codes as ssp_constitutive_sds_branch(2, ...)
 * and S, DS within a few ulps of it, with the elastic points finished in a first pass
 * and the plastic branches run only on the listed points.  scratch: 1 + n_int int32 (caller
 * allocated; a count then the listed points).  Replaces the reference's NumPy
 * constitutive_problem_2D (src/slope_stability/constitutive/problem.py:143-475) in the operator. */
int ssp_constitutive_2d_sds_binned(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                                   const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                                   int32_t *scratch, void *stream);

/* S, DS and the branch code of every point (2D or 3D); the branch codes drive the plastic-only
 * tangent correction (ssp_tangent_plastic_correction).  Same arithmetic as ssp_constitutive_3d_sds /
 * ssp_constitutive_2d. */
int ssp_constitutive_sds_branch(int dim, const double *E, const double *c_bar, const double *sin_phi,
                                const double *shear, const double *lame, int n_int, double *S_out, double *DS_out,
                                int8_t *branch_out, void *stream);

/* The 3D return mapping in three passes over the same arithmetic (replaces
 * constitutive_problem_3d_sds_batch_c, constitutive_3d_batch.h:15-25): pass A bounds every point's
 * trial yield function from its invariants (FP32, with a margin that covers FP32 and eigenvalue
 * rounding) and finishes the points it proves elastic with the elastic branch's FP64 arithmetic;
 * pass B runs the FP64 eigen-decomposition and branch decision on the other points (a dense list)
 * and finishes elastic and apex ones; pass C finishes the smooth-face, left-edge and right-edge
 * points one branch per warp from the decision record pass B leaves in their DS rows.  Results
 * equal ssp_constitutive_sds_branch's (same branch codes; the same FP64 operations).  scratch is
 * caller-allocated device memory of 3*n_int + 4 int32 (counters and point lists); it is
 * overwritten.  Outputs as ssp_constitutive_sds_branch. */
int ssp_constitutive_3d_sds_binned(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                                   const double *lame, int n_int, double *S_out, double *DS_out, int8_t *branch_out,
                                   int32_t *scratch, void *stream);

/* No counterpart in the reference.  ssp_constitutive_3d_sds_binned for the mixed-precision form:
 * the same branches, multipliers and S (FP64, bitwise the same), the plastic points' DS in
 * double-float arithmetic on the FP32 pipe (per-point FP64 coefficients, compensated sums of
 * products per entry, about 2^-46 of the terms' magnitude).  A point whose smallest eigenvalue gap is
 * below 1e-3 of max|e|, or whose coefficients leave the float range, gets the FP64 DS. */
int ssp_constitutive_3d_sds_binned_mixed(const double *E, const double *c_bar, const double *sin_phi,
                                         const double *shear, const double *lame, int n_int, double *S_out,
                                         double *DS_out, int8_t *branch_out, int32_t *scratch, void *stream);

/* No counterpart in the reference.  ssp_constitutive_3d_sds_binned for callers that cannot
 * allocate device memory, e.g. a constitutive hook called from inside another solver's assembly
 * loop: it is handed device pointers to its inputs and outputs only, the host framework owns and
 * budgets all device memory, and a cudaMalloc there would also synchronise the device mid-loop.
 * The caller passes inputs and outputs as for ssp_constitutive_3d_sds_binned, but no scratch:
 * the point lists live in a fixed array inside this library (static device memory of
 * 4 + 3*SSP_NOALLOC_MAX_POINTS int32, about 24 MiB, which every GPU that loads the library holds
 * until the process exits).  Nothing is allocated: no cudaMalloc, cudaFree or allocating library
 * call.
 *   - n_int above SSP_NOALLOC_MAX_POINTS returns SSP_ERR_TOO_LARGE before any work.
 *   - The first call on each device looks up the array's device address (cudaGetSymbolAddress,
 *     with that device current) and caches it for the life of the process; make that first call
 *     before any stream capture.  A reset of the device's context (cudaDeviceReset, or a release
 *     of its primary context) invalidates the cached address: do not call this entry point on a
 *     device after resetting it.
 *   - Every call on a device shares the one array and leaves the last call's lists in it; the
 *     counters are cleared at the start of each call.  Calls that overlap on the GPU (different
 *     streams, or host threads sharing a device) race on the array: serialise them. */
#define SSP_NOALLOC_MAX_POINTS 2097152
int ssp_constitutive_3d_sds_binned_noalloc(const double *E, const double *c_bar, const double *sin_phi,
                                           const double *shear, const double *lame, int n_int, double *S_out,
                                           double *DS_out, int8_t *branch_out, void *stream);

/* Replaces constitutive_problem_2D (src/slope_stability/constitutive/problem.py:143-475), which the
 * reference has only in NumPy: E [n_int][3] -> S [n_int][4] ([s11,s22,s12,s33]), DS [n_int][9]
 * (DS_out may be NULL for stress only). */
int ssp_constitutive_2d(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                        const double *bulk, const double *lame, int n_int, double *S_out, double *DS_out, void *stream);

/* Replaces potential_3D / potential_2D (src/slope_stability/constitutive/problem.py:1111-1190,
 * 1029-1108) and the weighted sum of ConstitutiveOperator.potential_energy (problem.py:2148-2157):
 *   psi_out[p]   = the Mohr-Coulomb potential energy density at point p (NULL: not written);
 *   branch_out[p] = its branch, 0 elastic, 1 smooth, 2 left edge, 3 right edge, 4 apex (NULL: not written);
 *   *total_out   = sum_p weight[p] * psi[p], one double on the device (NULL: not computed; weight
 *                  and partial are then unused and may be NULL).
 * E is [n_int][6] (3D) or [n_int][3] (2D); bulk enters the apex branch.  partial is caller scratch
 * of SSP_POTENTIAL_PARTIALS doubles; the sum is deterministic (fixed grid, fixed trees) for a
 * given n_int.  Two launches when total_out is given, one otherwise. */
#define SSP_POTENTIAL_PARTIALS 1024
int ssp_potential_energy(int dim, const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                         const double *bulk, const double *lame, const double *weight, int n_int, double *psi_out,
                         int8_t *branch_out, double *partial, double *total_out, void *stream);

/* Replaces reduction(c0, phi, psi, lam, Davis_type) (src/slope_stability/constitutive/reduction.py:14-78).
 * davis_type is 'A', 'B' or 'C'; lam must be > 0. */
int ssp_reduction(const double *c0, const double *phi, const double *psi, int n_int, double lam, char davis_type,
                  double *c_bar_out, double *sin_phi_out, void *stream);

/* ------------------------------------------------------------------ geometry */

/* Replaces the dphi/weight part of _assemble_3d / _assemble_2d (src/slope_stability/fem/assembly.py:139-245,
 * 50-136).  coord [dim][n_nodes], elem [n_p][n_elem] (int64), dhat [dim][n_p][n_q] reference
 * gradients, wf [n_q]; outputs dphi* [n_elem*n_q][n_p], weight [n_elem*n_q] (dphi3 unused in 2D). */
int ssp_geometry(int dim, const double *coord, const int64_t *elem, const double *dhat, const double *wf, int n_nodes,
                 int n_elem, int n_p, int n_q, double *dphi1, double *dphi2, double *dphi3, double *weight,
                 void *stream);

/* ------------------------------------------------------------------ strain / force */

/* Replaces assemble_overlap_strain_3d_c (src/slope_stability/cython/assemble_tangent_values_3d.h:40-51).
 * Adds n_u, the length of u_overlap, for bounds checking. */
int ssp_assemble_overlap_strain_3d(const double *dphi1, const double *dphi2, const double *dphi3,
                                   const double *u_overlap, int n_u, const int32_t *elem_dof_lids, int n_int,
                                   int n_elem, int n_p, int n_q, double *out_values, void *stream);

/* 2D counterpart of the strain kernel; replaces overlap_B @ u_overlap
 * (src/slope_stability/fem/distributed_tangent.py:906-907) for plane strain. */
int ssp_assemble_overlap_strain_2d(const double *dphi1, const double *dphi2, const double *u_overlap, int n_u,
                                   const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                   double *out_values, void *stream);

/* hi + lo float pairs of FP64 values: out_pairs[2 i], out_pairs[2 i + 1] = split of
 * x[i] * (scale ? scale[i / group] : 1) (the product in FP64; hi = the value truncated to 24 bits,
 * lo = the rest rounded to a float).  The inputs of the compensated kernels below. */
int ssp_split_f64(const double *x, const double *scale, long long n, int group, float *out_pairs, void *stream);

/* Mixed-precision form of ssp_assemble_overlap_strain_3d and ssp_assemble_force_element (3D): the
 * same sums in compensated double-float arithmetic on the FP32 pipe (product rounding errors
 * recovered with FMAs, sums kept as hi + lo pairs), widened to FP64 once per output.  Inputs are
 * hi + lo pairs from ssp_split_f64: the gradients (strain), w * gradient (force; scale = weight,
 * group = n_p) and the overlap displacements; the force kernel splits the FP64 stresses itself.  The strain is formed from displacement
 * differences to the element's first node (sum of the basis gradients = 0), so no digits cancel.
 * Relative error against the FP64 kernels ~1e-13; the force is still accumulated into out_values
 * with FP64 reductions.  No reference counterpart. */
int ssp_assemble_overlap_strain_3d_mixed(const float *dphi1_hl, const float *dphi2_hl, const float *dphi3_hl,
                                         const float *u_hl, int n_u, const int32_t *elem_dof_lids, int n_int,
                                         int n_elem, int n_p, int n_q, double *out_values, void *stream);
int ssp_assemble_force_element_mixed(const float *wdphi1_hl, const float *wdphi2_hl, const float *wdphi3_hl,
                                     const double *stress, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                     int n_rows, double *out_values, void *stream);

/* The same strain and force for affine (straight-sided) tetrahedra, whose gradients are
 * J^{-T} ghat(q): jinv_hl [n_elem][3][3] hi + lo pairs of each element's J^{-1} (row-major),
 * ghat_hl [n_q][n_p][3] hi + lo pairs of the reference-element gradient table, w_hl [n_int] of the
 * point weights.  Reads 9 pairs per element instead of 3 n_p pairs per point; the caller checks
 * that its elements are affine.  No reference counterpart. */
int ssp_assemble_overlap_strain_3d_affine_mixed(const float *jinv_hl, const float *ghat_hl, const float *u_hl, int n_u,
                                                const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                                double *out_values, void *stream);
int ssp_assemble_force_element_affine_mixed(const float *jinv_hl, const float *ghat_hl, const float *w_hl,
                                            const double *stress, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                            int n_rows, double *out_values, void *stream);

/* Straight-sided P1 / P4 tetrahedra in FP64 (no reference counterpart; same results as
 * ssp_assemble_overlap_strain_3d / ssp_assemble_force_element within rounding): the gradients are
 * J^{-T} ghat(q), so the kernels read J^{-1} per element (jinv [n_elem][3][3] row-major) and the
 * reference element's gradient table (ghat [n_q][n_p][3]) instead of per-point gradients.  The
 * force entry zeroes out_values first; elem_row as in ssp_assemble_force_element.  Tables of more
 * than 48 KiB of shared memory return SSP_ERR_UNSUPPORTED. */
int ssp_assemble_overlap_strain_3d_affine(const double *jinv, const double *ghat, const double *u_overlap, int n_u,
                                          const int32_t *elem_dof_lids, int n_int, int n_elem, int n_p, int n_q,
                                          double *out_values, void *stream);
int ssp_assemble_force_element_affine(const double *jinv, const double *ghat, const double *stress,
                                      const double *weight, const int32_t *elem_row, int n_elem, int n_p, int n_q,
                                      int n_rows, double *out_values, void *stream);

/* Straight-sided P2 tetrahedra (no reference counterpart; same results as
 * ssp_assemble_overlap_strain_3d / ssp_assemble_force_element within rounding): the strain and
 * the owned force through the barycentric form of the quadratic basis, from J^{-1} per element
 * (jinv [n_elem][3][3], row k = the gradient of barycentric coordinate k+1) and the quadrature
 * points' barycentric coordinates (bary [n_q][4]) instead of per-point gradients.  Local node order
 * of the reference's P2 tetrahedron: vertices 0-3, edges 01, 12, 02, 13, 23, 03.  The force
 * entry zeroes out_values first; elem_row as in ssp_assemble_force_element. */
int ssp_assemble_overlap_strain_3d_p2_affine(const double *jinv, const double *bary, const double *u_overlap, int n_u,
                                             const int32_t *elem_dof_lids, int n_int, int n_elem, int n_q,
                                             double *out_values, void *stream);
int ssp_assemble_force_element_p2_affine(const double *jinv, const double *bary, const double *stress,
                                         const double *weight, const int32_t *elem_row, int n_elem, int n_q,
                                         int n_rows, double *out_values, void *stream);
/* The same two in the mixed form's double-float arithmetic (hi + lo float pairs of J^{-1}, of the
 * barycentric coordinates, of the displacements and of the weights, as the _affine_mixed entries
 * take them); FP64 outputs, about 1e-13 relative. */
int ssp_assemble_overlap_strain_3d_p2_affine_mixed(const float *jinv_hl, const float *bary_hl, const float *u_hl,
                                                   int n_u, const int32_t *elem_dof_lids, int n_int, int n_elem, int n_q,
                                                   double *out_values, void *stream);
int ssp_assemble_force_element_p2_affine_mixed(const float *jinv_hl, const float *bary_hl, const float *w_hl,
                                               const double *stress, const int32_t *elem_row, int n_elem, int n_q,
                                               int n_rows, double *out_values, void *stream);

/* Replaces assemble_force_3d_rows_c (src/slope_stability/cython/assemble_tangent_values_3d.h:53-68).
 * Deterministic row gather; rows without slots come out 0. */
int ssp_assemble_force_3d_rows(const double *dphi1, const double *dphi2, const double *dphi3, const double *stress,
                               const double *weight, const int32_t *row_slot_ptr, const int32_t *slot_elem,
                               const uint8_t *slot_lrow, int n_int, int n_rows, int n_slots, int n_p, int n_q,
                               double *out_values, void *stream);

/* Owned internal force by element scatter, 2D or 3D: the same F = B^T (w S) restricted to owned
 * free rows (distributed_tangent.py:845-883, 910-934).  elem_row [n_elem][dim*n_p] gives the owned
 * free row of each local dof or -1.  out_values [n_rows] is zeroed first. */
int ssp_assemble_force_element(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                               const double *stress, const double *weight, const int32_t *elem_row, int n_elem,
                               int n_p, int n_q, int n_rows, double *out_values, void *stream);

/* ------------------------------------------------------------------ tangent CSR values */

/* Replaces assemble_tangent_values_3d_rows_c (src/slope_stability/cython/assemble_tangent_values_3d.h:21-38).
 * out_values [nnz_out] is zeroed first; constrained diagonals are left at 0 as in the reference
 * kernel (the caller sets them, see ssp_finish_values). */
int ssp_assemble_tangent_values_3d_rows(const double *dphi1, const double *dphi2, const double *dphi3, const double *ds,
                                        const double *weight, const int32_t *row_slot_ptr, const int32_t *slot_elem,
                                        const uint8_t *slot_lrow, const int32_t *slot_pos, int n_int, int n_rows,
                                        int n_slots, int n_p, int n_q, int nnz_out, double *out_values, void *stream);

/* Replaces assemble_tangent_values_3d_p2_c (src/slope_stability/cython/assemble_tangent_values_3d.h:6-19):
 * element-dense K_e through scatter_map [n_elem][(3 n_p)^2] (-1 = skipped). */
int ssp_assemble_tangent_values_3d_p2(const double *dphi1, const double *dphi2, const double *dphi3, const double *ds,
                                      const double *weight, const int32_t *scatter_map, int n_int, int n_elem, int n_p,
                                      int n_q, int nnz_out, double *out_values, void *stream);

/* The element kernel behind ssp_assemble_tangent_values_3d_p2, for 2D and 3D, with a symmetric
 * variant (symmetric != 0: evaluates alpha <= beta only; valid when every DS block is symmetric,
 * which holds for tangents from ssp_constitutive_*).  accumulate == 0 zeroes out_values first.
 * 2D also replaces the Python loop of distributed_tangent.py:1437-1484. */
int ssp_tangent_element(int dim, int symmetric, const double *dphi1, const double *dphi2, const double *dphi3,
                        const double *ds, const double *weight, const int32_t *scatter_map, int n_elem, int n_p, int n_q,
                        long long nnz_out, double *out_values, int accumulate, void *stream);

/* Tangent by elastic predictor and plastic correction: adds
 *     sum over points with branch != 0 of  B^T (w * scale * (DS - D_el)) B
 * to out_values (no zeroing), where D_el is the elastic tangent the return mapping emits for
 * (shear, lame).  Added to the elastic tangent of the same mesh (assembled once from
 * ssp_elastic_tangent_blocks), this equals the element sum of the reference's tangent kernels
 * (assemble_tangent_values_3d.c:13-214) up to rounding, with FP64 work only for plastic points. */
int ssp_tangent_plastic_correction(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                                   const double *ds, const double *weight, const int8_t *branch, const double *shear,
                                   const double *lame, const int32_t *scatter_map, int n_elem, int n_p, int n_q,
                                   long long nnz_out, double scale, double *out_values, const int32_t *elem_list,
                                   const int32_t *elem_count, void *stream);

/* The elements with at least one point whose branch is not elastic: list_out[0 .. *count_out)
 * (device memory; count_out is zeroed first; the order is unspecified).  Passed as elem_list /
 * elem_count to the plastic-correction entry points, which then visit only those elements (both
 * NULL: every element). */
int ssp_plastic_elements(const int8_t *branch, int n_elem, int n_q, int32_t *list_out, int32_t *count_out,
                         void *stream);

/* No reference counterpart.  The plastic elements (elements with a point whose branch is not 0)
 * split by their number of plastic points: fewer than min_points into list_few, at least
 * min_points into list_many (each n_elem long; the counts are zeroed first). */
int ssp_plastic_elements_split(const int8_t *branch, int n_elem, int n_q, int min_points, int32_t *list_few,
                               int32_t *count_few, int32_t *list_many, int32_t *count_many, void *stream);

/* No reference counterpart; the same result as ssp_tangent_plastic_correction (3D P2) to rounding.
 * The plastic correction of straight-sided P2 tetrahedra in moment form: with the gradients linear
 * in the barycentric coordinates, an element's correction is assembled from the ten moments
 * sum_q lambda_qm lambda_qn w_q s (DS_q - D_el,q) of its plastic points (jinv [n_elem][3][3], row k
 * the gradient of barycentric coordinate k+1; bary [n_q][4] the points' barycentric coordinates),
 * about 7,500 + 261 n_pl FP64 operations per element instead of about 1,935 per plastic point
 * (fewer from five plastic points up).
 * Visits the elements of elem_list[0 .. *elem_count) (e.g. list_many of ssp_plastic_elements_split);
 * n_q <= 11. */
int ssp_tangent_plastic_correction_p2_moments(const double *jinv, const double *bary, const double *ds,
                                              const double *weight, const int8_t *branch, const double *shear,
                                              const double *lame, const int32_t *scatter_map, int n_elem, int n_q,
                                              long long nnz_out, double scale, double *out_values,
                                              const int32_t *elem_list, const int32_t *elem_count, void *stream);

/* Mixed-precision form of ssp_tangent_plastic_correction_p2_moments: DS - D_el and w * scale are
 * formed in FP64 and rounded to FP32 by bit operations; the moments, beta^T M beta and the element
 * matrix in FP32 (about 2e-7 of the correction's scale); the element sums widened exactly and added
 * to the FP64 CSR values with FP64 reductions.  Cheaper than ssp_tangent_plastic_correction_mixed
 * from one plastic point up. */
int ssp_tangent_plastic_correction_p2_moments_mixed(const double *jinv, const double *bary, const double *ds,
                                                    const double *weight, const int8_t *branch, const double *shear,
                                                    const double *lame, const int32_t *scatter_map, int n_elem, int n_q,
                                                    long long nnz_out, double scale, double *out_values,
                                                    const int32_t *elem_list, const int32_t *elem_count, void *stream);

/* Mixed-precision form of ssp_tangent_plastic_correction.  H = B^T (w * scale * (DS - D_el)) is
 * formed in FP64 and split into hi + lo parts.  P1/P2 elements: the products B^T H are taken and
 * accumulated in FP32 on the CUDA cores.  P4 elements (3D, 35 nodes, 24 points): the element's
 * contraction over (point, strain component) runs on the tensor cores (tcgen05.mma kind::tf32,
 * H and B both split into TF32 hi + lo, hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor
 * memory).  The element sums are added to the FP64 CSR values with FP64 atomics.  The return mapping that produced DS (eigendecomposition, branch tests, plastic
 * multipliers) is FP64.  Relative error of the assembled tangent against the FP64 form is about
 * 1e-7 (tested <= 1e-6).  No reference counterpart: the reference assembles in FP64 only. */
int ssp_tangent_plastic_correction_mixed(int dim, const double *dphi1, const double *dphi2, const double *dphi3,
                                         const double *ds, const double *weight, const int8_t *branch,
                                         const double *shear, const double *lame, const int32_t *scatter_map,
                                         int n_elem, int n_p, int n_q, long long nnz_out, double scale,
                                         double *out_values, const int32_t *elem_list,
                                         const int32_t *elem_count, void *stream);

/* Per-point elastic tangent blocks [n_int][n_s*n_s] of the return mapping's elastic branch. */
/* Test support for the tensor-core tangent: D[128][112] = A[128][K] * B[112][K]^T (row-major FP32,
 * inputs rounded to TF32) through the shared-memory layout, descriptors and tensor-memory read-back
 * of the P4 kernel, one CTA; K in {8, 16, 24}; convention 1 swaps the descriptor's leading and
 * stride byte offsets (0 is the kernel's).  No reference counterpart. */
int ssp_tc_tf32_probe(const float *A, const float *B, int K, int convention, float *D, void *stream);

/* Test support for the bounded waits of the tensor-core kernels (no reference counterpart): one
 * CTA takes tensor memory, waits on an mbarrier that nothing arrives on for at most limit_clocks SM
 * clocks (1 .. 2e9), then frees the tensor memory and returns.  On expiry it sets SSP_DEV_TIMEOUT
 * in the device status word and writes 1 to *expired (a device int), else 0.  No tensor-core
 * operation is issued, so nothing is left in flight. */
int ssp_tc_wait_probe(long long limit_clocks, int *expired, void *stream);

/* DS rows [n_int][n_s*n_s] of the points whose branch code is 0 (elastic) set to the elastic matrix
 * the return mapping emits for them (bit for bit); other rows untouched.  Completes the DS of a
 * return mapping run with SSP_RM_PLASTIC_DS_ONLY.  No reference counterpart. */
int ssp_fill_elastic_ds(int dim, const int8_t *branch, const double *shear, const double *lame, int n_int,
                        double *ds_inout, void *stream);

int ssp_elastic_tangent_blocks(int dim, const double *shear, const double *lame, int n_int, double *ds_out,
                               void *stream);

/* out = (1-r) base + r elastic_values (the regularised blend of problem.py:1614-1615 applied to
 * a precomputed base). */
int ssp_blend_values(double *out_values, const double *base, const double *elastic_values, double r, long long nnz,
                     void *stream);

/* Constrained diagonals := 1.0 (distributed_tangent.py:1606-1607), then, when elastic_values is
 * not NULL, values := (1-r) values + r elastic_values (constitutive/problem.py:1614-1615). */
int ssp_finish_values(double *values, long long nnz, const int32_t *constrained_diag_positions, int n_diag,
                      const double *elastic_values, double r, void *stream);

/* dst[i] = src[idx[i]] (owned free rows of a force vector, problem.py:1008-1015). */
int ssp_gather(const double *src, const int32_t *idx, int n, double *dst, void *stream);

/* 1 if host_ptr is pinned, device-mapped host memory (cudaHostAlloc / cudaMallocHost memory, or
 * registered memory, under unified addressing) that kernels can store to, else 0.  The copy entry
 * points below address it through its device mapping (cudaPointerGetAttributes). */
int ssp_host_writable(const void *host_ptr);

/* dst[0..n) := src[0..n), both device memory, by a grid-stride kernel on the SMs (16-byte vectors
 * where both are aligned) rather than a memcpy: the operator's copy of a tangent's starting values,
 * which is then a kernel node when the build is captured in a CUDA graph.  No reference counterpart. */
int ssp_copy_device(const double *src, long long n, double *dst, void *stream);
/* The CSR rows r with row_mark[r] != 0 of src copied into dst (both device memory, the same
 * pattern indptr): restores a values array to its starting values where the previous build's
 * plastic-element corrections changed it.  No reference counterpart. */
int ssp_copy_rows_device(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows, long long nnz,
                         double *dst, void *stream);

/* No reference counterpart.  ssp_copy_rows_device with a grid of blocks_per_sm (1..8) 256-thread
 * blocks per SM (ssp_copy_rows_device: 8), for a copy issued on a second stream beside long kernels:
 * with a small share it runs beside them rather than ahead of them, at a lower rate of its own. */
int ssp_copy_rows_device_share(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows,
                               long long nnz, double *dst, int blocks_per_sm, void *stream);

/* dst_host[0..n) = src[0..n) written by the SMs into pinned, device-mapped host memory
 * (ssp_host_writable(dst_host) must hold, else SSP_ERR_INVALID); asynchronous on the stream.
 * The operator's host hand-off of the CSR values; no reference counterpart. */
int ssp_copy_out(const double *src, long long n, double *dst_host, void *stream);

/* No counterpart in the reference.  row_mark[r] = 1 (not cleared first) for every owned row
 * r = elem_row[e][a] (a < n_ld, r >= 0) of the elements e of elem_list[0 .. *elem_count): the rows
 * a plastic correction of those elements writes. */
int ssp_mark_element_rows(const int32_t *elem_row, int n_elem, int n_ld, const int32_t *elem_list,
                          const int32_t *elem_count, int n_rows, uint8_t *row_mark, void *stream);

/* No counterpart in the reference.  The CSR rows r with row_mark[r] != 0 of src (device) stored to
 * the same positions of dst_host (pinned, device-mapped host memory: ssp_host_writable), by the SMs.
 * Refreshes a host mirror of the tangent values whose other rows are known to be unchanged. */
int ssp_copy_rows_out(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows, long long nnz,
                      double *dst_host, void *stream);

/* No reference counterpart.  ssp_copy_rows_out with a grid of blocks_per_sm (1..8) 256-thread blocks
 * per SM (ssp_copy_rows_out: 4, which leaves half of each SM's threads to the kernels beside it). */
int ssp_copy_rows_out_share(const double *src, const int32_t *indptr, const uint8_t *row_mark, int n_rows,
                            long long nnz, double *dst_host, int blocks_per_sm, void *stream);

/* Reads the device status word (SSP_DEV_* bits); clear != 0 resets it.  Synchronous. */
int ssp_device_status(int *status_out, int clear);

/* ------------------------------------------------------------------ learned branch proposal */

/* No counterpart in the reference (it has no learned component).  A 6 -> 32 -> 32 -> 5 ReLU MLP
 * proposes each point's return branch from FP32 trial-strain features; points are binned by the
 * proposal and the exact FP64 return mapping runs bin by bin.  The parameters are one FP32 vector
 * of SSP_MLP_PARAMS values: W1[32][6], b1[32], W2[32][32], b2[32], W3[5][32], b3[5]. */
#define SSP_MLP_PARAMS 1445

/* Features X [n][6] (FP32) of the trial strains E [n][6]. */
int ssp_branch_features(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                        const double *lame, int n, float *X, void *stream);

/* Predicted branch (argmax) of every feature row.  mode 0: FP32 on the CUDA cores; 1: weights and
 * activations rounded to BF16, FP32 accumulation, CUDA cores; 2: the same BF16 network on the tensor
 * cores (tcgen05.mma kind::f16, FP32 accumulation in tensor memory; the inference the binning of
 * ssp_constitutive_3d_sds_learned uses). */
int ssp_mlp_predict(const float *params, const float *X, int n, int mode, int8_t *pred, void *stream);

/* Softmax cross-entropy of a batch against labels [n] (branch codes 0..4): grad [SSP_MLP_PARAMS]
 * receives the gradient summed over the batch, loss_sum the summed loss, correct the number of
 * argmax hits (all three are zeroed first). */
int ssp_mlp_loss_grad(const float *params, const float *X, const int8_t *labels, int n, float *grad,
                      float *loss_sum, int *correct, void *stream);

/* One Adam step on params with moments m, v (all SSP_MLP_PARAMS long); the gradient is scaled by
 * grad_scale first (e.g. 1/batch); step counts from 1. */
int ssp_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, float beta1, float beta2,
                 float eps, float grad_scale, void *stream);

/* The 3D return mapping with learned binning: the binned return mapping's elastic screen (pass A),
 * then a branch proposal by the MLP (tensor-core inference) for the points the screen listed,
 * which are binned by it; the exact FP64 decision pass runs over the five bins, then the branch
 * finish pass.  Same outputs as ssp_constitutive_sds_branch.  scratch is caller-allocated device
 * memory of 8*n_int + 12 int32 (the binned layout of 3*n_int + 4, then 8 bin counters and five
 * bins of n_int), overwritten. */
int ssp_constitutive_3d_sds_learned(const float *params, const double *E, const double *c_bar,
                                    const double *sin_phi, const double *shear, const double *lame, int n_int,
                                    double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                    void *stream);
/* The learned return mapping of the mixed-precision form (DS as ssp_constitutive_3d_sds_binned_mixed). */
int ssp_constitutive_3d_sds_learned_mixed(const float *params, const double *E, const double *c_bar,
                                          const double *sin_phi, const double *shear, const double *lame, int n_int,
                                          double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                          void *stream);

/* No counterpart in the reference: the trivial branch predictor beside the network.  The return
 * mapping with the points the elastic screen lists binned by given branch codes proposal [n_int]
 * (e.g. the previous Newton iteration's branch_out; codes outside 0..4 go to the elastic bin), then
 * the exact decision and finish passes as in ssp_constitutive_3d_sds_learned.  Same outputs, same
 * scratch layout; proposal must not alias branch_out. */
int ssp_constitutive_3d_sds_proposed(const int8_t *proposal, const double *E, const double *c_bar,
                                     const double *sin_phi, const double *shear, const double *lame, int n_int,
                                     double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                     void *stream);
/* The same in the mixed-precision form (DS as ssp_constitutive_3d_sds_binned_mixed). */
int ssp_constitutive_3d_sds_proposed_mixed(const int8_t *proposal, const double *E, const double *c_bar,
                                           const double *sin_phi, const double *shear, const double *lame, int n_int,
                                           double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                           void *stream);

/* No counterpart in the reference: every screened form of the 3D return mapping behind one entry.
 * Pass A (the FP32 elastic screen) finishes the points it proves elastic; the listed points are
 * binned by `bins` -- SSP_BINS_EXACT: one list, exact FP64 decision then one branch per warp
 * (ssp_constitutive_3d_sds_binned; scratch 3*n_int + 4 int32); SSP_BINS_LEARNED: the MLP's
 * proposal, bin_source = the FP32 parameter vector (ssp_constitutive_3d_sds_learned); SSP_BINS_GIVEN:
 * given branch codes, bin_source = int8 [n_int] not aliasing branch_out
 * (ssp_constitutive_3d_sds_proposed); the last two need scratch of 8*n_int + 12 int32.
 * options: SSP_RM_COMPENSATED_DS -- the plastic DS in double-float arithmetic (the mixed form);
 * SSP_RM_PLASTIC_DS_ONLY -- the DS rows of points that return elastic are not written (they equal
 * the elastic matrix; the tangent's plastic corrections never read them; ssp_fill_elastic_ds
 * writes them when a caller needs every row).  S and branch_out are always complete. */
#define SSP_BINS_EXACT 0
#define SSP_BINS_LEARNED 1
#define SSP_BINS_GIVEN 2
#define SSP_RM_COMPENSATED_DS 1
#define SSP_RM_PLASTIC_DS_ONLY 2
int ssp_constitutive_3d_sds_screened(const double *E, const double *c_bar, const double *sin_phi,
                                     const double *shear, const double *lame, int n_int, double *S_out,
                                     double *DS_out, int8_t *branch_out, int32_t *scratch, int bins,
                                     const void *bin_source, int options, void *stream);

/* ------------------------------------------------------------------ pattern (host) */

/* Fixed owned-row CSR pattern and element->CSR maps, built on the host in C++; replaces the
 * dictionary loops of prepare_owned_tangent_pattern (src/slope_stability/fem/distributed_tangent.py:
 * 297-478, 937-1175) with bit-identical output.  All pointers of the pattern API are HOST pointers.
 *
 * elem is [n_p][n_elem] int64 (global node ids), free_mask is [dim*n_nodes] (dof dim*node+comp,
 * nonzero = free, i.e. q_mask flattened in Fortran order); the owned node block is [node0, node1). */
typedef struct ssp_pattern ssp_pattern;

int ssp_pattern_build(int dim, int n_nodes, int n_p, int n_elem, const int64_t *elem, const uint8_t *free_mask,
                      int node0, int node1, ssp_pattern **out);

/* sizes[0..6] = n_overlap_elements, n_overlap_nodes, n_rows, nnz, n_slots, n_constrained, n_ld */
int ssp_pattern_sizes(const ssp_pattern *p, int64_t *sizes);

/* Copies one named array into dst (host, caller-sized from ssp_pattern_sizes).  Names and types:
 *   "overlap_elements" int64 [n_ov_el]        "overlap_nodes" int64 [n_ov_nodes]
 *   "overlap_element_dof_lids" int32 [n_ov_el][n_ld]   "owned_local_overlap_dofs" int64 [n_rows]
 *   "indptr" int32 [n_rows+1]   "indices" int32 [nnz]   "constrained_diag_positions" int32
 *   "scatter_map" int32 [n_ov_el][n_ld*n_ld]   "row_slot_ptr" int32 [n_rows+1]
 *   "slot_elem" int32 [n_slots]   "slot_lrow" uint8 [n_slots]   "slot_pos" int32 [n_slots][n_ld]
 *   "elem_row" int32 [n_ov_el][n_ld]   "owned_free_mask" uint8 [n_rows] */
int ssp_pattern_copy(const ssp_pattern *p, const char *name, void *dst);

void ssp_pattern_free(ssp_pattern *p);

#ifdef __cplusplus
}
#endif

#endif /* SSP_GB300_H */
