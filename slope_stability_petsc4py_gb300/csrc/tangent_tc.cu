// Mixed-precision plastic-correction tangent of P4 tetrahedra on the tensor cores (tcgen05).
//
// For an element whose plastic points are q (branch != elastic), the correction of the
// elastic-predictor tangent (assembly.cu, tangent_element_kernel in correction mode) is
//   K_e = sum_q B_q^T dD_q B_q,   dD_q = s w_q (DS_q - D_el,q),   B_q: 6 x 105,
// which is one dense contraction over kappa = (q, m), m a strain component:
//   K_e[alpha][beta] = sum_kappa H[alpha][kappa] Bk[kappa][beta],
//   H[alpha][(q, m)] = (B_q^T dD_q)[alpha][m],   Bk[(q, m)][beta] = B_q[m][beta].
// The compensated D*B term: the gradients and dD are split into hi + lo float pairs by bit
// operations and every H entry is a compensated dot product of three double-float terms on the
// FP32 pipe (about 46 significant bits; GB300's FP64 pipe is a small fraction of its FP32 rate).  Both operands are then split
// into TF32 pairs, x = hi + lo with hi = tf32(x), lo = tf32(x - hi), and the tensor cores form
// hi*hi and hi*lo + lo*hi (the three-product TF32 scheme: about 22 significant bits per product)
// in two FP32 accumulators in tensor memory.
//
// Accuracy.  A tensor-core MMA rounds its FP32 result once per instruction, so errors grow with
// the number of MMAs that feed one accumulator.  The points of an element are taken in groups of
// four (K = 24, three K = 8 steps); each group has its own pair of accumulators (hi*hi: three
// MMAs, cross terms: six, 2^-11 smaller), and the CUDA cores add every group's two partial sums
// into compensated (Kahan) FP32 sums in registers (widened exactly to FP64 once per element).  Two accumulator pairs alternate between groups (ping-pong), so the tensor
// cores multiply group g while the CUDA cores drain group g - 1 and build group g + 1.  The FP64
// element sums are added to the CSR values with FP64 reductions through the element->CSR map, on
// both mirror positions of alpha <= beta, so the correction is exactly symmetric.
//
// Tile: M = 128 rows (alpha, 105 used), N = 112 columns (beta, 105 used).  One CTA of 512 threads
// per SM, grid-striding over elements; it owns all 512 tensor-memory columns (two accumulator
// pairs at columns 0 / 128 and 256 / 384).  One thread issues the MMAs and commits each group to
// the mbarrier of its buffer.  Warp w drains accumulator lanes 32 (w % 4) .. + 31 (its lane
// quarter), columns 28 (w / 4) .. + 27.  The element's FP64 sums are staged in shared memory and
// scattered row by row, so the reductions of a warp fall on neighbouring entries of one CSR row.
//
// Operand layout in shared memory: K-major, no swizzle, in 8-row x 16-byte core matrices:
// byte offset(row, kappa) = ((kappa / 4) * (rows / 8) + row / 8) * 128 + (row % 8) * 16 + (kappa % 4) * 4,
// so the core matrices of one row group are 128 B apart along M/N (the descriptor's stride byte
// offset) and rows/8 * 128 B apart along K (its leading byte offset).
//
// Every wait on an mbarrier is bounded (about one second of SM clocks); on expiry the CTA sets
// SSP_DEV_TIMEOUT, stops, and still releases its tensor memory.
#include "ssp_internal.cuh"
#include "tcgen05.cuh"

namespace ssp {
namespace {

using namespace tc;

constexpr int kNP = 35, kNQ = 24, kNLD = 105, kNS = 6;
constexpr int kM = 128, kN = 112, kPts = 4, kK = kPts * kNS;  // 24 = three K steps of 8
constexpr int kThreads = 512;
constexpr int kScatterBatch = 8;                               // map entries a thread loads before its reductions
constexpr int kTmemCols = 512;                                 // two (hi*hi, cross) accumulator pairs
constexpr int kColsPerWarp = kN / 4;                           // 28 accumulator columns per drain warp
constexpr uint32_t kLboA = (kM / 8) * 128, kLboB = (kN / 8) * 128, kSbo = 128;
constexpr int kABytes = kM * kK * 4, kBBytes = kN * kK * 4;
static_assert(kABytes % 1024 == 0 && kBBytes % 128 == 0, "operand tiles keep 128-byte alignment");
static_assert(kColsPerWarp % 4 == 0, "drain loads four columns at a time");

// Instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t kIdesc = tc::idesc(tc::kFmtTF32, kM, kN);

struct Stage {  // one group of four points, operands split hi / lo
    uint32_t a_hi[kABytes / 4];
    uint32_t a_lo[kABytes / 4];
    uint32_t b_hi[kBBytes / 4];
    uint32_t b_lo[kBBytes / 4];
};
struct PointData {  // inputs of the group being built, as double-float (hi + lo) pairs
    df32 g[kPts][3][kNP];
    df32 dD[kPts][kNS * kNS];
};
struct RawInputs {  // FP64 inputs of the next group, copied ahead by cp.async
    double g[kPts * 3 * kNP];
    double ds[kPts * kNS * kNS], w[kPts * kNS * kNS], sh[kPts * kNS * kNS], la[kPts * kNS * kNS];
};
struct Smem {
    Stage stage[2];
    PointData pts;
    RawInputs raw;
    double ke[kNLD * kNLD];  // the element's FP64 sums (upper triangle used), staged for a row-wise scatter
    unsigned long long mbar[2];
    uint32_t tmem_slot;
    int abort;
    int nq[2];
    int sq[kNQ];
};
// Dynamic shared memory requested: more than half of an SM's, so one CTA (which owns all of the
// SM's tensor memory) is resident per SM.
constexpr size_t kSmemBytes = sizeof(Smem) > 120 * 1024 ? sizeof(Smem) : 120 * 1024;
static_assert(sizeof(Smem) <= 227 * 1024, "shared memory of one CTA");

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
// A double-float value as two TF32 parts: hi = tf32(x.hi), lo = tf32((x.hi - hi) + x.lo); the
// subtraction is exact (hi is x.hi rounded to 10 mantissa bits).
__device__ __forceinline__ void split_tf32(df32 x, uint32_t &hi, uint32_t &lo) {
    hi = to_tf32(x.hi);
    lo = to_tf32(__fadd_rn(__fsub_rn(x.hi, __uint_as_float(hi)), x.lo));
}

// 32 lanes x 16 consecutive FP32 columns of the accumulator (this warp's lane quarter), waited for.
__device__ __forceinline__ void tmem_ld16f(uint32_t taddr, float *v) {
    uint32_t r[16];
    tmem_ld16(taddr, r);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
// The 28 accumulator columns col0 .. col0 + 27 of this thread's lane.
__device__ __forceinline__ void tmem_ld28(uint32_t taddr0, uint32_t *r) {
    tmem_ld16(taddr0, r);
    tmem_ld8(taddr0 + 16, r + 16);
    tmem_ld4(taddr0 + 24, r + 24);
}

// Compensated (Kahan) running sums of the groups' partials: sum[j] - comp[j] is the element's
// value of column j; each group adds its hi*hi and cross partials.
__device__ __forceinline__ void drain_add(uint32_t taddr_hh, uint32_t taddr_x, float *sum, float *comp) {
    uint32_t rh[kColsPerWarp], rx[kColsPerWarp];
    tmem_ld28(taddr_hh, rh);
    tmem_ld28(taddr_x, rx);
    tmem_wait_ld();
#pragma unroll
    for (int j = 0; j < kColsPerWarp; ++j) {
        const float x = __fadd_rn(__uint_as_float(rh[j]), __uint_as_float(rx[j]));
        const float y = __fsub_rn(x, comp[j]);
        const float t = __fadd_rn(sum[j], y);
        comp[j] = __fsub_rn(__fsub_rn(t, sum[j]), y);
        sum[j] = t;
    }
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

__device__ __forceinline__ double elastic_d3(int i, int j, double G, double lam) {
    if (i < 3 && j < 3) return i == j ? 2.0 * G + lam : lam;
    if (i == j) return G;
    return 0.0;
}

// Every thread waits for the commit of group parity b (bounded), then adds that group's two
// accumulators to its compensated sums.
__device__ __forceinline__ void drain_group(Smem &S, uint32_t tmem, int b, uint32_t &phase_bits, uint32_t lane_col,
                                            float *sum, float *comp) {
    if (!mbar_wait(smem_u32(&S.mbar[b]), (phase_bits >> b) & 1u)) {
        S.abort = 1;
        flag(SSP_DEV_TIMEOUT);
    }
    phase_bits ^= 1u << b;
    fence_after_sync();
    const uint32_t base = tmem + lane_col + 256u * b;
    drain_add(base, base + 128u, sum, comp);  // hi * hi, hi * lo + lo * hi
    fence_before_sync();                      // these reads precede the next MMAs into this pair
}

__global__ void __launch_bounds__(kThreads, 1) correction_tc_p4_kernel(
    const double *__restrict__ d1, const double *__restrict__ d2, const double *__restrict__ d3,
    const double *__restrict__ DS, const double *__restrict__ w, const int8_t *__restrict__ branch,
    const double *__restrict__ shear, const double *__restrict__ lame, const int32_t *__restrict__ emap, int n_elem,
    long long nnz, double scale, double *__restrict__ values, const int32_t *__restrict__ elist,
    const int32_t *__restrict__ elist_count) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lq = warp & 3, cq = warp >> 2;  // drain lane quarter and column quarter
    const uint32_t lane_col = (static_cast<uint32_t>(32 * lq) << 16) + static_cast<uint32_t>(kColsPerWarp * cq);

    // zero both stages once: the padding rows (alpha >= 105, beta >= 105) are never written again
    for (int i = tid; i < (int)(sizeof(Stage) * 2 / 4); i += kThreads) reinterpret_cast<uint32_t *>(S.stage)[i] = 0u;
    if (tid == 0) {
        mbar_init(smem_u32(&S.mbar[0]));
        mbar_init(smem_u32(&S.mbar[1]));
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = S.tmem_slot;
    uint32_t phase_bits = 0;
    int parity = 0;

    const long long n_iter = elist ? static_cast<long long>(*elist_count) : static_cast<long long>(n_elem);
    for (long long it = blockIdx.x; it < n_iter; it += gridDim.x, parity ^= 1) {
        long long e = it;
        if (elist) {
            e = elist[it];
            if (e < 0 || e >= n_elem) {  // uniform across the CTA
                if (tid == 0) flag(SSP_DEV_BAD_INDEX);
                continue;
            }
        }
        const long long g0 = e * kNQ;
        if (warp == 0) {
            const bool pl = lane < kNQ && branch[g0 + lane] != 0;
            const unsigned mask = __ballot_sync(0xffffffffu, pl);
            if (pl) S.sq[__popc(mask & ((1u << lane) - 1u))] = lane;
            if (lane == 0) S.nq[parity] = __popc(mask);
        }
        __syncthreads();
        const int nq = S.nq[parity];
        if (nq == 0) continue;  // uniform across the CTA
        const int groups = (nq + kPts - 1) / kPts;
        float sum[kColsPerWarp], comp[kColsPerWarp];
#pragma unroll
        for (int j = 0; j < kColsPerWarp; ++j) sum[j] = comp[j] = 0.0f;
        // the raw FP64 inputs of a group are copied into shared memory one group ahead (cp.async, in
        // flight while the current group's H is formed and multiplied): thread t < 420 one gradient
        // value, thread t < 144 one DS entry with its point's w, shear and lame; each thread later
        // converts only the entries it copied itself
        // (indices recomputed from tid where used: cheaper than keeping them live across the loop)
        auto load_group = [&](int grp) {
            if (tid < kPts * 3 * kNP) {
                const int gi_pi = tid / (3 * kNP), gi_r = (tid % (3 * kNP)) / kNP, gi_a = tid % kNP;
                const int k = grp * kPts + gi_pi;
                if (k < nq) {
                    const long long src = (g0 + S.sq[k]) * kNP + gi_a;
                    cp_async8(&S.raw.g[tid], (gi_r == 0 ? d1 : (gi_r == 1 ? d2 : d3)) + src);
                }
            }
            if (tid < kPts * kNS * kNS) {
                const int k = grp * kPts + tid / (kNS * kNS);
                if (k < nq) {
                    const long long gq = g0 + S.sq[k];
                    cp_async8(&S.raw.ds[tid], DS + gq * (kNS * kNS) + tid % (kNS * kNS));
                    cp_async8(&S.raw.w[tid], w + gq);
                    cp_async8(&S.raw.sh[tid], shear + gq);
                    cp_async8(&S.raw.la[tid], lame + gq);
                }
            }
            cp_async_commit();
        };
        load_group(0);
        for (int grp = 0; grp < groups; ++grp) {
            const int b = grp & 1;  // stage buffer and accumulator pair; both were released by drain(grp - 2)
            // inputs of the group's points as hi + lo pairs (absent slots are zero): the gradients,
            // and w s (DS - D_el) with the FP64 subtraction only where D_el is nonzero
            cp_async_wait_all();
            if (tid < kPts * 3 * kNP) {
                const int gi_pi = tid / (3 * kNP), gi_r = (tid % (3 * kNP)) / kNP, gi_a = tid % kNP;
                const int k = grp * kPts + gi_pi;
                S.pts.g[gi_pi][gi_r][gi_a] = k < nq ? df_from_f64(S.raw.g[tid]) : df32{0.0f, 0.0f};
            }
            if (tid < kPts * kNS * kNS) {
                const int di_pi = tid / (kNS * kNS), di_kk = tid % (kNS * kNS);
                const int k = grp * kPts + di_pi;
                df32 v{0.0f, 0.0f};
                if (k < nq) {
                    double d = S.raw.ds[tid];
                    const double de = elastic_d3(di_kk % kNS, di_kk / kNS, S.raw.sh[tid], S.raw.la[tid]);
                    if (de != 0.0) d -= de;
                    v = df_mul(df_from_f64(d), df_from_f64(scale * S.raw.w[tid]));
                }
                S.pts.dD[di_pi][di_kk] = v;
            }
            __syncthreads();
            if (grp + 1 < groups) load_group(grp + 1);
            Stage &st = S.stage[b];
            unsigned char *a_hi = reinterpret_cast<unsigned char *>(st.a_hi);
            unsigned char *a_lo = reinterpret_cast<unsigned char *>(st.a_lo);
            unsigned char *b_hi = reinterpret_cast<unsigned char *>(st.b_hi);
            unsigned char *b_lo = reinterpret_cast<unsigned char *>(st.b_lo);
            if (tid < kPts * kNLD) {
                // H = B^T dD for one (point, alpha), all six strain components: compensated dot
                // products of three terms on the FP32 pipe; alpha = 3 * node + component
                const int pi = tid / kNLD, alpha = tid - pi * kNLD;
                const int a = alpha / 3, c = alpha - 3 * a;
                const df32 ga = S.pts.g[pi][0][a], gb = S.pts.g[pi][1][a], gc = S.pts.g[pi][2][a];
                const int k0 = bt_row3(c, 0), k1 = bt_row3(c, 1), k2 = bt_row3(c, 2);
                const df32 *D = S.pts.dD[pi];
#pragma unroll
                for (int m = 0; m < kNS; ++m) {
                    const df32 h = df_dot3(ga, D[k0 + kNS * m], gb, D[k1 + kNS * m], gc, D[k2 + kNS * m]);
                    uint32_t hi, lo;
                    split_tf32(h, hi, lo);
                    const int off = kmaj_off<4>(alpha, pi * kNS + m, kM);
                    *reinterpret_cast<uint32_t *>(a_hi + off) = hi;
                    *reinterpret_cast<uint32_t *>(a_lo + off) = lo;
                }
            } else {
                // the nonzeros of Bk: g[pi][r][bn] at beta = 3 bn + cp, kappa = 6 pi + bt_row3(cp, r); the
                // other entries are zero in every group and were zeroed once
                for (int i = tid - kPts * kNLD; i < kPts * 3 * kNP * 3; i += kThreads - kPts * kNLD) {
                    const int cp = i % 3, rest = i / 3, bn = rest % kNP, pr = rest / kNP, r = pr % 3, pi = pr / 3;
                    uint32_t hi, lo;
                    split_tf32(S.pts.g[pi][r][bn], hi, lo);
                    const int off = kmaj_off<4>(3 * bn + cp, pi * kNS + bt_row3(cp, r), kN);
                    *reinterpret_cast<uint32_t *>(b_hi + off) = hi;
                    *reinterpret_cast<uint32_t *>(b_lo + off) = lo;
                }
            }
            fence_async_smem();  // generic-proxy writes -> visible to the tensor cores
            __syncthreads();
            if (S.abort) break;
            if (tid == 0) {
                fence_after_sync();
                const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_hi), bl = smem_u32(b_lo);
                const uint32_t t_hh = tmem + 256u * b, t_x = t_hh + 128u;
#pragma unroll
                for (int s = 0; s < kK / 8; ++s) {
                    const uint32_t oa = s * 2 * kLboA, ob = s * 2 * kLboB;
                    mma_tf32(t_hh, smem_desc(ah + oa, kLboA, kSbo), smem_desc(bh + ob, kLboB, kSbo), kIdesc, s != 0 ? 1u : 0u);
                    mma_tf32(t_x, smem_desc(ah + oa, kLboA, kSbo), smem_desc(bl + ob, kLboB, kSbo), kIdesc, s != 0 ? 1u : 0u);
                    mma_tf32(t_x, smem_desc(al + oa, kLboA, kSbo), smem_desc(bh + ob, kLboB, kSbo), kIdesc, 1u);
                }
                mma_commit(smem_u32(&S.mbar[b]));
            }
            if (grp >= 1) drain_group(S, tmem, b ^ 1, phase_bits, lane_col, sum, comp);
        }
        if (S.abort) break;
        drain_group(S, tmem, (groups - 1) & 1, phase_bits, lane_col, sum, comp);
        __syncthreads();  // also orders this element's shared-memory reads before the next element's writes
        if (S.abort) break;
        // stage the upper triangle, then scatter every entry row by row (consecutive threads ->
        // consecutive columns of one CSR row, so the reductions of a warp share cache lines)
        const int row = 32 * lq + lane;
        if (row < kNLD) {
#pragma unroll
            for (int j = 0; j < kColsPerWarp; ++j) {
                const int beta = kColsPerWarp * cq + j;
                if (beta >= row && beta < kNLD) S.ke[row * kNLD + beta] = df_to_f64({sum[j], -comp[j]});
            }
        }
        __syncthreads();
        // the element's map row (44 KB, not staged) is read kScatterBatch entries per thread at a
        // time, so a thread's loads are in flight together before its reductions
        const int32_t *em = emap + (long long)e * kNLD * kNLD;
        for (int base = tid; base < kNLD * kNLD; base += kThreads * kScatterBatch) {
            int32_t p[kScatterBatch];
#pragma unroll
            for (int u = 0; u < kScatterBatch; ++u) {
                const int idx = base + u * kThreads;
                p[u] = idx < kNLD * kNLD ? em[idx] : -1;
            }
#pragma unroll
            for (int u = 0; u < kScatterBatch; ++u) {
                const int idx = base + u * kThreads;
                if (p[u] < 0) continue;
                const int a = idx / kNLD, bcol = idx - a * kNLD;
                const double val = bcol >= a ? S.ke[idx] : S.ke[bcol * kNLD + a];
                if (p[u] < nnz) red_add(values + p[u], val);
                else flag(SSP_DEV_BAD_INDEX);
            }
        }
    }
    // all tensor-core work of this CTA has been waited for (or abandoned after a timeout)
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// Layout / descriptor check: D[128][112] = A[128][K] B[112][K]^T through the same shared-memory
// layout, descriptors and tensor-memory read-back as the kernel above (one CTA, K = 8, 16 or 24).
// convention 0 passes (leading, stride) byte offsets as (K-direction, row-direction) core-matrix
// strides, convention 1 swaps them.  Operands sit in a 64 KiB buffer so either reading stays
// inside it.
__global__ void __launch_bounds__(128, 1) tc_probe_kernel(const float *__restrict__ A, const float *__restrict__ B,
                                                          int K, int convention, float *__restrict__ D) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sa = smem_raw, *sb = smem_raw + 32768;
    unsigned long long *mbar = reinterpret_cast<unsigned long long *>(smem_raw + 65536);
    uint32_t *slot = reinterpret_cast<uint32_t *>(smem_raw + 65536 + 8);
    int *abort_flag = reinterpret_cast<int *>(smem_raw + 65536 + 12);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < 65536 / 4; i += 128) reinterpret_cast<uint32_t *>(smem_raw)[i] = 0u;
    __syncthreads();
    for (int i = tid; i < kM * K; i += 128) {
        const int r = i / K, k = i % K;
        *reinterpret_cast<uint32_t *>(sa + kmaj_off<4>(r, k, kM)) = to_tf32(A[i]);
    }
    for (int i = tid; i < kN * K; i += 128) {
        const int r = i / K, k = i % K;
        *reinterpret_cast<uint32_t *>(sb + kmaj_off<4>(r, k, kN)) = to_tf32(B[i]);
    }
    if (tid == 0) {
        mbar_init(smem_u32(mbar));
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        const uint32_t la = convention == 0 ? kLboA : kSbo, sa_ = convention == 0 ? kSbo : kLboA;
        const uint32_t lb = convention == 0 ? kLboB : kSbo, sb_ = convention == 0 ? kSbo : kLboB;
        for (int s = 0; s < K / 8; ++s)
            mma_tf32(tmem, smem_desc(smem_u32(sa) + s * 2 * kLboA, la, sa_), smem_desc(smem_u32(sb) + s * 2 * kLboB, lb, sb_),
                     kIdesc, s != 0 ? 1u : 0u);
        mma_commit(smem_u32(mbar));
        if (!mbar_wait(smem_u32(mbar), 0)) {
            *abort_flag = 1;
            flag(SSP_DEV_TIMEOUT);
        }
    }
    __syncthreads();
    fence_after_sync();
    if (*abort_flag == 0) {
        for (int ch = 0; ch < kN / 16; ++ch) {
            float v[16];
            tmem_ld16f(tmem + (static_cast<uint32_t>(32 * warp) << 16) + ch * 16, v);
            const int row = 32 * warp + lane;
#pragma unroll
            for (int j = 0; j < 16; ++j) D[row * kN + ch * 16 + j] = v[j];
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

// The expiry path of the bounded waits, exercised without a tensor-core operation: warp 0 takes
// tensor memory as the kernels do, thread 0 waits on an mbarrier nothing ever arrives on, with a
// limit of `limit` clocks; on expiry it sets SSP_DEV_TIMEOUT, and the CTA frees the tensor memory
// and returns, as the kernels do when a wait expires.
__global__ void __launch_bounds__(128) tc_wait_probe_kernel(long long limit, int *expired) {
    __shared__ uint32_t slot;
    __shared__ __align__(8) uint64_t mbar;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) tmem_alloc(&slot, 32);
    if (tid == 0) {
        mbar_init(smem_u32(&mbar));
        mbar_init_fence();
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = slot;
    if (tid == 0) {
        const bool done = mbar_wait(smem_u32(&mbar), 0, limit);
        *expired = done ? 0 : 1;
        if (!done) flag(SSP_DEV_TIMEOUT);
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tmem, 32);
    }
}

}  // namespace

int correction_tc_p4(const double *d1, const double *d2, const double *d3, const double *DS, const double *w,
                     const int8_t *branch, const double *shear, const double *lame, const int32_t *emap, int n_elem,
                     long long nnz, double scale, double *values, const int32_t *elist, const int32_t *elist_count,
                     cudaStream_t st) {
    const size_t smem = kSmemBytes;
    if (cudaFuncSetAttribute(correction_tc_p4_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess)
        return SSP_ERR_CUDA;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = sms;  // one CTA per SM: each owns the SM's 512 tensor-memory columns
    if (grid > n_elem) grid = n_elem;
    correction_tc_p4_kernel<<<static_cast<unsigned>(grid), kThreads, smem, st>>>(d1, d2, d3, DS, w, branch, shear, lame,
                                                                                   emap, n_elem, nnz, scale, values,
                                                                                   elist, elist_count);
    return launch_status();
}

}  // namespace ssp

using namespace ssp;

extern "C" int ssp_tc_wait_probe(long long limit_clocks, int *expired, void *stream) {
    if (limit_clocks <= 0 || limit_clocks > kWaitLimitClocks || !expired) return SSP_ERR_INVALID;
    tc_wait_probe_kernel<<<1, 128, 0, as_stream(stream)>>>(limit_clocks, expired);
    return launch_status();
}

extern "C" int ssp_tc_tf32_probe(const float *A, const float *B, int K, int convention, float *D, void *stream) {
    if ((K != 8 && K != 16 && K != 24) || (convention != 0 && convention != 1) || !A || !B || !D)
        return SSP_ERR_INVALID;
    const int smem = 65536 + 64;
    if (cudaFuncSetAttribute(tc_probe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return SSP_ERR_CUDA;
    tc_probe_kernel<<<1, 128, smem, as_stream(stream)>>>(A, B, K, convention, D);
    return launch_status();
}
