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
// four (K = 24, three K = 8 steps), and two consecutive groups of an element (a batch) share a pair
// of accumulators (hi*hi: up to six MMAs, cross terms: up to twelve, 2^-11 smaller); every batch's
// two partial sums are added into compensated (Kahan) FP32 sums of the element (widened exactly
// to FP64 once per element).  The FP64
// element sums are added to the CSR values with FP64 reductions through the element->CSR map, on
// both mirror positions of alpha <= beta, so the correction is exactly symmetric.
//
// Tile: M = 128 rows (alpha, 105 used), N = 112 columns (beta, 105 used).  One CTA of 512 threads
// per SM, grid-striding over elements; it owns all 512 tensor-memory columns (two accumulator
// pairs at columns 0 / 128 and 256 / 384, alternating between batches).  The warps specialise:
// warps 0-7 build each group's operands into one of two stage buffers and one of their threads
// issues the group's MMAs; warps 8-15 drain each accumulator pair into the element's compensated
// sums, which live in shared memory, and scatter the finished element.  The roles hand off through
// mbarriers (the MMA commit of a stage buffer, the MMA commit of a batch into a pair, and the
// eight drain warps' release of the pair) and synchronise inside a role with named barriers, so
// the builders form group g + 1 while the tensor cores multiply group g and the drain warps read
// the previous batch or scatter the previous element.
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
constexpr uint32_t kLboA = (kM / 8) * 128, kLboB = (kN / 8) * 128, kSbo = 128;
constexpr int kABytes = kM * kK * 4, kBBytes = kN * kK * 4;
static_assert(kABytes % 1024 == 0 && kBBytes % 128 == 0, "operand tiles keep 128-byte alignment");

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
// Warp roles: warps 0-7 build the operands (inputs converted to double-float, H = B^T dD and B
// split into TF32 pairs, one thread issuing the MMAs); warps 8-15 drain the accumulators into the
// element's compensated sums and scatter them.  Drain warp w owns tensor-memory lane quarter w % 4
// (TMEM rows 32 (w % 4) ..+ 31, the row each lane reads) and the column half (w - 8) / 4.
constexpr int kBuildThreads = 256, kDrainThreads = 256;
constexpr int kDrainCols = kN / 2;                     // 56 accumulator columns per drain thread
constexpr int kKeStride = kN + 1;                      // float2 row stride of the element sums (spreads banks)
constexpr int kBarBuild = 1, kBarDrain = 2;            // named barriers of the two roles
struct Smem {
    Stage stage[2];
    PointData pts;
    RawInputs raw;
    float2 ke[kNLD * kKeStride];  // the element's compensated FP32 sums (s, c), upper triangle used
    unsigned long long stage_free[2];  // commit of the MMAs that read stage buffer b (count 1)
    unsigned long long acc_full[2];    // commit of a batch's MMAs into accumulator pair b (count 1)
    unsigned long long acc_empty[2];   // the eight drain warps have read pair b (count 8)
    uint32_t tmem_slot;
    int abort;   // any role gave up on a wait (the device status has SSP_DEV_TIMEOUT)
    int babort;  // the builders stop (read only after a builders' barrier)
    int dabort;  // the drainers stop (read only after a drainers' barrier)
    int nq;
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

__device__ __forceinline__ void named_bar(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_count(uint32_t addr, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(addr), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t addr) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(addr) : "memory");
}
__device__ __forceinline__ long long element_at(const int32_t *elist, long long it, int n_elem) {
    if (!elist) return it;
    const long long e = elist[it];
    return (e < 0 || e >= n_elem) ? -1 : e;
}

// Builders: per group of four plastic points, the inputs (copied one group ahead by cp.async, each
// thread converting the entries it copied), then H = B^T dD (compensated double-float dot products)
// and the nonzeros of B, both split into TF32 pairs, into the stage buffer of the group's parity;
// one thread issues the nine MMAs into the accumulator pair of the batch's parity and commits them
// to stage_free (and, after a batch's last group, to acc_full).  A stage buffer is rewritten only
// after the MMAs that read it (two groups back) have completed, an accumulator pair only after the
// drain warps have read it (acc_empty, two batches back).
__device__ __forceinline__ void build_role(Smem &S, uint32_t tmem, const double *__restrict__ d1,
                                           const double *__restrict__ d2, const double *__restrict__ d3,
                                           const double *__restrict__ DS, const double *__restrict__ w,
                                           const int8_t *__restrict__ branch, const double *__restrict__ shear,
                                           const double *__restrict__ lame, int n_elem, double scale,
                                           const int32_t *__restrict__ elist, long long n_iter) {
    const int bt = threadIdx.x, warp = bt >> 5, lane = bt & 31;
    uint32_t G = 0;   // the CTA's running group count (stage buffer G & 1)
    uint32_t Bn = 0;  // the CTA's running batch count (accumulator pair Bn & 1; the drain warps count the same)
    for (long long it = blockIdx.x; it < n_iter; it += gridDim.x) {
        const long long e = element_at(elist, it, n_elem);
        if (e < 0) {  // uniform
            if (bt == 0) flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        const long long g0 = e * kNQ;
        if (warp == 0) {
            const bool pl = lane < kNQ && branch[g0 + lane] != 0;
            const unsigned mask = __ballot_sync(0xffffffffu, pl);
            if (pl) S.sq[__popc(mask & ((1u << lane) - 1u))] = lane;
            if (lane == 0) S.nq = __popc(mask);
        }
        named_bar(kBarBuild, kBuildThreads);
        const int nq = S.nq;
        if (nq == 0) continue;  // uniform
        const int groups = (nq + kPts - 1) / kPts;
        // raw FP64 inputs of group grp: thread t copies gradient values t, t + 256 (< 420) and,
        // for t < 144, one DS entry with its point's w, shear and lame
        auto load_group = [&](int grp) {
            for (int i = bt; i < kPts * 3 * kNP; i += kBuildThreads) {
                const int gi_pi = i / (3 * kNP), gi_r = (i % (3 * kNP)) / kNP, gi_a = i % kNP;
                const int k = grp * kPts + gi_pi;
                if (k < nq) {
                    const long long src = (g0 + S.sq[k]) * kNP + gi_a;
                    cp_async8(&S.raw.g[i], (gi_r == 0 ? d1 : (gi_r == 1 ? d2 : d3)) + src);
                }
            }
            if (bt < kPts * kNS * kNS) {
                const int k = grp * kPts + bt / (kNS * kNS);
                if (k < nq) {
                    const long long gq = g0 + S.sq[k];
                    cp_async8(&S.raw.ds[bt], DS + gq * (kNS * kNS) + bt % (kNS * kNS));
                    cp_async8(&S.raw.w[bt], w + gq);
                    cp_async8(&S.raw.sh[bt], shear + gq);
                    cp_async8(&S.raw.la[bt], lame + gq);
                }
            }
            cp_async_commit();
        };
        load_group(0);
        for (int grp = 0; grp < groups; ++grp, ++G) {
            const int b = G & 1, pb = Bn & 1;
            // a batch is two consecutive groups of the element (the last one alone when their number is odd)
            const bool first = (grp & 1) == 0, last = (grp & 1) == 1 || grp + 1 == groups;
            cp_async_wait_all();
            for (int i = bt; i < kPts * 3 * kNP; i += kBuildThreads) {
                const int gi_pi = i / (3 * kNP), gi_r = (i % (3 * kNP)) / kNP, gi_a = i % kNP;
                const int k = grp * kPts + gi_pi;
                S.pts.g[gi_pi][gi_r][gi_a] = k < nq ? df_from_f64(S.raw.g[i]) : df32{0.0f, 0.0f};
            }
            if (bt < kPts * kNS * kNS) {
                const int di_pi = bt / (kNS * kNS), di_kk = bt % (kNS * kNS);
                const int k = grp * kPts + di_pi;
                df32 v{0.0f, 0.0f};
                if (k < nq) {
                    double d = S.raw.ds[bt];
                    const double de = elastic_d3(di_kk % kNS, di_kk / kNS, S.raw.sh[bt], S.raw.la[bt]);
                    if (de != 0.0) d -= de;
                    v = df_mul(df_from_f64(d), df_from_f64(scale * S.raw.w[bt]));
                }
                S.pts.dD[di_pi][di_kk] = v;
            }
            if (bt == 0) {  // stage b was last read by the MMAs of group G - 2
                if (S.abort) {
                    S.babort = 1;
                } else if (G >= 2 && !mbar_wait(smem_u32(&S.stage_free[b]), ((G - 2) >> 1) & 1u)) {
                    S.babort = S.abort = 1;
                    flag(SSP_DEV_TIMEOUT);
                }
            }
            named_bar(kBarBuild, kBuildThreads);  // inputs converted, stage b free
            if (S.babort) {
                cp_async_wait_all();
                return;
            }
            if (grp + 1 < groups) load_group(grp + 1);
            Stage &st = S.stage[b];
            unsigned char *a_hi = reinterpret_cast<unsigned char *>(st.a_hi);
            unsigned char *a_lo = reinterpret_cast<unsigned char *>(st.a_lo);
            unsigned char *b_hi = reinterpret_cast<unsigned char *>(st.b_hi);
            unsigned char *b_lo = reinterpret_cast<unsigned char *>(st.b_lo);
            // H = B^T dD: item (point, alpha, half) forms three strain components of one row,
            // compensated dot products of three terms on the FP32 pipe; alpha = 3 * node + component
            for (int i = bt; i < kPts * kNLD * 2; i += kBuildThreads) {
                const int half = i & 1, rest = i >> 1;
                const int pi = rest / kNLD, alpha = rest - pi * kNLD;
                const int a = alpha / 3, c = alpha - 3 * a;
                const df32 ga = S.pts.g[pi][0][a], gb = S.pts.g[pi][1][a], gc = S.pts.g[pi][2][a];
                const int k0 = bt_row3(c, 0), k1 = bt_row3(c, 1), k2 = bt_row3(c, 2);
                const df32 *D = S.pts.dD[pi];
#pragma unroll
                for (int mm = 0; mm < 3; ++mm) {
                    const int m = 3 * half + mm;
                    const df32 h = df_dot3(ga, D[k0 + kNS * m], gb, D[k1 + kNS * m], gc, D[k2 + kNS * m]);
                    uint32_t hi, lo;
                    split_tf32(h, hi, lo);
                    const int off = kmaj_off<4>(alpha, pi * kNS + m, kM);
                    *reinterpret_cast<uint32_t *>(a_hi + off) = hi;
                    *reinterpret_cast<uint32_t *>(a_lo + off) = lo;
                }
            }
            // the nonzeros of Bk: g[pi][r][bn] at beta = 3 bn + cp, kappa = 6 pi + bt_row3(cp, r); the
            // other entries are zero in every group and were zeroed once
            for (int i = bt; i < kPts * 3 * kNP * 3; i += kBuildThreads) {
                const int cp = i % 3, rest = i / 3, bn = rest % kNP, pr = rest / kNP, r = pr % 3, pi = pr / 3;
                uint32_t hi, lo;
                split_tf32(S.pts.g[pi][r][bn], hi, lo);
                const int off = kmaj_off<4>(3 * bn + cp, pi * kNS + bt_row3(cp, r), kN);
                *reinterpret_cast<uint32_t *>(b_hi + off) = hi;
                *reinterpret_cast<uint32_t *>(b_lo + off) = lo;
            }
            fence_async_smem();  // generic-proxy writes -> visible to the tensor cores
            named_bar(kBarBuild, kBuildThreads);  // stage b complete
            if (bt == 0) {
                bool ok = !S.abort;
                if (ok && first && Bn >= 2 && !mbar_wait(smem_u32(&S.acc_empty[pb]), ((Bn - 2) >> 1) & 1u)) {
                    ok = false;
                    S.abort = 1;
                    flag(SSP_DEV_TIMEOUT);
                }
                if (ok) {
                    fence_after_sync();
                    const uint32_t ah = smem_u32(a_hi), al = smem_u32(a_lo), bh = smem_u32(b_hi), bl = smem_u32(b_lo);
                    const uint32_t t_hh = tmem + 256u * pb, t_x = t_hh + 128u;
#pragma unroll
                    for (int s = 0; s < kK / 8; ++s) {
                        const uint32_t oa = s * 2 * kLboA, ob = s * 2 * kLboB;
                        const uint32_t acc = (s != 0 || !first) ? 1u : 0u;  // a batch's first MMAs overwrite
                        mma_tf32(t_hh, smem_desc(ah + oa, kLboA, kSbo), smem_desc(bh + ob, kLboB, kSbo), kIdesc, acc);
                        mma_tf32(t_x, smem_desc(ah + oa, kLboA, kSbo), smem_desc(bl + ob, kLboB, kSbo), kIdesc, acc);
                        mma_tf32(t_x, smem_desc(al + oa, kLboA, kSbo), smem_desc(bh + ob, kLboB, kSbo), kIdesc, 1u);
                    }
                    mma_commit(smem_u32(&S.stage_free[b]));
                    if (last) mma_commit(smem_u32(&S.acc_full[pb]));
                } else {
                    S.babort = 1;  // seen by the builders after their next barrier
                }
            }
            if (last) ++Bn;
        }
    }
    cp_async_wait_all();
}

// Drain warps: per batch, one lane waits for the commit (acc_full of the batch's parity), the warp
// reads its 32 accumulator rows x 56 columns of both accumulators (hi * hi, cross terms) and adds
// their sum into the element's compensated sums in shared memory (upper triangle only), then
// releases the pair (acc_empty).  After an element's last group the 256 drain threads scatter the
// element's sums to both mirror positions through the element -> CSR map with FP64 reductions.
__device__ __forceinline__ void drain_role(Smem &S, uint32_t tmem, const int8_t *__restrict__ branch,
                                           const int32_t *__restrict__ emap, int n_elem, long long nnz,
                                           double *__restrict__ values, const int32_t *__restrict__ elist,
                                           long long n_iter) {
    const int dt = threadIdx.x - kBuildThreads, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int lq = warp & 3, chalf = (warp - kBuildThreads / 32) >> 2;
    const int row = 32 * lq + lane, col0 = kDrainCols * chalf;
    const uint32_t lane_col = (static_cast<uint32_t>(32 * lq) << 16) + static_cast<uint32_t>(col0);
    float2 *kr = S.ke + row * kKeStride;  // this lane's row of sums (row < kNLD)
    uint32_t Bn = 0;  // running batch count, as the builders count it
    for (long long it = blockIdx.x; it < n_iter; it += gridDim.x) {
        const long long e = element_at(elist, it, n_elem);
        if (e < 0) continue;  // uniform (the builders flag it)
        const bool pl = lane < kNQ && branch[e * kNQ + lane] != 0;
        const int nq = __popc(__ballot_sync(0xffffffffu, pl));
        if (nq == 0) continue;
        const int groups = (nq + kPts - 1) / kPts;
        if (row < kNLD) {
            for (int j = 0; j < kDrainCols; ++j) {
                const int c = col0 + j;
                if (c >= row && c < kNLD) kr[c] = make_float2(0.0f, 0.0f);
            }
        }
        bool skipped = false;
        const int batches = (groups + 1) / 2;
        for (int bi = 0; bi < batches; ++bi, ++Bn) {
            const int b = Bn & 1;
            int ok = 0;
            if (lane == 0) {
                ok = !S.abort;
                if (ok && !mbar_wait(smem_u32(&S.acc_full[b]), (Bn >> 1) & 1u)) {
                    ok = 0;
                    S.abort = 1;
                    flag(SSP_DEV_TIMEOUT);
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (ok) {
                fence_after_sync();
                const uint32_t base = tmem + lane_col + 256u * b;
#pragma unroll
                for (int part = 0; part < 2; ++part) {  // 28 columns at a time
                    uint32_t rh[28], rx[28];
                    const uint32_t t0 = base + 28u * part;
                    tmem_ld16(t0, rh);
                    tmem_ld8(t0 + 16u, rh + 16);
                    tmem_ld4(t0 + 24u, rh + 24);
                    tmem_ld16(t0 + 128u, rx);
                    tmem_ld8(t0 + 144u, rx + 16);
                    tmem_ld4(t0 + 152u, rx + 24);
                    tmem_wait_ld();
                    if (row < kNLD) {
#pragma unroll
                        for (int j = 0; j < 28; ++j) {
                            const int c = col0 + 28 * part + j;
                            if (c >= row && c < kNLD) {
                                const float x = __fadd_rn(__uint_as_float(rh[j]), __uint_as_float(rx[j]));
                                const float2 v = kr[c];
                                const float y = __fsub_rn(x, v.y);
                                const float t = __fadd_rn(v.x, y);
                                kr[c] = make_float2(t, __fsub_rn(__fsub_rn(t, v.x), y));
                            }
                        }
                    }
                }
                fence_before_sync();  // these reads precede the next MMAs into this pair
            } else {
                skipped = true;
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&S.acc_empty[b]));
        }
        if (skipped && lane == 0) S.dabort = 1;
        named_bar(kBarDrain, kDrainThreads);  // the element's sums are complete
        if (S.dabort) return;
        // every entry, row by row (consecutive threads -> consecutive columns of one CSR row, so the
        // reductions of a warp share cache lines); the map row (44 KB, not staged) is read
        // kScatterBatch entries per thread at a time, so a thread's loads are in flight together
        const int32_t *em = emap + e * kNLD * kNLD;
        for (int base = dt; base < kNLD * kNLD; base += kDrainThreads * kScatterBatch) {
            int32_t pp[kScatterBatch];
#pragma unroll
            for (int u = 0; u < kScatterBatch; ++u) {
                const int idx = base + u * kDrainThreads;
                pp[u] = idx < kNLD * kNLD ? em[idx] : -1;
            }
#pragma unroll
            for (int u = 0; u < kScatterBatch; ++u) {
                const int idx = base + u * kDrainThreads;
                if (pp[u] < 0) continue;
                const int a = idx / kNLD, bcol = idx - a * kNLD;
                const float2 v = bcol >= a ? S.ke[a * kKeStride + bcol] : S.ke[bcol * kKeStride + a];
                const double val = df_to_f64({v.x, -v.y});
                if (pp[u] < nnz) red_add(values + pp[u], val);
                else flag(SSP_DEV_BAD_INDEX);
            }
        }
        named_bar(kBarDrain, kDrainThreads);  // the sums are read before their owners reset them
    }
}

__global__ void __launch_bounds__(kThreads, 1) correction_tc_p4_kernel(
    const double *__restrict__ d1, const double *__restrict__ d2, const double *__restrict__ d3,
    const double *__restrict__ DS, const double *__restrict__ w, const int8_t *__restrict__ branch,
    const double *__restrict__ shear, const double *__restrict__ lame, const int32_t *__restrict__ emap, int n_elem,
    long long nnz, double scale, double *__restrict__ values, const int32_t *__restrict__ elist,
    const int32_t *__restrict__ elist_count) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    // zero both stages once: the padding rows (alpha >= 105, beta >= 105) are never written again
    for (int i = tid; i < (int)(sizeof(Stage) * 2 / 4); i += kThreads) reinterpret_cast<uint32_t *>(S.stage)[i] = 0u;
    if (tid == 0) {
        mbar_init(smem_u32(&S.stage_free[0]));
        mbar_init(smem_u32(&S.stage_free[1]));
        mbar_init(smem_u32(&S.acc_full[0]));
        mbar_init(smem_u32(&S.acc_full[1]));
        mbar_init_count(smem_u32(&S.acc_empty[0]), kDrainThreads / 32);
        mbar_init_count(smem_u32(&S.acc_empty[1]), kDrainThreads / 32);
        S.abort = S.babort = S.dabort = 0;
        mbar_init_fence();
    }
    if (warp == 0) tmem_alloc(&S.tmem_slot, kTmemCols);
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = S.tmem_slot;
    const long long n_iter = elist ? static_cast<long long>(*elist_count) : static_cast<long long>(n_elem);
    if (tid < kBuildThreads)
        build_role(S, tmem, d1, d2, d3, DS, w, branch, shear, lame, n_elem, scale, elist, n_iter);
    else
        drain_role(S, tmem, branch, emap, n_elem, nnz, values, elist, n_iter);
    // every MMA has been drained (or abandoned after a timeout)
    fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        fence_after_sync();
        tmem_dealloc(tmem, kTmemCols);
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
