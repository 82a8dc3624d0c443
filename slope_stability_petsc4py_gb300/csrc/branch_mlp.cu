// Learned branch proposal for the 3D return mapping.
//
// A small MLP (6 -> 32 -> 32 -> 5, ReLU) maps cheap FP32 invariants of the trial strain to one of
// the five return branches of constitutive_3D_kernel.h:116-350 (elastic, smooth face, left edge,
// right edge, apex).  In the learned return mapping the points that the exact kernel's FP32 elastic
// screen cannot settle (those near or past the yield surface) get a proposal, are binned by it, and
// the exact FP64 decision pass runs bin by bin, so each warp mostly follows one branch's checks.
// The exact kernel decides and computes every result; a wrong proposal only costs time.  The
// network is trained on the GPU
// by the kernels below (forward, backward, Adam), on (features, branch) pairs produced by the
// exact return mapping.
//
// Parameters are one FP32 vector of SSP_MLP_PARAMS values: W1[32][6], b1[32], W2[32][32], b2[32],
// W3[5][32], b3[5].  Inference rounds weights and activations to BF16 and accumulates in FP32.
#include <cuda_bf16.h>

#include "ssp_internal.cuh"
#include "tcgen05.cuh"

namespace ssp {

namespace {

constexpr int kIn = 6, kH = 32, kOut = 5;
constexpr int oW1 = 0, ob1 = oW1 + kH * kIn, oW2 = ob1 + kH, ob2 = oW2 + kH * kH, oW3 = ob2 + kH,
              ob3 = oW3 + kOut * kH, kParams = ob3 + kOut;
static_assert(kParams == SSP_MLP_PARAMS, "parameter count");

__device__ __forceinline__ float slog(float x) { return copysignf(log1pf(fabsf(x)), x); }

// Features of one point (FP32): deviatoric and volumetric trial strain measured against the
// cohesion, the Lode parameter, sin(phi) and the Lame ratio.
__device__ __forceinline__ void features(const double *E, double c_bar, double sin_phi, double shear, double lame,
                                         float *x) {
    const float t0 = (float)E[0], t1 = (float)E[1], t2 = (float)E[2];
    const float t3 = 0.5f * (float)E[3], t4 = 0.5f * (float)E[4], t5 = 0.5f * (float)E[5];
    const float I1 = t0 + t1 + t2;
    const float m = I1 * (1.0f / 3.0f);
    const float d0 = t0 - m, d1 = t1 - m, d2 = t2 - m;
    const float J2 = 0.5f * (d0 * d0 + d1 * d1 + d2 * d2) + t3 * t3 + t4 * t4 + t5 * t5;
    const float J3 = d0 * d1 * d2 + 2.0f * t3 * t4 * t5 - d0 * t4 * t4 - d1 * t5 * t5 - d2 * t3 * t3;
    const float k = (float)(2.0 * shear / fmax(c_bar, 1e-300));
    const float rJ2 = sqrtf(J2);
    float lode = J2 > 0.0f ? 2.598076211f * J3 / (J2 * rJ2) : 0.0f;
    lode = fminf(1.0f, fmaxf(-1.0f, lode));
    const float s = (float)sin_phi, lr = (float)(lame / shear);
    x[0] = slog(k * rJ2);
    x[1] = slog(k * I1);
    x[2] = slog(lr * s * k * I1);
    x[3] = lode;
    x[4] = s;
    x[5] = lr / (lr + 2.0f);
}

__global__ void features_kernel(const double *__restrict__ E, const double *__restrict__ c_bar,
                                const double *__restrict__ sin_phi, const double *__restrict__ shear,
                                const double *__restrict__ lame, int n, float *__restrict__ X) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float x[kIn];
    features(E + 6ll * p, c_bar[p], sin_phi[p], shear[p], lame[p], x);
#pragma unroll
    for (int i = 0; i < kIn; ++i) X[(long long)p * kIn + i] = x[i];
}

__device__ __forceinline__ float bf(float v) { return __bfloat162float(__float2bfloat16(v)); }

// Forward pass of one sample with parameters in shared memory.  BF16 mode rounds the weights
// (already rounded in shared memory) and every activation to BF16.
template <bool BF16>
__device__ __forceinline__ int forward_argmax(const float *P, const float *x_in) {
    float x[kIn], h1[kH], h2[kH];
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = BF16 ? bf(x_in[i]) : x_in[i];
#pragma unroll
    for (int j = 0; j < kH; ++j) {
        float a = P[ob1 + j];
#pragma unroll
        for (int i = 0; i < kIn; ++i) a = fmaf(P[oW1 + j * kIn + i], x[i], a);
        h1[j] = BF16 ? bf(fmaxf(a, 0.0f)) : fmaxf(a, 0.0f);
    }
#pragma unroll
    for (int j = 0; j < kH; ++j) {
        float a = P[ob2 + j];
#pragma unroll
        for (int i = 0; i < kH; ++i) a = fmaf(P[oW2 + j * kH + i], h1[i], a);
        h2[j] = BF16 ? bf(fmaxf(a, 0.0f)) : fmaxf(a, 0.0f);
    }
    int best = 0;
    float bz = -3.0e38f;
#pragma unroll
    for (int o = 0; o < kOut; ++o) {
        float a = P[ob3 + o];
#pragma unroll
        for (int i = 0; i < kH; ++i) a = fmaf(P[oW3 + o * kH + i], h2[i], a);
        if (a > bz) {
            bz = a;
            best = o;
        }
    }
    return best;
}

__device__ __forceinline__ void load_params(const float *__restrict__ params, float *P, bool round_bf16) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) P[i] = round_bf16 ? bf(params[i]) : params[i];
    __syncthreads();
}

__global__ void predict_kernel(const float *__restrict__ params, const float *__restrict__ X, int n, int bf16,
                               int8_t *__restrict__ pred) {
    __shared__ float P[kParams];
    load_params(params, P, bf16 != 0);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float x[kIn];
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = X[(long long)p * kIn + i];
    pred[p] = static_cast<int8_t>(bf16 ? forward_argmax<true>(P, x) : forward_argmax<false>(P, x));
}

// Loss and parameter gradient of a batch (softmax cross-entropy, summed over samples).  A block
// handles TILE samples: each thread runs its sample forward and backward and leaves the
// activations and their gradients in shared memory; the block then reduces the outer products
// into the parameter gradient and adds its partial sums to grad with FP32 atomics.
constexpr int TILE = 128;
struct TileBuf {
    float x[TILE][kIn];
    float h1[TILE][kH];
    float h2[TILE][kH];
    float g1[TILE][kH];   // dLoss/d(pre-activation 1)
    float g2[TILE][kH];   // dLoss/d(pre-activation 2)
    float g3[TILE][kOut]; // dLoss/d(logits)
};

__global__ void __launch_bounds__(TILE) loss_grad_kernel(const float *__restrict__ params,
                                                         const float *__restrict__ X,
                                                         const int8_t *__restrict__ labels, int n,
                                                         float *__restrict__ grad, float *__restrict__ loss_sum,
                                                         int *__restrict__ correct) {
    __shared__ float P[kParams];
    extern __shared__ __align__(16) unsigned char tile_raw[];
    TileBuf &T = *reinterpret_cast<TileBuf *>(tile_raw);
    load_params(params, P, false);
    const int tid = threadIdx.x;
    const long long s = (long long)blockIdx.x * TILE + tid;
    float loss = 0.0f;
    int ok = 0;
    if (s < n) {
        float *x = T.x[tid], *h1 = T.h1[tid], *h2 = T.h2[tid];
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = X[s * kIn + i];
        for (int j = 0; j < kH; ++j) {
            float a = P[ob1 + j];
#pragma unroll
            for (int i = 0; i < kIn; ++i) a = fmaf(P[oW1 + j * kIn + i], x[i], a);
            h1[j] = fmaxf(a, 0.0f);
        }
        for (int j = 0; j < kH; ++j) {
            float a = P[ob2 + j];
            for (int i = 0; i < kH; ++i) a = fmaf(P[oW2 + j * kH + i], h1[i], a);
            h2[j] = fmaxf(a, 0.0f);
        }
        float z[kOut], zmax = -3.0e38f;
        int arg = 0;
        for (int o = 0; o < kOut; ++o) {
            float a = P[ob3 + o];
            for (int i = 0; i < kH; ++i) a = fmaf(P[oW3 + o * kH + i], h2[i], a);
            z[o] = a;
            if (a > zmax) {
                zmax = a;
                arg = o;
            }
        }
        float se = 0.0f;
        for (int o = 0; o < kOut; ++o) se += expf(z[o] - zmax);
        int y = labels[s];
        if (y < 0 || y >= kOut) {  // not a branch code: counted as class 0 and reported
            flag(SSP_DEV_BAD_INDEX);
            y = 0;
        }
        loss = logf(se) + zmax - z[y];
        ok = (arg == y);
        for (int o = 0; o < kOut; ++o) T.g3[tid][o] = expf(z[o] - zmax) / se - (o == y ? 1.0f : 0.0f);
        for (int i = 0; i < kH; ++i) {
            float a = 0.0f;
            for (int o = 0; o < kOut; ++o) a = fmaf(P[oW3 + o * kH + i], T.g3[tid][o], a);
            T.g2[tid][i] = h2[i] > 0.0f ? a : 0.0f;
        }
        for (int i = 0; i < kH; ++i) {
            float a = 0.0f;
            for (int j = 0; j < kH; ++j) a = fmaf(P[oW2 + j * kH + i], T.g2[tid][j], a);
            T.g1[tid][i] = h1[i] > 0.0f ? a : 0.0f;
        }
    } else {
        for (int i = 0; i < kIn; ++i) T.x[tid][i] = 0.0f;
        for (int i = 0; i < kH; ++i) T.h1[tid][i] = T.h2[tid][i] = T.g1[tid][i] = T.g2[tid][i] = 0.0f;
        for (int o = 0; o < kOut; ++o) T.g3[tid][o] = 0.0f;
    }
    // block sums of loss and hits
    for (int off = 16; off > 0; off >>= 1) {
        loss += __shfl_down_sync(0xffffffffu, loss, off);
        ok += __shfl_down_sync(0xffffffffu, ok, off);
    }
    if ((tid & 31) == 0) {
        atomicAdd(loss_sum, loss);
        atomicAdd(correct, ok);
    }
    __syncthreads();
    // parameter gradient: outer products summed over the tile
    for (int k = tid; k < kParams; k += TILE) {
        float a = 0.0f;
        if (k < ob1) {
            const int j = k / kIn, i = k % kIn;
            for (int t = 0; t < TILE; ++t) a = fmaf(T.g1[t][j], T.x[t][i], a);
        } else if (k < oW2) {
            const int j = k - ob1;
            for (int t = 0; t < TILE; ++t) a += T.g1[t][j];
        } else if (k < ob2) {
            const int j = (k - oW2) / kH, i = (k - oW2) % kH;
            for (int t = 0; t < TILE; ++t) a = fmaf(T.g2[t][j], T.h1[t][i], a);
        } else if (k < oW3) {
            const int j = k - ob2;
            for (int t = 0; t < TILE; ++t) a += T.g2[t][j];
        } else if (k < ob3) {
            const int o = (k - oW3) / kH, i = (k - oW3) % kH;
            for (int t = 0; t < TILE; ++t) a = fmaf(T.g3[t][o], T.h2[t][i], a);
        } else {
            const int o = k - ob3;
            for (int t = 0; t < TILE; ++t) a += T.g3[t][o];
        }
        atomicAdd(grad + k, a);
    }
}

__global__ void adam_kernel(float *__restrict__ params, const float *__restrict__ grad, float *__restrict__ m,
                            float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2,
                            float gscale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = grad[i] * gscale;
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// The network on the tensor cores: a CTA of 128 threads takes tiles of 128 points; each layer is
// one tcgen05.mma kind::f16 chain (BF16 operands in shared memory, FP32 accumulator in tensor
// memory): [128 x 16] x [16 x 32] (the 6 features, zero-padded), [128 x 32] x [32 x 32],
// [128 x 32] x [32 x 16] (5 logits, zero-padded).  Thread t owns point row t: it writes its
// operand row, and after each MMA reads its accumulator row (tcgen05.ld, lane t), adds the bias,
// applies ReLU and rounds to BF16 for the next layer.  The same BF16 rounding of weights and
// activations as forward_argmax<true>; the accumulation order is the tensor core's.
// FROM_LIST: the points listed by the binned return mapping's screen (count scratch[0], indices
// from scratch + 4), features from their trial strain, each point appended to the list of its
// proposed branch (counts at scratch + 4 + 3 n, lists of n entries from scratch + 12 + 3 n);
// otherwise features from X and the argmax stored in pred.
constexpr int kTcTile = 128, kTcCols = 64;  // layer 1 -> columns 0-31, layer 2 -> 32-63, layer 3 -> 0-15
struct MlpSmem {
    alignas(128) unsigned char w1[32 * 16 * 2];
    alignas(128) unsigned char w2[32 * 32 * 2];
    alignas(128) unsigned char w3[16 * 32 * 2];
    alignas(128) unsigned char a1[kTcTile * 16 * 2];
    alignas(128) unsigned char a2[kTcTile * 32 * 2];
    alignas(128) unsigned char a3[kTcTile * 32 * 2];
    float b1[kH], b2[kH], b3[8];
    unsigned long long mbar;
    uint32_t tmem_slot;
    int abort;
};
// more than a ninth of an SM's 228 KB of shared memory, so at most eight CTAs (8 x 64 tensor-memory
// columns, all of the SM's 512) are resident on an SM and every allocation succeeds at once
constexpr size_t kMlpSmemBytes = 26 * 1024;
static_assert(sizeof(MlpSmem) <= kMlpSmemBytes, "MLP shared memory");

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}
// One row of 8 * chunks BF16 values (from v) into the K-major tile at row r.
template <int CHUNKS>
__device__ __forceinline__ void store_row_bf16(unsigned char *tile, int r, const float *v) {
#pragma unroll
    for (int c = 0; c < CHUNKS; ++c) {
        uint4 q;
        q.x = pack_bf16(v[8 * c + 0], v[8 * c + 1]);
        q.y = pack_bf16(v[8 * c + 2], v[8 * c + 3]);
        q.z = pack_bf16(v[8 * c + 4], v[8 * c + 5]);
        q.w = pack_bf16(v[8 * c + 6], v[8 * c + 7]);
        *reinterpret_cast<uint4 *>(tile + tc::kmaj_off<2>(r, 8 * c, kTcTile)) = q;
    }
}
// Issue one layer (K / 16 MMAs), commit, wait for it (bounded; on expiry flag and return false).
__device__ __forceinline__ bool mlp_layer(MlpSmem &S, const unsigned char *a, const unsigned char *b, int n_rows_b,
                                          int K, uint32_t tmem_d, uint32_t id, uint32_t &phase) {
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        const uint32_t lbo_a = (kTcTile / 8) * 128, lbo_b = (n_rows_b / 8) * 128;
        for (int s = 0; s < K / 16; ++s)
            tc::mma_f16(tmem_d, tc::smem_desc(tc::smem_u32(a) + s * 2 * lbo_a, lbo_a, 128),
                        tc::smem_desc(tc::smem_u32(b) + s * 2 * lbo_b, lbo_b, 128), id, s != 0 ? 1u : 0u);
        tc::mma_commit(tc::smem_u32(&S.mbar));
    }
    if (!tc::mbar_wait(tc::smem_u32(&S.mbar), phase)) {
        S.abort = 1;
        flag(SSP_DEV_TIMEOUT);
    }
    phase ^= 1u;
    __syncthreads();  // every thread leaves on the same decision
    tc::fence_after_sync();
    return S.abort == 0;
}

template <bool FROM_LIST>
__global__ void __launch_bounds__(kTcTile, 8) mlp_tc_kernel(const float *__restrict__ params, const float *__restrict__ X,
                                                         const double *__restrict__ E,
                                                         const double *__restrict__ c_bar,
                                                         const double *__restrict__ sin_phi,
                                                         const double *__restrict__ shear,
                                                         const double *__restrict__ lame, int n,
                                                         int8_t *__restrict__ pred, int32_t *__restrict__ scratch) {
    extern __shared__ __align__(128) unsigned char mlp_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(mlp_raw);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // weights as BF16 B operands (N x K, K-major), zero-padded; biases as FP32
    for (int i = tid; i < 32 * 16; i += kTcTile) {
        const int nn = i / 16, k = i % 16;
        *reinterpret_cast<__nv_bfloat16 *>(S.w1 + tc::kmaj_off<2>(nn, k, 32)) =
            __float2bfloat16_rn(k < kIn ? params[oW1 + nn * kIn + k] : 0.0f);
    }
    for (int i = tid; i < 32 * 32; i += kTcTile) {
        const int nn = i / 32, k = i % 32;
        *reinterpret_cast<__nv_bfloat16 *>(S.w2 + tc::kmaj_off<2>(nn, k, 32)) = __float2bfloat16_rn(params[oW2 + i]);
    }
    for (int i = tid; i < 16 * 32; i += kTcTile) {
        const int nn = i / 32, k = i % 32;
        *reinterpret_cast<__nv_bfloat16 *>(S.w3 + tc::kmaj_off<2>(nn, k, 16)) =
            __float2bfloat16_rn(nn < kOut ? params[oW3 + nn * kH + k] : 0.0f);
    }
    if (tid < kH) {
        S.b1[tid] = params[ob1 + tid];
        S.b2[tid] = params[ob2 + tid];
    }
    if (tid < 8) S.b3[tid] = tid < kOut ? params[ob3 + tid] : 0.0f;
    if (tid == 0) {
        tc::mbar_init(tc::smem_u32(&S.mbar));
        S.abort = 0;
        tc::mbar_init_fence();
    }
    if (warp == 0) tc::tmem_alloc(&S.tmem_slot, kTcCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem_slot;
    const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
    constexpr uint32_t id32 = tc::idesc(tc::kFmtBF16, kTcTile, 32), id16 = tc::idesc(tc::kFmtBF16, kTcTile, 16);
    uint32_t phase = 0;
    const int cnt = FROM_LIST ? scratch[0] : n;
    const int tiles = (cnt + kTcTile - 1) / kTcTile;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int i_item = tile * kTcTile + tid;
        int p = i_item < cnt ? i_item : -1;
        if (FROM_LIST && p >= 0) {
            p = scratch[4 + p];
            if (p < 0 || p >= n) {
                flag(SSP_DEV_BAD_INDEX);
                p = -1;
            }
        }
        float v[32];
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = 0.0f;
        if (p >= 0) {
            if (FROM_LIST) {
                features(E + 6ll * p, c_bar[p], sin_phi[p], shear[p], lame[p], v);
            } else {
#pragma unroll
                for (int i = 0; i < kIn; ++i) v[i] = X[(long long)p * kIn + i];
            }
        }
        store_row_bf16<2>(S.a1, tid, v);
        if (!mlp_layer(S, S.a1, S.w1, 32, 16, tmem, id32, phase)) break;
        {
            uint32_t r[32];
            tc::tmem_ld16(tmem + lane_base, r);
            tc::tmem_ld16(tmem + lane_base + 16, r + 16);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = fmaxf(__uint_as_float(r[j]) + S.b1[j], 0.0f);
        }
        store_row_bf16<4>(S.a2, tid, v);
        if (!mlp_layer(S, S.a2, S.w2, 32, 32, tmem + 32, id32, phase)) break;
        {
            uint32_t r[32];
            tc::tmem_ld16(tmem + lane_base + 32, r);
            tc::tmem_ld16(tmem + lane_base + 48, r + 16);
            tc::tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = fmaxf(__uint_as_float(r[j]) + S.b2[j], 0.0f);
        }
        store_row_bf16<4>(S.a3, tid, v);
        // layer 1's accumulator columns are free again: every thread has read them
        if (!mlp_layer(S, S.a3, S.w3, 16, 32, tmem, id16, phase)) break;
        int best = 0;
        {
            uint32_t r[16];
            tc::tmem_ld16(tmem + lane_base, r);
            tc::tmem_wait_ld();
            float bz = -3.0e38f;
#pragma unroll
            for (int o = 0; o < kOut; ++o) {
                const float a = __uint_as_float(r[o]) + S.b3[o];
                if (a > bz) {
                    bz = a;
                    best = o;
                }
            }
        }
        if (FROM_LIST) {
            const int b = p >= 0 ? best : -1;
            int32_t *counts = scratch + 4 + 3ll * n, *lists = scratch + 12 + 3ll * n;
#pragma unroll
            for (int k = 0; k < kOut; ++k) {
                const unsigned mask = __ballot_sync(0xffffffffu, b == k);
                if (mask == 0u) continue;
                const int leader = __ffs(mask) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(counts + k, __popc(mask));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (b == k) lists[(long long)k * n + base + __popc(mask & ((1u << lane) - 1u))] = p;
            }
        } else if (p >= 0) {
            pred[p] = static_cast<int8_t>(best);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, kTcCols);
    }
}

template <bool FROM_LIST>
int launch_mlp_tc(const float *params, const float *X, const double *E, const double *c_bar, const double *sin_phi,
                  const double *shear, const double *lame, int n, int8_t *pred, int32_t *scratch, cudaStream_t st) {
    auto kernel = mlp_tc_kernel<FROM_LIST>;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kMlpSmemBytes)) !=
        cudaSuccess)
        return SSP_ERR_CUDA;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)sms * 8;
    const long long tiles = (n + kTcTile - 1) / kTcTile;
    if (grid > tiles) grid = tiles;
    kernel<<<static_cast<unsigned>(grid), kTcTile, kMlpSmemBytes, st>>>(params, X, E, c_bar, sin_phi, shear, lame, n, pred,
                                                                        scratch);
    return launch_status();
}

// The trivial predictor beside the network: each point listed by pass A goes to the bin of a given
// branch code (the previous Newton iteration's, for instance); codes outside 0..4 go to bin 0.
// Same list layout as the network's proposal (five lists of stride n after the 8 counters).
__global__ void __launch_bounds__(256) propose_given_kernel(const int8_t *__restrict__ proposal, int n,
                                                            int32_t *__restrict__ scratch) {
    const int cnt = scratch[0];
    const int32_t *listed = scratch + 4;
    int32_t *counts = scratch + 4 + 3ll * n, *lists = scratch + 12 + 3ll * n;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    const int iters = (cnt + stride - 1) / stride;
    for (int it = 0; it < iters; ++it) {  // whole warps iterate together (the appends are warp-collective)
        const int i = it * stride + blockIdx.x * blockDim.x + threadIdx.x;
        int p = -1, b = -1;
        if (i < cnt) {
            p = listed[i];
            if (p < 0 || p >= n) {
                flag(SSP_DEV_BAD_INDEX);
                p = -1;
            } else {
                b = proposal[p];
                if (b < 0 || b >= kOut) b = 0;
            }
        }
#pragma unroll
        for (int k = 0; k < kOut; ++k) {
            const unsigned mask = __ballot_sync(0xffffffffu, b == k);
            if (mask == 0u) continue;
            const int leader = __ffs(mask) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(counts + k, __popc(mask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (b == k) lists[(long long)k * n + base + __popc(mask & ((1u << lane) - 1u))] = p;
        }
    }
}

// Pass A, the given codes' bins for its listed points, then passes B (over the five bins) and C.
int proposed_return_mapping(const int8_t *proposal, const double *E, const double *c_bar, const double *sin_phi,
                            const double *shear, const double *lame, int n_int, double *S_out, double *DS_out,
                            int8_t *branch_out, int32_t *scratch, bool compensated_ds, cudaStream_t st,
                            bool write_elastic_ds = true) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!proposal || !E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    if (proposal == branch_out) return SSP_ERR_INVALID;  // pass A overwrites the codes it reads
    int32_t *counts = scratch + 4 + 3ll * n_int, *lists = scratch + 12 + 3ll * n_int;
    if (cudaMemsetAsync(counts, 0, 8 * sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    int rc = binned_screen(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, st,
                           write_elastic_ds);
    if (rc != SSP_OK) return rc;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)sms * 8;
    const long long need = (n_int + 255) / 256;
    if (grid > need) grid = need;
    propose_given_kernel<<<static_cast<unsigned>(grid), 256, 0, st>>>(proposal, n_int, scratch);
    rc = launch_status();
    if (rc != SSP_OK) return rc;
    return binned_decide_finish(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, lists,
                                counts, kOut, n_int, compensated_ds, st);
}

// Pass A of the binned return mapping, the proposal for its listed points, then passes B (over
// the five proposal bins) and C.
int learned_return_mapping(const float *params, const double *E, const double *c_bar, const double *sin_phi,
                           const double *shear, const double *lame, int n_int, double *S_out, double *DS_out,
                           int8_t *branch_out, int32_t *scratch, bool compensated_ds, cudaStream_t st,
                           bool write_elastic_ds = true) {
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!params || !E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    int32_t *counts = scratch + 4 + 3ll * n_int, *lists = scratch + 12 + 3ll * n_int;
    if (cudaMemsetAsync(counts, 0, 8 * sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    int rc = binned_screen(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, st,
                           write_elastic_ds);
    if (rc != SSP_OK) return rc;
    rc = launch_mlp_tc<true>(params, nullptr, E, c_bar, sin_phi, shear, lame, n_int, nullptr, scratch, st);
    if (rc != SSP_OK) return rc;
    return binned_decide_finish(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, lists,
                                counts, kOut, n_int, compensated_ds, st);
}

}  // namespace
}  // namespace ssp

using namespace ssp;

extern "C" {

int ssp_branch_features(const double *E, const double *c_bar, const double *sin_phi, const double *shear,
                        const double *lame, int n, float *X, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!E || !c_bar || !sin_phi || !shear || !lame || !X) return SSP_ERR_INVALID;
    features_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(E, c_bar, sin_phi, shear, lame, n, X);
    return launch_status();
}

int ssp_mlp_predict(const float *params, const float *X, int n, int mode, int8_t *pred, void *stream) {
    if (n < 0 || mode < 0 || mode > 2) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!params || !X || !pred) return SSP_ERR_INVALID;
    if (mode == 2)
        return launch_mlp_tc<false>(params, X, nullptr, nullptr, nullptr, nullptr, nullptr, n, pred, nullptr,
                                    as_stream(stream));
    predict_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(params, X, n, mode, pred);
    return launch_status();
}

int ssp_mlp_loss_grad(const float *params, const float *X, const int8_t *labels, int n, float *grad,
                      float *loss_sum, int *correct, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (!params || !grad || !loss_sum || !correct || (n > 0 && (!X || !labels))) return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(grad, 0, sizeof(float) * kParams, st) != cudaSuccess ||
        cudaMemsetAsync(loss_sum, 0, sizeof(float), st) != cudaSuccess ||
        cudaMemsetAsync(correct, 0, sizeof(int), st) != cudaSuccess)
        return SSP_ERR_CUDA;
    if (n == 0) return SSP_OK;
    const size_t smem = sizeof(TileBuf);
    if (cudaFuncSetAttribute(loss_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SSP_ERR_CUDA;
    loss_grad_kernel<<<grid_for(n, TILE), TILE, smem, st>>>(params, X, labels, n, grad, loss_sum, correct);
    return launch_status();
}

int ssp_mlp_adam(float *params, const float *grad, float *m, float *v, int step, float lr, float beta1, float beta2,
                 float eps, float grad_scale, void *stream) {
    if (step < 1 || !params || !grad || !m || !v) return SSP_ERR_INVALID;
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<grid_for(kParams, 256), 256, 0, as_stream(stream)>>>(params, grad, m, v, kParams, lr, beta1, beta2, eps,
                                                                      c1, c2, grad_scale);
    return launch_status();
}

int ssp_constitutive_3d_sds_learned(const float *params, const double *E, const double *c_bar,
                                    const double *sin_phi, const double *shear, const double *lame, int n_int,
                                    double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                    void *stream) {
    return learned_return_mapping(params, E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch,
                                  false, as_stream(stream));
}

int ssp_constitutive_3d_sds_proposed(const int8_t *proposal, const double *E, const double *c_bar,
                                     const double *sin_phi, const double *shear, const double *lame, int n_int,
                                     double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                     void *stream) {
    return proposed_return_mapping(proposal, E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out,
                                   scratch, false, as_stream(stream));
}

int ssp_constitutive_3d_sds_proposed_mixed(const int8_t *proposal, const double *E, const double *c_bar,
                                           const double *sin_phi, const double *shear, const double *lame, int n_int,
                                           double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                           void *stream) {
    return proposed_return_mapping(proposal, E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out,
                                   scratch, true, as_stream(stream));
}

int ssp_constitutive_3d_sds_screened(const double *E, const double *c_bar, const double *sin_phi,
                                     const double *shear, const double *lame, int n_int, double *S_out,
                                     double *DS_out, int8_t *branch_out, int32_t *scratch, int bins,
                                     const void *bin_source, int options, void *stream) {
    if (n_int < 0 || (options & ~(SSP_RM_COMPENSATED_DS | SSP_RM_PLASTIC_DS_ONLY)) != 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    const bool comp = (options & SSP_RM_COMPENSATED_DS) != 0;
    const bool write_el = (options & SSP_RM_PLASTIC_DS_ONLY) == 0;
    cudaStream_t st = as_stream(stream);
    switch (bins) {
    case SSP_BINS_EXACT: {
        if (!E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
            return SSP_ERR_INVALID;
        const int rc = binned_screen(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch, st,
                                     write_el);
        if (rc != SSP_OK) return rc;
        return binned_decide_finish(E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch,
                                    scratch + 4, scratch, 1, 0, comp, st);
    }
    case SSP_BINS_LEARNED:
        return learned_return_mapping(static_cast<const float *>(bin_source), E, c_bar, sin_phi, shear, lame, n_int,
                                      S_out, DS_out, branch_out, scratch, comp, st, write_el);
    case SSP_BINS_GIVEN:
        return proposed_return_mapping(static_cast<const int8_t *>(bin_source), E, c_bar, sin_phi, shear, lame, n_int,
                                       S_out, DS_out, branch_out, scratch, comp, st, write_el);
    default:
        return SSP_ERR_INVALID;
    }
}

int ssp_constitutive_3d_sds_learned_mixed(const float *params, const double *E, const double *c_bar,
                                          const double *sin_phi, const double *shear, const double *lame, int n_int,
                                          double *S_out, double *DS_out, int8_t *branch_out, int32_t *scratch,
                                          void *stream) {
    return learned_return_mapping(params, E, c_bar, sin_phi, shear, lame, n_int, S_out, DS_out, branch_out, scratch,
                                  true, as_stream(stream));
}

}  // extern "C"
