// Learned branch proposal for the 3D return mapping.
//
// A small MLP (6 -> 32 -> 32 -> 5, ReLU) maps cheap FP32 invariants of the trial strain to one of
// the five return branches of constitutive_3D_kernel.h:116-350 (elastic, smooth face, left edge,
// right edge, apex).  Points are binned by the proposed branch and the exact FP64 return mapping
// then runs bin by bin, so each warp mostly executes one branch's code.  The exact kernel decides
// and computes every result; a wrong proposal only costs time.  The network is trained on the GPU
// by the kernels below (forward, backward, Adam), on (features, branch) pairs produced by the
// exact return mapping.
//
// Parameters are one FP32 vector of SSP_MLP_PARAMS values: W1[32][6], b1[32], W2[32][32], b2[32],
// W3[5][32], b3[5].  Inference rounds weights and activations to BF16 and accumulates in FP32.
#include <cuda_bf16.h>

#include "ssp_internal.cuh"

namespace ssp {

// defined in constitutive.cu
__device__ int mc3d_point_ext(const double *E, double c_bar, double sin_phi, double shear, double lame, double *S,
                              double *DS);

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

// Proposal + binning: features, BF16 MLP, argmax, and a warp-aggregated append of the point to
// the list of its proposed branch.  scratch = 8 counters, then five lists of n entries.
__global__ void __launch_bounds__(128) propose_bin_kernel(const float *__restrict__ params,
                                                          const double *__restrict__ E,
                                                          const double *__restrict__ c_bar,
                                                          const double *__restrict__ sin_phi,
                                                          const double *__restrict__ shear,
                                                          const double *__restrict__ lame, int n,
                                                          int32_t *__restrict__ scratch) {
    __shared__ float P[kParams];
    load_params(params, P, true);
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    int b = -1;
    if (p < n) {
        float x[kIn];
        features(E + 6ll * p, c_bar[p], sin_phi[p], shear[p], lame[p], x);
        b = forward_argmax<true>(P, x);
    }
    const unsigned lane = threadIdx.x & 31u;
    int32_t *lists = scratch + 8;
#pragma unroll
    for (int k = 0; k < kOut; ++k) {
        const unsigned mask = __ballot_sync(0xffffffffu, b == k);
        if (mask == 0u) continue;
        const int leader = __ffs(mask) - 1;
        int base = 0;
        if ((int)lane == leader) base = atomicAdd(scratch + k, __popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (b == k) lists[(long long)k * n + base + __popc(mask & ((1u << lane) - 1u))] = p;
    }
}

// The exact FP64 return mapping over the five proposal lists (blockIdx.y = list).
__global__ void __launch_bounds__(128) exact_over_bins_kernel(const double *__restrict__ E,
                                                              const double *__restrict__ c_bar,
                                                              const double *__restrict__ sin_phi,
                                                              const double *__restrict__ shear,
                                                              const double *__restrict__ lame, int n,
                                                              double *__restrict__ S, double *__restrict__ DS,
                                                              int8_t *__restrict__ branch,
                                                              const int32_t *__restrict__ scratch) {
    const int k = blockIdx.y;
    const int cnt = scratch[k];
    const int32_t *list = scratch + 8 + (long long)k * n;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int p = list[i];
        if (p < 0 || p >= n) {
            flag(SSP_DEV_BAD_INDEX);
            continue;
        }
        double e[6], s[6], ds[36];
#pragma unroll
        for (int j = 0; j < 6; ++j) e[j] = E[6ll * p + j];
        const int b = mc3d_point_ext(e, c_bar[p], sin_phi[p], shear[p], lame[p], s, ds);
        double2 *S2 = reinterpret_cast<double2 *>(S + 6ll * p);
#pragma unroll
        for (int j = 0; j < 3; ++j) S2[j] = make_double2(s[2 * j], s[2 * j + 1]);
        double2 *D2 = reinterpret_cast<double2 *>(DS + 36ll * p);
#pragma unroll
        for (int j = 0; j < 18; ++j) D2[j] = make_double2(ds[2 * j], ds[2 * j + 1]);
        branch[p] = static_cast<int8_t>(b);
    }
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

int ssp_mlp_predict(const float *params, const float *X, int n, int bf16, int8_t *pred, void *stream) {
    if (n < 0) return SSP_ERR_INVALID;
    if (n == 0) return SSP_OK;
    if (!params || !X || !pred) return SSP_ERR_INVALID;
    predict_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(params, X, n, bf16, pred);
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
    if (n_int < 0) return SSP_ERR_INVALID;
    if (n_int == 0) return SSP_OK;
    if (!params || !E || !c_bar || !sin_phi || !shear || !lame || !S_out || !DS_out || !branch_out || !scratch)
        return SSP_ERR_INVALID;
    cudaStream_t st = as_stream(stream);
    if (cudaMemsetAsync(scratch, 0, 8 * sizeof(int32_t), st) != cudaSuccess) return SSP_ERR_CUDA;
    propose_bin_kernel<<<grid_for(n_int, 128), 128, 0, st>>>(params, E, c_bar, sin_phi, shear, lame, n_int, scratch);
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long gx = (long long)sms * 8;
    const long long need = (n_int + 127) / 128;
    if (gx > need) gx = need;
    exact_over_bins_kernel<<<dim3(static_cast<unsigned>(gx), kOut), 128, 0, st>>>(E, c_bar, sin_phi, shear, lame, n_int,
                                                                                   S_out, DS_out, branch_out, scratch);
    return launch_status();
}

}  // extern "C"
