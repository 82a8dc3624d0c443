// Measurement probe (not part of the product library): a stream of independent FP64 fused
// multiply-adds, used by the benchmark to measure the FP64 issue rate of the device the hot path
// runs on (the denominator of its FP64 roofline).  Built into _build/libssp_fp64_probe.so.
#include "../ssp_internal.cuh"

namespace ssp {
namespace {

__global__ void dfma_probe_kernel(int iters, double seed, double *__restrict__ out) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + 1e-3 * (threadIdx.x + k);
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace ssp

extern "C" int ssp_probe_dfma(int iters, int blocks, int threads, double *out, void *stream) {
    if (iters <= 0 || blocks <= 0 || threads <= 0 || threads > 1024 || !out) return SSP_ERR_INVALID;
    ssp::dfma_probe_kernel<<<blocks, threads, 0, ssp::as_stream(stream)>>>(iters, 1.0, out);
    return ssp::launch_status();
}
