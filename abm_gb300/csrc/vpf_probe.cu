// vpf_probe.cu -- throughput probes that measure the FP32 (FFMA) and MUFU (SFU) pipe peaks of
// the running GPU, the denominators of the roofline fraction reported for the VPF kernels.
#include "../../include/abm_vpf.h"
#include "vpf_host.h"

namespace abm {

// 8 independent FFMA chains per thread, `iters` rounds: 16 * iters FP32 ops per thread.
__global__ void probe_ffma_kernel(int iters, float a, float b, float *sink) {
    float r0 = threadIdx.x * 1e-7f, r1 = r0 + 1e-3f, r2 = r0 + 2e-3f, r3 = r0 + 3e-3f;
    float r4 = r0 + 4e-3f, r5 = r0 + 5e-3f, r6 = r0 + 6e-3f, r7 = r0 + 7e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            r0 = fmaf(r0, a, b); r1 = fmaf(r1, a, b); r2 = fmaf(r2, a, b); r3 = fmaf(r3, a, b);
            r4 = fmaf(r4, a, b); r5 = fmaf(r5, a, b); r6 = fmaf(r6, a, b); r7 = fmaf(r7, a, b);
        }
    }
    const float s = r0 + r1 + r2 + r3 + r4 + r5 + r6 + r7;
    if (s == 1234.5f) sink[threadIdx.x] = s;  // keeps the chains live
}

__device__ __forceinline__ float mufu_rsq(float x) {
    float r;
    asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// 8 independent MUFU.RSQ chains per thread (x -> rsqrt(x) stays near 1): 32 * iters ops.
__global__ void probe_mufu_kernel(int iters, float *sink) {
    float r0 = 1.f + threadIdx.x * 1e-7f, r1 = r0 + 1e-3f, r2 = r0 + 2e-3f, r3 = r0 + 3e-3f;
    float r4 = r0 + 4e-3f, r5 = r0 + 5e-3f, r6 = r0 + 6e-3f, r7 = r0 + 7e-3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            r0 = mufu_rsq(r0); r1 = mufu_rsq(r1); r2 = mufu_rsq(r2); r3 = mufu_rsq(r3);
            r4 = mufu_rsq(r4); r5 = mufu_rsq(r5); r6 = mufu_rsq(r6); r7 = mufu_rsq(r7);
        }
    }
    const float s = r0 + r1 + r2 + r3 + r4 + r5 + r6 + r7;
    if (s == 1234.5f) sink[threadIdx.x] = s;
}

}  // namespace abm

extern "C" int abm_probe_pipe_peak(int32_t kind, int32_t blocks, int32_t threads, int32_t iters,
                                   float *sink_dev, double *ops_out, void *stream) {
    using namespace abm;
    if (blocks <= 0 || threads <= 0 || threads > 1024 || iters <= 0 || !sink_dev || !ops_out)
        return set_error(ABM_ERR_INVALID_ARG, "abm_probe_pipe_peak: bad launch shape");
    cudaStream_t s = (cudaStream_t)stream;
    if (kind == 0) {
        probe_ffma_kernel<<<blocks, threads, 0, s>>>(iters, 0.999999f, 1e-7f, sink_dev);
        *ops_out = 64.0 * iters * (double)blocks * threads;   // 32 FFMA = 64 FP32 ops
    } else if (kind == 1) {
        probe_mufu_kernel<<<blocks, threads, 0, s>>>(iters, sink_dev);
        *ops_out = 32.0 * iters * (double)blocks * threads;
    } else {
        return set_error(ABM_ERR_INVALID_ARG, "abm_probe_pipe_peak: kind=%d", kind);
    }
    return check_cuda(cudaGetLastError(), "abm_probe_pipe_peak launch");
}
