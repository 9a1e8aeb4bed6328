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

// The same with packed FP32x2 FMAs (FFMA2): 8 chains of float2, 32 * iters FP32 FMAs.
__global__ void probe_ffma2_kernel(int iters, float a, float b, float *sink) {
    const float2 A = make_float2(a, a), B = make_float2(b, b);
    float2 r0 = make_float2(threadIdx.x * 1e-7f, 1e-4f), r1 = make_float2(1e-3f, 2e-3f);
    float2 r2 = make_float2(3e-3f, 4e-3f), r3 = make_float2(5e-3f, 6e-3f);
    float2 r4 = make_float2(7e-3f, 8e-3f), r5 = make_float2(9e-3f, 1e-2f);
    float2 r6 = make_float2(1.1e-2f, 1.2e-2f), r7 = make_float2(1.3e-2f, 1.4e-2f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            r0 = __ffma2_rn(r0, A, B); r1 = __ffma2_rn(r1, A, B); r2 = __ffma2_rn(r2, A, B);
            r3 = __ffma2_rn(r3, A, B); r4 = __ffma2_rn(r4, A, B); r5 = __ffma2_rn(r5, A, B);
            r6 = __ffma2_rn(r6, A, B); r7 = __ffma2_rn(r7, A, B);
        }
    }
    const float s = r0.x + r1.x + r2.x + r3.x + r4.x + r5.x + r6.x + r7.x + r0.y + r1.y + r2.y +
                    r3.y + r4.y + r5.y + r6.y + r7.y;
    if (s == 1234.5f) sink[threadIdx.x] = s;
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
    } else if (kind == 2) {
        probe_ffma2_kernel<<<blocks, threads, 0, s>>>(iters, 0.999999f, 1e-7f, sink_dev);
        *ops_out = 128.0 * iters * (double)blocks * threads;  // 32 FFMA2 = 64 FMAs
    } else if (kind == 1) {
        probe_mufu_kernel<<<blocks, threads, 0, s>>>(iters, sink_dev);
        *ops_out = 32.0 * iters * (double)blocks * threads;
    } else {
        return set_error(ABM_ERR_INVALID_ARG, "abm_probe_pipe_peak: kind=%d", kind);
    }
    return check_cuda(cudaGetLastError(), "abm_probe_pipe_peak launch");
}
