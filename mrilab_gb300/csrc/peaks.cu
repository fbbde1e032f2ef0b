// FP32 / MUFU throughput probes (libmrl_peaks.so, used by bench.py only).
//
// The roofline denominators for the scan kernels are the FP32 pipe (FFMA)
// and the multi-function unit (sin/cos/ex2/rsqrt); the driver-measured
// peaks cover HBM and bf16 tensor throughput only, so these two are
// measured here on the same GPU: independent FFMA chains (scalar and packed
// f32x2) and MUFU sin chains across every SM, timed with CUDA events.
#include <cuda_runtime.h>

namespace {

__global__ void ffma_probe(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    if (x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7 == 12345.f) out[0] = x0;
}

// the same chains with packed two-lane FMA (fma.rn.f32x2, 4 flops each)
__global__ void ffma2_probe(float *out, int iters, float a, float b) {
    const float2 av = make_float2(a, a), bv = make_float2(b, b);
    float2 x0 = make_float2(threadIdx.x * 1e-3f, threadIdx.x * 2e-3f);
    float2 x1 = make_float2(x0.x + 1.f, x0.y + 1.f), x2 = make_float2(x0.x + 2.f, x0.y + 2.f);
    float2 x3 = make_float2(x0.x + 3.f, x0.y + 3.f), x4 = make_float2(x0.x + 4.f, x0.y + 4.f);
    float2 x5 = make_float2(x0.x + 5.f, x0.y + 5.f), x6 = make_float2(x0.x + 6.f, x0.y + 6.f);
    float2 x7 = make_float2(x0.x + 7.f, x0.y + 7.f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = __ffma2_rn(x0, av, bv); x1 = __ffma2_rn(x1, av, bv); x2 = __ffma2_rn(x2, av, bv);
            x3 = __ffma2_rn(x3, av, bv); x4 = __ffma2_rn(x4, av, bv); x5 = __ffma2_rn(x5, av, bv);
            x6 = __ffma2_rn(x6, av, bv); x7 = __ffma2_rn(x7, av, bv);
        }
    }
    const float s = x0.x + x1.x + x2.x + x3.x + x4.x + x5.x + x6.x + x7.x + x0.y + x1.y + x2.y + x3.y + x4.y +
                    x5.y + x6.y + x7.y;
    if (s == 12345.f) out[0] = s;
}

__global__ void mufu_probe(float *out, int iters) {
    float x0 = threadIdx.x * 1e-3f, x1 = x0 + .1f, x2 = x0 + .2f, x3 = x0 + .3f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 16; ++k) {
            x0 = __sinf(x0); x1 = __sinf(x1); x2 = __sinf(x2); x3 = __sinf(x3);
        }
    }
    if (x0 + x1 + x2 + x3 == 12345.f) out[0] = x0;
}

}  // namespace

extern "C" {

// Measured FFMA throughput in FP32 TFLOP/s (2 flops per FFMA) and MUFU
// throughput in Gop/s on the current device; returns 0 on success.
int mrl_probe_peaks(double *fp32_tflops, double *mufu_gops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 4096;
    ffma_probe<<<blocks, threads>>>(out, 64, 0.999f, 1e-3f);  // warm-up
    cudaEventRecord(e0);
    ffma_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *fp32_tflops = (double)blocks * threads * iters * 16 * 8 * 2 / (ms * 1e-3) / 1e12;
    mufu_probe<<<blocks, threads>>>(out, 64);
    cudaEventRecord(e0);
    mufu_probe<<<blocks, threads>>>(out, iters / 4);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    *mufu_gops = (double)blocks * threads * (iters / 4) * 16 * 4 / (ms * 1e-3) / 1e9;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

// Measured packed FFMA (f32x2) throughput in FP32 TFLOP/s (4 flops per
// instruction) on the current device; returns 0 on success.
int mrl_probe_ffma2(double *fp32x2_tflops) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    float *out = nullptr;
    if (cudaMalloc(&out, sizeof(float)) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256, iters = 2048;
    ffma2_probe<<<blocks, threads>>>(out, 64, 0.999f, 1e-3f);  // warm-up
    cudaEventRecord(e0);
    ffma2_probe<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    *fp32x2_tflops = (double)blocks * threads * iters * 16 * 8 * 4 / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // extern "C"
