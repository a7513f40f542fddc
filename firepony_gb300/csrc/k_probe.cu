// FP32 SIMT throughput probe: the roofline denominator of the FP32 BAQ HMM, measured on the device it runs on
// instead of assumed. Every thread runs 8 independent multiply-add chains (scalar fmaf, or the packed
// two-lane __ffma2_rn), one resident grid of SMs x 8 blocks x 256 threads, timed with CUDA events. No
// reference counterpart (a measurement utility of this engine).
#include <cuda_runtime.h>

#include "firepony_gb300.h"

namespace {

constexpr int PROBE_THREADS = 256;
constexpr int PROBE_ITERS = 4096;

__global__ void __launch_bounds__(PROBE_THREADS) k_fma_probe(float *out, float a, float b) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = float(threadIdx.x + j);
    for (int i = 0; i < PROBE_ITERS; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = fmaf(x[j], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) s += x[j];
    if (s == 1234.5f) out[blockIdx.x] = s;  // keeps the chains live; never true for the inputs used
}

__global__ void __launch_bounds__(PROBE_THREADS) k_fma2_probe(float *out, float a, float b) {
    float2 x[8];
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll
    for (int j = 0; j < 8; j++) x[j] = make_float2(float(threadIdx.x + j), float(j));
    for (int i = 0; i < PROBE_ITERS; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) x[j] = __ffma2_rn(x[j], a2, b2);
    }
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++) s += x[j].x + x[j].y;
    if (s == 1234.5f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" fp_status fp_measure_fp32_peak(int device, int packed, double *tflops) {
    if (!tflops) return FP_BAD_INPUT;
    *tflops = 0.0;
    if (cudaSetDevice(device) != cudaSuccess) return FP_DEVICE_ERROR;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        return FP_DEVICE_ERROR;
    float *out = nullptr;
    if (cudaMalloc(&out, size_t(sms) * 8 * sizeof(float)) != cudaSuccess) return FP_OOM;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const unsigned blocks = unsigned(sms) * 8;
    // a multiplier just below 1 and a small addend keep every value a normal number
    const float a = 0.99999f, b = 1e-3f;
    float best_ms = 0.0f;
    for (int rep = 0; rep < 4; rep++) {  // the first launch is a warm-up; best of the others
        cudaEventRecord(e0);
        if (packed) k_fma2_probe<<<blocks, PROBE_THREADS>>>(out, a, b);
        else k_fma_probe<<<blocks, PROBE_THREADS>>>(out, a, b);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && (best_ms == 0.0f || ms < best_ms)) best_ms = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || best_ms <= 0.0f) return FP_DEVICE_ERROR;
    const double flops = double(blocks) * PROBE_THREADS * PROBE_ITERS * 8 * 2 * (packed ? 2 : 1);
    *tflops = flops / (double(best_ms) * 1e-3) / 1e12;
    return FP_OK;
}
