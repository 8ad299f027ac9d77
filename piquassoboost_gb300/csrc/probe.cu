// Pipe-throughput probes used as roofline denominators.
//
// The measured peaks cover HBM copy bandwidth and bf16 tensor rates
// only; the permanent kernels are bound by the FP64 pipe (FP64 product) or
// by FP32/ALU issue (double-float product), so the library measures those
// two peaks itself: a grid of independent FMA chains, 8 per thread, timed
// with CUDA events after a warm-up launch.
#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {
namespace {

constexpr int kProbeIters = 4096;
constexpr int kChains = 8;

__global__ void probe_dfma(double* out, double a, double b) {
    double x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) x[i] = fma(x[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += x[i];
    if (s == 123.456) out[0] = s;  // never true; keeps the chains live
}

__global__ void probe_ffma(float* out, float a, float b) {
    float x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < 4 * kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) x[i] = fmaf(x[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += x[i];
    if (s == 123.456f) out[0] = s;
}

}  // namespace
}  // namespace gbperm

using namespace gbperm;

extern "C" int gbperm_probe_peak(int kind, double* tflops) {
    if (!tflops) return fail(GBPERM_ERR_ARG, "gbperm_probe_peak: null output");
    if (kind != 0 && kind != 1) return fail(GBPERM_ERR_ARG, "gbperm_probe_peak: kind must be 0 (FP64) or 1 (FP32)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_probe_peak");
    int sms = device_sms(dev);
    const int threads = 256, blocks = sms * 8;
    void* buf = nullptr;
    e = cudaMalloc(&buf, 256);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_probe_peak: cudaMalloc");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0);
        if (kind == 0) probe_dfma<<<blocks, threads>>>((double*)buf, 1.0000001, 1e-9);
        else probe_ffma<<<blocks, threads>>>((float*)buf, 1.0000001f, 1e-9f);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // launch 0 is the warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_probe_peak: kernel");
    double fmas = (double)blocks * threads * kChains * (kind == 0 ? kProbeIters : 4.0 * kProbeIters);
    *tflops = 2.0 * fmas / (best * 1e-3) / 1e12;
    return GBPERM_OK;
}
