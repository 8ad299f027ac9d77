// Pipe-throughput probes used as roofline denominators.
//
// The measured peaks cover HBM copy bandwidth and bf16 tensor rates
// only; the permanent kernels are bound by the FP64 pipe (FP64 product), by
// FP32/ALU issue (double-float product) or by the integer multiply-add pipe
// (integer-mantissa product), so the library measures those peaks itself:
// a grid of independent chains, 8 per thread, timed with CUDA events after
// a warm-up launch.  Kinds:
//   0  FP64 FMA (DFMA)                    TFLOP/s, 2 flops per FMA
//   1  FP32 FMA (FFMA)                    TFLOP/s, 2 flops per FMA
//   2  FP64 tensor MMA (mma.sync m8n8k4)  TFLOP/s, 2*8*8*4 flops per warp MMA
//   3  32x32->64 multiply-add (mad.wide.s32, IMAD.WIDE)   tera-ops/s (lane ops)
//   4  32-bit multiply-add (mad.lo.s32, IMAD)             tera-ops/s (lane ops)
//   5  variable funnel shift (shf.l.wrap.b32)             tera-ops/s (lane ops)
//   6  64-bit add (add.s64)                               tera-ops/s (lane ops)
//   7  leading-bit search (bfind.s32)                     tera-ops/s (lane ops)
//   8  32-bit add (add.s32)                               tera-ops/s (lane ops)
// Kinds 5-8 price the integer-mantissa product's non-multiply instructions
// (renormalising shifts, column-sum updates, leading-bit searches).
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

// FP64 tensor core: each warp keeps kChains independent 8x8 accumulators
// and feeds them the same A/B fragments (one f64 each per lane).
__global__ void probe_dmma(double* out, double a, double b) {
    double acc[kChains][2];
#pragma unroll
    for (int i = 0; i < kChains; ++i) acc[i][0] = acc[i][1] = threadIdx.x * 1e-3 + i;
    const double fa = a + threadIdx.x * 1e-6, fb = b;
    for (int it = 0; it < kProbeIters / 4; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(acc[i][0]), "+d"(acc[i][1])
                         : "d"(fa), "d"(fb));
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += acc[i][0] + acc[i][1];
    if (s == 123.456) out[0] = s;
}

__global__ void probe_imad_wide(long long* out, int a, int b) {
    long long x[kChains];
    int m[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
        x[i] = threadIdx.x + i;
        m[i] = a + (int)threadIdx.x + i;
    }
    for (int it = 0; it < 4 * kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) asm volatile("mad.wide.s32 %0, %1, %2, %0;" : "+l"(x[i]) : "r"(m[i]), "r"(b));
    }
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += x[i];
    if (s == 123456789) out[0] = s;
}

__global__ void probe_imad(int* out, int a, int b) {
    int x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x + i;
    for (int it = 0; it < 4 * kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) asm volatile("mad.lo.s32 %0, %0, %1, %2;" : "+r"(x[i]) : "r"(a), "r"(b));
    }
    int s = 0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += x[i];
    if (s == 123456789) out[0] = s;
}

// Integer ALU probes: OP 0 = shf.l.wrap.b32, 1 = bfind.s32, 2 = add.s32.
// The step loop is kept rolled (16 chains per trip, one instruction each):
// unrolled, the assembler may merge consecutive adds of one chain into a
// three-input add and report twice the rate.  The trip's counter and branch
// make the figure a few percent low.
constexpr int kAluChains = 16;

template <int OP>
__global__ void probe_alu32(int* out, int a, int b) {
    unsigned int x[kAluChains];
#pragma unroll
    for (int i = 0; i < kAluChains; ++i) x[i] = threadIdx.x * 7u + i;
    const unsigned int y = (unsigned int)a, z = (unsigned int)b;
#pragma unroll 1
    for (int it = 0; it < 2 * kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kAluChains; ++i) {
            if (OP == 0) asm volatile("shf.l.wrap.b32 %0, %1, %0, %2;" : "+r"(x[i]) : "r"(z), "r"(y));
            if (OP == 1) asm volatile("bfind.s32 %0, %0;" : "+r"(x[i]));
            if (OP == 2) asm volatile("add.s32 %0, %0, %1;" : "+r"(x[i]) : "r"(y));
        }
    }
    unsigned int s = 0;
#pragma unroll
    for (int i = 0; i < kAluChains; ++i) s ^= x[i];
    if (s == 123456789u) out[0] = (int)s;
}

__global__ void probe_add64(long long* out, long long a) {
    long long x[kAluChains];
#pragma unroll
    for (int i = 0; i < kAluChains; ++i) x[i] = threadIdx.x * 7ll + i;
#pragma unroll 1
    for (int it = 0; it < 2 * kProbeIters; ++it) {
#pragma unroll
        for (int i = 0; i < kAluChains; ++i) asm volatile("add.s64 %0, %0, %1;" : "+l"(x[i]) : "l"(a));
    }
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kAluChains; ++i) s ^= x[i];
    if (s == 123456789) out[0] = s;
}

}  // namespace
}  // namespace gbperm

using namespace gbperm;

extern "C" int gbperm_probe_peak(int kind, double* tflops) {
    if (!tflops) return fail(GBPERM_ERR_ARG, "gbperm_probe_peak: null output");
    if (kind < 0 || kind > 8)
        return fail(GBPERM_ERR_ARG,
                    "gbperm_probe_peak: kind must be 0 (FP64), 1 (FP32), 2 (FP64 MMA), 3 (IMAD.WIDE), 4 (IMAD), "
                    "5 (funnel shift), 6 (64-bit add), 7 (bfind) or 8 (32-bit add)");
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
        else if (kind == 1) probe_ffma<<<blocks, threads>>>((float*)buf, 1.0000001f, 1e-9f);
        else if (kind == 2) probe_dmma<<<blocks, threads>>>((double*)buf, 1.0000001, 1e-9);
        else if (kind == 3) probe_imad_wide<<<blocks, threads>>>((long long*)buf, 3, 5);
        else if (kind == 4) probe_imad<<<blocks, threads>>>((int*)buf, 3, 5);
        else if (kind == 5) probe_alu32<0><<<blocks, threads>>>((int*)buf, 3, 5);
        else if (kind == 6) probe_add64<<<blocks, threads>>>((long long*)buf, 977);
        else if (kind == 7) probe_alu32<1><<<blocks, threads>>>((int*)buf, 3, 5);
        else probe_alu32<2><<<blocks, threads>>>((int*)buf, 3, 5);
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
    double ops;
    if (kind == 0) ops = 2.0 * blocks * threads * kChains * (double)kProbeIters;
    else if (kind == 1) ops = 2.0 * blocks * threads * kChains * 4.0 * kProbeIters;
    else if (kind == 2) ops = 2.0 * 8 * 8 * 4 * (blocks * threads / 32.0) * kChains * (kProbeIters / 4);
    else if (kind <= 4) ops = (double)blocks * threads * kChains * 4.0 * kProbeIters;
    else ops = (double)blocks * threads * kAluChains * 2.0 * kProbeIters;
    *tflops = ops / (best * 1e-3) / 1e12;
    return GBPERM_OK;
}
