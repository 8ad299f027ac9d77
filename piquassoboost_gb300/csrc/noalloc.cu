// Plain permanent with library-owned scratch: an entry point that allocates
// no device memory.
//
// Who needs it: callers whose device memory belongs to another allocator
// (a framework that has reserved the whole pool for its own caching
// allocator) and callers that must not pay cudaMalloc's implicit device-wide
// synchronisation inside a latency-critical loop.  gbperm_perm_dev already
// takes device inputs and outputs, but it also wants a caller-provided
// workspace; this variant needs none.
//
// The scratch (fixed-point copies of the matrix, the block partial sums and
// the completion counter of the plain kernels) lives in one file-scope
// __device__ array of kNoAllocScratchBytes.  Every GPU that loads the library
// holds it until the process exits.  Host code cannot use the array's name
// as a device address, so the first call on each device, with that device
// current, looks the address up with cudaGetSymbolAddress and caches it.
// That first call should therefore come before any stream capture.  The
// cached address belongs to the device's primary context: a
// cudaDeviceReset() while the library is in use leaves it stale, so do not
// reset a device between calls.
//
// Trivial shapes (0 x 0, rows >= cols + 2) are answered by a one-thread
// kernel that writes the constant on the stream: no host copy and no
// synchronisation, like every other call of this entry point.
//
// All calls share the one array and it keeps the last call's contents: the
// kernels overwrite every value they read before reading it, and the
// completion counter is cleared by each launch.  Calls that overlap on the
// GPU (different streams, or different host threads with no ordering between
// them) race on the array; callers must serialise them, e.g. on one stream.
#include <cstring>
#include <mutex>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

namespace {

// 256 KiB: two 64 x 64 fixed-point tables (128 KiB) plus block partials of
// the largest grid this library launches, with room to spare.
constexpr size_t kNoAllocScratchBytes = 256 * 1024;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

int scratch_for_current_device(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_noalloc: cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: device index out of range");
    std::lock_guard<std::mutex> g(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_noalloc: cudaGetSymbolAddress");
        g_scratch_ptr[dev] = ptr;
    }
    *out = g_scratch_ptr[dev];
    return GBPERM_OK;
}

// The constant result of a trivial shape (no scratch, no host copy).
__global__ void noalloc_const_kernel(double v, double* out2, double* out4) {
    out2[0] = v;
    out2[1] = 0.0;
    if (out4) {
        out4[0] = v;
        out4[1] = out4[2] = out4[3] = 0.0;
    }
}

}  // namespace

}  // namespace gbperm

using namespace gbperm;

extern "C" size_t gbperm_perm_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int gbperm_perm_noalloc(const void* dA, int64_t rows, int64_t cols, int64_t ld, int arith, void* d_out,
                                   void* d_out_dd, void* stream) {
    if (rows < 0 || cols < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: negative shape");
    if (!d_out) return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: null output");
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: unknown arithmetic");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double hv[4];
    if (plain_trivial(rows, cols, hv, hv)) {
        noalloc_const_kernel<<<1, 1, 0, st>>>(hv[0], static_cast<double*>(d_out), static_cast<double*>(d_out_dd));
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? GBPERM_OK : cuda_fail(e, "gbperm_perm_noalloc");
    }
    if (!dA) return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: null matrix");
    if (ld < cols) return fail(GBPERM_ERR_ARG, "gbperm_perm_noalloc: ld < cols");
    if (rows > GBPERM_MAX_DIM || cols > GBPERM_MAX_DIM)
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_noalloc: matrix larger than 64 x 64");
    PlainPlan plan = plan_plain((int)rows, (int)cols,
                                arith == GBPERM_ARITH_DF32 && cols <= kDfMaxCols ? GBPERM_ARITH_DF32 : GBPERM_ARITH_FP64);
    size_t need = plain_ws_layout((int)rows, (int)cols, plan.max_grid(), nullptr);
    if (need > kNoAllocScratchBytes)
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_noalloc: needs " + std::to_string(need) +
                                              " bytes of scratch, more than the fixed " +
                                              std::to_string(kNoAllocScratchBytes));
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    return run_plain_dev(static_cast<const double2*>(dA), ld, (int)rows, (int)cols, scratch, kNoAllocScratchBytes,
                         static_cast<double*>(d_out), static_cast<double*>(d_out_dd), st, plan);
}
