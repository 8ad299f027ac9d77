// C ABI (include/gbperm.h): validation, workspace management and dispatch.
//
// The reference's wrappers throw std::string from C++ and turn it into a
// Python exception (GlynnPermanentCalculator_Wrapper.hpp:234-237); here every
// failure is a status code plus a per-thread message.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

thread_local std::string t_err;

int fail(int code, const std::string& msg) {
    t_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    return fail(GBPERM_ERR_CUDA, m);
}

Options g_opt;

int device_sms(int dev) {
    static std::mutex mu;
    static std::unordered_map<int, int> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(dev);
    if (it != cache.end()) return it->second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
    cache[dev] = sms;
    return sms;
}

cudaError_t allow_max_dynamic_smem(const void* kernel) {
    static std::mutex mu;
    static std::unordered_map<const void*, unsigned long long> done;  // kernel -> bitmask of devices
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    std::lock_guard<std::mutex> g(mu);
    auto it = done.find(kernel);
    if (it != done.end() && (it->second & bit)) return cudaSuccess;
    int optin = 0;
    e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa{};
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    const int dyn = optin - (int)fa.sharedSizeBytes;
    if (dyn > 0) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
        if (e != cudaSuccess) return e;
    }
    done[kernel] |= bit;
    return cudaSuccess;
}

ThreadCtx& thread_ctx() {
    thread_local ThreadCtx c;
    return c;
}

int ThreadCtx::ensure(size_t bytes) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return fail(GBPERM_ERR_NO_DEVICE, "no CUDA device visible: the GB300 permanent library needs a GPU");
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (device != dev) {
        // a new device for this thread: release the old device's stream,
        // events and workspace with that device current, then start afresh
        if (device >= 0) {
            if (cudaSetDevice(device) == cudaSuccess) {
                if (dbuf) cudaFree(dbuf);
                if (ev0) cudaEventDestroy(ev0);
                if (ev1) cudaEventDestroy(ev1);
                if (stream) cudaStreamDestroy(stream);
            }
            cudaGetLastError();
            e = cudaSetDevice(dev);
            if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
        }
        stream = nullptr;
        ev0 = ev1 = nullptr;
        dbuf = nullptr;
        dcap = 0;
        device = dev;
        e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
        e = cudaEventCreate(&ev0);
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
        e = cudaEventCreate(&ev1);
        if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    }
    if (bytes > dcap) {
        if (dbuf) cudaFree(dbuf);
        dbuf = nullptr;
        dcap = 0;
        size_t want = align_up(bytes, 1 << 20);
        e = cudaMalloc(&dbuf, want);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(workspace)");
        dcap = want;
    }
    return GBPERM_OK;
}

bool all_finite(const double* A, int64_t rows, int64_t cols, int64_t ld) {
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < 2 * cols; ++j)
            if (!std::isfinite(A[2 * i * ld + j])) return false;
    return true;
}

int ceil_log2_u64(unsigned long long x) {
    int l = 0;
    while ((1ull << l) < x && l < 63) ++l;
    return l;
}

// ------------------------------------------------------------------ plain

// Segment length and grid for `seg_threads` threads per segment.
static void plain_geometry(int rows, int grid_full, int seg_threads, int* grid, int* seg_log2) {
    int slog = rows - 1;
    // aim at >= 64 segments per segment-slot of a full grid (load balance
    // within ~1.5%) while keeping segments >= 16 steps when possible
    unsigned long long slots = (unsigned long long)grid_full * (128ull / seg_threads);
    int l = slog - ceil_log2_u64(64ull * slots);
    if (l < 4) l = slog < 4 ? slog : 4;
    if (l > slog) l = slog;
    if (l < 0) l = 0;
    int64_t force = g_opt.plain_seg_log2.load();
    if (force >= 0) l = (int)(force > slog ? slog : force);
    if (l > 31) l = 31;  // the integer-mantissa kernel counts steps in 32 bits
    unsigned long long nseg = 1ull << (slog - l);
    unsigned long long per_block = 128ull / seg_threads;
    unsigned long long need = (nseg + per_block - 1) / per_block;
    int g = (int)(need < (unsigned long long)grid_full ? need : (unsigned long long)grid_full);
    int64_t fg = g_opt.plain_grid.load();
    if (fg > 0) g = (int)fg;
    if (g < 1) g = 1;
    *grid = g;
    *seg_log2 = l;
}

int plain_arith(int64_t rows, int64_t cols, int arith) {
    if (arith != GBPERM_ARITH_DF32) return arith;
    if (cols > kDfMaxCols || (rows == cols && rows > g_opt.df_max_rows.load())) return GBPERM_ARITH_FX64;
    return arith;
}

PlainPlan plan_plain(int rows, int cols, int arith) {
    PlainPlan p;
    p.df = arith == GBPERM_ARITH_DF32;
    p.fx = arith == GBPERM_ARITH_FX64;
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = device_sms(dev);
    // the double-float kernel's twin is the integer-mantissa kernel: it
    // recomputes on the device when the range check fails or the estimate
    // is above the bar
    if (p.df) p.fx = true;
    if (p.fx) {
        fx_shape(cols, (int)g_opt.plain_fx_group.load(), &p.cpl_fx, &p.grp_fx);
        plain_geometry(rows, sms * plain_fx_blocks_per_sm(rows, p.cpl_fx, p.grp_fx), p.grp_fx, &p.grid_fx,
                       &p.seg_log2_fx);
    } else {
        plain_geometry(rows, sms * plain_blocks_per_sm(rows, cols), plain_group(cols), &p.grid, &p.seg_log2);
    }
    if (p.df) {
        df_shape(cols, (int)g_opt.plain_df_group.load(), &p.cpl, &p.grp);
        plain_geometry(rows, sms * plain_df_blocks_per_sm(rows, p.cpl, p.grp), p.grp, &p.grid_df, &p.seg_log2_df);
    }
    return p;
}

size_t plain_ws_layout(int rows, int cols, int grid, PlainWs* w) {
    size_t off = 0;
    size_t mat = align_up((size_t)rows * cols * sizeof(longlong2), 256);
    if (w) w->a1 = off;
    off += mat;
    if (w) w->a2 = off;
    off += mat;
    if (w) w->exp = off;
    off += 256;
    if (w) w->scale = off;
    off += 256;
    if (w) w->kern = off;
    off += plain_workspace_bytes(grid);
    return off;
}

int run_plain_dev(const double2* dA, int64_t ld, int rows, int cols, void* ws, size_t ws_bytes,
                  double* d_out2, double* d_out4, cudaStream_t st, const PlainPlan& plan, double* d_err) {
    PlainWs w;
    size_t need = plain_ws_layout(rows, cols, plan.max_grid(), &w);
    if (ws_bytes < need) return fail(GBPERM_ERR_ARG, "gbperm: workspace too small");
    char* base = static_cast<char*>(ws);
    PrepArgs pa;
    pa.col_e_out = nullptr;
    pa.A = dA;
    pa.ld = ld;
    pa.rows = rows;
    pa.cols = cols;
    pa.row_w = nullptr;
    pa.col_w = nullptr;
    pa.norm_shift = rows - 1;
    pa.a1 = reinterpret_cast<longlong2*>(base + w.a1);
    pa.a2 = reinterpret_cast<longlong2*>(base + w.a2);
    pa.exp_out = reinterpret_cast<int*>(base + w.exp);
    pa.df = plan.df ? 1 : 0;
    pa.df_info = reinterpret_cast<int*>(base + w.scale);
    // the Gray sum is multilinear in the rows only for square matrices
    // (for rows != cols it is a different polynomial of the entries)
    pa.row_balance = rows == cols ? 1 : 0;
    pa.exp_fp64_out = pa.exp_out + 1;
    cudaError_t e = launch_prepare(pa, st);
    if (e != cudaSuccess) return cuda_fail(e, "prepare launch");
    if (plan.df) {
        // the double-float kernel returns at once if the device range check
        // failed; its integer-mantissa twin below returns at once unless that
        // check failed or the double-float result's error estimate was above
        // the bar
        double* err = d_err ? d_err : reinterpret_cast<double*>(base + w.scale + 8);
        e = cudaMemsetAsync(err, 0, sizeof(double), st);
        if (e != cudaSuccess) return cuda_fail(e, "plain df error slot");
        e = launch_plain_df(pa.a1, pa.a2, pa.exp_out, pa.df_info, rows, cols, plan.cpl, plan.grp, plan.grid_df,
                            plan.seg_log2_df, base + w.kern, d_out2, d_out4, err, g_opt.df_escalate.load() != 0, st);
        if (e != cudaSuccess) return cuda_fail(e, "plain df launch");
    } else if (plan.fx && d_err) {
        e = cudaMemsetAsync(d_err, 0, sizeof(double), st);
        if (e != cudaSuccess) return cuda_fail(e, "plain fx error slot");
    }
    if (plan.fx) {
        // scaled by the exponent without the double-float boost
        e = launch_plain_fx(pa.a1, pa.a2, pa.exp_fp64_out, plan.df ? pa.df_info : nullptr, rows, cols, plan.cpl_fx,
                            plan.grp_fx, plan.grid_fx, plan.seg_log2_fx, base + w.kern, d_out2, d_out4, st);
        if (e != cudaSuccess) return cuda_fail(e, "plain fx launch");
        return GBPERM_OK;
    }
    e = launch_plain(pa.a1, pa.a2, pa.exp_fp64_out, nullptr, rows, cols, plan.grid, plan.seg_log2, base + w.kern,
                     d_out2, d_out4, st);
    if (e != cudaSuccess) return cuda_fail(e, "plain launch");
    return GBPERM_OK;
}

// Trivial shapes shared by the plain entry points; returns true when `out`
// has been filled without any GPU work.
bool plain_trivial(int64_t rows, int64_t cols, double* out, double* out_dd) {
    double v = -1.0;
    if (rows == 0 || cols == 0) v = 1.0;
    else if (rows >= cols + 2) v = 0.0;
    if (v < 0.0) return false;
    out[0] = v;
    out[1] = 0.0;
    if (out_dd) {
        out_dd[0] = v;
        out_dd[1] = out_dd[2] = out_dd[3] = 0.0;
    }
    return true;
}

}  // namespace gbperm

using namespace gbperm;

extern "C" {

int gbperm_version(void) { return 100; }

const char* gbperm_last_error(void) { return t_err.c_str(); }

int gbperm_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

int gbperm_set_option(const char* key, int64_t value) {
    if (!key) return fail(GBPERM_ERR_ARG, "gbperm_set_option: null key");
    std::atomic<int64_t>* slot = g_opt.find(key);
    if (!slot) return fail(GBPERM_ERR_ARG, std::string("gbperm_set_option: unknown key ") + key);
    slot->store(value);
    return GBPERM_OK;
}

int64_t gbperm_get_option(const char* key) {
    if (!key) return 0;
    std::atomic<int64_t>* slot = g_opt.find(key);
    return slot ? slot->load() : 0;
}

size_t gbperm_perm_workspace_size(int64_t rows, int64_t cols) {
    if (rows <= 0 || cols <= 0 || rows > GBPERM_MAX_DIM || cols > GBPERM_MAX_DIM) return 256;
    // the largest of the arithmetics' needs (grids may differ)
    PlainPlan plan = plan_plain((int)rows, (int)cols, cols <= kDfMaxCols ? GBPERM_ARITH_DF32 : GBPERM_ARITH_FX64);
    PlainPlan p64 = plan_plain((int)rows, (int)cols, GBPERM_ARITH_FP64);
    const int g = plan.max_grid() > p64.max_grid() ? plan.max_grid() : p64.max_grid();
    return plain_ws_layout((int)rows, (int)cols, g, nullptr);
}

int gbperm_perm_dev(const void* dA, int64_t rows, int64_t cols, int64_t ld, int arith, void* d_out,
                    void* d_out_dd, void* workspace, size_t workspace_bytes, void* stream) {
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: unknown arithmetic");
    if (rows < 0 || cols < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: negative shape");
    if (!d_out) return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: null output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double hv[4];
    if (plain_trivial(rows, cols, hv, hv)) {
        hv[1] = 0.0;
        hv[2] = hv[3] = 0.0;
        double h2[2] = {hv[0], 0.0};
        cudaError_t e = cudaMemcpyAsync(d_out, h2, sizeof(h2), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && d_out_dd) e = cudaMemcpyAsync(d_out_dd, hv, sizeof(hv), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        return e == cudaSuccess ? GBPERM_OK : cuda_fail(e, "gbperm_perm_dev");
    }
    if (!dA || !workspace) return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: null pointer");
    if (ld < cols) return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: ld < cols");
    if (rows > GBPERM_MAX_DIM || cols > GBPERM_MAX_DIM)
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_dev: matrix larger than 64 x 64");
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_dev: workspace must be 256-byte aligned");
    PlainPlan plan = plan_plain((int)rows, (int)cols, plain_arith(rows, cols, arith));
    return run_plain_dev(static_cast<const double2*>(dA), ld, (int)rows, (int)cols, workspace,
                         workspace_bytes, static_cast<double*>(d_out), static_cast<double*>(d_out_dd), st,
                         plan);
}

int gbperm_perm(const double* A, int64_t rows, int64_t cols, int64_t ld, int arith, double* out,
                double* out_dd, gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!out) return fail(GBPERM_ERR_ARG, "gbperm_perm: null output");
    if (rows < 0 || cols < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm: negative shape");
    if (plain_trivial(rows, cols, out, out_dd)) return GBPERM_OK;
    if (!A) return fail(GBPERM_ERR_ARG, "gbperm_perm: null matrix");
    if (ld < cols) return fail(GBPERM_ERR_ARG, "gbperm_perm: ld < cols");
    if (rows > GBPERM_MAX_DIM || cols > GBPERM_MAX_DIM)
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm: matrix larger than 64 x 64");
    if (!all_finite(A, rows, cols, ld)) {
        out[0] = out[1] = NAN;
        if (out_dd) out_dd[0] = out_dd[1] = out_dd[2] = out_dd[3] = NAN;
        return GBPERM_OK;
    }
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_perm: unknown arithmetic");
    // the double-float product where the size rule and the host range check
    // allow it, else the integer-mantissa product alone
    const int a = plain_arith(rows, cols, arith);
    bool df = false;
    int boost = 0;
    if (a == GBPERM_ARITH_DF32) df = df_boost(A, rows, cols, ld, nullptr, nullptr, &boost, rows == cols);
    const bool fx = a == GBPERM_ARITH_FX64 || (a == GBPERM_ARITH_DF32 && !df);
    PlainPlan plan = plan_plain((int)rows, (int)cols,
                                df ? GBPERM_ARITH_DF32 : (fx ? GBPERM_ARITH_FX64 : GBPERM_ARITH_FP64));
    size_t mat_bytes = align_up((size_t)rows * cols * sizeof(double2), 256);
    size_t ws = plain_ws_layout((int)rows, (int)cols, plan.max_grid(), nullptr);
    ThreadCtx& c = thread_ctx();
    int rc = c.ensure(mat_bytes + 256 + ws);
    if (rc) return rc;
    char* base = static_cast<char*>(c.dbuf);
    double2* dA = reinterpret_cast<double2*>(base);
    double* dout = reinterpret_cast<double*>(base + mat_bytes);  // 6 doubles: out2, out4
    void* dws = base + mat_bytes + 256;
    cudaError_t e = cudaMemcpy2DAsync(dA, cols * sizeof(double2), A, ld * sizeof(double2),
                                      cols * sizeof(double2), rows, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm: upload");
    if (stats) cudaEventRecord(c.ev0, c.stream);
    rc = run_plain_dev(dA, cols, (int)rows, (int)cols, dws, ws, dout, dout + 2, c.stream, plan, dout + 6);
    if (rc) return rc;
    if (stats) cudaEventRecord(c.ev1, c.stream);
    double h[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    e = cudaMemcpyAsync(h, dout, (df ? 7 : 6) * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm: download");
    e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm: kernel");
    out[0] = h[0];
    out[1] = h[1];
    if (out_dd) std::memcpy(out_dd, h + 2, 4 * sizeof(double));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        stats->kernel_ms = ms;
        stats->steps = std::ldexp(1.0, (int)rows - 1);
        stats->flops = 8.0 * (double)cols * stats->steps;
        stats->launches = df ? 3 : 2;
        stats->grid = df ? plan.grid_df : (plan.fx ? plan.grid_fx : plan.grid);
        stats->seg_log2 = df ? plan.seg_log2_df : (plan.fx ? plan.seg_log2_fx : plan.seg_log2);
        // h[6]: the double-float estimate, -1 when the device range check
        // sent the matrix to the twin; above the bar the integer-mantissa
        // twin recomputed
        const bool ran_df = df && h[6] >= 0.0;
        const bool used_df = ran_df && (h[6] <= kDfEscalate || g_opt.df_escalate.load() == 0);
        stats->arith = used_df ? GBPERM_ARITH_DF32 : (plan.fx ? GBPERM_ARITH_FX64 : GBPERM_ARITH_FP64);
        stats->err_est = ran_df ? h[6] : 0.0;
    }
    return GBPERM_OK;
}

}  // extern "C"
