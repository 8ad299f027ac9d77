// Permanent and its full gradient in one Gray-code sweep (GB300).
//
// There is no reference function for this; it is the adjoint of the plain
// BBFG sum (BBFGPermanentCalculator.hpp:87-235):
//   dperm/da_kl = 2^-(n-1) sum_delta s(delta) delta_k W_l(delta),
//   W_l = prod_{j != l} c_j(delta),  s = prod_i delta_i,
// i.e. perm of A with row k and column l removed.
//
// Per step, W is formed from prefix and suffix products of the column sums
// (no division), in double-float arithmetic on the FP32 pipe, and
// X = s W is added to a running sum Q.  The n x n accumulation uses the Gray
// structure: delta_r only changes when row r flips, so by telescoping
//   sum_t delta_r(t) X(t) = delta_r(T) Q(T) + sum_{flips of r at k} 2 delta_r(k-1) Q(k-1),
// and each step touches ONE row of G (the row that flips, warp-uniform)
// instead of all n.  Q is folded into G and restarted every kChunk steps to
// keep the running sums small (bounded rounding growth).
//
// Layout: GROUP = 4 lanes share a Gray walk, lane g owns columns
// [g*CPL, (g+1)*CPL); the 8 groups of a warp walk 8 aligned ranges in
// lockstep.  The per-step row update of G is a reduce-scatter over the 8
// groups (lane (g, grp) ends with column g*CPL + grp), added into the warp's
// own n x n double-float G tile in shared memory.  Warp tiles are written to
// global memory and summed in a fixed order by a finalize kernel.
#include <cmath>
#include <cstring>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
constexpr int kGroup = 4;
constexpr int kGroups = 32 / kGroup;  // walks per warp
constexpr int kChunk = 256;           // steps between folds of Q into G

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
}

__device__ __forceinline__ cf shfl_cf(const cf& v, int src) {
    return cf{__shfl_sync(0xffffffffu, v.rh, src), __shfl_sync(0xffffffffu, v.rl, src),
              __shfl_sync(0xffffffffu, v.ih, src), __shfl_sync(0xffffffffu, v.il, src)};
}

__device__ __forceinline__ cf cf_add(const cf& a, const cf& b) {
    cf r = a;
    df_acc(r.rh, r.rl, b.rh, b.rl);
    df_acc(r.ih, r.il, b.ih, b.il);
    return r;
}

__device__ __forceinline__ cf cf_scale_sign(const cf& a, unsigned int sbit) {
    return cf{__uint_as_float(__float_as_uint(a.rh) ^ sbit), __uint_as_float(__float_as_uint(a.rl) ^ sbit),
              __uint_as_float(__float_as_uint(a.ih) ^ sbit), __uint_as_float(__float_as_uint(a.il) ^ sbit)};
}

struct GradArgs {
    const longlong2* a1;
    const longlong2* a2;
    int n;
    int seg_log2;              // each walk covers 2^seg_log2 Gray steps
    unsigned long long nseg;   // walks (multiple of kGroups, or smaller total)
    const int* df_info;        // {boost, ok}
    float4* warp_g;            // per warp: n x n complex double-float tiles (re_h, re_l, im_h, im_l)
    float4* warp_p;            // per warp: permanent partial
};

// Reduce-scatter of v[0..CPL) over the kGroups groups of a warp (lanes with
// equal g): afterwards lane (g, grp) holds, in v[0], the sum over groups of
// column g*CPL + (grp % CPL) (CPL <= kGroups).  The ownership pattern is
// fixed: at each halving stage with mask m, the lane with (grp & m) keeps
// the upper half.
template <int CPL>
__device__ __forceinline__ cf reduce_scatter(cf (&v)[CPL], int grp) {
    int lanes_per_col = kGroups;  // groups still sharing each column slot
    int width = CPL;
    int base = 0;                 // first column index this lane still holds
#pragma unroll
    for (int m = kGroups / 2; m >= 1; m >>= 1) {
        if (width > 1) {
            const int half = width / 2;
            const bool upper = (grp & m) != 0;
#pragma unroll
            for (int c = 0; c < CPL / 2; ++c) {
                if (c < half) {
                    // send the half I drop, receive the matching half I keep
                    cf send = upper ? v[c] : v[c + half];
                    cf recv = shfl_xor_cf(send, m * kGroup);
                    cf keep = upper ? v[c + half] : v[c];
                    v[c] = cf_add(keep, recv);
                }
            }
            if (upper) base += half;
            width = half;
        } else {
            cf recv = shfl_xor_cf(v[0], m * kGroup);
            v[0] = cf_add(v[0], recv);
        }
        lanes_per_col >>= 1;
    }
    (void)base;
    return v[0];
}

// Column owned by lane (g, grp) after reduce_scatter<CPL>.
template <int CPL>
__device__ __forceinline__ int scatter_col(int g, int grp) {
    int width = CPL, base = 0;
#pragma unroll
    for (int m = kGroups / 2; m >= 1; m >>= 1) {
        if (width > 1) {
            const int half = width / 2;
            if (grp & m) base += half;
            width = half;
        }
    }
    return g * CPL + base;
}

template <int CPL>
__global__ void __launch_bounds__(kThreads) grad_kernel(GradArgs p) {
    constexpr int NP = CPL * kGroup;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);           // n x NP
    longlong2* s_a2 = s_a1 + p.n * NP;                                  // n x NP
    float4* s_g = reinterpret_cast<float4*>(s_a2 + p.n * NP);           // (warps) x n x NP
    const int n = p.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane % kGroup, grp = lane / kGroup;
    const int j0 = g * CPL;
    float4* G = s_g + (size_t)warp * n * NP;
    for (int e = threadIdx.x; e < n * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        longlong2 z = make_longlong2(0, 0);
        s_a1[e] = j < n ? p.a1[r * n + j] : z;
        s_a2[e] = j < n ? p.a2[r * n + j] : z;
    }
    for (int e = lane; e < n * NP; e += 32) G[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    if (p.df_info[1] == 0) return;  // range check failed: finalize writes NaN
    const DfConv cv = make_dfconv(p.df_info[0]);
    const int my_col = scatter_col<CPL>(g, grp);
    // with CPL < kGroups the last stages are all-reduces: one lane per column writes
    const bool writer = (grp & (kGroups / CPL - 1)) == 0;
    const unsigned long long L = 1ull << p.seg_log2;
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (kThreads / 32);
    const unsigned long long gwarp = (unsigned long long)blockIdx.x * (kThreads / 32) + warp;
    long long cre[CPL], cim[CPL];
    cf Q[CPL];
    float prh = 0.f, prl = 0.f, pih = 0.f, pil = 0.f;  // permanent partial (group leader)

    // fold Q into every row of G: G[r] += delta_r * Q (the end term), then Q = 0
    auto fold_all = [&](unsigned long long idx, bool active) {
        const unsigned long long gray = idx ^ (idx >> 1);
        for (int r = 0; r < n; ++r) {
            // delta_r = -1 when bit (n-1-r) of the Gray code is set (row 0: +1)
            const bool neg = r > 0 && ((gray >> (n - 1 - r)) & 1ull);
            cf v[CPL];
#pragma unroll
            for (int c = 0; c < CPL; ++c) v[c] = active ? cf_scale_sign(Q[c], neg ? 0x80000000u : 0u) : cf{0.f, 0.f, 0.f, 0.f};
            cf s = reduce_scatter<CPL>(v, grp);
            if (writer && my_col < n) {
                float4 gg = G[r * NP + my_col];
                df_acc(gg.x, gg.y, s.rh, s.rl);
                df_acc(gg.z, gg.w, s.ih, s.il);
                G[r * NP + my_col] = gg;
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) Q[c] = cf{0.f, 0.f, 0.f, 0.f};
    };

    for (unsigned long long wb = gwarp * kGroups; wb < p.nseg; wb += warps_total * kGroups) {
        const unsigned long long s_raw = wb + grp;
        const bool active = s_raw < p.nseg;
        const unsigned long long i0 = (active ? s_raw : 0ull) << p.seg_log2;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cre[c] = s_a1[j0 + c].x;
            cim[c] = s_a1[j0 + c].y;
            Q[c] = cf{0.f, 0.f, 0.f, 0.f};
        }
        for (int r = 1; r < n; ++r) {
            const long long m = -(long long)((g0 >> (n - 1 - r)) & 1ull);
            const longlong2* a = s_a1 + r * NP + j0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                longlong2 v = a[c];
                cre[c] += (v.x ^ m) - m;
                cim[c] += (v.y ^ m) - m;
            }
        }
        unsigned int sbit = (unsigned int)(__popcll(g0) & 1) << 31;
        for (unsigned long long k = 0; k < L; ++k) {
            const unsigned long long idx = i0 + k;
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;          // warp-uniform
                const int r = n - 1 - b;                            // the row that flips
                const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;  // new delta_r = -1
                if ((k % kChunk) == 0) {
                    // chunk boundary: end term at idx-1 for every row, Q = 0;
                    // the flip term of this step would then add 2 * 0
                    fold_all(idx - 1, active);
                } else {
                    // flip term: G[r] += 2 delta_r(k-1) Q(k-1); delta_r(k-1) = +1
                    // when the row now turns -1
                    {
                    cf v[CPL];
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        cf q = Q[c];
                        q.rh *= 2.f; q.rl *= 2.f; q.ih *= 2.f; q.il *= 2.f;
                        v[c] = active ? cf_scale_sign(q, sub ? 0u : 0x80000000u) : cf{0.f, 0.f, 0.f, 0.f};
                    }
                    cf s = reduce_scatter<CPL>(v, grp);
                    if (writer && my_col < n) {
                        float4 gg = G[r * NP + my_col];
                        df_acc(gg.x, gg.y, s.rh, s.rl);
                        df_acc(gg.z, gg.w, s.ih, s.il);
                        G[r * NP + my_col] = gg;
                    }
                }
                }
                const longlong2* a = s_a2 + r * NP + j0;
                if (sub) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c];
                        cre[c] -= v.x;
                        cim[c] -= v.y;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c];
                        cre[c] += v.x;
                        cim[c] += v.y;
                    }
                }
                sbit ^= 0x80000000u;
            }
            // column values (padded columns act as 1)
            cf x[CPL];
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (j0 + c < n) {
                    fix_to_df_magic(cre[c], cv, x[c].rh, x[c].rl);
                    fix_to_df_magic(cim[c], cv, x[c].ih, x[c].il);
                } else {
                    x[c] = cf{1.f, 0.f, 0.f, 0.f};
                }
            }
            // partial product of my columns, then the product of the other
            // three lanes' partials (gathered in the group)
            cf part = x[0];
#pragma unroll
            for (int c = 1; c < CPL; ++c) part = cf_mul(part, x[c]);
            const int lbase = lane - g;
            cf o1 = shfl_cf(part, lbase + ((g + 1) & 3));
            cf o2 = shfl_cf(part, lbase + ((g + 2) & 3));
            cf o3 = shfl_cf(part, lbase + ((g + 3) & 3));
            cf excl = cf_mul(cf_mul(o1, o2), o3);
            // permanent term (leader)
            if (g == 0 && active) {
                cf tot = cf_scale_sign(cf_mul(excl, part), sbit);
                df_acc(prh, prl, tot.rh, tot.rl);
                df_acc(pih, pil, tot.ih, tot.il);
            }
            // W_c = excl * prod_{c' < c} x_c' * prod_{c' > c} x_c' (prefix/suffix)
            cf pre[CPL];
            pre[0] = cf_scale_sign(excl, sbit);  // fold the sign s(delta) in once
#pragma unroll
            for (int c = 1; c < CPL; ++c) pre[c] = cf_mul(pre[c - 1], x[c - 1]);
            cf suf{1.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c = CPL - 1; c >= 0; --c) {
                cf w = (c == CPL - 1) ? pre[c] : cf_mul(pre[c], suf);
                Q[c] = cf_add(Q[c], w);
                if (c > 0) suf = (c == CPL - 1) ? x[c] : cf_mul(suf, x[c]);
            }
        }
        // end term of the walk
        fold_all(i0 + L - 1, active);
    }
    __syncwarp();
    // write the warp's G tile and permanent partial
    float4* outg = p.warp_g + (size_t)gwarp * n * n;
    for (int e = lane; e < n * n; e += 32) {
        int r = e / n, j = e % n;
        outg[e] = G[r * NP + j];
    }
    // permanent: sum the 8 leaders' partials
    cf pp{prh, prl, pih, pil};
#pragma unroll
    for (int m = kGroup; m < 32; m <<= 1) pp = cf_add(pp, shfl_xor_cf(pp, m));
    if (lane == 0) p.warp_p[gwarp] = make_float4(pp.rh, pp.rl, pp.ih, pp.il);
}

// Sum the warp tiles (fixed order) in double-double, scale, write the
// gradient (complex128, n x n row-major) and the permanent.
__global__ void grad_finalize_kernel(const float4* warp_g, const float4* warp_p, int nwarps, int n,
                                     const int* exp_in, const int* col_e, const int* df_info, double* grad,
                                     double* perm2, double* perm4) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int boost = df_info[0];
    if (df_info[1] == 0) {
        if (e < n * n) grad[2 * e] = grad[2 * e + 1] = nan("");
        if (e == 0) {
            perm2[0] = perm2[1] = nan("");
            if (perm4) perm4[0] = perm4[1] = perm4[2] = perm4[3] = nan("");
        }
        return;
    }
    if (e < n * n) {
        cdd acc{{0.0, 0.0}, {0.0, 0.0}};
        for (int w = 0; w < nwarps; ++w) {
            float4 v = warp_g[(size_t)w * n * n + e];
            acc.re = dd_add(acc.re, dd{(double)v.x, (double)v.y});
            acc.im = dd_add(acc.im, dd{(double)v.z, (double)v.w});
        }
        const int l = e % n;
        // W_l omits column l: remove its factor from the permanent's scale
        const int ex = *exp_in - (col_e[l] - boost);
        double r2[2];
        write_result(acc, ex, r2, nullptr);
        grad[2 * e] = r2[0];
        grad[2 * e + 1] = r2[1];
    }
    if (e == 0) {
        cdd acc{{0.0, 0.0}, {0.0, 0.0}};
        for (int w = 0; w < nwarps; ++w) {
            float4 v = warp_p[w];
            acc.re = dd_add(acc.re, dd{(double)v.x, (double)v.y});
            acc.im = dd_add(acc.im, dd{(double)v.z, (double)v.w});
        }
        write_result(acc, *exp_in, perm2, perm4);
    }
}

// Per-column exponents e_j of the fixed-point scaling (the prepare kernel
// keeps them internal; recomputed here identically).
__global__ void col_exp_kernel(const double2* A, long long ld, int n, int* col_e) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double br = 0.0, bi = 0.0;
    for (int i = 0; i < n; ++i) {
        double2 a = A[(long long)i * ld + j];
        br += fabs(a.x);
        bi += fabs(a.y);
    }
    double b = fmax(br, bi) * (1.0 + 1e-12);
    int e = 0;
    if (b > 0.0) frexp(b, &e);
    col_e[j] = e;
}

template <int CPL>
size_t grad_smem(int n) {
    return 2ull * n * CPL * kGroup * sizeof(longlong2) + (size_t)(kThreads / 32) * n * CPL * kGroup * sizeof(float4);
}

}  // namespace

struct GradPlan {
    int cpl = 8;
    int grid = 1;
    int seg_log2 = 0;
    unsigned long long nseg = 1;
    int nwarps = 1;
};

static GradPlan plan_grad(int n) {
    GradPlan gp;
    gp.cpl = n <= 16 ? 4 : 8;
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = device_sms(dev);
    int nb = 0;
    size_t smem = gp.cpl == 4 ? grad_smem<4>(n) : grad_smem<8>(n);
    if (gp.cpl == 4) {
        cudaFuncSetAttribute(grad_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, grad_kernel<4>, kThreads, smem);
    } else {
        cudaFuncSetAttribute(grad_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, grad_kernel<8>, kThreads, smem);
    }
    if (nb < 1) nb = 1;
    int grid_full = sms * nb;
    int slog = n - 1;
    // walks of >= 2 kChunk steps when possible; >= 8 walks per resident group slot
    unsigned long long slots = (unsigned long long)grid_full * (kThreads / 32) * kGroups;
    int l = slog - ceil_log2_u64(8ull * slots);
    if (l < 9) l = 9;
    if (l > slog) l = slog;
    gp.seg_log2 = l;
    gp.nseg = 1ull << (slog - l);
    unsigned long long warps_needed = (gp.nseg + kGroups - 1) / kGroups;
    unsigned long long blocks_needed = (warps_needed + 3) / 4;
    gp.grid = (int)(blocks_needed < (unsigned long long)grid_full ? blocks_needed : (unsigned long long)grid_full);
    if (gp.grid < 1) gp.grid = 1;
    gp.nwarps = gp.grid * (kThreads / 32);
    return gp;
}

static size_t grad_ws_bytes(int n, const GradPlan& gp) {
    size_t mat = align_up((size_t)n * n * sizeof(longlong2), 256);
    return 2 * mat + 256 + 256 + align_up((size_t)n * sizeof(int), 256) +
           align_up((size_t)gp.nwarps * n * n * sizeof(float4), 256) + align_up((size_t)gp.nwarps * sizeof(float4), 256);
}

// Device-side gradient: dA (n x n complex128, ld), grad out (n x n complex128
// row-major), perm out (2 doubles) and optional perm dd (4 doubles).
static int run_grad_dev(const double2* dA, long long ld, int n, void* ws, size_t ws_bytes, double* d_grad,
                        double* d_perm, double* d_perm4, cudaStream_t st, GradPlan* used) {
    GradPlan gp = plan_grad(n);
    if (used) *used = gp;
    if (ws_bytes < grad_ws_bytes(n, gp)) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad: workspace too small");
    char* base = static_cast<char*>(ws);
    size_t mat = align_up((size_t)n * n * sizeof(longlong2), 256);
    size_t off = 0;
    longlong2* a1 = reinterpret_cast<longlong2*>(base + off);
    off += mat;
    longlong2* a2 = reinterpret_cast<longlong2*>(base + off);
    off += mat;
    int* exp_out = reinterpret_cast<int*>(base + off);
    off += 256;
    int* df_info = reinterpret_cast<int*>(base + off);
    off += 256;
    int* col_e = reinterpret_cast<int*>(base + off);
    off += align_up((size_t)n * sizeof(int), 256);
    float4* warp_g = reinterpret_cast<float4*>(base + off);
    off += align_up((size_t)gp.nwarps * n * n * sizeof(float4), 256);
    float4* warp_p = reinterpret_cast<float4*>(base + off);
    PrepArgs pa;
    pa.A = dA;
    pa.ld = ld;
    pa.rows = n;
    pa.cols = n;
    pa.row_w = nullptr;
    pa.col_w = nullptr;
    pa.norm_shift = n - 1;
    pa.a1 = a1;
    pa.a2 = a2;
    pa.exp_out = exp_out;
    pa.df = 1;
    pa.df_info = df_info;
    cudaError_t e = launch_prepare(pa, st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: prepare");
    col_exp_kernel<<<1, 64, 0, st>>>(dA, ld, n, col_e);
    GradArgs g;
    g.a1 = a1;
    g.a2 = a2;
    g.n = n;
    g.seg_log2 = gp.seg_log2;
    g.nseg = gp.nseg;
    g.df_info = df_info;
    g.warp_g = warp_g;
    g.warp_p = warp_p;
    if (gp.cpl == 4) grad_kernel<4><<<gp.grid, kThreads, grad_smem<4>(n), st>>>(g);
    else grad_kernel<8><<<gp.grid, kThreads, grad_smem<8>(n), st>>>(g);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: kernel");
    // the boost is read on the device by the finalize kernel via df_info
    grad_finalize_kernel<<<(n * n + 127) / 128, 128, 0, st>>>(warp_g, warp_p, gp.nwarps, n, exp_out, col_e,
                                                            df_info, d_grad, d_perm, d_perm4);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: finalize");
    return GBPERM_OK;
}

}  // namespace gbperm

using namespace gbperm;

extern "C" {

size_t gbperm_perm_grad_workspace_size(int64_t n) {
    if (n <= 0 || n > 32) return 256;
    return grad_ws_bytes((int)n, plan_grad((int)n));
}

int gbperm_perm_grad_dev(const void* dA, int64_t n, int64_t ld, void* d_perm, void* d_perm_dd, void* d_grad,
                         void* workspace, size_t workspace_bytes, void* stream) {
    if (n < 1 || n > 32) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_grad: n must be in 1..32");
    if (!dA || !d_perm || !d_grad || !workspace) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: null pointer");
    if (ld < n) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: ld < n");
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: workspace must be 256-byte aligned");
    return run_grad_dev(static_cast<const double2*>(dA), ld, (int)n, workspace, workspace_bytes,
                        static_cast<double*>(d_grad), static_cast<double*>(d_perm), static_cast<double*>(d_perm_dd),
                        static_cast<cudaStream_t>(stream), nullptr);
}

int gbperm_perm_grad(const double* A, int64_t n, int64_t ld, double* perm, double* perm_dd, double* grad,
                     gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!perm || !grad) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad: null output");
    if (n < 1 || n > 32) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_grad: n must be in 1..32");
    if (!A || ld < n) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad: bad matrix");
    if (!all_finite(A, n, n, ld)) {
        perm[0] = perm[1] = NAN;
        for (int64_t e = 0; e < 2 * n * n; ++e) grad[e] = NAN;
        return GBPERM_OK;
    }
    int boost = 0;
    if (!df_boost(A, n, n, ld, nullptr, nullptr, &boost))
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_grad: matrix dynamic range beyond the double-float product");
    GradPlan gp = plan_grad((int)n);
    size_t mat_bytes = align_up((size_t)n * n * sizeof(double2), 256);
    size_t ws = grad_ws_bytes((int)n, gp);
    ThreadCtx& c = thread_ctx();
    int rc = c.ensure(mat_bytes * 2 + 256 + ws);
    if (rc) return rc;
    char* base = static_cast<char*>(c.dbuf);
    double2* dA = reinterpret_cast<double2*>(base);
    double* dgrad = reinterpret_cast<double*>(base + mat_bytes);
    double* dperm = reinterpret_cast<double*>(base + 2 * mat_bytes);
    void* dws = base + 2 * mat_bytes + 256;
    cudaError_t e = cudaMemcpy2DAsync(dA, n * sizeof(double2), A, ld * sizeof(double2), n * sizeof(double2), n,
                                      cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: upload");
    if (stats) cudaEventRecord(c.ev0, c.stream);
    GradPlan used;
    rc = run_grad_dev(dA, n, (int)n, dws, ws, dgrad, dperm, dperm + 2, c.stream, &used);
    if (rc) return rc;
    if (stats) cudaEventRecord(c.ev1, c.stream);
    double h[6];
    e = cudaMemcpyAsync(grad, dgrad, (size_t)n * n * sizeof(double2), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dperm, sizeof(h), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: kernel");
    perm[0] = h[0];
    perm[1] = h[1];
    if (perm_dd) std::memcpy(perm_dd, h + 2, 4 * sizeof(double));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        stats->kernel_ms = ms;
        stats->steps = std::ldexp(1.0, (int)n - 1);
        stats->flops = 8.0 * (double)n * stats->steps;
        stats->launches = 4;
        stats->grid = used.grid;
        stats->seg_log2 = used.seg_log2;
        stats->arith = GBPERM_ARITH_DF32;
    }
    return GBPERM_OK;
}

}  // extern "C"
