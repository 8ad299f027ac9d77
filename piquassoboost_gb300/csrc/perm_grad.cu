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
// Per step and lane (CPL columns): prefix products of the lane's columns
// (which also give its partial product), the other three lanes' partials
// (shuffles), then a suffix chain seeded with the signed exclusive product,
// so W_c = prefix_c x suffix_c: 3 CPL - 1 double-float complex products for
// the CPL gradient columns, one more for the permanent term on the group's
// first lane.  Running sums are added
// with an exact two-sum of the high parts and renormalised every 8 steps.
//
// Layout: GROUP = 4 lanes share a Gray walk, lane g owns columns
// [g*CPL, (g+1)*CPL); the 8 groups of a warp walk 8 aligned ranges in
// lockstep.  The per-step row update of G is a reduce-scatter over the 8
// groups (lane (g, grp) ends with column g*CPL + grp), added into the warp's
// own n x n double-float G tile in shared memory.  The flip sign is the same
// for all 8 walks except at the middle step of a walk, so it is applied after
// the reduction.  Warp tiles are written to global memory and summed in a
// fixed order by two finalize kernels.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
constexpr int kGroup = 4;
constexpr int kGroups = 32 / kGroup;  // walks per warp
constexpr int kChunk = 1024;          // steps between folds of Q into G
constexpr int kFinWarps = 64;         // warp tiles per partial of the first finalize stage

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
}

__device__ __forceinline__ cf shfl_cf(const cf& v, int src) {
    return cf{__shfl_sync(0xffffffffu, v.rh, src), __shfl_sync(0xffffffffu, v.rl, src),
              __shfl_sync(0xffffffffu, v.ih, src), __shfl_sync(0xffffffffu, v.il, src)};
}

// a += b without renormalisation: exact two-sum of the high parts, the low
// parts and the rounding error collected in the low word.  Over m such adds
// the low word stays below ~m 2^-24 of the running magnitude, so a
// renormalisation every few adds keeps the pair accurate to ~2^-44.
__device__ __forceinline__ void df_add_lazy(float& ah, float& al, float bh, float bl) {
    float s, e;
    two_sum_f(ah, bh, s, e);
    ah = s;
    al = __fadd_rn(al, __fadd_rn(bl, e));
}

__device__ __forceinline__ void df_renorm(float& h, float& l) {
    float s, e;
    two_sum_f(h, l, s, e);
    h = s;
    l = e;
}

__device__ __forceinline__ cf cf_add_lazy(const cf& a, const cf& b) {
    cf r = a;
    df_add_lazy(r.rh, r.rl, b.rh, b.rl);
    df_add_lazy(r.ih, r.il, b.ih, b.il);
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
    unsigned long long nseg;   // walks
    const int* df_info;        // {boost, ok}
    float4* warp_g;            // per warp: n x n complex double-float tiles (re_h, re_l, im_h, im_l)
    float4* warp_p;            // per warp: permanent partial
};

// Reduce-scatter of v[0..CPL) over the kGroups groups of a warp (lanes with
// equal g): afterwards lane (g, grp) holds, in v[0], the sum over groups of
// column g*CPL + (grp % CPL) (CPL <= kGroups).  The ownership pattern is
// fixed: at each halving stage with mask m, the lane with (grp & m) keeps
// the upper half.  The sums are lazily normalised pairs.
template <int CPL>
__device__ __forceinline__ cf reduce_scatter(cf (&v)[CPL], int grp) {
    int width = CPL;
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
                    v[c] = cf_add_lazy(keep, recv);
                }
            }
            width = half;
        } else {
            cf recv = shfl_xor_cf(v[0], m * kGroup);
            v[0] = cf_add_lazy(v[0], recv);
        }
    }
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
    const bool writer = (grp & (kGroups / CPL - 1)) == 0 && my_col < n;
    const int L = p.seg_log2;
    const unsigned long long Lsteps = 1ull << L;
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (kThreads / 32);
    const unsigned long long gwarp = (unsigned long long)blockIdx.x * (kThreads / 32) + warp;
    const int lbase = lane - g;
    long long cre[CPL], cim[CPL];
    cf Q[CPL];
    float prh = 0.f, prl = 0.f, pih = 0.f, pil = 0.f;  // permanent partial (group leader)

    auto g_add = [&](int r, const cf& s) {
        if (writer) {
            float4 gg = G[r * NP + my_col];
            df_acc(gg.x, gg.y, s.rh, s.rl);
            df_acc(gg.z, gg.w, s.ih, s.il);
            G[r * NP + my_col] = gg;
        }
    };
    // fold Q into every row of G: G[r] += delta_r * Q (the end term), then Q = 0
    auto fold_all = [&](unsigned long long idx) {
        const unsigned long long gray = idx ^ (idx >> 1);
        for (int r = 0; r < n; ++r) {
            // delta_r = -1 when bit (n-1-r) of the Gray code is set (row 0: +1)
            const bool neg = r > 0 && ((gray >> (n - 1 - r)) & 1ull);
            cf v[CPL];
#pragma unroll
            for (int c = 0; c < CPL; ++c) v[c] = cf_scale_sign(Q[c], neg ? 0x80000000u : 0u);
            g_add(r, reduce_scatter<CPL>(v, grp));
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) Q[c] = cf{0.f, 0.f, 0.f, 0.f};
    };

    for (unsigned long long wb = gwarp * kGroups; wb < p.nseg; wb += warps_total * kGroups) {
        const unsigned long long s_raw = wb + grp;
        const bool active = s_raw < p.nseg;
        const unsigned long long i0 = (active ? s_raw : 0ull) << L;
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
        // inactive walks (past the end of the range) carry weight 0
        const float wgt = active ? 1.f : 0.f;
        for (unsigned long long k = 0; k < Lsteps; ++k) {
            const unsigned long long idx = i0 + k;
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;                  // warp-uniform
                const int r = n - 1 - b;                                    // the row that flips
                const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;  // new delta_r = -1
                if ((k % kChunk) == 0) {
                    // chunk boundary: end term at idx-1 for every row, Q = 0;
                    // the flip term of this step would then add 2 * 0
                    fold_all(idx - 1);
                } else if (b + 1 < L) {
                    // flip term G[r] += 2 delta_r(k-1) Q(k-1), delta_r(k-1) = +1
                    // when the row now turns -1; bits b, b+1 of idx are bits
                    // of k here, so the sign is the same for all walks
                    cf v[CPL];
#pragma unroll
                    for (int c = 0; c < CPL; ++c) v[c] = Q[c];
                    cf s = reduce_scatter<CPL>(v, grp);
                    const float f = sub ? 2.f : -2.f;
                    s.rh = __fmul_rn(s.rh, f);
                    s.rl = __fmul_rn(s.rl, f);
                    s.ih = __fmul_rn(s.ih, f);
                    s.il = __fmul_rn(s.il, f);
                    g_add(r, s);
                } else {
                    // middle step of the walk: the sign depends on the walk
                    cf v[CPL];
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        cf q = Q[c];
                        q.rh = __fmul_rn(q.rh, 2.f);
                        q.rl = __fmul_rn(q.rl, 2.f);
                        q.ih = __fmul_rn(q.ih, 2.f);
                        q.il = __fmul_rn(q.il, 2.f);
                        v[c] = cf_scale_sign(q, sub ? 0u : 0x80000000u);
                    }
                    g_add(r, reduce_scatter<CPL>(v, grp));
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
            // prefix products pre[c] = prod_{c' < c} x_c' (pre[0] = 1 is implicit);
            // the last one times x[CPL-1] is the lane's partial product
            cf pre[CPL];
            cf part = x[0];
            if (CPL > 1) {
                pre[1] = x[0];
#pragma unroll
                for (int c = 2; c < CPL; ++c) pre[c] = cf_mul(pre[c - 1], x[c - 1]);
                part = cf_mul(pre[CPL - 1], x[CPL - 1]);
            }
            // product of the other three lanes' partials (gathered in the group)
            cf o1 = shfl_cf(part, lbase + ((g + 1) & 3));
            cf o2 = shfl_cf(part, lbase + ((g + 2) & 3));
            cf o3 = shfl_cf(part, lbase + ((g + 3) & 3));
            cf seed = cf_scale_sign(cf_mul(cf_mul(o1, o2), o3), sbit);  // s(delta) folded in once
            seed.rh = __fmul_rn(seed.rh, wgt);
            seed.rl = __fmul_rn(seed.rl, wgt);
            seed.ih = __fmul_rn(seed.ih, wgt);
            seed.il = __fmul_rn(seed.il, wgt);
            // permanent term (leader)
            if (g == 0) {
                cf t = cf_mul(seed, part);
                df_add_lazy(prh, prl, t.rh, t.rl);
                df_add_lazy(pih, pil, t.ih, t.il);
            }
            // W_c = seed * prod_{c' > c} x_c' * pre[c]
            cf suf = seed;
#pragma unroll
            for (int c = CPL - 1; c >= 0; --c) {
                cf w = (c == 0) ? suf : cf_mul(pre[c], suf);
                Q[c] = cf_add_lazy(Q[c], w);
                if (c > 0) suf = cf_mul(suf, x[c]);
            }
            if ((k & 7ull) == 7ull) {
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    df_renorm(Q[c].rh, Q[c].rl);
                    df_renorm(Q[c].ih, Q[c].il);
                }
                df_renorm(prh, prl);
                df_renorm(pih, pil);
            }
        }
        // end term of the walk
        fold_all(i0 + Lsteps - 1);
    }
    __syncwarp();
    // write the warp's G tile and permanent partial
    float4* outg = p.warp_g + (size_t)gwarp * n * n;
    for (int e = lane; e < n * n; e += 32) {
        int r = e / n, j = e % n;
        outg[e] = G[r * NP + j];
    }
    // permanent: sum the 8 leaders' partials
    df_renorm(prh, prl);
    df_renorm(pih, pil);
    cf pp{prh, prl, pih, pil};
#pragma unroll
    for (int m = kGroup; m < 32; m <<= 1) {
        cf o = shfl_xor_cf(pp, m);
        df_acc(pp.rh, pp.rl, o.rh, o.rl);
        df_acc(pp.ih, pp.il, o.ih, o.il);
    }
    if (lane == 0) p.warp_p[gwarp] = make_float4(pp.rh, pp.rl, pp.ih, pp.il);
}

// First finalize stage: element e < n*n of the gradient (e == n*n: the
// permanent) summed over kFinWarps consecutive warp tiles, in double-float,
// one partial per (chunk, element).  Every SM takes part.
__global__ void grad_partial_kernel(const float4* warp_g, const float4* warp_p, int nwarps, int n,
                                    float4* part) {
    const int ne = n * n + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int w0 = blockIdx.y * kFinWarps;
    const int w1 = min(w0 + kFinWarps, nwarps);
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int w = w0; w < w1; ++w) {
        const float4 v = e < n * n ? warp_g[(size_t)w * n * n + e] : warp_p[w];
        df_acc(rh, rl, v.x, v.y);
        df_acc(ih, il, v.z, v.w);
    }
    part[(size_t)blockIdx.y * ne + e] = make_float4(rh, rl, ih, il);
}

// Second stage: sum the chunk partials in a fixed order in double-double,
// scale, write the gradient (complex128, n x n row-major) and the permanent.
__global__ void grad_finalize_kernel(const float4* part, int nchunks, int n, const int* exp_in, const int* col_e,
                                     const int* df_info, double* grad, double* perm2, double* perm4) {
    const int ne = n * n + 1;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    if (df_info[1] == 0) {
        if (e < n * n) {
            grad[2 * e] = grad[2 * e + 1] = nan("");
        } else {
            perm2[0] = perm2[1] = nan("");
            if (perm4) perm4[0] = perm4[1] = perm4[2] = perm4[3] = nan("");
        }
        return;
    }
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    for (int c = 0; c < nchunks; ++c) {
        const float4 v = part[(size_t)c * ne + e];
        acc.re = dd_add(acc.re, dd{(double)v.x, (double)v.y});
        acc.im = dd_add(acc.im, dd{(double)v.z, (double)v.w});
    }
    if (e < n * n) {
        const int l = e % n;
        // W_l omits column l: remove its factor from the permanent's scale
        const int ex = *exp_in - (col_e[l] - df_info[0]);
        double r2[2];
        write_result(acc, ex, r2, nullptr);
        grad[2 * e] = r2[0];
        grad[2 * e + 1] = r2[1];
    } else {
        write_result(acc, *exp_in, perm2, perm4);
    }
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
    int nchunks = 1;  // partials of the first finalize stage
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
    const int grid_full = sms * nb;
    const int slog = n - 1;
    // walk length 2^l: the walks are dealt to the resident walk slots in
    // passes, so the time goes as passes x (2^l + per-walk cost), the
    // per-walk cost (start-up and the final fold of n rows) being about
    // 0.2 n + 16 steps.  Ties go to the longer walk.
    const unsigned long long slots = (unsigned long long)grid_full * (kThreads / 32) * kGroups;
    double best = 1e300;
    int best_l = slog;
    for (int l = slog; l >= 0; --l) {
        const unsigned long long nseg = 1ull << (slog - l);
        const double passes = (double)((nseg + slots - 1) / slots);
        const double cost = passes * (std::ldexp(1.0, l) + 0.2 * n + 16.0);
        if (cost < best * (1.0 - 1e-9)) {
            best = cost;
            best_l = l;
        }
    }
    gp.seg_log2 = best_l;
    gp.nseg = 1ull << (slog - best_l);
    unsigned long long warps_needed = (gp.nseg + kGroups - 1) / kGroups;
    unsigned long long blocks_needed = (warps_needed + 3) / 4;
    gp.grid = (int)(blocks_needed < (unsigned long long)grid_full ? blocks_needed : (unsigned long long)grid_full);
    if (gp.grid < 1) gp.grid = 1;
    gp.nwarps = gp.grid * (kThreads / 32);
    gp.nchunks = (gp.nwarps + kFinWarps - 1) / kFinWarps;
    return gp;
}

static size_t grad_ws_bytes(int n, const GradPlan& gp) {
    size_t mat = align_up((size_t)n * n * sizeof(longlong2), 256);
    return 2 * mat + 256 + 256 + align_up((size_t)n * sizeof(int), 256) +
           align_up((size_t)gp.nwarps * n * n * sizeof(float4), 256) + align_up((size_t)gp.nwarps * sizeof(float4), 256) +
           align_up((size_t)gp.nchunks * (n * n + 1) * sizeof(float4), 256);
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
    off += align_up((size_t)gp.nwarps * sizeof(float4), 256);
    float4* fin_part = reinterpret_cast<float4*>(base + off);
    PrepArgs pa;
    pa.col_e_out = col_e;
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
    const int ne = n * n + 1;
    grad_partial_kernel<<<dim3((ne + 127) / 128, gp.nchunks), 128, 0, st>>>(warp_g, warp_p, gp.nwarps, n, fin_part);
    grad_finalize_kernel<<<(ne + 127) / 128, 128, 0, st>>>(fin_part, gp.nchunks, n, exp_out, col_e, df_info, d_grad,
                                                          d_perm, d_perm4);
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
