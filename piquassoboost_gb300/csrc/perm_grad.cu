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
#include <string>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"
#include "gbperm_fx.cuh"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
constexpr int kGroup = 4;
constexpr int kGroups = 32 / kGroup;  // walks per warp
constexpr int kChunk = 4096;          // steps between folds of Q into G
constexpr int kHot = 8;               // rows of G kept in shared memory (the 8 that flip most often)
constexpr int kFinWarps = 64;         // warp tiles per partial of the first finalize stage

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
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

// One launch serves a batch of equal-size matrices: blockIdx.y is the
// matrix, blockIdx.x the block within it; every per-matrix array is
// consecutive in the matrix index.
struct GradArgs {
    const longlong2* a1;       // per matrix n x n
    const longlong2* a2;
    int n;
    int seg_log2;              // each walk covers 2^seg_log2 Gray steps
    unsigned long long nseg;   // walks per matrix
    const int* df_info;        // per matrix {boost, ok}
    float4* warp_g;            // per matrix and warp: n x n complex double-float tiles (re_h, re_l, im_h, im_l);
                               // the integer-mantissa twin stores double2 tiles (16 bytes too) here
    double* warp_s2 = nullptr; // double-float sweep: per matrix and warp, sum of |term 2^40|^2
    const int* gate = nullptr; // integer-mantissa twin: run only for matrices whose gate[2 i + 1]
                               // is 0 (the double-float product is not in use); null: always
};

// Reduce-scatter of v[0..CPL) over the kGroups walks of a warp (lanes with
// equal g), without selects: every lane keeps the lower half of its
// positions and receives its partner's upper half at each halving stage.
// That adds the same column on both sides because lane (g, grp) stores its
// columns in the order column = position ^ perm_mask<CPL>(grp): the partner
// across stage bit m has the matching bit of the mask flipped, so its upper
// positions hold this lane's lower-position columns.  Afterwards lane
// (g, grp) holds, in v[0], the sum over walks of column g*CPL +
// perm_mask<CPL>(grp); with CPL < kGroups the last stages are all-reduces.
// The sums are lazily normalised pairs.
template <int CPL>
__device__ __forceinline__ int perm_mask(int grp) {
    // log2(kGroups / CPL) low bits of grp are all-reduce stages
    return CPL == 8 ? grp : CPL == 4 ? (grp >> 1) : CPL == 2 ? (grp >> 2) : 0;
}

template <int CPL>
__device__ __forceinline__ cf reduce_scatter(cf (&v)[CPL]) {
    int width = CPL;
#pragma unroll
    for (int m = kGroups / 2; m >= 1; m >>= 1) {
        if (width > 1) {
            const int half = width / 2;
#pragma unroll
            for (int c = 0; c < CPL / 2; ++c)
                if (c < half) v[c] = cf_add_lazy(v[c], shfl_xor_cf(v[c + half], m * kGroup));
            width = half;
        } else {
            v[0] = cf_add_lazy(v[0], shfl_xor_cf(v[0], m * kGroup));
        }
    }
    return v[0];
}

template <int CPL>
__global__ void __launch_bounds__(kThreads, 3) grad_kernel(GradArgs p) {
    constexpr int NP = CPL * kGroup;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a2 = reinterpret_cast<longlong2*>(smem_raw);           // n x NP (interleaved)
    float4* s_g = reinterpret_cast<float4*>(s_a2 + p.n * NP);           // (warps) x kHot x NP
    const int n = p.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane % kGroup, grp = lane / kGroup;
    const int j0 = g * CPL;
    const size_t inst = blockIdx.y;
    const longlong2* A1 = p.a1 + inst * n * n;
    const longlong2* A2 = p.a2 + inst * n * n;
    const int* dfi = p.df_info + 2 * inst;
    // G: the kHot rows that flip most often (rows n-kHot .. n-1) live in a
    // per-warp shared-memory tile; the other rows, which flip at most once
    // every 2^kHot steps, accumulate straight into the warp's own tile in
    // global memory (L2-resident), which is also the kernel's output.
    const int hot0 = n > kHot ? n - kHot : 0;
    float4* G = s_g + (size_t)warp * kHot * NP;
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (kThreads / 32);
    const unsigned long long gwarp = (unsigned long long)blockIdx.x * (kThreads / 32) + warp;
    const size_t slot = inst * warps_total + gwarp;
    float4* outg = p.warp_g + slot * n * n;
    // the step's row table, interleaved by lane: column j = g*CPL + c of row r
    // sits at r*NP + c*kGroup + g, so the four lanes of a walk read four
    // adjacent 16-byte words (one wavefront) when they fetch their c-th column
    for (int e = threadIdx.x; e < n * NP; e += blockDim.x) {
        const int r = e / NP, q = e % NP;
        const int j = (q % kGroup) * CPL + q / kGroup;
        s_a2[e] = j < n ? A2[r * n + j] : make_longlong2(0, 0);
    }
    for (int e = lane; e < kHot * NP; e += 32) G[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int e = lane; e < hot0 * n; e += 32) outg[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    if (dfi[1] == 0) return;  // range check failed: finalize writes NaN
    const DfConv cv = make_dfconv(dfi[0]);
    // register position c of this lane holds column j0 + (c ^ pm)
    const int pm = perm_mask<CPL>(grp);
    const int my_col = j0 + pm;
    // with CPL < kGroups the last stages are all-reduces: one lane per column writes
    const bool writer = (grp & (kGroups / CPL - 1)) == 0 && my_col < n;
    const int L = p.seg_log2;
    const unsigned long long Lsteps = 1ull << L;
    long long cre[CPL], cim[CPL];
    cf Q[CPL];
    // this thread's sum of |term 2^40|^2, in shared memory: a register pair
    // more would make the 8-column shape spill
    __shared__ double s_s2t[kThreads];
    __shared__ float s_s2f[kThreads];  // the same since the last fold, in float
    s_s2t[threadIdx.x] = 0.0;
    s_s2f[threadIdx.x] = 0.f;

    auto g_add = [&](int r, const cf& s) {
        if (writer) {
            float4* dst = r >= hot0 ? G + (r - hot0) * NP + my_col : outg + r * n + my_col;  // r warp-uniform
            float4 gg = *dst;
            df_acc(gg.x, gg.y, s.rh, s.rl);
            df_acc(gg.z, gg.w, s.ih, s.il);
            *dst = gg;
        }
    };

    for (unsigned long long wb = gwarp * kGroups; wb < p.nseg; wb += warps_total * kGroups) {
        const unsigned long long s_raw = wb + grp;
        const bool active = s_raw < p.nseg;
        const unsigned long long i0 = (active ? s_raw : 0ull) << L;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
        // walk-start column sums from the fixed-point matrix in global
        // memory (once per walk): row 0 plus rows 1.. with their signs
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            const int j = j0 + (c ^ pm);
            const longlong2 v = j < n ? A1[j] : make_longlong2(0, 0);
            cre[c] = v.x;
            cim[c] = v.y;
            Q[c] = cf{0.f, 0.f, 0.f, 0.f};
        }
        for (int r = 1; r < n; ++r) {
            const long long m = -(long long)((g0 >> (n - 1 - r)) & 1ull);
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int j = j0 + (c ^ pm);
                const longlong2 v = j < n ? A1[r * n + j] : make_longlong2(0, 0);
                cre[c] += (v.x ^ m) - m;
                cim[c] += (v.y ^ m) - m;
            }
        }
        unsigned int sbit = (unsigned int)(__popcll(g0) & 1) << 31;
        // inactive walks (past the end of the range) carry weight 0
        const float wgt = active ? 1.f : 0.f;
        for (unsigned long long k0 = 0; k0 < Lsteps; k0 += kChunk) {
            const unsigned long long kend = k0 + kChunk < Lsteps ? k0 + kChunk : Lsteps;
            for (unsigned long long k = k0; k < kend; ++k) {
                const unsigned long long idx = i0 + k;
                if (k != 0) {
                    const int b = __ffsll((long long)k) - 1;                  // warp-uniform
                    const int r = n - 1 - b;                                    // the row that flips
                    const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;  // new delta_r = -1
                    // flip term G[r] += 2 delta_r(k-1) Q(k-1), delta_r(k-1) = +1 when
                    // the row now turns -1 (Q is zero right after a fold).  Bits b,
                    // b+1 of idx are bits of k unless b is the walk's top bit, so the
                    // sign is the same for all walks and is applied after the
                    // reduction; at the middle step it is applied per walk before.
                    const bool mid = b + 1 >= L;
                    cf v[CPL];
#pragma unroll
                    for (int c = 0; c < CPL; ++c) v[c] = Q[c];
                    if (mid) {
#pragma unroll
                        for (int c = 0; c < CPL; ++c) {
                            cf q = v[c];
                            q.rh = __fmul_rn(q.rh, 2.f);
                            q.rl = __fmul_rn(q.rl, 2.f);
                            q.ih = __fmul_rn(q.ih, 2.f);
                            q.il = __fmul_rn(q.il, 2.f);
                            v[c] = cf_scale_sign(q, sub ? 0u : 0x80000000u);
                        }
                    }
                    cf s = reduce_scatter<CPL>(v);
                    const float f = mid ? 1.f : (sub ? 2.f : -2.f);
                    s.rh = __fmul_rn(s.rh, f);
                    s.rl = __fmul_rn(s.rl, f);
                    s.ih = __fmul_rn(s.ih, f);
                    s.il = __fmul_rn(s.il, f);
                    g_add(r, s);
                    // column sums: -/+ 2 a_r
                    const long long m = sub ? -1ll : 0ll;
                    const longlong2* a = s_a2 + r * NP + g;
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v2 = a[(c ^ pm) * kGroup];
                        cre[c] += (v2.x ^ m) - m;
                        cim[c] += (v2.y ^ m) - m;
                    }
                    sbit ^= 0x80000000u;
                }
                // column values (padded columns act as 1)
                cf x[CPL];
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    if (j0 + (c ^ pm) < n) {
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
                // product of the other three lanes' partials: the partner's
                // partial (lane g^1) times the other pair's product (g^2, g^3)
                const cf o1 = shfl_xor_cf(part, 1);
                const cf pair = cf_mul(part, o1);
                const cf o23 = shfl_xor_cf(pair, 2);
                // |term|^2 = |pair|^2 |o23|^2, each factor scaled by 2^20 (the
                // range boost centres the terms near 2^-40), for the error
                // estimate: one walk's lane g = 0 adds it
                if (g == 0) {
                    const float ar = pair.rh * 0x1p20f, ai = pair.ih * 0x1p20f;
                    const float br = o23.rh * 0x1p20f, bi = o23.ih * 0x1p20f;
                    s_s2f[threadIdx.x] = fmaf(fmaf(ar, ar, ai * ai), fmaf(br, br, bi * bi), s_s2f[threadIdx.x]);
                }
                cf seed = cf_scale_sign(cf_mul(o1, o23), sbit);  // s(delta) folded in once
                seed.rh = __fmul_rn(seed.rh, wgt);
                seed.rl = __fmul_rn(seed.rl, wgt);
                seed.ih = __fmul_rn(seed.ih, wgt);
                seed.il = __fmul_rn(seed.il, wgt);
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
                }
            }
            s_s2t[threadIdx.x] += (double)s_s2f[threadIdx.x];
            s_s2f[threadIdx.x] = 0.f;
            // end of a chunk (or of the walk): fold Q into every row of G,
            // G[r] += delta_r(kend-1) * Q, then restart Q
            const unsigned long long idx = i0 + kend - 1;
            const unsigned long long gray = idx ^ (idx >> 1);
            for (int r = 0; r < n; ++r) {
                // delta_r = -1 when bit (n-1-r) of the Gray code is set (row 0: +1)
                const bool neg = r > 0 && ((gray >> (n - 1 - r)) & 1ull);
                cf v[CPL];
#pragma unroll
                for (int c = 0; c < CPL; ++c) v[c] = cf_scale_sign(Q[c], neg ? 0x80000000u : 0u);
                g_add(r, reduce_scatter<CPL>(v));
            }
#pragma unroll
            for (int c = 0; c < CPL; ++c) Q[c] = cf{0.f, 0.f, 0.f, 0.f};
        }
    }
    __syncwarp();
    // the hot rows of the warp's tile go to its global tile (the other rows
    // are there already)
    for (int e = lane; e < (n - hot0) * n; e += 32) {
        const int rr = e / n, j = e % n;
        outg[(hot0 + rr) * n + j] = G[rr * NP + j];
    }
    if (p.warp_s2) {
        const double s2 = warp_sum_d(s_s2t[threadIdx.x]);
        if (lane == 0) p.warp_s2[slot] = s2;
    }
}

// ------------------------------------------------ integer-mantissa twin
// The same sweep with the product on 64-bit integer mantissas
// (gbperm_fx.cuh): prefix, partial, butterfly and suffix products as above,
// each multiply keeping 55-57 significant bits; the running sums Q, the
// reduce-scatter of the flipping row and the G tiles in double (FP64 pipe).
// Padded columns hold the exact column value 1 (2^62 in the fixed point),
// which the integer multiply passes through to within half a unit.  It is
// the double-float sweep's fallback for matrices whose range check fails or
// whose error estimate is above 1e-10 (gate), and the whole sweep when the
// integer-mantissa product is requested (no gate).
template <int CPL>
__device__ __forceinline__ double2 reduce_scatter_d(double2 (&v)[CPL]) {
    int width = CPL;
#pragma unroll
    for (int m = kGroups / 2; m >= 1; m >>= 1) {
        if (width > 1) {
            const int half = width / 2;
#pragma unroll
            for (int c = 0; c < CPL / 2; ++c)
                if (c < half) {
                    v[c].x += __shfl_xor_sync(0xffffffffu, v[c + half].x, m * kGroup);
                    v[c].y += __shfl_xor_sync(0xffffffffu, v[c + half].y, m * kGroup);
                }
            width = half;
        } else {
            v[0].x += __shfl_xor_sync(0xffffffffu, v[0].x, m * kGroup);
            v[0].y += __shfl_xor_sync(0xffffffffu, v[0].y, m * kGroup);
        }
    }
    return v[0];
}

template <int CPL>
__global__ void __launch_bounds__(kThreads, 3) grad_fx_kernel(GradArgs p) {
    constexpr int NP = CPL * kGroup;
    constexpr long long kOne = 1ll << GBPERM_FIX_BITS;  // the column value 1
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a2 = reinterpret_cast<longlong2*>(smem_raw);           // n x NP (interleaved)
    double2* s_g = reinterpret_cast<double2*>(s_a2 + p.n * NP);         // (warps) x kHot x NP
    const int n = p.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane % kGroup, grp = lane / kGroup;
    const int j0 = g * CPL;
    const size_t inst = blockIdx.y;
    if (p.gate && p.gate[2 * inst + 1] != 0) return;  // the double-float result stands
    const longlong2* A1 = p.a1 + inst * n * n;
    const longlong2* A2 = p.a2 + inst * n * n;
    const int hot0 = n > kHot ? n - kHot : 0;
    double2* G = s_g + (size_t)warp * kHot * NP;
    const unsigned long long warps_total = (unsigned long long)gridDim.x * (kThreads / 32);
    const unsigned long long gwarp = (unsigned long long)blockIdx.x * (kThreads / 32) + warp;
    const size_t slot = inst * warps_total + gwarp;
    double2* outg = reinterpret_cast<double2*>(p.warp_g) + slot * n * n;
    for (int e = threadIdx.x; e < n * NP; e += blockDim.x) {
        const int r = e / NP, q = e % NP;
        const int j = (q % kGroup) * CPL + q / kGroup;
        s_a2[e] = j < n ? A2[r * n + j] : make_longlong2(0, 0);
    }
    for (int e = lane; e < kHot * NP; e += 32) G[e] = make_double2(0.0, 0.0);
    for (int e = lane; e < hot0 * n; e += 32) outg[e] = make_double2(0.0, 0.0);
    __syncthreads();
    const int pm = perm_mask<CPL>(grp);
    const int my_col = j0 + pm;
    const bool writer = (grp & (kGroups / CPL - 1)) == 0 && my_col < n;
    const int L = p.seg_log2;
    const unsigned long long Lsteps = 1ull << L;
    long long cre[CPL], cim[CPL];
    double2 Q[CPL];

    auto g_add = [&](int r, const double2& v) {
        if (writer) {
            double2* dst = r >= hot0 ? G + (r - hot0) * NP + my_col : outg + r * n + my_col;  // r warp-uniform
            double2 gg = *dst;
            gg.x += v.x;
            gg.y += v.y;
            *dst = gg;
        }
    };

    for (unsigned long long wb = gwarp * kGroups; wb < p.nseg; wb += warps_total * kGroups) {
        const unsigned long long s_raw = wb + grp;
        const bool active = s_raw < p.nseg;
        const unsigned long long i0 = (active ? s_raw : 0ull) << L;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            const int j = j0 + (c ^ pm);
            const longlong2 v = j < n ? A1[j] : make_longlong2(kOne, 0);
            cre[c] = v.x;
            cim[c] = v.y;
            Q[c] = make_double2(0.0, 0.0);
        }
        for (int r = 1; r < n; ++r) {
            const long long m = -(long long)((g0 >> (n - 1 - r)) & 1ull);
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int j = j0 + (c ^ pm);
                const longlong2 v = j < n ? A1[r * n + j] : make_longlong2(0, 0);
                cre[c] += (v.x ^ m) - m;
                cim[c] += (v.y ^ m) - m;
            }
        }
        unsigned long long sbit = (unsigned long long)(__popcll(g0) & 1) << 63;
        for (unsigned long long k0 = 0; k0 < Lsteps; k0 += kChunk) {
            const unsigned long long kend = k0 + kChunk < Lsteps ? k0 + kChunk : Lsteps;
            for (unsigned long long k = k0; k < kend; ++k) {
                const unsigned long long idx = i0 + k;
                if (k != 0) {
                    const int b = __ffsll((long long)k) - 1;                  // warp-uniform
                    const int r = n - 1 - b;                                    // the row that flips
                    const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;  // new delta_r = -1
                    const bool mid = b + 1 >= L;
                    double2 v[CPL];
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        v[c] = Q[c];
                        if (mid) {
                            const double f = sub ? 2.0 : -2.0;
                            v[c].x *= f;
                            v[c].y *= f;
                        }
                    }
                    double2 sv = reduce_scatter_d<CPL>(v);
                    if (!mid) {
                        const double f = sub ? 2.0 : -2.0;
                        sv.x *= f;
                        sv.y *= f;
                    }
                    g_add(r, sv);
                    const long long m = sub ? -1ll : 0ll;
                    const longlong2* a = s_a2 + r * NP + g;
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v2 = a[(c ^ pm) * kGroup];
                        cre[c] += (v2.x ^ m) - m;
                        cim[c] += (v2.y ^ m) - m;
                    }
                    sbit ^= 0x8000000000000000ull;
                }
                // prefix products pre[c] = prod_{c' < c} x_c' (normalised,
                // shift counts spre), the lane's partial product `part`
                fxl pre[CPL];
                int spre[CPL];
                fxl part;
                int spart;
                if (CPL > 1) {
                    spre[1] = fx_norm_col(cre[0], cim[0], pre[1]);
#pragma unroll
                    for (int c = 2; c < CPL; ++c) {
                        long long rr, ri;
                        fx_mul(pre[c - 1], fx_col(cre[c - 1], cim[c - 1]), rr, ri);
                        spre[c] = spre[c - 1] - 1 + fx_norm(rr, ri, pre[c]);
                    }
                    long long rr, ri;
                    fx_mul(pre[CPL - 1], fx_col(cre[CPL - 1], cim[CPL - 1]), rr, ri);
                    spart = spre[CPL - 1] - 1 + fx_norm(rr, ri, part);
                } else {
                    spart = fx_norm_col(cre[0], cim[0], part);
                }
                // product of the other three lanes' partials (fx_mul is
                // symmetric, so partners compute identical values)
                const fxl o1 = shfl_xor_fxl(part, 1);
                const int so1 = __shfl_xor_sync(0xffffffffu, spart, 1);
                fxl pair;
                int spair;
                {
                    long long rr, ri;
                    fx_mul(part, o1, rr, ri);
                    spair = spart + so1 - 1 + fx_norm(rr, ri, pair);
                }
                const fxl o23 = shfl_xor_fxl(pair, 2);
                const int so23 = __shfl_xor_sync(0xffffffffu, spair, 2);
                fxl suf;
                int ssuf;
                {
                    long long rr, ri;
                    fx_mul(o1, o23, rr, ri);
                    ssuf = so1 + so23 - 1 + fx_norm(rr, ri, suf);
                }
                // W_c = pre[c] * (others) * prod_{c' > c} x_c', signed, into Q
#pragma unroll
                for (int c = CPL - 1; c >= 0; --c) {
                    long long wr, wi;
                    int sw;
                    if (c == 0) {
                        wr = fx_join(suf.rh, suf.rl);
                        wi = fx_join(suf.ih, suf.il);
                        sw = ssuf;
                    } else {
                        fx_mul(pre[c], suf, wr, wi);
                        sw = spre[c] + ssuf - 1;
                    }
                    if (active) {
                        const int e = -61 - sw;
                        Q[c].x += __longlong_as_double(__double_as_longlong(fx_to_double_alu(wr, e)) ^ (long long)sbit);
                        Q[c].y += __longlong_as_double(__double_as_longlong(fx_to_double_alu(wi, e)) ^ (long long)sbit);
                    }
                    if (c > 0) {
                        long long rr, ri;
                        fx_mul(suf, fx_col(cre[c], cim[c]), rr, ri);
                        ssuf = ssuf - 1 + fx_norm(rr, ri, suf);
                    }
                }
            }
            // end of a chunk (or of the walk): G[r] += delta_r(kend-1) Q, restart Q
            const unsigned long long idx = i0 + kend - 1;
            const unsigned long long gray = idx ^ (idx >> 1);
            for (int r = 0; r < n; ++r) {
                const bool neg = r > 0 && ((gray >> (n - 1 - r)) & 1ull);
                double2 v[CPL];
#pragma unroll
                for (int c = 0; c < CPL; ++c) v[c] = neg ? make_double2(-Q[c].x, -Q[c].y) : Q[c];
                g_add(r, reduce_scatter_d<CPL>(v));
            }
#pragma unroll
            for (int c = 0; c < CPL; ++c) Q[c] = make_double2(0.0, 0.0);
        }
    }
    __syncwarp();
    for (int e = lane; e < (n - hot0) * n; e += 32) {
        const int rr = e / n, j = e % n;
        outg[(hot0 + rr) * n + j] = G[rr * NP + j];
    }
}

// Finalize stages of the twin: kFinWarps warp tiles per partial summed in
// double in a fixed order, then the partials in double-double; the exponent
// is the FP64 one (no boost).  Gated like the sweep.
__global__ void grad_partial_fx_kernel(const double2* warp_g, int nwarps, int n, double2* part, const int* gate) {
    const int ne = n * n;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const size_t inst = blockIdx.z;
    if (gate && gate[2 * inst + 1] != 0) return;
    warp_g += inst * nwarps * n * n;
    part += inst * gridDim.y * ne;
    const int w0 = blockIdx.y * kFinWarps;
    const int w1 = min(w0 + kFinWarps, nwarps);
    double re = 0.0, im = 0.0;
    for (int w = w0; w < w1; ++w) {
        const double2 v = warp_g[(size_t)w * n * n + e];
        re += v.x;
        im += v.y;
    }
    part[(size_t)blockIdx.y * ne + e] = make_double2(re, im);
}

__global__ void grad_finalize_fx_kernel(const double2* part, int nchunks, int n, const int* exp64, const int* col_e,
                                        const int* row_k, const int* gate, double* grad) {
    const int ne = n * n;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const size_t inst = blockIdx.y;
    if (gate && gate[2 * inst + 1] != 0) return;
    part += inst * nchunks * ne;
    exp64 += inst;
    col_e += inst * n;
    row_k += inst * n;
    grad += inst * 2 * n * n;
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    for (int c = 0; c < nchunks; ++c) {
        const double2 v = part[(size_t)c * ne + e];
        acc.re = dd_add_d(acc.re, v.x);
        acc.im = dd_add_d(acc.im, v.y);
    }
    const int l = e % n, k = e / n;
    double r2[2];
    write_result(acc, *exp64 - col_e[l] - row_k[k], r2, nullptr);
    grad[2 * e] = r2[0];
    grad[2 * e + 1] = r2[1];
}

// First finalize stage: element e of the gradient summed over kFinWarps
// consecutive warp tiles, in double-float, one partial per (chunk, element).
// Every SM takes part.
__global__ void grad_partial_kernel(const float4* warp_g, int nwarps, int n, float4* part) {
    const int ne = n * n;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const size_t inst = blockIdx.z;  // matrix of a batch
    warp_g += inst * nwarps * n * n;
    part += inst * gridDim.y * ne;
    const int w0 = blockIdx.y * kFinWarps;
    const int w1 = min(w0 + kFinWarps, nwarps);
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int w = w0; w < w1; ++w) {
        const float4 v = warp_g[(size_t)w * n * n + e];
        df_acc(rh, rl, v.x, v.y);
        df_acc(ih, il, v.z, v.w);
    }
    part[(size_t)blockIdx.y * ne + e] = make_float4(rh, rl, ih, il);
}

// Second stage: sum the chunk partials in a fixed order in double-double,
// scale, write the gradient (complex128, n x n row-major).
__global__ void grad_finalize_kernel(const float4* part, int nchunks, int n, const int* exp_in, const int* col_e,
                                     const int* row_k, const int* df_info, double* grad) {
    const int ne = n * n;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const size_t inst = blockIdx.y;  // matrix of a batch
    part += inst * nchunks * ne;
    exp_in += inst;
    col_e += inst * n;
    row_k += inst * n;
    df_info += 2 * inst;
    grad += inst * 2 * n * n;
    if (df_info[1] == 0) {
        grad[2 * e] = grad[2 * e + 1] = nan("");
        return;
    }
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    for (int c = 0; c < nchunks; ++c) {
        const float4 v = part[(size_t)c * ne + e];
        acc.re = dd_add(acc.re, dd{(double)v.x, (double)v.y});
        acc.im = dd_add(acc.im, dd{(double)v.z, (double)v.w});
    }
    const int l = e % n, k = e / n;
    // the minor omits row k and column l: remove column l's factor (its
    // 2^-e_l scaling and the range boost) and row k's 2^-k_k balancing
    // from the permanent's scale
    const int ex = *exp_in - (col_e[l] - df_info[0]) - row_k[k];
    double r2[2];
    write_result(acc, ex, r2, nullptr);
    grad[2 * e] = r2[0];
    grad[2 * e + 1] = r2[1];
}

__device__ __forceinline__ dd two_prod(double a, double b) {
    const double p = a * b;
    return dd{p, fma(a, b, -p)};
}

// The permanent from its gradient: perm is linear in every row, so
// perm = sum_l a_kl dperm/da_kl for each row k (Laplace expansion along k).
// One warp per matrix: lane k estimates the condition
// sum_l |a_kl| |G_kl| / |sum| of row k in plain FP64, and the
// best-conditioned row is then summed in double-double (products exact by
// FMA) with one term per lane, so the sweep needs no separate permanent
// term.
//
// Two passes share it.  After the double-float sweep (est != null): a matrix
// whose range check failed gets NaN here (its twin pass follows); otherwise
// lane 0 also forms the relative rounding-error estimate of the sweep,
//     sqrt(n) 2^-46 sqrt(sum |term 2^40|^2) 2^-40 / |perm 2^-exp|,
// (the model of the forward double-float kernels; the gradient entries are
// minors of the same matrix) and, when it is above 1e-10 and `escalate` is
// set, clears df_info[1] so that the integer-mantissa twin queued behind
// recomputes the gradient and the permanent.  After the twin (est == null):
// matrices whose df_info[1] is set keep the double-float values (df_info
// null: every matrix is the twin's).
__global__ void grad_perm_kernel(const double2* A, long long ld, long long stride, int n, const double* grad,
                                 int* df_info, double* perm2, double* perm4, const double* warp_s2, int nwarps,
                                 const int* exp_in, double* est, int escalate) {
    const size_t inst = blockIdx.x;
    const int k = threadIdx.x;
    A += inst * stride;
    grad += inst * 2 * n * n;
    if (df_info) df_info += 2 * inst;
    perm2 += 2 * inst;
    if (perm4) perm4 += 4 * inst;
    if (est) {
        if (df_info[1] == 0) {
            if (k == 0) {
                perm2[0] = perm2[1] = nan("");
                if (perm4) perm4[0] = perm4[1] = perm4[2] = perm4[3] = nan("");
                est[inst] = -1.0;
            }
            return;
        }
    } else if (df_info && df_info[1] != 0) {
        return;
    }
    // condition estimate of every row's expansion in plain FP64 (it only
    // picks the row): |sum| and sum_l |a_kl| |G_kl| in the 1-norm of C
    double cond = INFINITY;
    if (k < n) {
        double sr = 0.0, si = 0.0, mag = 0.0;
        for (int l = 0; l < n; ++l) {
            const double2 a = A[(long long)k * ld + l];
            const double gr = grad[2 * (k * n + l)], gi = grad[2 * (k * n + l) + 1];
            sr = fma(a.x, gr, fma(-a.y, gi, sr));
            si = fma(a.x, gi, fma(a.y, gr, si));
            mag += (fabs(a.x) + fabs(a.y)) * (fabs(gr) + fabs(gi));
        }
        const double absv = fabs(sr) + fabs(si);
        cond = absv > 0.0 ? mag / absv : (mag > 0.0 ? INFINITY : 1.0);
    }
    int best = k;
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        const double oc = __shfl_xor_sync(0xffffffffu, cond, m);
        const int ob = __shfl_xor_sync(0xffffffffu, best, m);
        if (oc < cond || (oc == cond && ob < best)) {
            cond = oc;
            best = ob;
        }
    }
    // the chosen row exactly: lane l holds a_bl G_bl (exact products as
    // double-doubles), summed by a butterfly; fl addition commutes and TwoSum
    // is exact, so every lane ends with the same total
    cdd s{{0.0, 0.0}, {0.0, 0.0}};
    if (k < n) {
        const double2 a = A[(long long)best * ld + k];
        const double gr = grad[2 * (best * n + k)], gi = grad[2 * (best * n + k) + 1];
        s.re = dd_add(two_prod(a.x, gr), two_prod(-a.y, gi));
        s.im = dd_add(two_prod(a.x, gi), two_prod(a.y, gr));
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
        cdd o;
        o.re.hi = __shfl_xor_sync(0xffffffffu, s.re.hi, m);
        o.re.lo = __shfl_xor_sync(0xffffffffu, s.re.lo, m);
        o.im.hi = __shfl_xor_sync(0xffffffffu, s.im.hi, m);
        o.im.lo = __shfl_xor_sync(0xffffffffu, s.im.lo, m);
        s = cdd_add(s, o);
    }
    if (k == 0) {
        perm2[0] = s.re.hi + s.re.lo;
        perm2[1] = s.im.hi + s.im.lo;
        if (perm4) {
            perm4[0] = s.re.hi;
            perm4[1] = s.im.hi;
            perm4[2] = s.re.lo;
            perm4[3] = s.im.lo;
        }
    }
    if (est) {
        // the sweep's sum of |term 2^40|^2 over the matrix's warps, in a fixed order
        double q = 0.0;
        for (int w = k; w < nwarps; w += 32) q += warp_s2[inst * nwarps + w];
        q = warp_sum_d(q);
        if (k == 0) {
            const double mag = ldexp(hypot(s.re.hi, s.im.hi), -exp_in[inst]);
            const double e = sqrt((double)n) * 0x1p-46 * sqrt(q) * 0x1p-40 / mag;
            est[inst] = e;
            if (escalate && !(e <= kDfEscalate)) df_info[1] = 0;
        }
    }
}

template <int CPL>
size_t grad_smem(int n) {
    return (size_t)n * CPL * kGroup * sizeof(longlong2) + (size_t)(kThreads / 32) * kHot * CPL * kGroup * sizeof(float4);
}

}  // namespace

struct GradPlan {
    int cpl = 8;
    int grid = 1;      // blocks per matrix
    int seg_log2 = 0;
    unsigned long long nseg = 1;
    int nwarps = 1;    // warps per matrix
    int nchunks = 1;   // partials per matrix in the first finalize stage
    int count = 1;     // matrices in one launch
};

// Largest batch one launch takes (gridDim.y); larger batches are cut.
constexpr int kMaxBatchLaunch = 65535;

// fx: plan for the integer-mantissa sweep alone (otherwise for the
// double-float sweep, whose twin then runs on the same plan)
static GradPlan plan_grad(int n, int count, bool fx = false) {
    GradPlan gp;
    gp.cpl = n <= 16 ? 4 : 8;
    gp.count = count;
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = device_sms(dev);
    int nb = 0;
    size_t smem = gp.cpl == 4 ? grad_smem<4>(n) : grad_smem<8>(n);
    const void* kern = gp.cpl == 4 ? (fx ? (const void*)grad_fx_kernel<4> : (const void*)grad_kernel<4>)
                                   : (fx ? (const void*)grad_fx_kernel<8> : (const void*)grad_kernel<8>);
    allow_max_dynamic_smem(kern);
    allow_max_dynamic_smem(gp.cpl == 4 ? (const void*)grad_fx_kernel<4> : (const void*)grad_fx_kernel<8>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kThreads, smem);
    if (nb < 1) nb = 1;
    const long long grid_full = (long long)sms * nb;
    const long long gx_max = std::max(1ll, grid_full / std::max(1, count));
    const int slog = n - 1;
    // walk length 2^l: a matrix's walks are dealt to its blocks' walk slots
    // in passes, and the matrices' blocks fill the GPU in waves, so the time
    // goes as waves x passes x (2^l + per-walk cost), the per-walk cost
    // (start-up and the final fold of n rows) being about 0.2 n + 16 steps.
    // Ties go to the longer walk.
    double best = 1e300;
    int best_l = slog;
    long long best_gx = 1;
    for (int l = slog; l >= 0; --l) {
        const unsigned long long nseg = 1ull << (slog - l);
        const unsigned long long blocks_needed = ((nseg + kGroups - 1) / kGroups + 3) / 4;
        const long long gx = std::max(1ll, std::min(gx_max, (long long)blocks_needed));
        const unsigned long long slots = (unsigned long long)gx * (kThreads / 32) * kGroups;
        const double passes = (double)((nseg + slots - 1) / slots);
        const double waves = std::ceil((double)count * (double)gx / (double)grid_full);
        const double cost = waves * passes * (std::ldexp(1.0, l) + 0.2 * n + 16.0);
        if (cost < best * (1.0 - 1e-9)) {
            best = cost;
            best_l = l;
            best_gx = gx;
        }
    }
    gp.seg_log2 = best_l;
    gp.nseg = 1ull << (slog - best_l);
    gp.grid = (int)best_gx;
    gp.nwarps = gp.grid * (kThreads / 32);
    gp.nchunks = (gp.nwarps + kFinWarps - 1) / kFinWarps;
    return gp;
}

// The integer-mantissa twin behind a double-float batch recomputes only the
// matrices handed over (usually a few: near-vanishing permanents), so its
// launch is planned as if for count / spread matrices: a handed-over
// matrix gets `spread` times the blocks the double-float sweep gave it,
// while the blocks of the others return at once.  spread <= 16, and the
// twin's per-warp tiles are kept within 64 MiB.
static GradPlan plan_grad_twin(int n, int count) {
    int spread = 16;
    GradPlan gp = plan_grad(n, std::max(1, count / spread), true);
    while (spread > 1 && (double)count * gp.nwarps * n * n * sizeof(float4) > 64.0 * 1024 * 1024) {
        spread >>= 1;
        gp = plan_grad(n, std::max(1, count / spread), true);
    }
    gp.count = count;
    return gp;
}

struct GradWs {
    size_t a1, a2, exp, exp64, dfi, cole, rowk, warp_g, part, warp_s2, est, total;
};

static GradWs grad_ws_layout(int n, const GradPlan& gp, const GradPlan* twin = nullptr) {
    GradWs w;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes, 256);
        return o;
    };
    const size_t c = (size_t)gp.count;
    w.a1 = take(c * n * n * sizeof(longlong2));
    w.a2 = take(c * n * n * sizeof(longlong2));
    w.exp = take(c * sizeof(int));
    w.exp64 = take(c * sizeof(int));
    w.dfi = take(c * 2 * sizeof(int));
    w.cole = take(c * n * sizeof(int));
    w.rowk = take(c * n * sizeof(int));
    const size_t tw = twin ? std::max(gp.nwarps, twin->nwarps) : gp.nwarps;
    const size_t tc = twin ? std::max(gp.nchunks, twin->nchunks) : gp.nchunks;
    w.warp_g = take(c * tw * n * n * sizeof(float4));
    w.part = take(c * tc * n * n * sizeof(float4));
    w.warp_s2 = take(c * gp.nwarps * sizeof(double));
    w.est = take(c * sizeof(double));
    w.total = off;
    return w;
}

static size_t grad_ws_bytes(int n, int count) {
    size_t most = 256;
    for (int done = 0; done < count; done += kMaxBatchLaunch) {
        const int c = std::min(kMaxBatchLaunch, count - done);
        const GradPlan twin = plan_grad_twin(n, c);
        most = std::max(most, grad_ws_layout(n, plan_grad(n, c, false), &twin).total);
        most = std::max(most, grad_ws_layout(n, plan_grad(n, c, true)).total);
        if (count > kMaxBatchLaunch) break;  // all full launches have the same layout; the last is smaller
    }
    return most;
}

// Device-side gradient of `count` matrices: matrix b is dA + b * stride
// (n x n complex128, leading dimension ld); grad out count x n x n complex128
// row-major, perm out count x 2 doubles, optional perm dd count x 4 doubles.
// arith GBPERM_ARITH_DF32: the double-float sweep, each matrix recomputed by
// the integer-mantissa twin on the device when its range check fails or its
// error estimate is above 1e-10 (d_est: count doubles receiving the
// estimates, -1 for a failed range check); GBPERM_ARITH_FX64: the twin alone.
// d_flags (count x 2 ints, optional): df_info after the run ({boost, ok}; ok
// 0 = the twin's values).
static int run_grad_dev(const double2* dA, long long ld, long long stride, int n, int count, void* ws,
                        size_t ws_bytes, double* d_grad, double* d_perm, double* d_perm4, cudaStream_t st,
                        GradPlan* used, int arith, double* d_est = nullptr, int* d_flags = nullptr) {
    const bool fx_only = arith == GBPERM_ARITH_FX64;
    const bool escalate = g_opt.df_escalate.load() != 0;
    for (int done = 0; done < count; done += kMaxBatchLaunch) {
        const int c = std::min(kMaxBatchLaunch, count - done);
        GradPlan gp = plan_grad(n, c, fx_only);
        if (used) *used = gp;
        // the twin's own launch shape (the same as gp when it runs alone)
        const GradPlan gt = fx_only ? gp : plan_grad_twin(n, c);
        const GradWs w = grad_ws_layout(n, gp, fx_only ? nullptr : &gt);
        if (ws_bytes < w.total) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad: workspace too small");
        char* base = static_cast<char*>(ws);
        longlong2* a1 = reinterpret_cast<longlong2*>(base + w.a1);
        longlong2* a2 = reinterpret_cast<longlong2*>(base + w.a2);
        int* exp_out = reinterpret_cast<int*>(base + w.exp);
        int* exp64 = reinterpret_cast<int*>(base + w.exp64);
        int* df_info = reinterpret_cast<int*>(base + w.dfi);
        int* col_e = reinterpret_cast<int*>(base + w.cole);
        int* row_k = reinterpret_cast<int*>(base + w.rowk);
        float4* warp_g = reinterpret_cast<float4*>(base + w.warp_g);
        float4* fin_part = reinterpret_cast<float4*>(base + w.part);
        double* warp_s2 = reinterpret_cast<double*>(base + w.warp_s2);
        double* est = d_est ? d_est + done : reinterpret_cast<double*>(base + w.est);
        PrepArgs pa;
        pa.col_e_out = col_e;
        pa.A = dA + (long long)done * stride;
        pa.ld = ld;
        pa.rows = n;
        pa.cols = n;
        pa.row_w = nullptr;
        pa.col_w = nullptr;
        pa.norm_shift = n - 1;
        pa.a1 = a1;
        pa.a2 = a2;
        pa.exp_out = exp_out;
        pa.df = fx_only ? 0 : 1;
        pa.df_info = df_info;
        pa.count = c;
        pa.a_stride = stride;
        pa.row_balance = 1;
        pa.row_k_out = row_k;
        pa.exp_fp64_out = exp64;
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
        const dim3 grid(gp.grid, c);
        const int ne = n * n;
        double* gout = d_grad + (size_t)done * 2 * n * n;
        const double2* Ab = dA + (long long)done * stride;
        double* pout = d_perm + (size_t)done * 2;
        double* p4 = d_perm4 ? d_perm4 + (size_t)done * 4 : nullptr;
        if (!fx_only) {
            g.warp_s2 = warp_s2;
            if (gp.cpl == 4) grad_kernel<4><<<grid, kThreads, grad_smem<4>(n), st>>>(g);
            else grad_kernel<8><<<grid, kThreads, grad_smem<8>(n), st>>>(g);
            e = cudaGetLastError();
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: kernel");
            // the boost is read on the device by the finalize kernel via df_info
            grad_partial_kernel<<<dim3((ne + 127) / 128, gp.nchunks, c), 128, 0, st>>>(warp_g, gp.nwarps, n,
                                                                                       fin_part);
            grad_finalize_kernel<<<dim3((ne + 127) / 128, c), 128, 0, st>>>(fin_part, gp.nchunks, n, exp_out,
                                                                            col_e, row_k, df_info, gout);
            grad_perm_kernel<<<c, 32, 0, st>>>(Ab, ld, stride, n, gout, df_info, pout, p4, warp_s2, gp.nwarps,
                                               exp_out, est, escalate ? 1 : 0);
            e = cudaGetLastError();
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: finalize");
        }
        // the integer-mantissa twin: every matrix (fx_only), or those the
        // range check or the error estimate handed over
        g.warp_s2 = nullptr;
        g.gate = fx_only ? nullptr : df_info;
        g.seg_log2 = gt.seg_log2;
        g.nseg = gt.nseg;
        const dim3 grid_t(gt.grid, c);
        if (gt.cpl == 4) grad_fx_kernel<4><<<grid_t, kThreads, grad_smem<4>(n), st>>>(g);
        else grad_fx_kernel<8><<<grid_t, kThreads, grad_smem<8>(n), st>>>(g);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: fx kernel");
        double2* part2 = reinterpret_cast<double2*>(fin_part);
        grad_partial_fx_kernel<<<dim3((ne + 127) / 128, gt.nchunks, c), 128, 0, st>>>(
            reinterpret_cast<const double2*>(warp_g), gt.nwarps, n, part2, g.gate);
        grad_finalize_fx_kernel<<<dim3((ne + 127) / 128, c), 128, 0, st>>>(part2, gt.nchunks, n, exp64, col_e,
                                                                           row_k, g.gate, gout);
        grad_perm_kernel<<<c, 32, 0, st>>>(Ab, ld, stride, n, gout, fx_only ? nullptr : df_info, pout, p4, nullptr,
                                           0, nullptr, nullptr, 0);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: fx finalize");
        if (d_flags) {
            if (fx_only) e = cudaMemsetAsync(d_flags + 2 * (size_t)done, 0, 2 * sizeof(int) * (size_t)c, st);
            else e = cudaMemcpyAsync(d_flags + 2 * (size_t)done, df_info, 2 * sizeof(int) * (size_t)c,
                                     cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_grad: flags");
        }
    }
    return GBPERM_OK;
}

// the gradient sweep's arithmetic (option "grad.arith")
static int grad_arith() {
    return g_opt.grad_arith.load() == GBPERM_ARITH_FX64 ? GBPERM_ARITH_FX64 : GBPERM_ARITH_DF32;
}

}  // namespace gbperm

using namespace gbperm;

extern "C" {

size_t gbperm_perm_grad_workspace_size(int64_t n) {
    if (n <= 0 || n > 32) return 256;
    return grad_ws_bytes((int)n, 1);
}

size_t gbperm_perm_grad_batched_workspace_size(int64_t n, int64_t count) {
    if (n <= 0 || n > 32 || count <= 0 || count > INT32_MAX) return 256;
    return grad_ws_bytes((int)n, (int)count);
}

int gbperm_perm_grad_dev(const void* dA, int64_t n, int64_t ld, void* d_perm, void* d_perm_dd, void* d_grad,
                         void* workspace, size_t workspace_bytes, void* stream) {
    if (n < 1 || n > 32) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_grad: n must be in 1..32");
    if (!dA || !d_perm || !d_grad || !workspace) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: null pointer");
    if (ld < n) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: ld < n");
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_dev: workspace must be 256-byte aligned");
    return run_grad_dev(static_cast<const double2*>(dA), ld, 0, (int)n, 1, workspace, workspace_bytes,
                        static_cast<double*>(d_grad), static_cast<double*>(d_perm), static_cast<double*>(d_perm_dd),
                        static_cast<cudaStream_t>(stream), nullptr, grad_arith());
}

int gbperm_perm_grad_batched_dev(const void* dA, int64_t n, int64_t count, int64_t ld, int64_t stride, void* d_perm,
                                 void* d_grad, void* workspace, size_t workspace_bytes, void* stream) {
    if (n < 1 || n > 32) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_grad_batched: n must be in 1..32");
    if (count < 0 || count > INT32_MAX) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_batched: bad count");
    if (count == 0) return GBPERM_OK;
    if (!dA || !d_perm || !d_grad || !workspace)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_batched_dev: null pointer");
    if (ld < n || stride < n * ld) return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_batched_dev: ld < n or stride < n ld");
    if (reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_grad_batched_dev: workspace must be 256-byte aligned");
    return run_grad_dev(static_cast<const double2*>(dA), ld, stride, (int)n, (int)count, workspace, workspace_bytes,
                        static_cast<double*>(d_grad), static_cast<double*>(d_perm), nullptr,
                        static_cast<cudaStream_t>(stream), nullptr, grad_arith());
}

// Host-buffer form shared by the single and batched entry points: count
// dense n x n matrices (matrix b at A + 2 b stride doubles, leading
// dimension ld), perms count x 2, grads count x n x n complex128.
static int perm_grad_host(const double* A, int64_t n, int64_t count, int64_t ld, int64_t stride, double* perms,
                          double* perm_dd, double* grads, gbperm_stats* stats, const char* who) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!perms || !grads) return fail(GBPERM_ERR_ARG, std::string(who) + ": null output");
    if (n < 1 || n > 32) return fail(GBPERM_ERR_TOO_LARGE, std::string(who) + ": n must be in 1..32");
    if (count < 0 || count > INT32_MAX) return fail(GBPERM_ERR_ARG, std::string(who) + ": bad count");
    if (count == 0) return GBPERM_OK;
    if (!A || ld < n || stride < n * ld) return fail(GBPERM_ERR_ARG, std::string(who) + ": bad matrix");
    // matrices beyond the double-float product's range are handed to the
    // integer-mantissa twin by the device range check
    const int arith = grad_arith();
    const size_t nn = (size_t)n * n;
    const size_t mat_bytes = align_up((size_t)count * nn * sizeof(double2), 256);
    const size_t perm_bytes = align_up((size_t)count * 6 * sizeof(double), 256);
    const size_t est_bytes = align_up((size_t)count * (sizeof(double) + 2 * sizeof(int)), 256);
    const size_t ws = grad_ws_bytes((int)n, (int)count);
    ThreadCtx& c = thread_ctx();
    int rc = c.ensure(mat_bytes * 2 + perm_bytes + est_bytes + ws);
    if (rc) return rc;
    char* base = static_cast<char*>(c.dbuf);
    double2* dA = reinterpret_cast<double2*>(base);
    double* dgrad = reinterpret_cast<double*>(base + mat_bytes);
    double* dperm = reinterpret_cast<double*>(base + 2 * mat_bytes);
    double* dest = reinterpret_cast<double*>(base + 2 * mat_bytes + perm_bytes);
    int* dflags = reinterpret_cast<int*>(dest + count);
    void* dws = base + 2 * mat_bytes + perm_bytes + est_bytes;
    // dense upload: matrix b as n rows of n complex128; non-finite matrices
    // are replaced by zeros on the device and answered with NaN
    std::vector<double2> h((size_t)count * nn);
    std::vector<char> bad((size_t)count, 0);
    for (int64_t b = 0; b < count; ++b) {
        const double* Ab = A + 2 * b * stride;
        bad[b] = !all_finite(Ab, n, n, ld);
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j)
                h[b * nn + i * n + j] = bad[b] ? make_double2(0.0, 0.0)
                                               : make_double2(Ab[2 * (i * ld + j)], Ab[2 * (i * ld + j) + 1]);
    }
    cudaError_t e = cudaMemcpyAsync(dA, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_fail(e, (std::string(who) + ": upload").c_str());
    if (stats) cudaEventRecord(c.ev0, c.stream);
    GradPlan used;
    rc = run_grad_dev(dA, n, (long long)nn, (int)n, (int)count, dws, ws, dgrad, dperm,
                      count == 1 ? dperm + 2 : nullptr, c.stream, &used, arith, dest, dflags);
    if (rc) return rc;
    if (stats) cudaEventRecord(c.ev1, c.stream);
    std::vector<double> hp(count == 1 ? 6 : 2 * (size_t)count);
    std::vector<double> hest((size_t)count, 0.0);
    std::vector<int> hflags(2 * (size_t)count, 0);
    e = cudaMemcpyAsync(grads, dgrad, (size_t)count * nn * sizeof(double2), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), dperm, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess && arith != GBPERM_ARITH_FX64)
        e = cudaMemcpyAsync(hest.data(), dest, hest.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hflags.data(), dflags, hflags.size() * sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(e, (std::string(who) + ": kernel").c_str());
    for (int64_t b = 0; b < count; ++b) {
        perms[2 * b] = bad[b] ? NAN : hp[2 * b];
        perms[2 * b + 1] = bad[b] ? NAN : hp[2 * b + 1];
        if (bad[b])
            for (size_t q = 0; q < 2 * nn; ++q) grads[2 * b * nn + q] = NAN;
    }
    if (perm_dd && count == 1) std::memcpy(perm_dd, hp.data() + 2, 4 * sizeof(double));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        stats->kernel_ms = ms;
        stats->steps = (double)count * std::ldexp(1.0, (int)n - 1);
        stats->flops = 8.0 * (double)n * stats->steps;
        const int launches_per = arith == GBPERM_ARITH_FX64 ? 5 : 9;
        stats->launches = launches_per * (int)((count + kMaxBatchLaunch - 1) / kMaxBatchLaunch);
        stats->grid = used.grid;
        stats->seg_log2 = used.seg_log2;
        // arith: FX64 when the twin produced any matrix's values; err_est:
        // the largest double-float estimate among the matrices it kept
        bool any_fx = arith == GBPERM_ARITH_FX64;
        double worst = 0.0;
        for (int64_t b = 0; b < count; ++b) {
            if (bad[b]) continue;
            if (hflags[2 * b + 1] == 0) any_fx = true;
            else if (hest[b] > worst) worst = hest[b];
        }
        stats->arith = any_fx ? GBPERM_ARITH_FX64 : GBPERM_ARITH_DF32;
        stats->err_est = worst;
    }
    return GBPERM_OK;
}

int gbperm_perm_grad(const double* A, int64_t n, int64_t ld, double* perm, double* perm_dd, double* grad,
                     gbperm_stats* stats) {
    return perm_grad_host(A, n, 1, ld, n * ld, perm, perm_dd, grad, stats, "gbperm_perm_grad");
}

int gbperm_perm_grad_batched(const double* A, int64_t n, int64_t count, double* perms, double* grads,
                             gbperm_stats* stats) {
    return perm_grad_host(A, n, count, n, n * n, perms, nullptr, grads, stats, "gbperm_perm_grad_batched");
}

}  // extern "C"
