// Batched plain permanents of many small matrices in one persistent launch.
//
// Replaces the sequential list branch of the reference's plain wrapper
// (GlynnPermanentCalculator_Wrapper.hpp:204-294) and the one-permanent-at-a-
// time loop of BatchednPermanentCalculator::calculate
// (BatchedPermanentCalculator.cpp:109-296), where each instance spins up its
// own TBB parallel region.
//
// Work list: every instance's Gray range is cut into aligned segments of
// 2^l_i steps; a work item is the SPI = 32 / GROUP consecutive segments one
// warp handles (one segment per lane group).  Items are ordered by instance
// cost, largest first (longest-processing-time order), and warps take them
// from an atomic counter until the list is empty, so small instances fill
// the tail behind the large ones.  Each item's double-double partial sum
// lands in its own slot; a finalize kernel adds an instance's slots in a
// fixed order (bitwise-reproducible results) and applies the scale.
//
// Arithmetic per instance as in the single-permanent kernels: exact int64
// column sums; FP64 product (GROUP = 1), the double-float product with lane
// groups (GROUP = 2/4) with the FP64 product as the per-instance fallback
// when the range check fails or the error estimate is above the bar, or the
// integer-mantissa product with lane groups (batched_fx_kernel).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <numeric>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"
#include "gbperm_fx.cuh"

namespace gbperm {

namespace {

constexpr int kThreads = 128;

struct BInst {              // device instance descriptor
    int rows, cols;
    long long a_off;        // offset (complex elements) of the instance in the packed input / fixed arrays
    int seg_log2;
    int item0, nitems;
    unsigned long long nseg;
};

struct BInstOut {           // written by the batched prepare kernel
    int exp;                // result exponent of the double-float product (with the boost)
    int exp64;              // result exponent of the FP64 product
    int boost;
    int ok;                 // double-float product in use (range check; cleared to redo in FP64)
    int finite;             // input finite
    int redo;               // the FP64 pass recomputes this instance
};

struct BItem {
    int inst;
    int pad;
    unsigned long long seg0;
};

struct BArgs {
    const double2* A;       // packed inputs (dense rows x cols each)
    longlong2* a1;
    longlong2* a2;
    const BInst* inst;
    BInstOut* iout;
    const BItem* items;
    int nitems;
    int ninst;
    unsigned int* counter;
    cdd* item_part;
    double* item_s2;        // per item: sum of |term 2^40|^2 of its double-float terms
    double* out;            // 2 doubles per instance (device)
    double* inst_est;       // per instance: relative error estimate (-1: FP64 product, -2: recomputed in FP64)
    int df;
    int escalate;           // mark double-float instances above the error bar for the FP64 pass
    int redo_only;          // the FP64 pass: only instances marked redo
};

// One block per instance (grid-stride): fixed point, exponent and
// double-float boost, as launch_prepare does for one matrix.
__global__ void batched_prepare_kernel(BArgs p) {
    __shared__ int s_e[64];
    __shared__ double s_typ[64];
    __shared__ int s_bad;
    for (int i = blockIdx.x; i < p.ninst; i += gridDim.x) {
        const BInst in = p.inst[i];
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        const double2* A = p.A + in.a_off;
        for (int j = threadIdx.x; j < in.cols; j += blockDim.x) {
            double br = 0.0, bi = 0.0, l2 = 0.0;
            bool fin = true;
            for (int r = 0; r < in.rows; ++r) {
                double2 a = A[r * in.cols + j];
                fin = fin && isfinite(a.x) && isfinite(a.y);
                br += fabs(a.x);
                bi += fabs(a.y);
                l2 += a.x * a.x + a.y * a.y;
            }
            if (!fin) atomicOr(&s_bad, 1);
            double b = fmax(br, bi) * (1.0 + 1e-12);
            int e = 0;
            if (b > 0.0 && fin) frexp(b, &e);
            s_e[j] = e;
            s_typ[j] = (b > 0.0 && fin) ? log2(sqrt(l2) / ldexp(1.0, e)) : -1e300;
            for (int r = 0; r < in.rows; ++r) {
                double2 a = A[r * in.cols + j];
                long long xr = fin ? __double2ll_rn(ldexp(a.x, GBPERM_FIX_BITS - e)) : 0;
                long long xi = fin ? __double2ll_rn(ldexp(a.y, GBPERM_FIX_BITS - e)) : 0;
                p.a1[in.a_off + r * in.cols + j] = make_longlong2(xr, xi);
                p.a2[in.a_off + r * in.cols + j] = make_longlong2(2 * xr, 2 * xi);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long tot = 0;
            double typ = 0.0;
            for (int j = 0; j < in.cols; ++j) {
                tot += s_e[j];
                typ += s_typ[j];
            }
            int o = 0, ok = 0;
            if (p.df && typ > -1e290) {
                o = (int)floor((-40.0 - typ) / (double)in.cols);
                int omax = (int)floor(118.0 / (double)in.cols - 0.5);
                if (o > omax) o = omax;
                ok = (typ + (double)o * (double)in.cols >= -100.0) ? 1 : 0;
                if (!ok) o = 0;
            }
            BInstOut r;
            r.exp = (int)(tot - (long long)o * in.cols - (in.rows - 1));
            r.exp64 = (int)(tot - (in.rows - 1));
            r.boost = o;
            r.ok = ok;
            r.finite = s_bad ? 0 : 1;
            r.redo = 0;
            p.iout[i] = r;
        }
        __syncthreads();
    }
}

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
}

// Persistent worker: each warp takes items from the counter.  GROUP lanes
// share a segment; lane g owns columns [g*CPL, (g+1)*CPL).  DF selects the
// double-float product (GROUP > 1 allowed) or the FP64 product (GROUP == 1).
template <int CPL, int GROUP, bool DF>
__global__ void __launch_bounds__(kThreads) batched_kernel(BArgs p) {
    const int lane = threadIdx.x & 31;
    const int g = lane % GROUP;
    const int grp = lane / GROUP;
    const int j0 = g * CPL;
    long long cre[CPL], cim[CPL];
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(p.counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= p.nitems) break;
        const BItem item = p.items[it];
        const BInstOut io = p.iout[item.inst];
        if (p.redo_only && !io.redo) continue;  // warp-uniform
        const BInst in = p.inst[item.inst];
        const int rows = in.rows, cols = in.cols;
        const unsigned long long s = item.seg0 + (unsigned long long)grp;
        const bool active = s < in.nseg && io.finite;
        const unsigned long long i0 = (active ? s : 0ull) << in.seg_log2;
        const unsigned long long L = 1ull << in.seg_log2;
        const longlong2* __restrict__ a1 = p.a1 + in.a_off;
        const longlong2* __restrict__ a2 = p.a2 + in.a_off;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            longlong2 v = (j0 + c < cols) ? __ldg(&a1[j0 + c]) : make_longlong2(0, 0);
            cre[c] = v.x;
            cim[c] = v.y;
        }
        for (int r = 1; r < rows; ++r) {
            const long long m = -(long long)((g0 >> (rows - 1 - r)) & 1ull);
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (j0 + c < cols) {
                    longlong2 v = __ldg(&a1[r * cols + j0 + c]);
                    cre[c] += (v.x ^ m) - m;
                    cim[c] += (v.y ^ m) - m;
                }
            }
        }
        cdd acc{{0.0, 0.0}, {0.0, 0.0}};
        double s2 = 0.0;  // double-float items: sum of |term 2^40|^2 (error estimate)
        const bool use_df = DF && io.ok;
        if (use_df) {
            const DfConv cv = make_dfconv(io.boost);
            unsigned int sbit = (unsigned int)(__popcll(g0) & 1) << 31;
            float brh = 0.f, brl = 0.f, bih = 0.f, bil = 0.f;
            float s2f = 0.f;  // sum of |term 2^40|^2 since the last fold
            for (unsigned long long k = 0; k < L; ++k) {
                if (k != 0) {
                    const int b = __ffsll((long long)k) - 1;
                    const unsigned long long idx = i0 + k;
                    const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;
                    const longlong2* a = a2 + (rows - 1 - b) * cols + j0;
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        if (j0 + c < cols) {
                            longlong2 v = __ldg(&a[c]);
                            if (sub) {
                                cre[c] -= v.x;
                                cim[c] -= v.y;
                            } else {
                                cre[c] += v.x;
                                cim[c] += v.y;
                            }
                        }
                    }
                    sbit ^= 0x80000000u;
                    if ((k & 255ull) == 0) {
                        acc.re = dd_add(acc.re, dd{(double)brh, (double)brl});
                        acc.im = dd_add(acc.im, dd{(double)bih, (double)bil});
                        brh = brl = bih = bil = 0.f;
                        s2 += (double)s2f;
                        s2f = 0.f;
                    }
                }
                cf pa{1.f, 0.f, 0.f, 0.f}, pb{1.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    if (j0 + c < cols) {
                        cf x;
                        fix_to_df_magic(cre[c], cv, x.rh, x.rl);
                        fix_to_df_magic(cim[c], cv, x.ih, x.il);
                        if (c == 0) pa = x;
                        else if (c == 1) pb = x;
                        else if (c & 1) pb = cf_mul(pb, x);
                        else pa = cf_mul(pa, x);
                    }
                }
                if (CPL > 1) pa = cf_mul(pa, pb);
#pragma unroll
                for (int m = 1; m < GROUP; m <<= 1) pa = cf_mul(pa, shfl_xor_cf(pa, m));
                if (g == 0 && active) {
                    df_acc(brh, brl, __uint_as_float(__float_as_uint(pa.rh) ^ sbit),
                           __uint_as_float(__float_as_uint(pa.rl) ^ sbit));
                    df_acc(bih, bil, __uint_as_float(__float_as_uint(pa.ih) ^ sbit),
                           __uint_as_float(__float_as_uint(pa.il) ^ sbit));
                    const float ur = pa.rh * 0x1p40f, ui = pa.ih * 0x1p40f;
                    s2f = fmaf(ur, ur, fmaf(ui, ui, s2f));
                }
            }
            acc.re = dd_add(acc.re, dd{(double)brh, (double)brl});
            acc.im = dd_add(acc.im, dd{(double)bih, (double)bil});
            s2 += (double)s2f;
        } else if (GROUP == 1) {
            // FP64 product (also the double-float fallback)
            unsigned long long neg = (unsigned long long)(__popcll(g0) & 1) << 63;
            double bre = 0.0, bim = 0.0;
            for (unsigned long long k = 0; k < L; ++k) {
                if (k != 0) {
                    const int b = __ffsll((long long)k) - 1;
                    const unsigned long long idx = i0 + k;
                    const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;
                    const longlong2* a = a2 + (rows - 1 - b) * cols + j0;
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        if (j0 + c < cols) {
                            longlong2 v = __ldg(&a[c]);
                            if (sub) {
                                cre[c] -= v.x;
                                cim[c] -= v.y;
                            } else {
                                cre[c] += v.x;
                                cim[c] += v.y;
                            }
                        }
                    }
                    neg ^= 0x8000000000000000ull;
                    if ((k & 255ull) == 0) {
                        acc.re = dd_add_d(acc.re, bre);
                        acc.im = dd_add_d(acc.im, bim);
                        bre = 0.0;
                        bim = 0.0;
                    }
                }
                cd pa{1.0, 0.0}, pb{1.0, 0.0};
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    if (c < cols) {
                        cd x{fix_to_double(cre[c]), fix_to_double(cim[c])};
                        if (c == 0) pa = x;
                        else if (c == 1) pb = x;
                        else if (c & 1) pb = cmul(pb, x);
                        else pa = cmul(pa, x);
                    }
                }
                if (CPL > 1 && cols > 1) pa = cmul(pa, pb);
                if (active) {
                    bre += __longlong_as_double(__double_as_longlong(pa.re) ^ (long long)neg);
                    bim += __longlong_as_double(__double_as_longlong(pa.im) ^ (long long)neg);
                }
            }
            acc.re = dd_add_d(acc.re, bre);
            acc.im = dd_add_d(acc.im, bim);
        } else {
            // GROUP > 1 and the range check failed: FP64 product of the lane's
            // columns, then the butterfly in FP64
            unsigned long long neg = (unsigned long long)(__popcll(g0) & 1) << 63;
            double bre = 0.0, bim = 0.0;
            for (unsigned long long k = 0; k < L; ++k) {
                if (k != 0) {
                    const int b = __ffsll((long long)k) - 1;
                    const unsigned long long idx = i0 + k;
                    const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;
                    const longlong2* a = a2 + (rows - 1 - b) * cols + j0;
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        if (j0 + c < cols) {
                            longlong2 v = __ldg(&a[c]);
                            if (sub) {
                                cre[c] -= v.x;
                                cim[c] -= v.y;
                            } else {
                                cre[c] += v.x;
                                cim[c] += v.y;
                            }
                        }
                    }
                    neg ^= 0x8000000000000000ull;
                    if ((k & 255ull) == 0) {
                        acc.re = dd_add_d(acc.re, bre);
                        acc.im = dd_add_d(acc.im, bim);
                        bre = 0.0;
                        bim = 0.0;
                    }
                }
                cd pa{1.0, 0.0};
#pragma unroll
                for (int c = 0; c < CPL; ++c)
                    if (j0 + c < cols) pa = cmul(pa, cd{fix_to_double(cre[c]), fix_to_double(cim[c])});
#pragma unroll
                for (int m = 1; m < GROUP; m <<= 1) {
                    cd o{__shfl_xor_sync(0xffffffffu, pa.re, m), __shfl_xor_sync(0xffffffffu, pa.im, m)};
                    pa = cmul(pa, o);
                }
                if (g == 0 && active) {
                    bre += __longlong_as_double(__double_as_longlong(pa.re) ^ (long long)neg);
                    bim += __longlong_as_double(__double_as_longlong(pa.im) ^ (long long)neg);
                }
            }
            acc.re = dd_add_d(acc.re, bre);
            acc.im = dd_add_d(acc.im, bim);
        }
        acc = warp_sum_cdd(acc);
        s2 = warp_sum_d(s2);
        if (lane == 0) {
            p.item_part[it] = acc;
            p.item_s2[it] = s2;
        }
    }
}

// Integer-mantissa worker (GBPERM_ARITH_FX64): the items of the FP64 /
// double-float worker with the product of perm_plain_fx.cu -- each
// instance's columns split evenly over the GROUP lanes of a walk (a lane
// holds ceil(cols / GROUP) of them), two product chains per lane on 31-bit
// limbs, a shuffle butterfly over the group, and the term converted to
// double (fx_to_double).  No range check and no redo pass.
template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads) batched_fx_kernel(BArgs p) {
    static_assert(GROUP >= 2, "lanes 0 and 1 of a group convert the two components");
    const int lane = threadIdx.x & 31;
    const int g = lane % GROUP;
    const int grp = lane / GROUP;
    long long cre[CPL], cim[CPL];
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(p.counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= p.nitems) break;
        const BItem item = p.items[it];
        const BInstOut io = p.iout[item.inst];
        const BInst in = p.inst[item.inst];
        const int rows = in.rows, cols = in.cols;
        const int cpl_i = (cols + GROUP - 1) / GROUP;
        const int j0 = g * cpl_i;
        const int nr = max(0, min(cpl_i, cols - j0));  // 0 for a lane past the columns
        const unsigned long long s = item.seg0 + (unsigned long long)grp;
        const bool active = s < in.nseg && io.finite;
        const unsigned long long i0 = (active ? s : 0ull) << in.seg_log2;
        const unsigned long long L = 1ull << in.seg_log2;
        const longlong2* __restrict__ a1 = p.a1 + in.a_off;
        const longlong2* __restrict__ a2 = p.a2 + in.a_off;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            longlong2 v = c < nr ? __ldg(&a1[j0 + c]) : make_longlong2(0, 0);
            cre[c] = v.x;
            cim[c] = v.y;
        }
        for (int r = 1; r < rows; ++r) {
            const long long m = -(long long)((g0 >> (rows - 1 - r)) & 1ull);
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (c < nr) {
                    longlong2 v = __ldg(&a1[r * cols + j0 + c]);
                    cre[c] += (v.x ^ m) - m;
                    cim[c] += (v.y ^ m) - m;
                }
            }
        }
        cdd acc{{0.0, 0.0}, {0.0, 0.0}};
        unsigned long long sbit = (unsigned long long)(__popcll(g0) & 1) << 63;
        // every lane of a group ends the butterfly with the same product:
        // lane 0 converts and sums its real part, lane 1 its imaginary part
        double b0 = 0.0;
        for (unsigned long long k = 0; k < L; ++k) {
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;
                const unsigned long long idx = i0 + k;
                const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;
                const longlong2* a = a2 + (rows - 1 - b) * cols + j0;
                if (sub) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c)
                        if (c < nr) {
                            longlong2 v = __ldg(&a[c]);
                            cre[c] -= v.x;
                            cim[c] -= v.y;
                        }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; ++c)
                        if (c < nr) {
                            longlong2 v = __ldg(&a[c]);
                            cre[c] += v.x;
                            cim[c] += v.y;
                        }
                }
                sbit ^= 0x8000000000000000ull;
                if ((k & 255ull) == 0) {
                    acc.re = dd_add_d(acc.re, b0);
                    b0 = 0.0;
                }
            }
            // the lane's partial product in two chains (sig: shift count)
            fxl ch[2];
            int sig = 0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (c < nr) {
                    if (c < 2) {
                        sig += fx_norm_col(cre[c], cim[c], ch[c]);
                    } else {
                        long long rr, ri;
                        fx_mul(ch[c & 1], fx_col(cre[c], cim[c]), rr, ri);
                        sig += fx_norm(rr, ri, ch[c & 1]) - 1;
                    }
                }
            }
            long long pr = 0, pi = 0;
            if (nr >= 2) {
                fx_mul(ch[0], ch[1], pr, pi);
                sig -= 1;
            } else if (nr == 1) {
                pr = fx_join(ch[0].rh, ch[0].rl);
                pi = fx_join(ch[0].ih, ch[0].il);
            }
            // a lane without columns enters the first stage with the value 1,
            // normalised (2^58 with shift count -3, so that two such lanes'
            // product stays within fx_norm's range); from the second stage on
            // it holds a product like every other lane
            bool have = nr > 0;
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) {
                fxl x;
                if (have) {
                    sig += fx_norm(pr, pi, x);
                } else {
                    x = fxl{1 << 27, 0, 0, 0};
                    sig = -3;
                }
                have = true;
                const fxl y = shfl_xor_fxl(x, m);
                sig += __shfl_xor_sync(0xffffffffu, sig, m) - 1;
                fx_mul(x, y, pr, pi);
            }
            if (g < 2 && active) {  // every shape has GROUP >= 2
                const int e = -61 - sig;
                b0 += __longlong_as_double(__double_as_longlong(fx_to_double(g == 0 ? pr : pi, e)) ^ (long long)sbit);
            }
        }
        acc.re = dd_add_d(acc.re, b0);
        if (g == 1) {  // lane 1 summed the imaginary part
            acc.im = acc.re;
            acc.re = dd{0.0, 0.0};
        }
        acc = warp_sum_cdd(acc);
        if (lane == 0) {
            p.item_part[it] = acc;
            p.item_s2[it] = 0.0;
        }
    }
}

// warp per instance: lane l sums items l, l + 32, ... in order, then a fixed
// butterfly (deterministic; a large instance has thousands of items)
__global__ void batched_finalize_kernel(BArgs p) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.ninst; i += nw) {  // warp-uniform
        const BInst in = p.inst[i];
        const BInstOut io = p.iout[i];
        if (p.redo_only && !io.redo) continue;
        if (!io.finite) {
            if (lane == 0) {
                p.out[2 * i] = nan("");
                p.out[2 * i + 1] = nan("");
                p.inst_est[i] = -1.0;
            }
            continue;
        }
        cdd tot{{0.0, 0.0}, {0.0, 0.0}};
        double q = 0.0;
        for (int k = lane; k < in.nitems; k += 32) {
            tot = cdd_add(tot, p.item_part[in.item0 + k]);
            q += p.item_s2[in.item0 + k];
        }
        tot = warp_sum_cdd(tot);
        q = warp_sum_d(q);
        if (lane == 0) {
            write_result(tot, io.ok ? io.exp : io.exp64, p.out + 2 * i, nullptr);
            if (p.redo_only) {
                p.inst_est[i] = -2.0;
            } else if (p.df && io.ok) {
                // relative rounding-error estimate of a double-float result,
                // as in the single-permanent kernels; above the bar the
                // instance goes to the FP64 pass that follows
                const double est =
                    sqrt((double)in.cols) * 0x1p-46 * sqrt(q) * 0x1p-40 / hypot(tot.re.hi, tot.im.hi);
                p.inst_est[i] = est;
                if (p.escalate && !(est <= kDfEscalate)) {
                    p.iout[i].ok = 0;
                    p.iout[i].redo = 1;
                }
            } else {
                p.inst_est[i] = -1.0;
            }
        }
    }
}

// Device-pointer results in the caller's slot order: slot i takes device
// instance dev_index[i], or the host-decided value trivial[i] (1, or 0 for
// rows >= cols + 2) when the instance never reached the device.
__global__ void batched_scatter_kernel(const double* dout, const int* dev_index, const double* trivial,
                                       long long count, double* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const int d = dev_index[i];
        out[2 * i] = d >= 0 ? dout[2 * d] : trivial[i];
        out[2 * i + 1] = d >= 0 ? dout[2 * d + 1] : 0.0;
    }
}

template <int CPL, int GROUP, bool DF>
int bps_t() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_kernel<CPL, GROUP, DF>, kThreads, 0);
    return nb > 0 ? nb : 1;
}

template <int CPL, int GROUP, bool DF>
void launch_t(const BArgs& a, int grid, cudaStream_t st) {
    batched_kernel<CPL, GROUP, DF><<<grid, kThreads, 0, st>>>(a);
}

// shapes: (CPL, GROUP, DF)
#define GBPERM_BATCH_SHAPES(X)                                                                          \
    X(16, 1, false) X(32, 1, false) X(48, 1, false) X(64, 1, false) X(4, 2, true) X(6, 2, true) X(8, 2, true) \
    X(10, 2, true) X(12, 2, true) X(14, 2, true) X(16, 2, true) X(20, 2, true) X(24, 2, true) X(8, 4, true)  \
    X(12, 4, true)

int batch_bps(int cpl, int grp, bool df) {
#define X(C, G, D) \
    if (cpl == C && grp == G && df == D) return bps_t<C, G, D>();
    GBPERM_BATCH_SHAPES(X)
#undef X
    return 0;
}

cudaError_t batch_launch(const BArgs& a, int cpl, int grp, bool df, int grid, cudaStream_t st) {
#define X(C, G, D) \
    if (cpl == C && grp == G && df == D) {  \
        launch_t<C, G, D>(a, grid, st);     \
        return cudaGetLastError();          \
    }
    GBPERM_BATCH_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

// integer-mantissa shapes (CPL, GROUP): an instance's columns are split
// evenly, so CPL only bounds ceil(cols / GROUP)
#define GBPERM_BATCH_FX_SHAPES(X) X(4, 2) X(8, 2) X(12, 2) X(16, 2) X(20, 2) X(16, 4)

int batch_fx_bps(int cpl, int grp) {
#define X(C, G)                                                                                          \
    if (cpl == C && grp == G) {                                                                          \
        int nb = 0;                                                                                      \
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batched_fx_kernel<C, G>, kThreads, 0);        \
        return nb > 0 ? nb : 1;                                                                          \
    }
    GBPERM_BATCH_FX_SHAPES(X)
#undef X
    return 0;
}

cudaError_t batch_fx_launch(const BArgs& a, int cpl, int grp, int grid, cudaStream_t st) {
#define X(C, G)                                                 \
    if (cpl == C && grp == G) {                                 \
        batched_fx_kernel<C, G><<<grid, kThreads, 0, st>>>(a);  \
        return cudaGetLastError();                              \
    }
    GBPERM_BATCH_FX_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

// lane pairs up to 40 columns (quads on request or above), the smallest CPL
// with CPL * GROUP >= cols
void batch_fx_shape(int cols, int group, int* cpl, int* grp) {
    static const int sfx[][2] = {{4, 2}, {8, 2}, {12, 2}, {16, 2}, {20, 2}, {16, 4}};
    const int want = (group == 4 || cols > 40) ? 4 : 2;
    for (auto& s : sfx)
        if (s[1] == want && s[0] * s[1] >= cols) {
            *cpl = s[0];
            *grp = s[1];
            return;
        }
    *cpl = 16;
    *grp = 4;
}

// smallest compiled shape covering `cols` columns for the arithmetic
void batch_shape(int cols, bool df, int group, int* cpl, int* grp) {
    static const int s64[][2] = {{16, 1}, {32, 1}, {48, 1}, {64, 1}};
    static const int sdf[][2] = {{4, 2},  {6, 2},  {8, 2},  {10, 2}, {12, 2},
                                 {14, 2}, {16, 2}, {20, 2}, {24, 2}, {8, 4}, {12, 4}};
    if (!df) {
        for (auto& s : s64)
            if (s[0] >= cols) {
                *cpl = s[0];
                *grp = 1;
                return;
            }
        *cpl = 64;
        *grp = 1;
        return;
    }
    // lane pairs: the widest instances dominate a batch's work, and GROUP = 2
    // with an exact column fit is the fastest plain shape measured on GB300
    int want = group > 0 ? group : 2;
    int best = -1;
    const int n = (int)(sizeof(sdf) / sizeof(sdf[0]));
    for (int i = 0; i < n; ++i)
        if (sdf[i][1] == want && sdf[i][0] * sdf[i][1] >= cols && (best < 0 || sdf[i][0] < sdf[best][0])) best = i;
    if (best < 0)
        for (int i = 0; i < n; ++i)
            if (sdf[i][0] * sdf[i][1] >= cols &&
                (best < 0 || sdf[i][0] * sdf[i][1] < sdf[best][0] * sdf[best][1]))
                best = i;
    *cpl = sdf[best][0];
    *grp = sdf[best][1];
}

}  // namespace

// ------------------------------------------------------------------- plan

struct BatchPlan {
    int device = -1;
    int64_t count = 0;
    int arith = GBPERM_ARITH_FP64;
    bool df = false;
    bool fx = false;                 // integer-mantissa worker (batched_fx_kernel)
    bool escalate = true;            // double-float instances above the error bar redone in FP64
    int cpl = 16, grp = 1;
    int grid = 1;
    int maxc = 1;                    // widest instance (columns)
    int64_t item_target_log2 = 0;
    std::vector<int> rows, cols;
    std::vector<long long> off;      // complex offsets of each instance in the packed input
    std::vector<int> dev_index;      // device instance index or -1 (trivial)
    std::vector<double> trivial;     // value for trivial instances
    long long total_elems = 0;       // packed complex elements
    int ninst = 0, nitems = 0;
    double steps = 0.0, flops = 0.0;
    // device buffers
    char* dbuf = nullptr;
    size_t dbytes = 0;
    char* item_buf = nullptr;        // work list + item partial sums
    size_t item_cap = 0;
    double2* dA = nullptr;
    longlong2 *da1 = nullptr, *da2 = nullptr;
    BInst* dinst = nullptr;
    BInstOut* diout = nullptr;
    BItem* ditems = nullptr;
    unsigned int* dcounter = nullptr;
    cdd* dpart = nullptr;
    double* ds2 = nullptr;           // per item |term|^2 sums
    double* dout = nullptr;
    double* dest = nullptr;          // per instance error estimates
    int* ddev_index = nullptr;       // dev_index on the device (slot -> device instance)
    double* dtrivial = nullptr;      // trivial values on the device
    // pinned host staging and the captured graph
    double* hin = nullptr;
    double* hout = nullptr;
    double* hest = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

static void plan_free(BatchPlan* p) {
    if (!p) return;
    if (p->graph) cudaGraphExecDestroy(p->graph);
    if (p->dbuf) cudaFree(p->dbuf);
    if (p->item_buf) cudaFree(p->item_buf);
    if (p->hin) cudaFreeHost(p->hin);
    if (p->hout) cudaFreeHost(p->hout);
    if (p->hest) cudaFreeHost(p->hest);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

static BArgs plan_args(BatchPlan* p) {
    BArgs a;
    a.A = p->dA;
    a.a1 = p->da1;
    a.a2 = p->da2;
    a.inst = p->dinst;
    a.iout = p->diout;
    a.items = p->ditems;
    a.nitems = p->nitems;
    a.ninst = p->ninst;
    a.counter = p->dcounter;
    a.item_part = p->dpart;
    a.item_s2 = p->ds2;
    a.out = p->dout;
    a.inst_est = p->dest;
    a.df = p->df ? 1 : 0;
    a.escalate = p->escalate ? 1 : 0;
    a.redo_only = 0;
    return a;
}

// Enqueue prepare + worker + finalize on the plan's stream (device input
// already in p->dA).
static cudaError_t plan_enqueue(BatchPlan* p) {
    if (p->ninst == 0) return cudaSuccess;
    BArgs a = plan_args(p);
    cudaError_t e = cudaMemsetAsync(p->dcounter, 0, sizeof(unsigned int), p->stream);
    if (e != cudaSuccess) return e;
    int pg = std::min(p->ninst, 4 * device_sms(p->device));
    batched_prepare_kernel<<<pg, 64, 0, p->stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = p->fx ? batch_fx_launch(a, p->cpl, p->grp, p->grid, p->stream)
              : batch_launch(a, p->cpl, p->grp, p->df, p->grid, p->stream);
    if (e != cudaSuccess) return e;
    batched_finalize_kernel<<<(p->ninst + 3) / 4, 128, 0, p->stream>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess || !(p->df && p->escalate)) return e;
    // the FP64 pass over the instances whose double-float estimate was above
    // the bar (usually none: the warps fetch every item and skip the rest)
    a.redo_only = 1;
    e = cudaMemsetAsync(p->dcounter, 0, sizeof(unsigned int), p->stream);
    if (e != cudaSuccess) return e;
    e = batch_launch(a, p->cpl, p->grp, p->df, p->grid, p->stream);
    if (e != cudaSuccess) return e;
    batched_finalize_kernel<<<(p->ninst + 3) / 4, 128, 0, p->stream>>>(a);
    return cudaGetLastError();
}

// Build instance descriptors and the LPT-ordered item list for the current
// item target, upload them.
static int plan_build_items(BatchPlan* p) {
    const int spi = 32 / p->grp;
    std::vector<int> order;
    for (int64_t i = 0; i < p->count; ++i)
        if (p->dev_index[i] >= 0) order.push_back((int)i);
    // largest first
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        double cx = std::ldexp((double)p->cols[x], p->rows[x]);
        double cy = std::ldexp((double)p->cols[y], p->rows[y]);
        return cx > cy;
    });
    std::vector<BInst> inst(p->ninst);
    std::vector<BItem> items;
    for (int i : order) {
        int d = p->dev_index[i];
        BInst b;
        b.rows = p->rows[i];
        b.cols = p->cols[i];
        b.a_off = p->off[i];
        int slog = b.rows - 1;
        // steps per item ~ 2^target; segment length = that / SPI
        int l = (int)p->item_target_log2 - ceil_log2_u64((unsigned long long)spi);
        if (l > slog) l = slog;
        if (l < 0) l = 0;
        b.seg_log2 = l;
        b.nseg = 1ull << (slog - l);
        b.item0 = (int)items.size();
        unsigned long long nit = (b.nseg + spi - 1) / spi;
        for (unsigned long long k = 0; k < nit; ++k) {
            BItem it;
            it.inst = d;
            it.pad = 0;
            it.seg0 = k * (unsigned long long)spi;
            items.push_back(it);
        }
        b.nitems = (int)nit;
        inst[d] = b;
    }
    p->nitems = (int)items.size();
    if (items.size() > p->item_cap) {
        if (p->item_buf) cudaFree(p->item_buf);
        p->item_buf = nullptr;
        p->item_cap = 0;
        size_t want = items.size() + items.size() / 4 + 64;
        cudaError_t ea = cudaMalloc(&p->item_buf, align_up(want * sizeof(BItem), 256) +
                                                      align_up(want * sizeof(cdd), 256) + want * sizeof(double));
        if (ea != cudaSuccess) return cuda_fail(ea, "batched: work list allocation");
        p->item_cap = want;
        p->ditems = reinterpret_cast<BItem*>(p->item_buf);
        p->dpart = reinterpret_cast<cdd*>(p->item_buf + align_up(want * sizeof(BItem), 256));
        p->ds2 = reinterpret_cast<double*>(p->item_buf + align_up(want * sizeof(BItem), 256) +
                                           align_up(want * sizeof(cdd), 256));
    }
    cudaError_t e = cudaMemcpy(p->dinst, inst.data(), inst.size() * sizeof(BInst), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !items.empty())
        e = cudaMemcpy(p->ditems, items.data(), items.size() * sizeof(BItem), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "batched: upload work list");
    return GBPERM_OK;
}

static int plan_capture(BatchPlan* p) {
    if (p->graph) {
        cudaGraphExecDestroy(p->graph);
        p->graph = nullptr;
    }
    if (p->ninst == 0) return GBPERM_OK;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "batched: begin capture");
    e = cudaMemcpyAsync(p->dA, p->hin, (size_t)p->total_elems * sizeof(double2), cudaMemcpyHostToDevice, p->stream);
    cudaError_t e2 = (e == cudaSuccess) ? plan_enqueue(p) : e;
    cudaError_t e3 = (e2 == cudaSuccess)
                         ? cudaMemcpyAsync(p->hout, p->dout, (size_t)p->ninst * 2 * sizeof(double),
                                           cudaMemcpyDeviceToHost, p->stream)
                         : e2;
    if (e3 == cudaSuccess && p->df)
        e3 = cudaMemcpyAsync(p->hest, p->dest, (size_t)p->ninst * sizeof(double), cudaMemcpyDeviceToHost, p->stream);
    e = cudaStreamEndCapture(p->stream, &g);
    if (e3 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(e3, "batched: capture");
    }
    if (e != cudaSuccess) return cuda_fail(e, "batched: end capture");
    e = cudaGraphInstantiate(&p->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "batched: instantiate graph");
    return GBPERM_OK;
}

}  // namespace gbperm

using namespace gbperm;

struct gbperm_batch_plan {
    BatchPlan* p;
};

extern "C" {

int gbperm_batch_plan_create(const int64_t* rows, const int64_t* cols, int64_t count, int arith,
                             gbperm_batch_plan** out_plan) {
    if (!out_plan) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_create: null plan pointer");
    *out_plan = nullptr;
    if (count < 0 || (count > 0 && (!rows || !cols))) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_create: bad sizes");
    if (count > (int64_t)1 << 28) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_batch_plan_create: too many instances");
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_create: unknown arithmetic");
    BatchPlan* p = new BatchPlan();
    p->count = count;
    p->arith = arith;
    int maxc = 1;
    double total_steps = 0.0;
    for (int64_t i = 0; i < count; ++i) {
        if (rows[i] < 0 || cols[i] < 0) {
            plan_free(p);
            return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_create: negative shape");
        }
        p->rows.push_back((int)rows[i]);
        p->cols.push_back((int)cols[i]);
        p->off.push_back(p->total_elems);
        p->total_elems += rows[i] * cols[i];
        double v = -1.0;
        if (rows[i] == 0 || cols[i] == 0) v = 1.0;
        else if (rows[i] >= cols[i] + 2) v = 0.0;
        if (v < 0.0 && (rows[i] > GBPERM_MAX_DIM || cols[i] > GBPERM_MAX_DIM)) {
            plan_free(p);
            return fail(GBPERM_ERR_TOO_LARGE, "gbperm_batch_plan_create: matrix larger than 64 x 64");
        }
        p->trivial.push_back(v < 0.0 ? 0.0 : v);
        p->dev_index.push_back(v < 0.0 ? p->ninst++ : -1);
        if (v < 0.0) {
            maxc = std::max(maxc, (int)cols[i]);
            total_steps += std::ldexp(1.0, (int)rows[i] - 1);
            p->flops += 8.0 * (double)cols[i] * std::ldexp(1.0, (int)rows[i] - 1);
        }
    }
    p->steps = total_steps;
    if (p->ninst > 0) {
        // a device is needed from here on: report its absence as such
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
            cudaGetLastError();
            plan_free(p);
            return fail(GBPERM_ERR_NO_DEVICE, "no CUDA device visible: the GB300 permanent library needs a GPU");
        }
    }
    cudaError_t e = cudaGetDevice(&p->device);
    if (e != cudaSuccess) {
        plan_free(p);
        return cuda_fail(e, "gbperm_batch_plan_create");
    }
    p->fx = arith == GBPERM_ARITH_FX64;
    p->df = arith == GBPERM_ARITH_DF32 && maxc <= kDfMaxCols;
    p->escalate = g_opt.df_escalate.load() != 0;
    p->maxc = maxc;
    if (p->fx) batch_fx_shape(maxc, (int)g_opt.batched_threads.load(), &p->cpl, &p->grp);
    else batch_shape(maxc, p->df, (int)g_opt.batched_threads.load(), &p->cpl, &p->grp);
    int bps = p->fx ? batch_fx_bps(p->cpl, p->grp) : batch_bps(p->cpl, p->grp, p->df);
    p->grid = device_sms(p->device) * bps;
    // item target: ~16 items per resident warp over the whole batch
    double warps = (double)p->grid * (kThreads / 32);
    double tgt = total_steps / std::max(1.0, warps * 16.0);
    int tl = 0;
    while (std::ldexp(1.0, tl) < tgt && tl < 40) ++tl;
    p->item_target_log2 = std::max(tl, 8);
    int64_t force = g_opt.batched_item_log2.load();
    if (force > 0) p->item_target_log2 = force;
    // device buffers (the work list is allocated with the items)
    size_t off = 0;
    auto take = [&](size_t b) {
        size_t o = off;
        off += align_up(b ? b : 1, 256);
        return o;
    };
    size_t oA = take((size_t)p->total_elems * sizeof(double2));
    size_t o1 = take((size_t)p->total_elems * sizeof(longlong2));
    size_t o2 = take((size_t)p->total_elems * sizeof(longlong2));
    size_t oI = take((size_t)std::max(1, p->ninst) * sizeof(BInst));
    size_t oO = take((size_t)std::max(1, p->ninst) * sizeof(BInstOut));
    size_t oC = take(sizeof(unsigned int));
    size_t oR = take((size_t)std::max(1, p->ninst) * 2 * sizeof(double));
    size_t oE = take((size_t)std::max(1, p->ninst) * sizeof(double));
    size_t oX = take((size_t)std::max<int64_t>(1, p->count) * sizeof(int));
    size_t oT = take((size_t)std::max<int64_t>(1, p->count) * sizeof(double));
    p->dbytes = off;
    e = cudaMalloc(&p->dbuf, p->dbytes);
    if (e == cudaSuccess) e = cudaMallocHost(&p->hin, std::max<size_t>(1, (size_t)p->total_elems) * sizeof(double2));
    if (e == cudaSuccess) e = cudaMallocHost(&p->hout, (size_t)std::max(1, p->ninst) * 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&p->hest, (size_t)std::max(1, p->ninst) * sizeof(double));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev1);
    if (e != cudaSuccess) {
        plan_free(p);
        return cuda_fail(e, "gbperm_batch_plan_create: allocation");
    }
    p->dA = reinterpret_cast<double2*>(p->dbuf + oA);
    p->da1 = reinterpret_cast<longlong2*>(p->dbuf + o1);
    p->da2 = reinterpret_cast<longlong2*>(p->dbuf + o2);
    p->dinst = reinterpret_cast<BInst*>(p->dbuf + oI);
    p->diout = reinterpret_cast<BInstOut*>(p->dbuf + oO);
    p->dcounter = reinterpret_cast<unsigned int*>(p->dbuf + oC);
    p->ddev_index = reinterpret_cast<int*>(p->dbuf + oX);
    p->dtrivial = reinterpret_cast<double*>(p->dbuf + oT);
    if (p->count > 0) {
        e = cudaMemcpy(p->ddev_index, p->dev_index.data(), (size_t)p->count * sizeof(int), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(p->dtrivial, p->trivial.data(), (size_t)p->count * sizeof(double), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            plan_free(p);
            return cuda_fail(e, "gbperm_batch_plan_create: upload");
        }
    }
    p->dout = reinterpret_cast<double*>(p->dbuf + oR);
    p->dest = reinterpret_cast<double*>(p->dbuf + oE);
    int rc = plan_build_items(p);
    if (rc == GBPERM_OK) rc = plan_capture(p);
    if (rc) {
        plan_free(p);
        return rc;
    }
    gbperm_batch_plan* h = new gbperm_batch_plan{p};
    *out_plan = h;
    return GBPERM_OK;
}

void gbperm_batch_plan_destroy(gbperm_batch_plan* plan) {
    if (!plan) return;
    plan_free(plan->p);
    delete plan;
}

int gbperm_batch_plan_run(gbperm_batch_plan* plan, const double* packed, double* out, gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!plan || !plan->p) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run: null plan");
    BatchPlan* p = plan->p;
    if (p->count > 0 && !out) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run: null output");
    if (p->total_elems > 0 && !packed) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run: null input");
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != p->device) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run: plan belongs to another device");
    // gather device instances into the pinned staging buffer (packed order)
    if (p->ninst > 0) {
        for (int64_t i = 0; i < p->count; ++i) {
            if (p->dev_index[i] < 0) continue;
            std::memcpy(p->hin + 2 * p->off[i], packed + 2 * p->off[i],
                        (size_t)p->rows[i] * p->cols[i] * sizeof(double2));
        }
        if (stats) cudaEventRecord(p->ev0, p->stream);
        cudaError_t e = cudaGraphLaunch(p->graph, p->stream);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_run: graph launch");
        if (stats) cudaEventRecord(p->ev1, p->stream);
        e = cudaStreamSynchronize(p->stream);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_run: kernels");
    }
    double worst = 0.0;  // largest estimate among the double-float results kept
    for (int64_t i = 0; i < p->count; ++i) {
        int d = p->dev_index[i];
        if (d < 0) {
            out[2 * i] = p->trivial[i];
            out[2 * i + 1] = 0.0;
        } else {
            out[2 * i] = p->hout[2 * d];
            out[2 * i + 1] = p->hout[2 * d + 1];
            // the estimate is -2 when the FP64 pass recomputed the instance
            // (its double-float estimate was above the bar; rare: one in
            // thousands of the k = 8..28 batches), -1 for the FP64 product
            if (p->df && p->hest[d] >= 0.0) worst = std::max(worst, p->hest[d]);
        }
    }
    if (stats && p->ninst > 0) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        stats->kernel_ms = ms;
        stats->steps = p->steps;
        stats->flops = p->flops;
        stats->launches = (p->df && p->escalate) ? 5 : 3;  // + the FP64 pass and its finalize
        stats->err_est = worst;
        stats->grid = p->grid;
        stats->seg_log2 = (int)p->item_target_log2;
        stats->arith = p->fx ? GBPERM_ARITH_FX64 : (p->df ? GBPERM_ARITH_DF32 : GBPERM_ARITH_FP64);
    }
    return GBPERM_OK;
}

int gbperm_batch_plan_run_dev(gbperm_batch_plan* plan, const void* d_packed, void* d_out, void* stream) {
    if (!plan || !plan->p) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run_dev: null plan");
    BatchPlan* p = plan->p;
    if (p->count == 0) return GBPERM_OK;
    if (!d_out || (p->total_elems > 0 && !d_packed)) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_run_dev: null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    if (p->ninst > 0) {
        // device-to-device gather of the non-trivial instances is the identity
        // on the packed layout
        e = cudaMemcpyAsync(p->dA, d_packed, (size_t)p->total_elems * sizeof(double2), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_run_dev: copy");
        cudaStream_t saved = p->stream;
        p->stream = st;
        e = plan_enqueue(p);
        p->stream = saved;
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_run_dev: launch");
    }
    // scatter: device instance d -> output slot i (trivial slots get their value)
    const long long cnt = (long long)p->count;
    const int sb = (int)std::min<long long>((cnt + 255) / 256, 1024);
    batched_scatter_kernel<<<sb, 256, 0, st>>>(p->dout, p->ddev_index, p->dtrivial, cnt, static_cast<double*>(d_out));
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_run_dev: scatter");
    return GBPERM_OK;
}

int gbperm_batch_plan_set_item_log2(gbperm_batch_plan* plan, int64_t item_log2) {
    if (!plan || !plan->p) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_set_item_log2: null plan");
    BatchPlan* p = plan->p;
    if (item_log2 < 0 || item_log2 > 40) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_set_item_log2: out of range");
    p->item_target_log2 = item_log2;
    int rc = plan_build_items(p);
    if (rc == GBPERM_OK) rc = plan_capture(p);
    return rc;
}

int64_t gbperm_batch_plan_get_item_log2(gbperm_batch_plan* plan) {
    return (plan && plan->p) ? plan->p->item_target_log2 : -1;
}

int gbperm_batch_plan_autotune(gbperm_batch_plan* plan, const double* packed, int reps, double* best_ms) {
    if (!plan || !plan->p) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_autotune: null plan");
    BatchPlan* p = plan->p;
    if (best_ms) *best_ms = 0.0;
    if (p->ninst == 0) return GBPERM_OK;
    if (p->total_elems > 0 && !packed) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_autotune: null input");
    if (reps < 1) reps = 1;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev != p->device) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_autotune: plan belongs to another device");
    for (int64_t i = 0; i < p->count; ++i) {
        if (p->dev_index[i] < 0) continue;
        std::memcpy(p->hin + 2 * p->off[i], packed + 2 * p->off[i], (size_t)p->rows[i] * p->cols[i] * sizeof(double2));
    }
    // candidates: lanes per segment (double-float: 2 or 4; FP64: 1) x work
    // item sizes around the size-based default; each is planned, captured and
    // timed on the real batch, the fastest is kept
    const int64_t base = p->item_target_log2;
    std::vector<int> groups = (p->df || p->fx) ? std::vector<int>{2, 4} : std::vector<int>{1};
    double best = 1e300;
    int best_grp = p->grp;
    int64_t best_log2 = base;
    for (int grp : groups) {
        for (int64_t dl = -2; dl <= 2; dl += 2) {
            const int64_t l2 = std::min<int64_t>(40, std::max<int64_t>(8, base + dl));
            int cpl = 0, gg = 0;
            if (p->fx) batch_fx_shape(p->maxc, grp, &cpl, &gg);
            else batch_shape(p->maxc, p->df, grp, &cpl, &gg);
            p->cpl = cpl;
            p->grp = gg;
            p->grid = device_sms(p->device) * (p->fx ? batch_fx_bps(cpl, gg) : batch_bps(cpl, gg, p->df));
            p->item_target_log2 = l2;
            int rc = plan_build_items(p);
            if (rc == GBPERM_OK) rc = plan_capture(p);
            if (rc) return rc;
            cudaError_t e = cudaGraphLaunch(p->graph, p->stream);  // warm-up
            if (e == cudaSuccess) e = cudaEventRecord(p->ev0, p->stream);
            for (int r = 0; r < reps && e == cudaSuccess; ++r) e = cudaGraphLaunch(p->graph, p->stream);
            if (e == cudaSuccess) e = cudaEventRecord(p->ev1, p->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_batch_plan_autotune: trial");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, p->ev0, p->ev1);
            const double per = (double)ms / reps;
            if (per < best) {
                best = per;
                best_grp = gg;
                best_log2 = l2;
            }
        }
    }
    int cpl = 0, gg = 0;
    if (p->fx) batch_fx_shape(p->maxc, best_grp, &cpl, &gg);
    else batch_shape(p->maxc, p->df, best_grp, &cpl, &gg);
    p->cpl = cpl;
    p->grp = gg;
    p->grid = device_sms(p->device) * (p->fx ? batch_fx_bps(cpl, gg) : batch_bps(cpl, gg, p->df));
    p->item_target_log2 = best_log2;
    int rc = plan_build_items(p);
    if (rc == GBPERM_OK) rc = plan_capture(p);
    if (rc) return rc;
    if (best_ms) *best_ms = best;
    return GBPERM_OK;
}

int gbperm_batch_plan_get_shape(gbperm_batch_plan* plan, int64_t* lanes_per_segment, int64_t* columns_per_lane) {
    if (!plan || !plan->p) return fail(GBPERM_ERR_ARG, "gbperm_batch_plan_get_shape: null plan");
    if (lanes_per_segment) *lanes_per_segment = plan->p->grp;
    if (columns_per_lane) *columns_per_lane = plan->p->cpl;
    return GBPERM_OK;
}

int gbperm_perm_batched(const double* packed, const int64_t* rows, const int64_t* cols, int64_t count, int arith,
                        double* out, gbperm_stats* stats) {
    gbperm_batch_plan* plan = nullptr;
    int rc = gbperm_batch_plan_create(rows, cols, count, arith, &plan);
    if (rc) return rc;
    rc = gbperm_batch_plan_run(plan, packed, out, stats);
    gbperm_batch_plan_destroy(plan);
    return rc;
}

}  // extern "C"
