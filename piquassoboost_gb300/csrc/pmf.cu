// One probability layer of the generalized Clifford & Clifford sampler.
//
// Replaces compute_pmf (piquassoboost/sampling/simulation_strategies/source/
// samplingHelperFunctions.cpp:78-342), called once per photon by the
// simulation strategies (CGeneralizedCliffordsBSimulationStrategy.cpp:298,
// CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp:262,
// CGeneralizedCliffordsBLossySimulationStrategy.cpp:350).  For every occupied
// input mode l the reference computes the repeated permanent of the sample
// (rows) against the input with one photon removed from l (columns) -- one
// task and one full Gray sweep per l on the CPU, or one multi-input batch on
// its FPGA path (GlynnPermanentCalculatorRepeatedInputBatch_DFE) -- and
// contracts them with the interferometer:
//   pmf[m] ~ | sum_l input[l] * perm_l * U[m][l] |^2,  normalised to sum 1.
//
// All these permanents share the row side (the sample), hence the Gray walk,
// the column sums and the binomial weights; they differ only in the product,
// where column l carries one power less:
//   perm_l = 2^-(N-1) sum_g sign w(g) x_l^(c_l - 1) prod_{j != l} x_j^(c_j).
// One sweep evaluates every perm_l with leave-one-out products (prefix and
// suffix products, no division).  G lanes share a segment; lane g owns
// columns [g*CPL, (g+1)*CPL), gathers the other lanes' partial products and
// forms  prefix x x_c^(c_c - 1) x suffix  for its own columns.  Column sums
// are exact int64 fixed point and the digit walk is the one of
// perm_repeated.cu; the product runs on the FP64 pipe.  A step costs about
// 4 C complex multiplies for all C permanents, against C - 1 per permanent
// (C^2 in all) in the per-mode form.  The double-float twin (pmf_df_kernel)
// is followed by a check kernel that estimates each permanent's rounding
// error and hands the layer to the FP64 kernel when any is above 1e-10.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"
#include "gbperm_fx.cuh"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
constexpr int kFinThreads = 256;

__device__ __forceinline__ cd shfl_cd(cd v, int src) {
    return cd{__shfl_sync(0xffffffffu, v.re, src), __shfl_sync(0xffffffffu, v.im, src)};
}

// x^e for e >= 1 by squaring.  Out of line: reached only for multiplicities
// above 1, and it keeps speculated multiplies off the common path.
__device__ __noinline__ cd cpow_pos(cd x, int e);

// z * x^e (e >= 1), out of line for the same reason
__device__ __noinline__ cd cmul_pow(cd z, cd x, int e) { return cmul(z, cpow_pos(x, e)); }

__device__ __noinline__ cd cpow_pos(cd x, int e) {
    cd acc = x;
    bool have = false;
    cd y = x;
    while (e > 0) {
        if (e & 1) {
            acc = have ? cmul(acc, y) : y;
            have = true;
        }
        e >>= 1;
        if (e) y = cmul(y, y);
    }
    return acc;
}

// Sum each column's per-thread partials -- column g*CPL + c is held by the
// threads t with t % G == g, at s_acc[c * kThreads + t] -- by a tree over t
// (strides kThreads/2 .. G keep the residue mod G) with the (t, c) pairs of
// each level spread over the block; the sum ends at s_acc[c * kThreads + g].
// A few dependent double-double adds per thread instead of kThreads/G in
// one thread: FP64 latency dominates this epilogue on GB300.  Fixed order.
template <int CPL, int G>
__device__ __forceinline__ void column_tree(cdd* s_acc) {
    for (int st = kThreads / 2; st >= G; st >>= 1) {
        for (int it = threadIdx.x; it < st * CPL; it += blockDim.x) {
            const int t = it % st, c = it / st;
            s_acc[c * kThreads + t] = cdd_add(s_acc[c * kThreads + t], s_acc[c * kThreads + t + st]);
        }
        __syncthreads();
    }
}

template <int CPL, int G>
__global__ void __launch_bounds__(kThreads) pmf_kernel(RepArgs p, cdd* col_part) {
    constexpr int NP = CPL * G;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cdd* s_acc = reinterpret_cast<cdd*>(smem_raw);                           // CPL x kThreads
    longlong2* s_a1 = reinterpret_cast<longlong2*>(s_acc + CPL * kThreads);  // R x NP
    longlong2* s_a2 = s_a1 + p.R * NP;                                       // nd x NP
    double* s_w = reinterpret_cast<double*>(s_a2 + p.nd * NP);               // P
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);      // P
    __shared__ int s_cpow[NP];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    // launched as the twin of pmf_df_kernel: run only when the range check
    // sent the product to FP64
    if (p.df_info && p.df_info[1] != 0) return;
    for (int e = threadIdx.x; e < R * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        s_a1[e] = j < C ? p.a1[r * C + j] : make_longlong2(0, 0);
    }
    for (int e = threadIdx.x; e < nd * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        s_a2[e] = j < C ? p.a2[r * C + j] : make_longlong2(0, 0);
    }
    for (long long e = threadIdx.x; e < (long long)p.P; e += blockDim.x) {
        s_w[e] = p.wlow[e];
        s_seq[e] = p.seq[e];
    }
    for (int e = threadIdx.x; e < NP; e += blockDim.x) s_cpow[e] = e < C ? p.cpow[e] : 0;
    for (int e = threadIdx.x; e < nd; e += blockDim.x) s_D[e] = p.D[e];
    for (int e = threadIdx.x; e < R; e += blockDim.x) s_r[e] = p.rcoef[e];
    for (int e = threadIdx.x; e < CPL * kThreads; e += blockDim.x) s_acc[e] = cdd{{0.0, 0.0}, {0.0, 0.0}};
    if (threadIdx.x == 0) {
        long long s = 1;
        for (int i = 0; i < q; ++i) {
            s_stride[i] = s;
            s *= (long long)(p.D[i] + 1);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const int j0 = g * CPL;
    const int lbase = lane - g;
    cdd* my_acc = s_acc + threadIdx.x;  // column c at my_acc[c * kThreads]
    // segments: each warp takes 32/G consecutive ones per pass; the loop
    // bound is warp-uniform so every shuffle runs with the full warp
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / G;
    const unsigned long long lane_seg = (unsigned long long)(lane / G);
    constexpr unsigned long long S = 32 / G;  // segments per warp
    const unsigned long long full = p.nseg / (2 * S) * (2 * S);
    long long cre[CPL], cim[CPL];

    for (unsigned long long hw = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / G;
         hw < p.nseg; hw += T) {
        const unsigned long long h_raw = parity_slot(hw + lane_seg, S, full);
        const bool active = h_raw < p.nseg;
        const unsigned long long h = active ? h_raw : 0ull;
        int gdig[kMaxDigits];
        {
            unsigned long long rem = h;
            int cnt[kMaxDigits];
            for (int i = q; i < nd; ++i) {
                unsigned long long L = (unsigned long long)(s_D[i] + 1);
                cnt[i] = (int)(rem % L);
                rem /= L;
            }
            int par = 0;
            for (int i = nd - 1; i >= 0; --i) {
                int c = i >= q ? cnt[i] : 0;
                int gg = par ? s_D[i] - c : c;
                gdig[i] = gg;
                par ^= gg & 1;
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cre[c] = 0;
            cim[c] = 0;
        }
        int gsum = 0;
        double whigh = 1.0;
        unsigned long long Gd = 0ull;  // low Gray digits, 4 bits each
        unsigned int dir = 0u;         // bit i set: low digit i moves up next
        long long widx = 0;
        for (int i = 0; i < R; ++i) {
            int gi = i < nd ? gdig[i] : 0;
            long long coef = (long long)(s_r[i] - 2 * gi);
            const longlong2* a = s_a1 + i * NP + j0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                longlong2 v = a[c];
                cre[c] += coef * v.x;
                cim[c] += coef * v.y;
            }
            if (i < nd) {
                gsum += gi;
                if (i < q) {
                    Gd |= (unsigned long long)gi << (4 * i);
                    if (gi == 0) dir |= 1u << i;
                    widx += (long long)gi * s_stride[i];
                } else {
                    whigh *= p.binom[s_D[i] * kBinomStride + gi];
                }
            }
        }
        double sgn = (gsum & 1) ? -whigh : whigh;
        if (!active) sgn = 0.0;
        cd blk[CPL];
#pragma unroll
        for (int c = 0; c < CPL; ++c) blk[c] = cd{0.0, 0.0};
        for (unsigned long long k = 0; k < p.P; ++k) {
            if (k != 0) {
                const int d = s_seq[k];  // warp-uniform
                const bool up = (dir >> d) & 1u;
                const int sh = 4 * d;
                int gv = (int)((Gd >> sh) & 15ull);
                gv += up ? 1 : -1;
                Gd = (Gd & ~(15ull << sh)) | ((unsigned long long)gv << sh);
                if (gv == 0 || gv == s_D[d]) dir ^= 1u << d;
                widx += up ? s_stride[d] : -s_stride[d];
                // up: one more -1 delta -> subtract 2 a (warp-uniform: a
                // warp's segments share their parity)
                const longlong2* a = s_a2 + d * NP + j0;
                if (up) {
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
                sgn = -sgn;
                if ((k & 255ull) == 0) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        cdd t = my_acc[c * kThreads];
                        t.re = dd_add_d(t.re, blk[c].re);
                        t.im = dd_add_d(t.im, blk[c].im);
                        my_acc[c * kThreads] = t;
                        blk[c] = cd{0.0, 0.0};
                    }
                }
            }
            // P_c = x_c^(c_c) (1 for padding columns)
            cd Pv[CPL];
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int e = s_cpow[j0 + c];
                cd x{fix_to_double(cre[c]), fix_to_double(cim[c])};
                Pv[c] = e == 1 ? x : (e == 0 ? cd{1.0, 0.0} : cpow_pos(x, e));
            }
            cd part = Pv[0];
#pragma unroll
            for (int c = 1; c < CPL; ++c) part = cmul(part, Pv[c]);
            // weight x product of the other lanes of the group
            cd run{sgn * s_w[widx], 0.0};
#pragma unroll
            for (int t = 1; t < G; ++t) run = cmul(run, shfl_cd(part, lbase + ((g + t) % G)));
            // suffix products: suf[c] = prod_{c' > c} P_c'
            cd suf[CPL];
            suf[CPL - 1] = cd{1.0, 0.0};
            if (CPL > 1) suf[CPL > 1 ? CPL - 2 : 0] = Pv[CPL - 1];
#pragma unroll
            for (int c = CPL - 3; c >= 0; --c) suf[c] = cmul(suf[c + 1], Pv[c + 1]);
            // leave-one-out: run (weight x other lanes x prefix) x x_c^(c_c - 1) x suffix
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int e = s_cpow[j0 + c];
                cd lo = c == CPL - 1 ? run : cmul(run, suf[c]);
                if (e > 1) {
                    cd x{fix_to_double(cre[c]), fix_to_double(cim[c])};
                    lo = cmul_pow(lo, x, e - 1);
                }
                blk[c].re += lo.re;
                blk[c].im += lo.im;
                if (c < CPL - 1) run = cmul(run, Pv[c]);
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cdd t = my_acc[c * kThreads];
            t.re = dd_add_d(t.re, blk[c].re);
            t.im = dd_add_d(t.im, blk[c].im);
            my_acc[c * kThreads] = t;
        }
    }
    __syncthreads();
    column_tree<CPL, G>(s_acc);
    for (int j = threadIdx.x; j < NP; j += blockDim.x) {
        const int gj = j / CPL, c = j % CPL;
        if (j < C) col_part[(size_t)blockIdx.x * C + j] = s_acc[c * kThreads + gj];
    }
}

// ------------------------------------------------ double-float product
// The same sweep with the product as float pairs on the FP32 pipe (the
// arithmetic of perm_repeated_df.cu, error ~2^-46 per complex multiply):
// per step and lane, powers P_c = x_c^(c_c), prefix products (which also give
// the lane's partial product), the other three lanes' partials by shuffle, a
// suffix chain seeded with weight x sign x those partials, and
// LO_c = prefix_c x suffix_c x x_c^(c_c - 1).  Running sums per column are
// lazily normalised float pairs (renormalised every 8 steps), folded into a
// double-double accumulator with the high-digit weight every 256 steps.
// The row tables are interleaved by lane (column g*CPL + c of row r at
// r*NP + c*4 + g) so a walk's four lanes read adjacent words.  Launched as the
// twin of pmf_kernel: whichever the range check does not select returns.

__device__ __forceinline__ cf shfl_cf(const cf& v, int src) {
    return cf{__shfl_sync(0xffffffffu, v.rh, src), __shfl_sync(0xffffffffu, v.rl, src),
              __shfl_sync(0xffffffffu, v.ih, src), __shfl_sync(0xffffffffu, v.il, src)};
}

// x^e by squaring (e >= 1).  Not inlined: it is reached only for columns
// of multiplicity > 1, and one copy instead of one per unrolled column keeps
// the kernel's loop body in the instruction cache.
__device__ __noinline__ cf cf_pow_pos(cf x, int e);

// z * x^e (e >= 1), out of line for the same reason
__device__ __noinline__ cf cf_mul_pow(cf z, cf x, int e) { return cf_mul(z, cf_pow_pos(x, e)); }

__device__ __noinline__ cf cf_pow_pos(cf x, int e) {
    cf acc = x;
    bool have = false;
    cf y = x;
    while (e > 0) {
        if (e & 1) {
            acc = have ? cf_mul(acc, y) : y;
            have = true;
        }
        e >>= 1;
        if (e) y = cf_mul(y, y);
    }
    return acc;
}

__device__ __forceinline__ void df_add_lazy2(float& ah, float& al, float bh, float bl) {
    float s, e;
    two_sum_f(ah, bh, s, e);
    ah = s;
    al = __fadd_rn(al, __fadd_rn(bl, e));
}

__device__ __forceinline__ void df_renorm2(float& h, float& l) {
    float s, e;
    two_sum_f(h, l, s, e);
    h = s;
    l = e;
}

template <int CPL>
__global__ void __launch_bounds__(kThreads) pmf_df_kernel(RepArgs p, cdd* col_part, double* col_s2) {
    constexpr int G = 4;
    constexpr int NP = CPL * G;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cdd* s_acc = reinterpret_cast<cdd*>(smem_raw);                           // CPL x kThreads
    double* s_s2 = reinterpret_cast<double*>(s_acc + CPL * kThreads);        // CPL x kThreads: sum |LO|^2
    longlong2* s_a1 = reinterpret_cast<longlong2*>(s_s2 + CPL * kThreads);   // R x NP (interleaved)
    longlong2* s_a2 = s_a1 + p.R * NP;                                       // nd x NP (interleaved)
    float2* s_w = reinterpret_cast<float2*>(s_a2 + p.nd * NP);               // P: weights as float pairs
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);      // P
    __shared__ int s_cpow[NP];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    if (p.df_info[1] == 0) return;  // range check failed: pmf_kernel runs instead
    for (int e = threadIdx.x; e < R * NP; e += blockDim.x) {
        const int r = e / NP, qq = e % NP, j = (qq % G) * CPL + qq / G;
        s_a1[e] = j < C ? p.a1[r * C + j] : make_longlong2(0, 0);
    }
    for (int e = threadIdx.x; e < nd * NP; e += blockDim.x) {
        const int r = e / NP, qq = e % NP, j = (qq % G) * CPL + qq / G;
        s_a2[e] = j < C ? p.a2[r * C + j] : make_longlong2(0, 0);
    }
    for (long long e = threadIdx.x; e < (long long)p.P; e += blockDim.x) {
        const double w = p.wlow[e];
        const float wh = (float)w;
        s_w[e] = make_float2(wh, (float)(w - (double)wh));
        s_seq[e] = p.seq[e];
    }
    for (int e = threadIdx.x; e < NP; e += blockDim.x) s_cpow[e] = e < C ? p.cpow[e] : 0;
    for (int e = threadIdx.x; e < nd; e += blockDim.x) s_D[e] = p.D[e];
    for (int e = threadIdx.x; e < R; e += blockDim.x) s_r[e] = p.rcoef[e];
    for (int e = threadIdx.x; e < CPL * kThreads; e += blockDim.x) s_acc[e] = cdd{{0.0, 0.0}, {0.0, 0.0}};
    for (int e = threadIdx.x; e < CPL * kThreads; e += blockDim.x) s_s2[e] = 0.0;
    if (threadIdx.x == 0) {
        long long st = 1;
        for (int i = 0; i < q; ++i) {
            s_stride[i] = st;
            st *= (long long)(p.D[i] + 1);
        }
    }
    __syncthreads();

    const DfConv cv = make_dfconv(p.df_info[0]);
    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const int lbase = lane - g;
    cdd* my_acc = s_acc + threadIdx.x;  // column c at my_acc[c * kThreads]
    int cp[CPL];
#pragma unroll
    for (int c = 0; c < CPL; ++c) cp[c] = s_cpow[g * CPL + c];
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / G;
    const unsigned long long lane_seg = (unsigned long long)(lane / G);
    constexpr unsigned long long S = 32 / G;  // segments per warp
    const unsigned long long full = p.nseg / (2 * S) * (2 * S);
    long long cre[CPL], cim[CPL];
    cf Q[CPL];
    float s2f[CPL];  // sum of |LO_c|^2 since the last fold (rounding-error estimate)
    double* my_s2 = s_s2 + threadIdx.x;

    for (unsigned long long hw = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / G;
         hw < p.nseg; hw += T) {
        const unsigned long long h_raw = parity_slot(hw + lane_seg, S, full);
        const bool active = h_raw < p.nseg;
        const unsigned long long h = active ? h_raw : 0ull;
        int gdig[kMaxDigits];
        {
            unsigned long long rem = h;
            int cnt[kMaxDigits];
            for (int i = q; i < nd; ++i) {
                unsigned long long L = (unsigned long long)(s_D[i] + 1);
                cnt[i] = (int)(rem % L);
                rem /= L;
            }
            int par = 0;
            for (int i = nd - 1; i >= 0; --i) {
                int c = i >= q ? cnt[i] : 0;
                int gg = par ? s_D[i] - c : c;
                gdig[i] = gg;
                par ^= gg & 1;
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cre[c] = 0;
            cim[c] = 0;
            Q[c] = cf{0.f, 0.f, 0.f, 0.f};
            s2f[c] = 0.f;
        }
        int gsum = 0;
        double whigh = 1.0;
        unsigned long long Gd = 0ull;  // low Gray digits, 4 bits each
        unsigned int dir = 0u;         // bit i set: low digit i moves up next
        long long widx = 0;
        for (int i = 0; i < R; ++i) {
            int gi = i < nd ? gdig[i] : 0;
            long long coef = (long long)(s_r[i] - 2 * gi);
            const longlong2* a = s_a1 + i * NP + g;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                longlong2 v = a[c * G];
                cre[c] += coef * v.x;
                cim[c] += coef * v.y;
            }
            if (i < nd) {
                gsum += gi;
                if (i < q) {
                    Gd |= (unsigned long long)gi << (4 * i);
                    if (gi == 0) dir |= 1u << i;
                    widx += (long long)gi * s_stride[i];
                } else {
                    whigh *= p.binom[s_D[i] * kBinomStride + gi];
                }
            }
        }
        unsigned int sbit = (unsigned int)(gsum & 1) << 31;
        const float wgt = active ? 1.f : 0.f;
        for (unsigned long long k = 0; k < p.P; ++k) {
            if (k != 0) {
                const int d = s_seq[k];  // warp-uniform
                const bool up = (dir >> d) & 1u;
                const int sh = 4 * d;
                int gv = (int)((Gd >> sh) & 15ull);
                gv += up ? 1 : -1;
                Gd = (Gd & ~(15ull << sh)) | ((unsigned long long)gv << sh);
                if (gv == 0 || gv == s_D[d]) dir ^= 1u << d;
                widx += up ? s_stride[d] : -s_stride[d];
                // up: one more -1 delta -> subtract 2 a (warp-uniform: a
                // warp's segments share their parity)
                const longlong2* a = s_a2 + d * NP + g;
                if (up) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c * G];
                        cre[c] -= v.x;
                        cim[c] -= v.y;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c * G];
                        cre[c] += v.x;
                        cim[c] += v.y;
                    }
                }
                sbit ^= 0x80000000u;
                if ((k & 255ull) == 0) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        cdd t = my_acc[c * kThreads];
                        t.re = dd_add(t.re, dd{(double)Q[c].rh * whigh, (double)Q[c].rl * whigh});
                        t.im = dd_add(t.im, dd{(double)Q[c].ih * whigh, (double)Q[c].il * whigh});
                        my_acc[c * kThreads] = t;
                        Q[c] = cf{0.f, 0.f, 0.f, 0.f};
                        my_s2[c * kThreads] += (double)s2f[c] * whigh * whigh;
                        s2f[c] = 0.f;
                    }
                }
            }
            // P_c = x_c^(c_c) (1 for padding columns)
            cf x[CPL], P[CPL];
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (cp[c] > 0) {
                    fix_to_df_magic(cre[c], cv, x[c].rh, x[c].rl);
                    fix_to_df_magic(cim[c], cv, x[c].ih, x[c].il);
                    P[c] = cp[c] == 1 ? x[c] : cf_pow_pos(x[c], cp[c]);
                } else {
                    x[c] = cf{1.f, 0.f, 0.f, 0.f};
                    P[c] = x[c];
                }
            }
            // prefix products pre[c] = prod_{c' < c} P_c'; the lane's partial
            cf pre[CPL];
            cf part = P[0];
            if (CPL > 1) {
                pre[1] = P[0];
#pragma unroll
                for (int c = 2; c < CPL; ++c) pre[c] = cf_mul(pre[c - 1], P[c - 1]);
                part = cf_mul(pre[CPL - 1], P[CPL - 1]);
            }
            cf o1 = shfl_cf(part, lbase + ((g + 1) & 3));
            cf o2 = shfl_cf(part, lbase + ((g + 2) & 3));
            cf o3 = shfl_cf(part, lbase + ((g + 3) & 3));
            // low-digit weight: exact integer table entry as a float pair
            const float2 w = s_w[widx];
            const float wh = __fmul_rn(w.x, wgt);
            const float wl = __fmul_rn(w.y, wgt);
            cf seed = cf_mul(cf_mul(cf_mul(o1, o2), o3), cf{wh, wl, 0.f, 0.f});
            seed = cf{__uint_as_float(__float_as_uint(seed.rh) ^ sbit), __uint_as_float(__float_as_uint(seed.rl) ^ sbit),
                      __uint_as_float(__float_as_uint(seed.ih) ^ sbit), __uint_as_float(__float_as_uint(seed.il) ^ sbit)};
            // LO_c = seed * prod_{c' > c} P_c' * pre[c] * x_c^(c_c - 1)
            cf suf = seed;
#pragma unroll
            for (int c = CPL - 1; c >= 0; --c) {
                cf lo = (c == 0) ? suf : cf_mul(pre[c], suf);
                if (cp[c] > 1) lo = cf_mul_pow(lo, x[c], cp[c] - 1);
                df_add_lazy2(Q[c].rh, Q[c].rl, lo.rh, lo.rl);
                df_add_lazy2(Q[c].ih, Q[c].il, lo.ih, lo.il);
                s2f[c] = fmaf(lo.rh, lo.rh, fmaf(lo.ih, lo.ih, s2f[c]));
                if (c > 0) suf = cf_mul(suf, P[c]);
            }
            if ((k & 7ull) == 7ull) {
#pragma unroll
                for (int c = 0; c < CPL; ++c) {
                    df_renorm2(Q[c].rh, Q[c].rl);
                    df_renorm2(Q[c].ih, Q[c].il);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cdd t = my_acc[c * kThreads];
            t.re = dd_add(t.re, dd{(double)Q[c].rh * whigh, (double)Q[c].rl * whigh});
            t.im = dd_add(t.im, dd{(double)Q[c].ih * whigh, (double)Q[c].il * whigh});
            my_acc[c * kThreads] = t;
            my_s2[c * kThreads] += (double)s2f[c] * whigh * whigh;
        }
    }
    __syncthreads();
    // column j = g*CPL + c is held by the threads t with t % G == g: sum them
    // in a fixed order
    for (int j = threadIdx.x; j < NP; j += blockDim.x) {
        const int gj = j / CPL, c = j % CPL;
        cdd b = s_acc[c * kThreads + gj];
        double bq = s_s2[c * kThreads + gj];
        for (int t = gj + G; t < kThreads; t += G) {
            b = cdd_add(b, s_acc[c * kThreads + t]);
            bq += s_s2[c * kThreads + t];
        }
        if (j < C) {
            col_part[(size_t)blockIdx.x * C + j] = b;
            col_s2[(size_t)blockIdx.x * C + j] = bq;
        }
    }
}

// Between the double-float kernel and its FP64 twin: sum each column's block
// partials and |LO|^2 sums (a warp per column, fixed order), estimate each
// leave-one-out permanent's relative rounding error as
// sqrt(nfac) 2^-46 sqrt(sum |LO|^2) / |perm|, and when the largest is above
// kDfEscalate (or not finite) clear df_info[1] so that the FP64 twin
// recomputes the whole layer.  err_out receives the largest estimate (-1
// when the range check had already sent the layer to the FP64 kernel).
__global__ void __launch_bounds__(kFinThreads) pmf_check_kernel(const cdd* col_part, const double* col_s2,
                                                                int nblocks, int C, double nfac, int* df_info,
                                                                double* err_out, int escalate) {
    __shared__ double s_max[kFinThreads / 32];
    if (df_info[1] == 0) {  // block-uniform: the double-float kernel did not run
        if (threadIdx.x == 0) *err_out = -1.0;
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double mx = 0.0;
    for (int j = warp; j < C; j += nw) {
        cdd tot{{0.0, 0.0}, {0.0, 0.0}};
        double q = 0.0;
        for (int b = lane; b < nblocks; b += 32) {
            tot = cdd_add(tot, col_part[(size_t)b * C + j]);
            q += col_s2[(size_t)b * C + j];
        }
        tot = warp_sum_cdd(tot);
        q = warp_sum_d(q);
        double est = sqrt(nfac) * 0x1p-46 * sqrt(q) / hypot(tot.re.hi, tot.im.hi);
        if (!(est == est)) est = INFINITY;
        mx = fmax(mx, est);
    }
    if (lane == 0) s_max[warp] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = s_max[0];
        for (int w = 1; w < nw; ++w) m = fmax(m, s_max[w]);
        *err_out = m;
        if (escalate && !(m <= kDfEscalate)) df_info[1] = 0;
    }
}

// Sum the block partials per column in a fixed order and scale: perm_l =
// sum * 2^(exp - e_l + o) (column l lost one factor of its 2^-e_l scaling
// and, in the double-float product, of the range boost 2^o; exp includes the
// boost over all factors, exp_fp64 is the exponent without it).
// Then the contraction with the interferometer and the normalisation, in the
// reference's order (input modes ascending, total over modes ascending).
__global__ void __launch_bounds__(kFinThreads) pmf_finalize_kernel(const cdd* col_part, int nblocks, int C,
                                                                   const int* exp_in, const int* exp_fp64,
                                                                   const int* col_e,
                                                                   const int* df_info, const int* col_mode,
                                                                   const double* cin_w,
                                                                   const double2* U, long long ldu, int m,
                                                                   double* pmf, double2* addends,
                                                                   double2* perm_out, unsigned int* done) {
    // one block per column: the double-double adds run on the FP64 pipe,
    // which retires under two FMA per clock per SM on GB300, so C blocks on
    // C SMs instead of one block for all columns (thread t takes blocks t,
    // t + blockDim, ... in order, then a fixed butterfly and warp order:
    // deterministic)
    __shared__ cdd s_warp[kFinThreads / 32];
    __shared__ bool s_last;
    __shared__ double s_tot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int j = blockIdx.x;
    cdd tot{{0.0, 0.0}, {0.0, 0.0}};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) tot = cdd_add(tot, col_part[(size_t)b * C + j]);
    // a tree over the lanes that hold partials only (ceil(log2 nblocks)
    // levels; a small layer's few blocks skip most of the butterfly)
    const int used = nblocks < 32 ? nblocks : 32;
    int span = 1;
    while (span < used) span <<= 1;
    for (int s = span >> 1; s > 0; s >>= 1) {
        cdd o{{__shfl_down_sync(0xffffffffu, tot.re.hi, s), __shfl_down_sync(0xffffffffu, tot.re.lo, s)},
              {__shfl_down_sync(0xffffffffu, tot.im.hi, s), __shfl_down_sync(0xffffffffu, tot.im.lo, s)}};
        if (lane + s < span) tot = cdd_add(tot, o);
    }
    if (lane == 0) s_warp[warp] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        cdd all = s_warp[0];
        for (int w = 1; w < nwarps; ++w) all = cdd_add(all, s_warp[w]);
        double o[2];
        // the double-float partials carry the range boost; the FP64 twin's
        // (it ran when the range check or the error estimate sent the layer
        // to it) do not
        const bool dfok = df_info && df_info[1];
        const int ex = dfok ? *exp_in - (col_e[j] - df_info[0]) : *exp_fp64 - col_e[j];
        write_result(all, ex, o, nullptr);
        perm_out[j] = make_double2(o[0], o[1]);
        __threadfence();
        s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // the last block: contraction with the interferometer and normalisation,
    // in the reference's order (input modes ascending, total over modes
    // ascending)
    __threadfence();
    const volatile double* pv = reinterpret_cast<const volatile double*>(perm_out);
    for (int i = threadIdx.x; i < m; i += blockDim.x) addends[i] = make_double2(0.0, 0.0);
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) addends[col_mode[c]] = make_double2(pv[2 * c], pv[2 * c + 1]);
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        double re = 0.0, im = 0.0;
        for (int c = 0; c < C; ++c) {
            const double2 u = U[(long long)i * ldu + col_mode[c]];
            const double pr = cin_w[c] * pv[2 * c], pi = cin_w[c] * pv[2 * c + 1];
            re += pr * u.x - pi * u.y;
            im += pr * u.y + pi * u.x;
        }
        pmf[i] = re * re + im * im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < m; ++i) t += pmf[i];
        s_tot = t;
        *done = 0u;  // ready for the next layer
    }
    __syncthreads();
    const double t = s_tot;
    for (int i = threadIdx.x; i < m; i += blockDim.x) pmf[i] = pmf[i] / t;
}

// ------------------------------------------ integer-mantissa product
// The same sweep with every product on 64-bit integer mantissas
// (gbperm_fx.cuh: 31-bit limbs, twelve mad.wide.s32 and a renormalising
// shift per complex multiply, 55-57 significant bits, no range limit): per
// step and lane the prefix products of the powers P_c = x_c^(c_c) (which
// end in the lane's partial product), the other lanes' partials by shuffle
// (limbs and shift count), then backwards LO_c = prefix_c x (others x
// suffix_c) x x_c^(c_c - 1) with P_c recomputed from the column sums: three
// multiplies per column and step, and no array of powers or suffixes kept
// in registers (the kernel fits 3 blocks per SM).  Each LO_c is
// converted to double (fx_to_double: one FP64-pipe conversion per
// component) and accumulated with the step's weight by one FP64 FMA per
// component, so the FP64 pipe carries 4 instructions per column and step
// where pmf_kernel needs about 14.  The
// row tables are interleaved by lane as in pmf_df_kernel.  No twin: the
// product needs no range check and is at least as accurate as FP64.

struct fxs {  // mantissa limbs and shift count: the value m 2^(-61 - s)
    fxl m;
    int s;
};

__device__ __forceinline__ fxs fxs_one() { return fxs{fxl{1 << 27, 0, 0, 0}, -3}; }  // 2^58 2^-58

__device__ __forceinline__ fxs fxs_mul(const fxs& a, const fxs& b) {
    long long rr, ri;
    fx_mul(a.m, b.m, rr, ri);
    fxs r;
    r.s = a.s + b.s - 1;
    r.s += fx_norm(rr, ri, r.m);
    return r;
}

// the column factor x = C 2^-62 of an exact column sum, normalised
__device__ __forceinline__ fxs fxs_col(long long cr, long long ci) {
    fxs r;
    r.s = fx_norm_col(cr, ci, r.m);
    return r;
}

// z x^e (e >= 1), out of line: only columns of multiplicity > 1 reach it
__device__ __noinline__ fxs fxs_mul_pow(fxs z, fxs x, int e) {
    for (int t = 0; t < e; ++t) z = fxs_mul(z, x);
    return z;
}

__device__ __forceinline__ fxs shfl_fxs(const fxs& v, int src) {
    return fxs{fxl{__shfl_sync(0xffffffffu, v.m.rh, src), __shfl_sync(0xffffffffu, v.m.rl, src),
                   __shfl_sync(0xffffffffu, v.m.ih, src), __shfl_sync(0xffffffffu, v.m.il, src)},
               __shfl_sync(0xffffffffu, v.s, src)};
}

template <int CPL, int G>
// 3 blocks per SM (168 registers, no spills): the extra warps cover the
// dependent integer chains
__global__ void __launch_bounds__(kThreads, 3) pmf_fx_kernel(RepArgs p, cdd* col_part) {
    constexpr int NP = CPL * G;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cdd* s_acc = reinterpret_cast<cdd*>(smem_raw);                           // CPL x kThreads
    longlong2* s_a1 = reinterpret_cast<longlong2*>(s_acc + CPL * kThreads);  // R x NP (interleaved)
    longlong2* s_a2 = s_a1 + p.R * NP;                                       // nd x NP (interleaved)
    double* s_w = reinterpret_cast<double*>(s_a2 + p.nd * NP);               // P
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);      // P
    __shared__ int s_cpow[NP];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    // column g*CPL + c of row r at r*NP + c*G + g: a walk's G lanes read
    // adjacent words
    for (int e = threadIdx.x; e < R * NP; e += blockDim.x) {
        const int r = e / NP, qq = e % NP, j = (qq % G) * CPL + qq / G;
        s_a1[e] = j < C ? p.a1[r * C + j] : make_longlong2(0, 0);
    }
    for (int e = threadIdx.x; e < nd * NP; e += blockDim.x) {
        const int r = e / NP, qq = e % NP, j = (qq % G) * CPL + qq / G;
        s_a2[e] = j < C ? p.a2[r * C + j] : make_longlong2(0, 0);
    }
    for (long long e = threadIdx.x; e < (long long)p.P; e += blockDim.x) {
        s_w[e] = p.wlow[e];
        s_seq[e] = p.seq[e];
    }
    for (int e = threadIdx.x; e < NP; e += blockDim.x) s_cpow[e] = e < C ? p.cpow[e] : 0;
    for (int e = threadIdx.x; e < nd; e += blockDim.x) s_D[e] = p.D[e];
    for (int e = threadIdx.x; e < R; e += blockDim.x) s_r[e] = p.rcoef[e];
    for (int e = threadIdx.x; e < CPL * kThreads; e += blockDim.x) s_acc[e] = cdd{{0.0, 0.0}, {0.0, 0.0}};
    if (threadIdx.x == 0) {
        long long st = 1;
        for (int i = 0; i < q; ++i) {
            s_stride[i] = st;
            st *= (long long)(p.D[i] + 1);
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int g = lane % G;
    const int lbase = lane - g;
    const int j0 = g * CPL;
    // the padding columns of the last lanes (j >= C) carry the exact value
    // 1 (column sum 2^62, power 0) and go through the products like the
    // others -- no per-column predicate; their leave-one-out sums are not
    // written
    unsigned int extra = 0u;  // bit c: column c has power > 1
#pragma unroll
    for (int c = 0; c < CPL; ++c)
        if (s_cpow[j0 + c] > 1) extra |= 1u << c;
    cdd* my_acc = s_acc + threadIdx.x;  // column c at my_acc[c * kThreads]
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / G;
    const unsigned long long lane_seg = (unsigned long long)(lane / G);
    constexpr unsigned long long S = 32 / G;  // segments per warp
    const unsigned long long full = p.nseg / (2 * S) * (2 * S);
    long long cre[CPL], cim[CPL];

    for (unsigned long long hw = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / G;
         hw < p.nseg; hw += T) {
        const unsigned long long h_raw = parity_slot(hw + lane_seg, S, full);
        const bool active = h_raw < p.nseg;
        const unsigned long long h = active ? h_raw : 0ull;
        int gdig[kMaxDigits];
        {
            unsigned long long rem = h;
            int cnt[kMaxDigits];
            for (int i = q; i < nd; ++i) {
                unsigned long long L = (unsigned long long)(s_D[i] + 1);
                cnt[i] = (int)(rem % L);
                rem /= L;
            }
            int par = 0;
            for (int i = nd - 1; i >= 0; --i) {
                int c = i >= q ? cnt[i] : 0;
                int gg = par ? s_D[i] - c : c;
                gdig[i] = gg;
                par ^= gg & 1;
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cre[c] = j0 + c < C ? 0 : (1ll << GBPERM_FIX_BITS);
            cim[c] = 0;
        }
        int gsum = 0;
        double whigh = 1.0;
        unsigned long long Gd = 0ull;  // low Gray digits, 4 bits each
        unsigned int dir = 0u;         // bit i set: low digit i moves up next
        long long widx = 0;
        for (int i = 0; i < R; ++i) {
            int gi = i < nd ? gdig[i] : 0;
            long long coef = (long long)(s_r[i] - 2 * gi);
            const longlong2* a = s_a1 + i * NP + g;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                longlong2 v = a[c * G];
                cre[c] += coef * v.x;
                cim[c] += coef * v.y;
            }
            if (i < nd) {
                gsum += gi;
                if (i < q) {
                    Gd |= (unsigned long long)gi << (4 * i);
                    if (gi == 0) dir |= 1u << i;
                    widx += (long long)gi * s_stride[i];
                } else {
                    whigh *= p.binom[s_D[i] * kBinomStride + gi];
                }
            }
        }
        double sgn = (gsum & 1) ? -whigh : whigh;
        if (!active) sgn = 0.0;
        cd blk[CPL];
#pragma unroll
        for (int c = 0; c < CPL; ++c) blk[c] = cd{0.0, 0.0};
        for (unsigned long long k = 0; k < p.P; ++k) {
            if (k != 0) {
                const int d = s_seq[k];  // warp-uniform
                const bool up = (dir >> d) & 1u;
                const int sh = 4 * d;
                int gv = (int)((Gd >> sh) & 15ull);
                gv += up ? 1 : -1;
                Gd = (Gd & ~(15ull << sh)) | ((unsigned long long)gv << sh);
                if (gv == 0 || gv == s_D[d]) dir ^= 1u << d;
                widx += up ? s_stride[d] : -s_stride[d];
                const longlong2* a = s_a2 + d * NP + g;
                if (up) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c * G];
                        cre[c] -= v.x;
                        cim[c] -= v.y;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c * G];
                        cre[c] += v.x;
                        cim[c] += v.y;
                    }
                }
                sgn = -sgn;
                if ((k & 255ull) == 0) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        cdd t = my_acc[c * kThreads];
                        t.re = dd_add_d(t.re, blk[c].re);
                        t.im = dd_add_d(t.im, blk[c].im);
                        my_acc[c * kThreads] = t;
                        blk[c] = cd{0.0, 0.0};
                    }
                }
            }
            // prefix products pre[c] = prod_{c' < c} P_c' and the lane's
            // partial product; P_c = x_c^(c_c) is recomputed from the column
            // sums in the backward pass instead of being kept
            fxs pre[CPL];
            fxs part = fxs_one();
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                fxs pc = fxs_col(cre[c], cim[c]);
                if ((extra >> c) & 1u) pc = fxs_mul_pow(pc, pc, s_cpow[j0 + c] - 1);
                pre[c] = part;
                part = (c == 0) ? pc : fxs_mul(part, pc);
            }
            // the other lanes' partials, then backwards:
            // LO_c = prefix_c x (others x suffix_c) x x_c^(c_c - 1)
            fxs run = shfl_fxs(part, lbase + ((g + 1) % G));
#pragma unroll
            for (int t = 2; t < G; ++t) run = fxs_mul(run, shfl_fxs(part, lbase + ((g + t) % G)));
            const double w = sgn * s_w[widx];
#pragma unroll
            for (int c = CPL - 1; c >= 0; --c) {
                fxs lo = (c == 0) ? run : fxs_mul(pre[c], run);
                if ((extra >> c) & 1u) lo = fxs_mul_pow(lo, fxs_col(cre[c], cim[c]), s_cpow[j0 + c] - 1);
                const int ex = -61 - lo.s;
                blk[c].re = fma(w, fx_to_double(fx_join(lo.m.rh, lo.m.rl), ex), blk[c].re);
                blk[c].im = fma(w, fx_to_double(fx_join(lo.m.ih, lo.m.il), ex), blk[c].im);
                if (c > 0) {
                    fxs pc = fxs_col(cre[c], cim[c]);
                    if ((extra >> c) & 1u) pc = fxs_mul_pow(pc, pc, s_cpow[j0 + c] - 1);
                    run = fxs_mul(run, pc);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cdd t = my_acc[c * kThreads];
            t.re = dd_add_d(t.re, blk[c].re);
            t.im = dd_add_d(t.im, blk[c].im);
            my_acc[c * kThreads] = t;
        }
    }
    __syncthreads();
    column_tree<CPL, G>(s_acc);
    for (int j = threadIdx.x; j < NP; j += blockDim.x) {
        const int gj = j / CPL, c = j % CPL;
        if (j < C) col_part[(size_t)blockIdx.x * C + j] = s_acc[c * kThreads + gj];
    }
}

template <int CPL, int G>
size_t pmf_smem(const RepArgs& a) {
    return (size_t)CPL * kThreads * sizeof(cdd) + (size_t)(a.R + a.nd) * CPL * G * sizeof(longlong2) +
           (size_t)a.P * (sizeof(double) + 1) + 16;
}

template <int CPL, int G>
int pmf_bps_t(const RepArgs& a) {
    int nb = 0;
    size_t smem = pmf_smem<CPL, G>(a);
    allow_max_dynamic_smem((const void*)pmf_kernel<CPL, G>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pmf_kernel<CPL, G>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

template <int CPL, int G>
cudaError_t pmf_launch_t(const RepArgs& a, cdd* col_part, int grid, cudaStream_t st) {
    size_t smem = pmf_smem<CPL, G>(a);
    cudaError_t e =
        allow_max_dynamic_smem((const void*)pmf_kernel<CPL, G>);
    if (e != cudaSuccess) return e;
    pmf_kernel<CPL, G><<<grid, kThreads, smem, st>>>(a, col_part);
    return cudaGetLastError();
}

// lane-group shape for C product columns: 4 lanes up to 32 columns, 8 above
void pmf_shape(int C, int* cpl, int* grp) {
    *grp = 4;
    if (C <= 4) *cpl = 1;
    else if (C <= 8) *cpl = 2;
    else if (C <= 16) *cpl = 4;
    else if (C <= 32) *cpl = 8;
    else *cpl = 8, *grp = 8;
}

int pmf_bps(const RepArgs& a, int cpl, int grp) {
    if (grp == 8) return pmf_bps_t<8, 8>(a);
    switch (cpl) {
        case 1: return pmf_bps_t<1, 4>(a);
        case 2: return pmf_bps_t<2, 4>(a);
        case 4: return pmf_bps_t<4, 4>(a);
        default: return pmf_bps_t<8, 4>(a);
    }
}

cudaError_t pmf_launch(const RepArgs& a, int cpl, int grp, cdd* col_part, int grid, cudaStream_t st) {
    if (grp == 8) return pmf_launch_t<8, 8>(a, col_part, grid, st);
    switch (cpl) {
        case 1: return pmf_launch_t<1, 4>(a, col_part, grid, st);
        case 2: return pmf_launch_t<2, 4>(a, col_part, grid, st);
        case 4: return pmf_launch_t<4, 4>(a, col_part, grid, st);
        default: return pmf_launch_t<8, 4>(a, col_part, grid, st);
    }
}

template <int CPL, int G>
int pmf_fx_bps_t(const RepArgs& a) {
    int nb = 0;
    size_t smem = pmf_smem<CPL, G>(a);
    allow_max_dynamic_smem((const void*)pmf_fx_kernel<CPL, G>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pmf_fx_kernel<CPL, G>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

template <int CPL, int G>
cudaError_t pmf_fx_launch_t(const RepArgs& a, cdd* col_part, int grid, cudaStream_t st) {
    size_t smem = pmf_smem<CPL, G>(a);
    cudaError_t e = allow_max_dynamic_smem((const void*)pmf_fx_kernel<CPL, G>);
    if (e != cudaSuccess) return e;
    pmf_fx_kernel<CPL, G><<<grid, kThreads, smem, st>>>(a, col_part);
    return cudaGetLastError();
}

int pmf_fx_bps(const RepArgs& a, int cpl, int grp) {
    if (grp == 8) return pmf_fx_bps_t<8, 8>(a);
    switch (cpl) {
        case 1: return pmf_fx_bps_t<1, 4>(a);
        case 2: return pmf_fx_bps_t<2, 4>(a);
        case 4: return pmf_fx_bps_t<4, 4>(a);
        default: return pmf_fx_bps_t<8, 4>(a);
    }
}

cudaError_t pmf_fx_launch(const RepArgs& a, int cpl, int grp, cdd* col_part, int grid, cudaStream_t st) {
    if (grp == 8) return pmf_fx_launch_t<8, 8>(a, col_part, grid, st);
    switch (cpl) {
        case 1: return pmf_fx_launch_t<1, 4>(a, col_part, grid, st);
        case 2: return pmf_fx_launch_t<2, 4>(a, col_part, grid, st);
        case 4: return pmf_fx_launch_t<4, 4>(a, col_part, grid, st);
        default: return pmf_fx_launch_t<8, 4>(a, col_part, grid, st);
    }
}

template <int CPL>
size_t pmf_df_smem(const RepArgs& a) {
    return pmf_smem<CPL, 4>(a) + (size_t)CPL * kThreads * sizeof(double);
}

template <int CPL>
int pmf_df_bps_t(const RepArgs& a) {
    int nb = 0;
    size_t smem = pmf_df_smem<CPL>(a);
    allow_max_dynamic_smem((const void*)pmf_df_kernel<CPL>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pmf_df_kernel<CPL>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

template <int CPL>
cudaError_t pmf_df_launch_t(const RepArgs& a, cdd* col_part, double* col_s2, int grid, cudaStream_t st) {
    size_t smem = pmf_df_smem<CPL>(a);
    cudaError_t e = allow_max_dynamic_smem((const void*)pmf_df_kernel<CPL>);
    if (e != cudaSuccess) return e;
    pmf_df_kernel<CPL><<<grid, kThreads, smem, st>>>(a, col_part, col_s2);
    return cudaGetLastError();
}

int pmf_df_bps(const RepArgs& a, int cpl) {
    switch (cpl) {
        case 1: return pmf_df_bps_t<1>(a);
        case 2: return pmf_df_bps_t<2>(a);
        case 4: return pmf_df_bps_t<4>(a);
        default: return pmf_df_bps_t<8>(a);
    }
}

cudaError_t pmf_df_launch(const RepArgs& a, int cpl, cdd* col_part, double* col_s2, int grid, cudaStream_t st) {
    switch (cpl) {
        case 1: return pmf_df_launch_t<1>(a, col_part, col_s2, grid, st);
        case 2: return pmf_df_launch_t<2>(a, col_part, col_s2, grid, st);
        case 4: return pmf_df_launch_t<4>(a, col_part, col_s2, grid, st);
        default: return pmf_df_launch_t<8>(a, col_part, col_s2, grid, st);
    }
}

// FP64 flops of one Gray step of pmf_kernel: per lane CPL-1 (partial
// product) + G-1 (gather) + CPL-2 (suffix) + 2 (CPL-1) (leave-one-out)
// complex products of 6 flops, plus 2 adds per column
double pmf_step_flops(int C, int cpl, int grp) {
    double cm = (double)(cpl - 1) + (grp - 1) + std::max(cpl - 2, 0) + 2.0 * (cpl - 1);
    return 6.0 * cm * grp + 2.0 * C;
}

}  // namespace

}  // namespace gbperm

using namespace gbperm;

extern "C" int gbperm_compute_pmf(const double* U, int64_t m, int64_t ld, const int64_t* sample,
                                  const int64_t* current_input, int arith, double* pmf, double* addends,
                                  gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: unknown arithmetic");
    bool fx = arith == GBPERM_ARITH_FX64;
    if (m <= 0) return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: no modes");
    if (!U || !sample || !current_input || !pmf) return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: null argument");
    if (ld < m) return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: ld < m");
    int64_t ns = 0, ni = 0;
    std::vector<int> cols;  // occupied input modes, ascending
    for (int64_t i = 0; i < m; ++i) {
        if (sample[i] < 0 || current_input[i] < 0)
            return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: negative occupation");
        ns += sample[i];
        ni += current_input[i];
        if (current_input[i] > 0) cols.push_back((int)i);
    }
    if (ni == 0) return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: empty input state");
    if (ns + 1 != ni)
        return fail(GBPERM_ERR_STATE_SUM,
                    "gbperm_compute_pmf: the input state must hold one photon more than the sample");
    if (ns > 64) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_compute_pmf: more than 64 photons in the sample");
    if (!all_finite(U, m, m, ld)) return fail(GBPERM_ERR_ARG, "gbperm_compute_pmf: non-finite interferometer");

    RepHost h;
    const bool first_photon = (ns == 0);
    if (!first_photon) {
        double triv[2];
        bool is_triv = false;
        int rc = repeated_plan(U, m, m, ld, current_input, m, sample, m, &h, triv, &is_triv, false, 1);
        if (rc) return rc;
    } else {
        h.C = (int)cols.size();
        h.col_src = cols;
    }
    const int C = h.C;
    if (C > 64) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_compute_pmf: more than 64 occupied input modes");
    RepArgs a{};
    int cpl = 1, grp = 4, grid = 1;
    bool df = false;
    if (!first_photon) {
        a.R = h.R;
        a.C = h.C;
        a.nd = h.nd;
        pmf_shape(C, &cpl, &grp);
        // double-float product for up to 32 columns (4 lanes x 8), up to the
        // df.pmf_max_photons size rule, when the dynamic range allows; the
        // device check decides between it and its FP64 twin.  Otherwise a
        // double-float request runs the integer-mantissa layer (faster than
        // the FP64 one and at least as accurate)
        if (arith == GBPERM_ARITH_DF32 && grp == 4 && ns <= g_opt.df_pmf_max_photons.load()) {
            int boost = 0;
            df = df_boost(h.M.data(), h.R, h.C, h.C, h.rcoef.data(), h.cpow.data(), &boost);
        }
        if (arith == GBPERM_ARITH_DF32 && !df) fx = true;
    }
    ThreadCtx& cx = thread_ctx();
    int rc = cx.ensure(0);  // device check before any runtime query
    if (rc) return rc;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!first_photon) {
        // both twins launch on one grid of grp lanes per segment; setup costs
        // (in steps) fitted to kernel times of 60-mode, 30-photon layers --
        // the double-float one flushes its per-column double-double
        // accumulators once per segment
        const unsigned long long sms = (unsigned long long)device_sms(dev);
        repeated_low_digits(
            &h,
            [&](unsigned long long P) {
                RepArgs t = a;
                t.P = P;
                int b = fx ? pmf_fx_bps(t, cpl, grp) : pmf_bps(t, cpl, grp);
                if (df) b = std::min(b, pmf_df_bps(t, cpl));
                return sms * (unsigned long long)b * (unsigned long long)(kThreads / grp);
            },
            df ? 20.0 : (fx ? 4.0 : 2.0));
        a.q = h.q;
        a.P = h.P;
        a.nseg = h.nseg;
        int bps = fx ? pmf_fx_bps(a, cpl, grp) : pmf_bps(a, cpl, grp);
        if (df) bps = std::min(bps, pmf_df_bps(a, cpl));
        unsigned long long full = (unsigned long long)device_sms(dev) * bps;
        unsigned long long per_block = (unsigned long long)(kThreads / grp);
        unsigned long long need = (h.nseg + per_block - 1) / per_block;
        grid = (int)std::max(1ull, std::min(full, need));
    }
    // device layout
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes, 256);
        return o;
    };
    const size_t o_U = take((size_t)m * m * sizeof(double2));
    const size_t o_M = take(h.M.size() * sizeof(double));
    const size_t o_a1 = take((size_t)h.R * C * sizeof(longlong2));
    const size_t o_a2 = take((size_t)h.R * C * sizeof(longlong2));
    const size_t o_ints = take((size_t)(h.R + h.nd + 3 * C + 64) * sizeof(int));
    const size_t o_cw = take((size_t)C * sizeof(double));
    const size_t o_wlow = take(h.wlow.size() * sizeof(double));
    const size_t o_seq = take(h.seq.size());
    const size_t o_binom = take((size_t)kBinomStride * kBinomStride * sizeof(double));
    const size_t o_exp = take(64);
    const size_t o_pmf = take((size_t)m * sizeof(double));
    const size_t o_add = take((size_t)m * sizeof(double2));  // 16-byte elements: own aligned region
    const size_t o_part = take((size_t)grid * C * sizeof(cdd));
    const size_t o_s2 = take((size_t)grid * C * sizeof(double));
    const size_t o_perm = take((size_t)C * sizeof(double2) + sizeof(unsigned int));
    rc = cx.ensure(off);
    if (rc) return rc;
    char* base = static_cast<char*>(cx.dbuf);
    cudaStream_t st = cx.stream;

    // interferometer, dense (ld = m) complex128
    std::vector<double> Ud((size_t)m * m * 2);
    for (int64_t i = 0; i < m; ++i)
        std::memcpy(&Ud[(size_t)i * m * 2], U + 2 * i * ld, (size_t)m * 2 * sizeof(double));
    std::vector<int> ints;
    ints.insert(ints.end(), h.rcoef.begin(), h.rcoef.end());
    ints.insert(ints.end(), h.D.begin(), h.D.end());
    ints.insert(ints.end(), h.cpow.begin(), h.cpow.end());
    const size_t i_cole = ints.size();
    ints.resize(ints.size() + C, 0);  // per-column exponents (written by the prepare kernel)
    const size_t i_mode = ints.size();
    ints.insert(ints.end(), h.col_src.begin(), h.col_src.end());
    std::vector<double> cw(C);
    for (int j = 0; j < C; ++j) cw[j] = (double)current_input[h.col_src[j]];
    cudaError_t e = cudaMemcpyAsync(base + o_U, Ud.data(), Ud.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !h.M.empty())
        e = cudaMemcpyAsync(base + o_M, h.M.data(), h.M.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + o_ints, ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + o_cw, cw.data(), cw.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !h.wlow.empty())
        e = cudaMemcpyAsync(base + o_wlow, h.wlow.data(), h.wlow.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !h.seq.empty())
        e = cudaMemcpyAsync(base + o_seq, h.seq.data(), h.seq.size(), cudaMemcpyHostToDevice, st);
    const std::vector<double>& bt = binom_table();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + o_binom, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: upload");
    int* d_ints = reinterpret_cast<int*>(base + o_ints);
    int* d_exp = reinterpret_cast<int*>(base + o_exp);
    cdd* d_part = reinterpret_cast<cdd*>(base + o_part);
    int nblocks = grid;
    std::vector<cdd> ones;
    std::vector<int> zero;
    if (stats) cudaEventRecord(cx.ev0, st);
    if (!first_photon) {
        PrepArgs pa;
        pa.A = reinterpret_cast<const double2*>(base + o_M);
        pa.ld = C;
        pa.rows = h.R;
        pa.cols = C;
        pa.row_w = d_ints;
        pa.col_w = d_ints + h.R + h.nd;
        pa.norm_shift = h.norm_shift;
        pa.a1 = reinterpret_cast<longlong2*>(base + o_a1);
        pa.a2 = reinterpret_cast<longlong2*>(base + o_a2);
        pa.exp_out = d_exp;
        pa.col_e_out = d_ints + i_cole;
        pa.df = df ? 1 : 0;
        pa.df_info = df ? d_exp + 4 : nullptr;
        pa.row_balance = 1;
        pa.exp_fp64_out = d_exp + 1;
        e = launch_prepare(pa, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: prepare");
        a.a1 = pa.a1;
        a.a2 = pa.a2;
        a.rcoef = d_ints;
        a.D = d_ints + h.R;
        a.cpow = d_ints + h.R + h.nd;
        a.wlow = reinterpret_cast<const double*>(base + o_wlow);
        a.seq = reinterpret_cast<const unsigned char*>(base + o_seq);
        a.binom = reinterpret_cast<const double*>(base + o_binom);
        a.df_info = pa.df_info;
        if (df) {
            double* d_s2 = reinterpret_cast<double*>(base + o_s2);
            e = pmf_df_launch(a, cpl, d_part, d_s2, grid, st);
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: df launch");
            // error estimate before the FP64 twin, which runs when it fails
            pmf_check_kernel<<<1, kFinThreads, 0, st>>>(d_part, d_s2, grid, C, (double)h.photons, d_exp + 4,
                                                        reinterpret_cast<double*>(d_exp + 8),
                                                        g_opt.df_escalate.load() != 0 ? 1 : 0);
            e = cudaGetLastError();
            if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: check launch");
        }
        // the integer-mantissa layer runs alone (no range check, no twin)
        e = fx ? pmf_fx_launch(a, cpl, grp, d_part, grid, st) : pmf_launch(a, cpl, grp, d_part, grid, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: launch");
    } else {
        // no sample yet: every permanent is of an empty matrix, i.e. 1
        ones.assign(C, cdd{{1.0, 0.0}, {0.0, 0.0}});
        zero.assign(2, 0);  // exponent with and without the boost
        e = cudaMemcpyAsync(d_part, ones.data(), C * sizeof(cdd), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_exp, zero.data(), 2 * sizeof(int), cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: upload");
        nblocks = 1;
    }
    double* d_pmf = reinterpret_cast<double*>(base + o_pmf);
    double2* d_add = reinterpret_cast<double2*>(base + o_add);
    double2* d_perm = reinterpret_cast<double2*>(base + o_perm);
    unsigned int* d_done = reinterpret_cast<unsigned int*>(d_perm + C);
    e = cudaMemsetAsync(d_done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: finalize counter");
    // one warp per column: a warp-wide double-double add costs the FP64
    // pipe the same whatever the partial count, so fewer, fuller warps
    pmf_finalize_kernel<<<C, 32, 0, st>>>(d_part, nblocks, C, d_exp, d_exp + 1, d_ints + i_cole,
                                          df ? d_exp + 4 : nullptr, d_ints + i_mode,
                                          reinterpret_cast<const double*>(base + o_cw),
                                          reinterpret_cast<const double2*>(base + o_U), m, (int)m, d_pmf, d_add,
                                          d_perm, d_done);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: finalize");
    if (stats) cudaEventRecord(cx.ev1, st);
    e = cudaMemcpyAsync(pmf, d_pmf, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && addends)
        e = cudaMemcpyAsync(addends, d_add, (size_t)m * sizeof(double2), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_compute_pmf: kernel");
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, cx.ev0, cx.ev1);
        stats->kernel_ms = ms;
        stats->steps = first_photon ? 0.0 : h.steps;
        stats->flops = first_photon ? 0.0 : pmf_step_flops(C, cpl, grp) * h.steps;
        stats->launches = first_photon ? 1 : (df ? 5 : 3);
        stats->grid = grid;
        stats->seg_log2 = h.q;
        int info[2] = {0, 0};
        double est = 0.0;
        if (df && !first_photon) {
            cudaMemcpy(info, d_exp + 4, sizeof(info), cudaMemcpyDeviceToHost);
            cudaMemcpy(&est, d_exp + 8, sizeof(est), cudaMemcpyDeviceToHost);
        }
        const bool used_df = df && !first_photon && info[1];
        stats->arith = fx ? GBPERM_ARITH_FX64 : (used_df ? GBPERM_ARITH_DF32 : GBPERM_ARITH_FP64);
        stats->err_est = (df && !first_photon && est >= 0.0) ? est : 0.0;
    }
    return GBPERM_OK;
}
