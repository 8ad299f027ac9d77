// Repeated-multiplicity permanent with the double-float product (GB300).
//
// Same sum, digit plan and exact int64 column sums as perm_repeated.cu
// (BBFGPermanentCalculatorRepeated.hpp:116-307); the product
// prod_j colsum_j^(c_j) runs as float pairs on the FP32 pipe, with lane groups
// as in perm_plain_df.cu: GROUP lanes walk one segment, lane g owns columns
// [g*CPL, (g+1)*CPL) and a shuffle butterfly multiplies the partials.  Every
// lane of a group tracks the same Gray digits (they are cheap integers), so
// the weights and signs need no exchange.  Segment loops run over warp-sized
// blocks of segments so all 32 lanes always reach the shuffles.  As in
// perm_plain_df.cu the sweep ends with a rounding-error estimate that hands
// the result to the integer-mantissa twin when it is above 1e-10 (at 30
// photons most bunched outputs are; the host then skips this kernel).
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
}

// x^e by squaring (e >= 1).  Not inlined: it is reached only for columns
// of multiplicity > 1, and one copy instead of one per unrolled column keeps
// the kernel's loop body in the instruction cache.
__device__ __noinline__ cf cf_pow(cf x, int e) {
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

template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads) repeated_df_kernel(RepArgs p) {
    constexpr int NP = CPL * GROUP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);            // R x NP
    longlong2* s_a2 = s_a1 + p.R * NP;                                   // nd x NP
    float2* s_w = reinterpret_cast<float2*>(s_a2 + p.nd * NP);           // P: weights as float pairs
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);  // P
    __shared__ int s_cpow[NP];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    if (p.df_info[1] == 0) {  // range check failed: the FP64 kernel runs instead
        if (blockIdx.x == 0 && threadIdx.x == 0 && p.err_out) *p.err_out = -1.0;
        return;
    }
    for (int e = threadIdx.x; e < R * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        s_a1[e] = j < C ? p.a1[r * C + j] : make_longlong2(0, 0);
    }
    for (int e = threadIdx.x; e < nd * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        s_a2[e] = j < C ? p.a2[r * C + j] : make_longlong2(0, 0);
    }
    // low-digit weights (exact integers) as float pairs, converted once here
    // instead of on the FP64 pipe every step
    for (long long e = threadIdx.x; e < (long long)p.P; e += blockDim.x) {
        const double w = p.wlow[e];
        const float wh = (float)w;
        s_w[e] = make_float2(wh, (float)(w - (double)wh));
        s_seq[e] = p.seq[e];
    }
    for (int e = threadIdx.x; e < NP; e += blockDim.x) s_cpow[e] = e < C ? p.cpow[e] : 0;
    for (int e = threadIdx.x; e < nd; e += blockDim.x) s_D[e] = p.D[e];
    for (int e = threadIdx.x; e < R; e += blockDim.x) s_r[e] = p.rcoef[e];
    if (threadIdx.x == 0) {
        long long s = 1;
        for (int i = 0; i < q; ++i) {
            s_stride[i] = s;
            s *= (long long)(p.D[i] + 1);
        }
    }
    __syncthreads();

    const DfConv cv = make_dfconv(p.df_info[0]);
    const int g = threadIdx.x % GROUP;
    const int j0 = g * CPL;
    const bool leader = (g == 0);
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    double s2 = 0.0;  // sum of |term 2^40|^2 (rounding-error estimate)
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / GROUP;
    const unsigned long long lane_seg = (threadIdx.x & 31) / GROUP;
    constexpr unsigned long long S = 32 / GROUP;  // segments per warp
    const unsigned long long full = p.nseg / (2 * S) * (2 * S);
    long long cre[CPL], cim[CPL];

    for (unsigned long long hw = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / GROUP;
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
        unsigned long long Gd = 0ull;
        unsigned int dir = 0u;
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
        unsigned int sbit = (unsigned int)(gsum & 1) << 31;
        float brh = 0.f, brl = 0.f, bih = 0.f, bil = 0.f;
        float s2f = 0.f;  // sum of |term 2^40|^2 (low-digit weight in, high-digit weight out)
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
                // warp-uniform: a warp's segments share their parity
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
                sbit ^= 0x80000000u;
                if ((k & 255ull) == 0) {
                    acc.re = dd_add(acc.re, dd{(double)brh * whigh, (double)brl * whigh});
                    acc.im = dd_add(acc.im, dd{(double)bih * whigh, (double)bil * whigh});
                    brh = brl = bih = bil = 0.f;
                    s2 += (double)s2f * whigh * whigh;
                    s2f = 0.f;
                }
            }
            // a lane's columns are contiguous, so padding (power 0) only ever
            // follows its real columns: the first one starts the product
            cf pa{1.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                const int e = s_cpow[j0 + c];  // 0 for padded columns
                if (e > 0) {
                    cf x;
                    fix_to_df_magic(cre[c], cv, x.rh, x.rl);
                    fix_to_df_magic(cim[c], cv, x.ih, x.il);
                    if (e > 1) x = cf_pow(x, e);
                    pa = c == 0 ? x : cf_mul(pa, x);
                }
            }
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) pa = cf_mul(pa, shfl_xor_cf(pa, m));
            if (leader && active) {
                // weight: exact integer table entry (<= 2^53 here) as a float pair
                const float2 w = s_w[widx];
                cf t = cf_mul(pa, cf{w.x, w.y, 0.f, 0.f});
                df_acc(brh, brl, __uint_as_float(__float_as_uint(t.rh) ^ sbit),
                       __uint_as_float(__float_as_uint(t.rl) ^ sbit));
                df_acc(bih, bil, __uint_as_float(__float_as_uint(t.ih) ^ sbit),
                       __uint_as_float(__float_as_uint(t.il) ^ sbit));
                const float ur = t.rh * 0x1p40f, ui = t.ih * 0x1p40f;
                s2f = fmaf(ur, ur, fmaf(ui, ui, s2f));
            }
        }
        acc.re = dd_add(acc.re, dd{(double)brh * whigh, (double)brl * whigh});
        acc.im = dd_add(acc.im, dd{(double)bih * whigh, (double)bil * whigh});
        s2 += (double)s2f * whigh * whigh;
    }

    df_grid_finish<kThreads>(acc, s2, p.block_part, p.block_s2, p.done, p.exp_in, p.out2, p.out4, p.err_out,
                             p.df_ok, (double)C);
}

template <int CPL, int GROUP>
size_t rep_df_smem(const RepArgs& a) {
    return (size_t)(a.R + a.nd) * CPL * GROUP * sizeof(longlong2) + (size_t)a.P * (sizeof(float2) + 1) + 16;
}

template <int CPL, int GROUP>
cudaError_t launch_rep_df_t(const RepArgs& a, int grid, cudaStream_t st) {
    size_t smem = rep_df_smem<CPL, GROUP>(a);
    cudaError_t e = allow_max_dynamic_smem((const void*)repeated_df_kernel<CPL, GROUP>);
    if (e != cudaSuccess) return e;
    repeated_df_kernel<CPL, GROUP><<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int rep_df_bps_t(const RepArgs& a) {
    int nb = 0;
    size_t smem = rep_df_smem<CPL, GROUP>(a);
    allow_max_dynamic_smem((const void*)repeated_df_kernel<CPL, GROUP>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, repeated_df_kernel<CPL, GROUP>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

#define GBPERM_REP_DF_SHAPES(X) \
    X(4, 2) X(6, 2) X(8, 2) X(10, 2) X(12, 2) X(14, 2) X(16, 2) X(18, 2) X(20, 2) X(24, 2)

}  // namespace

void repeated_df_shape(int cols, int* cpl, int* grp) {
    static const int c2[] = {4, 6, 8, 10, 12, 14, 16, 18, 20, 24};
    *grp = 2;
    *cpl = 24;
    for (int c : c2)
        if (2 * c >= cols) {
            *cpl = c;
            return;
        }
}

int repeated_df_blocks_per_sm(const RepArgs& a, int cpl, int grp) {
#define X(C, G) \
    if (cpl == C && grp == G) return rep_df_bps_t<C, G>(a);
    GBPERM_REP_DF_SHAPES(X)
#undef X
    return 1;
}

cudaError_t launch_repeated_df(RepArgs a, int cpl, int grp, int grid, void* ws, bool escalate, cudaStream_t st) {
    char* w = static_cast<char*>(ws);
    a.block_part = reinterpret_cast<cdd*>(w);
    a.done = reinterpret_cast<unsigned int*>(w + align_up((size_t)grid * sizeof(cdd), 256));
    a.block_s2 = reinterpret_cast<double*>(w + align_up((size_t)grid * sizeof(cdd), 256) + 256);
    a.df_ok = escalate ? const_cast<int*>(a.df_info) + 1 : nullptr;
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
#define X(C, G) \
    if (cpl == C && grp == G) return launch_rep_df_t<C, G>(a, grid, st);
    GBPERM_REP_DF_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

}  // namespace gbperm
