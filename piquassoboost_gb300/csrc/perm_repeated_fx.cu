// Repeated-multiplicity permanent with the integer-mantissa product (GB300
// integer pipes).
//
// Same sum, digit plan and exact int64 column sums as perm_repeated.cu
// (BBFGPermanentCalculatorRepeated.hpp:116-307); the product
// prod_j colsum_j^(c_j) runs on 64-bit integer mantissas in 31-bit limbs
// (gbperm_fx.cuh), with lane groups as in perm_repeated_df.cu: GROUP lanes
// walk one segment, lane g owns columns [g*CPL, (g+1)*CPL), forms their
// partial product in two interleaved chains, and a shuffle butterfly
// multiplies the GROUP partials.  Every lane of a group tracks the same Gray
// digits, so the weights and signs need no exchange.  Lanes 0 and 1 of the
// group convert the term's real and imaginary parts to double (fx_to_double)
// and accumulate weight x term with one FP64 FMA each.  No range check, error estimate or FP64
// twin: each multiply keeps 55-57 significant bits.
#include "gbperm_fx.cuh"
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;

template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads) repeated_fx_kernel(RepArgs p) {
    constexpr int NP = CPL * GROUP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);            // R x NP
    longlong2* s_a2 = s_a1 + p.R * NP;                                   // nd x NP
    double* s_w = reinterpret_cast<double*>(s_a2 + p.nd * NP);           // P
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);  // P
    __shared__ int s_cpow[NP];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    // launched as the twin of the double-float kernel: run only when the
    // range check or the error estimate handed the permanent over
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
    if (threadIdx.x == 0) {
        long long s = 1;
        for (int i = 0; i < q; ++i) {
            s_stride[i] = s;
            s *= (long long)(p.D[i] + 1);
        }
    }
    __syncthreads();

    const int g = threadIdx.x % GROUP;
    // lane g owns columns [g CPL, (g + 1) CPL); the host picks CPL =
    // ceil(C / 2) for lane pairs, so only the last lane may hold padding
    // columns, which carry the exact value 1 (column sum 2^62 at every step)
    // and are multiplied like the others: no per-column predicate
    const int j0 = g * CPL;
    // bit c: this lane's column c has power > 1 (the step loop runs the
    // common power-1 multiply unconditionally); power 0 among the real
    // columns cannot occur (the host drops empty columns), padding columns
    // have power 0 and value 1
    unsigned int extra = 0u;
#pragma unroll
    for (int c = 0; c < CPL; ++c)
        if (s_cpow[j0 + c] > 1) extra |= 1u << c;
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
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
            cre[c] = j0 + c < C ? 0 : (1ll << GBPERM_FIX_BITS);
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
        unsigned long long sbit = (unsigned long long)(gsum & 1) << 63;
        // the lanes of a group end the butterfly with the same product: with
        // GROUP >= 2 lane 0 converts and sums its real part in b0 and lane 1
        // its imaginary part
        double b0 = 0.0, b1 = 0.0;
        const unsigned int P = (unsigned int)p.P;  // at most 4096 (low-digit table)
        for (unsigned int k = 0; k < P; ++k) {
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
                sbit ^= 0x8000000000000000ull;
                if ((k & 255u) == 0) {
                    acc.re = dd_add_d(acc.re, b0 * whigh);
                    b0 = 0.0;
                    if (GROUP == 1) {
                        acc.im = dd_add_d(acc.im, b1 * whigh);
                        b1 = 0.0;
                    }
                }
            }
            // prod_c colsum_c^(power_c) of this lane's columns (padding
            // columns: 1), in two chains; sig: shift count (shifts minus
            // multiplies)
            fxl ch[2];
            int sig = 0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                // a column of power e multiplies its chain e times by the
                // same column factor (the host lays the columns out so that
                // column c of every lane group has nearly the same power: the
                // extra multiplies diverge little)
                const fxl y = fx_col(cre[c], cim[c]);
                if (c < 2) {
                    sig += fx_norm_col(cre[c], cim[c], ch[c]);
                } else {
                    long long rr, ri;
                    fx_mul(ch[c & 1], y, rr, ri);
                    sig += fx_norm(rr, ri, ch[c & 1]) - 1;
                }
                if ((extra >> c) & 1u) {
                    const int e = s_cpow[j0 + c];
                    for (int t = 1; t < e; ++t) {
                        long long rr, ri;
                        fx_mul(ch[c & 1], y, rr, ri);
                        sig += fx_norm(rr, ri, ch[c & 1]) - 1;
                    }
                }
            }
            long long pr, pi;
            fx_mul(ch[0], ch[1], pr, pi);  // every shape has CPL >= 5
            sig -= 1;
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) {
                fxl x;
                sig += fx_norm(pr, pi, x);
                const fxl y = shfl_xor_fxl(x, m);
                sig += __shfl_xor_sync(0xffffffffu, sig, m) - 1;
                fx_mul(x, y, pr, pi);
            }
            if (active && (GROUP == 1 || g < 2)) {
                const int ex = -61 - sig;
                const double w = s_w[widx];
                const long long v0 = GROUP == 1 || g == 0 ? pr : pi;
                const double t0 = __longlong_as_double(__double_as_longlong(fx_to_double(v0, ex)) ^ (long long)sbit);
                b0 = fma(w, t0, b0);
                if (GROUP == 1) {
                    const double t1 =
                        __longlong_as_double(__double_as_longlong(fx_to_double(pi, ex)) ^ (long long)sbit);
                    b1 = fma(w, t1, b1);
                }
            }
        }
        acc.re = dd_add_d(acc.re, b0 * whigh);
        if (GROUP == 1) acc.im = dd_add_d(acc.im, b1 * whigh);
    }
    if (GROUP > 1 && g == 1) {  // lane 1 summed the imaginary part
        acc.im = acc.re;
        acc.re = dd{0.0, 0.0};
    }

    // block reduction (double-double, fixed order); the last block sums the
    // block partials with all its threads
    __shared__ cdd s_warp[kThreads / 32];
    __shared__ bool s_last;
    acc = warp_sum_cdd(acc);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_warp[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        cdd b = s_warp[0];
        for (int w = 1; w < kThreads / 32; ++w) b = cdd_add(b, s_warp[w]);
        p.block_part[blockIdx.x] = b;
        __threadfence();
        unsigned int t = atomicAdd(p.done, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        cdd tot{{0.0, 0.0}, {0.0, 0.0}};
        for (unsigned int bk = threadIdx.x; bk < gridDim.x; bk += blockDim.x) {
            const volatile double* qv = reinterpret_cast<const volatile double*>(&p.block_part[bk]);
            cdd v{{qv[0], qv[1]}, {qv[2], qv[3]}};
            tot = cdd_add(tot, v);
        }
        tot = warp_sum_cdd(tot);
        if (lane == 0) s_warp[warp] = tot;
        __syncthreads();
        if (threadIdx.x == 0) {
            cdd all = s_warp[0];
            for (int w = 1; w < kThreads / 32; ++w) all = cdd_add(all, s_warp[w]);
            write_result(all, *p.exp_in, p.out2, p.out4);
            *p.done = 0u;
        }
    }
}

template <int CPL, int GROUP>
size_t rep_fx_smem(const RepArgs& a) {
    return (size_t)(a.R + a.nd) * CPL * GROUP * sizeof(longlong2) + (size_t)a.P * (sizeof(double) + 1) + 16;
}

template <int CPL, int GROUP>
cudaError_t launch_rep_fx_t(const RepArgs& a, int grid, cudaStream_t st) {
    cudaError_t e = allow_max_dynamic_smem((const void*)repeated_fx_kernel<CPL, GROUP>);
    if (e != cudaSuccess) return e;
    repeated_fx_kernel<CPL, GROUP><<<grid, kThreads, rep_fx_smem<CPL, GROUP>(a), st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int rep_fx_bps_t(const RepArgs& a) {
    int nb = 0;
    allow_max_dynamic_smem((const void*)repeated_fx_kernel<CPL, GROUP>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, repeated_fx_kernel<CPL, GROUP>, kThreads,
                                                  rep_fx_smem<CPL, GROUP>(a));
    return nb > 0 ? nb : 1;
}

// one lane up to 8 columns; lane pairs with an even column count per lane up
// to 40; lane quads up to 64.  Every lane keeps at least one real column.
// lane pairs with CPL = ceil(C / 2) exactly (the unrolled column loop runs
// CPL slots whatever a lane's share, so a rounded-up CPL costs a slot per
// step), quads above 40 columns
#define GBPERM_REP_FX_SHAPES(X)                                                                        \
    X(8, 1) X(5, 2) X(6, 2) X(7, 2) X(8, 2) X(9, 2) X(10, 2) X(11, 2) X(12, 2) X(13, 2) X(14, 2) X(15, 2) \
    X(16, 2) X(17, 2) X(18, 2) X(19, 2) X(20, 2) X(12, 4) X(16, 4)

}  // namespace

void repeated_fx_shape(int cols, int* cpl, int* grp) {
    if (cols <= 8) {
        *cpl = 8;
        *grp = 1;
        return;
    }
    if (cols <= 40) {
        *grp = 2;
        *cpl = (cols + 1) / 2;  // 5..20
        return;
    }
    *grp = 4;
    *cpl = cols <= 48 ? 12 : 16;
}

int repeated_fx_blocks_per_sm(const RepArgs& a, int cpl, int grp) {
#define X(C, G) \
    if (cpl == C && grp == G) return rep_fx_bps_t<C, G>(a);
    GBPERM_REP_FX_SHAPES(X)
#undef X
    return 1;
}

cudaError_t launch_repeated_fx(RepArgs a, int cpl, int grp, int grid, void* ws, cudaStream_t st) {
    char* w = static_cast<char*>(ws);
    a.block_part = reinterpret_cast<cdd*>(w);
    a.done = reinterpret_cast<unsigned int*>(w + align_up((size_t)grid * sizeof(cdd), 256));
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
#define X(C, G) \
    if (cpl == C && grp == G) return launch_rep_fx_t<C, G>(a, grid, st);
    GBPERM_REP_FX_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

}  // namespace gbperm
