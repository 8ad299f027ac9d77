// Plain Glynn / BBFG permanent with the integer-mantissa product (GB300
// integer pipes).
//
// Same sum, Gray order and exact int64 column sums as perm_plain.cu
// (BBFGPermanentCalculator.hpp:87-235).  The n-term complex product runs on
// 64-bit integer mantissas split into 31-bit limbs (gbperm_fx.cuh): twelve
// mad.wide.s32 and a renormalising funnel shift per complex multiply, each
// keeping 55-57 significant bits.  No FP32 range boost, range check or
// error estimate is needed: the product is at least as accurate as the FP64
// kernel's and its exponent is an int.
//
// Lane groups as in perm_plain_df.cu: GROUP consecutive lanes share one Gray
// segment, lane g owns columns [g*CPL, (g+1)*CPL), forms their partial
// product in kChains interleaved chains, and a shuffle butterfly multiplies
// the GROUP partials.  Lanes 0 and 1 of the group convert the term's real
// and imaginary parts to double (fx_to_double) and sum them in double
// (256 steps) folded into a double-double accumulator; the grid
// reduction is the double-double, fixed-order one of the other plain kernels.
#include "gbperm_fx.cuh"
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
constexpr int kChains = 2;

template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads, (CPL <= 16 ? 4 : 3)) plain_fx_kernel(PlainArgs p) {
    constexpr int NP = CPL * GROUP;  // padded columns
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);
    longlong2* s_a2 = s_a1 + p.rows * NP;
    const int rows = p.rows, cols = p.cols;
    // launched as the twin of the double-float kernel: run only when the
    // range check or the error estimate handed the permanent over
    if (p.df_info && p.df_info[1] != 0) return;
    // padding columns (j >= cols) hold the exact value 1 = 2^62 in row 0
    // and 0 elsewhere, so their column sum is 1 at every step and every lane
    // multiplies all CPL of its columns without a per-column predicate
    // (measured 4-10% faster than predicating the padding out)
    for (int e = threadIdx.x; e < rows * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        longlong2 z = make_longlong2(0, 0);
        s_a1[e] = j < cols ? p.a1[r * cols + j] : (r == 0 ? make_longlong2(1ll << GBPERM_FIX_BITS, 0) : z);
        s_a2[e] = j < cols ? p.a2[r * cols + j] : z;
    }
    __syncthreads();

    const int g = threadIdx.x % GROUP;
    const int j0 = g * CPL;
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    const unsigned int L = 1u << p.seg_log2;  // seg_log2 <= 31 (plain_geometry)
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / GROUP;
    long long cre[CPL], cim[CPL];
    // warp-sized blocks of segments: every lane makes the same number of
    // trips (the butterfly shuffles need all 32 lanes); a group whose
    // segment is past the end computes on segment 0 and does not accumulate
    const unsigned long long lane_seg = (threadIdx.x & 31) / GROUP;
    for (unsigned long long sw = ((unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) / GROUP;
         sw < p.nseg; sw += T) {
        const unsigned long long s_raw = sw + lane_seg;
        const bool active = s_raw < p.nseg;
        const unsigned long long s = active ? s_raw : 0ull;
        const unsigned long long i0 = s << p.seg_log2;
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int c = 0; c < CPL; ++c) {
            cre[c] = s_a1[j0 + c].x;
            cim[c] = s_a1[j0 + c].y;
        }
        for (int r = 1; r < rows; ++r) {
            const long long m = -(long long)((g0 >> (rows - 1 - r)) & 1ull);
            const longlong2* a = s_a1 + r * NP + j0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                longlong2 v = a[c];
                cre[c] += (v.x ^ m) - m;
                cim[c] += (v.y ^ m) - m;
            }
        }
        unsigned long long sbit = (unsigned long long)(__popcll(g0) & 1) << 63;
        // the lanes of a group end the butterfly with the same product: with
        // GROUP >= 2 lane 0 converts and sums its real part in b0 and lane 1
        // its imaginary part (half the conversions of one lane doing both)
        double b0 = 0.0, b1 = 0.0;
        for (unsigned int k = 0; k < L; ++k) {
            if (k != 0) {
                const int b = __ffs((int)k) - 1;  // warp-uniform
                const longlong2* a = s_a2 + (rows - 1 - b) * NP + j0;
                if (b + 1 < p.seg_log2) {
                    // below the segment boundary bit the new delta depends on
                    // k alone: Gray bit b becomes 1 ^ (bit b + 1 of k)
                    const bool sub = !((k >> (b + 1)) & 1u);
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
                } else {
                    // k = L/2: the direction depends on the segment
                    const unsigned long long idx = i0 + k;
                    const long long m = -(long long)(((idx >> b) ^ (idx >> (b + 1))) & 1ull);
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c];
                        cre[c] += (v.x ^ m) - m;
                        cim[c] += (v.y ^ m) - m;
                    }
                }
                sbit ^= 0x8000000000000000ull;
                if ((k & 255u) == 0) {
                    acc.re = dd_add_d(acc.re, b0);
                    b0 = 0.0;
                    if (GROUP == 1) {
                        acc.im = dd_add_d(acc.im, b1);
                        b1 = 0.0;
                    }
                }
            }
            // partial product of this lane's columns in kChains chains; sig
            // tracks the product's shift count (shifts minus multiplies)
            fxl ch[kChains];
            int sig = 0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (c < kChains) {
                    sig += fx_norm_col(cre[c], cim[c], ch[c]);
                } else {
                    long long rr, ri;
                    fx_mul(ch[c % kChains], fx_col(cre[c], cim[c]), rr, ri);
                    sig += fx_norm(rr, ri, ch[c % kChains]) - 1;
                }
            }
            long long pr, pi;
            fx_mul(ch[0], ch[1], pr, pi);  // every shape has CPL >= 2
            sig -= 1;
            // butterfly over the lane group; fx_mul is symmetric in its
            // operands, so every lane of the group ends with the same product
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) {
                fxl x;
                sig += fx_norm(pr, pi, x);
                const fxl y = shfl_xor_fxl(x, m);
                sig += __shfl_xor_sync(0xffffffffu, sig, m) - 1;
                fx_mul(x, y, pr, pi);
            }
            if (active && (GROUP == 1 || g < 2)) {
                const int e = -61 - sig;
                const double t0 = fx_to_double(GROUP == 1 || g == 0 ? pr : pi, e);
                b0 += __longlong_as_double(__double_as_longlong(t0) ^ (long long)sbit);
                if (GROUP == 1) {
                    const double t1 = fx_to_double(pi, e);
                    b1 += __longlong_as_double(__double_as_longlong(t1) ^ (long long)sbit);
                }
            }
        }
        acc.re = dd_add_d(acc.re, b0);
        if (GROUP == 1) acc.im = dd_add_d(acc.im, b1);
    }
    if (GROUP > 1 && g == 1) {  // lane 1 summed the imaginary part
        acc.im = acc.re;
        acc.re = dd{0.0, 0.0};
    }

    // block reduction (double-double, fixed order), then the last block sums
    // the block partials with all its threads
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
            const volatile double* q = reinterpret_cast<const volatile double*>(&p.block_part[bk]);
            cdd v{{q[0], q[1]}, {q[2], q[3]}};
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
size_t fx_smem(int rows) {
    return 2ull * rows * CPL * GROUP * sizeof(longlong2);
}

template <int CPL, int GROUP>
cudaError_t launch_fx_t(const PlainArgs& a, int grid, cudaStream_t st) {
    cudaError_t e = allow_max_dynamic_smem((const void*)plain_fx_kernel<CPL, GROUP>);
    if (e != cudaSuccess) return e;
    plain_fx_kernel<CPL, GROUP><<<grid, kThreads, fx_smem<CPL, GROUP>(a.rows), st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int fx_bps_t(int rows) {
    int nb = 0;
    allow_max_dynamic_smem((const void*)plain_fx_kernel<CPL, GROUP>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, plain_fx_kernel<CPL, GROUP>, kThreads,
                                                  fx_smem<CPL, GROUP>(rows));
    return nb > 0 ? nb : 1;
}

// (CPL, GROUP) shapes compiled: one lane up to 8 columns, lane pairs up to
// 40, lane quads above (and from 22 columns on request); fx_shape() picks
// CPL = ceil(cols / GROUP), which leaves every lane at least one real column
#define GBPERM_FX_SHAPES(X)                                                                                   \
    X(8, 1) X(5, 2) X(6, 2) X(7, 2) X(8, 2) X(9, 2) X(10, 2) X(11, 2) X(12, 2) X(13, 2) X(14, 2) X(15, 2)    \
    X(16, 2) X(17, 2) X(18, 2) X(19, 2) X(20, 2) X(6, 4) X(7, 4) X(8, 4) X(9, 4) X(10, 4) X(11, 4) X(12, 4)  \
    X(13, 4) X(14, 4) X(15, 4) X(16, 4)

}  // namespace

void fx_shape(int cols, int group, int* cpl, int* grp) {
    if (cols <= 8) {
        *cpl = 8;
        *grp = 1;
    } else if (cols <= 40 && !(group == 4 && cols > 21)) {
        *grp = 2;
        *cpl = (cols + 1) / 2;
    } else {
        *grp = 4;
        *cpl = (cols + 3) / 4;
    }
}

int plain_fx_blocks_per_sm(int rows, int cpl, int grp) {
#define X(C, G) \
    if (cpl == C && grp == G) return fx_bps_t<C, G>(rows);
    GBPERM_FX_SHAPES(X)
#undef X
    return 1;
}

cudaError_t launch_plain_fx(const longlong2* a1, const longlong2* a2, const int* exp_in, const int* gate, int rows,
                            int cols, int cpl, int grp, int grid, int seg_log2, void* ws, double* out2,
                            double* out4, cudaStream_t st) {
    PlainArgs a;
    a.a1 = a1;
    a.a2 = a2;
    a.rows = rows;
    a.cols = cols;
    a.seg_log2 = seg_log2;
    a.nseg = 1ull << (rows - 1 - seg_log2);
    char* w = static_cast<char*>(ws);
    a.block_part = reinterpret_cast<cdd*>(w);
    a.done = reinterpret_cast<unsigned int*>(w + align_up((size_t)grid * sizeof(cdd), 256));
    a.exp_in = exp_in;
    a.df_info = gate;
    a.out2 = out2;
    a.out4 = out4;
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
#define X(C, G) \
    if (cpl == C && grp == G) return launch_fx_t<C, G>(a, grid, st);
    GBPERM_FX_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

}  // namespace gbperm
