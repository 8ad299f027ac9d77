// Plain Glynn / BBFG permanent with the double-float product (GB300 FP32 pipe).
//
// Same sum, Gray order and exact int64 column sums as perm_plain.cu
// (BBFGPermanentCalculator.hpp:87-235).  On this chip the FP32 pipe issues
// ~70x more FMAs than the FP64 pipe, so the n-term complex product runs as
// unevaluated float pairs (~2^-46 relative error per complex multiply) and
// the column sums reach it through integer-only conversions.
//
// Lane groups: GROUP consecutive lanes share one Gray segment; lane g owns
// columns [g*CPL, (g+1)*CPL).  Each lane forms the partial product of its
// columns and a shuffle butterfly multiplies the GROUP partials, so a thread
// holds only CPL column sums (4 CPL registers) and the SM keeps more warps
// in flight to hide the float-pair dependency chains.  The changed row is
// still warp-uniform (aligned segments of equal length).
//
// Accuracy guard: the leaders also sum |term|^2, and the grid finish
// (df_grid_finish) turns it into an estimate of the result's relative
// rounding error; above 1e-10 it clears the range-check flag, so the
// integer-mantissa twin (perm_plain_fx.cu), launched next on the same
// stream, recomputes.
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;
#ifndef GBPERM_DF_CHAINS
#define GBPERM_DF_CHAINS 2
#endif
constexpr int kChains = GBPERM_DF_CHAINS;  // independent product chains per lane

__device__ __forceinline__ cf shfl_xor_cf(const cf& v, int m) {
    return cf{__shfl_xor_sync(0xffffffffu, v.rh, m), __shfl_xor_sync(0xffffffffu, v.rl, m),
              __shfl_xor_sync(0xffffffffu, v.ih, m), __shfl_xor_sync(0xffffffffu, v.il, m)};
}

template <int CPL, int GROUP>
// up to 18 columns per lane the kernel fits 128 registers (4 blocks per SM),
// above that 168 (3 blocks); the allocator is held to those, which it
// otherwise gives up for a few more live values
__global__ void __launch_bounds__(kThreads, (CPL <= 18 ? 4 : 3)) plain_df_kernel(PlainArgs p) {
    constexpr int NP = CPL * GROUP;  // padded columns
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);
    longlong2* s_a2 = s_a1 + p.rows * NP;
    const int rows = p.rows, cols = p.cols;
    if (p.df_info[1] == 0) {  // range check failed: the FP64 kernel runs instead
        if (blockIdx.x == 0 && threadIdx.x == 0 && p.err_out) *p.err_out = -1.0;
        return;
    }
    for (int e = threadIdx.x; e < rows * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        longlong2 z = make_longlong2(0, 0);
        s_a1[e] = j < cols ? p.a1[r * cols + j] : z;
        s_a2[e] = j < cols ? p.a2[r * cols + j] : z;
    }
    __syncthreads();

    const DfConv cv = make_dfconv(p.df_info[0]);
    const int g = threadIdx.x % GROUP;
    const int j0 = g * CPL;
    const bool leader = (g == 0);
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    // sum of |term 2^40|^2 (rounding-error estimate), per thread in shared
    // memory: a register pair more would cost the 18-column shape a block
    // per SM
    __shared__ double s_s2t[kThreads];
    s_s2t[threadIdx.x] = 0.0;
    const unsigned long long L = 1ull << p.seg_log2;
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / GROUP;
    long long cre[CPL], cim[CPL];
    // The loop runs over warp-sized blocks of segments so that every lane of
    // a warp makes the same number of trips (the product butterfly shuffles
    // need all 32 lanes); a group whose segment is past the end computes on
    // segment 0 and does not accumulate.
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
        unsigned int sbit = (unsigned int)(__popcll(g0) & 1) << 31;
        float brh = 0.f, brl = 0.f, bih = 0.f, bil = 0.f;
        float s2f = 0.f;  // sum of |term 2^40|^2 since the last fold
        for (unsigned long long k = 0; k < L; ++k) {
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;  // warp-uniform
                const longlong2* a = s_a2 + (rows - 1 - b) * NP + j0;
                if (b + 1 < p.seg_log2) {
                    // the new delta is Gray bit b of i0 + k; below the segment
                    // boundary bit it depends on k alone: a uniform branch
                    const bool sub = ((k >> b) ^ (k >> (b + 1))) & 1ull;
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
                    // k = L/2: the direction depends on the segment (once per segment)
                    const unsigned long long idx = i0 + k;
                    const long long m = -(long long)(((idx >> b) ^ (idx >> (b + 1))) & 1ull);
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c];
                        cre[c] += (v.x ^ m) - m;
                        cim[c] += (v.y ^ m) - m;
                    }
                }
                sbit ^= 0x80000000u;
                if ((k & 255ull) == 0) {
                    acc.re = dd_add(acc.re, dd{(double)brh, (double)brl});
                    acc.im = dd_add(acc.im, dd{(double)bih, (double)bil});
                    brh = brl = bih = bil = 0.f;
                    s_s2t[threadIdx.x] += (double)s2f;
                    s2f = 0.f;
                }
            }
            // partial product of this lane's columns in kChains independent
            // chains (ILP); padded columns hold zero sums and are skipped
            cf ch[kChains];
#pragma unroll
            for (int t = 0; t < kChains; ++t) ch[t] = cf{1.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (j0 + c < cols) {
                    cf x;
                    fix_to_df_magic(cre[c], cv, x.rh, x.rl);
                    fix_to_df_magic(cim[c], cv, x.ih, x.il);
                    if (c < kChains) ch[c] = x;
                    else ch[c % kChains] = cf_mul(ch[c % kChains], x);
                }
            }
#pragma unroll
            for (int w = 1; w < kChains; w <<= 1)
#pragma unroll
                for (int t = 0; t + w < kChains; t += 2 * w)
                    if (t + w < CPL) ch[t] = cf_mul(ch[t], ch[t + w]);
            cf pa = ch[0];
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) pa = cf_mul(pa, shfl_xor_cf(pa, m));
            if (leader && active) {
                df_acc(brh, brl, __uint_as_float(__float_as_uint(pa.rh) ^ sbit),
                       __uint_as_float(__float_as_uint(pa.rl) ^ sbit));
                df_acc(bih, bil, __uint_as_float(__float_as_uint(pa.ih) ^ sbit),
                       __uint_as_float(__float_as_uint(pa.il) ^ sbit));
                // terms sit near 2^-40 (the range boost centres them there)
                const float ur = pa.rh * 0x1p40f, ui = pa.ih * 0x1p40f;
                s2f = fmaf(ur, ur, fmaf(ui, ui, s2f));
            }
        }
        acc.re = dd_add(acc.re, dd{(double)brh, (double)brl});
        acc.im = dd_add(acc.im, dd{(double)bih, (double)bil});
        s_s2t[threadIdx.x] += (double)s2f;
    }

    df_grid_finish<kThreads>(acc, s_s2t[threadIdx.x], p.block_part, p.block_s2, p.done, p.exp_in, p.out2, p.out4, p.err_out,
                             p.df_ok, (double)cols);
}

template <int CPL, int GROUP>
size_t df_smem(int rows) {
    return 2ull * rows * CPL * GROUP * sizeof(longlong2);
}

template <int CPL, int GROUP>
cudaError_t launch_df_t(const PlainArgs& a, int grid, cudaStream_t st) {
    size_t smem = df_smem<CPL, GROUP>(a.rows);
    cudaError_t e = allow_max_dynamic_smem((const void*)plain_df_kernel<CPL, GROUP>);
    if (e != cudaSuccess) return e;
    plain_df_kernel<CPL, GROUP><<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int df_bps_t(int rows) {
    int nb = 0;
    size_t smem = df_smem<CPL, GROUP>(rows);
    allow_max_dynamic_smem((const void*)plain_df_kernel<CPL, GROUP>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, plain_df_kernel<CPL, GROUP>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

// (CPL, GROUP) shapes compiled; chosen by df_shape()
#define GBPERM_DF_SHAPES(X)                                                                                  \
    X(8, 1) X(4, 2) X(5, 2) X(6, 2) X(7, 2) X(8, 2) X(9, 2) X(10, 2) X(11, 2) X(12, 2) X(13, 2) X(14, 2) X(15, 2) \
    X(16, 2) X(17, 2) X(18, 2) X(19, 2) X(20, 2) X(22, 2) X(24, 2) X(6, 4) X(8, 4) X(9, 4) X(10, 4) X(12, 4)

}  // namespace

// Lane-group shape for a column count: GROUP lanes x CPL columns >= cols.
// `group` forces GROUP (1, 2, 4, 8) when > 0.
void df_shape(int cols, int group, int* cpl, int* grp) {
    static const int shapes[][2] = {{8, 1},  {4, 2},  {5, 2},  {6, 2},  {7, 2},  {8, 2},  {9, 2},
                                    {10, 2}, {11, 2}, {12, 2}, {13, 2}, {14, 2}, {15, 2}, {16, 2},
                                    {17, 2}, {18, 2}, {19, 2}, {20, 2}, {22, 2}, {24, 2}, {6, 4},
                                    {8, 4},  {9, 4},  {10, 4}, {12, 4}};
    // lane groups of 2 measured best on GB300 for 20 <= n <= 36 (fewest
    // instructions per term at 3-4 resident warps per scheduler)
    int want = group;
    if (want <= 0) want = cols <= 8 ? 1 : 2;
    int best = -1;
    for (int i = 0; i < (int)(sizeof(shapes) / sizeof(shapes[0])); ++i) {
        if (shapes[i][1] != want || shapes[i][0] * shapes[i][1] < cols) continue;
        if (best < 0 || shapes[i][0] < shapes[best][0]) best = i;
    }
    if (best < 0) {  // fall back to the widest shape that fits
        for (int i = 0; i < (int)(sizeof(shapes) / sizeof(shapes[0])); ++i)
            if (shapes[i][0] * shapes[i][1] >= cols &&
                (best < 0 || shapes[i][0] * shapes[i][1] < shapes[best][0] * shapes[best][1]))
                best = i;
    }
    *cpl = shapes[best][0];
    *grp = shapes[best][1];
}

int plain_df_blocks_per_sm(int rows, int cpl, int grp) {
#define X(C, G) \
    if (cpl == C && grp == G) return df_bps_t<C, G>(rows);
    GBPERM_DF_SHAPES(X)
#undef X
    return 1;
}

cudaError_t launch_plain_df(const longlong2* a1, const longlong2* a2, const int* exp_in, const int* df_info,
                            int rows, int cols, int cpl, int grp, int grid, int seg_log2, void* ws,
                            double* out2, double* out4, double* err_out, bool escalate, cudaStream_t st) {
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
    a.df_info = df_info;
    a.out2 = out2;
    a.out4 = out4;
    a.block_s2 = reinterpret_cast<double*>(w + align_up((size_t)grid * sizeof(cdd), 256) + 256);
    a.err_out = err_out;
    a.df_ok = escalate ? const_cast<int*>(df_info) + 1 : nullptr;
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
#define X(C, G) \
    if (cpl == C && grp == G) return launch_df_t<C, G>(a, grid, st);
    GBPERM_DF_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

}  // namespace gbperm
