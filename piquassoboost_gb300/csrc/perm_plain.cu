// Plain Glynn / BBFG permanent of one rows x cols complex matrix (GB300).
//
// Replaces BBFGPermanentCalculator_Tasks::calculate
// (piquassoboost/sampling/source/BBFGPermanentCalculator.hpp:87-235) and the
// recursive GlynnPermanentCalculator (GlynnPermanentCalculator.hpp:47-201):
//   perm = 2^-(rows-1) * sum_{delta in {+-1}^rows, delta_0 = +1}
//          (prod_i delta_i) * prod_j (sum_i delta_i a_ij)
// over the binary-reflected Gray code of rows 1..rows-1 (bit b of the Gray
// code <-> row rows-1-b, as in the reference).
//
// Work split: the 2^(rows-1) Gray indices are cut into aligned segments of
// L = 2^l steps.  Inside an aligned segment the changed row at local step k is
// rows-1-ctz(k) for every segment, so all lanes of a warp touch the same row
// at the same time (a shared-memory broadcast); only the add/subtract
// direction is per lane.  Up to 8 columns each thread walks segments t,
// t+T, t+2T, ... holding every column sum (plain_kernel); from 9 columns on
// a group of 2 or 4 lanes shares each segment, every lane holding an even
// share of the column sums (plain_group_kernel).
// Column sums are exact 64-bit fixed point (no drift); the product runs in
// FP64; terms are summed in double per 256 steps and folded into a
// double-double accumulator; the grid reduction is double-double and its
// order is fixed, so results are bitwise reproducible.
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;


template <int NMAX>
__global__ void __launch_bounds__(kThreads) plain_kernel(PlainArgs p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);
    longlong2* s_a2 = s_a1 + p.rows * NMAX;
    const int rows = p.rows, cols = p.cols;
    // launched as the twin of the double-float kernel: run only when the
    // prepare kernel's range check sent the product to FP64
    if (p.df_info && p.df_info[1] != 0) return;
    for (int e = threadIdx.x; e < rows * NMAX; e += blockDim.x) {
        int r = e / NMAX, j = e % NMAX;
        longlong2 z = make_longlong2(0, 0);
        s_a1[e] = j < cols ? p.a1[r * cols + j] : z;
        s_a2[e] = j < cols ? p.a2[r * cols + j] : z;
    }
    __syncthreads();

    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    const unsigned long long L = 1ull << p.seg_log2;
    const unsigned long long T = (unsigned long long)gridDim.x * blockDim.x;
    long long cre[NMAX], cim[NMAX];

    for (unsigned long long s = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; s < p.nseg;
         s += T) {
        const unsigned long long i0 = s << p.seg_log2;
        // exact segment-start sums: row 0 plus/minus rows 1..rows-1 by the Gray bits
        const unsigned long long g0 = i0 ^ (i0 >> 1);
#pragma unroll
        for (int j = 0; j < NMAX; ++j) {
            cre[j] = s_a1[j].x;
            cim[j] = s_a1[j].y;
        }
        for (int r = 1; r < rows; ++r) {
            const long long m = -(long long)((g0 >> (rows - 1 - r)) & 1ull);  // 0 (+) or -1 (-)
            const longlong2* a = s_a1 + r * NMAX;
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                longlong2 v = a[j];
                cre[j] += (v.x ^ m) - m;
                cim[j] += (v.y ^ m) - m;
            }
        }
        unsigned long long neg = (unsigned long long)(__popcll(g0) & 1) << 63;
        double bre = 0.0, bim = 0.0;
        for (unsigned long long k = 0; k < L; ++k) {
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;  // warp-uniform
                const unsigned long long idx = i0 + k;
                const bool sub = ((idx >> b) ^ (idx >> (b + 1))) & 1ull;
                const longlong2* a = s_a2 + (rows - 1 - b) * NMAX;
                if (sub) {
#pragma unroll
                    for (int j = 0; j < NMAX; ++j)
                        if (j < cols) {
                            longlong2 v = a[j];
                            cre[j] -= v.x;
                            cim[j] -= v.y;
                        }
                } else {
#pragma unroll
                    for (int j = 0; j < NMAX; ++j)
                        if (j < cols) {
                            longlong2 v = a[j];
                            cre[j] += v.x;
                            cim[j] += v.y;
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
            // product of the column sums, two interleaved chains for ILP;
            // the term sign goes into the first factor's sign bit (integer op)
            cd pa, pb;
            pa.re = __longlong_as_double(__double_as_longlong(fix_to_double(cre[0])) ^ (long long)neg);
            pa.im = __longlong_as_double(__double_as_longlong(fix_to_double(cim[0])) ^ (long long)neg);
            pb.re = 1.0;
            pb.im = 0.0;
            if (cols > 1) {
                pb.re = fix_to_double(cre[1]);
                pb.im = fix_to_double(cim[1]);
            }
#pragma unroll
            for (int j = 2; j < NMAX; j += 2) {
                if (j < cols) pa = cmul(pa, cd{fix_to_double(cre[j]), fix_to_double(cim[j])});
                if (j + 1 < cols) pb = cmul(pb, cd{fix_to_double(cre[j + 1]), fix_to_double(cim[j + 1])});
            }
            if (cols > 1) pa = cmul(pa, pb);
            bre += pa.re;
            bim += pa.im;
        }
        acc.re = dd_add_d(acc.re, bre);
        acc.im = dd_add_d(acc.im, bim);
    }

    // block reduction (double-double, fixed order)
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
        // the last block sums the block partials: thread t takes partials
        // t, t + blockDim, ... in order, then a fixed butterfly and the warp
        // order -- deterministic, and not one thread's serial chain of L2
        // loads and dependent double-double adds
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

// FP64 product with lane groups, for 9 or more columns.  GROUP consecutive
// lanes share one Gray segment; lane g owns an even share of the columns
// (columns [g c, g c + nr) with c = ceil(cols / GROUP)), forms their partial
// product in two chains, and a shuffle butterfly multiplies the GROUP
// partials.  plain_kernel<NMAX> keeps all NMAX column sums in one thread
// (255 registers and two warps per scheduler at n = 28, which leaves the
// FP64 pipe waiting on dependent multiplies); here a thread holds
// ceil(cols / GROUP) of them.  The butterfly adds one complex multiply per
// step and lane pair.  Same sum, Gray order, exact column sums and
// double-double accumulation as plain_kernel.
template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads, (CPL <= 16 ? 4 : 3)) plain_group_kernel(PlainArgs p) {
    constexpr int NP = CPL * GROUP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);
    longlong2* s_a2 = s_a1 + p.rows * NP;
    const int rows = p.rows, cols = p.cols;
    if (p.df_info && p.df_info[1] != 0) return;
    for (int e = threadIdx.x; e < rows * NP; e += blockDim.x) {
        int r = e / NP, j = e % NP;
        longlong2 z = make_longlong2(0, 0);
        s_a1[e] = j < cols ? p.a1[r * cols + j] : z;
        s_a2[e] = j < cols ? p.a2[r * cols + j] : z;
    }
    __syncthreads();

    const int g = threadIdx.x % GROUP;
    const int cpl_i = (cols + GROUP - 1) / GROUP;
    const int j0 = g * cpl_i;
    // real columns of this lane (>= 4: the host picks GROUP = 2 from 9
    // columns on and GROUP = 4 from 41)
    const int nr = cols - j0 < cpl_i ? cols - j0 : cpl_i;
    const bool leader = (g == 0);
    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    const unsigned long long L = 1ull << p.seg_log2;
    const unsigned long long T = ((unsigned long long)gridDim.x * blockDim.x) / GROUP;
    long long cre[CPL], cim[CPL];
    // warp-sized blocks of segments: every lane makes the same number of
    // trips (the butterfly shuffles need all 32 lanes); a group whose segment
    // is past the end computes on segment 0 and does not accumulate
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
        unsigned long long neg = (unsigned long long)(__popcll(g0) & 1) << 63;
        double bre = 0.0, bim = 0.0;
        for (unsigned long long k = 0; k < L; ++k) {
            if (k != 0) {
                const int b = __ffsll((long long)k) - 1;  // warp-uniform
                const longlong2* a = s_a2 + (rows - 1 - b) * NP + j0;
                if (b + 1 < p.seg_log2) {
                    // below the segment boundary bit the direction depends on k alone
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
                    const unsigned long long idx = i0 + k;
                    const long long m = -(long long)(((idx >> b) ^ (idx >> (b + 1))) & 1ull);
#pragma unroll
                    for (int c = 0; c < CPL; ++c) {
                        longlong2 v = a[c];
                        cre[c] += (v.x ^ m) - m;
                        cim[c] += (v.y ^ m) - m;
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
            // this lane's partial product in two interleaved chains
            cd pa{fix_to_double(cre[0]), fix_to_double(cim[0])};
            cd pb{fix_to_double(cre[1]), fix_to_double(cim[1])};
#pragma unroll
            for (int c = 2; c < CPL; c += 2) {
                if (c < nr) pa = cmul(pa, cd{fix_to_double(cre[c]), fix_to_double(cim[c])});
                if (c + 1 < nr) pb = cmul(pb, cd{fix_to_double(cre[c + 1]), fix_to_double(cim[c + 1])});
            }
            cd pr = cmul(pa, pb);
            // butterfly over the lane group: cmul is symmetric in its
            // operands, so every lane of the group ends with the same product
#pragma unroll
            for (int m = 1; m < GROUP; m <<= 1) {
                const cd y{__shfl_xor_sync(0xffffffffu, pr.re, m), __shfl_xor_sync(0xffffffffu, pr.im, m)};
                pr = cmul(pr, y);
            }
            if (leader && active) {
                bre += __longlong_as_double(__double_as_longlong(pr.re) ^ (long long)neg);
                bim += __longlong_as_double(__double_as_longlong(pr.im) ^ (long long)neg);
            }
        }
        acc.re = dd_add_d(acc.re, bre);
        acc.im = dd_add_d(acc.im, bim);
    }

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
size_t group_smem(int rows) {
    return 2ull * rows * CPL * GROUP * sizeof(longlong2);
}

template <int CPL, int GROUP>
cudaError_t launch_group_t(const PlainArgs& a, int grid, cudaStream_t st) {
    cudaError_t e = allow_max_dynamic_smem((const void*)plain_group_kernel<CPL, GROUP>);
    if (e != cudaSuccess) return e;
    plain_group_kernel<CPL, GROUP><<<grid, kThreads, group_smem<CPL, GROUP>(a.rows), st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int group_bps_t(int rows) {
    int nb = 0;
    allow_max_dynamic_smem((const void*)plain_group_kernel<CPL, GROUP>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, plain_group_kernel<CPL, GROUP>, kThreads,
                                                  group_smem<CPL, GROUP>(rows));
    return nb > 0 ? nb : 1;
}

// (CPL, GROUP) shapes of the lane-group kernel: pairs for 9..40 columns,
// quads for 41..64 (CPL = ceil(cols / GROUP))
#define GBPERM_FP64_GROUP_SHAPES(X)                                                                          \
    X(5, 2) X(6, 2) X(7, 2) X(8, 2) X(9, 2) X(10, 2) X(11, 2) X(12, 2) X(13, 2) X(14, 2) X(15, 2) X(16, 2) \
    X(17, 2) X(18, 2) X(19, 2) X(20, 2) X(11, 4) X(12, 4) X(13, 4) X(14, 4) X(15, 4) X(16, 4)

void group_shape(int cols, int* cpl, int* grp) {
    if (cols <= 8) {
        *cpl = 0;
        *grp = 1;
    } else if (cols <= 40) {
        *grp = 2;
        *cpl = (cols + 1) / 2;
    } else {
        *grp = 4;
        *cpl = (cols + 3) / 4;
    }
}

template <int NMAX>
cudaError_t launch_plain_t(const PlainArgs& a, int grid, cudaStream_t st) {
    size_t smem = 2ull * a.rows * NMAX * sizeof(longlong2);
    auto kern = plain_kernel<NMAX>;
    cudaError_t e = allow_max_dynamic_smem((const void*)kern);
    if (e != cudaSuccess) return e;
    kern<<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int NMAX>
int blocks_per_sm_t(int rows) {
    int nb = 0;
    size_t smem = 2ull * rows * NMAX * sizeof(longlong2);
    auto kern = plain_kernel<NMAX>;
    allow_max_dynamic_smem((const void*)kern);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kThreads, smem);
    return nb > 0 ? nb : 1;
}

}  // namespace

int plain_bucket(int cols) {
    if (cols <= 8) return 8;
    if (cols <= 16) return 16;
    if (cols <= 24) return 24;
    if (cols <= 32) return 32;
    if (cols <= 40) return 40;
    if (cols <= 48) return 48;
    if (cols <= 56) return 56;
    return 64;
}

int plain_group(int cols) {
    int cpl, grp;
    group_shape(cols, &cpl, &grp);
    return grp;
}

int plain_blocks_per_sm(int rows, int cols) {
    int cpl, grp;
    group_shape(cols, &cpl, &grp);
    if (grp > 1) {
#define X(C, G) \
    if (cpl == C && grp == G) return group_bps_t<C, G>(rows);
        GBPERM_FP64_GROUP_SHAPES(X)
#undef X
        return 1;
    }
    return blocks_per_sm_t<8>(rows);  // up to 8 columns: one thread holds every column sum
}

size_t plain_workspace_bytes(int grid) {
    // block partials + completion counter + per-block |term|^2 sums
    return align_up((size_t)grid * sizeof(cdd), 256) + 256 + align_up((size_t)grid * sizeof(double), 256);
}

// Launch the plain kernel on device data that is already in fixed point
// (launch_prepare).  ws must hold plain_workspace_bytes(grid).
cudaError_t launch_plain(const longlong2* a1, const longlong2* a2, const int* exp_in,
                         const int* df_info, int rows, int cols, int grid, int seg_log2, void* ws,
                         double* out2, double* out4, cudaStream_t st) {
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
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    int cpl, grp;
    group_shape(cols, &cpl, &grp);
    if (grp > 1) {
#define X(C, G) \
    if (cpl == C && grp == G) return launch_group_t<C, G>(a, grid, st);
        GBPERM_FP64_GROUP_SHAPES(X)
#undef X
        return cudaErrorInvalidValue;
    }
    return launch_plain_t<8>(a, grid, st);  // up to 8 columns
}

}  // namespace gbperm
