// Repeated-row / repeated-column permanent (GB300).
//
// Replaces BBFGPermanentCalculatorRepeated_Tasks::calculate
// (piquassoboost/sampling/source/BBFGPermanentCalculatorRepeated.hpp:116-307)
// and the recursive GlynnPermanentCalculatorRepeated (GlynnPermanent
// CalculatorRepeated.hpp:48-258).  With row multiplicities r_i, column
// multiplicities c_j and one copy of one row kept at delta = +1:
//   perm = 2^-(sum r - 1) * sum_g (-1)^(sum g) prod_i C(D_i, g_i)
//          * prod_j (sum_i (r_i - 2 g_i) a_ij)^(c_j)
// where g_i in [0, D_i] counts the -1 deltas among the free copies of row i
// (D_i = r_i, and r_f - 1 for the row holding the fixed copy).  The g vector
// runs over the reflected mixed-radix Gray code (radices D_i + 1), so one
// step changes one g_i by +-1 and moves one row's coefficient by -+2.
//
// Work split: the digits are split into q low digits (changing inside a
// segment) and high digits (fixed per segment).  Segments are aligned blocks
// of P = prod_{i<q} (D_i + 1) steps, so the changed digit at local step k is
// the same for every segment (a shared-memory table, warp-uniform); only the
// direction is per lane, tracked Knuth-style (a digit reverses after it
// reaches an end).  The low-digit binomial weight is a table indexed by the
// low Gray digits; the high-digit weight is constant per segment.
// Column sums are exact 64-bit fixed point; product and accumulation as in
// the plain kernel.
#include "gbperm_internal.h"

namespace gbperm {

namespace {

constexpr int kThreads = 128;

// x^e by squaring (e >= 1).  Out of line: reached only for multiplicities
// above 1, and it keeps speculated multiplies off the common path.
__device__ __noinline__ cd cd_pow(cd x, int e) {
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

template <int NMAX>
__global__ void __launch_bounds__(kThreads) repeated_kernel(RepArgs p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    longlong2* s_a1 = reinterpret_cast<longlong2*>(smem_raw);            // R x NMAX
    longlong2* s_a2 = s_a1 + p.R * NMAX;                                 // nd x NMAX (digit rows)
    double* s_w = reinterpret_cast<double*>(s_a2 + p.nd * NMAX);         // P
    unsigned char* s_seq = reinterpret_cast<unsigned char*>(s_w + p.P);  // P
    __shared__ int s_cpow[NMAX];
    __shared__ int s_D[kMaxDigits], s_r[kMaxRows];
    __shared__ long long s_stride[kMaxDigits];
    const int R = p.R, C = p.C, nd = p.nd, q = p.q;
    // launched as the twin of the double-float kernel: run only when the
    // range check sent the product to FP64
    if (p.df_info && p.df_info[1] != 0) return;
    for (int e = threadIdx.x; e < R * NMAX; e += blockDim.x) {
        int r = e / NMAX, j = e % NMAX;
        s_a1[e] = j < C ? p.a1[r * C + j] : make_longlong2(0, 0);
    }
    for (int e = threadIdx.x; e < nd * NMAX; e += blockDim.x) {
        int r = e / NMAX, j = e % NMAX;
        s_a2[e] = j < C ? p.a2[r * C + j] : make_longlong2(0, 0);
    }
    for (long long e = threadIdx.x; e < (long long)p.P; e += blockDim.x) {
        s_w[e] = p.wlow[e];
        s_seq[e] = p.seq[e];
    }
    for (int e = threadIdx.x; e < NMAX; e += blockDim.x) s_cpow[e] = e < C ? p.cpow[e] : 0;
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

    cdd acc{{0.0, 0.0}, {0.0, 0.0}};
    const unsigned long long T = (unsigned long long)gridDim.x * blockDim.x;
    long long cre[NMAX], cim[NMAX];

    const unsigned long long full = p.nseg / 64ull * 64ull;  // parity blocks of two warps' segments
    for (unsigned long long u = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; u < p.nseg; u += T) {
        const unsigned long long h = parity_slot(u, 32ull, full);
        // --- decode the segment: high counter digits from h, Gray digits
        // from the top down (reflected when the digits above sum to odd);
        // low digits start at counter 0, i.e. at one end.
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
                int g = par ? s_D[i] - c : c;
                gdig[i] = g;
                par ^= g & 1;
            }
        }
        // --- segment-start column sums, sign, weights
#pragma unroll
        for (int j = 0; j < NMAX; ++j) {
            cre[j] = 0;
            cim[j] = 0;
        }
        int gsum = 0;
        double whigh = 1.0;
        unsigned long long G = 0ull;   // low Gray digits, 4 bits each
        unsigned int dir = 0u;         // bit i set: low digit i moves up next
        long long widx = 0;
        for (int i = 0; i < R; ++i) {
            int g = i < nd ? gdig[i] : 0;
            long long coef = (long long)(s_r[i] - 2 * g);
            const longlong2* a = s_a1 + i * NMAX;
#pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                longlong2 v = a[j];
                cre[j] += coef * v.x;
                cim[j] += coef * v.y;
            }
            if (i < nd) {
                gsum += g;
                if (i < q) {
                    G |= (unsigned long long)g << (4 * i);
                    if (g == 0) dir |= 1u << i;
                    widx += (long long)g * s_stride[i];
                } else {
                    whigh *= p.binom[s_D[i] * kBinomStride + g];
                }
            }
        }
        unsigned long long neg = (unsigned long long)(gsum & 1) << 63;

        double bre = 0.0, bim = 0.0;
        for (unsigned long long k = 0; k < p.P; ++k) {
            if (k != 0) {
                const int d = s_seq[k];  // warp-uniform
                const bool up = (dir >> d) & 1u;
                const int sh = 4 * d;
                int g = (int)((G >> sh) & 15ull);
                g += up ? 1 : -1;
                G = (G & ~(15ull << sh)) | ((unsigned long long)g << sh);
                if (g == 0 || g == s_D[d]) dir ^= 1u << d;
                widx += up ? s_stride[d] : -s_stride[d];
                // up: one more -1 delta -> subtract 2 a (warp-uniform: a
                // warp's segments share their parity)
                const longlong2* a = s_a2 + d * NMAX;
                if (up) {
#pragma unroll
                    for (int j = 0; j < NMAX; ++j) {
                        if (j < C) {
                            longlong2 v = a[j];
                            cre[j] -= v.x;
                            cim[j] -= v.y;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < NMAX; ++j) {
                        if (j < C) {
                            longlong2 v = a[j];
                            cre[j] += v.x;
                            cim[j] += v.y;
                        }
                    }
                }
                neg ^= 0x8000000000000000ull;
                if ((k & 255ull) == 0) {
                    acc.re = dd_add_d(acc.re, bre * whigh);
                    acc.im = dd_add_d(acc.im, bim * whigh);
                    bre = 0.0;
                    bim = 0.0;
                }
            }
            // prod_j colsum_j^(c_j); the sign goes into factor 0; powers above
            // 1 (rare) through an out-of-line helper, so the common path holds
            // exactly one complex multiply per column
            cd pr;
            {
                cd x0{fix_to_double(cre[0]), fix_to_double(cim[0])};
                const int e0 = s_cpow[0];
                if (e0 != 1) x0 = cd_pow(x0, e0);
                pr.re = __longlong_as_double(__double_as_longlong(x0.re) ^ (long long)neg);
                pr.im = __longlong_as_double(__double_as_longlong(x0.im) ^ (long long)neg);
            }
#pragma unroll
            for (int j = 1; j < NMAX; ++j) {
                if (j < C) {
                    cd x{fix_to_double(cre[j]), fix_to_double(cim[j])};
                    const int e = s_cpow[j];
                    if (e != 1) x = cd_pow(x, e);
                    pr = cmul(pr, x);
                }
            }
            const double w = s_w[widx];
            bre = fma(w, pr.re, bre);
            bim = fma(w, pr.im, bim);
        }
        acc.re = dd_add_d(acc.re, bre * whigh);
        acc.im = dd_add_d(acc.im, bim * whigh);
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
        // the last block sums the block partials: thread t takes partials
        // t, t + blockDim, ... in order, then a fixed butterfly and the warp
        // order -- deterministic, and not one thread's serial chain of L2
        // loads and dependent double-double adds
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

template <int NMAX>
size_t rep_smem(const RepArgs& a) {
    return (size_t)(a.R + a.nd) * NMAX * sizeof(longlong2) + (size_t)a.P * (sizeof(double) + 1) + 16;
}

template <int NMAX>
cudaError_t launch_rep_t(const RepArgs& a, int grid, cudaStream_t st) {
    size_t smem = rep_smem<NMAX>(a);
    cudaError_t e = allow_max_dynamic_smem((const void*)repeated_kernel<NMAX>);
    if (e != cudaSuccess) return e;
    repeated_kernel<NMAX><<<grid, kThreads, smem, st>>>(a);
    return cudaGetLastError();
}

template <int NMAX>
int rep_bps_t(const RepArgs& a) {
    int nb = 0;
    size_t smem = rep_smem<NMAX>(a);
    allow_max_dynamic_smem((const void*)repeated_kernel<NMAX>);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, repeated_kernel<NMAX>, kThreads, smem);
    return nb > 0 ? nb : 1;
}

}  // namespace

int repeated_blocks_per_sm(const RepArgs& a) {
    switch (plain_bucket(a.C)) {
        case 8: return rep_bps_t<8>(a);
        case 16: return rep_bps_t<16>(a);
        case 24: return rep_bps_t<24>(a);
        case 32: return rep_bps_t<32>(a);
        case 40: return rep_bps_t<40>(a);
        case 48: return rep_bps_t<48>(a);
        case 56: return rep_bps_t<56>(a);
        default: return rep_bps_t<64>(a);
    }
}

size_t repeated_workspace_bytes(int grid) {
    // block partials + completion counter + per-block |term|^2 sums (double-float kernel)
    return align_up((size_t)grid * sizeof(cdd), 256) + 256 + align_up((size_t)grid * sizeof(double), 256);
}

cudaError_t launch_repeated(RepArgs a, int grid, void* ws, cudaStream_t st) {
    char* w = static_cast<char*>(ws);
    a.block_part = reinterpret_cast<cdd*>(w);
    a.done = reinterpret_cast<unsigned int*>(w + align_up((size_t)grid * sizeof(cdd), 256));
    cudaError_t e = cudaMemsetAsync(a.done, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    switch (plain_bucket(a.C)) {
        case 8: return launch_rep_t<8>(a, grid, st);
        case 16: return launch_rep_t<16>(a, grid, st);
        case 24: return launch_rep_t<24>(a, grid, st);
        case 32: return launch_rep_t<32>(a, grid, st);
        case 40: return launch_rep_t<40>(a, grid, st);
        case 48: return launch_rep_t<48>(a, grid, st);
        case 56: return launch_rep_t<56>(a, grid, st);
        default: return launch_rep_t<64>(a, grid, st);
    }
}

}  // namespace gbperm
