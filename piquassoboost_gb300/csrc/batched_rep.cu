// Many repeated-multiplicity permanents of one interferometer in one
// persistent launch, integer-mantissa product.
//
// Replaces BatchednPermanentCalculator::calculate
// (piquassoboost/sampling/source/BatchedPermanentCalculator.cpp:109-296): the
// reference takes one interferometer and a list of (input, output) state
// pairs and evaluates them one at a time, each through adaptInterferometer
// and the repeated (multiplicity) calculator (:118-143).  Here every pair is
// planned on the host as a repeated permanent (compaction of empty modes,
// the cheaper orientation, the fixed copy, the low digits walked inside a
// segment: host_repeated.cu), all instances' tables are packed into one
// device arena, and a persistent kernel walks them all.
//
// Work items: a warp takes one item from an atomic counter; an item holds
// up to SPI = 32 / GROUP segments of ONE instance, all of the same parity
// h & 1.  The parity of a segment's high digits fixes its whole low-digit
// walk (which digit moves, up or down), so every lane group of the warp
// moves the same row in the same direction at every step.  Items are dealt
// largest instance first (longest-processing-time order).  Each item's
// double-double sum lands in its own slot; a finalize kernel adds an
// instance's slots in a fixed order and applies the scale, so results are
// bitwise reproducible.
//
// Arithmetic: exact int64 column sums and the integer-mantissa product of
// gbperm_fx.cuh, with column powers, the low-digit binomial weight applied
// by one FP64 FMA per component and the high-digit weight per segment.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"
#include "gbperm_fx.cuh"

namespace gbperm {

namespace {

constexpr int kThreads = 128;

struct RInst {                 // device descriptor of one repeated instance
    int R, C, nd, q;           // rows (digit rows first), columns, digit rows, low digits
    unsigned long long P;      // steps per segment (low-digit table length)
    unsigned long long nseg;   // segments
    long long m_off;           // offset (complex elements) of the R x C matrix and its fixed-point tables
    int i_off;                 // offset of rcoef (R), D (nd), cpow (C) in the int arena
    long long t_off;           // offset of wlow (P doubles) and seq (P bytes) in the table arenas
    int norm_shift;            // the sum is scaled by 2^-norm_shift
    int item0, nitems;
};

struct RInstOut {              // written by the prepare kernel
    int exp;
    int finite;
};

struct RItem {
    int inst;
    int par;                   // segment parity of the item
    unsigned long long base;   // segments base + 2 grp + par, grp < SPI
};

struct RArgs {
    const double2* M;          // packed compact matrices
    longlong2* a1;             // fixed point a (same layout as M)
    longlong2* a2;             // fixed point 2 a
    const int* ints;
    const double* wlow;
    const unsigned char* seq;
    const double* binom;       // 65 x 65
    const RInst* inst;
    RInstOut* iout;
    const RItem* items;
    int nitems, ninst;
    unsigned int* counter;
    cdd* item_part;
    double* out;               // 2 doubles per device instance
};

// One block per instance (grid-stride): row balancing by powers of two,
// column bounds with the row coefficients as weights, int64 fixed point and
// the result exponent, as launch_prepare does for one repeated matrix.
__global__ void rep_prepare_kernel(RArgs p) {
    __shared__ int s_k[kMaxRows];
    __shared__ int s_e[GBPERM_MAX_DIM];
    __shared__ int s_bad;
    for (int i = blockIdx.x; i < p.ninst; i += gridDim.x) {
        const RInst in = p.inst[i];
        const double2* A = p.M + in.m_off;
        const int* w = p.ints + in.i_off;          // rcoef
        const int* cpow = w + in.R + in.nd;
        if (threadIdx.x == 0) s_bad = 0;
        __syncthreads();
        for (int r = threadIdx.x; r < in.R; r += blockDim.x) {
            double mx = 0.0;
            bool fin = true;
            for (int j = 0; j < in.C; ++j) {
                const double2 a = A[r * in.C + j];
                fin = fin && isfinite(a.x) && isfinite(a.y);
                mx = fmax(mx, fmax(fabs(a.x), fabs(a.y)));
            }
            int k = 0;
            if (mx > 0.0 && fin) frexp(mx, &k);
            s_k[r] = k;
            if (!fin) atomicOr(&s_bad, 1);
        }
        __syncthreads();
        for (int j = threadIdx.x; j < in.C; j += blockDim.x) {
            double br = 0.0, bi = 0.0;
            for (int r = 0; r < in.R; ++r) {
                const double2 a = A[r * in.C + j];
                br += (double)w[r] * fabs(ldexp(a.x, -s_k[r]));
                bi += (double)w[r] * fabs(ldexp(a.y, -s_k[r]));
            }
            const double b = fmax(br, bi) * (1.0 + 1e-12);
            int e = 0;
            if (b > 0.0 && isfinite(b)) frexp(b, &e);
            s_e[j] = e;
            for (int r = 0; r < in.R; ++r) {
                const double2 a = A[r * in.C + j];
                const bool ok = !s_bad;
                const long long xr = ok ? __double2ll_rn(ldexp(a.x, GBPERM_FIX_BITS - e - s_k[r])) : 0;
                const long long xi = ok ? __double2ll_rn(ldexp(a.y, GBPERM_FIX_BITS - e - s_k[r])) : 0;
                p.a1[in.m_off + r * in.C + j] = make_longlong2(xr, xi);
                p.a2[in.m_off + r * in.C + j] = make_longlong2(2 * xr, 2 * xi);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            long long tot = 0;
            for (int j = 0; j < in.C; ++j) tot += (long long)s_e[j] * cpow[j];
            for (int r = 0; r < in.R; ++r) tot += (long long)s_k[r] * w[r];
            p.iout[i].exp = (int)(tot - in.norm_shift);
            p.iout[i].finite = s_bad ? 0 : 1;
        }
        __syncthreads();
    }
}

template <int CPL, int GROUP>
__global__ void __launch_bounds__(kThreads) rep_batched_kernel(RArgs p) {
    __shared__ long long s_str[kThreads / 32][16];  // per warp: low-digit strides of its item's instance
    const int lane = threadIdx.x & 31;
    const int g = lane % GROUP;
    const int grp = lane / GROUP;
    long long cre[CPL], cim[CPL];
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(p.counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= p.nitems) break;
        const RItem item = p.items[it];
        const RInst in = p.inst[item.inst];
        const RInstOut io = p.iout[item.inst];
        const int R = in.R, C = in.C, nd = in.nd, q = in.q;
        const int* rcoef = p.ints + in.i_off;
        const int* Dg = rcoef + R;
        const int* cpow = Dg + nd;
        const longlong2* __restrict__ a1 = p.a1 + in.m_off;
        const longlong2* __restrict__ a2 = p.a2 + in.m_off;
        const double* __restrict__ wl = p.wlow + in.t_off;
        const unsigned char* __restrict__ sq = p.seq + in.t_off;
        // this lane's real columns: the instance's columns split evenly over
        // the group (a warp runs the longest lane's columns, so an even split
        // costs ceil(C / GROUP) column updates per step, not CPL); 0 for a
        // lane past the instance's columns
        const int cpl_i = (C + GROUP - 1) / GROUP;
        const int j0 = g * cpl_i;
        const int nr = max(0, min(cpl_i, C - j0));
        // bit c: this lane's column c has power > 1 (loaded once per item;
        // the step loop runs the common power-1 multiply unconditionally)
        unsigned int extra = 0u;
#pragma unroll
        for (int c = 0; c < CPL; ++c)
            if (c < nr && __ldg(&cpow[j0 + c]) > 1) extra |= 1u << c;
        const unsigned long long h_raw = item.base + 2ull * (unsigned long long)grp + (unsigned long long)item.par;
        const bool active = h_raw < in.nseg && io.finite;
        const unsigned long long h = h_raw < in.nseg ? h_raw : item.base + (unsigned long long)item.par;
        // --- decode the segment (as repeated_kernel): high counter digits
        // from h, Gray digits from the top down, low digits at one end
        int gdig[kMaxDigits];
        {
            unsigned long long rem = h;
            int cnt[kMaxDigits];
            for (int i = q; i < nd; ++i) {
                const unsigned long long Ld = (unsigned long long)(__ldg(&Dg[i]) + 1);
                cnt[i] = (int)(rem % Ld);
                rem /= Ld;
            }
            int par = 0;
            for (int i = nd - 1; i >= 0; --i) {
                const int c = i >= q ? cnt[i] : 0;
                const int gg = par ? __ldg(&Dg[i]) - c : c;
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
        long long widx = 0, stride = 1;
        long long* strides = s_str[threadIdx.x >> 5];
        __syncwarp();  // the previous item's strides are no longer read
        for (int i = 0; i < R; ++i) {
            const int gi = i < nd ? gdig[i] : 0;
            const long long coef = (long long)(__ldg(&rcoef[i]) - 2 * gi);
            const longlong2* a = a1 + i * C + j0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (c < nr) {
                    const longlong2 v = __ldg(&a[c]);
                    cre[c] += coef * v.x;
                    cim[c] += coef * v.y;
                }
            }
            if (i < nd) {
                gsum += gi;
                if (i < q) {
                    Gd |= (unsigned long long)gi << (4 * i);
                    if (gi == 0) dir |= 1u << i;
                    if (lane == 0) strides[i] = stride;
                    widx += (long long)gi * stride;
                    stride *= (long long)(__ldg(&Dg[i]) + 1);
                } else {
                    whigh *= __ldg(&p.binom[__ldg(&Dg[i]) * kBinomStride + gi]);
                }
            }
        }
        __syncwarp();  // strides written by lane 0 (the same for every lane: one instance per item)
        unsigned long long sbit = (unsigned long long)(gsum & 1) << 63;
        cdd acc{{0.0, 0.0}, {0.0, 0.0}};
        // every lane of a group ends the butterfly with the same product:
        // with GROUP >= 2 lane 0 converts and sums its real part in b0 and
        // lane 1 its imaginary part
        double b0 = 0.0, b1 = 0.0;
        const unsigned int P = (unsigned int)in.P;  // at most 4096 (low-digit table)
        for (unsigned int k = 0; k < P; ++k) {
            if (k != 0) {
                const int d = __ldg(&sq[k]);  // warp-uniform (one instance per item)
                const bool up = (dir >> d) & 1u;  // warp-uniform (one parity per item)
                const int sh = 4 * d;
                int gv = (int)((Gd >> sh) & 15ull);
                gv += up ? 1 : -1;
                Gd = (Gd & ~(15ull << sh)) | ((unsigned long long)gv << sh);
                if (gv == 0 || gv == __ldg(&Dg[d])) dir ^= 1u << d;
                widx += up ? strides[d] : -strides[d];
                const longlong2* a = a2 + d * C + j0;
                if (up) {
#pragma unroll
                    for (int c = 0; c < CPL; ++c)
                        if (c < nr) {
                            const longlong2 v = __ldg(&a[c]);
                            cre[c] -= v.x;
                            cim[c] -= v.y;
                        }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; ++c)
                        if (c < nr) {
                            const longlong2 v = __ldg(&a[c]);
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
            // this lane's partial product in two chains; a lane without
            // columns enters the butterfly with the value 1
            fxl ch[2];
            int sig = 0;
#pragma unroll
            for (int c = 0; c < CPL; ++c) {
                if (c < nr) {
                    // a column of power e multiplies its chain e times by the
                    // same column factor; powers above 1 are rare
                    const fxl y = fx_col(cre[c], cim[c]);
                    if (c < 2) {
                        sig += fx_norm_col(cre[c], cim[c], ch[c]);
                    } else {
                        long long rr, ri;
                        fx_mul(ch[c & 1], y, rr, ri);
                        sig += fx_norm(rr, ri, ch[c & 1]) - 1;
                    }
                    if ((extra >> c) & 1u) {
                        const int e = __ldg(&cpow[j0 + c]);
                        for (int t = 1; t < e; ++t) {
                            long long rr, ri;
                            fx_mul(ch[c & 1], y, rr, ri);
                            sig += fx_norm(rr, ri, ch[c & 1]) - 1;
                        }
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
            if (active && (GROUP == 1 || g < 2)) {
                const int ex = -61 - sig;
                const double w = __ldg(&wl[widx]);
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
        if (GROUP > 1 && g == 1) {  // lane 1 summed the imaginary part
            acc.im = acc.re;
            acc.re = dd{0.0, 0.0};
        }
        acc = warp_sum_cdd(acc);
        if (lane == 0) p.item_part[it] = acc;
    }
}

// warp per instance: lane l sums items l, l + 32, ... in order, then a fixed
// butterfly; scale by the instance's exponent
__global__ void rep_finalize_kernel(RArgs p) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < p.ninst; i += nw) {
        const RInst in = p.inst[i];
        const RInstOut io = p.iout[i];
        if (!io.finite) {
            if (lane == 0) p.out[2 * i] = p.out[2 * i + 1] = nan("");
            continue;
        }
        cdd tot{{0.0, 0.0}, {0.0, 0.0}};
        for (int k = lane; k < in.nitems; k += 32) tot = cdd_add(tot, p.item_part[in.item0 + k]);
        tot = warp_sum_cdd(tot);
        if (lane == 0) write_result(tot, io.exp, p.out + 2 * i, nullptr);
    }
}

template <int CPL, int GROUP>
cudaError_t launch_rep_batched_t(const RArgs& a, int grid, cudaStream_t st) {
    rep_batched_kernel<CPL, GROUP><<<grid, kThreads, 0, st>>>(a);
    return cudaGetLastError();
}

template <int CPL, int GROUP>
int rep_batched_bps_t() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, rep_batched_kernel<CPL, GROUP>, kThreads, 0);
    return nb > 0 ? nb : 1;
}

// (CPL, GROUP): one lane up to 8 columns, lane pairs up to 40
#define GBPERM_REP_BATCH_SHAPES(X) \
    X(8, 1) X(6, 2) X(8, 2) X(10, 2) X(12, 2) X(14, 2) X(16, 2) X(18, 2) X(20, 2)

void rep_batch_shape(int cmax, int* cpl, int* grp) {
    if (cmax <= 8) {
        *cpl = 8;
        *grp = 1;
        return;
    }
    *grp = 2;
    const int half = (cmax + 1) / 2;
    *cpl = half <= 6 ? 6 : (half + 1) / 2 * 2;
}

int rep_batched_bps(int cpl, int grp) {
#define X(C, G) \
    if (cpl == C && grp == G) return rep_batched_bps_t<C, G>();
    GBPERM_REP_BATCH_SHAPES(X)
#undef X
    return 1;
}

cudaError_t launch_rep_batched(const RArgs& a, int cpl, int grp, int grid, cudaStream_t st) {
#define X(C, G) \
    if (cpl == C && grp == G) return launch_rep_batched_t<C, G>(a, grid, st);
    GBPERM_REP_BATCH_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
}

// Largest column count the persistent repeated batch takes (lane pairs).
constexpr int kRepBatchMaxCols = 40;

// slot i of the caller's order takes device instance dev_index[i], or the
// host-decided value trivial[i] (1: no photons) when it never reached the
// device
__global__ void rep_scatter_kernel(const double* dout, const int* dev_index, const double* trivial,
                                   long long count, double* out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
         i += (long long)gridDim.x * blockDim.x) {
        const int d = dev_index[i];
        out[2 * i] = d >= 0 ? dout[2 * d] : trivial[2 * i];
        out[2 * i + 1] = d >= 0 ? dout[2 * d + 1] : trivial[2 * i + 1];
    }
}

}  // namespace

}  // namespace gbperm

using namespace gbperm;

struct gbperm_rep_batch {
    int device = -1;
    cudaStream_t stream = nullptr;
    long long count = 0;        // state pairs
    int ninst = 0, nitems = 0;  // device instances and work items
    int cpl = 8, grp = 1, grid = 1;
    double steps = 0.0, flops = 0.0, mul_ops = 0.0;
    void* dbuf = nullptr;
    RArgs args{};
    int* d_index = nullptr;
    double* d_trivial = nullptr;
    double* d_slots = nullptr;  // 2 count doubles in the caller's order
    double* h_slots = nullptr;  // pinned copy of d_slots
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

// counter reset, prepare, persistent worker, finalize and the slot-order
// scatter, on one stream
cudaError_t rep_batch_enqueue(gbperm_rep_batch* p, double* slots, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(p->args.counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    if (p->ninst > 0) {
        rep_prepare_kernel<<<std::min(p->ninst, 4096), 64, 0, st>>>(p->args);
        e = launch_rep_batched(p->args, p->cpl, p->grp, p->grid, st);
        if (e != cudaSuccess) return e;
        rep_finalize_kernel<<<std::max(1, std::min((p->ninst + 3) / 4, 4096)), 128, 0, st>>>(p->args);
    }
    const long long c = p->count;
    rep_scatter_kernel<<<(int)std::min<long long>((c + 255) / 256, 4096), 256, 0, st>>>(p->args.out, p->d_index,
                                                                                          p->d_trivial, c, slots);
    return cudaGetLastError();
}

}  // namespace

extern "C" {

int gbperm_rep_batch_create(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mults,
                            int64_t ncol, const int64_t* row_mults, int64_t nrow, int64_t count, int arith,
                            gbperm_rep_batch** out) {
    if (!out) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_create: null output");
    *out = nullptr;
    if (arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_create: the persistent repeated batch runs GBPERM_ARITH_FX64");
    if (count < 0 || rows < 0 || cols < 0 || nrow < 0 || ncol < 0)
        return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_create: negative size");
    if ((ncol > 0 && !col_mults) || (nrow > 0 && !row_mults))
        return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_create: null states");
    int rc = thread_ctx().ensure(0);  // a device must be visible
    if (rc) return rc;
    // plan every pair on the host (the reference's adaptInterferometer and
    // repeated calculator set-up, host_repeated.cu)
    std::vector<RepHost> hs;
    std::vector<int> dev_index((size_t)count, -1);
    std::vector<double> trivial(2 * (size_t)count, 0.0);
    int cmax = 1;
    for (int64_t i = 0; i < count; ++i) {
        RepHost h;
        double tv[2];
        bool is_triv = false;
        rc = repeated_plan(A, rows, cols, ld, col_mults + i * ncol, ncol, row_mults + i * nrow, nrow, &h, tv, &is_triv,
                           true, 0);
        if (rc) return rc;
        if (is_triv) {
            trivial[2 * i] = tv[0];
            trivial[2 * i + 1] = tv[1];
            continue;
        }
        if (h.C > kRepBatchMaxCols)
            return fail(GBPERM_ERR_TOO_LARGE, "gbperm_rep_batch_create: an instance has more than 40 occupied "
                                              "modes on its product side");
        dev_index[i] = (int)hs.size();
        cmax = std::max(cmax, h.C);
        hs.push_back(std::move(h));
    }
    gbperm_rep_batch* p = new gbperm_rep_batch();
    p->count = count;
    p->ninst = (int)hs.size();
    rep_batch_shape(cmax, &p->cpl, &p->grp);
    const int spi = 32 / p->grp;
    // segment length per instance: one item's SPI lane groups share it
    for (RepHost& h : hs) {
        deal_columns_by_power(&h, p->grp, (h.C + p->grp - 1) / p->grp);
        repeated_low_digits(&h, [spi](unsigned long long) { return (unsigned long long)spi; }, 8.0);
        p->steps += h.steps;
        p->flops += h.flops;
        p->mul_ops += 12.0 * (double)(h.photons - 1) * h.steps;
    }
    // instances by cost, largest first; an instance's items are contiguous
    std::vector<int> order(hs.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return hs[a].steps * hs[a].C > hs[b].steps * hs[b].C;
    });
    std::vector<RInst> insts(hs.size());
    std::vector<RItem> items;
    long long m_off = 0, t_off = 0;
    int i_off = 0;
    for (size_t k = 0; k < hs.size(); ++k) {
        const RepHost& h = hs[k];
        RInst& in = insts[k];
        in.R = h.R;
        in.C = h.C;
        in.nd = h.nd;
        in.q = h.q;
        in.P = h.P;
        in.nseg = h.nseg;
        in.m_off = m_off;
        in.i_off = i_off;
        in.t_off = t_off;
        in.norm_shift = h.norm_shift;
        m_off += (long long)h.R * h.C;
        i_off += h.R + h.nd + h.C;
        t_off += (long long)h.P;
    }
    for (int k : order) {
        RInst& in = insts[k];
        in.item0 = (int)items.size();
        const unsigned long long blk = 2ull * (unsigned long long)spi;
        for (unsigned long long b = 0; b * blk < in.nseg; ++b)
            for (int par = 0; par < 2; ++par)
                if (b * blk + (unsigned long long)par < in.nseg) items.push_back(RItem{k, par, b * blk});
        in.nitems = (int)items.size() - in.item0;
        if (items.size() > (size_t)INT32_MAX / 2) {
            delete p;
            return fail(GBPERM_ERR_TOO_LARGE, "gbperm_rep_batch_create: too many work items");
        }
    }
    p->nitems = (int)items.size();
    // host images of the arenas
    std::vector<double> M(2 * (size_t)m_off);
    std::vector<int> ints((size_t)i_off);
    std::vector<double> wlow((size_t)t_off);
    std::vector<unsigned char> seq((size_t)t_off);
    for (size_t k = 0; k < hs.size(); ++k) {
        const RepHost& h = hs[k];
        const RInst& in = insts[k];
        std::memcpy(&M[2 * (size_t)in.m_off], h.M.data(), h.M.size() * sizeof(double));
        int* ip = &ints[(size_t)in.i_off];
        std::copy(h.rcoef.begin(), h.rcoef.end(), ip);
        std::copy(h.D.begin(), h.D.end(), ip + h.R);
        std::copy(h.cpow.begin(), h.cpow.end(), ip + h.R + h.nd);
        std::memcpy(&wlow[(size_t)in.t_off], h.wlow.data(), h.wlow.size() * sizeof(double));
        std::memcpy(&seq[(size_t)in.t_off], h.seq.data(), h.seq.size());
    }
    const std::vector<double>& bt = binom_table();
    // device arena
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes > 0 ? bytes : 1, 256);
        return o;
    };
    const size_t oM = take(M.size() * sizeof(double)), oA1 = take((size_t)m_off * sizeof(longlong2)),
                 oA2 = take((size_t)m_off * sizeof(longlong2)), oI = take(ints.size() * sizeof(int)),
                 oW = take(wlow.size() * sizeof(double)), oS = take(seq.size()),
                 oB = take(bt.size() * sizeof(double)), oIn = take(insts.size() * sizeof(RInst)),
                 oIo = take(insts.size() * sizeof(RInstOut)), oIt = take(items.size() * sizeof(RItem)),
                 oC = take(sizeof(unsigned int)), oP = take(items.size() * sizeof(cdd)),
                 oO = take(2 * insts.size() * sizeof(double)), oX = take((size_t)count * sizeof(int)),
                 oT = take(2 * (size_t)count * sizeof(double)), oSl = take(2 * (size_t)count * sizeof(double));
    cudaError_t e = cudaGetDevice(&p->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&p->dbuf, off);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->h_slots, std::max<size_t>(16, 2 * (size_t)count * sizeof(double)));
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&p->ev1);
    if (e != cudaSuccess) {
        gbperm_rep_batch_destroy(p);
        return cuda_fail(e, "gbperm_rep_batch_create: allocation");
    }
    char* b = static_cast<char*>(p->dbuf);
    RArgs& a = p->args;
    a.M = reinterpret_cast<const double2*>(b + oM);
    a.a1 = reinterpret_cast<longlong2*>(b + oA1);
    a.a2 = reinterpret_cast<longlong2*>(b + oA2);
    a.ints = reinterpret_cast<const int*>(b + oI);
    a.wlow = reinterpret_cast<const double*>(b + oW);
    a.seq = reinterpret_cast<const unsigned char*>(b + oS);
    a.binom = reinterpret_cast<const double*>(b + oB);
    a.inst = reinterpret_cast<const RInst*>(b + oIn);
    a.iout = reinterpret_cast<RInstOut*>(b + oIo);
    a.items = reinterpret_cast<const RItem*>(b + oIt);
    a.nitems = p->nitems;
    a.ninst = p->ninst;
    a.counter = reinterpret_cast<unsigned int*>(b + oC);
    a.item_part = reinterpret_cast<cdd*>(b + oP);
    a.out = reinterpret_cast<double*>(b + oO);
    p->d_index = reinterpret_cast<int*>(b + oX);
    p->d_trivial = reinterpret_cast<double*>(b + oT);
    p->d_slots = reinterpret_cast<double*>(b + oSl);
    struct Up {
        size_t o;
        const void* src;
        size_t n;
    } ups[] = {{oM, M.data(), M.size() * sizeof(double)},
               {oI, ints.data(), ints.size() * sizeof(int)},
               {oW, wlow.data(), wlow.size() * sizeof(double)},
               {oS, seq.data(), seq.size()},
               {oB, bt.data(), bt.size() * sizeof(double)},
               {oIn, insts.data(), insts.size() * sizeof(RInst)},
               {oIt, items.data(), items.size() * sizeof(RItem)},
               {oX, dev_index.data(), dev_index.size() * sizeof(int)},
               {oT, trivial.data(), trivial.size() * sizeof(double)}};
    for (const Up& u : ups)
        if (u.n > 0 && e == cudaSuccess) e = cudaMemcpyAsync(b + u.o, u.src, u.n, cudaMemcpyHostToDevice, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) {
        gbperm_rep_batch_destroy(p);
        return cuda_fail(e, "gbperm_rep_batch_create: upload");
    }
    const int sms = device_sms(p->device);
    p->grid = sms * rep_batched_bps(p->cpl, p->grp);
    // the host run as one CUDA graph: the enqueue above plus the copy back
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = rep_batch_enqueue(p, p->d_slots, p->stream);
        if (e2 == cudaSuccess && count > 0)
            e2 = cudaMemcpyAsync(p->h_slots, p->d_slots, 2 * (size_t)count * sizeof(double), cudaMemcpyDeviceToHost,
                                 p->stream);
        e = cudaStreamEndCapture(p->stream, &graph);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        gbperm_rep_batch_destroy(p);
        return cuda_fail(e, "gbperm_rep_batch_create: graph");
    }
    *out = p;
    return GBPERM_OK;
}

int gbperm_rep_batch_run(gbperm_rep_batch* p, double* out, gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (!p) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_run: null plan");
    if (p->count > 0 && !out) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_run: null output");
    cudaError_t e = cudaSetDevice(p->device);
    if (e == cudaSuccess) e = cudaEventRecord(p->ev0, p->stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(p->exec, p->stream);
    if (e == cudaSuccess) e = cudaEventRecord(p->ev1, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_rep_batch_run");
    if (p->count > 0) std::memcpy(out, p->h_slots, 2 * (size_t)p->count * sizeof(double));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        stats->kernel_ms = ms;
        stats->steps = p->steps;
        stats->flops = p->flops;
        stats->launches = p->ninst > 0 ? 4 : 1;
        stats->grid = p->grid;
        stats->arith = GBPERM_ARITH_FX64;
    }
    return GBPERM_OK;
}

int gbperm_rep_batch_run_dev(gbperm_rep_batch* p, void* d_out, void* stream) {
    if (!p) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_run_dev: null plan");
    if (p->count > 0 && !d_out) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_run_dev: null output");
    cudaError_t e = rep_batch_enqueue(p, static_cast<double*>(d_out), static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? GBPERM_OK : cuda_fail(e, "gbperm_rep_batch_run_dev");
}

int gbperm_rep_batch_info(const gbperm_rep_batch* p, double* steps, double* flops, double* mul_ops,
                          int64_t* items) {
    if (!p) return fail(GBPERM_ERR_ARG, "gbperm_rep_batch_info: null plan");
    if (steps) *steps = p->steps;
    if (flops) *flops = p->flops;
    if (mul_ops) *mul_ops = p->mul_ops;
    if (items) *items = p->nitems;
    return GBPERM_OK;
}

void gbperm_rep_batch_destroy(gbperm_rep_batch* p) {
    if (!p) return;
    if (p->device >= 0) cudaSetDevice(p->device);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->h_slots) cudaFreeHost(p->h_slots);
    if (p->dbuf) cudaFree(p->dbuf);
    if (p->stream) cudaStreamDestroy(p->stream);
    cudaGetLastError();
    delete p;
}

}  // extern "C"
