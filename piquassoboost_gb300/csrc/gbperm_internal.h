// Internal declarations shared by the kernel translation units and the C-ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "gbperm_common.cuh"

namespace gbperm {

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Lift a kernel's dynamic shared-memory limit to the device's opt-in maximum
// (less the kernel's static shared memory), once per kernel and device.  The
// attribute is process-wide: setting it to each launch's own size lets a
// second host thread lower it between another thread's set and launch.  The
// size passed at launch (and to the occupancy query) still decides
// occupancy.
cudaError_t allow_max_dynamic_smem(const void* kernel);

// ---------------------------------------------------------------- prepare
// Per-matrix fixed-point preparation (device).  For each column j with
// weight sum  B_j = max(sum_i w_i |Re a_ij|, sum_i w_i |Im a_ij|)  the column
// is scaled by 2^-e_j with e_j = floor(log2 B_j) + 1 (so scaled B_j < 1) and
// a_ij, 2 a_ij are written as int64 fixed point with unit 2^-62.
// exp_out[0] = sum_j cm_j e_j - (total multiplicity - 1): the caller's final
// sum is multiplied by 2^exp_out[0].
struct PrepArgs {
    const double2* A;        // rows x cols complex128, leading dimension ld (elements)
    long long ld;
    int rows, cols;
    const int* row_w;        // rows weights (nullptr -> 1)
    const int* col_w;        // column powers (nullptr -> 1)
    int norm_shift;          // subtract from the exponent: total row weight - 1
    longlong2* a1;           // rows x cols
    longlong2* a2;           // rows x cols
    int* exp_out;            // 1 int
    int* col_e_out;          // optional: per-column scaling exponents e_j (cols ints)
    int df;                  // 1: also decide the double-float range boost
    int* df_info;            // {o, ok}: boost and range-check result (ok = 0:
                             // the kernel must use the FP64 product)
    // batch of equal-shape matrices, one block each: matrix b starts at
    // A + b * a_stride and writes a1/a2 + b*rows*cols, exp_out + b,
    // col_e_out + b*cols, df_info + 2b
    int count = 1;
    long long a_stride = 0;
    // 1: scale row i by 2^-k_i first (k_i: binary exponent of its largest
    // component) and add sum_i w_i k_i to exp_out.  Exact, and it removes
    // the cancellation that unequal row norms cause in the Gray sum.  Valid
    // when the sum is multilinear in the (expanded) rows: square plain
    // matrices, the repeated and leave-one-out sums, and the gradient (whose
    // entry (k, l) then takes exponent exp - e_l - k_k: row_k_out); off for
    // rectangular matrices
    int row_balance = 0;
    // optional: the exponent without the double-float boost, for the FP64
    // twin when it takes over from a double-float kernel that ran
    int* exp_fp64_out = nullptr;
    // optional: the row scaling exponents k_i (rows ints per matrix), for
    // results that lose a row (the gradient's minors)
    int* row_k_out = nullptr;
};
cudaError_t launch_prepare(const PrepArgs& a, cudaStream_t st);

// ------------------------------------------------------------------ plain
struct PlainArgs {
    const longlong2* a1;   // rows x cols fixed-point a_ij (unit 2^-62 after column scaling)
    const longlong2* a2;   // rows x cols fixed-point 2 a_ij
    int rows, cols;
    int seg_log2;          // L = 2^seg_log2
    unsigned long long nseg;
    cdd* block_part;       // gridDim.x partial sums
    unsigned int* done;    // completion counter (zero before the launch)
    const int* exp_in;     // final scale exponent (from the prepare kernel)
    const int* df_info;    // {boost, ok} from the prepare kernel, or null (FP64 only)
    double* out2;          // complex128 result
    double* out4;          // optional: {re_hi, im_hi, re_lo, im_lo} of the scaled result
    // double-float kernel only: per-block sums of |term|^2 (terms scaled by
    // 2^40) and the relative rounding-error estimate of the result
    double* block_s2 = nullptr;
    double* err_out = nullptr;
    int* df_ok = nullptr;  // writable df_info[1]: cleared to hand the result to the twin
};

// A double-float result whose estimated relative rounding error exceeds this
// (the 1e-10 accuracy bar) is recomputed by the twin kernel (integer-mantissa
// for plain and repeated permanents and the gradient, FP64 for pmf layers
// and the plain batch plans).  The
// estimate sat above the measured error in every case checked (2-8x
// typically; Haar, rescaled, Gaussian and positive matrices, n = 16-36).
constexpr double kDfEscalate = 1e-10;

int plain_bucket(int cols);
int plain_blocks_per_sm(int rows, int cols);
// Lanes sharing one Gray segment in the FP64 plain kernel: 1 up to 8
// columns (one thread holds every column sum), 2 up to 40, 4 above
int plain_group(int cols);
void df_shape(int cols, int group, int* cpl, int* grp);
int plain_df_blocks_per_sm(int rows, int cpl, int grp);
cudaError_t launch_plain_df(const longlong2* a1, const longlong2* a2, const int* exp_in, const int* df_info,
                            int rows, int cols, int cpl, int grp, int grid, int seg_log2, void* ws,
                            double* out2, double* out4, double* err_out, bool escalate, cudaStream_t st);
size_t plain_workspace_bytes(int grid);
cudaError_t launch_plain(const longlong2* a1, const longlong2* a2, const int* exp_in,
                         const int* df_info, int rows, int cols, int grid, int seg_log2, void* ws,
                         double* out2, double* out4, cudaStream_t st);

// Integer-mantissa product (perm_plain_fx.cu): lane-group shape for a column
// count, occupancy and launch.  No range check.  gate: the double-float
// kernel's {boost, ok} flags when launched as its twin (the kernel returns at
// once while ok is set), else null.
// group: 0 = by column count (lane pairs up to 40 columns), 4 = lane quads
// from 22 columns on
void fx_shape(int cols, int group, int* cpl, int* grp);
int plain_fx_blocks_per_sm(int rows, int cpl, int grp);
cudaError_t launch_plain_fx(const longlong2* a1, const longlong2* a2, const int* exp_in, const int* gate, int rows,
                            int cols, int cpl, int grp, int grid, int seg_log2, void* ws, double* out2,
                            double* out4, cudaStream_t st);

// Range boost o for the double-float product (host): columns are first
// scaled to their L1 bound (< 1); o then centres the typical term
// (prod of column 2-norms) near 2^-40 while keeping the largest possible
// term (every |colsum| at its bound, times sqrt 2) below 2^118.  Returns
// false when no o satisfies both (then the FP64 kernel must be used).
// row_balance: the rows are scaled first as PrepArgs::row_balance does.
bool df_boost(const double* A, int64_t rows, int64_t cols, int64_t ld, const int* row_w,
              const int* col_w, int* boost, bool row_balance = true);
constexpr int kDfMaxCols = 48;

// --------------------------------------------------------------- repeated
constexpr int kMaxDigits = 64;
constexpr int kMaxRows = 64;
constexpr int kBinomStride = 65;  // binom[n * 65 + k] = C(n, k), n, k <= 64

struct RepArgs {
    const longlong2* a1;      // R x C fixed-point a_ij; rows 0..nd-1 are the Gray digits
    const longlong2* a2;      // nd x C fixed-point 2 a_ij
    int R, C, nd, q;          // rows, columns, digit rows, low digits
    const int* rcoef;         // R: base coefficient r_i (coefficient = r_i - 2 g_i)
    const int* D;             // nd: digit ranges (g_i in [0, D_i])
    const int* cpow;          // C: column powers c_j
    const double* wlow;       // P: prod_{i<q} C(D_i, g_i) by low Gray index
    const unsigned char* seq; // P: digit changed at local step k (entry 0 unused)
    const double* binom;      // 65 x 65 binomial table
    unsigned long long P;     // steps per segment
    unsigned long long nseg;  // segments
    cdd* block_part;
    unsigned int* done;
    const int* exp_in;
    const int* df_info;       // {boost, ok} or null (FP64 only)
    double* out2;
    double* out4;
    // double-float kernel only (as in PlainArgs)
    double* block_s2 = nullptr;
    double* err_out = nullptr;
    int* df_ok = nullptr;
};
int repeated_blocks_per_sm(const RepArgs& a);
void repeated_df_shape(int cols, int* cpl, int* grp);
int repeated_df_blocks_per_sm(const RepArgs& a, int cpl, int grp);
cudaError_t launch_repeated_df(RepArgs a, int cpl, int grp, int grid, void* ws, bool escalate, cudaStream_t st);
size_t repeated_workspace_bytes(int grid);
// integer-mantissa product (perm_repeated_fx.cu): no range check, no twin
void repeated_fx_shape(int cols, int* cpl, int* grp);
int repeated_fx_blocks_per_sm(const RepArgs& a, int cpl, int grp);
cudaError_t launch_repeated_fx(RepArgs a, int cpl, int grp, int grid, void* ws, cudaStream_t st);
cudaError_t launch_repeated(RepArgs a, int grid, void* ws, cudaStream_t st);

// Scale a double-double complex sum by 2^e and store it: out2 = {re, im}
// (rounded to double), out4 (optional) = {re_hi, im_hi, re_lo, im_lo}.
__device__ __forceinline__ void write_result(cdd v, int e, double* out2, double* out4) {
    double rh = ldexp(v.re.hi, e), rl = ldexp(v.re.lo, e);
    double ih = ldexp(v.im.hi, e), il = ldexp(v.im.lo, e);
    out2[0] = rh + rl;
    out2[1] = ih + il;
    if (out4) {
        out4[0] = rh;
        out4[1] = ih;
        out4[2] = rl;
        out4[3] = il;
    }
}

// End of a double-float Gray sweep, shared by the plain and repeated
// double-float kernels.  Every block publishes its threads' double-double
// sum and sum of |term 2^40|^2; the last block to arrive sums all blocks'
// with every thread (strided, then a fixed butterfly and the warp order, so
// the result is reproducible), writes the sum scaled by 2^exp_in and the
// estimate
//     sqrt(nfac) 2^-46 sqrt(sum |term|^2) / |sum|
// of its relative rounding error (each term carries ~2^-46 sqrt(nfac)
// relative error, independent between terms), and when that is above
// kDfEscalate (or not finite) clears *df_ok so that the twin launched next
// on the stream recomputes and overwrites the result.
template <int THREADS>
__device__ __forceinline__ void df_grid_finish(cdd acc, double s2, cdd* block_part, double* block_s2,
                                               unsigned int* done, const int* exp_in, double* out2, double* out4,
                                               double* err_out, int* df_ok, double nfac) {
    __shared__ cdd s_warp[THREADS / 32];
    __shared__ double s_wq[THREADS / 32];
    __shared__ bool s_last;
    acc = warp_sum_cdd(acc);
    s2 = warp_sum_d(s2);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_warp[warp] = acc;
        s_wq[warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        cdd b = s_warp[0];
        double q = s_wq[0];
        for (int w = 1; w < THREADS / 32; ++w) {
            b = cdd_add(b, s_warp[w]);
            q += s_wq[w];
        }
        block_part[blockIdx.x] = b;
        block_s2[blockIdx.x] = q;
        __threadfence();
        unsigned int t = atomicAdd(done, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;  // block-uniform
    __threadfence();
    cdd tot{{0.0, 0.0}, {0.0, 0.0}};
    double tq = 0.0;
    for (unsigned int bk = threadIdx.x; bk < gridDim.x; bk += blockDim.x) {
        const volatile double* qv = reinterpret_cast<const volatile double*>(&block_part[bk]);
        cdd v{{qv[0], qv[1]}, {qv[2], qv[3]}};
        tot = cdd_add(tot, v);
        tq += *reinterpret_cast<const volatile double*>(&block_s2[bk]);
    }
    tot = warp_sum_cdd(tot);
    tq = warp_sum_d(tq);
    if (lane == 0) {
        s_warp[warp] = tot;
        s_wq[warp] = tq;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        cdd all = s_warp[0];
        double q2 = s_wq[0];
        for (int w = 1; w < THREADS / 32; ++w) {
            all = cdd_add(all, s_warp[w]);
            q2 += s_wq[w];
        }
        write_result(all, *exp_in, out2, out4);
        const double est = sqrt(nfac) * 0x1p-46 * sqrt(q2) * 0x1p-40 / hypot(all.re.hi, all.im.hi);
        if (err_out) *err_out = est;
        if (df_ok && !(est <= kDfEscalate)) *df_ok = 0;
        *done = 0u;
    }
}

}  // namespace gbperm
