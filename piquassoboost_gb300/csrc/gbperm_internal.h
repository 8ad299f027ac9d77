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
};

int plain_bucket(int cols);
int plain_blocks_per_sm(int rows, int cols);
void df_shape(int cols, int group, int* cpl, int* grp);
int plain_df_blocks_per_sm(int rows, int cpl, int grp);
cudaError_t launch_plain_df(const longlong2* a1, const longlong2* a2, const int* exp_in, const int* df_info,
                            int rows, int cols, int cpl, int grp, int grid, int seg_log2, void* ws,
                            double* out2, double* out4, cudaStream_t st);
size_t plain_workspace_bytes(int grid);
cudaError_t launch_plain(const longlong2* a1, const longlong2* a2, const int* exp_in,
                         const int* df_info, int rows, int cols, int grid, int seg_log2, void* ws,
                         double* out2, double* out4, cudaStream_t st);

// Range boost o for the double-float product (host): columns are first
// scaled to their L1 bound (< 1); o then centres the typical term
// (prod of column 2-norms) near 2^-40 while keeping the largest possible
// term (every |colsum| at its bound, times sqrt 2) below 2^118.  Returns
// false when no o satisfies both (then the FP64 kernel must be used).
bool df_boost(const double* A, int64_t rows, int64_t cols, int64_t ld, const int* row_w,
              const int* col_w, int* boost);
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
};
int repeated_blocks_per_sm(const RepArgs& a);
void repeated_df_shape(int cols, int* cpl, int* grp);
int repeated_df_blocks_per_sm(const RepArgs& a, int cpl, int grp);
cudaError_t launch_repeated_df(RepArgs a, int cpl, int grp, int grid, void* ws, cudaStream_t st);
size_t repeated_workspace_bytes(int grid);
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

}  // namespace gbperm
