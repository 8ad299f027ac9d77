// Host-side internals of the C ABI: options, per-thread context, plans.
#pragma once
#include <atomic>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "gbperm_internal.h"

namespace gbperm {

extern thread_local std::string t_err;
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

struct Options {
    std::atomic<int64_t> plain_seg_log2{-1};
    std::atomic<int64_t> plain_grid{0};
    std::atomic<int64_t> repeated_low_digits{-1};
    std::atomic<int64_t> batched_threads{0};
    std::atomic<int64_t> plain_df_group{0};
    std::atomic<int64_t> batched_item_log2{0};
    std::atomic<int64_t> df_escalate{1};
    std::atomic<int64_t> plain_fx_group{0};
    std::atomic<int64_t> grad_arith{1};
    // the double-float product is tried first only up to these sizes (plain:
    // rows of a square matrix; repeated and pmf: photons of the permanents);
    // above them its error estimate mostly exceeds 1e-10 (plain, repeated)
    // and the accurate product alone is faster than the double-float pass
    // plus its twin.  For the pmf layer the double-float kernel measured no
    // faster than the FP64 one up to 20 photons and escalated from 24 on, so
    // its rule defaults to 0: the fast mode runs the integer-mantissa layer
    std::atomic<int64_t> df_max_rows{36};
    std::atomic<int64_t> df_max_photons{24};
    std::atomic<int64_t> df_pmf_max_photons{0};
    std::atomic<int64_t>* find(const char* key) {
        if (!std::strcmp(key, "plain.seg_log2")) return &plain_seg_log2;
        if (!std::strcmp(key, "plain.grid")) return &plain_grid;
        if (!std::strcmp(key, "repeated.low_digits")) return &repeated_low_digits;
        if (!std::strcmp(key, "batched.threads")) return &batched_threads;
        if (!std::strcmp(key, "plain.df_group")) return &plain_df_group;
        if (!std::strcmp(key, "batched.item_log2")) return &batched_item_log2;
        if (!std::strcmp(key, "df.escalate")) return &df_escalate;
        if (!std::strcmp(key, "plain.fx_group")) return &plain_fx_group;
        if (!std::strcmp(key, "grad.arith")) return &grad_arith;
        if (!std::strcmp(key, "df.max_rows")) return &df_max_rows;
        if (!std::strcmp(key, "df.max_photons")) return &df_max_photons;
        if (!std::strcmp(key, "df.pmf_max_photons")) return &df_pmf_max_photons;
        return nullptr;
    }
};
extern Options g_opt;

int device_sms(int dev);
bool all_finite(const double* A, int64_t rows, int64_t cols, int64_t ld);
int ceil_log2_u64(unsigned long long x);

// Per-thread stream, timing events and a growable device buffer used by the
// host-pointer entry points.  Resources are kept until the process exits.
struct ThreadCtx {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void* dbuf = nullptr;
    size_t dcap = 0;
    int ensure(size_t bytes);
};
ThreadCtx& thread_ctx();

struct PlainPlan {
    int grid = 1;          // FP64 kernel
    int seg_log2 = 0;
    bool df = false;       // double-float kernel requested
    int grid_df = 1;
    int seg_log2_df = 0;
    int cpl = 8, grp = 1;  // double-float lane-group shape
    bool fx = false;       // integer-mantissa kernel: alone, or as the double-float kernel's twin
    int grid_fx = 1;
    int seg_log2_fx = 0;
    int cpl_fx = 8, grp_fx = 1;
    int max_grid() const {
        int g = grid;
        if (df && grid_df > g) g = grid_df;
        if (fx && grid_fx > g) g = grid_fx;
        return g;
    }
};
struct PlainWs {
    size_t a1 = 0, a2 = 0, exp = 0, scale = 0, kern = 0;
};
// arith: GBPERM_ARITH_*; the caller maps DF32 to FP64 beyond kDfMaxCols or
// when the host range check fails
PlainPlan plan_plain(int rows, int cols, int arith);
// The arithmetic a plain request runs: DF32 becomes FX64 beyond kDfMaxCols
// columns or above the df.max_rows size rule
int plain_arith(int64_t rows, int64_t cols, int arith);
size_t plain_ws_layout(int rows, int cols, int grid, PlainWs* w);
// d_err: optional device double that receives the double-float product's
// relative rounding-error estimate (0 when the FP64 product runs)
int run_plain_dev(const double2* dA, int64_t ld, int rows, int cols, void* ws, size_t ws_bytes,
                  double* d_out2, double* d_out4, cudaStream_t st, const PlainPlan& plan,
                  double* d_err = nullptr);
bool plain_trivial(int64_t rows, int64_t cols, double* out, double* out_dd);

// Repeated-multiplicity plan built on the host (host_repeated.cu).
struct RepHost {
    bool transpose = false;
    int R = 0, C = 0, nd = 0, q = 0, photons = 0;
    int norm_shift = 0;           // the sum is scaled by 2^-norm_shift
    unsigned long long P = 1, nseg = 1;
    double steps = 0.0, flops = 0.0;
    std::vector<double> M;        // R x C complex128 (interleaved), digit rows first
    std::vector<int> rcoef, D, cpow;
    std::vector<int> col_src;     // original column index of each column of M
    std::vector<double> wlow;
    std::vector<unsigned char> seq;
};
struct RepWs {
    size_t M = 0, a1 = 0, a2 = 0, ints = 0, wlow = 0, seq = 0, binom = 0, exp = 0, out = 0, kern = 0;
};
// col_surplus: photons the column side holds beyond the row side (1 for the
// leave-one-out sums of the pmf layer).  chinhuh: the Chin-Huh form of the
// same sum -- Gray digits over the input (column) side, no fixed copy, so the
// prefactor is 2^-N (CChinHuhPermanentCalculator.cpp:48-201).
int repeated_plan(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                  int64_t ncol, const int64_t* row_mult, int64_t nrow, RepHost* h, double* trivial,
                  bool* is_trivial, bool allow_transpose, int col_surplus, bool chinhuh = false);
// Reorder the product-side columns (M, cpow, col_src) for a kernel whose
// lane groups of `group` lanes hold `cpl` contiguous columns each: the
// columns sorted by power are dealt slot by slot across the lanes, so that
// slot c of every lane holds nearly the same power and the lanes' extra
// multiplies for powers above 1 line up.  A permutation of the columns
// leaves the repeated permanent unchanged.
void deal_columns_by_power(RepHost* h, int group, int cpl);
// Split the Gray range into segments of P = prod_{i<q} (D_i + 1) steps: the
// q low digits walk inside a segment from the tables wlow / seq, the high
// digits are decoded once per segment.  q minimises
//   ceil(nseg / slots(P)) * (P + seg_cost)
// over P <= 4096 -- the passes of the slowest segment slot times its steps
// plus the per-segment setup expressed in steps -- where slots(P) is the
// number of segments the launch runs at once for that table size.  Fills q,
// P, nseg, wlow and seq.
void repeated_low_digits(RepHost* h, const std::function<unsigned long long(unsigned long long)>& slots,
                         double seg_cost);
const std::vector<double>& binom_table();
size_t repeated_ws_layout(const RepHost& h, int grid, RepWs* w);

}  // namespace gbperm
