// Host side of the repeated-multiplicity permanent: validation with the
// reference's semantics, compaction, orientation, digit plan and launch.
//
// Reference semantics (BBFGPermanentCalculatorRepeated.cpp:75-141, .hpp
// :74-141; ChinHuhPermanentCalculator_Wrapper.hpp:367-375):
//   * col_mult is the input state, row_mult the output state;
//   * rows == 0 -> 1; sum(col_mult) != sum(row_mult) -> error;
//     sum == 0 -> 1;
//   * only the first len(row_mult) rows / len(col_mult) columns are used.
// Rows and columns of zero multiplicity do not change the value and are
// dropped; the permanent is invariant under transposition (with the roles of
// the multiplicities swapped), so the orientation with the shorter Gray code
// is used.  The fixed delta = +1 copy goes to the row of smallest
// multiplicity, as in the reference (which prepends that row, .hpp:78-94).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

const std::vector<double>& binom_table() {
    static std::vector<double> t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.assign(kBinomStride * kBinomStride, 0.0);
        unsigned long long C[kBinomStride][kBinomStride];  // exact: C(64, 32) < 2^64
        std::memset(C, 0, sizeof(C));
        for (int n = 0; n < kBinomStride; ++n) {
            C[n][0] = 1;
            for (int k = 1; k <= n; ++k) C[n][k] = C[n - 1][k - 1] + (k <= n - 1 ? C[n - 1][k] : 0);
        }
        for (int n = 0; n < kBinomStride; ++n)
            for (int k = 0; k <= n; ++k) t[n * kBinomStride + k] = (double)C[n][k];
    });
    return t;
}

int repeated_plan(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                  int64_t ncol, const int64_t* row_mult, int64_t nrow, RepHost* h, double* trivial,
                  bool* is_trivial, bool allow_transpose, int col_surplus, bool chinhuh) {
    *is_trivial = false;
    if (rows == 0) {
        trivial[0] = 1.0;
        trivial[1] = 0.0;
        *is_trivial = true;
        return GBPERM_OK;
    }
    if (nrow > rows) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: output state longer than the matrix rows");
    if (ncol > cols) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: input state longer than the matrix columns");
    if (nrow > 0 && !row_mult) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: null output state");
    if (ncol > 0 && !col_mult) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: null input state");
    int64_t sr = 0, sc = 0;
    for (int64_t i = 0; i < nrow; ++i) {
        if (row_mult[i] < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: negative occupation");
        sr += row_mult[i];
    }
    for (int64_t j = 0; j < ncol; ++j) {
        if (col_mult[j] < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: negative occupation");
        sc += col_mult[j];
    }
    if (sr + col_surplus != sc)
        return fail(GBPERM_ERR_STATE_SUM,
                    "BBFGPermanentCalculatorRepeated_Tasks::calculate:  Number of input and output states should be equal");
    if (sr == 0 || cols == 0) {
        trivial[0] = 1.0;
        trivial[1] = 0.0;
        *is_trivial = true;
        return GBPERM_OK;
    }
    if (sr > 64) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_repeated: more than 64 photons");
    if (!A) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: null matrix");
    if (ld < cols) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: ld < cols");

    std::vector<int> ri, ci;  // occupied row / column indices
    for (int64_t i = 0; i < nrow; ++i)
        if (row_mult[i] > 0) ri.push_back((int)i);
    for (int64_t j = 0; j < ncol; ++j)
        if (col_mult[j] > 0) ci.push_back((int)j);
    if (ri.size() > (size_t)kMaxRows || ci.size() > (size_t)GBPERM_MAX_DIM)
        return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_repeated: more than 64 occupied modes");

    // log2 of the Gray length of one orientation: prod (D_i + 1) with the
    // fixed copy on the smallest multiplicity
    auto gray_len = [](const std::vector<int>& idx, const int64_t* mult) {
        int64_t mn = INT64_MAX;
        for (int i : idx) mn = std::min(mn, mult[i]);
        double t = 0.0;
        for (int i : idx) t += std::log2((double)(mult[i] + 1));
        return t + std::log2((double)mn / (double)(mn + 1));
    };
    const double t_rows = gray_len(ri, row_mult), t_cols = gray_len(ci, col_mult);
    bool transpose = chinhuh || (allow_transpose && t_cols < t_rows);
    h->transpose = transpose;
    const std::vector<int>& gi = transpose ? ci : ri;   // Gray-code side (rows of M)
    const std::vector<int>& pj = transpose ? ri : ci;   // product side (columns of M)
    const int64_t* gm = transpose ? col_mult : row_mult;
    const int64_t* pm = transpose ? row_mult : col_mult;
    int R = (int)gi.size(), C = (int)pj.size();
    if (C > GBPERM_MAX_DIM) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_repeated: more than 64 occupied modes");

    // fixed copy: first occurrence of the smallest multiplicity (none in the
    // Chin-Huh form)
    int fixed = 0;
    for (int i = 1; i < R; ++i)
        if (gm[gi[i]] < gm[gi[fixed]]) fixed = i;
    if (chinhuh) fixed = -1;

    struct RowInfo {
        int src;   // index into gi
        int r;     // multiplicity
        int D;     // digit range
    };
    std::vector<RowInfo> digits, consts;
    for (int i = 0; i < R; ++i) {
        int r = (int)gm[gi[i]];
        int D = (i == fixed) ? r - 1 : r;
        if (D >= 1) digits.push_back({i, r, D});
        else consts.push_back({i, r, D});
    }
    // small ranges first: they can be low digits (4-bit packed, D <= 15)
    std::stable_sort(digits.begin(), digits.end(),
                     [](const RowInfo& a, const RowInfo& b) { return (a.D <= 15) > (b.D <= 15); });
    long double total = 1.0L;
    for (auto& d : digits) total *= (long double)(d.D + 1);
    if (total > 9.0e18L) return fail(GBPERM_ERR_TOO_LARGE, "gbperm_perm_repeated: Gray range beyond 2^63");
    unsigned long long T = 1ull;
    for (auto& d : digits) T *= (unsigned long long)(d.D + 1);

    h->R = R;
    h->C = C;
    h->nd = (int)digits.size();
    h->q = 0;
    h->P = 1;
    h->nseg = T;
    h->steps = (double)T;
    h->photons = (int)sr;
    h->norm_shift = chinhuh ? (int)sr : (int)sr - 1;
    // matrix M (rows: digits then constants) as complex128, dense
    h->M.assign((size_t)R * C * 2, 0.0);
    h->rcoef.clear();
    h->D.clear();
    std::vector<RowInfo> order = digits;
    order.insert(order.end(), consts.begin(), consts.end());
    for (int r = 0; r < R; ++r) {
        int src = gi[order[r].src];
        for (int c = 0; c < C; ++c) {
            int dst = pj[c];
            int64_t ii = transpose ? dst : src, jj = transpose ? src : dst;
            h->M[2 * ((size_t)r * C + c)] = A[2 * (ii * ld + jj)];
            h->M[2 * ((size_t)r * C + c) + 1] = A[2 * (ii * ld + jj) + 1];
        }
        h->rcoef.push_back(order[r].r);
        if (r < h->nd) h->D.push_back(order[r].D);
    }
    h->cpow.clear();
    h->col_src.clear();
    for (int c = 0; c < C; ++c) {
        h->cpow.push_back((int)pm[pj[c]]);
        h->col_src.push_back(pj[c]);
    }
    double fl = 0.0;  // algorithmic flops: colsum updates + product + accumulate
    int mults = 0;
    for (int c = 0; c < C; ++c) mults += h->cpow[c];
    mults -= 1;
    fl = (2.0 * C + 6.0 * mults + 2.0) * (double)T;
    h->flops = fl;
    return GBPERM_OK;
}

void deal_columns_by_power(RepHost* h, int group, int cpl) {
    const int C = h->C;
    if (group <= 1 || C <= 1 || C > group * cpl) return;
    // sorted by power, largest first; ties keep their order
    std::vector<int> s(C);
    for (int c = 0; c < C; ++c) s[c] = c;
    std::stable_sort(s.begin(), s.end(), [h](int a, int b) { return h->cpow[a] > h->cpow[b]; });
    // lane l holds positions [l cpl, l cpl + n_l); slot c of every lane in
    // turn takes the next columns of the sorted list
    std::vector<int> perm(C, -1);  // perm[new position] = old column
    int next = 0;
    for (int c = 0; c < cpl && next < C; ++c)
        for (int l = 0; l < group && next < C; ++l) {
            const int pos = l * cpl + c;
            if (pos < C && c < std::min(cpl, C - l * cpl)) perm[pos] = s[next++];
        }
    std::vector<double> M(h->M.size());
    std::vector<int> cp(C), src(C);
    for (int j = 0; j < C; ++j) {
        const int o = perm[j];
        for (int r = 0; r < h->R; ++r) {
            M[2 * ((size_t)r * C + j)] = h->M[2 * ((size_t)r * C + o)];
            M[2 * ((size_t)r * C + j) + 1] = h->M[2 * ((size_t)r * C + o) + 1];
        }
        cp[j] = h->cpow[o];
        src[j] = h->col_src[o];
    }
    h->M.swap(M);
    h->cpow.swap(cp);
    h->col_src.swap(src);
}

void repeated_low_digits(RepHost* h, const std::function<unsigned long long(unsigned long long)>& slots,
                         double seg_cost) {
    const unsigned long long T = h->nseg * h->P;
    // candidates: prefixes of the digit list with ranges <= 15 (4-bit packed
    // in the kernels) and at most 4096 table entries
    int qmax = 0;
    unsigned long long Pmax = 1ull;
    while (qmax < h->nd && qmax < 16 && h->D[qmax] <= 15 &&
           Pmax * (unsigned long long)(h->D[qmax] + 1) <= 4096ull) {
        Pmax *= (unsigned long long)(h->D[qmax] + 1);
        ++qmax;
    }
    int q = 0;
    const int64_t force_q = g_opt.repeated_low_digits.load();
    if (force_q >= 0) {
        q = (int)std::min<int64_t>(force_q, qmax);
    } else {
        double best = 0.0;
        unsigned long long P = 1ull;
        for (int c = 0; c <= qmax; ++c) {
            if (c > 0) P *= (unsigned long long)(h->D[c - 1] + 1);
            const unsigned long long nseg = T / P;
            const unsigned long long s = std::max(1ull, slots(P));
            const double cost = (double)((nseg + s - 1) / s) * ((double)P + seg_cost);
            if (c == 0 || cost < best) {
                best = cost;
                q = c;
            }
        }
    }
    unsigned long long P = 1ull;
    for (int i = 0; i < q; ++i) P *= (unsigned long long)(h->D[i] + 1);
    h->q = q;
    h->P = P;
    h->nseg = T / P;
    // low-digit tables: binomial weight of each low-digit combination and the
    // digit that moves at each step of the reflected mixed-radix Gray walk.
    // An odometer over the q low digits (g[i] in [0, D_i], digit 0 fastest)
    // gives both without divisions: the digit that moves at step k is the
    // number of digits that wrap when k - 1 becomes k, and only the suffix
    // products of the digits that changed are recomputed.  Every weight is
    // an integer below 2^45 (D_i <= 15 and prod (D_i + 1) <= 4096 bound
    // sum D_i by 45, and C(D, g) <= 2^D), so the products are exact in any
    // order.
    h->wlow.assign(P, 1.0);
    h->seq.assign(P, 0);
    const std::vector<double>& bt = binom_table();
    int g[16] = {0};      // q <= 16
    double suf[17];       // suf[i] = prod_{j >= i} C(D_j, g_j)
    suf[q] = 1.0;
    for (int i = q - 1; i >= 0; --i) suf[i] = suf[i + 1] * bt[h->D[i] * kBinomStride];
    for (unsigned long long k = 0; k < P; ++k) {
        if (k > 0) {
            int d = 0;
            while (++g[d] > h->D[d]) {  // k < P: some digit below q takes the carry
                g[d] = 0;
                ++d;
            }
            h->seq[k] = (unsigned char)d;
            for (int i = d; i >= 0; --i) suf[i] = suf[i + 1] * bt[h->D[i] * kBinomStride + g[i]];
        }
        h->wlow[k] = suf[0];
    }
}

size_t repeated_ws_layout(const RepHost& h, int grid, RepWs* w) {
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align_up(bytes, 256);
        return o;
    };
    RepWs l;
    l.M = take(h.M.size() * sizeof(double));
    l.a1 = take((size_t)h.R * h.C * sizeof(longlong2));
    l.a2 = take((size_t)h.R * h.C * sizeof(longlong2));
    l.ints = take((size_t)(h.R + h.nd + h.C + 64) * sizeof(int));
    l.wlow = take(h.wlow.size() * sizeof(double));
    l.seq = take(h.seq.size());
    l.binom = take((size_t)kBinomStride * kBinomStride * sizeof(double));
    l.exp = take(64);  // exponent int at +0, double-float info {boost, ok} at +16
    l.out = take(8 * sizeof(double));
    l.kern = take(repeated_workspace_bytes(grid));
    if (w) *w = l;
    return off;
}

}  // namespace gbperm

using namespace gbperm;

static int run_repeated(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                        int64_t ncol, const int64_t* row_mult, int64_t nrow, int arith, double* out, double* out_dd,
                        gbperm_stats* stats, bool chinhuh) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32 && arith != GBPERM_ARITH_FX64)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: unknown arithmetic");
    if (!out) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: null output");
    if (rows < 0 || cols < 0 || nrow < 0 || ncol < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated: negative size");
    RepHost h;
    double triv[2];
    bool is_triv = false;
    int rc = repeated_plan(A, rows, cols, ld, col_mult, ncol, row_mult, nrow, &h, triv, &is_triv, true, 0, chinhuh);
    if (rc) return rc;
    if (is_triv) {
        out[0] = triv[0];
        out[1] = triv[1];
        if (out_dd) {
            out_dd[0] = triv[0];
            out_dd[1] = triv[1];
            out_dd[2] = out_dd[3] = 0.0;
        }
        return GBPERM_OK;
    }
    if (!all_finite(h.M.data(), h.R, h.C, h.C)) {
        out[0] = out[1] = NAN;
        if (out_dd) out_dd[0] = out_dd[1] = out_dd[2] = out_dd[3] = NAN;
        return GBPERM_OK;
    }
    // double-float product when requested, within the size rule, and the
    // dynamic range allows it; otherwise (and as its twin) the
    // integer-mantissa product
    bool df = false;
    int dcpl = 0, dgrp = 0, grid_df = 1;
    if (arith == GBPERM_ARITH_DF32 && h.C <= kDfMaxCols && h.photons <= g_opt.df_max_photons.load()) {
        int boost = 0;
        std::vector<int> cw(h.cpow.begin(), h.cpow.end());
        df = df_boost(h.M.data(), h.R, h.C, h.C, h.rcoef.data(), cw.data(), &boost);
    }
    if (df) repeated_df_shape(h.C, &dcpl, &dgrp);
    const bool fx = arith == GBPERM_ARITH_FX64 || arith == GBPERM_ARITH_DF32;
    int xcpl = 0, xgrp = 0, grid_fx = 1;
    if (fx) repeated_fx_shape(h.C, &xcpl, &xgrp);
    if (df) deal_columns_by_power(&h, dgrp, dcpl);
    else if (fx) deal_columns_by_power(&h, xgrp, xcpl);
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long sms = (unsigned long long)device_sms(dev);
    RepArgs a{};
    a.R = h.R;
    a.C = h.C;
    a.nd = h.nd;
    // segment length for the kernel that does the work: one thread per
    // segment in the FP64 kernel, dgrp lanes per segment in the double-float
    // one; setup costs (in steps) fitted to kernel times at 30 photons
    repeated_low_digits(
        &h,
        [&](unsigned long long P) {
            RepArgs t = a;
            t.P = P;
            if (df) return sms * (unsigned long long)repeated_df_blocks_per_sm(t, dcpl, dgrp) * (128ull / dgrp);
            if (fx) return sms * (unsigned long long)repeated_fx_blocks_per_sm(t, xcpl, xgrp) * (128ull / xgrp);
            return sms * (unsigned long long)repeated_blocks_per_sm(t) * 128ull;
        },
        df ? 6.5 : (fx ? 4.0 : 2.0));
    a.q = h.q;
    a.P = h.P;
    a.nseg = h.nseg;
    int bps = repeated_blocks_per_sm(a);
    unsigned long long grid_full = sms * bps;
    unsigned long long need = (h.nseg + 127ull) / 128ull;
    int grid = (int)std::max(1ull, std::min(grid_full, need));
    if (df) {
        unsigned long long gfull = sms * repeated_df_blocks_per_sm(a, dcpl, dgrp);
        unsigned long long per_block = 128ull / (unsigned long long)dgrp;
        unsigned long long need_df = (h.nseg + per_block - 1) / per_block;
        grid_df = (int)std::max(1ull, std::min(gfull, need_df));
    }
    if (fx) {
        unsigned long long gfull = sms * repeated_fx_blocks_per_sm(a, xcpl, xgrp);
        unsigned long long per_block = 128ull / (unsigned long long)xgrp;
        unsigned long long need_fx = (h.nseg + per_block - 1) / per_block;
        grid_fx = (int)std::max(1ull, std::min(gfull, need_fx));
    }
    RepWs w;
    size_t bytes = repeated_ws_layout(h, std::max(std::max(grid, grid_df), grid_fx), &w);
    ThreadCtx& c = thread_ctx();
    rc = c.ensure(bytes);
    if (rc) return rc;
    char* base = static_cast<char*>(c.dbuf);
    cudaStream_t st = c.stream;
    std::vector<int> ints;
    ints.insert(ints.end(), h.rcoef.begin(), h.rcoef.end());
    ints.insert(ints.end(), h.D.begin(), h.D.end());
    ints.insert(ints.end(), h.cpow.begin(), h.cpow.end());
    cudaError_t e = cudaMemcpyAsync(base + w.M, h.M.data(), h.M.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + w.ints, ints.data(), ints.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + w.wlow, h.wlow.data(), h.wlow.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + w.seq, h.seq.data(), h.seq.size(), cudaMemcpyHostToDevice, st);
    const std::vector<double>& bt = binom_table();
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + w.binom, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: upload");
    const int* d_ints = reinterpret_cast<const int*>(base + w.ints);
    PrepArgs pa;
    pa.col_e_out = nullptr;
    pa.A = reinterpret_cast<const double2*>(base + w.M);
    pa.ld = h.C;
    pa.rows = h.R;
    pa.cols = h.C;
    pa.row_w = d_ints;
    pa.col_w = d_ints + h.R + h.nd;
    pa.norm_shift = h.norm_shift;
    pa.a1 = reinterpret_cast<longlong2*>(base + w.a1);
    pa.a2 = reinterpret_cast<longlong2*>(base + w.a2);
    pa.exp_out = reinterpret_cast<int*>(base + w.exp);
    pa.df = df ? 1 : 0;
    pa.df_info = df ? reinterpret_cast<int*>(base + w.exp + 16) : nullptr;
    pa.row_balance = 1;
    pa.exp_fp64_out = pa.exp_out + 1;
    if (stats) cudaEventRecord(c.ev0, st);
    e = launch_prepare(pa, st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: prepare");
    a.a1 = pa.a1;
    a.a2 = pa.a2;
    a.rcoef = d_ints;
    a.D = d_ints + h.R;
    a.cpow = d_ints + h.R + h.nd;
    a.wlow = reinterpret_cast<const double*>(base + w.wlow);
    a.seq = reinterpret_cast<const unsigned char*>(base + w.seq);
    a.binom = reinterpret_cast<const double*>(base + w.binom);
    a.exp_in = pa.exp_out;
    a.df_info = pa.df_info;
    double* dout = reinterpret_cast<double*>(base + w.out);
    a.out2 = dout;
    a.out4 = dout + 2;
    if (df) {
        // dout[6]: the double-float estimate (-1 when the range check fails)
        a.err_out = dout + 6;
        e = cudaMemsetAsync(a.err_out, 0, sizeof(double), st);
        if (e == cudaSuccess)
            e = launch_repeated_df(a, dcpl, dgrp, grid_df, base + w.kern, g_opt.df_escalate.load() != 0, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: df launch");
    }
    // the twin (or the product alone) scales by the exponent without the
    // double-float boost; as the twin it returns at once unless the range
    // check failed or the estimate was above the bar
    a.exp_in = pa.exp_fp64_out;
    a.err_out = nullptr;
    if (fx) {
        e = launch_repeated_fx(a, xcpl, xgrp, grid_fx, base + w.kern, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: fx launch");
    } else {
        e = launch_repeated(a, grid, base + w.kern, st);
        if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: launch");
    }
    if (stats) cudaEventRecord(c.ev1, st);
    double hres[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    e = cudaMemcpyAsync(hres, dout, (df ? 7 : 6) * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "gbperm_perm_repeated: kernel");
    out[0] = hres[0];
    out[1] = hres[1];
    if (out_dd) std::memcpy(out_dd, hres + 2, 4 * sizeof(double));
    if (stats) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        stats->kernel_ms = ms;
        stats->steps = h.steps;
        stats->flops = h.flops;
        stats->launches = df ? 3 : 2;
        stats->grid = df ? grid_df : (fx ? grid_fx : grid);
        stats->seg_log2 = h.q;
        const bool ran_df = df && hres[6] >= 0.0;
        const bool used_df = ran_df && (hres[6] <= kDfEscalate || g_opt.df_escalate.load() == 0);
        stats->arith = used_df ? GBPERM_ARITH_DF32 : (fx ? GBPERM_ARITH_FX64 : GBPERM_ARITH_FP64);
        stats->err_est = ran_df ? hres[6] : 0.0;
    }
    return GBPERM_OK;
}

extern "C" int gbperm_perm_repeated(const double* A, int64_t rows, int64_t cols, int64_t ld,
                                    const int64_t* col_mult, int64_t ncol, const int64_t* row_mult,
                                    int64_t nrow, int arith, double* out, double* out_dd,
                                    gbperm_stats* stats) {
    return run_repeated(A, rows, cols, ld, col_mult, ncol, row_mult, nrow, arith, out, out_dd, stats, false);
}

extern "C" int gbperm_perm_chinhuh(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                                   int64_t ncol, const int64_t* row_mult, int64_t nrow, int arith, double* out,
                                   double* out_dd, gbperm_stats* stats) {
    return run_repeated(A, rows, cols, ld, col_mult, ncol, row_mult, nrow, arith, out, out_dd, stats, true);
}
