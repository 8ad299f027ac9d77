// Many repeated-multiplicity permanents of one interferometer.
//
// Replaces BatchednPermanentCalculator::calculate
// (piquassoboost/sampling/source/BatchedPermanentCalculator.cpp:109-296),
// which the generalized Clifford simulation strategies fill with (input,
// output) state pairs (CGeneralizedCliffordsSimulationStrategy.cpp:411-423)
// and then evaluate one repeated permanent at a time, and the list branch of
// the repeated wrapper (ChinHuhPermanentCalculator_Wrapper.hpp:233-323).
//
// Each pair is either expanded into its plain N x N matrix (row i of the
// interferometer repeated output[i] times, column j repeated input[j]
// times; N = photons) and joins one persistent batched launch, or, when the
// multiplicities make the mixed-radix Gray code much shorter than the plain
// one, runs as its own repeated launch.  Both give the same permanent.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gbperm.h"
#include "gbperm_capi_internal.h"

namespace gbperm {

namespace {

// Largest photon number expanded into the batched plain launch.
constexpr int64_t kExpandMax = 40;

// Gray steps of the repeated form in its cheaper orientation: prod (m + 1)
// over the occupied modes, with one copy of the smallest multiplicity fixed.
double repeated_steps(const int64_t* mult, int64_t len) {
    double t = 1.0;
    int64_t mn = INT64_MAX;
    for (int64_t i = 0; i < len; ++i)
        if (mult[i] > 0) {
            t *= (double)(mult[i] + 1);
            mn = std::min(mn, mult[i]);
        }
    return mn == INT64_MAX ? 1.0 : t * (double)mn / (double)(mn + 1);
}

}  // namespace

}  // namespace gbperm

using namespace gbperm;

extern "C" int gbperm_perm_repeated_batched(const double* A, int64_t rows, int64_t cols, int64_t ld,
                                            const int64_t* col_mults, int64_t ncol, const int64_t* row_mults,
                                            int64_t nrow, int64_t count, int arith, double* out,
                                            gbperm_stats* stats) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    if (arith == GBPERM_ARITH_FX64) {
        // integer-mantissa product: every pair in one persistent
        // multiplicity launch; pairs with more than 40 occupied product-side
        // modes fall back to the launches below with the FP64 product
        gbperm_rep_batch* plan = nullptr;
        int rc = gbperm_rep_batch_create(A, rows, cols, ld, col_mults, ncol, row_mults, nrow, count, arith, &plan);
        if (rc == GBPERM_OK) {
            rc = gbperm_rep_batch_run(plan, out, stats);
            gbperm_rep_batch_destroy(plan);
            return rc;
        }
        if (rc != GBPERM_ERR_TOO_LARGE) return rc;
        arith = GBPERM_ARITH_FP64;
    }
    if (arith != GBPERM_ARITH_FP64 && arith != GBPERM_ARITH_DF32)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: unknown arithmetic");
    if (count < 0 || rows < 0 || cols < 0 || nrow < 0 || ncol < 0)
        return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: negative size");
    if (count == 0) return GBPERM_OK;
    if (!out) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: null output");
    if ((ncol > 0 && !col_mults) || (nrow > 0 && !row_mults))
        return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: null states");
    if (nrow > rows) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: output state longer than the matrix rows");
    if (ncol > cols) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: input state longer than the matrix columns");
    if (rows > 0 && (!A || ld < cols)) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: bad matrix");
    // validate every pair first: one bad pair fails the whole call, as the
    // reference's list branch raises
    std::vector<int64_t> photons(count, 0);
    for (int64_t i = 0; i < count; ++i) {
        const int64_t* cm = col_mults + i * ncol;
        const int64_t* rm = row_mults + i * nrow;
        int64_t sc = 0, sr = 0;
        for (int64_t j = 0; j < ncol; ++j) {
            if (cm[j] < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: negative occupation");
            sc += cm[j];
        }
        for (int64_t j = 0; j < nrow; ++j) {
            if (rm[j] < 0) return fail(GBPERM_ERR_ARG, "gbperm_perm_repeated_batched: negative occupation");
            sr += rm[j];
        }
        if (sc != sr)
            return fail(GBPERM_ERR_STATE_SUM,
                        "BBFGPermanentCalculatorRepeated_Tasks::calculate:  Number of input and output states should be "
                        "equal");
        photons[i] = sr;
    }
    // split: expanded into the batched plain launch, or a repeated launch
    std::vector<int64_t> ksz;
    std::vector<int64_t> which;  // pair index of each expanded instance
    std::vector<double> packed;
    std::vector<int64_t> solo;
    for (int64_t i = 0; i < count; ++i) {
        const int64_t N = photons[i];
        if (N == 0 || rows == 0 || cols == 0) {
            out[2 * i] = 1.0;
            out[2 * i + 1] = 0.0;
            continue;
        }
        const double t_rep = std::min(repeated_steps(col_mults + i * ncol, ncol), repeated_steps(row_mults + i * nrow, nrow));
        const double t_plain = std::ldexp(1.0, (int)std::min<int64_t>(N, 1000) - 1);
        if (N <= kExpandMax && t_plain <= 4.0 * t_rep) {
            const int64_t* cm = col_mults + i * ncol;
            const int64_t* rm = row_mults + i * nrow;
            std::vector<int64_t> rsrc, csrc;
            for (int64_t r = 0; r < nrow; ++r)
                for (int64_t q = 0; q < rm[r]; ++q) rsrc.push_back(r);
            for (int64_t c = 0; c < ncol; ++c)
                for (int64_t q = 0; q < cm[c]; ++q) csrc.push_back(c);
            const size_t base = packed.size();
            packed.resize(base + 2 * (size_t)N * N);
            for (int64_t r = 0; r < N; ++r)
                for (int64_t c = 0; c < N; ++c) {
                    const double* a = A + 2 * (rsrc[r] * ld + csrc[c]);
                    packed[base + 2 * (r * N + c)] = a[0];
                    packed[base + 2 * (r * N + c) + 1] = a[1];
                }
            ksz.push_back(N);
            which.push_back(i);
        } else {
            solo.push_back(i);
        }
    }
    double kernel_ms = 0.0, steps = 0.0, flops = 0.0;
    int launches = 0;
    if (!ksz.empty()) {
        std::vector<double> res(2 * ksz.size());
        gbperm_stats st{};
        int rc = gbperm_perm_batched(packed.data(), ksz.data(), ksz.data(), (int64_t)ksz.size(), arith, res.data(),
                                     stats ? &st : nullptr);
        if (rc) return rc;
        for (size_t b = 0; b < ksz.size(); ++b) {
            out[2 * which[b]] = res[2 * b];
            out[2 * which[b] + 1] = res[2 * b + 1];
        }
        kernel_ms += st.kernel_ms;
        steps += st.steps;
        flops += st.flops;
        launches += st.launches;
    }
    for (int64_t i : solo) {
        gbperm_stats st{};
        int rc = gbperm_perm_repeated(A, rows, cols, ld, col_mults + i * ncol, ncol, row_mults + i * nrow, nrow, arith,
                                      out + 2 * i, nullptr, stats ? &st : nullptr);
        if (rc) return rc;
        kernel_ms += st.kernel_ms;
        steps += st.steps;
        flops += st.flops;
        launches += st.launches;
    }
    if (stats) {
        stats->kernel_ms = kernel_ms;
        stats->steps = steps;
        stats->flops = flops;
        stats->launches = launches;
        stats->arith = arith;
    }
    return GBPERM_OK;
}
