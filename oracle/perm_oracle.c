/*
 * CPU oracle for the Glynn / BBFG permanent calculators.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * calculators (piquassoboost, sampling/source/ permanent calculators), used by
 * the tests as the expected values and by bench.py as the CPU baseline.  The
 * product library never links or calls it.
 *
 * Parity pin: tests/test_oracle.py checks every entry point against the golden
 * values of the reference's unittests/test_permanent.py:47-251 and against
 * fixtures generated by running the reference's own C++ calculators
 * (tests/golden/make_golden.py, oracle/build_ref.sh).
 *
 * Two precisions are built from one body (perm_oracle_body.h):
 *   _d : IEEE double, the reference's lib 6/7 arithmetic;
 *   _q : IEEE binary128 (113-bit significand) -- __float128 on x86-64 and
 *        long double on AArch64, where long double is binary128.  This is the
 *        extended-precision oracle.  (The reference's own "long double" is the
 *        x87 64-bit-significand type on x86; binary128 is strictly wider.)
 * Results are returned as double-double pairs so that the extended oracle
 * keeps its extra digits: out = {re_hi, im_hi, re_lo, im_lo}.
 *
 * Threading mirrors the reference's work split (BBFGPermanentCalculator.hpp
 * :119-134): the Gray range is cut into 4 x threads contiguous segments; each
 * segment's partial sum is stored by segment index and the partials are added
 * in index order, so results do not depend on thread timing.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#if defined(__x86_64__) || defined(__i386__)
typedef __float128 quad_t_;
#elif defined(__aarch64__)
typedef long double quad_t_;
_Static_assert(sizeof(long double) == 16, "AArch64 long double must be binary128");
#else
#error "binary128 type unknown for this architecture"
#endif

static __thread char g_err[256];

const char* orc_last_error(void) { return g_err; }

static int set_err(int code, const char* msg) {
    snprintf(g_err, sizeof(g_err), "%s", msg);
    return code;
}

/* Exact binomial coefficient, common_functionalities.cpp:131-160 (Pascal row). */
static __int128 orc_binom128(int n, int k) {
    if (k < 0 || k > n) return 0;
    __int128 C[130];
    if (k > 128) return 0;
    memset(C, 0, sizeof(C));
    C[0] = 1;
    for (int i = 1; i <= n; i++)
        for (int j = (i < k ? i : k); j > 0; j--) C[j] = C[j] + C[j - 1];
    return C[k];
}

#define R double
#define CX cx_d
#define SFX(x) x##_d
#include "perm_oracle_body.h"
#undef R
#undef CX
#undef SFX

#define R quad_t_
#define CX cx_q
#define SFX(x) x##_q
#include "perm_oracle_body.h"
#undef R
#undef CX
#undef SFX

static void put_d(cx_d v, double* out) {
    out[0] = v.re;
    out[1] = v.im;
    out[2] = 0.0;
    out[3] = 0.0;
}

static void put_q(cx_q v, double* out) {
    double rh = (double)v.re, ih = (double)v.im;
    out[0] = rh;
    out[1] = ih;
    out[2] = (double)(v.re - (quad_t_)rh);
    out[3] = (double)(v.im - (quad_t_)ih);
}

static int hw_threads(int nthreads) {
    if (nthreads > 0) return nthreads;
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

/* ---------------------------------------------------------------- pool */
typedef struct {
    int kind;   /* 0 plain, 1 repeated */
    int prec;   /* 0 double, 1 quad */
    const double* A;
    int64_t rows, cols, ld;
    const void* A1;
    const void* A2;
    const int* rm;
    int64_t nrm;
    const int* cm;
    int64_t ncm;
    uint64_t total;    /* plain: Idx_max (or the range length); repeated: Idx_max */
    uint64_t base;     /* plain: first Gray index of the range */
    int64_t njobs;
    atomic_llong next;
    cx_d* part_d;
    cx_q* part_q;
} job_t;

static void run_job(job_t* J, int64_t j) {
    uint64_t wb = J->total / (uint64_t)J->njobs;
    uint64_t o0 = (uint64_t)j * wb;
    if (J->kind == 0) {
        uint64_t o1 = (j == J->njobs - 1) ? J->total : (uint64_t)(j + 1) * wb;
        o0 += J->base;
        o1 += J->base;
        if (J->prec == 0)
            J->part_d[j] = bbfg_segment_d((const cx_d*)J->A1, (const cx_d*)J->A2, J->rows, J->cols, o0, o1);
        else
            J->part_q[j] = bbfg_segment_q((const cx_q*)J->A1, (const cx_q*)J->A2, J->rows, J->cols, o0, o1);
    } else {
        uint64_t o1 = (j == J->njobs - 1) ? J->total - 1 : (uint64_t)(j + 1) * wb - 1;
        if (J->prec == 0)
            J->part_d[j] = rep_segment_d(J->A, J->ld, J->rm, J->nrm, J->cm, J->ncm, o0, o1);
        else
            J->part_q[j] = rep_segment_q(J->A, J->ld, J->rm, J->nrm, J->cm, J->ncm, o0, o1);
    }
}

static void* worker(void* arg) {
    job_t* J = (job_t*)arg;
    for (;;) {
        long long j = atomic_fetch_add(&J->next, 1);
        if (j >= J->njobs) break;
        run_job(J, (int64_t)j);
    }
    return NULL;
}

static void run_pool(job_t* J, int nthreads) {
    int nt = nthreads < J->njobs ? nthreads : (int)J->njobs;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)(nt > 0 ? nt : 1));
    atomic_store(&J->next, 0);
    for (int t = 1; t < nt; ++t) pthread_create(&th[t], NULL, worker, J);
    worker(J);
    for (int t = 1; t < nt; ++t) pthread_join(th[t], NULL);
    free(th);
}

/* ------------------------------------------------------------ plain BBFG */
/* BBFGPermanentCalculator::calculate, BBFGPermanentCalculator.cpp:89-126 and
 * BBFGPermanentCalculator.hpp:87-235.  prec: 0 double, 1 binary128. */
int orc_bbfg(const double* A, int64_t rows, int64_t cols, int64_t ld, int prec, int nthreads,
             double* out) {
    if (rows == 0 || cols == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (rows >= cols + 2) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return 0;
    }
    if (rows > 63) return set_err(3, "orc_bbfg: too many rows");
    int nt = hw_threads(nthreads);
    job_t J;
    memset(&J, 0, sizeof(J));
    J.kind = 0; J.prec = prec; J.A = A; J.rows = rows; J.cols = cols; J.ld = ld;
    J.total = 1ULL << (rows - 1);
    int64_t conc = 4 * (int64_t)nt;
    J.njobs = conc < (int64_t)J.total ? conc : (int64_t)J.total;
    if (prec == 0) {
        cx_d *A1, *A2;
        make_a12_d(A, rows, cols, ld, &A1, &A2);
        J.A1 = A1; J.A2 = A2;
        J.part_d = (cx_d*)calloc((size_t)J.njobs, sizeof(cx_d));
        run_pool(&J, nt);
        free(A1); free(A2);
        acc_t_d acc = {0, 0, 0, 0};
        for (int64_t j = 0; j < J.njobs; ++j) acc_add_d(&acc, J.part_d[j]);
        cx_d r = acc_get_d(&acc);
        double s = pow2_neg_d(rows - 1);
        r.re *= s; r.im *= s;
        put_d(r, out);
        free(J.part_d);
    } else {
        cx_q *A1, *A2;
        make_a12_q(A, rows, cols, ld, &A1, &A2);
        J.A1 = A1; J.A2 = A2;
        J.part_q = (cx_q*)calloc((size_t)J.njobs, sizeof(cx_q));
        run_pool(&J, nt);
        free(A1); free(A2);
        acc_t_q acc = {0, 0, 0, 0};
        for (int64_t j = 0; j < J.njobs; ++j) acc_add_q(&acc, J.part_q[j]);
        cx_q r = acc_get_q(&acc);
        quad_t_ s = pow2_neg_q(rows - 1);
        r.re *= s; r.im *= s;
        put_q(r, out);
        free(J.part_q);
    }
    return 0;
}

/* Partial plain BBFG sum over the Gray indices [idx_begin, idx_end) (no
 * 2^-(rows-1) normalisation), with the same 4 x threads segmentation.  Used
 * to time a bounded sample of a large permanent.  prec: 0 double (lib 7),
 * 1 binary128 (lib 8 where long double is binary128, as on AArch64). */
int orc_bbfg_range_prec(const double* A, int64_t rows, int64_t cols, int64_t ld, int prec, int nthreads,
                        uint64_t idx_begin, uint64_t idx_end, double* out) {
    if (rows < 1 || cols < 1 || rows > 63) return set_err(3, "orc_bbfg_range: bad shape");
    if (idx_end > (1ULL << (rows - 1)) || idx_begin >= idx_end) return set_err(1, "orc_bbfg_range: bad range");
    if (prec != 0 && prec != 1) return set_err(1, "orc_bbfg_range: prec must be 0 or 1");
    int nt = hw_threads(nthreads);
    job_t J;
    memset(&J, 0, sizeof(J));
    J.kind = 0; J.prec = prec; J.A = A; J.rows = rows; J.cols = cols; J.ld = ld;
    J.total = idx_end - idx_begin;
    J.base = idx_begin;
    int64_t conc = 4 * (int64_t)nt;
    J.njobs = conc < (int64_t)J.total ? conc : (int64_t)J.total;
    if (prec == 0) {
        cx_d *A1, *A2;
        make_a12_d(A, rows, cols, ld, &A1, &A2);
        J.A1 = A1; J.A2 = A2;
        J.part_d = (cx_d*)calloc((size_t)J.njobs, sizeof(cx_d));
        run_pool(&J, nt);
        acc_t_d acc = {0, 0, 0, 0};
        for (int64_t j = 0; j < J.njobs; ++j) acc_add_d(&acc, J.part_d[j]);
        put_d(acc_get_d(&acc), out);
        free(A1); free(A2); free(J.part_d);
    } else {
        cx_q *A1, *A2;
        make_a12_q(A, rows, cols, ld, &A1, &A2);
        J.A1 = A1; J.A2 = A2;
        J.part_q = (cx_q*)calloc((size_t)J.njobs, sizeof(cx_q));
        run_pool(&J, nt);
        acc_t_q acc = {0, 0, 0, 0};
        for (int64_t j = 0; j < J.njobs; ++j) acc_add_q(&acc, J.part_q[j]);
        put_q(acc_get_q(&acc), out);
        free(A1); free(A2); free(J.part_q);
    }
    return 0;
}

int orc_bbfg_range(const double* A, int64_t rows, int64_t cols, int64_t ld, int nthreads,
                   uint64_t idx_begin, uint64_t idx_end, double* out) {
    return orc_bbfg_range_prec(A, rows, cols, ld, 0, nthreads, idx_begin, idx_end, out);
}

/* --------------------------------------------------------- repeated BBFG */
/* BBFGPermanentCalculatorRepeated::calculate, BBFGPermanentCalculatorRepeated
 * .cpp:75-141 and _Tasks ctor/calculate, .hpp:74-307.
 * col_mult = the input state, row_mult = the output state. */
int orc_bbfg_repeated(const double* A, int64_t rows, int64_t cols, int64_t ld,
                      const int64_t* col_mult, int64_t ncol, const int64_t* row_mult,
                      int64_t nrow, int prec, int nthreads, double* out) {
    if (rows == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (nrow > rows) return set_err(1, "orc_bbfg_repeated: more row multiplicities than rows");
    if (ncol > cols) return set_err(1, "orc_bbfg_repeated: more column multiplicities than columns");
    int* rin = (int*)malloc(sizeof(int) * (size_t)(nrow + 1));
    int* cm = (int*)malloc(sizeof(int) * (size_t)(ncol + 1));
    for (int64_t i = 0; i < nrow; ++i) rin[i] = (int)row_mult[i];
    for (int64_t j = 0; j < ncol; ++j) cm[j] = (int)col_mult[j];
    /* ctor: prepend the first row of smallest nonzero multiplicity with
     * multiplicity 1 (BBFGPermanentCalculatorRepeated.hpp:78-94). */
    int64_t imin = -1;
    for (int64_t i = 0; i < nrow; ++i)
        if (rin[i] != 0 && (imin < 0 || rin[i] < rin[imin])) imin = i;
    int* rm;
    int64_t nrm;
    double* M;
    int64_t Mld, Mrows;
    if (nrow > 0 && imin >= 0) {
        nrm = nrow + 1;
        rm = (int*)malloc(sizeof(int) * (size_t)nrm);
        rm[0] = 1;
        for (int64_t i = 0; i < nrow; ++i) rm[i + 1] = rin[i];
        rm[1 + imin]--;
        Mrows = rows + 1;
        Mld = cols;
        M = (double*)malloc(sizeof(double) * 2 * (size_t)(Mrows * cols));
        for (int64_t j = 0; j < cols; ++j) {
            M[2 * j] = A[2 * (imin * ld + j)];
            M[2 * j + 1] = A[2 * (imin * ld + j) + 1];
        }
        for (int64_t i = 0; i < rows; ++i)
            for (int64_t j = 0; j < cols; ++j) {
                M[2 * ((i + 1) * Mld + j)] = A[2 * (i * ld + j)];
                M[2 * ((i + 1) * Mld + j) + 1] = A[2 * (i * ld + j) + 1];
            }
    } else {
        nrm = nrow;
        rm = (int*)malloc(sizeof(int) * (size_t)(nrm + 1));
        for (int64_t i = 0; i < nrow; ++i) rm[i] = rin[i];
        Mrows = rows;
        Mld = cols;
        M = (double*)malloc(sizeof(double) * 2 * (size_t)(rows * cols));
        for (int64_t i = 0; i < rows; ++i)
            for (int64_t j = 0; j < cols; ++j) {
                M[2 * (i * Mld + j)] = A[2 * (i * ld + j)];
                M[2 * (i * Mld + j) + 1] = A[2 * (i * ld + j) + 1];
            }
    }
    free(rin);
    int rc = 0;
    int64_t sr = 0, sc = 0;
    for (int64_t i = 0; i < nrm; ++i) sr += rm[i];
    for (int64_t j = 0; j < ncol; ++j) sc += cm[j];
    if (sr != sc) {
        rc = set_err(2, "BBFGPermanentCalculatorRepeated_Tasks::calculate:  Number of input and output states should be equal");
        goto done;
    }
    if (Mrows == 0 || cols == 0 || sr == 0 || sc == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        goto done;
    }
    if (Mrows == 1) {
        /* BBFGPermanentCalculatorRepeated.hpp:130-140 */
        if (prec == 0) {
            cx_d p = {1.0, 0.0};
            for (int64_t j = 0; j < ncol; ++j)
                for (int k = 0; k < cm[j]; ++k) p = cx_mul_d(p, ld_d(M, Mld, 0, j));
            put_d(p, out);
        } else {
            cx_q p = {1, 0};
            for (int64_t j = 0; j < ncol; ++j)
                for (int k = 0; k < cm[j]; ++k) p = cx_mul_q(p, ld_q(M, Mld, 0, j));
            put_q(p, out);
        }
        goto done;
    }
    {
        if (sr > 64) { rc = set_err(3, "orc_bbfg_repeated: too many photons"); goto done; }
        uint64_t total = 1;
        for (int64_t i = 1; i < nrm; ++i) {
            uint64_t l = (uint64_t)(rm[i] + 1);
            if (total > (UINT64_MAX >> 1) / l) { rc = set_err(3, "orc_bbfg_repeated: Gray range too large"); goto done; }
            total *= l;
        }
        int nt = hw_threads(nthreads);
        job_t J;
        memset(&J, 0, sizeof(J));
        J.kind = 1; J.prec = prec; J.A = M; J.ld = Mld; J.rm = rm; J.nrm = nrm; J.cm = cm;
        J.ncm = ncol; J.total = total;
        int64_t conc = 4 * (int64_t)nt;
        J.njobs = conc < (int64_t)total ? conc : (int64_t)total;
        if (prec == 0) {
            J.part_d = (cx_d*)calloc((size_t)J.njobs, sizeof(cx_d));
            run_pool(&J, nt);
            acc_t_d acc = {0, 0, 0, 0};
            for (int64_t j = 0; j < J.njobs; ++j) acc_add_d(&acc, J.part_d[j]);
            cx_d r = acc_get_d(&acc);
            double s = pow2_neg_d(sr - 1);
            r.re *= s; r.im *= s;
            put_d(r, out);
            free(J.part_d);
        } else {
            J.part_q = (cx_q*)calloc((size_t)J.njobs, sizeof(cx_q));
            run_pool(&J, nt);
            acc_t_q acc = {0, 0, 0, 0};
            for (int64_t j = 0; j < J.njobs; ++j) acc_add_q(&acc, J.part_q[j]);
            cx_q r = acc_get_q(&acc);
            quad_t_ s = pow2_neg_q(sr - 1);
            r.re *= s; r.im *= s;
            put_q(r, out);
            free(J.part_q);
        }
    }
done:
    free(rm);
    free(cm);
    free(M);
    return rc;
}

/* ------------------------------------------------------- recursive Glynn */
/* GlynnPermanentCalculator<..>::calculate, GlynnPermanentCalculator.hpp
 * :47-136: the initial column sums take every row with delta = +1. */
int orc_glynn_recursive(const double* A, int64_t rows, int64_t cols, int64_t ld, int prec,
                        double* out) {
    if (rows == 0 || cols == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (rows >= cols + 2) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return 0;
    }
    if (rows > 40) return set_err(3, "orc_glynn_recursive: too many rows");
    if (prec == 0) {
        cx_d* cs = (cx_d*)calloc((size_t)cols, sizeof(cx_d));
        for (int64_t j = 0; j < cols; ++j)
            for (int64_t i = 0; i < rows; ++i) {
                cx_d a = ld_d(A, ld, i, j);
                cs[j].re += a.re;
                cs[j].im += a.im;
            }
        acc_t_d acc = {0, 0, 0, 0};
        glynn_rec_d(A, rows, cols, ld, cs, 1, 1, &acc);
        cx_d r = acc_get_d(&acc);
        double s = pow2_neg_d(rows - 1);
        r.re *= s; r.im *= s;
        put_d(r, out);
        free(cs);
    } else {
        cx_q* cs = (cx_q*)calloc((size_t)cols, sizeof(cx_q));
        for (int64_t j = 0; j < cols; ++j)
            for (int64_t i = 0; i < rows; ++i) {
                cx_q a = ld_q(A, ld, i, j);
                cs[j].re += a.re;
                cs[j].im += a.im;
            }
        acc_t_q acc = {0, 0, 0, 0};
        glynn_rec_q(A, rows, cols, ld, cs, 1, 1, &acc);
        cx_q r = acc_get_q(&acc);
        quad_t_ s = pow2_neg_q(rows - 1);
        r.re *= s; r.im *= s;
        put_q(r, out);
        free(cs);
    }
    return 0;
}

/* ---------------------------------------------- recursive repeated Glynn */
/* GlynnPermanentCalculatorRepeated<..>::calculate and Task, Glynn
 * PermanentCalculatorRepeated.hpp:48-193: the first nonzero row keeps one
 * copy fixed at +1 (its delta limit is multiplicity - 1). */
int orc_glynn_repeated(const double* A, int64_t rows, int64_t cols, int64_t ld,
                       const int64_t* col_mult, const int64_t* row_mult, int prec, double* out) {
    int64_t sin_ = 0, sout = 0;
    for (int64_t j = 0; j < cols; ++j) sin_ += col_mult[j];
    for (int64_t i = 0; i < rows; ++i) sout += row_mult[i];
    if (sin_ != sout)
        return set_err(2, "GlynnPermanentCalculatorRepeated::calculate:  Number of input and output states should be equal");
    if (rows == 0 || sin_ == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (sout > 40) return set_err(3, "orc_glynn_repeated: too many photons");
    int* lim = (int*)malloc(sizeof(int) * (size_t)rows);
    int* cm = (int*)malloc(sizeof(int) * (size_t)(cols > 0 ? cols : 1));
    for (int64_t j = 0; j < cols; ++j) cm[j] = (int)col_mult[j];
    int64_t imin = rows;
    for (int64_t i = 0; i < rows; ++i) {
        if (row_mult[i] > 0) {
            if (imin > i) { lim[i] = (int)row_mult[i] - 1; imin = i; }
            else lim[i] = (int)row_mult[i];
        } else lim[i] = 0;
    }
    if (imin == rows) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        free(lim); free(cm);
        return 0;
    }
    if (prec == 0) {
        cx_d* cs = (cx_d*)calloc((size_t)(cols > 0 ? cols : 1), sizeof(cx_d));
        for (int64_t j = 0; j < cols; ++j)
            for (int64_t i = 0; i < rows; ++i) {
                cx_d a = ld_d(A, ld, i, j);
                cs[j].re += (double)row_mult[i] * a.re;
                cs[j].im += (double)row_mult[i] * a.im;
            }
        acc_t_d acc = {0, 0, 0, 0};
        glynn_rep_rec_d(A, rows, cols, ld, lim, cm, cs, 1, imin, 1, &acc);
        cx_d r = acc_get_d(&acc);
        double s = pow2_neg_d(sout - 1);
        r.re *= s; r.im *= s;
        put_d(r, out);
        free(cs);
    } else {
        cx_q* cs = (cx_q*)calloc((size_t)(cols > 0 ? cols : 1), sizeof(cx_q));
        for (int64_t j = 0; j < cols; ++j)
            for (int64_t i = 0; i < rows; ++i) {
                cx_q a = ld_q(A, ld, i, j);
                cs[j].re += (quad_t_)row_mult[i] * a.re;
                cs[j].im += (quad_t_)row_mult[i] * a.im;
            }
        acc_t_q acc = {0, 0, 0, 0};
        glynn_rep_rec_q(A, rows, cols, ld, lim, cm, cs, 1, imin, 1, &acc);
        cx_q r = acc_get_q(&acc);
        quad_t_ s = pow2_neg_q(sout - 1);
        r.re *= s; r.im *= s;
        put_q(r, out);
        free(cs);
    }
    free(lim);
    free(cm);
    return 0;
}

/* ------------------------------------------------------------- Chin-Huh */
/* CChinHuhPermanentCalculator::calculate, CChinHuhPermanentCalculator.cpp:
 * 48-201 (repeated lib 0); see SFX(chinhuh). */
int orc_chinhuh(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* col_mult,
                const int64_t* row_mult, int prec, double* out) {
    int64_t sin_ = 0, sout = 0;
    double steps = 1.0;
    for (int64_t j = 0; j < cols; ++j) {
        sin_ += col_mult[j];
        steps *= (double)(col_mult[j] + 1);
    }
    for (int64_t i = 0; i < rows; ++i) sout += row_mult[i];
    if (sin_ != sout)
        return set_err(2, "CChinHuhPermanentCalculator::calculate:  Number of input and output states should be equal");
    if (rows == 0 || sin_ == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (steps > 1e8) return set_err(3, "orc_chinhuh: too many terms for the oracle");
    if (prec == 0) put_d(chinhuh_d(A, rows, cols, ld, col_mult, row_mult, sin_), out);
    else put_q(chinhuh_q(A, rows, cols, ld, col_mult, row_mult, sin_), out);
    return 0;
}

/* ---------------------------------------------------------- simple Glynn */
/* GlynnPermanentCalculatorSimple.hpp:61-168.  Non-square input returns 0
 * (the reference prints a message and returns 0). */
int orc_glynn_simple(const double* A, int64_t rows, int64_t cols, int64_t ld, int prec,
                     double* out) {
    if (rows == 0 || cols == 0) {
        out[0] = 1.0; out[1] = 0.0; out[2] = 0.0; out[3] = 0.0;
        return 0;
    }
    if (rows != cols) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return 0;
    }
    if (rows > 30) return set_err(3, "orc_glynn_simple: too many rows");
    if (prec == 0) put_d(simple_d(A, rows, ld), out);
    else put_q(simple_q(A, rows, ld), out);
    return 0;
}

/* ------------------------------------------------- submatrix extraction */
/* adaptInterferometer, BatchedPermanentCalculator.cpp:412-451: keep the rows
 * of nonzero output occupation and the columns of nonzero input occupation. */
int orc_adapt_interferometer(const double* U, int64_t m, int64_t ld, const int64_t* input_state,
                             const int64_t* output_state, double* out, int64_t* out_rows,
                             int64_t* out_cols) {
    int64_t nr = 0, nc = 0;
    for (int64_t i = 0; i < m; ++i) nr += output_state[i] > 0;
    for (int64_t j = 0; j < m; ++j) nc += input_state[j] > 0;
    *out_rows = nr;
    *out_cols = nc;
    if (!out) return 0;
    int64_t r = 0;
    for (int64_t i = 0; i < m; ++i) {
        if (output_state[i] <= 0) continue;
        int64_t c = 0;
        for (int64_t j = 0; j < m; ++j) {
            if (input_state[j] <= 0) continue;
            out[2 * (r * nc + c)] = U[2 * (i * ld + j)];
            out[2 * (r * nc + c) + 1] = U[2 * (i * ld + j) + 1];
            ++c;
        }
        ++r;
    }
    return 0;
}

/* adaptInterferometerGlynnMultiplied, BatchedPermanentCalculator.cpp:367-399:
 * row i repeated output_state[i] times, column j input_state[j] times. */
int orc_adapt_interferometer_multiplied(const double* U, int64_t m, int64_t ld,
                                        const int64_t* input_state, const int64_t* output_state,
                                        double* out, int64_t* out_n) {
    int64_t n = 0;
    for (int64_t j = 0; j < m; ++j) n += input_state[j];
    *out_n = n;
    if (!out) return 0;
    int64_t r = 0;
    for (int64_t i = 0; i < m; ++i)
        for (int64_t rr = 0; rr < output_state[i]; ++rr) {
            int64_t c = 0;
            for (int64_t j = 0; j < m; ++j)
                for (int64_t cc = 0; cc < input_state[j]; ++cc) {
                    out[2 * (r * n + c)] = U[2 * (i * ld + j)];
                    out[2 * (r * n + c) + 1] = U[2 * (i * ld + j) + 1];
                    ++c;
                }
            ++r;
        }
    return 0;
}

/* --------------------------------------------------------- compute_pmf */
/* compute_pmf, sampling/simulation_strategies/source/samplingHelperFunctions
 * .cpp:78-342 (its CPU branch): for every occupied input mode idx, the
 * repeated permanent of the sample (rows) against the input with one photon
 * removed from idx (columns), then
 *   pmf[mdx] ~ | sum_idx input[idx] * addend[idx] * U[mdx][idx] |^2,
 * normalised to sum 1.  addends (2m doubles, may be NULL) receives the
 * permanents, zero for unoccupied modes. */
int orc_compute_pmf(const double* U, int64_t m, int64_t ld, const int64_t* sample, const int64_t* current_input,
                    int prec, int nthreads, double* pmf, double* addends) {
    double* add = (double*)calloc((size_t)(2 * m), sizeof(double));
    int64_t* inp = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    int64_t* fin = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    int64_t* fout = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    double* sub = (double*)malloc(sizeof(double) * 2 * (size_t)(m * m));
    int rc = 0;
    for (int64_t idx = 0; idx < m && rc == 0; ++idx) {
        if (current_input[idx] <= 0) continue;
        for (int64_t j = 0; j < m; ++j) inp[j] = current_input[j];
        inp[idx]--;
        int64_t nr = 0, nc = 0;
        orc_adapt_interferometer(U, m, ld, inp, sample, sub, &nr, &nc);
        int64_t a = 0, b = 0;
        for (int64_t j = 0; j < m; ++j) {
            if (inp[j] > 0) fin[a++] = inp[j];
            if (sample[j] > 0) fout[b++] = sample[j];
        }
        double o4[4];
        rc = orc_bbfg_repeated(sub, nr, nc, nc > 0 ? nc : 1, fin, a, fout, b, prec, nthreads, o4);
        add[2 * idx] = o4[0];
        add[2 * idx + 1] = o4[1];
    }
    if (rc == 0) {
        double total = 0.0;
        for (int64_t mdx = 0; mdx < m; ++mdx) {
            double re = 0.0, im = 0.0;
            for (int64_t idx = 0; idx < m; ++idx) {
                if (current_input[idx] == 0) continue;
                double ur = U[2 * (mdx * ld + idx)], ui = U[2 * (mdx * ld + idx) + 1];
                double pr = (double)current_input[idx] * add[2 * idx];
                double pi = (double)current_input[idx] * add[2 * idx + 1];
                re += pr * ur - pi * ui;
                im += pr * ui + pi * ur;
            }
            pmf[mdx] = re * re + im * im;
            total += pmf[mdx];
        }
        for (int64_t mdx = 0; mdx < m; ++mdx) pmf[mdx] /= total;
        if (addends) memcpy(addends, add, sizeof(double) * 2 * (size_t)m);
    }
    free(add);
    free(inp);
    free(fin);
    free(fout);
    free(sub);
    return rc;
}

/* ------------------------------------------------- Clifford & Clifford B */
/* MT19937 (Matsumoto & Nishimura, ACM TOMACS 8(1), 1998; the generator that
 * std::mt19937 specifies), restated from the published algorithm: 624-word
 * state, initialised by x_i = 1812433253 (x_{i-1} xor (x_{i-1} >> 30)) + i,
 * twisted 624 words at a time and tempered on output. */
typedef struct {
    uint32_t x[624];
    int i;
} orc_mt_t;

static void orc_mt_seed(orc_mt_t* g, uint32_t s) {
    g->x[0] = s;
    for (int i = 1; i < 624; ++i) g->x[i] = 1812433253u * (g->x[i - 1] ^ (g->x[i - 1] >> 30)) + (uint32_t)i;
    g->i = 624;
}

static uint32_t orc_mt_next(orc_mt_t* g) {
    if (g->i >= 624) {
        for (int k = 0; k < 624; ++k) {
            const uint32_t y = (g->x[k] & 0x80000000u) | (g->x[(k + 1) % 624] & 0x7fffffffu);
            g->x[k] = g->x[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        g->i = 0;
    }
    uint32_t y = g->x[g->i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

/* CGeneralizedCliffordsBSimulationStrategy::simulate without MPI
 * (simulation_strategies/source/CGeneralizedCliffordsBSimulationStrategy.cpp
 * :137-283) and fill_r_sample (:287-316), with the helpers of
 * samplingHelperFunctions.cpp: the generator seeded with the low 32 bits of
 * `seed` (:60-62), a photon of the working input list picked by
 * generator() % size (:68-74, update_input_by_single_photon :378-405), one
 * compute_pmf layer per photon, and the output mode drawn as the first index
 * whose running pmf sum reaches generator() / (2^32 - 1) (sample_from_pmf
 * :351-375; index 0 when no sum reaches it).  out: nsamples x m occupations.
 * transmissivity >= 0: the uniform-losses strategy
 * (CGeneralizedCliffordsBUniformLossesSimulationStrategy.cpp:110-322): each
 * sample first draws its photon count k, the first k whose running sum of
 * binom(n, k) eta^k (1 - eta)^(n - k), eta = transmissivity^2, reaches
 * generator() / (2^32 - 1) (or 1), and places k photons; < 0: lossless. */
int orc_sample_b(const double* U, int64_t m, int64_t ld, const int64_t* input_state, int64_t nsamples,
                 uint64_t seed, double transmissivity, int prec, int nthreads, int64_t* out) {
    orc_mt_t g;
    orc_mt_seed(&g, (uint32_t)seed);
    int64_t np = 0;
    for (int64_t i = 0; i < m; ++i) {
        if (input_state[i] < 0) return set_err(1, "orc_sample_b: negative occupation");
        np += input_state[i];
    }
    int64_t* particles = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
    int64_t* working = (int64_t*)malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
    int64_t* current = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
    double* pmf = (double*)malloc(sizeof(double) * (size_t)m);
    int64_t k = 0;
    for (int64_t i = 0; i < m; ++i)
        for (int64_t c = 0; c < input_state[i]; ++c) particles[k++] = i;
    double* law = (double*)malloc(sizeof(double) * (size_t)(np + 1));
    if (transmissivity >= 0.0) {
        const double eta = transmissivity * transmissivity;
        for (int64_t i = 0; i <= np; ++i) {
            int64_t b = 1;
            for (int64_t q = 1; q <= i; ++q) b = b * (np - i + q) / q;
            law[i] = (double)b * pow(eta, (double)i) * pow(1.0 - eta, (double)(np - i));
        }
    }
    int rc = 0;
    for (int64_t s = 0; s < nsamples && rc == 0; ++s) {
        int64_t* sample = out + s * m;
        memset(sample, 0, sizeof(int64_t) * (size_t)m);
        memset(current, 0, sizeof(int64_t) * (size_t)m);
        memcpy(working, particles, sizeof(int64_t) * (size_t)np);
        int64_t nw = np, ns = 0, target = np;
        if (transmissivity >= 0.0) {
            const double u = (double)orc_mt_next(&g) / 4294967295.0;
            int64_t q = 0;
            double w = law[0];
            while (w < u && w < 1.0 && q < np) {
                ++q;
                w += law[q];
            }
            target = q;
        }
        while (target > ns && rc == 0) {
            const int64_t r = (int64_t)(orc_mt_next(&g) % (uint32_t)nw);
            current[working[r]]++;
            memmove(working + r, working + r + 1, sizeof(int64_t) * (size_t)(nw - r - 1));
            nw--;
            rc = orc_compute_pmf(U, m, ld, sample, current, prec, nthreads, pmf, NULL);
            if (rc) break;
            const double u = (double)orc_mt_next(&g) / 4294967295.0;
            int64_t pick = 0;
            double acc = 0.0;
            for (int64_t i = 0; i < m; ++i) {
                acc = acc + pmf[i];
                if (acc >= u) {
                    pick = i;
                    break;
                }
            }
            sample[pick]++;
            ns++;
        }
    }
    free(particles);
    free(working);
    free(current);
    free(pmf);
    free(law);
    return rc;
}
