/*
 * Precision-generic body of the CPU oracle.  Included twice by perm_oracle.c:
 * once with R = double (suffix _d) and once with R = a 113-bit binary128 type
 * (suffix _q).  Each function restates one reference calculator; the reference
 * file:line it follows is given above it.  Oracle-only test infrastructure.
 *
 * Required macros: R (real type), CX (complex struct name), SFX(name) (suffix).
 */

typedef struct { R re, im; } CX;

static inline CX SFX(cx_mul)(CX a, CX b) {
    CX r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}

/* Neumaier-compensated complex accumulator (stands in for the reference's
 * multi-bucket ComplexM, PicComplexM.hpp:42-285; both exist only to make the
 * 2^(n-1)-term sum accurate). */
typedef struct { R re, im, cre, cim; } SFX(acc_t);

static inline void SFX(acc_add)(SFX(acc_t) * a, CX v) {
    R t = a->re + v.re;
    if ((a->re >= 0 ? a->re : -a->re) >= (v.re >= 0 ? v.re : -v.re)) a->cre += (a->re - t) + v.re;
    else a->cre += (v.re - t) + a->re;
    a->re = t;
    t = a->im + v.im;
    if ((a->im >= 0 ? a->im : -a->im) >= (v.im >= 0 ? v.im : -v.im)) a->cim += (a->im - t) + v.im;
    else a->cim += (v.im - t) + a->im;
    a->im = t;
}

static inline CX SFX(acc_get)(const SFX(acc_t) * a) {
    CX r;
    r.re = a->re + a->cre;
    r.im = a->im + a->cim;
    return r;
}

static inline CX SFX(ld)(const double* A, int64_t ld, int64_t i, int64_t j) {
    CX r;
    r.re = (R)A[2 * (i * ld + j)];
    r.im = (R)A[2 * (i * ld + j) + 1];
    return r;
}

static R SFX(pow2_neg)(int64_t k) {
    R s = (R)1;
    for (int64_t i = 0; i < k; ++i) s *= (R)0.5;
    return s;
}

/* ------------------------------------------------------------------------
 * Plain BBFG, one Gray-code segment [off0, off1).
 * Follows BBFGPermanentCalculator.hpp:128-221: the segment start sums are
 * built exactly from row 0 plus/minus the other rows by the Gray bits of the
 * start index (bit b of the Gray code <-> row rows-1-b), then each step flips
 * the row rows-1-ctz(idx) and adds/subtracts twice that row.
 * The reference keeps a plain per-thread sum (`addend_loc`); the oracle keeps
 * a compensated one per segment.
 * ---------------------------------------------------------------------- */
static CX SFX(bbfg_segment)(const CX* A1, const CX* A2, int64_t rows, int64_t cols,
                            uint64_t off0, uint64_t off1) {
    /* A1 = the matrix, A2 = twice the matrix (the reference's mtx2,
     * BBFGPermanentCalculator.hpp:107-110), both dense rows x cols. */
    CX* colsum = (CX*)malloc(sizeof(CX) * (size_t)cols);
    char* delta = (char*)calloc((size_t)rows, 1);
    SFX(acc_t) acc = {0, 0, 0, 0};
    int parity = 1;
    for (int64_t j = 0; j < cols; ++j) colsum[j] = A1[j];
    uint64_t g = off0 ^ (off0 >> 1);
    for (int64_t r = rows - 1; r > 0; --r) {
        const CX* a = A1 + r * cols;
        if (g & 1ULL) {
            for (int64_t j = 0; j < cols; ++j) {
                colsum[j].re -= a[j].re;
                colsum[j].im -= a[j].im;
            }
            parity = -parity;
            delta[r] = 1;
        } else {
            for (int64_t j = 0; j < cols; ++j) {
                colsum[j].re += a[j].re;
                colsum[j].im += a[j].im;
            }
            delta[r] = 0;
        }
        g >>= 1;
    }
    {
        CX p = colsum[0];
        for (int64_t j = 1; j < cols; ++j) p = SFX(cx_mul)(p, colsum[j]);
        if (parity < 0) { p.re = -p.re; p.im = -p.im; }
        SFX(acc_add)(&acc, p);
    }
    /* plain block sums of 256 terms, folded into the compensated sum */
    CX blk;
    blk.re = (R)0;
    blk.im = (R)0;
    for (uint64_t idx = off0 + 1; idx < off1; ++idx) {
        if ((idx & 255u) == 0) {
            SFX(acc_add)(&acc, blk);
            blk.re = (R)0;
            blk.im = (R)0;
        }
        int64_t row = rows - 1 - (int64_t)__builtin_ctzll(idx);
        delta[row] ^= 1;
        parity = -parity;
        const CX* a = A2 + row * cols;
        CX p;
        p.re = (R)parity;
        p.im = (R)0;
        if (delta[row]) {
            for (int64_t j = 0; j < cols; ++j) {
                colsum[j].re -= a[j].re;
                colsum[j].im -= a[j].im;
                p = SFX(cx_mul)(p, colsum[j]);
            }
        } else {
            for (int64_t j = 0; j < cols; ++j) {
                colsum[j].re += a[j].re;
                colsum[j].im += a[j].im;
                p = SFX(cx_mul)(p, colsum[j]);
            }
        }
        blk.re += p.re;
        blk.im += p.im;
    }
    SFX(acc_add)(&acc, blk);
    free(colsum);
    free(delta);
    return SFX(acc_get)(&acc);
}

/* Dense copies of A and 2A in the working precision. */
static void SFX(make_a12)(const double* A, int64_t rows, int64_t cols, int64_t ld, CX** A1,
                          CX** A2) {
    *A1 = (CX*)malloc(sizeof(CX) * (size_t)(rows * cols));
    *A2 = (CX*)malloc(sizeof(CX) * (size_t)(rows * cols));
    for (int64_t i = 0; i < rows; ++i)
        for (int64_t j = 0; j < cols; ++j) {
            CX a = SFX(ld)(A, ld, i, j);
            (*A1)[i * cols + j] = a;
            (*A2)[i * cols + j].re = a.re * (R)2;
            (*A2)[i * cols + j].im = a.im * (R)2;
        }
}

/* ------------------------------------------------------------------------
 * Repeated-row BBFG over one mixed-radix segment [off0, off1] (inclusive).
 * Follows BBFGPermanentCalculatorRepeated.hpp:193-288 with the n-ary Gray
 * counter of n_aryGrayCodeCounter.cpp:114-240 restated inline:
 *   counter digits are little-endian mixed radix (digit 0 fastest);
 *   gray digit j = counter_j, reflected (limit_j-1-counter_j) when the sum of
 *   the gray digits above j is odd;
 *   one step increments the counter and changes exactly one gray digit.
 * Gray digit g_i is the number of -1 deltas among the rm[i+1] copies of row
 * i+1; its weight is C(rm[i+1], g_i) (exact 128-bit integers, as the
 * reference's piq_int128_t).  M is the (possibly row-prepended) matrix.
 * ---------------------------------------------------------------------- */
static CX SFX(rep_segment)(const double* M, int64_t ld, const int* rm, int64_t nrm,
                           const int* cm, int64_t ncm, uint64_t off0, uint64_t off1) {
    int64_t nd = nrm - 1;
    int* lim = (int*)malloc(sizeof(int) * (size_t)(nd > 0 ? nd : 1));
    int* cnt = (int*)malloc(sizeof(int) * (size_t)(nd > 0 ? nd : 1));
    int* gray = (int*)malloc(sizeof(int) * (size_t)(nd > 0 ? nd : 1));
    CX* colsum = (CX*)malloc(sizeof(CX) * (size_t)(ncm > 0 ? ncm : 1));
    SFX(acc_t) acc = {0, 0, 0, 0};
    for (int64_t i = 0; i < nd; ++i) lim[i] = rm[i + 1] + 1;
    /* counter initialisation, n_aryGrayCodeCounter.cpp:114-140 */
    uint64_t o = off0;
    for (int64_t i = 0; i < nd; ++i) {
        cnt[i] = (int)(o % (uint64_t)lim[i]);
        o /= (uint64_t)lim[i];
    }
    {
        int par = 0;
        for (int64_t j = nd - 1; j >= 0; --j) {
            gray[j] = par ? lim[j] - 1 - cnt[j] : cnt[j];
            par ^= (gray[j] & 1);
        }
    }
    /* segment-start sums and weight, BBFGPermanentCalculatorRepeated.hpp:199-243 */
    __int128 binom = 1;
    int minus_all = 0;
    for (int64_t j = 0; j < ncm; ++j) colsum[j] = SFX(ld)(M, ld, 0, j);
    for (int64_t i = 0; i < nd; ++i) {
        int r = rm[i + 1];
        for (int64_t j = 0; j < ncm; ++j) {
            CX a = SFX(ld)(M, ld, i + 1, j);
            colsum[j].re += a.re * (R)(r - 2 * gray[i]);
            colsum[j].im += a.im * (R)(r - 2 * gray[i]);
        }
        minus_all += gray[i];
        binom *= orc_binom128(r, gray[i]);
    }
    int parity = (minus_all % 2 == 0) ? 1 : -1;
    {
        CX p;
        p.re = (R)parity;
        p.im = (R)0;
        for (int64_t j = 0; j < ncm; ++j)
            for (int k = 0; k < cm[j]; ++k) p = SFX(cx_mul)(p, colsum[j]);
        p.re *= (R)binom;
        p.im *= (R)binom;
        SFX(acc_add)(&acc, p);
    }
    for (uint64_t idx = off0 + 1; idx <= off1; ++idx) {
        /* counter increment, n_aryGrayCodeCounter.cpp:203-218 */
        int64_t d = 0;
        while (d < nd && cnt[d] == lim[d] - 1) { cnt[d] = 0; ++d; }
        if (d >= nd) break;
        cnt[d]++;
        /* locate the changed gray digit, n_aryGrayCodeCounter.cpp:222-234 */
        int par = 0, changed = -1, vprev = 0, vnew = 0;
        for (int64_t j = nd - 1; j >= 0; --j) {
            int gv = par ? lim[j] - 1 - cnt[j] : cnt[j];
            par ^= (gv & 1);
            if (gv != gray[j]) {
                vprev = gray[j];
                vnew = gv;
                gray[j] = gv;
                changed = (int)j;
                break;
            }
        }
        parity = -parity;
        CX p;
        p.re = (R)parity;
        p.im = (R)0;
        for (int64_t j = 0; j < ncm; ++j) {
            CX a = SFX(ld)(M, ld, changed + 1, j);
            if (vprev < vnew) {
                colsum[j].re -= (R)2 * a.re;
                colsum[j].im -= (R)2 * a.im;
            } else {
                colsum[j].re += (R)2 * a.re;
                colsum[j].im += (R)2 * a.im;
            }
            for (int k = 0; k < cm[j]; ++k) p = SFX(cx_mul)(p, colsum[j]);
        }
        /* exact weight update, BBFGPermanentCalculatorRepeated.hpp:279-280 */
        int r = rm[changed + 1];
        binom = vnew < vprev ? binom * vprev / (r - vnew) : binom * (r - vprev) / vnew;
        p.re *= (R)binom;
        p.im *= (R)binom;
        SFX(acc_add)(&acc, p);
    }
    free(lim);
    free(cnt);
    free(gray);
    free(colsum);
    return SFX(acc_get)(&acc);
}

/* ------------------------------------------------------------------------
 * Recursive Glynn, GlynnPermanentCalculator.hpp:146-201: every node adds
 * sign * prod(colsum) and spawns children that subtract 2*row idx for
 * idx in [index_min, rows).
 * ---------------------------------------------------------------------- */
static void SFX(glynn_rec)(const double* A, int64_t rows, int64_t cols, int64_t ld,
                           const CX* colsum, int sign, int64_t index_min, SFX(acc_t) * acc) {
    CX p;
    p.re = (R)1;
    p.im = (R)0;
    for (int64_t j = 0; j < cols; ++j) p = SFX(cx_mul)(p, colsum[j]);
    if (sign < 0) { p.re = -p.re; p.im = -p.im; }
    SFX(acc_add)(acc, p);
    CX* nc = (CX*)malloc(sizeof(CX) * (size_t)cols);
    for (int64_t idx = index_min; idx < rows; ++idx) {
        for (int64_t j = 0; j < cols; ++j) {
            CX a = SFX(ld)(A, ld, idx, j);
            nc[j].re = colsum[j].re - (R)2 * a.re;
            nc[j].im = colsum[j].im - (R)2 * a.im;
        }
        SFX(glynn_rec)(A, rows, cols, ld, nc, -sign, idx + 1, acc);
    }
    free(nc);
}

/* Recursive repeated Glynn, GlynnPermanentCalculatorRepeated.hpp:203-258. */
static void SFX(glynn_rep_rec)(const double* A, int64_t rows, int64_t cols, int64_t ld,
                               const int* limits, const int* cm, const CX* colsum, int sign,
                               int64_t index_min, int64_t mult, SFX(acc_t) * acc) {
    CX p;
    p.re = (R)1;
    p.im = (R)0;
    for (int64_t j = 0; j < cols; ++j)
        for (int k = 0; k < cm[j]; ++k) p = SFX(cx_mul)(p, colsum[j]);
    R w = (R)(mult * sign);
    p.re *= w;
    p.im *= w;
    SFX(acc_add)(acc, p);
    CX* nc = (CX*)malloc(sizeof(CX) * (size_t)cols);
    for (int64_t idx = index_min; idx < rows; ++idx) {
        int ls = sign;
        for (int64_t j = 0; j < cols; ++j) nc[j] = colsum[j];
        for (int k = 1; k <= limits[idx]; ++k) {
            for (int64_t j = 0; j < cols; ++j) {
                CX a = SFX(ld)(A, ld, idx, j);
                nc[j].re -= (R)2 * a.re;
                nc[j].im -= (R)2 * a.im;
            }
            ls = -ls;
            SFX(glynn_rep_rec)(A, rows, cols, ld, limits, cm, nc, ls, idx + 1,
                               mult * (int64_t)orc_binom128(limits[idx], k), acc);
        }
    }
    free(nc);
}

/* ------------------------------------------------------------------------
 * Simple Glynn, GlynnPermanentCalculatorSimple.hpp:61-168: deltas over the
 * columns (delta_c = -1 when bit n-1-c of d is set, column 0 fixed at +1),
 * product over the rows, plain binary order.
 * ---------------------------------------------------------------------- */
static CX SFX(simple)(const double* A, int64_t n, int64_t ld) {
    SFX(acc_t) acc = {0, 0, 0, 0};
    uint64_t P = 1ULL << (n - 1);
    for (uint64_t d = 0; d < P; ++d) {
        CX prod;
        prod.re = (R)1;
        prod.im = (R)0;
        for (int64_t r = 0; r < n; ++r) {
            CX s = SFX(ld)(A, ld, r, 0);
            for (int64_t c = 1; c < n; ++c) {
                CX a = SFX(ld)(A, ld, r, c);
                if ((d >> (n - 1 - c)) & 1ULL) {
                    s.re -= a.re;
                    s.im -= a.im;
                } else {
                    s.re += a.re;
                    s.im += a.im;
                }
            }
            prod = SFX(cx_mul)(prod, s);
        }
        if (__builtin_popcountll(d) & 1) { prod.re = -prod.re; prod.im = -prod.im; }
        SFX(acc_add)(&acc, prod);
    }
    CX r = SFX(acc_get)(&acc);
    R s = SFX(pow2_neg)(n - 1);
    r.re *= s;
    r.im *= s;
    return r;
}

/* ------------------------------------------------------------------------
 * Chin-Huh form of the repeated permanent, CChinHuhPermanentCalculator.cpp:
 * 48-201: every vector v with 0 <= v_j <= in_j over the input (column)
 * multiplicities, in odometer order, contributes
 *   (-1)^{|v|} prod_j C(in_j, v_j) prod_i (sum_j (in_j - 2 v_j) a_ij)^{out_i}
 * (rows i with out_i = 0 skipped), and the sum is divided by 2^N.  The
 * powers are repeated products here.
 * ---------------------------------------------------------------------- */
static CX SFX(chinhuh)(const double* A, int64_t rows, int64_t cols, int64_t ld, const int64_t* in,
                       const int64_t* out, int64_t photons) {
    int64_t* v = (int64_t*)calloc((size_t)(cols > 0 ? cols : 1), sizeof(int64_t));
    SFX(acc_t) acc = {0, 0, 0, 0};
    for (;;) {
        int64_t vs = 0;
        R w = (R)1;
        for (int64_t j = 0; j < cols; ++j) {
            vs += v[j];
            w *= (R)orc_binom128((int)in[j], (int)v[j]);
        }
        if (vs & 1) w = -w;
        CX prod = {(R)1, (R)0};
        for (int64_t i = 0; i < rows; ++i) {
            if (out[i] == 0) continue;
            CX s = {(R)0, (R)0};
            for (int64_t j = 0; j < cols; ++j) {
                CX a = SFX(ld)(A, ld, i, j);
                R coef = (R)(in[j] - 2 * v[j]);
                s.re += coef * a.re;
                s.im += coef * a.im;
            }
            for (int64_t q = 0; q < out[i]; ++q) prod = SFX(cx_mul)(prod, s);
        }
        prod.re *= w;
        prod.im *= w;
        SFX(acc_add)(&acc, prod);
        int64_t j = 0;
        while (j < cols) {
            if (v[j] < in[j]) {
                v[j]++;
                break;
            }
            v[j] = 0;
            ++j;
        }
        if (j == cols) break;
    }
    free(v);
    CX r = SFX(acc_get)(&acc);
    R s = SFX(pow2_neg)(photons);
    r.re *= s;
    r.im *= s;
    return r;
}
