// Shared device/host helpers for the GB300 permanent kernels.
//
// Number formats used on the device:
//   * column sums: exact two's-complement 64-bit fixed point per component.
//     Every column j is pre-scaled on the host by a power of two 2^s_j so that
//     sum_i |Re a_ij| and sum_i |Im a_ij| (times the row multiplicity) stay
//     below 1; the fixed-point unit is 2^-62.  Adding or subtracting a row is
//     exact, so column sums never drift, whatever the segment length.
//   * the n-term product: IEEE double (FP64 pipe), fed by an integer-only
//     int64 -> double conversion (no FP64 instruction spent on it);
//   * term accumulation: double per block of steps, folded into a
//     double-double (TwoSum) accumulator; the cross-thread reduction is
//     double-double throughout.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define GBPERM_FIX_BITS 62

namespace gbperm {

struct dd {  // double-double: value = hi + lo, |lo| <= ulp(hi)/2
    double hi, lo;
};

struct cdd {  // complex double-double
    dd re, im;
};

__host__ __device__ __forceinline__ dd two_sum(double a, double b) {
    double s = a + b;
    double bb = s - a;
    double e = (a - (s - bb)) + (b - bb);
    return dd{s, e};
}

__host__ __device__ __forceinline__ dd dd_add(dd a, dd b) {
    dd s = two_sum(a.hi, b.hi);
    dd t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ dd dd_add_d(dd a, double b) {
    dd s = two_sum(a.hi, b);
    s.lo += a.lo;
    return two_sum(s.hi, s.lo);
}

__host__ __device__ __forceinline__ cdd cdd_add(cdd a, cdd b) {
    return cdd{dd_add(a.re, b.re), dd_add(a.im, b.im)};
}

__device__ __forceinline__ dd shfl_xor_dd(dd v, int m) {
    return dd{__shfl_xor_sync(0xffffffffu, v.hi, m), __shfl_xor_sync(0xffffffffu, v.lo, m)};
}

// Warp-wide double-double sum (every lane ends with the total).
__device__ __forceinline__ cdd warp_sum_cdd(cdd v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) {
        cdd o{shfl_xor_dd(v.re, m), shfl_xor_dd(v.im, m)};
        v = cdd_add(v, o);
    }
    return v;
}

// Warp-wide double sum (every lane ends with the total).
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

// Exact int64 fixed point (unit 2^-62) -> double, round-to-nearest-up on the
// dropped bits, using integer instructions only.  x == 0 maps to +0.0.
__device__ __forceinline__ double fix_to_double(long long x) {
    unsigned long long s = (unsigned long long)(x >> 63);            // 0 or all ones
    unsigned long long m = ((unsigned long long)x ^ s) - s;          // |x| < 2^63
    int lz = __clzll((long long)m);                                  // 64 when m == 0
    unsigned long long mn = m << (lz & 63);                          // bit 63 set (m != 0)
    // value = m * 2^-62 = (mn / 2^63) * 2^(1 - lz): biased exponent 1024 - lz.
    unsigned long long bits = ((unsigned long long)(1023 - lz) << 52) + (mn >> 11);
    bits += (mn >> 10) & 1ull;                                       // round (carry may bump exponent)
    bits |= s & 0x8000000000000000ull;
    bits = (m == 0ull) ? 0ull : bits;
    return __longlong_as_double((long long)bits);
}

// Complex double helpers (FP64 pipe).
struct cd {
    double re, im;
};

__device__ __forceinline__ cd cmul(cd a, cd b) {
    cd r;
    r.re = fma(a.re, b.re, -a.im * b.im);
    r.im = fma(a.re, b.im, a.im * b.re);
    return r;
}

// ---------------------------------------------------------- double-float
// Unevaluated float pairs h + l on the FP32 pipe ("df").  Products keep the
// exact error of the leading product (FMA) and the first-order cross terms;
// the pair is not renormalised after a multiply (|l| stays below ~2^-22 |z|),
// which keeps the error of a complex product near 2^-46 |z|.
//
// The error-free steps below only hold with every add and multiply rounded
// on its own: a multiply that the compiler fused into a following add (its
// default FMA contraction) would already carry the product's exact value,
// which the separately computed error term then adds a second time.  The
// primitives therefore use __fadd_rn / __fsub_rn / __fmul_rn, which are
// never contracted; the FMAs they need are written out as fmaf.
struct cf {  // complex double-float
    float rh, rl, ih, il;
};

// Knuth's TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ cf cf_mul(const cf& x, const cf& y) {
    cf z;
    // real part: xr*yr - xi*yi
    const float p1 = __fmul_rn(x.rh, y.rh);
    const float e1 = fmaf(x.rh, y.rh, -p1);
    const float p2 = __fmul_rn(x.ih, y.ih);
    const float e2 = fmaf(x.ih, y.ih, -p2);
    float s, t;
    two_sum_f(p1, -p2, s, t);
    float u = __fadd_rn(__fsub_rn(e1, e2), t);
    u = fmaf(x.rh, y.rl, u);
    u = fmaf(x.rl, y.rh, u);
    u = fmaf(-x.ih, y.il, u);
    u = fmaf(-x.il, y.ih, u);
    z.rh = s;
    z.rl = u;
    // imaginary part: xr*yi + xi*yr
    const float q1 = __fmul_rn(x.rh, y.ih);
    const float f1 = fmaf(x.rh, y.ih, -q1);
    const float q2 = __fmul_rn(x.ih, y.rh);
    const float f2 = fmaf(x.ih, y.rh, -q2);
    float s2, t2;
    two_sum_f(q1, q2, s2, t2);
    float v = __fadd_rn(__fadd_rn(f1, f2), t2);
    v = fmaf(x.rh, y.il, v);
    v = fmaf(x.rl, y.ih, v);
    v = fmaf(x.ih, y.rl, v);
    v = fmaf(x.il, y.rh, v);
    z.ih = s2;
    z.il = v;
    return z;
}

// int64 fixed point -> float pair with three exact 21-bit chunks:
// x = c2 2^42 + c1 2^21 + c0 (c2 signed, c1, c0 in [0, 2^21)).  s2, s1, s0
// are the powers of two 2^(o-20), 2^(o-41), 2^(o-62) (o: the matrix's range
// boost).  The leading pair is combined with Fast2Sum, valid because
// |f2| >= 2^(o-20) > f1 whenever c2 != 0.
__device__ __forceinline__ void fix_to_df(long long x, float s2, float s1, float s0, float& h, float& l) {
    const int c2 = (int)(x >> 42);
    const int c1 = (int)((x >> 21) & 0x1FFFFFll);
    const int c0 = (int)(x & 0x1FFFFFll);
    const float f2 = __fmul_rn(__int2float_rn(c2), s2);
    const float f1 = __fmul_rn(__int2float_rn(c1), s1);
    const float f0 = __fmul_rn(__int2float_rn(c0), s0);
    h = __fadd_rn(f2, f1);
    const float e = __fsub_rn(f1, __fsub_rn(h, f2));
    l = __fadd_rn(e, f0);
}

// int64 fixed point -> float pair without conversion instructions.  The three
// chunks are written straight into float mantissas whose exponents carry the
// chunk units ("magic number" conversion): for 0 <= c < 2^23,
//   as_float(bits(2^(23+u)) | c) - 2^(23+u) = c 2^u   exactly,
// and the signed top chunk is offset by 2^22 first.  m[0..2] are the magic
// bit patterns for the units 2^(o-20), 2^(o-41), 2^(o-62) of chunks c2, c1,
// c0; off[0..2] the matching float offsets (off[0] includes the 2^22 shift).
struct DfConv {
    unsigned int m2, m1, m0;
    float o2, o1, o0;
};

__host__ __device__ inline DfConv make_dfconv(int boost) {
    DfConv c;
    // unit exponents of the chunks
    const int u2 = boost - 20, u1 = boost - 41, u0 = boost - 62;
    c.m2 = (unsigned int)(127 + 23 + u2) << 23;
    c.m1 = (unsigned int)(127 + 23 + u1) << 23;
    c.m0 = (unsigned int)(127 + 23 + u0) << 23;
    // 2^(23+u) (+ 2^(22+u) for the offset top chunk)
    union {
        unsigned int u;
        float f;
    } a, b, d;
    a.u = c.m2;
    b.u = c.m1;
    d.u = c.m0;
    c.o2 = a.f * 1.5f;  // 2^(23+u2) + 2^(22+u2)
    c.o1 = b.f;
    c.o0 = d.f;
    return c;
}

__device__ __forceinline__ void fix_to_df_magic(long long x, const DfConv& k, float& h, float& l) {
    const unsigned int lo = (unsigned int)x;
    const unsigned int hi = (unsigned int)((unsigned long long)x >> 32);
    const int c2 = ((int)hi >> 10) + (1 << 22);                      // bits 42..63, offset
    const unsigned int c1 = __funnelshift_r(lo, hi, 21) & 0x1FFFFFu;  // bits 21..41
    const unsigned int c0 = lo & 0x1FFFFFu;                           // bits 0..20
    const float f2 = __fsub_rn(__uint_as_float(k.m2 + (unsigned int)c2), k.o2);
    const float f1 = __fsub_rn(__uint_as_float(k.m1 | c1), k.o1);
    const float f0 = __fsub_rn(__uint_as_float(k.m0 | c0), k.o0);
    h = __fadd_rn(f2, f1);
    const float e = __fsub_rn(f1, __fsub_rn(h, f2));
    l = __fadd_rn(e, f0);
}

// Segment of work slot u for the mixed-radix Gray sweeps.  Consecutive
// segments differ by +-1 in one high Gray digit, so the parity of the high
// digits is h & 1, and that parity alone fixes the start of the low digits
// and hence the whole walk inside a segment (which digit moves, up or down).
// A warp's S consecutive slots (S a power of two: segments per warp) are
// given segments of one parity -- within each block of 2S slots the first S
// take the block's even segments and the last S its odd ones -- so every
// step's direction is warp-uniform.  Slots at or past `full` (nseg rounded
// down to a multiple of 2S) keep u.
__device__ __forceinline__ unsigned long long parity_slot(unsigned long long u, unsigned long long S,
                                                          unsigned long long full) {
    if (u >= full) return u;
    const unsigned long long r = u & (2 * S - 1);
    return (u - r) + (r < S ? 2 * r : 2 * (r - S) + 1);
}

// df accumulator: a += (h, l), renormalised
__device__ __forceinline__ void df_acc(float& ah, float& al, float h, float l) {
    float s, e;
    two_sum_f(ah, h, s, e);
    e = __fadd_rn(e, __fadd_rn(al, l));
    ah = __fadd_rn(s, e);
    al = __fsub_rn(e, __fsub_rn(ah, s));
}

}  // namespace gbperm
