// Integer-mantissa complex product ("fx") for the GB300 permanent kernels.
//
// On GB300 the FP64 pipe retires about 1.6 FMA per clock per SM, while the
// 32-bit integer multiply-add (IMAD, IMAD.WIDE) and the ALU run at tens of
// lanes per clock.  The column sums of the Gray sweep are already exact
// two's-complement 64-bit fixed point, so the n-term product can stay in
// integers: every factor is a complex number with 64-bit integer components
// and a shared binary exponent, split into 31-bit limbs
//     v = h 2^31 + l,   h signed, l in [0, 2^31),
// and a complex multiply is twelve 32x32->64 multiply-adds (mad.wide.s32)
// plus a renormalising shift.  Each multiply keeps 55-57 significant bits
// (the FP64 product keeps 53), so the product is at least as accurate as the
// FP64 kernel's while it runs on the integer pipes.
//
// Value convention: a mantissa m with shift count sigma stands for
//     m * 2^(-61 - sigma).
// A column sum C (unit 2^-62, |C| <= 2^62 per component; 2^62 is the exact
// value 1 a padding column carries) enters as y = C >> 1
// with sigma = 0.  fx_mul returns R = x y / 2^62 (sigma_R = sigma_x +
// sigma_y - 1); fx_norm shifts R left by s (sigma += s).  A chain of k
// multiplies over factors with sigma = 0 therefore ends with
// sigma = (sum of the shifts) - k.
//
// Range invariants (what keeps every intermediate inside int64):
//   * normalised operands: |component| <= 2^59, so |h| <= 2^28;
//   * column factors: |component| <= 2^61, so |h| <= 2^30;
//   * the cross sum of fx_mul is at most 2^30 + 2 * 2^59 + 2 * 2^61 < 2^63;
//   * |x y| / 2^62 <= (sqrt2 2^59)(sqrt2 2^61) / 2^62 = 2^59, so R's
//     components are at most 2^59 + 2 and its high word at most 2^27,
//     which fx_norm handles with a shift s in [-1, 27].
#pragma once
#include "gbperm_common.cuh"

namespace gbperm {

struct fxl {  // limbs of a complex mantissa: re = rh 2^31 + rl, im = ih 2^31 + il
    int rh, rl, ih, il;
};

// Limbs of the column factor y = C >> 1 (C: int64 column sum, |C| <= 2^62):
// the high limb is C's high word, the low limb C's low word shifted right by
// one (bits 1..31 of C).
__device__ __forceinline__ fxl fx_col(long long cr, long long ci) {
    fxl y;
    y.rh = (int)(cr >> 32);
    y.rl = (int)((unsigned int)cr >> 1);
    y.ih = (int)(ci >> 32);
    y.il = (int)((unsigned int)ci >> 1);
    return y;
}

// d = a b + c with a 32x32->64 signed multiply-add (one IMAD.WIDE).
__device__ __forceinline__ long long madw(int a, int b, long long c) {
    long long d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// R = x y / 2^62 rounded to nearest up to the dropped low-limb products
// (error below 1.5 units of R).  x: normalised, y: a column factor or
// normalised (the cross-sum bound above needs x normalised).  Twelve
// accumulating 32x32->64 multiply-adds; the subtracted products take a
// negated 32-bit limb (|limb| < 2^31, so the negation is exact).
__device__ __forceinline__ void fx_mul(const fxl& x, const fxl& y, long long& re, long long& im) {
    const int nih = -x.ih, nil = -x.il;
    long long mr = madw(x.rh, y.rl, 1ll << 30);
    long long mi = madw(x.rh, y.il, 1ll << 30);
    mr = madw(x.rl, y.rh, mr);
    mi = madw(x.rl, y.ih, mi);
    mr = madw(nih, y.il, mr);
    mi = madw(x.ih, y.rl, mi);
    mr = madw(nil, y.ih, mr);
    mi = madw(x.il, y.rh, mi);
    re = madw(nih, y.ih, madw(x.rh, y.rh, mr >> 31));
    im = madw(x.ih, y.rh, madw(x.rh, y.ih, mi >> 31));
}

// Bit position of the leading non-sign bit of the larger of two signed
// high words (PTX bfind.s32: for a negative word the most significant 0),
// -1 when both are 0 or -1.  Two bfind and a max measured 3-4% faster in
// the plain kernel than one bfind on the OR of the one's-complement
// magnitudes (fewer ALU-pipe instructions).
__device__ __forceinline__ int fx_lead2(int hr, int hi) {
    int fr, fi;
    asm("bfind.s32 %0, %1;" : "=r"(fr) : "r"(hr));
    asm("bfind.s32 %0, %1;" : "=r"(fi) : "r"(hi));
    return max(fr, fi);
}

// Normalise R (components at most 2^59 + 2 in magnitude) to limbs whose
// larger component has its leading bit at 58 (|component| <= 2^59); returns
// the left shift s in [-1, 27] (s = 27 when |R| < 2^32: such tiny values are
// shifted as far as the limb split allows).
__device__ __forceinline__ int fx_norm(long long re, long long im, fxl& x) {
    const unsigned int lr = (unsigned int)re, li = (unsigned int)im;
    const int hr = (int)(re >> 32), hi = (int)(im >> 32);
    const int f = fx_lead2(hr, hi);    // -1 when both high words are 0 or -1
    const int ls = 27 - f;             // s + 1, in [0, 28]
    // high limb = (R << s) >> 31 = the high word of R << (s + 1)
    x.rh = (int)__funnelshift_l(lr, (unsigned int)hr, ls);
    x.ih = (int)__funnelshift_l(li, (unsigned int)hi, ls);
    x.rl = (int)((lr << ls) >> 1);
    x.il = (int)((li << ls) >> 1);
    return 26 - f;
}

// Normalise a column factor y = C >> 1 (|component| <= 2^61) as the first
// factor of a product chain: same target as fx_norm, shift s in [-3, 27].
__device__ __forceinline__ int fx_norm_col(long long cr, long long ci, fxl& x) {
    const long long yr = cr >> 1, yi = ci >> 1;
    const int hr = (int)(yr >> 32), hi = (int)(yi >> 32);
    const int f = fx_lead2(hr, hi);    // <= 29
    const int s = 26 - f;
    long long vr, vi;
    if (s >= 0) {
        vr = yr << s;
        vi = yi << s;
    } else {
        vr = yr >> (-s);
        vi = yi >> (-s);
    }
    x.rh = (int)(vr >> 31);
    x.rl = (int)(vr & 0x7FFFFFFFll);
    x.ih = (int)(vi >> 31);
    x.il = (int)(vi & 0x7FFFFFFFll);
    return s;
}

// The value of the limbs as int64 components (for the final conversion).
__device__ __forceinline__ long long fx_join(int h, int l) { return ((long long)h << 31) + (long long)l; }

// x 2^e as a double: the int64 -> double conversion (cvt.rn.f64.s64, round
// to nearest even) with e added to its exponent field; 0 when x == 0 or when
// the result would be below the normal range.  Against fx_to_double_alu it
// trades about twenty ALU-pipe instructions for one FP64-pipe conversion:
// measured 1.3% faster in the plain kernel and 27% in the pmf kernel.
__device__ __forceinline__ double fx_to_double(long long x, int e) {
    const long long b = __double_as_longlong((double)x);
    const int be = (int)(((unsigned long long)b >> 52) & 0x7FFull) + e;  // biased exponent of the result
    return (x == 0 || be <= 0) ? 0.0 : __longlong_as_double(b + ((long long)e << 52));
}

// The same value assembled with integer instructions only (round half away
// from zero on the dropped bits), for kernels whose FP64 pipe is already
// the busy one: the gradient sweep adds one double per column and step, and
// measured 16% slower with the FP64-pipe conversion.
__device__ __forceinline__ double fx_to_double_alu(long long x, int e) {
    const unsigned long long s = (unsigned long long)(x >> 63);
    const unsigned long long m = ((unsigned long long)x ^ s) - s;
    const int lz = __clzll((long long)m);
    const unsigned long long mn = m << (lz & 63);
    // x 2^e = (mn / 2^63) 2^(63 - lz + e): biased exponent be = 1086 - lz + e;
    // the leading mantissa bit (bit 52 of mn >> 11) adds the last 1
    const int be = 1086 - lz + e;
    unsigned long long bits = ((unsigned long long)(be - 1) << 52) + (mn >> 11);
    bits += (mn >> 10) & 1ull;
    bits |= s & 0x8000000000000000ull;
    return (m == 0ull || be <= 0) ? 0.0 : __longlong_as_double((long long)bits);
}

__device__ __forceinline__ fxl shfl_xor_fxl(const fxl& v, int lanemask) {
    return fxl{__shfl_xor_sync(0xffffffffu, v.rh, lanemask), __shfl_xor_sync(0xffffffffu, v.rl, lanemask),
               __shfl_xor_sync(0xffffffffu, v.ih, lanemask), __shfl_xor_sync(0xffffffffu, v.il, lanemask)};
}

}  // namespace gbperm
