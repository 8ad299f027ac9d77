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

}  // namespace gbperm
