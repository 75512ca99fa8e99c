// xdem_df.cuh -- FP32-pipe helpers of the mixed-precision step.
//
// GB300 issues FP64 arithmetic and FP64<->FP32 conversions at about 1/64 of
// its FP32 rate, so the mixed form keeps exactly one kind of FP64 operation
// in its per-sphere work: the addition of an FP32 increment to an FP64 state
// value.  Everything else that needs more than FP32 precision is done here
// with integer bit operations (conversions, splits) or with unevaluated
// float pairs ("double-float", hi + lo, about 48 significant bits; the
// error-free transformations are Knuth's TwoSum, Dekker's FastTwoSum and the
// FMA-based TwoProduct).
//
// Conventions of the conversions below: finite inputs below the FP32 normal
// range flush to a signed zero, results beyond FLT_MAX give an infinity,
// NaN stays NaN.
#pragma once

#include <cuda_runtime.h>

namespace xdem {

// ---------------------------------------------------------------- conversions
// double -> float, round to nearest even, on the integer pipes.  In the
// FP32 normal range the exponent is rebiased on the high word (the bias has
// no low-word bits) and the 29 dropped mantissa bits are rounded by adding
// 0x0fffffff plus the lowest kept bit, so that a halfway case rounds to
// even; a carry runs on into the exponent, reaching 0x7f800000 (infinity)
// past FLT_MAX.  Two compares of the high word pick the flushed zero, the
// overflow infinity and NaN.
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
    const unsigned int sign = hi & 0x80000000u;
    const unsigned int ah = hi & 0x7fffffffu;  // high word of |x|
    const unsigned long long t = ((unsigned long long)(ah - (896u << 20)) << 32) | lo;
    unsigned int r = (unsigned int)((t + 0x0fffffffull + ((lo >> 29) & 1u)) >> 29);
    r = ah < (897u << 20) ? 0u : r;           // below FLT_MIN: a signed zero
    r = ah >= (1151u << 20) ? 0x7f800000u : r;  // beyond FLT_MAX, infinity
    r = (ah > 0x7ff00000u || (ah == 0x7ff00000u && lo != 0u)) ? 0x7fc00000u : r;  // NaN
    return __uint_as_float(sign | r);
}

// float -> double, exact, on the integer pipes.
__device__ __forceinline__ double f2d(float f)
{
    const unsigned int u = __float_as_uint(f);
    const unsigned int sign = u & 0x80000000u;
    int e = (int)((u >> 23) & 0xffu);
    unsigned int m = u & 0x7fffffu;
    if (e == 0) {
        if (m == 0u) return __hiloint2double((int)sign, 0);
        const int s = __clz(m) - 8;  // normalise a subnormal: bit 23 becomes the leading one
        m = (m << s) & 0x7fffffu;
        e = 1 - s;
    }
    const unsigned int de = e == 255 ? 0x7ffu : (unsigned int)(e + 896);
    return __hiloint2double((int)(sign | (de << 20) | (m >> 3)), (int)(m << 29));
}

// ---------------------------------------------------------------- float pairs
struct df { float hi, lo; };

__device__ __forceinline__ df two_sum(float a, float b)
{
    const float s = a + b;
    const float bp = s - a;
    return df{s, (a - (s - bp)) + (b - bp)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b)  // |a| >= |b|
{
    const float s = a + b;
    return df{s, b - (s - a)};
}
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = a * b;
    return df{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ float df_f(df a) { return a.hi + a.lo; }
__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_add(df a, df b)
{
    const df s = two_sum(a.hi, b.hi);
    const df t = two_sum(a.lo, b.lo);
    df r = fast_two_sum(s.hi, s.lo + t.hi);
    return fast_two_sum(r.hi, r.lo + t.lo);
}
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b)
{
    const df s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, s.lo + a.lo);
}
__device__ __forceinline__ df df_mul(df a, df b)
{
    const df p = two_prod(a.hi, b.hi);
    return fast_two_sum(p.hi, p.lo + (a.hi * b.lo + a.lo * b.hi));
}
__device__ __forceinline__ df df_mul_f(df a, float b)
{
    const df p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// double -> (hi, lo) with hi the double truncated to 24 significant bits and
// lo the remainder truncated to 24 bits: |x - (hi + lo)| <= 2^-47 |x| for
// 2^-78 <= |x| < 2^127 (below that the remainder leaves the FP32 normal range
// and lo is 0).  Integer pipes only.  Doubles below the FP32 normal range
// give (0, 0).
__device__ __forceinline__ df split_d(double x)
{
    const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
    const unsigned int sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ffu);
    const int fe = e - 896;
    const unsigned int m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const bool nan = e == 0x7ff && ((hi & 0xfffffu) | lo);
    if (e == 0x7ff || fe >= 255) return df{__uint_as_float(sign | 0x7f800000u | (nan ? 0x400000u : 0u)), 0.f};
    if (fe <= 0) return df{__uint_as_float(sign), 0.f};
    const float h = __uint_as_float(sign | ((unsigned int)fe << 23) | m);
    const unsigned int rest = lo & 0x1fffffffu;  // value rest * 2^(e - 1075)
    if (rest == 0u) return df{h, 0.f};
    const int lz = __clz(rest);                    // >= 3
    const int le = (31 - lz) + e - 948;            // FP32 biased exponent of rest's leading bit
    if (le <= 0) return df{h, 0.f};
    const unsigned int mm = ((rest << lz) << 1) >> 9;  // 23 bits after the leading one
    return df{h, __uint_as_float(sign | ((unsigned int)le << 23) | mm)};
}

// ---------------------------------------------------------------- compensated sums
// Running FP32 sum with the rounding error of every addition kept (TwoSum):
// hi + lo carries about 48 significant bits.
struct CSum {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float b)
    {
        const float t = hi + b;
        const float bp = t - hi;
        lo += (hi - (t - bp)) + (b - bp);
        hi = t;
    }
    __device__ __forceinline__ void add(const CSum& o)
    {
        add(o.hi);
        lo += o.lo;
    }
    __device__ __forceinline__ float value() const { return hi + lo; }
};

}  // namespace xdem
