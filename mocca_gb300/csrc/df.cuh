// df.cuh -- double-float arithmetic for the mixed-precision kernels.
//
// A value is carried as the unevaluated sum hi + lo of two floats (48
// significant bits).  Products use the exact FMA residual (TwoProduct) and
// sums Knuth's TwoSum (Dekker 1971, "A floating-point technique for
// extending the available precision", Numer. Math. 18; Knuth, TAOCP vol. 2,
// 4.2.2).  GB300 issues FP32 at ~70x its FP64 rate, so a double-float
// operation (~10-20 FP32 instructions) is several times cheaper than one FP64
// operation while keeping ~1e-14 relative accuracy.  The rounded products and
// the TwoSum steps use the _rn intrinsics so that the compiler cannot fuse
// them into FMAs, which would change the roundings the error terms rely on.
#pragma once

#include <cuda_runtime.h>

namespace mg {

struct dfl {
    float h, l;
};

__device__ __forceinline__ dfl df_from(double x) {
    const float h = (float)x;
    return dfl{h, (float)(x - (double)h)};
}

__device__ __forceinline__ double df_to(dfl a) { return (double)a.h + (double)a.l; }

// float -> double by bit moves (normal floats; zero and subnormals give 0):
// no FP64-pipe conversion
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    if (e == 0u) return 0.0;
    const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    const unsigned lo = u << 29;
    return __hiloint2double((int)hi, (int)lo);
}

// double-float -> FP64 with one FP64 add (parts below 2^-126 are dropped)
__device__ __forceinline__ double df_to_fast(dfl a) { return f2d_bits(a.h) + f2d_bits(a.l); }

// FP64 -> double-float with integer instructions only.  FP64 adds and the
// FP64 <-> FP32 conversions issue at the (low) FP64 rate on GB300, so the hot
// loops split their FP64 inputs from the bit pattern: hi keeps the sign, the
// exponent and the leading 23 mantissa bits (truncated), lo is the remaining
// 29 bits converted with one integer-to-float conversion and scaled by an
// exact power of two.  hi + lo equals x to 2^-47 relative.  |x| below 2^-126
// gives 0 and lo is dropped below |x| ~ 2^-74 (far below the grid values);
// inf and nan keep their class in hi.
__device__ __forceinline__ dfl df_split(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(b >> 32);
    const int e = (int)((hw >> 20) & 0x7ffu) - 1023;   // unbiased exponent
    if (e < -126) return dfl{0.0f, 0.0f};
    if (e > 127) return dfl{(float)x, 0.0f};   // inf / nan / out of float range
    const unsigned sign = hw & 0x80000000u;
    const unsigned mant23 = (unsigned)((b >> 29) & 0x7fffffu);
    const float h = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | mant23);
    const unsigned rem = (unsigned)(b & 0x1fffffffu);
    float l = 0.0f;
    if (e - 52 + 127 >= 1) {
        const float scale = __uint_as_float(sign | ((unsigned)(e - 52 + 127) << 23));
        l = __fmul_rn(__uint2float_rn(rem), scale);
    }
    return dfl{h, l};
}

// a stored double-float value (float2 {hi, lo} in memory)
__device__ __forceinline__ dfl df_ld(const float2* p) {
    const float2 v = *p;
    return dfl{v.x, v.y};
}

__device__ __forceinline__ void df_st(float2* p, dfl a) { *p = make_float2(a.h, a.l); }

__device__ __forceinline__ dfl df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
    return dfl{s, e};
}

// renormalise so that |lo| <= ulp(hi) / 2 (Fast2Sum, |hi| >= |lo|)
__device__ __forceinline__ dfl df_norm(dfl a) {
    const float s = __fadd_rn(a.h, a.l);
    return dfl{s, __fsub_rn(a.l, __fsub_rn(s, a.h))};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
    dfl s = df_two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return df_norm(s);
}

__device__ __forceinline__ dfl df_neg(dfl a) { return dfl{-a.h, -a.l}; }

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return df_norm(dfl{p, e});
}

// a * b + c
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    dfl s = df_two_sum(p, c.h);
    s.l += e + c.l;
    return df_norm(s);
}

// accumulate a * b into an unnormalised running sum (sh, sl): the lo part
// collects the rounding errors and is folded in once at the end (df_to)
__device__ __forceinline__ void df_acc(float& sh, float& sl, dfl a, dfl b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    const dfl s = df_two_sum(sh, p);
    sh = s.h;
    sl += s.l + e;
}

}  // namespace mg
