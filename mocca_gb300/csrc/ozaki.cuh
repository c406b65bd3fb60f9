// ozaki.cuh -- exact-digit BF16 products on the tcgen05 tensor cores.
//
// An FP64 operand row (a grid line, a spinor chunk, a point's spinor values,
// a matrix row) is scaled by a power of two chosen from its largest exponent
// and rounded to a signed integer of 47 bits, then written as six balanced
// base-256 digits (|d| <= 128), each exact in BF16.  Digit a is stored
// pre-scaled by 2^(-8a), so the product of digit a of one row and digit b of
// another carries its weight 2^(-8(a+b)) by itself.  Products are exact in
// FP32; sums of up to 2^8 products of one weight stay below 2^22 and are
// exact too.  Pairs of weight 0, 1 and 2 go to three accumulators that stay
// exact; all pairs of weight 3..5 share a fourth, whose FP32 rounding sits
// near 2^-48 of the result; pairs of weight 6 and above (below 2^-48) are
// dropped.  The epilogue adds the four accumulators as a double-float and
// multiplies by the two powers of two: 2^(E_row + E_col - 12), E being the
// exponent of each row's largest entry (2^E <= max < 2^(E+1)).
//
// After Ozaki, Ogita, Oishi, Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication", Numer.
// Algorithms 59 (2012), with integer digits as in Ootomo, Ozaki, Yokota,
// "DGEMM on integer matrix multiplication unit", IJHPCA 2024.
#pragma once

#include <stdint.h>

#include <cmath>
#include <cstring>

#include "df.cuh"
#include "tc.cuh"

namespace mg {
namespace oz {

constexpr int kDigits = 6;                       // digits per operand entry
constexpr int kCmax = 5;                         // largest kept digit weight a + b
constexpr long long kDigitBias = 0x8080808080LL; // 128 in each of the five lower digits
constexpr int kPairs = 21;                       // pairs with a + b <= kCmax
constexpr uint32_t kAccs = 4;                    // accumulators per output

// float bit pattern of (u - 128) * 2^(-8A) for byte u of w, selected by sel
template <int A>
__device__ __forceinline__ uint32_t low_digit(uint32_t w, uint32_t sel) {
    constexpr uint32_t ebits = (uint32_t)(150 - 8 * A) << 23;   // 2^(23-8A), even exponent
    constexpr float off = (float)(8388608.0 + 128.0) * (1.0f / (float)(1ull << (8 * A)));
    const float f = __uint_as_float(__byte_perm(w, ebits, sel)) - off;
    return __float_as_uint(f);
}

// Biased exponent field of an FP64 value (0 for zero and subnormals).
__device__ __forceinline__ int bexp(double v) {
    return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7FF);
}

// round(v * 2^f) for a row whose largest biased exponent is emax, with
// f = 8 kDigits - 2 - (emax - 1023): |result| <= 2^47.  Zero and subnormal v
// give 0, as do values 2^62 below the row's largest.
__device__ __forceinline__ long long fixed(double v, int emax) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    const int sh = (54 - 8 * kDigits) + (emax - e);   // >= 6
    long long X = 0;
    if (e != 0 && sh < 62) {
        const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        X = (long long)((m + (1ull << (sh - 1))) >> sh);
        if (b >> 63) X = -X;
    }
    return X;
}

// The same fixed-point value of a float (part of a double-float), exact when
// the float's bits lie above 2^-f, rounded otherwise.
__device__ __forceinline__ long long fixed_f(float v, int emax) {
    const uint32_t u = __float_as_uint(v);
    const int ef = (int)((u >> 23) & 0xFFu);
    if (ef == 0) return 0;
    const long long m = (long long)((u & 0x7FFFFFu) | 0x800000u);
    // v * 2^f = m * 2^sh with f = 8 kDigits - 2 - (emax - 1023)
    const int sh = ef - 150 + (8 * kDigits - 2) - (emax - 1023);
    long long X;
    if (sh >= 0) X = sh < 39 ? (m << sh) : 0;   // above the row bound: not reached
    else if (sh > -40) X = (m + (1ll << (-sh - 1))) >> (-sh);
    else X = 0;
    return (u >> 31) ? -X : X;
}

// The pre-scaled digits (top digit first) of a fixed-point value X
// (|X| <= 2^47), as FP32 bit patterns whose upper halves are the exact BF16
// values.
__device__ __forceinline__ void digits_fixed(long long X, uint32_t (&d)[kDigits]) {
    const unsigned long long Y = (unsigned long long)(X + kDigitBias);
    const uint32_t ylo = (uint32_t)Y, yhi = (uint32_t)(Y >> 32);
    const int top = (int)yhi >> 8;   // Y >> 40 (arithmetic), in [-128, 128]
    d[0] = __float_as_uint(__int_as_float(0x4B400000 + top) - 12582912.0f);
    // digit a (a = 1..5) is byte (5 - a) of Y, biased by 128
    d[1] = low_digit<1>(yhi, 0x7540);
    d[2] = low_digit<2>(ylo, 0x7543);
    d[3] = low_digit<3>(ylo, 0x7542);
    d[4] = low_digit<4>(ylo, 0x7541);
    d[5] = low_digit<5>(ylo, 0x7540);
}

// The pre-scaled digits of v (top digit first) for a row whose largest
// biased exponent is emax.
__device__ __forceinline__ void digits(double v, int emax, uint32_t (&d)[kDigits]) {
    digits_fixed(fixed(v, emax), d);
}

// Digits of 8 fixed-point values of a row as one 16-byte core-matrix row per
// digit plane.
__device__ __forceinline__ void digits8_fixed(const long long (&X)[8], uint4 (&w)[kDigits]) {
    uint32_t x[kDigits][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        uint32_t d0[kDigits], d1[kDigits];
        digits_fixed(X[2 * h], d0);
        digits_fixed(X[2 * h + 1], d1);
#pragma unroll
        for (int a = 0; a < kDigits; ++a) x[a][h] = __byte_perm(d0[a], d1[a], 0x7632);
    }
#pragma unroll
    for (int a = 0; a < kDigits; ++a) w[a] = make_uint4(x[a][0], x[a][1], x[a][2], x[a][3]);
}

// Digits of 8 consecutive values of a row, packed as one 16-byte core-matrix
// row per digit plane.
__device__ __forceinline__ void digits8(const double (&v)[8], int emax, uint4 (&w)[kDigits]) {
    uint32_t x[kDigits][4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        uint32_t d0[kDigits], d1[kDigits];
        digits(v[2 * h], emax, d0);
        digits(v[2 * h + 1], emax, d1);
#pragma unroll
        for (int a = 0; a < kDigits; ++a) x[a][h] = __byte_perm(d0[a], d1[a], 0x7632);
    }
#pragma unroll
    for (int a = 0; a < kDigits; ++a) w[a] = make_uint4(x[a][0], x[a][1], x[a][2], x[a][3]);
}

// a0 + a1 + a2 + a3 as a normalised double-float.  a0 is an integer below
// 2^22, a1 a multiple of 2^-8 below 2^15, a2 a multiple of 2^-16 below 2^8
// (all exact); a3 is the small rounded remainder.  With a1 = i1 + f1
// (integer and fractional parts), a0 + i1 and f1 + a2 are exact float sums;
// one TwoSum of those two is exact, and a3 joins the low part before the
// final renormalisation (it is far below the high part).
__device__ __forceinline__ dfl combine4(float a0, float a1, float a2, float a3) {
    const float i1 = truncf(a1);
    const float f1 = __fsub_rn(a1, i1);
    const dfl s = df_two_sum(__fadd_rn(a0, i1), __fadd_rn(f1, a2));
    return df_norm(dfl{s.h, __fadd_rn(s.l, a3)});
}

// 2^x as a float for -126 <= x <= 127, 0 below (values under 2^-126 are
// dropped; they are far below the grid values)
__device__ __forceinline__ float pow2f(int x) {
    return x < -126 ? 0.0f : __int_as_float((min(x, 127) + 127) << 23);
}

// Issue the kPairs digit-pair MMAs of one K stage: A planes at aBase +
// a * aPlane, B planes at bBase + b * bPlane, KSTEPS MMAs of K = 16 each,
// accumulators at tmem + g * N (g = min(a + b, 3)).  accumulate: the first
// MMA of each accumulator adds to what it holds (later K stages).
template <int KSTEPS>
__device__ __forceinline__ void issue_pairs(uint32_t tmem, int N, uint32_t idesc, uint32_t aBase,
                                            uint32_t aPlane, uint32_t aSbo, uint32_t bBase,
                                            uint32_t bPlane, uint32_t bSbo, bool accumulate) {
    bool started[4] = {accumulate, accumulate, accumulate, accumulate};
#pragma unroll
    for (int c = 0; c <= kCmax; ++c) {
        const int g = c < 3 ? c : 3;
#pragma unroll
        for (int a = 0; a < kDigits; ++a) {
            const int b = c - a;
            if (b < 0 || b >= kDigits) continue;
#pragma unroll
            for (int ks = 0; ks < KSTEPS; ++ks) {
                tc::mma_bf16(tmem + (uint32_t)(g * N),
                             tc::desc_sbo(aBase + a * aPlane + ks * tc::kKStep, aSbo),
                             tc::desc_sbo(bBase + b * bPlane + ks * tc::kKStep, bSbo), idesc,
                             started[g] ? 1u : 0u);
                started[g] = true;
            }
        }
    }
}

// Host form of the digits: BF16 bit patterns of the pre-scaled digits of
// round(x * 2^g), top first.
inline void host_digits(double x, int g, uint16_t* out) {
    const long long X = std::llrint(std::ldexp(x, g));
    const long long Y = X + kDigitBias;
    for (int b = kDigits - 1; b >= 1; --b) {
        const int j = kDigits - 1 - b;   // byte position
        const int d = (int)((Y >> (8 * j)) & 0xFF) - 128;
        const float f = std::ldexp((float)d, -8 * b);
        uint32_t u;
        std::memcpy(&u, &f, 4);
        out[b] = (uint16_t)(u >> 16);
    }
    const float f = (float)(Y >> (8 * (kDigits - 1)));
    uint32_t u;
    std::memcpy(&u, &f, 4);
    out[0] = (uint16_t)(u >> 16);
}

// The power g = 8 kDigits - 2 - E used for a row whose largest |entry| is mx,
// and E itself (0 for an all-zero row).
inline int host_row_exponent(double mx) {
    if (!(mx > 0.0)) return 0;
    int fe;
    std::frexp(mx, &fe);   // mx = f * 2^fe, 0.5 <= f < 1
    return fe - 1;
}

}  // namespace oz
}  // namespace mg
