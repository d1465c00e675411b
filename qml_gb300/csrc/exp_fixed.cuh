// exp(x) for x <= 0 in 64-bit fixed point, for the tensor-core Gaussian epilogues.
#pragma once

#include <cstdint>

#include "exp2_table.cuh"

namespace {

// exp(x) for the Gaussian epilogues, x <= 0 after clamping, by table-driven reduction
// (P. T. P. Tang, "Table-driven implementation of the exponential function in IEEE
// floating-point arithmetic", ACM TOMS 15(2), 1989) carried out in 64-bit fixed
// point, because FP64 instructions cost ~64 cycles of a scheduler's FP64 pipe on this
// GPU and the integer ones one or two:
//   |x| = (256 n + j) ln2/256 - r,  exp(x) = 2^-n 2^(-j/256) e^r,  |r| <= ln2/512.
// - X = |x| 2^53 exactly from x's bits (truncated below 2^-53; |x| < 700 so X < 2^63);
//   k = 256 n + j = round(|x| 256/ln2) from the high word of X (256/ln2 2^54).
// - r = k ln2/256 - |x| in 128 bits (ln2/256 to 2^-116), then to 2^-63.
// - e^r = 1 + r + r^2/2 + c: r^2 from one 64 x 64 multiply, c = r^3/6 + r^4/24 in FP32
//   (|c| < 4.2e-10, FP32's error on it below 3e-17), all summed in units of 2^-62.
// - 2^(-j/256) from a table in units of 2^-63; the 61-bit product is rounded once to
//   53 bits (nearest, ties to even) and 2^-n goes into the exponent bits.
// Against the host libm over 4M points per range of [-700, 0], [-1, 0], [-1e-3, 0],
// [-5, -4] and [-700, -600]: at most 2 ulp, 94% identical away from 0.  x > 0 (and
// +NaN) is clamped to 0, as the distance formula can round slightly above it;
// x <= -700 and -NaN go to the library exp.
__device__ __forceinline__ double exp_nonpos(double x)
{
    const long long xs = __double_as_longlong(x);
    if (xs >= 0) return 1.0;
    if ((unsigned long long)xs >= 0xC085E00000000000ull) return exp(x);  // bits of -700.0
    const unsigned long long u = (unsigned long long)xs & 0x7fffffffffffffffull;
    const int sh = (int)(u >> 52) - 1022;  // X = |x| 2^53 = m 2^sh
    const unsigned long long m = (u & 0xfffffffffffffull) | 0x10000000000000ull;
    const unsigned long long X = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> (-sh)) : 0ull);
    const unsigned int k = (unsigned int)((__umul64hi(X, kExpK256Q54) + (1ull << 42)) >> 43);
    // R = k ln2/256 - |x| in units of 2^-116: k L - X 2^63, two words
    const unsigned long long plo = (unsigned long long)k * kExpL256Lo, xlo = X << 63;
    const unsigned long long phi = __umul64hi((unsigned long long)k, kExpL256Lo) +
                                   (unsigned long long)k * kExpL256Hi;
    const unsigned long long rhi = phi - (X >> 1) - (plo < xlo ? 1ull : 0ull);
    const long long r = (long long)((rhi << 11) | ((plo - xlo) >> 53));  // units of 2^-63
    const long long r2 = __mul64hi(r, r);                                // r^2, 2^-62
    const float rf = __int2float_rn((int)(r >> 24)) * 1.8189894035458565e-12f;  // 2^-39
    const float c = rf * rf * rf * __fmaf_rn(rf, 1.0f / 24.0f, 1.0f / 6.0f);
    const long long p = (1ll << 62) + (r >> 1) + (r2 >> 1) +
                        (long long)__float2int_rn(c * 4.611686018427388e18f);  // e^r, 2^-62
    const unsigned long long V = __umul64hi(kExp2NegQ63[k & 255], (unsigned long long)p);
    const int lz = __clzll((long long)V);
    const unsigned long long W = V << lz;
    const unsigned int rem = (unsigned int)(W & 0x7ffull);
    unsigned long long mant = W >> 11;
    mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    // value = mant 2^-52 2^(2 - lz - n); mant's leading bit carries into the exponent
    return __longlong_as_double((long long)(((unsigned long long)(1024 - lz - (int)(k >> 8)) << 52) + mant));
}

}  // namespace
