// 1/sqrt(p) for p > 0 without an FP64 square root or division.  An FP64
// instruction holds its scheduler's FP64 pipe for about 64 cycles, and sqrt or
// division take about ten times that; this takes five FP64 instructions.
#pragma once

#include <cstdint>

namespace {

// FP32 rsqrtf of p's leading bits gives ~23 bits, and one Halley step (cubic
// convergence for f(y) = 1/y^2 - p) brings it to full FP64 precision:
//   e = 1 - p y^2,  y <- y + y e (1/2 + 3/8 e).
// The FP32 <-> FP64 moves are done on the bits.  Outside [2^-120, 2^120] p is first
// scaled by an even power of two into [1, 4).
__device__ __forceinline__ double rsqrt_halley(double p)
{
    double q = p;
    int h = 0;
    const int ed = (int)((unsigned long long)__double_as_longlong(p) >> 52);
    if (ed < 1023 - 120 || ed > 1023 + 120) {
        const int ex = ilogb(p) & ~1;
        q = scalbn(p, -ex);
        h = -ex / 2;
    }
    const unsigned long long qb = (unsigned long long)__double_as_longlong(q);
    // q truncated to FP32: exponent rebiased from 1023 to 127, top 23 mantissa bits
    const uint32_t fb = (uint32_t)(((qb >> 52) - 896ull) << 23) | (uint32_t)((qb >> 29) & 0x7fffffull);
    const uint32_t yb = __float_as_uint(rsqrtf(__uint_as_float(fb)));
    // the FP32 estimate (a normal positive float) as an exact double
    double y = __longlong_as_double((long long)((((unsigned long long)(yb >> 23) + 896ull) << 52) |
                                                ((unsigned long long)(yb & 0x7fffffu) << 29)));
    const double e = fma(-q * y, y, 1.0);
    y = fma(y * e, fma(0.375, e, 0.5), y);
    return h != 0 ? scalbn(y, h) : y;
}

}  // namespace
