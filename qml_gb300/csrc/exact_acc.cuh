// Exact sums of FP64 products in 256-bit fixed point, on the integer pipes.
//
// An accumulator holds a two's-complement integer l (four 64-bit limbs) and a frame
// f: its value is l * 2^f.  A product u*v of doubles is formed exactly from the
// 53-bit significands (64 x 64 -> 128-bit multiply) and added at its exponent.  The
// frame is kept ACC_HEAD bits below the largest product seen, so a product lands at
// bit s = E - f <= ACC_HEAD (E its exponent, value < 2^(E+106)) and up to 2^17
// products fit below bit 255.  When a larger product arrives the frame rises and
// the accumulator is shifted right: only bits 2^-132 below the largest term are ever
// dropped, so the sum is exact to far beyond FP64 and does not depend on the order
// of the additions.  Rounding to FP64 happens once, at the end (nearest, ties to
// even).  No FP64 instruction is used.
#pragma once

#include <cstdint>

namespace qmlg {

constexpr int ACC_HEAD = 132;
constexpr int ACC_EMPTY = -(1 << 30);

struct Acc {
    unsigned long long l0, l1, l2, l3;
    int f;
    int bad;  // a non-finite input was seen
};

__device__ __forceinline__ void acc_init(Acc &a)
{
    a.l0 = a.l1 = a.l2 = a.l3 = 0ull;
    a.f = ACC_EMPTY;
    a.bad = 0;
}

__device__ __forceinline__ void acc_addc(Acc &a, unsigned long long x0, unsigned long long x1,
                                         unsigned long long x2, unsigned long long x3)
{
    asm("add.cc.u64 %0, %0, %4;\n\t"
        "addc.cc.u64 %1, %1, %5;\n\t"
        "addc.cc.u64 %2, %2, %6;\n\t"
        "addc.u64 %3, %3, %7;"
        : "+l"(a.l0), "+l"(a.l1), "+l"(a.l2), "+l"(a.l3)
        : "l"(x0), "l"(x1), "l"(x2), "l"(x3));
}

__device__ __forceinline__ void acc_subc(Acc &a, unsigned long long x0, unsigned long long x1,
                                         unsigned long long x2, unsigned long long x3)
{
    asm("sub.cc.u64 %0, %0, %4;\n\t"
        "subc.cc.u64 %1, %1, %5;\n\t"
        "subc.cc.u64 %2, %2, %6;\n\t"
        "subc.u64 %3, %3, %7;"
        : "+l"(a.l0), "+l"(a.l1), "+l"(a.l2), "+l"(a.l3)
        : "l"(x0), "l"(x1), "l"(x2), "l"(x3));
}

// Arithmetic right shift of the 256-bit integer by k >= 0.
__device__ __forceinline__ void acc_sar(Acc &a, int k)
{
    if (k <= 0) return;
    const unsigned long long sg = (unsigned long long)((long long)a.l3 >> 63);
    if (k >= 256) {
        a.l0 = a.l1 = a.l2 = a.l3 = sg;
        return;
    }
    const int w = k >> 6, b = k & 63;
#pragma unroll
    for (int t = 0; t < 3; ++t)
        if (w > t) {
            a.l0 = a.l1;
            a.l1 = a.l2;
            a.l2 = a.l3;
            a.l3 = sg;
        }
    if (b) {
        a.l0 = (a.l0 >> b) | (a.l1 << (64 - b));
        a.l1 = (a.l1 >> b) | (a.l2 << (64 - b));
        a.l2 = (a.l2 >> b) | (a.l3 << (64 - b));
        a.l3 = (unsigned long long)((long long)a.l3 >> b);
    }
}

// Moves the frame up to nf (no-op if it is already there).
__device__ __forceinline__ void acc_raise(Acc &a, int nf)
{
    if (nf <= a.f) return;
    if (a.f != ACC_EMPTY) acc_sar(a, nf - a.f);
    a.f = nf;
}

// Adds (neg ? -1 : 1) * (hi:lo) * 2^E, (hi:lo) < 2^106.
__device__ __forceinline__ void acc_add_mag(Acc &a, unsigned long long hi, unsigned long long lo,
                                            int E, bool neg)
{
    if ((hi | lo) == 0ull) return;
    if (E - a.f > ACC_HEAD) acc_raise(a, E - ACC_HEAD);
    int s = E - a.f;
    if (s < 0) {
        // below the frame: the low bits are dropped
        if (s <= -128) return;
        const int k = -s;
        if (k >= 64) {
            lo = hi >> (k - 64);
            hi = 0ull;
        } else {
            lo = (lo >> k) | (hi << (64 - k));
            hi >>= k;
        }
        s = 0;
    }
    const int w = s >> 6, b = s & 63;  // w <= 2 since s <= ACC_HEAD
    const unsigned long long t0 = lo << b;
    const unsigned long long t1 = b ? ((hi << b) | (lo >> (64 - b))) : hi;
    const unsigned long long t2 = b ? (hi >> (64 - b)) : 0ull;
    const unsigned long long x0 = w == 0 ? t0 : 0ull;
    const unsigned long long x1 = w == 0 ? t1 : (w == 1 ? t0 : 0ull);
    const unsigned long long x2 = w == 0 ? t2 : (w == 1 ? t1 : t0);
    const unsigned long long x3 = w == 0 ? 0ull : (w == 1 ? t2 : t1);
    if (neg) acc_subc(a, x0, x1, x2, x3);
    else acc_addc(a, x0, x1, x2, x3);
}

// The common case of acc_add_mag, with no branch but the sign: a product that lands
// inside the frame (0 <= s <= ACC_HEAD).  Anything else (the first product, one
// above the head or below the frame, a zero) takes acc_add_mag.
__device__ __forceinline__ void acc_add_mag_fast(Acc &a, unsigned long long hi, unsigned long long lo,
                                                 int E, bool neg)
{
    const int s = E - a.f;
    if (s < 0 || s > ACC_HEAD) {
        acc_add_mag(a, hi, lo, E, neg);
        return;
    }
    // (hi:lo) << s in 32-bit words: a funnel shift by b = s mod 32 gives five words
    // q0..q4, which then move up by h = (s >> 5) & 1 words and w = s >> 6 limbs (w <= 2)
    const int b = s & 31, h = (s >> 5) & 1, w = s >> 6;
    const uint32_t p0 = (uint32_t)lo, p1 = (uint32_t)(lo >> 32), p2 = (uint32_t)hi,
                   p3 = (uint32_t)(hi >> 32);
    const uint32_t q0 = p0 << b, q1 = __funnelshift_l(p0, p1, b), q2 = __funnelshift_l(p1, p2, b),
                   q3 = __funnelshift_l(p2, p3, b), q4 = __funnelshift_l(p3, 0u, b);
    // three limbs t0, t1, t2 of (hi:lo) << (s mod 64)
    const unsigned long long t0 = h ? ((unsigned long long)q0 << 32) : (((unsigned long long)q1 << 32) | q0);
    const unsigned long long t1 = h ? (((unsigned long long)q2 << 32) | q1) : (((unsigned long long)q3 << 32) | q2);
    const unsigned long long t2 = h ? (((unsigned long long)q4 << 32) | q3) : (unsigned long long)q4;
    const unsigned long long x0 = w == 0 ? t0 : 0ull;
    const unsigned long long x1 = w == 0 ? t1 : (w == 1 ? t0 : 0ull);
    const unsigned long long x2 = w == 0 ? t2 : (w == 1 ? t1 : t0);
    const unsigned long long x3 = w == 0 ? 0ull : (w == 1 ? t2 : t1);
    if (neg) acc_subc(a, x0, x1, x2, x3);
    else acc_addc(a, x0, x1, x2, x3);
}

// The 106-bit product of two significands below 2^53, each given as its low 32 bits
// and its high 21: four 32 x 32 -> 64-bit multiplies; hi < 2^43.
__device__ __forceinline__ void mul53(uint32_t alo, uint32_t ahi, uint32_t blo, uint32_t bhi,
                                      unsigned long long &hi, unsigned long long &lo)
{
    const unsigned long long p00 = (unsigned long long)alo * blo;
    unsigned long long mid = (unsigned long long)ahi * blo + (p00 >> 32);  // < 2^53 + 2^32
    mid += (unsigned long long)alo * bhi;                                  // < 2^54 + 2^32
    hi = (unsigned long long)ahi * bhi + (mid >> 32);
    lo = (mid << 32) | (p00 & 0xffffffffull);
}

// Significand (with the hidden bit) and exponent: v = m * 2^e.
__device__ __forceinline__ void dbl_split(double v, unsigned long long &m, int &e, bool &neg,
                                          int &bad)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int ef = (int)((u >> 52) & 0x7ff);
    m = u & 0xfffffffffffffull;
    if (ef) m |= 0x10000000000000ull;
    e = (ef ? ef : 1) - 1075;
    neg = (u >> 63) != 0ull;
    if (ef == 0x7ff) bad = 1;
}

// a += (negate ? -1 : 1) * u * v, exactly.
__device__ __forceinline__ void acc_add_prod(Acc &a, double u, double v, bool negate = false)
{
    unsigned long long mu, mv;
    int eu, ev;
    bool nu, nv;
    dbl_split(u, mu, eu, nu, a.bad);
    dbl_split(v, mv, ev, nv, a.bad);
    acc_add_mag(a, __umul64hi(mu, mv), mu * mv, eu + ev, (nu != nv) != negate);
}

// a += (negate ? -1 : 1) * b  (frames aligned to the larger one).
__device__ __forceinline__ void acc_add_acc(Acc &a, Acc b, bool negate = false)
{
    a.bad |= b.bad;
    if (b.f == ACC_EMPTY) return;
    if (a.f == ACC_EMPTY) {
        a.l0 = a.l1 = a.l2 = a.l3 = 0ull;
        a.f = b.f;
    }
    if (b.f > a.f) acc_raise(a, b.f);
    else acc_sar(b, a.f - b.f);
    if (negate) acc_subc(a, b.l0, b.l1, b.l2, b.l3);
    else acc_addc(a, b.l0, b.l1, b.l2, b.l3);
}

// The value rounded to FP64 (nearest, ties to even).
__device__ __forceinline__ double acc_to_double(Acc a)
{
    if (a.bad) return __longlong_as_double(0x7ff8000000000000ll);
    if (a.f == ACC_EMPTY) return 0.0;
    const bool neg = (long long)a.l3 < 0;
    if (neg) {
        Acc z;
        acc_init(z);
        z.f = a.f;
        acc_subc(z, a.l0, a.l1, a.l2, a.l3);
        a = z;
    }
    int h;  // top set bit
    if (a.l3) h = 255 - __clzll((long long)a.l3);
    else if (a.l2) h = 191 - __clzll((long long)a.l2);
    else if (a.l1) h = 127 - __clzll((long long)a.l1);
    else if (a.l0) h = 63 - __clzll((long long)a.l0);
    else return 0.0;
    // 64-bit window of bits [h-63, h] and whether any bit below it is set
    unsigned long long win, sticky = 0ull;
    const int sh = h - 63;
    if (sh <= 0) {
        win = a.l0 << (-sh);
    } else {
        const int q = sh >> 6, b = sh & 63;
        const unsigned long long L0 = q == 0 ? a.l0 : (q == 1 ? a.l1 : (q == 2 ? a.l2 : a.l3));
        const unsigned long long L1 = q == 0 ? a.l1 : (q == 1 ? a.l2 : (q == 2 ? a.l3 : 0ull));
        win = b ? ((L0 >> b) | (L1 << (64 - b))) : L0;
        sticky = b ? (L0 & ((1ull << b) - 1ull)) : 0ull;
        if (q >= 1) sticky |= a.l0;
        if (q >= 2) sticky |= a.l1;
        if (q >= 3) sticky |= a.l2;
    }
    unsigned long long m = win >> 11;  // 53 bits
    const unsigned long long rest = win & 0x7ffull;
    if (rest > 0x400ull || (rest == 0x400ull && (sticky != 0ull || (m & 1ull)))) ++m;
    int E = a.f + sh + 11;  // value = m * 2^E
    if (m == (1ull << 53)) {
        m >>= 1;
        ++E;
    }
    const int field = E + 52 + 1023;
    if (field >= 0x7ff) return neg ? -INFINITY : INFINITY;
    if (field <= 0) {
        const double v = ldexp((double)m, E);  // subnormal range (rare)
        return neg ? -v : v;
    }
    const unsigned long long bits = ((unsigned long long)(neg ? 1 : 0) << 63) |
                                    ((unsigned long long)field << 52) | (m & 0xfffffffffffffull);
    return __longlong_as_double((long long)bits);
}

}  // namespace qmlg
