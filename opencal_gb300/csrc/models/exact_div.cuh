/*
 * exact_div.cuh -- IEEE-754 double division by a small positive integer
 * (1..9), correctly rounded to nearest-even, computed with integer
 * arithmetic on the significand; division by a fixed divisor through its
 * reciprocal with a provably exact correction; <= and > on the integer pipe.
 *
 * Why: the SCIDDICA-T and SCIARA-fv2 outflow computations divide a running
 * sum by the number of cells left in the minimisation (1..5 with the von
 * Neumann neighbourhood, 1..9 with Moore's).  On GB300 the FP64 pipe is
 * narrow (about 1/64 of the FP32/integer rate per SM), and a double
 * division expands into a sequence of several FP64 instructions; the integer
 * formulation below costs a few tens of full-rate integer instructions and
 * returns the same bits.
 *
 * Method (long division with round-half-even, no floating point):
 *   x = (-1)^s * M * 2^(E-52), M in [2^52, 2^53) for normal x.
 *   Choose t so that Q = floor(M * 2^t / c) lies in [2^53, 2^54): one bit
 *   beyond the 53 result bits.  The result significand is Q >> 1, the
 *   dropped bit is the round bit and a non-zero remainder (or a set round
 *   bit together with an odd result) decides rounding up.  Division of a
 *   64-bit integer by 3, 5, 7, 9 uses multiply-high identities (division by
 *   invariant integers, Granlund & Montgomery 1994):
 *     n / 3 = mulhi(n, 0xAAAAAAAAAAAAAAAB) >> 1      (all 64-bit n)
 *     n / 5 = mulhi(n, 0xCCCCCCCCCCCCCCCD) >> 2      (all 64-bit n)
 *     n / 7 = mulhi(n, ceil(2^66 / 7)) >> 2          (n < 2^66 / 6)
 *     n / 9 = mulhi(n, ceil(2^66 / 9)) >> 2          (n < 2^66 / 8)
 *   (here n < 2^58).  c = 1, 2, 4, 8 only change the exponent, and
 *   x / 6 = (x / 3) / 2 exactly (halving is exact away from underflow).
 * Zeros, subnormals, infinities, NaNs and results that would underflow take
 * the ordinary division (`x / c`), so every input is handled.
 * Tested against the division of the host and of the device on random and
 * edge-case inputs (tests/test_exact_div.py).
 */
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define CAL_HD __host__ __device__ __forceinline__
#else
#define CAL_HD static inline
#endif

CAL_HD uint64_t cal_mulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((unsigned __int128)a * (unsigned __int128)b) >> 64);
#endif
}

CAL_HD int64_t cal_d2i(double x)
{
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(x);
#else
    int64_t b;
    __builtin_memcpy(&b, &x, sizeof b);
    return b;
#endif
}

CAL_HD double cal_i2d(int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(b);
#else
    double x;
    __builtin_memcpy(&x, &b, sizeof x);
    return x;
#endif
}

/* x / c for c in 1..9, bit-identical to the IEEE quotient */
CAL_HD double cal_div_small(double x, int c)
{
    const int64_t bits = cal_d2i(x);
    const int64_t sign = bits & (int64_t)0x8000000000000000ULL;
    const int exp = (int)((bits >> 52) & 0x7ff);
    if (c == 1)
        return x;
    /* zero, subnormal, inf, nan, or exponent close to underflow: plain division */
    if (exp == 0 || exp == 0x7ff || exp < 8)
        return x / (double)c;
    if (c == 2 || c == 4 || c == 8) /* exact scaling: only the exponent changes */
        return cal_i2d(bits - ((int64_t)(c == 2 ? 1 : c == 4 ? 2 : 3) << 52));
    const int half = c == 6; /* x / 6 = (x / 3) / 2 */
    const int d = half ? 3 : c;
    const uint64_t M = ((uint64_t)bits & 0x000fffffffffffffULL) | 0x0010000000000000ULL; /* [2^52, 2^53) */
    /* shift t so that M*2^t/d lies in [2^53, 2^54): 54 significant bits
     * (53 + round bit); k = smallest shift that can reach d*2^53 */
    const int k = d == 3 ? 2 : d == 9 ? 4 : 3;
    const int t = ((M << k) >= (uint64_t)d * 0x0020000000000000ULL) ? k : k + 1;
    const uint64_t n = M << t;
    uint64_t q;
    if (d == 3)
        q = cal_mulhi64(n, 0xAAAAAAAAAAAAAAABULL) >> 1;
    else if (d == 5)
        q = cal_mulhi64(n, 0xCCCCCCCCCCCCCCCDULL) >> 2;
    else if (d == 7)
        q = cal_mulhi64(n, 0x924924924924924AULL) >> 2;
    else
        q = cal_mulhi64(n, 0x71C71C71C71C71C8ULL) >> 2;
    const uint64_t rem = n - q * (uint64_t)d;
    uint64_t sig = q >> 1;
    const uint64_t round_bit = q & 1;
    if (round_bit && (rem != 0 || (sig & 1)))
        sig++;
    /* value = q * 2^(E-52-t) = sig * 2^(E-52-t+1); sig in [2^52, 2^53] */
    int e = exp - t + 1 - half;
    if (sig == 0x0020000000000000ULL) { /* rounding carried into a new bit */
        sig >>= 1;
        e++;
    }
    return cal_i2d(sign | ((int64_t)e << 52) | (int64_t)(sig & 0x000fffffffffffffULL));
}

/* Division by a fixed divisor b through y = RN(1/b), exactly rounded:
 *   q = RN(a y),  r = a - b q (exact, one FMA),  a / b ~ RN(q + r y)  (one FMA).
 * Markstein's theorem (P. Markstein, IBM J. Res. Dev. 34(1), 1990; also
 * Muller et al., Handbook of Floating-Point Arithmetic, section on
 * Newton-Raphson division with an FMA): if q is a faithful rounding of a/b
 * and y approximates 1/b with relative error below 2^-53, then r is exact
 * and RN(q + r y) = RN(a/b), barring underflow and overflow.  q = RN(a y) is
 * faithful when |y b - 1| < 2^-55 (then |a y - a/b| < ulp(a/b) / 4), which
 * the host checks for the divisor once (cal_recip_exact_ok, which also
 * keeps b in [2^-16, 2^16]); a outside [2^-800, 2^800] in magnitude, zeros
 * included, takes the plain division, so that q and r stay far from
 * underflow and overflow. */
CAL_HD bool cal_recip_exact_ok(double b, double y)
{
    if (!(b >= 0x1p-16 && b <= 0x1p16))
        return false;
    const double e = fma(y, b, -1.0); /* exact when |y b - 1| < 2^-50: y b is a multiple of 2^-106 */
    return e < 0x1p-55 && e > -0x1p-55;
}

CAL_HD double cal_div_recip(double a, double b, double y)
{
    const int ea = (int)((cal_d2i(a) >> 52) & 0x7ff);
    if (ea < 1023 - 800 || ea > 1023 + 800)
        return a / b;
    const double q = a * y;
    const double r = fma(-q, b, a);
    return fma(r, y, q);
}

/* a <= b as IEEE compares doubles, on the bit patterns when both are
 * non-negative and not NaN (integer pipe); otherwise the FP comparison */
CAL_HD bool cal_le(double a, double b)
{
    const int64_t ba = cal_d2i(a), bb = cal_d2i(b);
    if ((ba | bb) >= 0 && ba <= (int64_t)0x7ff0000000000000LL && bb <= (int64_t)0x7ff0000000000000LL)
        return ba <= bb;
    return a <= b;
}

/* a > b (IEEE, false with a NaN), on the bit patterns when both are
 * non-negative and not NaN */
CAL_HD bool cal_gt(double a, double b)
{
    const int64_t ba = cal_d2i(a), bb = cal_d2i(b);
    if ((ba | bb) >= 0 && ba <= (int64_t)0x7ff0000000000000LL && bb <= (int64_t)0x7ff0000000000000LL)
        return ba > bb;
    return a > b;
}

/* x > 0 (IEEE: false for zeros of either sign and NaN) on the integer pipe */
CAL_HD bool cal_pos(double x)
{
    const int64_t b = cal_d2i(x);
    return b > 0 && b <= (int64_t)0x7ff0000000000000LL;
}
