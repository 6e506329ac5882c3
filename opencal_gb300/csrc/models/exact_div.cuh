/*
 * exact_div.cuh -- IEEE-754 double division by a small positive integer
 * (1..5), correctly rounded to nearest-even, computed with integer
 * arithmetic on the significand.
 *
 * Why: the SCIDDICA-T outflow computation divides a running sum by the
 * number of cells left in the minimisation (1..5).  On GB300 the FP64 pipe
 * is narrow (about 1/64 of the FP32/integer rate per SM), and a double
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
 *   64-bit integer by 3 or 5 uses the exact multiply-high identities
 *     n / 3 = mulhi(n, 0xAAAAAAAAAAAAAAAB) >> 1
 *     n / 5 = mulhi(n, 0xCCCCCCCCCCCCCCCD) >> 2      (for all 64-bit n)
 *   (division by invariant integers, Granlund & Montgomery 1994).
 *   c = 1, 2, 4 only change the exponent.
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

/* x / c for c in 1..5, bit-identical to the IEEE quotient */
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
    if (c == 2 || c == 4) /* exact scaling: only the exponent changes */
        return cal_i2d(bits - ((int64_t)(c == 2 ? 1 : 2) << 52));
    const uint64_t M = ((uint64_t)bits & 0x000fffffffffffffULL) | 0x0010000000000000ULL; /* [2^52, 2^53) */
    /* shift so that the quotient has 54 significant bits (53 + round bit) */
    int t;
    uint64_t n, q;
    if (c == 3) {
        /* M*2^t/3 in [2^53, 2^54): t = 2 if M*4 >= 3*2^53, else 3 */
        t = (M * 4 >= 3ULL * 0x0020000000000000ULL) ? 2 : 3;
        n = M << t;
        q = cal_mulhi64(n, 0xAAAAAAAAAAAAAAABULL) >> 1;
    } else { /* c == 5: M*2^t/5 in [2^53, 2^54): t = 3 if M*8 >= 5*2^53, else 4 */
        t = (M * 8 >= 5ULL * 0x0020000000000000ULL) ? 3 : 4;
        n = M << t;
        q = cal_mulhi64(n, 0xCCCCCCCCCCCCCCCDULL) >> 2;
    }
    const uint64_t rem = n - q * (uint64_t)c;
    uint64_t sig = q >> 1;
    const uint64_t round_bit = q & 1;
    if (round_bit && (rem != 0 || (sig & 1)))
        sig++;
    /* value = q * 2^(E-52-t) = sig * 2^(E-52-t+1); sig in [2^52, 2^53] */
    int e = exp - t + 1;
    if (sig == 0x0020000000000000ULL) { /* rounding carried into a new bit */
        sig >>= 1;
        e++;
    }
    return cal_i2d(sign | ((int64_t)e << 52) | (int64_t)(sig & 0x000fffffffffffffULL));
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
