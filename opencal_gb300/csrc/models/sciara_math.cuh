/*
 * sciara_math.cuh -- the transcendental parts of SCIARA-fv2's transition
 * function, written for a GPU whose FP64 pipe is narrow.  The reference
 * (OpenCAL-OMP/examples/calomp_sciara-fv2/source/Sciara.cpp) evaluates
 *
 *   powerLaw(k1, k2, T) = pow(10, k1 + k2 T)                 (Sciara.cpp:19-21)
 *   theta_k = atan(dz_k / w),  flow iff h0 > hc cos(theta_k)  (Sciara.cpp:53, 82)
 *   aus = 1 + 3 pow(T, 3) K / (C h),  T' = T / pow(aus, 1/3)  (Sciara.cpp:147-150)
 *
 * per lava cell and step: two pow, up to eight atan and eight cos, two more
 * pow.  Here each is the same quantity by an identity:
 *
 *   10^x                   exp10(x)
 *   h0 > hc cos(atan(dz/w)) with cos(atan(x)) = 1 / sqrt(1 + x^2), dz > 0,
 *                          hc > 0:  h0 > 0 and h0^2 (w^2 + dz^2) > hc^2 w^2
 *   pow(T, 3)              T * T * T
 *   pow(aus, 1/3)          cbrt(aus)
 *
 * Each differs from the C library's form by rounding only (a few ulp); the
 * shear test can decide differently from the reference only where h0 and
 * hc cos(theta) agree to the last bits.  The device-process program
 * (sciara.cu) and the split step (sciara_batch.cu) share these functions and
 * so agree bit for bit; against the C library they agree to a relative
 * 1e-10 over hundreds of steps.
 */
#ifndef OPENCAL_GB300_SCIARA_MATH_CUH
#define OPENCAL_GB300_SCIARA_MATH_CUH

static __device__ __forceinline__ double sci_power_law(double k1, double k2, double T)
{
    return exp10(k1 + k2 * T);
}

/* h0 > hc * cos(atan(dz / w)) for dz > 0, w > 0, hc > 0 */
static __device__ __forceinline__ bool sci_shear_exceeded(double h0, double hc, double dz, double w)
{
    return h0 > 0 && h0 * h0 * (w * w + dz * dz) > hc * hc * (w * w);
}

/* T' = T / pow(aus, 1/3), aus = 1 + 3 T^3 eps sigma clock cool / (rho cv h
 * ac), in the reference's operation order; sets *aus */
static __device__ __forceinline__ double sci_cool(double T, double h, double eps, double sigma, double clock,
                                                  double cool, double rho, double cv, double ac, double* aus)
{
    *aus = 1.0 + (3 * (T * T * T) * eps * sigma * clock * cool) / (rho * cv * h * ac);
    return T / cbrt(*aus);
}

/* The same three quantities written as the reference writes them, with
 * CUDA's pow, atan and cos in place of the C library's (the
 * device-process program selects them with cal_sciara_set_math(1)): the
 * difference from the C library is then CUDA's own rounding of those
 * functions alone. */
static __device__ __forceinline__ double sci_power_law_libm(double k1, double k2, double T)
{
    const double log_value = k1 + k2 * T;
    return pow(10.0, log_value);
}

static __device__ __forceinline__ bool sci_shear_exceeded_libm(double h0, double hc, double dz, double w)
{
    const double theta = atan(dz / w);
    return h0 > hc * cos(theta);
}

static __device__ __forceinline__ double sci_cool_libm(double T, double h, double eps, double sigma, double clock,
                                                       double cool, double rho, double cv, double ac, double* aus)
{
    *aus = 1.0 + (3 * pow(T, 3.0) * eps * sigma * clock * cool) / (rho * cv * h * ac);
    return T / pow(*aus, 1.0 / 3.0);
}

#endif
