/*
 * detmath.h — deterministic double-precision cbrt, acos, sin and cos.
 *
 * The PLIC plane-constant solve (Scardovelli & Zaleski inverse, reference src/VF.jl:164-214)
 * calls cbrt, acos, sin and cos.  Host libm and the CUDA device library may differ in the last
 * bit for these functions, and ELVIRA's strict "<" argmin over candidate normals
 * (src/ELVIRA.jl:129) then breaks exact ties between mirror-image candidates differently on
 * the two sides.  A CPU restatement and the FP64 GPU path therefore use the functions below,
 * which are built only from IEEE-754 operations whose results are fully specified
 * (+, -, *, /, sqrt, frexp, ldexp).  Compiled without FMA contraction (-ffp-contract=off on
 * gcc, -fmad=false on nvcc) they return identical bits on x86-64, aarch64 and sm_103a.
 *
 * Methods (all textbook mathematics, no vendor library code):
 *   cbrt : x = f * 2^e (frexp), e = 3q + r, Newton iteration y <- y - (y - m/y^2)/3 on
 *          m = f * 2^r from a quadratic least-squares start, then y * 2^q (ldexp).
 *   asin : Maclaurin series  asin(s) = sum (2n)! / (4^n (n!)^2 (2n+1)) s^(2n+1)  on |s| <= 1/2.
 *   acos : pi/2 - asin(x) for |x| <= 1/2; half-angle identities 2 asin(sqrt((1-x)/2)) and
 *          pi - 2 asin(sqrt((1+x)/2)) outside; pi and pi/2 carried as two-double sums.
 *   sin, cos : reduction by the nearest multiple of pi/2 (two-constant split), then the
 *          Maclaurin series of sin and cos on |r| <= pi/4 (terms through r^19 / r^18).
 * Accuracy against libm (a few ulp at most) is checked by tests/test_oracle_pins.py.
 */
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define DETM_FN __host__ __device__ __forceinline__
#else
#define DETM_FN static inline
#endif

DETM_FN double detm_cbrt(double x)
{
    if (x != x || x == 0.0 || x == INFINITY || x == -INFINITY) return x;
    const double ax = x < 0.0 ? -x : x;
    int e;
    const double f = frexp(ax, &e); /* ax = f * 2^e, f in [0.5, 1) */
    int q = e / 3, r = e % 3;
    if (r < 0) { r += 3; q -= 1; }
    const double m = ldexp(f, r); /* m in [0.5, 4) */
    double y = 0.65149417 + m * (0.37688818 + m * (-0.03680669));
    for (int it = 0; it < 5; ++it) y = y - (y - m / (y * y)) / 3.0;
    y = ldexp(y, q);
    return x < 0.0 ? -y : y;
}

/* asin on |s| <= 0.5 (callers guarantee the range). */
DETM_FN double detm_asin_small(double s)
{
    const double z = s * s;
    double p = 0.0022014739737101384;
    p = 0.002338091892111975 + z * p;
    p = 0.0024894486782468836 + z * p;
    p = 0.00265787063820729 + z * p;
    p = 0.002846178401108942 + z * p;
    p = 0.0030578216492580306 + z * p;
    p = 0.003297059503473485 + z * p;
    p = 0.0035692053938259347 + z * p;
    p = 0.003880964558837669 + z * p;
    p = 0.004240907093679363 + z * p;
    p = 0.004660143486915096 + z * p;
    p = 0.005153309682319905 + z * p;
    p = 0.005740037670841924 + z * p;
    p = 0.006447210311889649 + z * p;
    p = 0.0073125258735988454 + z * p;
    p = 0.008390335809616815 + z * p;
    p = 0.009761609529194078 + z * p;
    p = 0.011551800896139705 + z * p;
    p = 0.01396484375 + z * p;
    p = 0.017352764423076924 + z * p;
    p = 0.022372159090909092 + z * p;
    p = 0.030381944444444444 + z * p;
    p = 0.044642857142857144 + z * p;
    p = 0.075 + z * p;
    p = 0.16666666666666666 + z * p;
    return s + s * (z * p);
}

DETM_FN double detm_acos(double x)
{
    const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
    const double PI_HI = 3.141592653589793, PI_LO = 1.2246467991473532e-16;
    if (x != x || x > 1.0 || x < -1.0) return NAN;
    if (x <= 0.5 && x >= -0.5) return PIO2_HI - (detm_asin_small(x) - PIO2_LO);
    if (x > 0.5) {
        const double s = sqrt((1.0 - x) * 0.5);
        return 2.0 * detm_asin_small(s);
    }
    const double s = sqrt((1.0 + x) * 0.5);
    return PI_HI - (2.0 * detm_asin_small(s) - PI_LO);
}

/* Maclaurin kernels on |r| <= pi/4. */
DETM_FN double detm_sin_kernel(double r)
{
    const double z = r * r;
    double p = -8.22063524662433e-18;
    p = 2.8114572543455206e-15 + z * p;
    p = -7.647163731819816e-13 + z * p;
    p = 1.6059043836821613e-10 + z * p;
    p = -2.505210838544172e-08 + z * p;
    p = 2.7557319223985893e-06 + z * p;
    p = -0.0001984126984126984 + z * p;
    p = 0.008333333333333333 + z * p;
    p = -0.16666666666666666 + z * p;
    return r + r * (z * p);
}

DETM_FN double detm_cos_kernel(double r)
{
    const double z = r * r;
    double p = -1.5619206968586225e-16;
    p = 4.779477332387385e-14 + z * p;
    p = -1.1470745597729725e-11 + z * p;
    p = 2.08767569878681e-09 + z * p;
    p = -2.755731922398589e-07 + z * p;
    p = 2.48015873015873e-05 + z * p;
    p = -0.001388888888888889 + z * p;
    p = 0.041666666666666664 + z * p;
    return (1.0 - 0.5 * z) + z * (z * p);
}

/* Reduction x = n*pi/2 + r.  n*PIO2_HI is exact for |n| <= 1 (|x| < 3pi/4), which covers
 * every call site (theta = acos(q)/3 in [0, pi/3]); larger |x| stay deterministic but lose
 * accuracy. */
DETM_FN double detm_reduce(double x, int* quadrant)
{
    const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
    const double t = x * 0.6366197723675814;
    const double n = t >= 0.0 ? floor(t + 0.5) : -floor(-t + 0.5);
    *quadrant = ((int)n) & 3;
    return (x - n * PIO2_HI) - n * PIO2_LO;
}

DETM_FN double detm_sin(double x)
{
    if (x != x || x == INFINITY || x == -INFINITY) return NAN;
    int q;
    const double r = detm_reduce(x, &q);
    switch (q) {
    case 0: return detm_sin_kernel(r);
    case 1: return detm_cos_kernel(r);
    case 2: return -detm_sin_kernel(r);
    default: return -detm_cos_kernel(r);
    }
}

DETM_FN double detm_cos(double x)
{
    if (x != x || x == INFINITY || x == -INFINITY) return NAN;
    int q;
    const double r = detm_reduce(x, &q);
    switch (q) {
    case 0: return detm_cos_kernel(r);
    case 1: return -detm_sin_kernel(r);
    case 2: return -detm_cos_kernel(r);
    default: return detm_sin_kernel(r);
    }
}
