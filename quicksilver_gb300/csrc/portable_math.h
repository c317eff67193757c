/* Natural logarithm, sine and cosine built only from IEEE 754 double
 * operations that every conforming implementation rounds the same way (+, -,
 * *, /, fused multiply-add, sqrt not used) and integer bit manipulation, so
 * that a CPU and a GPU evaluating them give the same bits for every
 * argument.
 *
 * Why: the tracking path calls log (the number of mean free paths to the
 * next collision, MC_Segment_Outcome.cc:77-84, CollisionEvent.cc:43) and sin /
 * cos (the azimuth of updateTrajectory, CollisionEvent.cc:29-33; the
 * isotropic source direction, DirectionCosine.cc:5-12).  The reference takes
 * them from the host's libm, the GPU build from the CUDA math library; they
 * round a few arguments per thousand differently in the last bit, so
 * trajectories agree only to ~1e-15 cm.  A build of this library and of the
 * oracle (and the reference itself, linked with --wrap) that all use the
 * functions below instead tracks bit-identical trajectories -- the check that
 * nothing but the elementary functions separates them.  Not used by the
 * default build.
 *
 * Methods (textbook argument reductions, Taylor coefficients; no minimax
 * fits, so more terms than a production library would need):
 *  - log: x = 2^k m with m in [sqrt(1/2), sqrt(2)), f = m - 1 (exact),
 *    s = f / (2 + f), log m = 2 atanh s = f - (f^2/2 - s (f^2/2 + R)) with
 *    R = sum_{j>=1} 2 s^{2j} / (2j + 1) (ten terms: |s| <= 0.1716), then
 *    k ln2 added in two parts (ln 2 rounded to 42 bits, so k ln2_hi is exact,
 *    and the rounded remainder), the large terms summed with their rounding
 *    errors carried (TwoSum, fused multiply-add) so that only the last
 *    addition rounds noticeably.
 *  - sin / cos: x = k pi/2 + r (Cody and Waite's reduction with pi/2 split
 *    into two 33-bit parts and a rounded third, exact products for
 *    |k| < 2^20, r kept as an unevaluated sum rh + rl), Taylor series of sin
 *    and cos about 0 on |r| <= pi/4 (through r^19 and r^20), the quadrant
 *    from k mod 4.  Arguments are supported for |x| < 2^19 pi / 2; others
 *    return NaN (the tracking path sees |x| < 2 pi).
 * Accuracy: within one unit in the last place (log close to correctly
 * rounded), checked against the host's libm over the random-number stream's
 * arguments.
 *
 * Plain C99 / CUDA C++: the oracle (C) and the CUDA kernels include it. */
#ifndef QSG_PORTABLE_MATH_H
#define QSG_PORTABLE_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define QSG_PM_FN __host__ __device__ __forceinline__
#else
#define QSG_PM_FN static inline
#endif

QSG_PM_FN uint64_t qsg_pm_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

QSG_PM_FN double qsg_pm_double(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

QSG_PM_FN double qsg_pm_fma(double a, double b, double c)
{
    return fma(a, b, c);   /* correctly rounded on every IEEE 754-2008 platform */
}

/* log(x) for x >= 0 (x = 0: -infinity; negative or NaN: NaN; +inf: +inf). */
QSG_PM_FN double qsg_log(double x)
{
    const double ln2_hi = 0x1.62e42fefa3800p-1;   /* ln 2 to 42 bits */
    const double ln2_lo = 0x1.ef35793c76730p-45;  /* RN(ln 2 - ln2_hi) */
    const double sqrt2 = 0x1.6a09e667f3bcdp+0;
    uint64_t ix = qsg_pm_bits(x);
    if (ix == 0) return qsg_pm_double(0xfff0000000000000ull);   /* log(+0) = -inf */
    if (ix >> 63) return qsg_pm_double(0x7ff8000000000000ull);  /* negative: NaN */
    int k = (int)(ix >> 52);
    if (k == 0x7ff) return x + x;                  /* inf or NaN */
    if (k == 0) {                                  /* subnormal: scale by 2^54 */
        ix = qsg_pm_bits(x * 0x1p54);
        k = (int)(ix >> 52) - 54;
    }
    k -= 1023;
    double m = qsg_pm_double((ix & 0x000fffffffffffffull) | 0x3ff0000000000000ull);   /* [1, 2) */
    if (m > sqrt2) {
        m = qsg_pm_double((ix & 0x000fffffffffffffull) | 0x3fe0000000000000ull);       /* [1/2, 1) */
        k += 1;
    }
    const double f = m - 1.0;                      /* exact */
    const double s = f / (2.0 + f);
    const double z = s * s;
    double R = 0x1.8618618618618p-4;               /* RN(2 / 21) */
    R = R * z + 0x1.af286bca1af28p-4;              /* 2 / 19 */
    R = R * z + 0x1.e1e1e1e1e1e1ep-4;              /* 2 / 17 */
    R = R * z + 0x1.1111111111111p-3;              /* 2 / 15 */
    R = R * z + 0x1.3b13b13b13b14p-3;              /* 2 / 13 */
    R = R * z + 0x1.745d1745d1746p-3;              /* 2 / 11 */
    R = R * z + 0x1.c71c71c71c71cp-3;              /* 2 / 9 */
    R = R * z + 0x1.2492492492492p-2;              /* 2 / 7 */
    R = R * z + 0x1.999999999999ap-2;              /* 2 / 5 */
    R = R * z + 0x1.5555555555555p-1;              /* 2 / 3 */
    R = R * z;
    /* log x = k ln2_hi + f - f^2/2 + s (f^2/2 + R) + k ln2_lo, summed with
       the rounding errors of the large terms carried exactly: f^2 = p + ep
       (fused multiply-add), f - p/2 = t1 + e1 and k ln2_hi + t1 = t2 + e2
       (Knuth's TwoSum); k ln2_hi is exact */
    const double dk = (double)k;
    const double p = f * f;
    const double ep = qsg_pm_fma(f, f, -p);
    const double hfsq = 0.5 * p;
    const double t1 = f - hfsq;
    const double b1 = t1 - f;
    const double e1 = (f - (t1 - b1)) + (-hfsq - b1);
    const double a = dk * ln2_hi;
    const double t2 = a + t1;
    const double b2 = t2 - a;
    const double e2 = (a - (t2 - b2)) + (t1 - b2);
    const double tail = ((e1 + e2) - 0.5 * ep) + (s * (hfsq + R) + dk * ln2_lo);
    return t2 + tail;
}

/* sin(x) and cos(x) for |x| < 2^19 pi / 2 (NaN outside). */
QSG_PM_FN void qsg_sincos(double x, double* sin_out, double* cos_out)
{
    const double two_over_pi = 0x1.45f306dc9c883p-1;
    const double pio2_1 = 0x1.921fb54400000p+0;    /* pi/2 to 33 bits */
    const double pio2_2 = 0x1.0b4611a600000p-34;   /* the next 33 bits */
    const double pio2_3 = 0x1.3198a2e037073p-69;   /* RN(the rest) */
    if (!(x > -0x1.921fb54442d18p+19 && x < 0x1.921fb54442d18p+19)) {   /* also inf and NaN */
        *sin_out = *cos_out = qsg_pm_double(0x7ff8000000000000ull);
        return;
    }
    /* k = x * 2/pi rounded to the nearest integer (ties to even), by the
       2^52 + 2^51 shift (its low mantissa bits are then k mod 4) */
    const double shift = 0x1.8p52;
    const double kk = x * two_over_pi + shift;
    const double kd = kk - shift;
    const int q = (int)(qsg_pm_bits(kk) & 3u);
    /* r = x - k pi/2 as rh + rl: k * pio2_1 and k * pio2_2 are exact (k has
       at most 20 bits), x - k pio2_1 is exact (Sterbenz: the two are within a
       factor of two, or k = 0) */
    const double t = qsg_pm_fma(-kd, pio2_1, x);
    const double w = kd * pio2_2;
    double rh = t - w;
    double rl = ((t - rh) - w) - kd * pio2_3;
    const double r = rh + rl;
    rl = (rh - r) + rl;
    rh = r;
    const double z = rh * rh;
    /* sin(rh + rl) = rh + rh^3 S(z) + rl (1 - z/2) to this accuracy */
    double S = -0x1.2f49b46814157p-57;             /* -1/19! */
    S = S * z + 0x1.952c77030ad4ap-49;             /* 1/17! */
    S = S * z - 0x1.ae7f3e733b81fp-41;             /* -1/15! */
    S = S * z + 0x1.6124613a86d09p-33;             /* 1/13! */
    S = S * z - 0x1.ae64567f544e4p-26;             /* -1/11! */
    S = S * z + 0x1.71de3a556c734p-19;             /* 1/9! */
    S = S * z - 0x1.a01a01a01a01ap-13;             /* -1/7! */
    S = S * z + 0x1.1111111111111p-7;              /* 1/5! */
    S = S * z - 0x1.5555555555555p-3;              /* -1/3! */
    const double sn = rh + ((rh * z) * S + rl * (1.0 - 0.5 * z));
    /* cos(rh + rl) = 1 - z/2 + z^2 C(z) - rh rl */
    double Cc = 0x1.e542ba4020225p-62;             /* 1/20! */
    Cc = Cc * z - 0x1.6827863b97d97p-53;           /* -1/18! */
    Cc = Cc * z + 0x1.ae7f3e733b81fp-45;           /* 1/16! */
    Cc = Cc * z - 0x1.93974a8c07c9dp-37;           /* -1/14! */
    Cc = Cc * z + 0x1.1eed8eff8d898p-29;           /* 1/12! */
    Cc = Cc * z - 0x1.27e4fb7789f5cp-22;           /* -1/10! */
    Cc = Cc * z + 0x1.a01a01a01a01ap-16;           /* 1/8! */
    Cc = Cc * z - 0x1.6c16c16c16c17p-10;           /* -1/6! */
    Cc = Cc * z + 0x1.5555555555555p-5;            /* 1/4! */
    /* 1 - z/2 carries the rounding errors of z = rh^2 (fused multiply-add)
       and of the subtraction (exact by Sterbenz's lemma) */
    const double ez = qsg_pm_fma(rh, rh, -z);
    const double hz = 0.5 * z;
    const double one_minus = 1.0 - hz;
    const double cs = one_minus + (((1.0 - one_minus) - hz) + ((z * z) * Cc - (rh * rl + 0.5 * ez)));
    switch (q) {
    case 0: *sin_out = sn; *cos_out = cs; break;
    case 1: *sin_out = cs; *cos_out = -sn; break;
    case 2: *sin_out = -sn; *cos_out = -cs; break;
    default: *sin_out = -cs; *cos_out = sn; break;
    }
}

QSG_PM_FN double qsg_sin(double x)
{
    double s, c;
    qsg_sincos(x, &s, &c);
    return s;
}

QSG_PM_FN double qsg_cos(double x)
{
    double s, c;
    qsg_sincos(x, &s, &c);
    return c;
}

#endif /* QSG_PORTABLE_MATH_H */
