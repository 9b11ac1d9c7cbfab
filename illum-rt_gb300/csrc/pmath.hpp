// Portable double-precision elementary functions for the synthetic scene generators.
//
// The generated scenes must be bit-identical on every host (x86-64 here, aarch64 on the GPU
// host), so nothing below calls libm transcendentals, whose last bit can differ between C
// libraries and ISAs. Each function uses only IEEE-754 add, subtract, multiply, divide and
// sqrt (all correctly rounded on both ISAs), range reduction with exactly representable
// constants, and truncated Taylor series (sin, cos, exp) or the atanh series for log. The
// translation unit must be compiled with -ffp-contract=off so that no product is fused into
// a following add. Accuracy is ~1e-15 relative, far below float rounding of the outputs.
#pragma once
#include <cmath>
#include <cstdint>

namespace grt_pm {

// pi/2 split into a head with 33 significant bits (so k * head is exact for |k| < 2^20) and a tail.
static const double PIO2_HI = 1.5707963267341256e+00;
static const double PIO2_LO = 6.0771005065061922e-11;
static const double PI = 3.141592653589793238462643383279502884;
static const double LN2_HI = 6.93147180369123816490e-01;
static const double LN2_LO = 1.90821492927058770002e-10;

// sin and cos of r with |r| <= pi/4, Taylor series to the 19th / 18th order term.
inline void sincos_kernel(double r, double *s, double *c) {
    double r2 = r * r;
    double ts = r, tc = 1.0, sum_s = r, sum_c = 1.0;
    for (int k = 1; k <= 9; ++k) {
        ts = -ts * r2 / double((2 * k) * (2 * k + 1));
        tc = -tc * r2 / double((2 * k - 1) * (2 * k));
        sum_s = sum_s + ts;
        sum_c = sum_c + tc;
    }
    *s = sum_s;
    *c = sum_c;
}

inline void sincos(double x, double *s, double *c) {
    double kf = std::nearbyint(x / (PI / 2));
    long k = (long)kf;
    double r = (x - kf * PIO2_HI) - kf * PIO2_LO;
    double sr, cr;
    sincos_kernel(r, &sr, &cr);
    switch (((k % 4) + 4) % 4) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

inline double sin(double x) { double s, c; sincos(x, &s, &c); return s; }
inline double cos(double x) { double s, c; sincos(x, &s, &c); return c; }
inline double tan(double x) { double s, c; sincos(x, &s, &c); return s / c; }

// Natural log for x > 0: x = m * 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh((m-1)/(m+1)).
inline double log(double x) {
    int e;
    double m = std::frexp(x, &e);  // exact: m in [0.5, 1)
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0);
    double s2 = s * s, term = s, sum = s;
    for (int k = 1; k <= 20; ++k) {
        term = term * s2;
        sum = sum + term / double(2 * k + 1);
    }
    return 2.0 * sum + double(e) * LN2_HI + double(e) * LN2_LO;
}

// exp(x) = 2^k * exp(r), r = x - k ln2 with |r| <= ln2/2, Taylor series to the 22nd term.
inline double exp(double x) {
    double kf = std::nearbyint(x / (LN2_HI + LN2_LO));
    double r = (x - kf * LN2_HI) - kf * LN2_LO;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 22; ++k) {
        term = term * r / double(k);
        sum = sum + term;
    }
    return std::ldexp(sum, (int)kf);
}

inline double cbrt(double x) {
    // Newton iterations on y^3 = x, started from the exponent; x > 0.
    int e;
    std::frexp(x, &e);
    double y = std::ldexp(1.0, e / 3);
    for (int i = 0; i < 60; ++i) y = y - (y * y * y - x) / (3.0 * y * y);
    return y;
}

}  // namespace grt_pm
