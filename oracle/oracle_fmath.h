// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU statement of the executor's own single-precision exp and sincos, the
// ones the device Gabor kernel evaluates per impulse. They are written from
// the mathematics, not taken from any library:
//   * argument reduction by Cody & Waite (x = n*c + r with c split into a
//     short head, whose products with n are exact, and a tail);
//   * Taylor polynomials of the reduced argument in Horner form;
//   * exp scales by 2^n through two exact power-of-two multiplies so that
//     subnormal results round once.
// Only IEEE add/sub/mul/div and float<->int conversions are used, so with
// -ffp-contract=off on the host and -fmad=false on the device both sides
// produce the same bits. Accuracy against double-precision libm is checked
// by the tests (exp: <= 2 ulp; sin/cos: <= 2^-23 absolute).
//
// The reference evaluates these Gabor terms with libm expf / sincosf
// (src/liboslnoise/gabornoise.h:117-118 through OSL/dual.h:830-835,
// :1122-1126); gabor_eval in oracle_gabor.h can run with either.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle {

inline float pow2i(int k) {  // 2^k for k in [-126, 127]
    uint32_t b = (uint32_t)(k + 127) << 23;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

inline float own_exp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return INFINITY;
    if (x < -103.972084f) return 0.0f;
    const float t = x * 1.4426950216293335f;
    const int n = (int)std::floor(t + 0.5f);
    const float fn = (float)n;
    const float r = (x - fn * 0.693359375f) - fn * -0.00021219444170128554f;
    float p = 0.00019841270113829523f;
    p = 0.0013888889225199819f + r * p;
    p = 0.008333333767950535f + r * p;
    p = 0.0416666679084301f + r * p;
    p = 0.1666666716337204f + r * p;
    p = 0.5f + r * p;
    p = 1.0f + r * p;
    p = 1.0f + r * p;
    const int n1 = n / 2, n2 = n - n / 2;
    return (p * pow2i(n1)) * pow2i(n2);
}

inline void own_sincos(float x, float* s, float* c) {
    if (!(std::fabs(x) <= 6000.0f)) {
        // outside the exact-reduction range (and NaN/inf): double precision
        double xd = (double)x;
        *s = (float)std::sin(xd);
        *c = (float)std::cos(xd);
        return;
    }
    const int k = (int)std::floor(x * 0.6366197466850281f + 0.5f);
    const float fk = (float)k;
    const float r = ((x - fk * 1.5703125f) - fk * 0.0004837512969970703f) - fk * 7.549790126404332e-08f;
    const float r2 = r * r;
    float sp = 2.7557318844628753e-06f;
    sp = -0.00019841270113829523f + r2 * sp;
    sp = 0.008333333767950535f + r2 * sp;
    sp = -0.1666666716337204f + r2 * sp;
    sp = r + (r * r2) * sp;
    float cp = -2.755731998149713e-07f;
    cp = 2.4801587642286904e-05f + r2 * cp;
    cp = -0.0013888889225199819f + r2 * cp;
    cp = 0.0416666679084301f + r2 * cp;
    cp = -0.5f + r2 * cp;
    cp = 1.0f + r2 * cp;
    switch (k & 3) {
    case 0: *s = sp; *c = cp; break;
    case 1: *s = cp; *c = -sp; break;
    case 2: *s = -sp; *c = -cp; break;
    default: *s = -cp; *c = sp; break;
    }
}


// Natural log for x > 0 (0 -> -inf, negative or NaN -> NaN): exponent split,
// mantissa folded into [sqrt(1/2), sqrt(2)), ln m = 2 atanh(s) with
// s = (m-1)/(m+1) as an odd series to s^11, ln 2 in a head and tail.
inline float own_log(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (x == INFINITY) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {  // subnormal: scale into the normal range
        x = x * 8388608.0f;
        e = -23;
    }
    uint32_t b;
    std::memcpy(&b, &x, 4);
    e += (int)(b >> 23) - 127;
    const uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = (m - 1.0f) / (m + 1.0f);
    const float s2 = s * s;
    float p = 0.0909090936f;
    p = 0.111111112f + s2 * p;
    p = 0.142857149f + s2 * p;
    p = 0.200000003f + s2 * p;
    p = 0.333333343f + s2 * p;
    p = 1.0f + s2 * p;
    const float fe = (float)e;
    return fe * 0.693359375f + ((s + s) * p + fe * -0.00021219444170128554f);
}

// x^y for x >= 0, y > 0 as own_exp(y * own_log(x)) (about 1e-5 relative
// for |y ln x| near 100): the sheen distribution's power.
inline float own_pow_pos(float x, float y) {
    if (x == 0.0f) return 0.0f;
    if (x == 1.0f) return 1.0f;
    return own_exp(y * own_log(x));
}

}  // namespace oracle
