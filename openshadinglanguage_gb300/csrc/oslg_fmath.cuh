// The executor's own single-precision exp, sincos, log and power for the
// Gabor impulse loop and the sheen distribution, where libm-accurate double
// evaluation would run on the FP64 pipe.
// Written from the mathematics: Cody & Waite argument reduction (a short
// constant head whose products with the integer multiple are exact, plus a
// tail), Taylor polynomials of the reduced argument in Horner form, and a
// 2^n scale by two exact power-of-two multiplies (subnormals round once).
// Only IEEE add/sub/mul and float<->int conversions: built with -fmad=false
// these give the same bits as the host statement of the same steps.
// Accuracy: exp within 2 ulp, sin/cos within 2^-23 absolute of libm.
#pragma once
#include <stdint.h>

namespace oslg {
namespace dev {

__device__ __forceinline__ float pow2i(int k) { return __uint_as_float((uint32_t)(k + 127) << 23); }

__device__ __forceinline__ float own_exp(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
    if (x < -103.972084f) return 0.0f;
    const float t = x * 1.4426950216293335f;
    const int n = (int)floorf(t + 0.5f);
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

__device__ __forceinline__ void own_sincos(float x, float* s, float* c) {
    if (!(fabsf(x) <= 6000.0f)) {
        // outside the exact-reduction range (and NaN/inf): double precision
        double xd = (double)x;
        *s = (float)sin(xd);
        *c = (float)cos(xd);
        return;
    }
    const int k = (int)floorf(x * 0.6366197466850281f + 0.5f);
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
__device__ __forceinline__ float own_log(float x) {
    if (!(x > 0.0f)) return x == 0.0f ? __int_as_float(0xff800000) : __int_as_float(0x7fc00000);
    if (x == __int_as_float(0x7f800000)) return x;
    int e = 0;
    if (x < 1.17549435e-38f) {  // subnormal: scale into the normal range
        x = x * 8388608.0f;
        e = -23;
    }
    const uint32_t b = __float_as_uint(x);
    e += (int)(b >> 23) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
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
__device__ __forceinline__ float own_pow_pos(float x, float y) {
    if (x == 0.0f) return 0.0f;
    if (x == 1.0f) return 1.0f;
    return own_exp(y * own_log(x));
}

}  // namespace dev
}  // namespace oslg
