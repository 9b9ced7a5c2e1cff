// The executor's own single-precision exp and sincos for the Gabor impulse
// loop, where libm-accurate double evaluation would run on the FP64 pipe.
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

}  // namespace dev
}  // namespace oslg
