// Fast float transcendentals of OpenImageIO 3.0 (OpenImageIO/fmath.h, the
// fast_* family), which the reference calls for every transcendental op in
// its default build (USE_FAST_MATH=ON, CMakeLists.txt:145-150;
// src/liboslexec/wide/wide_optranscendental.cpp:34-66 and
// wide_optrigonometric.cpp:16-47). OpenImageIO is not part of the reference
// tree; the algorithms below are restated from its published sources:
//   exp2   range reduction to [0,1) + degree-5 polynomial, exponent added
//          to the bits; exp = exp2(x / ln 2); expm1 = exp - 1 except a
//          quadratic near 0
//   log2   exponent + degree-8 polynomial in the mantissa - 1 (two halves);
//          log = log2 * ln 2, log10 = log2 * ln 2 / ln 10
//   pow    "safe" pow: 0 for a negative base with a non-integer exponent,
//          exp2(y * log2|x|) with the sign of odd integer exponents
//   erf    Abramowitz & Stegun 7.1.28; erfc = 1 - erf
//   cbrt   Hacker's Delight initial guess + two Newton steps
//   sin/cos/tan  SLEEF-style Cody-Waite reduction by pi/2 (four parts)
//          and minimax polynomials; out-of-range results clamp to 0
//   asin/acos    sqrt(1 - |x|) times a cubic; atan/atan2 a rational
//          function tuned so atan(1) = pi/4
//   sinh/cosh/tanh   from exp, sinh a degree-7 polynomial on [-1, 1]
// Multiply-adds are separate multiplies and adds (no fused rounding), as
// the rest of the executor.
#pragma once

namespace oslg {
namespace dev {
namespace fm {

__device__ __forceinline__ float madd(float a, float b, float c) { return a * b + c; }
// round half away from zero; saturated to the int range (the reduction is
// meaningless there anyway) so host and device agree for huge arguments
__device__ __forceinline__ int rint_half_away(float x) {
    float t = x + copysignf(0.5f, x);
    if (!(t >= -2147483648.0f)) t = -2147483648.0f;
    if (!(t < 2147483648.0f)) t = 2147483520.0f;
    return (int)t;
}
// OpenImageIO's clamp: a NaN becomes the low bound
__device__ __forceinline__ float clampf(float x, float lo, float hi) {
    if (!(lo <= x)) x = lo;
    if (!(x <= hi)) x = hi;
    return x;
}

__device__ __forceinline__ float exp2(float xv) {
    float x = clampf(xv, -126.0f, 126.0f);
    const int m = (int)x;
    x -= (float)m;
    x = 1.0f - (1.0f - x);
    float r = 1.33336498402e-3f;
    r = madd(x, r, 9.810352697968e-3f);
    r = madd(x, r, 5.551834031939e-2f);
    r = madd(x, r, 0.2401793301105f);
    r = madd(x, r, 0.693144857883f);
    r = madd(x, r, 1.0f);
    return __uint_as_float(__float_as_uint(r) + ((uint32_t)m << 23));
}
__device__ __forceinline__ float exp(float x) { return exp2(x * 1.44269504088896340736f); }
__device__ __forceinline__ float expm1(float x) {
    if (fabsf(x) < 1e-5f) {
        x = 1.0f - (1.0f - x);
        return madd(0.5f, x * x, x);
    }
    return exp(x) - 1.0f;
}
__device__ __forceinline__ float log2(float xv) {
    const float x = clampf(xv, 1.17549435e-38f, 3.40282347e+38f);
    const uint32_t bits = __float_as_uint(x);
    const int e = (int)(bits >> 23) - 127;
    const float f = __uint_as_float((bits & 0x007FFFFFu) | 0x3f800000u) - 1.0f;
    const float f2 = f * f, f4 = f2 * f2;
    float hi = madd(f, -0.00931049621349f, 0.05206469089414f);
    float lo = madd(f, 0.47868480909345f, -0.72116591947498f);
    hi = madd(f, hi, -0.13753123777116f);
    hi = madd(f, hi, 0.24187369696082f);
    hi = madd(f, hi, -0.34730547155299f);
    lo = madd(f, lo, 1.442689881667200f);
    return ((f4 * hi) + (f * lo)) + (float)e;
}
__device__ __forceinline__ float log(float x) { return log2(x) * 0.693147180559945309417f; }
__device__ __forceinline__ float log10(float x) { return log2(x) * 0.301029995663981195214f; }
__device__ __forceinline__ float safe_pow(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return 0.0f;
    if (y == 1.0f) return x;
    if (y == 2.0f) return fminf(x * x, 3.40282347e+38f);
    float sign = 1.0f;
    if (x < 0.0f) {
        // only integer exponents of a negative base: |y| >= 2^24 is an
        // even integer; otherwise the bits below the binary point decide
        const int yb = __float_as_int(y) & 0x7fffffff;
        if (yb >= 0x4b800000) {
        } else if (yb >= 0x3f800000) {
            const int k = (yb >> 23) - 127;
            const int j = yb >> (23 - k);
            if ((j << (23 - k)) != yb) return 0.0f;
            sign = __int_as_float(0x3f800000 | (j << 31));
        } else {
            return 0.0f;
        }
    }
    return sign * exp2(y * log2(fabsf(x)));
}
__device__ __forceinline__ float erf(float x) {
    const float a1 = 0.0705230784f, a2 = 0.0422820123f, a3 = 0.0092705272f, a4 = 0.0001520143f,
                a5 = 0.0002765672f, a6 = 0.0000430638f;
    const float a = fabsf(x);
    const float b = 1.0f - (1.0f - a);
    const float r = madd(madd(madd(madd(madd(madd(a6, b, a5), b, a4), b, a3), b, a2), b, a1), b, 1.0f);
    const float s = r * r, t = s * s, u = t * t, v = u * u;
    return copysignf(1.0f - 1.0f / v, x);
}
__device__ __forceinline__ float erfc(float x) { return 1.0f - erf(x); }
__device__ __forceinline__ float cbrt(float x) {
    const float x0 = fabsf(x);
    float a = __int_as_float(0x2a5137a0 + __float_as_int(x0) / 3);
    a = 0.333333333f * (2.0f * a + x0 / (a * a));
    a = 0.333333333f * (2.0f * a + x0 / (a * a));
    a = x0 == 0.0f ? 0.0f : a;
    return copysignf(a, x);
}
// x - q * (pi / 2) * scale in four parts (scale 2: q counts multiples of pi)
__device__ __forceinline__ float reduce(float x, float qf, float scale) {
    x = madd(qf, -0.78515625f * scale, x);
    x = madd(qf, -0.00024187564849853515625f * scale, x);
    x = madd(qf, -3.7747668102383613586e-08f * scale, x);
    x = madd(qf, -1.2816720341285448015e-12f * scale, x);
    return x;
}
__device__ __forceinline__ void sincos(float x, float* sine, float* cosine) {
    const int q = rint_half_away(x * 0.318309886183790671538f);
    x = reduce(x, (float)q, 4.0f);
    x = 1.57079632679489661923f - (1.57079632679489661923f - x);
    const float s = x * x;
    if ((q & 1) != 0) x = -x;
    float su = 2.6083159809786593541503e-06f;
    su = madd(su, s, -0.0001981069071916863322258f);
    su = madd(su, s, +0.00833307858556509017944336f);
    su = madd(su, s, -0.166666597127914428710938f);
    su = madd(s, su * x, x);
    float cu = -2.71811842367242206819355e-07f;
    cu = madd(cu, s, +2.47990446951007470488548e-05f);
    cu = madd(cu, s, -0.00138888787478208541870117f);
    cu = madd(cu, s, +0.0416666641831398010253906f);
    cu = madd(cu, s, -0.5f);
    cu = madd(cu, s, +1.0f);
    if ((q & 1) != 0) cu = -cu;
    if (fabsf(su) > 1.0f) su = 0.0f;
    if (fabsf(cu) > 1.0f) cu = 0.0f;
    *sine = su;
    *cosine = cu;
}
__device__ __forceinline__ float sin(float x) { float s, c; sincos(x, &s, &c); return s; }
__device__ __forceinline__ float cos(float x) { float s, c; sincos(x, &s, &c); return c; }
__device__ __forceinline__ float tan(float x) {
    const int q = rint_half_away(x * 0.636619772367581343076f);
    x = reduce(x, (float)q, 2.0f);
    if ((q & 1) == 0) x = 0.785398163397448309616f - (0.785398163397448309616f - x);
    const float s = x * x;
    float u = 0.00927245803177356719970703f;
    u = madd(u, s, 0.00331984995864331722259521f);
    u = madd(u, s, 0.0242998078465461730957031f);
    u = madd(u, s, 0.0534495301544666290283203f);
    u = madd(u, s, 0.133383005857467651367188f);
    u = madd(u, s, 0.333331853151321411132812f);
    u = madd(s, u * x, x);
    if ((q & 1) != 0) u = -1.0f / u;
    return u;
}
__device__ __forceinline__ float acos_core(float m) {
    return sqrtf(1.0f - m) * (1.5707963267f + m * (-0.213300989f + m * (0.077980478f + m * -0.02164095f)));
}
__device__ __forceinline__ float acos(float x) {
    const float f = fabsf(x);
    const float m = f < 1.0f ? 1.0f - (1.0f - f) : 1.0f;
    const float a = acos_core(m);
    return x < 0.0f ? 3.14159265358979323846f - a : a;
}
__device__ __forceinline__ float asin(float x) {
    const float f = fabsf(x);
    const float m = f < 1.0f ? 1.0f - (1.0f - f) : 1.0f;
    return copysignf(1.57079632679489661923f - acos_core(m), x);
}
__device__ __forceinline__ float atan_core(float s) {
    const float t = s * s;
    return s * madd(0.430165678f, t, 1.0f) / madd(madd(0.0579354987f, t, 0.763007998f), t, 1.0f);
}
__device__ __forceinline__ float atan(float x) {
    const float a = fabsf(x);
    const float k = a > 1.0f ? 1.0f / a : a;
    float r = atan_core(1.0f - (1.0f - k));
    if (a > 1.0f) r = 1.570796326794896557998982f - r;
    return copysignf(r, x);
}
__device__ __forceinline__ float atan2(float y, float x) {
    const float a = fabsf(x), b = fabsf(y);
    const bool steep = b > a;
    const float k = b == 0.0f ? 0.0f : (a == b ? 1.0f : (steep ? a / b : b / a));
    float r = atan_core(1.0f - (1.0f - k));
    if (steep) r = 1.570796326794896557998982f - r;
    if (__float_as_uint(x) & 0x80000000u) r = 3.14159265358979323846f - r;
    return copysignf(r, y);
}
__device__ __forceinline__ float sinh(float x) {
    float a = fabsf(x);
    if (a > 1.0f) {
        const float e = exp(a);
        return copysignf(0.5f * e - 0.5f / e, x);
    }
    a = 1.0f - (1.0f - a);
    const float a2 = a * a;
    float r = 2.03945513931e-4f;
    r = madd(r, a2, 8.32990277558e-3f);
    r = madd(r, a2, 0.1666673421859f);
    r = madd(r * a, a2, a);
    return copysignf(r, x);
}
__device__ __forceinline__ float cosh(float x) {
    const float e = exp(fabsf(x));
    return 0.5f * e + 0.5f / e;
}
__device__ __forceinline__ float tanh(float x) {
    const float e = exp(2.0f * fabsf(x));
    return copysignf(1.0f - 2.0f / (1.0f + e), x);
}

}  // namespace fm
}  // namespace dev
}  // namespace oslg
