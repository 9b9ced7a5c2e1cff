// Test infrastructure: the oracle's restatement of OpenImageIO 3.0's fast
// float transcendentals (OpenImageIO/fmath.h, fast_* functions), which the
// reference calls for its transcendental ops in the default build
// (USE_FAST_MATH=ON: CMakeLists.txt:145-150,
// src/liboslexec/wide/wide_optranscendental.cpp:34-66,
// wide_optrigonometric.cpp:16-47, constant folding constfold.cpp:1786-1818).
// OpenImageIO is a dependency outside the reference tree; these follow its
// published algorithms (Cody-Waite reduction and minimax polynomials for
// sin/cos/tan after SLEEF, exponent/mantissa split for exp2/log2,
// Abramowitz & Stegun 7.1.28 for erf, Hacker's Delight cube root) with
// unfused multiply-adds. Pinned by testsuite/exponential (exp2 and erfc
// differ from correctly rounded values in the printed digits) and
// testsuite/hyperb.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle_fm {

inline uint32_t ubits(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
inline float ufloat(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }
// unfused: the oracle is built with -ffp-contract=off
inline float mad(float a, float b, float c) { return a * b + c; }
const float kMinF = 1.17549435e-38f, kMaxF = 3.40282347e+38f;
// OpenImageIO's clamp: a NaN becomes the low bound
inline float clamp_lo_nan(float v, float lo, float hi) {
    if (!(lo <= v)) v = lo;
    if (!(v <= hi)) v = hi;
    return v;
}

inline float exp2f_(float xv) {
    float x = clamp_lo_nan(xv, -126.0f, 126.0f);
    int m = (int)x;
    x = x - (float)m;
    x = 1.0f - (1.0f - x);
    float r = 1.33336498402e-3f;
    r = mad(x, r, 9.810352697968e-3f);
    r = mad(x, r, 5.551834031939e-2f);
    r = mad(x, r, 0.2401793301105f);
    r = mad(x, r, 0.693144857883f);
    r = mad(x, r, 1.0f);
    return ufloat(ubits(r) + ((uint32_t)m << 23));
}
inline float expf_(float x) { return exp2f_(x * 1.44269504088896340736f); }
inline float expm1f_(float x) {
    if (std::fabs(x) < 1e-5f) {
        x = 1.0f - (1.0f - x);
        return mad(0.5f, x * x, x);
    }
    return expf_(x) - 1.0f;
}
inline float log2f_(float xv) {
    float x = clamp_lo_nan(xv, kMinF, kMaxF);
    uint32_t b = ubits(x);
    int e = (int)(b >> 23) - 127;
    float f = ufloat((b & 0x007FFFFFu) | 0x3f800000u) - 1.0f;
    float f2 = f * f;
    float f4 = f2 * f2;
    float hi = mad(f, -0.00931049621349f, 0.05206469089414f);
    float lo = mad(f, 0.47868480909345f, -0.72116591947498f);
    hi = mad(f, hi, -0.13753123777116f);
    hi = mad(f, hi, 0.24187369696082f);
    hi = mad(f, hi, -0.34730547155299f);
    lo = mad(f, lo, 1.442689881667200f);
    float p = f4 * hi;
    float q = f * lo;
    return (p + q) + (float)e;
}
inline float logf_(float x) { return log2f_(x) * 0.693147180559945309417f; }
inline float log10f_(float x) { return log2f_(x) * 0.301029995663981195214f; }
inline float safe_powf_(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return 0.0f;
    if (y == 1.0f) return x;
    if (y == 2.0f) { float s = x * x; return s < kMaxF ? s : kMaxF; }
    float sign = 1.0f;
    if (x < 0.0f) {
        int32_t yb;
        std::memcpy(&yb, &y, 4);
        yb &= 0x7fffffff;
        if (yb >= 0x4b800000) {
            // |y| >= 2^24: an even integer
        } else if (yb >= 0x3f800000) {
            int k = (yb >> 23) - 127;
            int j = yb >> (23 - k);
            if ((j << (23 - k)) != yb) return 0.0f;
            sign = ufloat(0x3f800000u | ((uint32_t)j << 31));
        } else {
            return 0.0f;
        }
    }
    return sign * exp2f_(y * log2f_(std::fabs(x)));
}
inline float erff_(float x) {
    const float c1 = 0.0705230784f, c2 = 0.0422820123f, c3 = 0.0092705272f, c4 = 0.0001520143f,
                c5 = 0.0002765672f, c6 = 0.0000430638f;
    float a = std::fabs(x);
    float b = 1.0f - (1.0f - a);
    float r = mad(mad(mad(mad(mad(mad(c6, b, c5), b, c4), b, c3), b, c2), b, c1), b, 1.0f);
    float s = r * r, t = s * s, u = t * t, v = u * u;
    return std::copysign(1.0f - 1.0f / v, x);
}
inline float erfcf_(float x) { return 1.0f - erff_(x); }
inline float cbrtf_(float x) {
    float x0 = std::fabs(x);
    int32_t xi;
    std::memcpy(&xi, &x0, 4);
    float a = ufloat((uint32_t)(0x2a5137a0 + xi / 3));
    a = 0.333333333f * (2.0f * a + x0 / (a * a));
    a = 0.333333333f * (2.0f * a + x0 / (a * a));
    if (x0 == 0.0f) a = 0.0f;
    return std::copysign(a, x);
}
// round half away from zero, saturated to the int range (NaN to its low end)
inline int round_half_away(float x) {
    float t = x + std::copysign(0.5f, x);
    if (!(t >= -2147483648.0f)) t = -2147483648.0f;
    if (!(t < 2147483648.0f)) t = 2147483520.0f;
    return (int)t;
}
// x - q * (pi/4) * scale, the constant split in four
inline float cody_waite(float x, float q, float scale) {
    x = mad(q, -0.78515625f * scale, x);
    x = mad(q, -0.00024187564849853515625f * scale, x);
    x = mad(q, -3.7747668102383613586e-08f * scale, x);
    x = mad(q, -1.2816720341285448015e-12f * scale, x);
    return x;
}
inline void sincosf_(float x, float& sine, float& cosine) {
    int q = round_half_away(x * 0.318309886183790671538f);
    x = cody_waite(x, (float)q, 4.0f);
    x = 1.57079632679489661923f - (1.57079632679489661923f - x);
    float s = x * x;
    if (q & 1) x = -x;
    float su = 2.6083159809786593541503e-06f;
    su = mad(su, s, -0.0001981069071916863322258f);
    su = mad(su, s, 0.00833307858556509017944336f);
    su = mad(su, s, -0.166666597127914428710938f);
    su = mad(s, su * x, x);
    float cu = -2.71811842367242206819355e-07f;
    cu = mad(cu, s, 2.47990446951007470488548e-05f);
    cu = mad(cu, s, -0.00138888787478208541870117f);
    cu = mad(cu, s, 0.0416666641831398010253906f);
    cu = mad(cu, s, -0.5f);
    cu = mad(cu, s, 1.0f);
    if (q & 1) cu = -cu;
    sine = std::fabs(su) > 1.0f ? 0.0f : su;
    cosine = std::fabs(cu) > 1.0f ? 0.0f : cu;
}
inline float sinf_(float x) { float s, c; sincosf_(x, s, c); return s; }
inline float cosf_(float x) { float s, c; sincosf_(x, s, c); return c; }
inline float tanf_(float x) {
    int q = round_half_away(x * 0.636619772367581343076f);
    x = cody_waite(x, (float)q, 2.0f);
    if ((q & 1) == 0) x = 0.785398163397448309616f - (0.785398163397448309616f - x);
    float s = x * x;
    float u = 0.00927245803177356719970703f;
    u = mad(u, s, 0.00331984995864331722259521f);
    u = mad(u, s, 0.0242998078465461730957031f);
    u = mad(u, s, 0.0534495301544666290283203f);
    u = mad(u, s, 0.133383005857467651367188f);
    u = mad(u, s, 0.333331853151321411132812f);
    u = mad(s, u * x, x);
    if (q & 1) u = -1.0f / u;
    return u;
}
inline float acos_poly(float m) {
    return std::sqrt(1.0f - m) * (1.5707963267f + m * (-0.213300989f + m * (0.077980478f + m * -0.02164095f)));
}
inline float acosf_(float x) {
    float f = std::fabs(x);
    float m = f < 1.0f ? 1.0f - (1.0f - f) : 1.0f;
    float a = acos_poly(m);
    return x < 0.0f ? 3.14159265358979323846f - a : a;
}
inline float asinf_(float x) {
    float f = std::fabs(x);
    float m = f < 1.0f ? 1.0f - (1.0f - f) : 1.0f;
    return std::copysign(1.57079632679489661923f - acos_poly(m), x);
}
inline float atan_ratio(float s) {
    float t = s * s;
    return s * mad(0.430165678f, t, 1.0f) / mad(mad(0.0579354987f, t, 0.763007998f), t, 1.0f);
}
inline float atanf_(float x) {
    float a = std::fabs(x);
    float k = a > 1.0f ? 1.0f / a : a;
    float r = atan_ratio(1.0f - (1.0f - k));
    if (a > 1.0f) r = 1.570796326794896557998982f - r;
    return std::copysign(r, x);
}
inline float atan2f_(float y, float x) {
    float a = std::fabs(x), b = std::fabs(y);
    bool steep = b > a;
    float k = b == 0.0f ? 0.0f : (a == b ? 1.0f : (steep ? a / b : b / a));
    float r = atan_ratio(1.0f - (1.0f - k));
    if (steep) r = 1.570796326794896557998982f - r;
    if (ubits(x) & 0x80000000u) r = 3.14159265358979323846f - r;
    return std::copysign(r, y);
}
inline float sinhf_(float x) {
    float a = std::fabs(x);
    if (a > 1.0f) {
        float e = expf_(a);
        return std::copysign(0.5f * e - 0.5f / e, x);
    }
    a = 1.0f - (1.0f - a);
    float a2 = a * a;
    float r = 2.03945513931e-4f;
    r = mad(r, a2, 8.32990277558e-3f);
    r = mad(r, a2, 0.1666673421859f);
    r = mad(r * a, a2, a);
    return std::copysign(r, x);
}
inline float coshf_(float x) {
    float e = expf_(std::fabs(x));
    return 0.5f * e + 0.5f / e;
}
inline float tanhf_(float x) {
    float e = expf_(2.0f * std::fabs(x));
    return std::copysign(1.0f - 2.0f / (1.0f + e), x);
}

}  // namespace oracle_fm
