// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of:
//   * SplineInterp::evaluate and the basis set (src/liboslexec/splineimpl.h:
//     43-83, :191-239), with OIIO::clamp(x, 0, 1) on Dual2 values;
//   * testrender's BSDF evaluation for the lobes the benchmark groups use:
//     Diffuse<0>::eval (src/testrender/shading.cpp:301-320),
//     Microfacet<GGXDist,0>::eval (:571-613, helpers :712-760, GGXDist
//     :472-508), fresnel_dielectric (src/testrender/optics.h:13-30),
//     TangentFrame (src/testrender/sampling.h:15-60), CompositeBSDF
//     prepare/eval (src/testrender/shading.h:322-374) and
//     MIS::update_eval (src/testrender/sampling.h:175-205).
// Vectors follow Imath Vec3 semantics (normalize divides by the length).
#pragma once
#include <cmath>

#include "oracle_dual.h"

namespace oracle {

struct SplineBasis {
    int step;
    float m[4][4];
};
inline const SplineBasis& spline_basis(int id) {
    static const SplineBasis set[6] = {
        { 1, { { -1.0f / 2.0f, 3.0f / 2.0f, -3.0f / 2.0f, 1.0f / 2.0f },
               { 2.0f / 2.0f, -5.0f / 2.0f, 4.0f / 2.0f, -1.0f / 2.0f },
               { -1.0f / 2.0f, 0.0f / 2.0f, 1.0f / 2.0f, 0.0f / 2.0f },
               { 0.0f / 2.0f, 2.0f / 2.0f, 0.0f / 2.0f, 0.0f / 2.0f } } },
        { 3, { { -1, 3, -3, 1 }, { 3, -6, 3, 0 }, { -3, 3, 0, 0 }, { 1, 0, 0, 0 } } },
        { 1, { { -1.0f / 6.0f, 3.0f / 6.0f, -3.0f / 6.0f, 1.0f / 6.0f },
               { 3.0f / 6.0f, -6.0f / 6.0f, 3.0f / 6.0f, 0.0f / 6.0f },
               { -3.0f / 6.0f, 0.0f / 6.0f, 3.0f / 6.0f, 0.0f / 6.0f },
               { 1.0f / 6.0f, 4.0f / 6.0f, 1.0f / 6.0f, 0.0f / 6.0f } } },
        { 2, { { 2, 1, -2, 1 }, { -3, -2, 3, -1 }, { 0, 1, 0, 0 }, { 1, 0, 0, 0 } } },
        { 1, { { 0, 0, 0, 0 }, { 0, 0, 0, 0 }, { 0, -1, 1, 0 }, { 0, 1, 0, 0 } } },
        { 1, { { 0, 0, 0, 0 }, { 0, 0, 0, 0 }, { 0, 0, 0, 0 }, { 0, 0, 0, 0 } } },
    };
    return set[(id >= 0 && id < 6) ? id : 0];
}

// One channel of SplineInterp::evaluate. knot(k) returns knot k (Dual2 if
// the knots carry derivatives). Returns the channel value (Dual2).
template <class KnotFn>
inline DF spline_channel(int basis, DF xval, bool x_derivs, bool knot_derivs, int knot_count, KnotFn knot) {
    const SplineBasis& B = spline_basis(basis);
    DF x = xval;
    if (!(0.0f <= x.v)) x = DF(0.0f);   // OIIO::clamp, lower bound first
    if (x.v > 1.0f) x = DF(1.0f);
    int nsegs = ((knot_count - 4) / B.step) + 1;
    x = x * (float)nsegs;
    int segnum = (int)x.v;
    if (segnum < 0) segnum = 0;
    if (segnum > nsegs - 1) segnum = nsegs - 1;
    if (basis == 5) return DF(knot(segnum + 1).v);
    x = x - (float)segnum;
    int s = segnum * B.step;
    DF P[4];
    for (int k = 0; k < 4; ++k) P[k] = knot(s + k);
    DF tk[4];
    for (int k = 0; k < 4; ++k) tk[k] = B.m[k][0] * P[0] + B.m[k][1] * P[1] + B.m[k][2] * P[2] + B.m[k][3] * P[3];
    if (!x_derivs && !knot_derivs) {
        float t = tk[0].v * x.v + tk[1].v;
        t = t * x.v + tk[2].v;
        t = t * x.v + tk[3].v;
        return DF(t);
    }
    if (!knot_derivs) {
        DF t = tk[0].v * x + tk[1].v;
        t = t * x + tk[2].v;
        t = t * x + tk[3].v;
        return t;
    }
    DF t = tk[0] * x + tk[1];
    t = t * x + tk[2];
    t = t * x + tk[3];
    return t;
}

// ---- BSDFs -----------------------------------------------------------------------
inline float dotv(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 crossv(const V3& a, const V3& b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float imath_len(const V3& a) {
    float l2 = dotv(a, a);
    if (l2 < 2.0f * 1.17549435e-38f) {
        float m = std::max(std::fabs(a.x), std::max(std::fabs(a.y), std::fabs(a.z)));
        if (m == 0.0f) return 0.0f;
        V3 b(a.x / m, a.y / m, a.z / m);
        return m * std::sqrt(dotv(b, b));
    }
    return std::sqrt(l2);
}
inline V3 imath_normalize(const V3& a) {
    float l = imath_len(a);
    if (l == 0.0f) return a;
    return V3(a.x / l, a.y / l, a.z / l);
}

struct TangentFrame {
    V3 u, v, w;
    static TangentFrame from_normal(const V3& n) {
        const float sign = std::copysign(1.0f, n.z);
        const float a = -1.0f / (sign + n.z);
        const float b = n.x * n.y * a;
        return { V3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x), V3(b, sign + n.y * n.y * a, -n.y), n };
    }
    static TangentFrame from_normal_and_tangent(const V3& n, const V3& t) {
        V3 x = t - n * dotv(n, t);
        float xlen2 = dotv(x, x);
        if (xlen2 > 0.0f) {
            x = x * (1.0f / std::sqrt(xlen2));
            return { x, crossv(n, x), n };
        }
        return from_normal(n);
    }
    V3 tolocal(const V3& a) const { return V3(dotv(a, u), dotv(a, v), dotv(a, w)); }
};

inline float fresnel_dielectric(float cosi, float eta) {
    if (eta == 0.0f) return 1.0f;
    if (cosi < 0.0f) eta = 1.0f / eta;
    float c = std::fabs(cosi);
    float g = eta * eta - 1.0f + c * c;
    if (g > 0.0f) {
        g = std::sqrt(g);
        float A = (g - c) / (g + c);
        float B = (c * (g + c) - 1.0f) / (c * (g - c) + 1.0f);
        return 0.5f * A * A * (1.0f + B * B);
    }
    return 1.0f;
}

struct Sample {
    V3 wi = V3(0.0f);
    V3 weight = V3(0.0f);
    float pdf = 0.0f;
    float roughness = 0.0f;
};

inline Sample diffuse_eval(const V3& N, const V3& wi) {
    Sample s;
    s.weight = V3(1.0f);
    s.pdf = std::max(dotv(N, wi), 0.0f) * float(M_1_PI);
    s.roughness = 1.0f;
    return s;
}

struct MicrofacetGGXRefl {
    V3 N, U;
    float xalpha, yalpha, eta;
    TangentFrame tf;
    MicrofacetGGXRefl(const V3& n, const V3& u, float ax, float ay, float e)
        : N(n), U(u), xalpha(ax), yalpha(ay), eta(e), tf(TangentFrame::from_normal_and_tangent(n, u)) {}
    static float SQR(float x) { return x * x; }
    static float F(float tan_m2) { return 1 / (float(M_PI) * (1 + tan_m2) * (1 + tan_m2)); }
    static float Lambda(float a2) { return 0.5f * (-1.0f + std::sqrt(1.0f + 1.0f / a2)); }
    float evalLambda(const V3& w) const {
        float cosTheta2 = SQR(w.z);
        float cosPhi2st2 = SQR(w.x * xalpha);
        float sinPhi2st2 = SQR(w.y * yalpha);
        return Lambda(cosTheta2 / (cosPhi2st2 + sinPhi2st2));
    }
    float evalD(const V3& Hr) const {
        float cosThetaM = Hr.z;
        if (cosThetaM > 0) {
            float cosPhi2st2 = SQR(Hr.x / xalpha);
            float sinPhi2st2 = SQR(Hr.y / yalpha);
            float cosThetaM2 = SQR(cosThetaM);
            float cosThetaM4 = SQR(cosThetaM2);
            float tanThetaM2 = (cosPhi2st2 + sinPhi2st2) / cosThetaM2;
            const float val = F(tanThetaM2) / (xalpha * yalpha * cosThetaM4);
            return (val == val) ? val : 0;
        }
        return 0;
    }
    V3 albedo(const V3& wo) const { return V3(fresnel_dielectric(dotv(N, wo), eta)); }
    Sample eval(const V3& wo, const V3& wi) const {
        const V3 wo_l = tf.tolocal(wo);
        const V3 wi_l = tf.tolocal(wi);
        Sample s;
        if (wo_l.z > 0 && wi_l.z > 0) {
            const V3 m = imath_normalize(wi_l + wo_l);
            const float D = evalD(m);
            const float Lo = evalLambda(wo_l);
            const float Li = evalLambda(wi_l);
            const float G2 = 1 / (Lo + Li + 1);
            const float G1 = 1 / (Lo + 1);
            const float Fr = fresnel_dielectric(dotv(m, wo_l), eta);
            s.pdf = (G1 * D * 0.25f) / wo_l.z;
            float out = G2 / G1;
            s.weight = V3(out * Fr);
            s.roughness = std::max(xalpha, yalpha);
        }
        return s;
    }
};

inline void mis_update_eval(V3* w, float* pdf, V3 ow, float opdf, float b) {
    if (b > 1.17549435e-38f) {
        opdf *= b;
        ow = ow * (1 / b);
        float mis;
        if (*pdf < opdf) mis = 1 / (1 + *pdf / opdf);
        else if (opdf < *pdf) mis = 1 - 1 / (1 + opdf / *pdf);
        else mis = 0.5f;
        *w = *w * (1 - mis) + ow * mis;
        *pdf += opdf;
    }
}

}  // namespace oracle
