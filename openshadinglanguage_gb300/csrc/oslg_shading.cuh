// Device spline, closure-tree and BSDF code for the sm_103a interpreter.
//
// * spline: SplineInterp::evaluate (src/liboslexec/splineimpl.h:191-239)
//   with the basis set of splineimpl.h:43-83.
// * closures: the reference's closure tree (src/include/OSL/oslclosure.h:
//   65-147; allocation rules src/liboslexec/opclosure.cpp:19-117) kept in a
//   per-point node pool inside the symbol heap. A closure value is the node
//   index + 1 (0 is the null closure).
// * BSDF: testrender's closure walk (src/testrender/shading.cpp:1450-1500),
//   Diffuse (:301-320), GGX microfacet reflection (:472-508, :571-800),
//   fresnel_dielectric (optics.h:13-30), TangentFrame (sampling.h:15-60) and
//   CompositeBSDF prepare/eval with MIS::update_eval (shading.h:319-374,
//   sampling.h:175-205).
#pragma once
#include "oslg_noise.cuh"
#include "oslg_program.h"

namespace oslg {
namespace dev {

// ---- spline -------------------------------------------------------------------
struct SplineBasisDev {
    int step;
    float m[4][4];
};
static __constant__ SplineBasisDev c_spline_basis[6] = {
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

// ---- small vector helpers (Imath Vec3 semantics) -------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 vmul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
// Imath Vec3::length with the tiny-vector rescale
__device__ __forceinline__ float vlen_imath(V3 a) {
    float l2 = vdot(a, a);
    if (l2 < 2.0f * 1.17549435e-38f) {
        float m = fmaxf(fabsf(a.x), fmaxf(fabsf(a.y), fabsf(a.z)));
        if (m == 0.0f) return 0.0f;
        V3 b = v3(a.x / m, a.y / m, a.z / m);
        return m * sqrtf(vdot(b, b));
    }
    return sqrtf(l2);
}
// Imath Vec3::normalize(): divide each component by the length
__device__ __forceinline__ V3 vnormalize_imath(V3 a) {
    float l = vlen_imath(a);
    if (l == 0.0f) return a;
    return v3(a.x / l, a.y / l, a.z / l);
}

// TangentFrame (sampling.h:15-60)
struct Frame {
    V3 u, v, w;
};
__device__ __forceinline__ Frame frame_from_normal(V3 n) {
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = n.x * n.y * a;
    Frame f;
    f.u = v3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.v = v3(b, sign + n.y * n.y * a, -n.y);
    f.w = n;
    return f;
}
__device__ __forceinline__ Frame frame_from_normal_and_tangent(V3 n, V3 t) {
    V3 x = vsub(t, vmul(n, vdot(n, t)));
    float xlen2 = vdot(x, x);
    if (xlen2 > 0.0f) {
        x = vmul(x, 1.0f / sqrtf(xlen2));
        Frame f;
        f.u = x;
        f.v = vcross(n, x);
        f.w = n;
        return f;
    }
    return frame_from_normal(n);
}
__device__ __forceinline__ V3 tolocal(const Frame& f, V3 a) { return v3(vdot(a, f.u), vdot(a, f.v), vdot(a, f.w)); }

// optics.h:13-30
__device__ __forceinline__ float fresnel_dielectric(float cosi, float eta) {
    if (eta == 0.0f) return 1.0f;
    if (cosi < 0.0f) eta = 1.0f / eta;
    float c = fabsf(cosi);
    float g = eta * eta - 1.0f + c * c;
    if (g > 0.0f) {
        g = sqrtf(g);
        float A = (g - c) / (g + c);
        float B = (c * (g + c) - 1.0f) / (c * (g - c) + 1.0f);
        return 0.5f * A * A * (1.0f + B * B);
    }
    return 1.0f;
}

struct BsdfSample {
    float w[3];
    float pdf;
    float roughness;
};

// Diffuse<0>::eval (shading.cpp:307-311)
__device__ __forceinline__ BsdfSample diffuse_eval(V3 N, V3 wi) {
    BsdfSample s;
    const float pdf = fmaxf(vdot(N, wi), 0.0f) * 0.318309886183790671538f;
    s.w[0] = s.w[1] = s.w[2] = 1.0f;
    s.pdf = pdf;
    s.roughness = 1.0f;
    return s;
}

// Microfacet<GGXDist, 0>::eval (shading.cpp:589-613 + helpers :712-760)
__device__ __forceinline__ float ggx_F(float tan_m2) {
    return 1.0f / (3.14159265358979323846f * (1.0f + tan_m2) * (1.0f + tan_m2));
}
__device__ __forceinline__ float ggx_Lambda(float a2) { return 0.5f * (-1.0f + sqrtf(1.0f + 1.0f / a2)); }
__device__ __forceinline__ float mf_lambda(V3 w, float ax, float ay) {
    float cosTheta2 = w.z * w.z;
    float c = w.x * ax, s = w.y * ay;
    return ggx_Lambda(cosTheta2 / (c * c + s * s));
}
__device__ __forceinline__ float mf_D(V3 m, float ax, float ay) {
    float cosThetaM = m.z;
    if (cosThetaM > 0.0f) {
        float cx = m.x / ax, sy = m.y / ay;
        float cosPhi2st2 = cx * cx, sinPhi2st2 = sy * sy;
        float cosThetaM2 = cosThetaM * cosThetaM;
        float cosThetaM4 = cosThetaM2 * cosThetaM2;
        float tanThetaM2 = (cosPhi2st2 + sinPhi2st2) / cosThetaM2;
        const float val = ggx_F(tanThetaM2) / (ax * ay * cosThetaM4);
        return (val == val) ? val : 0.0f;
    }
    return 0.0f;
}
__device__ __forceinline__ BsdfSample microfacet_ggx_refl_eval(const Frame& tf, float ax, float ay, float eta,
                                                               V3 wo, V3 wi) {
    BsdfSample s;
    s.w[0] = s.w[1] = s.w[2] = 0.0f;
    s.pdf = 0.0f;
    s.roughness = 0.0f;
    const V3 wo_l = tolocal(tf, wo);
    const V3 wi_l = tolocal(tf, wi);
    if (wo_l.z > 0.0f && wi_l.z > 0.0f) {
        const V3 m = vnormalize_imath(vadd(wi_l, wo_l));
        const float D = mf_D(m, ax, ay);
        const float Lo = mf_lambda(wo_l, ax, ay);
        const float Li = mf_lambda(wi_l, ax, ay);
        const float G2 = 1.0f / (Lo + Li + 1.0f);
        const float G1 = 1.0f / (Lo + 1.0f);
        const float Fr = fresnel_dielectric(vdot(m, wo_l), eta);
        float pdf = (G1 * D * 0.25f) / wo_l.z;
        float out = G2 / G1;
        float w = out * Fr;
        s.w[0] = s.w[1] = s.w[2] = w;
        s.pdf = pdf;
        s.roughness = fmaxf(ax, ay);
    }
    return s;
}

// MIS::update_eval (sampling.h:175-205)
__device__ __forceinline__ void mis_update_eval(float* w, float* pdf, const float* ow_in, float opdf, float b) {
    if (b > 1.17549435e-38f) {
        opdf *= b;
        float inv = 1.0f / b;
        float ow[3] = { ow_in[0] * inv, ow_in[1] * inv, ow_in[2] * inv };
        float mis;
        if (*pdf < opdf) mis = 1.0f / (1.0f + *pdf / opdf);
        else if (opdf < *pdf) mis = 1.0f - 1.0f / (1.0f + opdf / *pdf);
        else mis = 0.5f;
        for (int c = 0; c < 3; ++c) w[c] = w[c] * (1.0f - mis) + ow[c] * mis;
        *pdf += opdf;
    }
}

}  // namespace dev
}  // namespace oslg
