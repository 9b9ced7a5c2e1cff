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
#include "oslg_fastmath.cuh"
#include "oslg_fmath.cuh"
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
    V3 wi;
};
__device__ __forceinline__ BsdfSample bsdf_zero() {
    BsdfSample s;
    s.w[0] = s.w[1] = s.w[2] = 0.0f;
    s.pdf = 0.0f;
    s.roughness = 0.0f;
    s.wi = v3(0.0f, 0.0f, 0.0f);
    return s;
}

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


// ---- sampling (wavefront path step) ------------------------------------------------
// TangentFrame::get (sampling.h:44-47)
__device__ __forceinline__ V3 frame_get(const Frame& f, float x, float y, float z) {
    return vadd(vadd(vmul(f.u, x), vmul(f.v, y)), vmul(f.w, z));
}
__device__ __forceinline__ V3 vneg(V3 a) { return v3(-a.x, -a.y, -a.z); }

// Sampling::to_unit_disk / sample_cosine_hemisphere (sampling.h:70-100); the
// reference's OIIO::fast_sincos is the executor's own sincos here
__device__ __forceinline__ void to_unit_disk(float& x, float& y) {
    const float PI_OVER_4 = 0.785398163397448309616f, PI_OVER_2 = 1.57079632679489661923f;
    float phi, r;
    const float a = 2 * x - 1, b = 2 * y - 1;
    if (a * a > b * b) {
        r = a;
        phi = PI_OVER_4 * (b / a);
    } else if (b != 0) {
        r = b;
        phi = PI_OVER_2 - PI_OVER_4 * (a / b);
    } else {
        r = 0;
        phi = 0;
    }
    own_sincos(phi, &x, &y);
    x *= r;
    y *= r;
}
// Diffuse<0>::sample (shading.cpp:313-319)
__device__ __forceinline__ BsdfSample diffuse_sample(V3 N, float rx, float ry) {
    to_unit_disk(rx, ry);
    const float cos_theta = sqrtf(fmaxf(1 - rx * rx - ry * ry, 0.0f));
    BsdfSample s;
    s.wi = frame_get(frame_from_normal(N), rx, ry, cos_theta);
    s.pdf = cos_theta * 0.318309886183790671538f;
    s.w[0] = s.w[1] = s.w[2] = 1.0f;
    s.roughness = 1.0f;
    return s;
}

// optics.h:34-66
__device__ __forceinline__ float fresnel_refraction(V3 I, V3 N, float eta, V3* T) {
    float cosi = -vdot(I, N);
    V3 Nn;
    float neta;
    if (cosi > 0) {
        neta = 1 / eta;
        Nn = N;
    } else {
        cosi = -cosi;
        neta = eta;
        Nn = vneg(N);
    }
    const float arg = 1.0f - (neta * neta * (1.0f - cosi * cosi));
    if (arg >= 0) {
        const float dnp = sqrtf(arg);
        const float nK = (neta * cosi) - dnp;
        *T = vadd(vmul(I, neta), vmul(Nn, nK));
        return 1 - fresnel_dielectric(cosi, eta);
    }
    *T = v3(0.0f, 0.0f, 0.0f);
    return 0;
}

struct GGXLobe {
    Frame tf;
    float ax, ay, eta;
    int refract;
};
__device__ __forceinline__ float ggx_D(const GGXLobe& g, V3 m) { return mf_D(m, g.ax, g.ay); }
__device__ __forceinline__ float ggx_albedo(const GGXLobe& g, V3 N, V3 wo) {
    if (g.refract == 2) return 1.0f;
    const float fr = fresnel_dielectric(vdot(N, wo), g.eta);
    return g.refract ? 1 - fr : fr;
}
// Microfacet<GGXDist, Refract>::eval (shading.cpp:589-652)
__device__ __forceinline__ BsdfSample ggx_eval(const GGXLobe& g, V3 wo, V3 wi) {
    const V3 wo_l = tolocal(g.tf, wo), wi_l = tolocal(g.tf, wi);
    BsdfSample s = bsdf_zero();
    s.wi = wi;
    if (g.refract == 0 || g.refract == 2) {
        if (wo_l.z > 0 && wi_l.z > 0) {
            const V3 m = vnormalize_imath(vadd(wi_l, wo_l));
            const float D = ggx_D(g, m);
            const float Lo = mf_lambda(wo_l, g.ax, g.ay), Li = mf_lambda(wi_l, g.ax, g.ay);
            const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
            const float Fr = fresnel_dielectric(vdot(m, wo_l), g.eta);
            const float pdf = (G1 * D * 0.25f) / wo_l.z;
            const float out = G2 / G1;
            s.roughness = fmaxf(g.ax, g.ay);
            if (g.refract == 2) {
                s.pdf = pdf * Fr;
                s.w[0] = s.w[1] = s.w[2] = out;
            } else {
                s.pdf = pdf;
                s.w[0] = s.w[1] = s.w[2] = out * Fr;
            }
            return s;
        }
    }
    if (g.refract == 1 || g.refract == 2) {
        if (wi_l.z < 0 && wo_l.z > 0.0f) {
            V3 ht = vneg(vadd(vmul(wi_l, g.eta), wo_l));
            if (g.eta < 1.0f) ht = vneg(ht);
            const V3 Ht = vnormalize_imath(ht);
            const float cosHO = vdot(Ht, wo_l);
            const float Ft = 1.0f - fresnel_dielectric(cosHO, g.eta);
            if (Ft > 0) {
                const float cosHI = vdot(Ht, wi_l);
                if (Ht.z <= 0.0f) return bsdf_zero();
                const float Dt = ggx_D(g, Ht);
                const float Lo = mf_lambda(wo_l, g.ax, g.ay), Li = mf_lambda(wi_l, g.ax, g.ay);
                const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
                const float invHt2 = 1 / vdot(ht, ht);
                const float pdf = (fabsf(cosHI * cosHO) * (g.eta * g.eta) * (G1 * Dt) * invHt2) / wo_l.z;
                const float out = G2 / G1;
                s.roughness = fmaxf(g.ax, g.ay);
                if (g.refract == 2) {
                    s.pdf = pdf * Ft;
                    s.w[0] = s.w[1] = s.w[2] = out;
                } else {
                    s.pdf = pdf;
                    s.w[0] = s.w[1] = s.w[2] = out * Ft;
                }
                return s;
            }
        }
    }
    return bsdf_zero();
}
// GGXDist::sampleSlope (shading.cpp:480-508)
__device__ __forceinline__ void ggx_sample_slope(float cos_theta, float randu, float randv, float* sx, float* sy) {
    const float c = cos_theta < 1e-6f ? 1e-6f : cos_theta;
    const float Q = (1 + c) * randu - c;
    const float num = c * sqrtf((1 - c) * (1 + c)) - Q * sqrtf((1 - Q) * (1 + Q));
    float den = (Q - c) * (Q + c);
    const float eps = 1.0f / 4294967296.0f;
    den = fabsf(den) < eps ? copysignf(eps, den) : den;
    *sx = num / den;
    const float Ru = 1 - 2 * randv;
    const float u2 = fabsf(Ru);
    const float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f))
                  / (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.0f) + 0.597999f);
    *sy = copysignf(1.0f, Ru) * z * sqrtf(1.0f + *sx * *sx);
}
// Microfacet::sampleMicronormal (shading.cpp:754-787)
__device__ __forceinline__ V3 ggx_sample_micronormal(const GGXLobe& g, V3 wo, float randu, float randv) {
    V3 swo = wo;
    swo.x *= g.ax;
    swo.y *= g.ay;
    swo = vnormalize_imath(swo);
    const float cos_theta = fmaxf(swo.z, 0.0f);
    float cos_phi = 1, sin_phi = 0;
    if (cos_theta < 0.99999f) {
        const float invnorm = 1 / sqrtf(swo.x * swo.x + swo.y * swo.y);
        cos_phi = swo.x * invnorm;
        sin_phi = swo.y * invnorm;
    }
    float slx, sly;
    ggx_sample_slope(cos_theta, randu, randv, &slx, &sly);
    float sx = cos_phi * slx - sin_phi * sly;
    float sy = sin_phi * slx + cos_phi * sly;
    sx *= g.ax;
    sy *= g.ay;
    const float mlen = sqrtf(sx * sx + sy * sy + 1);
    return v3(fabsf(sx) < mlen ? -sx / mlen : 1.0f, fabsf(sy) < mlen ? -sy / mlen : 1.0f, 1.0f / mlen);
}
// Microfacet::sample (shading.cpp:628-700)
__device__ __forceinline__ BsdfSample ggx_sample(const GGXLobe& g, V3 wo, float rx, float ry, float rz) {
    const V3 wo_l = tolocal(g.tf, wo);
    const float cosNO = wo_l.z;
    if (!(cosNO > 0)) return bsdf_zero();
    const V3 m = ggx_sample_micronormal(g, wo_l, rx, ry);
    const float cosMO = vdot(m, wo_l);
    const float F = fresnel_dielectric(cosMO, g.eta);
    BsdfSample s = bsdf_zero();
    if (g.refract == 0 || (g.refract == 2 && rz < F)) {
        const V3 wi_l = vsub(vmul(m, 2.0f * cosMO), wo_l);
        const float D = ggx_D(g, m);
        const float Lo = mf_lambda(wo_l, g.ax, g.ay), Li = mf_lambda(wi_l, g.ax, g.ay);
        const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
        s.wi = frame_get(g.tf, wi_l.x, wi_l.y, wi_l.z);
        const float pdf = (G1 * D * 0.25f) / cosNO;
        const float out = G2 / G1;
        s.roughness = fmaxf(g.ax, g.ay);
        if (g.refract == 2) {
            s.pdf = pdf * F;
            s.w[0] = s.w[1] = s.w[2] = out;
        } else {
            s.pdf = pdf;
            s.w[0] = s.w[1] = s.w[2] = F * out;
        }
        return s;
    }
    const V3 M = frame_get(g.tf, m.x, m.y, m.z);
    V3 wi;
    const float Ft = fresnel_refraction(vneg(wo), M, g.eta, &wi);
    const V3 wi_l = tolocal(g.tf, wi);
    const float cosHO = vdot(m, wo_l), cosHI = vdot(m, wi_l);
    const float D = ggx_D(g, m);
    const float Lo = mf_lambda(wo_l, g.ax, g.ay), Li = mf_lambda(wi_l, g.ax, g.ay);
    const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
    const V3 ht = vneg(vadd(vmul(wi_l, g.eta), wo_l));
    const float invHt2 = 1.0f / vdot(ht, ht);
    const float pdf = (fabsf(cosHI * cosHO) * (g.eta * g.eta) * (G1 * D) * invHt2) / fabsf(wo_l.z);
    const float out = G2 / G1;
    s.wi = wi;
    s.roughness = fmaxf(g.ax, g.ay);
    if (g.refract == 2) {
        s.pdf = pdf * Ft;
        s.w[0] = s.w[1] = s.w[2] = out;
    } else {
        s.pdf = pdf;
        s.w[0] = s.w[1] = s.w[2] = Ft * out;
    }
    return s;
}

// BSDL (libbsdl/include/BSDL/tools.h:196-275, :459-508; bsdf_impl.h:51-78)
__device__ __forceinline__ float bsdl_cos_quadrant(float x) {
    const float x2 = x * x;
    float cp = 0.01578646f + -0.00029826362f * x2;
    cp = -0.30837047f + cp * x2;
    cp = 0.99998736f + cp * x2;
    return cp;
}
__device__ __forceinline__ float bsdl_sin_quadrant(float x) {
    const float x2 = x * x;
    float sp = 0.0024843954015523195266723632812500f + -0.0000341485538228880614042282104492f * x2;
    sp = -0.0807407423853874206542968750000000f + sp * x2;
    sp = 0.7853975892066955566406250000000000f + sp * x2;
    return sp * x;
}
__device__ __forceinline__ V3 bsdl_sample_cos_hemisphere(float randu, float randv) {
    const float a = 2 * randu - 1, qa = fabsf(a);
    const float b = 2 * randv - 1, qb = fabsf(b);
    const float rad = qa > qb ? qa : qb;
    const float phi = qa > qb ? qb / qa : ((qa == qb) ? 1.0f : 2 - qa / qb);
    const float x = copysignf(rad * bsdl_cos_quadrant(phi), a);
    const float y = copysignf(rad * bsdl_sin_quadrant(phi), b);
    return v3(x, y, sqrtf(1 - rad * rad));
}
__device__ __forceinline__ Frame bsdl_frame(V3 z) {
    const float s = copysignf(1.0f, z.z);
    const float a = -1.0f / (s + z.z);
    const float b = z.x * z.y * a;
    Frame f;
    f.u = v3(1.0f + s * z.x * z.x * a, s * b, -s * z.x);
    f.v = v3(b, s + z.y * z.y * a, -z.y);
    f.w = z;
    return f;
}
__device__ __forceinline__ V3 bsdl_world(const Frame& f, V3 a) {
    return v3(f.u.x * a.x + f.v.x * a.y + f.w.x * a.z, f.u.y * a.x + f.v.y * a.y + f.w.y * a.z,
              f.u.z * a.x + f.v.z * a.y + f.w.z * a.z);
}
__device__ __forceinline__ float bsdl_max_abs(V3 v) { return fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z))); }
__device__ __forceinline__ V3 bsdl_visible_normal(V3 wo, V3 Ngf, V3 N) {
    if (vdot(wo, N) > 0.0f) return N;
    V3 V = vcross(wo, N);
    if (bsdl_max_abs(V) < 1e-4f) {
        V = vcross(wo, Ngf);
        if (bsdl_max_abs(V) < 1e-4f) {
            const float s = copysignf(1.0f, wo.z);
            const float a = -1.0f / (s + wo.z);
            V = v3(wo.x * wo.y * a, s + wo.y * wo.y * a, -wo.y);
        } else {
            V = vnormalize_imath(V);
        }
    } else {
        V = vnormalize_imath(V);
    }
    return vnormalize_imath(vadd(vcross(V, wo), vmul(wo, 1e-4f)));
}
__device__ __forceinline__ float bsdl_clamp(float x, float a, float b) { return fminf(fmaxf(x, a), b); }

// oren_nayar as testrender builds it: BSDL OrenNayarDiffuseLobe, energy
// compensation off, albedo 1 (libbsdl MTX/bsdf_oren_nayar_diffuse_impl.h:41-113)
__device__ __forceinline__ BsdfSample on_eval_local(float rough, V3 wo, V3 wi) {
    BsdfSample s = bsdf_zero();
    const float cosNI = bsdl_clamp(wi.z, 0.0f, 1.0f);
    const float cosNO = bsdl_clamp(wo.z, 0.0f, 1.0f);
    if (cosNI <= 0.0f || cosNO <= 0.0f) return s;
    const float cosIO = bsdl_clamp(vdot(wo, wi), -1.0f, 1.0f);
    const float sv = cosIO - cosNI * cosNO;
    const float pdf = cosNI * (1.0f / 3.14159265358979323846f);
    const float s2 = rough * rough;
    const float A = 1.0f - 0.50f * s2 / (s2 + 0.33f);
    const float B = 0.45f * s2 / (s2 + 0.09f);
    const float stinv = sv > 0.0f ? sv / fmaxf(cosNI, cosNO) : 0.0f;
    const float f_ss = A + B * stinv;
    s.wi = wi;
    s.w[0] = s.w[1] = s.w[2] = 1.0f * f_ss;
    s.pdf = pdf;
    s.roughness = 1.0f;
    return s;
}

// oren_nayar_diffuse_bsdf as testrender builds it: BSDL OrenNayarDiffuseLobe
// with the closure's albedo, and with energy_compensation the energy
// preserving "FON" form (libbsdl MTX/bsdf_oren_nayar_diffuse_impl.h:27-98:
// single scattering AF (1 + sigma s/max(cosNI, cosNO)) plus the multiple
// scattering term from the directional albedo E_FON). acos is evaluated
// in double precision and rounded, where BSDL calls its fast acos.
__device__ __forceinline__ float on_fon_E(float sigma, float mu) {
    constexpr float c1 = 0.5f - 2.0f / (3.0f * 3.14159265358979323846f);
    const float AF = 1.0f / (1.0f + c1 * sigma);
    const float BF = sigma * AF;
    const float Si = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    const float G = Si * ((float)acos((double)mu) - Si * mu)
                  + 2.0f * ((Si / fmaxf(mu, 1e-7f)) * (1.0f - Si * Si * Si) - Si) * (1.0f / 3.0f);
    return AF + (BF * (1 / 3.14159265358979323846f)) * G;
}
__device__ __forceinline__ BsdfSample on_mx_eval_local(float rough, const float* albedo, bool energy, V3 wo, V3 wi) {
    if (!energy) {
        BsdfSample s = on_eval_local(rough, wo, wi);
        for (int c = 0; c < 3; ++c) s.w[c] = albedo[c] * s.w[c];
        return s;
    }
    BsdfSample s = bsdf_zero();
    const float cosNI = bsdl_clamp(wi.z, 0.0f, 1.0f);
    const float cosNO = bsdl_clamp(wo.z, 0.0f, 1.0f);
    if (cosNI <= 0.0f || cosNO <= 0.0f) return s;
    const float cosIO = bsdl_clamp(vdot(wo, wi), -1.0f, 1.0f);
    const float sv = cosIO - cosNI * cosNO;
    const float pdf = cosNI * (1.0f / 3.14159265358979323846f);
    constexpr float c1 = 0.5f - 2.0f / (3.0f * 3.14159265358979323846f);
    constexpr float c2 = 2.0f / 3.0f - 28.0f / (15.0f * 3.14159265358979323846f);
    const float AF = 1.0f / (1.0f + c1 * rough);
    const float stinv = sv > 0.0f ? sv / fmaxf(cosNI, cosNO) : sv;
    const float f_ss = AF * (1.0f + rough * stinv);
    const float EFo = on_fon_E(rough, cosNO);
    const float EFi = on_fon_E(rough, cosNI);
    const float avgEF = AF * (1.0f + c2 * rough);
    const float f_ms = fmaxf(1e-7f, 1.0f - EFo) * fmaxf(1e-7f, 1.0f - EFi) / fmaxf(1e-7f, 1.0f - avgEF);
    for (int c = 0; c < 3; ++c) {
        const float a = albedo[c];
        const float rho_ms = (a * a) * avgEF / (1 - a * fmaxf(0.0f, 1.0f - avgEF));
        s.w[c] = a * f_ss + rho_ms * f_ms;
    }
    s.wi = wi;
    s.pdf = pdf;
    s.roughness = 1.0f;
    return s;
}

// sheen_bsdf as testrender builds it: BSDL mtx::SheenLobe (libbsdl
// MTX/bsdf_sheen_impl.h:19-80). Mode 0: Conty-Kulla with the MaterialX
// albedo fit and the non-legacy visibility term (:80-260; Conty Estevez and
// Kulla, "Production Friendly Microfacet Sheen BRDF", 2017; sin^(1/a) uses
// the executor's own float power where BSDL calls OIIO::fast_pow). Mode 1:
// Zeltner, Burley and Chiang, "Practical Multiple-Scattering Sheen Using
// Linearly Transformed Cosines" (2022): the LTC coefficients (A, B, R)
// bilinearly interpolated from the paper's 32 x 32 table over roughness and
// cos theta_o, sampled through the LTC, albedo R (:267-357).
struct SheenLobeDev {
    Frame f;
    float tint[3];
    float rough;  // regularized roughness (reported)
    float a;      // distribution roughness: [0.06, 1] (mode 0), [0.02, 1] (mode 1)
    float emiss;
    bool backfacing;
    bool zeltner;
};
static __constant__ float c_zeltner_ltc[32 * 32 * 3] = {
#include "oslg_zeltner_ltc.inc"
};
__device__ __forceinline__ void zeltner_fetch(float a, float cosNO, float* o) {
    const float almost_one = 0.999999940395355224609375f;
    const float row = bsdl_clamp(a, 0.0f, almost_one) * 31.0f;
    const float col = bsdl_clamp(cosNO, 0.0f, almost_one) * 31.0f;
    const float r = floorf(row), c = floorf(col);
    const float rf = bsdl_clamp(row - r, 0.0f, 1.0f), cf = bsdl_clamp(col - c, 0.0f, 1.0f);
    const int i0 = ((int)r * 32 + (int)c) * 3, i1 = i0 + 32 * 3;
    for (int k = 0; k < 3; ++k) {
        const float lo = (1 - cf) * c_zeltner_ltc[i0 + k] + cf * c_zeltner_ltc[i0 + 3 + k];
        const float hi = (1 - cf) * c_zeltner_ltc[i1 + k] + cf * c_zeltner_ltc[i1 + 3 + k];
        o[k] = (1 - rf) * lo + rf * hi;
    }
}
// the LTC evaluation at local direction wi with coefficients ltc
__device__ __forceinline__ BsdfSample zeltner_eval(float a, V3 wi, const float* ltc) {
    BsdfSample s = bsdf_zero();
    const float ai = ltc[0], bi = ltc[1];
    const V3 o = v3(ai * wi.x + bi * wi.z, ai * wi.y, wi.z);
    const float len2 = o.x * o.x + o.y * o.y + o.z * o.z;
    const float j = ai / len2;
    const float pdf = j * j * fmaxf(o.z, 0.0f) * (1.0f / 3.14159265358979323846f);
    if (pdf > 1.17549435e-38f) {
        s.wi = wi;
        s.w[0] = s.w[1] = s.w[2] = ltc[2];
        s.pdf = pdf;
        s.roughness = a;
    }
    return s;
}
__device__ __forceinline__ float sheen_albedo_fit(float c, float r) {
    float x = 13.67300f + -68.78018f * c;
    float y = 1.0f + 61.57746f * c;
    x = x + 799.08825f * r;
    y = y + 442.78211f * r;
    x = x + -905.00061f * c * r;
    y = y + 2597.49308f * c * r;
    x = x + 60.28956f * c * c;
    y = y + 121.81241f * c * c;
    x = x + 1086.96473f * r * r;
    y = y + 3045.55075f * r * r;
    return bsdl_clamp(x / y, 0.0f, 1.0f);
}
__device__ __forceinline__ SheenLobeDev sheen_make(V3 N, const float* albedo, float roughness, V3 wo,
                                                   float path_roughness, bool backfacing, int mode = 0) {
    SheenLobeDev L;
    L.f = bsdl_frame(bsdl_visible_normal(wo, N, N));
    for (int c = 0; c < 3; ++c) L.tint[c] = albedo[c];
    L.rough = 1.0f - (1.0f - bsdl_clamp(roughness, 0.0f, 1.0f)) * (1.0f - path_roughness);
    L.zeltner = mode == 1;
    L.a = L.zeltner ? bsdl_clamp(fmaxf(0.02f, sqrtf(L.rough)), 0.02f, 1.0f)
                    : bsdl_clamp(fmaxf(0.06f, L.rough), 0.06f, 1.0f);
    L.backfacing = backfacing;
    const float cosNO = bsdl_clamp(vdot(L.f.w, wo), 0.0f, 1.0f);
    const float tmax = fmaxf(fmaxf(L.tint[0], L.tint[1]), L.tint[2]);
    float alb;
    if (L.zeltner) {
        float ltc[3];
        zeltner_fetch(L.a, cosNO, ltc);
        alb = ltc[2];
    } else {
        alb = sheen_albedo_fit(cosNO, L.a);
    }
    L.emiss = backfacing ? 1.0f : 1.0f - fminf(alb * tmax, 1.0f);
    return L;
}
// SheenMicrofacet<ContyKullaDist<false>>::eval in the lobe frame
__device__ __forceinline__ BsdfSample sheen_mf_eval(float a, V3 wo, V3 wi) {
    BsdfSample s = bsdf_zero();
    const float cosNO = wo.z, cosNI = wi.z;
    if (cosNI <= 1e-5f || cosNO <= 1e-5f) return s;
    const V3 H = vnormalize_imath(vadd(wo, wi));
    const float ct = bsdl_clamp(H.z, 0.0f, 1.0f);
    const float st = sqrtf(1.0f - ct * ct);
    const float pi = 3.14159265358979323846f, one_over_pi = 1.0f / pi;
    const float D = own_pow_pos(st, 1 / a) * (2 + 1 / a) * 0.5f * one_over_pi;
    if (D < 1e-6f) return s;
    const float ci = fminf(1.0f, wi.z), co = fminf(1.0f, wo.z);
    const float G2 = (ci * co) / (ci + co - ci * co);
    s.wi = wi;
    s.w[0] = s.w[1] = s.w[2] = D * G2 * 0.5f * pi / cosNO;
    s.pdf = 0.5f * one_over_pi;
    return s;
}
__device__ __forceinline__ BsdfSample sheen_eval(const SheenLobeDev& L, V3 wo, V3 wi) {
    const V3 wo_l = tolocal(L.f, wo), wi_l = tolocal(L.f, wi);
    BsdfSample s = bsdf_zero();
    if (!(wi_l.z > 0 && wo_l.z >= 0) || L.backfacing) {
        s.wi = wi;
        return s;
    }
    if (L.zeltner) {
        if (wo_l.z >= 0 && wi_l.z > 0) {
            float ltc[3];
            zeltner_fetch(L.a, wo_l.z, ltc);
            s = zeltner_eval(L.a, wi_l, ltc);
        }
    } else {
        s = sheen_mf_eval(L.a, wo_l, wi_l);
    }
    for (int c = 0; c < 3; ++c) s.w[c] *= L.tint[c];
    s.roughness = L.rough;
    s.wi = wi;
    return s;
}
__device__ __forceinline__ BsdfSample sheen_sample(const SheenLobeDev& L, V3 wo, float rx, float ry) {
    if (L.backfacing) return bsdf_zero();
    if (L.zeltner) {
        const V3 wo_l = tolocal(L.f, wo);
        if (wo_l.z < 0) return bsdf_zero();
        float ltc[3];
        zeltner_fetch(L.a, wo_l.z, ltc);
        const V3 c = bsdl_sample_cos_hemisphere(rx, ry);
        BsdfSample s = zeltner_eval(L.a, vnormalize_imath(v3(c.x - c.z * ltc[1], c.y, ltc[0] * c.z)), ltc);
        for (int k = 0; k < 3; ++k) s.w[k] *= L.tint[k];
        s.roughness = L.rough;
        s.wi = bsdl_world(L.f, s.wi);
        return s;
    }
    const float a = 2 * rx - 1, qa = fabsf(a);
    const float b = 2 * ry - 1, qb = fabsf(b);
    const float rad = qa > qb ? qa : qb;
    const float phi = qa > qb ? qb / qa : ((qa == qb) ? 1.0f : 2 - qa / qb);
    const float x = copysignf(rad * bsdl_cos_quadrant(phi), a);
    const float y = copysignf(rad * bsdl_sin_quadrant(phi), b);
    const float cos_theta = 1 - rad * rad;
    const float sin_theta = sqrtf(2 - rad * rad);
    const V3 wi_l = v3(sin_theta * x, sin_theta * y, cos_theta);
    BsdfSample s = sheen_mf_eval(L.a, tolocal(L.f, wo), wi_l);
    for (int c = 0; c < 3; ++c) s.w[c] *= L.tint[c];
    s.roughness = L.rough;
    s.wi = bsdl_world(L.f, s.wi);
    return s;
}


// ---- BSDL mtx::DielectricLobe (libbsdl MTX/bsdf_dielectric_impl.h) --------------------
// dielectric_bsdf(N, U, reflection_tint, transmission_tint, roughness_x,
// roughness_y, ior, distribution) as testrender wraps it (BSDL_WRAP,
// shading.cpp:73-115: Nf = Ngf = N, outer IOR 1, no spectral sampling):
// GGX microfacets (microfacet_tools_impl.h GGXDist) with reflection only
// (Turquin multiple-scattering, :343-391) when the transmission tint is
// black, else reflection + refraction sampled with bounded visible normals
// and renormalized by the tabulated energy 1 - E_ms. The energy tables are
// baked at build time by gen_bsdl_luts.cpp, the way BSDL's genluts does.
// "absorption" (a colour keyword parameter) scales the reflection-only
// lobe's opacity; the thin-film and dispersion keywords change nothing in
// this configuration (no thin film is set on the lobe, lambda_0 is 0).
#define OSLG_LUT_QUAL static __device__ const
#include "oslg_bsdl_luts.inc"
#undef OSLG_LUT_QUAL

// The dielectric's construction, evaluation and sampling are calls except
// in a kernel specialized to one group: a persistent batch body instantiates
// a lobe's code once per lobe position and MIS pair (inlined, that would
// multiply its compile time), and the interpreter carries every lobe kind,
// where inlining this one would cost registers on every path.
#if defined(OSLG_SPEC) && !defined(OSLG_SPEC_BATCH)
#define OSLG_DIEL_FN __forceinline__
#else
#define OSLG_DIEL_FN __noinline__
#endif

// BSDL's MIN / MAX / CLAMP / LERP (tools.h:84-117)
__device__ __forceinline__ float bmin(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float bmax(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float bclamp(float x, float a, float b) { return bmin(bmax(x, a), b); }
__device__ __forceinline__ float blerp(float f, float a, float b) {
    f = bclamp(f, 0.0f, 1.0f);
    return (1 - f) * a + f * b;
}
__device__ __forceinline__ float bsqr(float x) { return x * x; }

// BSDL Frame(Z, X) (tools.h:483-495)
__device__ __forceinline__ Frame bsdl_frame_zx(V3 z, V3 x) {
    if (bsdl_max_abs(x) < 1e-4f || fabsf(vdot(z, vnormalize_imath(x))) > 0.999f) return bsdl_frame(z);
    Frame f;
    f.w = z;
    f.v = vnormalize_imath(vcross(z, x));
    f.u = vcross(f.v, z);
    return f;
}

// TabulatedEnergyCurve<T>::Emiss_eval (microfacet_tools_impl.h:113-212) over
// a baked table [NF][16 roughness][16 cosines]; cosines (i/15)^2 when SQ,
// else i/15. The roughness index is kept inside the table (BSDL reads past
// it for roughness above 1).
template <int NF, bool SQ>
__device__ __forceinline__ float lut_cosine(int i) {
    const float t = float(i) * (1.0f / 15);
    return fmaxf(SQ ? t * t : t, 1e-6f);
}
template <int NF>
__device__ __forceinline__ float lut_interp(const float* T, float rough, float findex, int i) {
    float rf = rough * 15;
    int ra = (int)rf;
    ra = ra < 0 ? 0 : (ra > 15 ? 15 : ra);
    const int rb = min(ra + 1, 15);
    rf -= ra;
    if (NF == 1) return blerp(rf, __ldg(T + ra * 16 + i), __ldg(T + rb * 16 + i));
    float ff = findex * (NF - 1);
    int fa = (int)ff;
    fa = fa < 0 ? 0 : (fa > NF - 1 ? NF - 1 : fa);
    const int fb = min(fa + 1, NF - 1);
    ff -= fa;
    return blerp(ff, blerp(rf, __ldg(T + (fa * 16 + ra) * 16 + i), __ldg(T + (fa * 16 + rb) * 16 + i)),
                 blerp(rf, __ldg(T + (fb * 16 + ra) * 16 + i), __ldg(T + (fb * 16 + rb) * 16 + i)));
}
template <int NF, bool SQ>
__device__ float lut_emiss(const float* T, float rough, float findex, float c) {
    float cos0 = lut_cosine<NF, SQ>(0);
    if (c <= cos0) return lut_interp<NF>(T, rough, findex, 0);
    for (int i = 1; i < 16; ++i) {
        const float cos1 = lut_cosine<NF, SQ>(i);
        if (c < cos1) {
            const float q = (c - cos0) / (cos1 - cos0);
            return blerp(q, lut_interp<NF>(T, rough, findex, i - 1), lut_interp<NF>(T, rough, findex, i));
        }
        cos0 = cos1;
    }
    return lut_interp<NF>(T, rough, findex, 15);
}

// GGXDist (microfacet_tools_decl.h:13-47, microfacet_tools_impl.h:17-112)
struct GGXDistDev {
    float ax, ay;
};
__device__ __forceinline__ GGXDistDev ggxd_make(float rough, float aniso, bool flip) {
    GGXDistDev d;
    d.ax = bsqr(rough);
    d.ay = d.ax;
    if (flip) aniso = -aniso;
    d.ax = fmaxf(d.ax * (1 + aniso), 1e-5f);
    d.ay = fmaxf(d.ay * (1 - aniso), 1e-5f);
    return d;
}
__device__ __forceinline__ float ggxd_D(const GGXDistDev& d, V3 h) {
    const float cp = bsqr(h.x / d.ax), sp = bsqr(h.y / d.ay), c2 = bsqr(h.z);
    const float s2 = cp + sp;
    return 1.0f / (3.14159265358979323846f * d.ax * d.ay * bsqr(c2 + s2));
}
__device__ __forceinline__ float ggxd_G1(const GGXDistDev& d, V3 w) {
    w = v3(w.x * d.ax, w.y * d.ay, w.z);
    return 2.0f * w.z / (w.z + vlen_imath(w));
}
__device__ __forceinline__ float ggxd_G2_G1(const GGXDistDev& d, V3 wi, V3 wo) {
    wi = v3(wi.x * d.ax, wi.y * d.ay, wi.z);
    wo = v3(wo.x * d.ax, wo.y * d.ay, wo.z);
    const float nl = vlen_imath(wi), nv = vlen_imath(wo);
    return wi.z * (wo.z + nv) / (wo.z * nl + wi.z * nv);
}
// Eto and Tokuyoshi, "Bounded VNDF Sampling for Smith-GGX Reflections"
// (eq. 5, 6, 8): the reflection-bounded micro normal and D_refl / D
__device__ __forceinline__ float ggxd_bvn_k(const GGXDistDev& d, V3 wo) {
    const float a = bclamp(bmin(d.ax, d.ay), 0.0f, 1.0f);
    const float s = 1 + sqrtf(bsqr(wo.x) + bsqr(wo.y));
    const float a2 = bsqr(a), s2 = bsqr(s);
    return (1 - a2) * s2 / (s2 + a2 * bsqr(wo.z));
}
__device__ __forceinline__ V3 ggxd_sample_for_refl(const GGXDistDev& d, V3 wo, float randu, float randv) {
    const V3 i_std = vnormalize_imath(v3(wo.x * d.ax, wo.y * d.ay, wo.z));
    const float phi = (2.0f * 3.14159265358979323846f) * randu;
    const float k = ggxd_bvn_k(d, wo);
    const float b = k * i_std.z;
    const float z = (1 - randv) * (1 + b) - b;
    const float st = sqrtf(bclamp(1 - bsqr(z), 0.0f, 1.0f));
    const V3 o_std = v3(st * fm::cos(phi), st * fm::sin(phi), z);
    const V3 m_std = vadd(i_std, o_std);
    return vnormalize_imath(v3(m_std.x * d.ax, m_std.y * d.ay, m_std.z));
}
__device__ __forceinline__ float ggxd_D_refl_D(const GGXDistDev& d, V3 wo) {
    const float l2 = (wo.x * d.ax) * (wo.x * d.ax) + (wo.y * d.ay) * (wo.y * d.ay);
    const float t = sqrtf(l2 + bsqr(wo.z));
    const float k = ggxd_bvn_k(d, wo);
    return 2 * wo.z / (k * wo.z + t);
}

// DielectricFresnel (MTX/bsdf_dielectric_impl.h:21-64)
__device__ __forceinline__ float diel_fresnel_eta(float e, bool backside) {
    if (backside) e = 1 / e;
    return e >= 1 ? bclamp(e, 1.001f, 5.0f) : bclamp(e, 1 / 5.0f, 1 / 1.001f);
}
__device__ __forceinline__ float diel_fresnel(float eta, float c) {
    float g = (eta - 1.0f) * (eta + 1.0f) + c * c;
    if (g > 0) {
        g = sqrtf(g);
        const float A = (g - c) / (g + c);
        const float B = (c * (g + c) - 1) / (c * (g - c) + 1);
        return 0.5f * A * A * (1 + B * B);
    }
    return 1.0f;
}
__device__ __forceinline__ float diel_table_index(float eta) {
    const float seta = bclamp(eta < 1 ? 1 / eta : eta, 1.001f, 5.0f);
    const float x = (seta - 1.001f) * (1 / (5.0f - 1.001f));
    return sqrtf(x);
}
// BSDL reflect / refract (tools.h:301-334)
__device__ __forceinline__ V3 bsdl_reflect(V3 E, V3 N) { return vsub(vmul(N, 2 * vdot(N, E)), E); }
__device__ __forceinline__ V3 bsdl_refract(V3 E, V3 N, float eta) {
    if (eta == 0) return v3(0.0f, 0.0f, 0.0f);
    float cosi = vdot(E, N), neta;
    V3 Nn;
    if (cosi > 0) {
        neta = 1 / eta;
        Nn = N;
    } else {
        cosi = -cosi;
        neta = eta;
        Nn = vneg(N);
    }
    const float arg = 1 - (neta * neta * (1 - (cosi * cosi)));
    if (arg >= 0) {
        const float dnp = sqrtf(arg);
        const float nK = (neta * cosi) - dnp;
        return vnormalize_imath(vadd(vmul(E, -neta), vmul(Nn, nK)));
    }
    return v3(0.0f, 0.0f, 0.0f);
}

struct DielLobeDev {
    Frame f;          // BSDL Frame(visible normal, U)
    GGXDistDev d;
    float eta;        // DielectricFresnel::eta
    float spec_ems;   // DielectricBSDF::E_ms (reflection only: MiniMicrofacetGGX)
    float ems;        // DielectricLobe::E_ms
    float rough;      // the lobe's (regularized) roughness
    float refl[3], refr[3], wo_abs[3];
    bool dorefl, dorefr;
};
// DielectricLobe::DielectricLobe (MTX/bsdf_dielectric_impl.h:245-316)
static __device__ OSLG_DIEL_FN DielLobeDev diel_make(V3 N, V3 U, const float* refl, const float* refr, float rx_in,
                                                 float ry_in, float ior, const float* absorption, V3 wo,
                                                 float path_rough, bool backfacing) {
    DielLobeDev D;
    D.f = bsdl_frame_zx(bsdl_visible_normal(wo, N, N), U);
    for (int c = 0; c < 3; ++c) {
        D.refl[c] = refl[c];
        D.refr[c] = refr[c];
        D.wo_abs[c] = 1.0f;
    }
    D.dorefl = bmax(refl[0], bmax(refl[1], refl[2])) > 0;
    D.dorefr = bmax(refr[0], bmax(refr[1], refr[2])) > 0;
    const float rx = bclamp(rx_in, 1e-4f, 2.0f), ry = bclamp(ry_in, 1e-4f, 2.0f);
    const float axr = fmaxf(rx, ry), ayr = fminf(rx, ry);
    const float b = ayr / axr;
    const float aniso = (1 - b) / (1 + b);
    const float roughness = 1.0f - (1.0f - sqrtf(axr / (1 + aniso))) * (1.0f - path_rough);
    const float cosNO = vdot(D.f.w, wo);
    const float IOR = bclamp(ior, 1.001f, 5.0f);
    D.eta = diel_fresnel_eta(IOR / 1.0f, backfacing);
    D.d = ggxd_make(roughness, aniso, rx < ry);
    D.spec_ems = D.dorefr ? 0.0f : lut_emiss<1, true>(kLutMiniGGX, roughness, 0.0f, cosNO);
    const float tix = diel_table_index(D.eta);
    D.ems = 0.0f;
    if (D.dorefl && !D.dorefr) D.ems = lut_emiss<32, false>(kLutDielReflFront, roughness, tix, cosNO);
    else if (D.dorefr)
        D.ems = lut_emiss<32, false>(backfacing ? kLutDielBothBack : kLutDielBothFront, roughness, tix, cosNO);
    D.rough = roughness;
    if (bmax(absorption[0], bmax(absorption[1], absorption[2])) > 0 && D.dorefl && !D.dorefr) {
        const float sinNO2 = 1 - bsqr(cosNO);
        const float inveta2 = bsqr(1 / D.eta);
        const float cos_p = sqrtf(1 - fminf(1.0f, inveta2 * sinNO2));
        const float dist = 1 / fmaxf(cos_p, 1.17549435e-38f);
        for (int c = 0; c < 3; ++c) D.wo_abs[c] = fm::exp(-absorption[c] * dist);
    }
    return D;
}
// eval_turquin_microms_reflection (microfacet_tools_impl.h:343-373) and
// DielectricBSDF::eval (MTX/bsdf_dielectric_impl.h:110-185), local frame;
// the weight is one value for all channels
__device__ __forceinline__ BsdfSample diel_spec_eval(const DielLobeDev& L, V3 wo, V3 wi) {
    BsdfSample s = bsdf_zero();
    const float cosNO = wo.z, cosNI = wi.z;
    if (!L.dorefr) {
        if (cosNI <= 0 || cosNO <= 0) return s;
        const V3 m = vnormalize_imath(vadd(wo, wi));
        const float cosMO = vdot(m, wo);
        const float D = ggxd_D(L.d, m);
        const float D_refl_D = ggxd_D_refl_D(L.d, wo);
        const float D_refl = D_refl_D * D;
        const float G1 = ggxd_G1(L.d, wo);
        const float pdf = D_refl / (4 * cosNO);
        const float out = ggxd_G2_G1(L.d, wi, wo) * G1 / D_refl_D;
        const float F = diel_fresnel(L.eta, cosMO);
        const float msf = L.spec_ems / fmaxf(0.01f, 1 - L.spec_ems);
        const float O = out * F * (1 + F * msf);
        s.w[0] = s.w[1] = s.w[2] = O;
        s.pdf = pdf;
        s.wi = wi;
        return s;
    }
    if (cosNI > 0) {
        const V3 m = vnormalize_imath(vadd(wo, wi));
        const float cosMO = vdot(m, wo);
        if (cosMO <= 0) return s;
        const float D = ggxd_D(L.d, m);
        const float G1 = ggxd_G1(L.d, wo);
        const float F = diel_fresnel(L.eta, cosMO);
        if (F <= 0) return s;
        const float D_refl_D = ggxd_D_refl_D(L.d, wo);
        const float D_refl = D_refl_D * D;
        const float out = F * (ggxd_G2_G1(L.d, wi, wo) * G1 / (D_refl_D * F));
        s.w[0] = s.w[1] = s.w[2] = out;
        s.pdf = D_refl / (4.0f * cosNO) * F;
        s.wi = wi;
        return s;
    }
    if (cosNI < 0) {
        const float eta = L.eta;
        const V3 Ht = vmul(vnormalize_imath(vadd(vmul(wi, eta), wo)), eta > 1 ? -1.0f : 1.0f);
        const float cosHO = vdot(Ht, wo), cosHI = vdot(Ht, wi);
        if (cosHO <= 0 || cosHI >= 0) return s;
        const float Ft = 1.0f - diel_fresnel(eta, cosHO);
        if (Ht.z <= 0 || Ft <= 0) return s;
        const float D = ggxd_D(L.d, Ht);
        const float G1 = ggxd_G1(L.d, wo);
        const float J = (-cosHI * cosHO * bsqr(eta)) / (wo.z * bsqr(cosHI * eta + cosHO));
        const float D_refl_D = ggxd_D_refl_D(L.d, wo);
        const float D_refl = D_refl_D * D;
        const float out = Ft * (ggxd_G2_G1(L.d, v3(wi.x, wi.y, -wi.z), wo) * G1 / (D_refl_D * Ft));
        s.w[0] = s.w[1] = s.w[2] = out;
        s.pdf = D_refl * J * Ft;
        s.wi = wi;
        return s;
    }
    return s;
}
// sample_turquin_microms_reflection (microfacet_tools_impl.h:375-391) and
// DielectricBSDF::sample (MTX/bsdf_dielectric_impl.h:187-216)
__device__ __forceinline__ BsdfSample diel_spec_sample(const DielLobeDev& L, V3 wo, float ru, float rv, float rw) {
    if (!L.dorefr) {
        if (wo.z <= 0) return bsdf_zero();
        const V3 m = ggxd_sample_for_refl(L.d, wo, ru, rv);
        const V3 wi = bsdl_reflect(wo, m);
        if (wi.z <= 0) return bsdf_zero();
        return diel_spec_eval(L, wo, wi);
    }
    const V3 m = ggxd_sample_for_refl(L.d, wo, ru, rv);
    const float cosMO = vdot(wo, m);
    if (cosMO <= 0) return bsdf_zero();
    const float F = diel_fresnel(L.eta, cosMO);
    const bool choose_reflect = rw < F;
    const V3 wi = choose_reflect ? bsdl_reflect(wo, m) : bsdl_refract(wo, m, L.eta);
    if ((choose_reflect && wi.z <= 0) || (!choose_reflect && wi.z >= 0)) return bsdf_zero();
    return diel_spec_eval(L, wo, wi);
}
// DielectricLobe::eval_impl / sample_impl (MTX/bsdf_dielectric_impl.h:318-
// 360) through BSDL_WRAP (world directions in and out)
__device__ __forceinline__ void diel_finish(const DielLobeDev& L, BsdfSample& s) {
    if (L.dorefr) {
        const float inv = 1 / fmaxf(0.01f, 1 - L.ems);
        for (int c = 0; c < 3; ++c) s.w[c] *= inv;
    }
}
static __device__ OSLG_DIEL_FN BsdfSample diel_eval(const DielLobeDev& L, V3 wo, V3 wi) {
    if (!L.dorefl && !L.dorefr) {
        BsdfSample z = bsdf_zero();
        z.wi = wi;
        return z;
    }
    BsdfSample s = diel_spec_eval(L, tolocal(L.f, wo), tolocal(L.f, wi));
    diel_finish(L, s);
    const float* tint = s.wi.z > 0 ? L.refl : L.refr;
    for (int c = 0; c < 3; ++c) s.w[c] *= tint[c];
    s.roughness = L.rough;
    s.wi = wi;
    return s;
}
static __device__ OSLG_DIEL_FN BsdfSample diel_sample(const DielLobeDev& L, V3 wo, float rx, float ry, float rz) {
    if (!L.dorefl && !L.dorefr) return bsdf_zero();
    BsdfSample s = diel_spec_sample(L, tolocal(L.f, wo), rx, ry, rz);
    diel_finish(L, s);
    if (bsdl_max_abs(s.wi) < 1e-4f) return bsdf_zero();
    const float* tint = s.wi.z > 0 ? L.refl : L.refr;
    for (int c = 0; c < 3; ++c) s.w[c] *= tint[c];
    s.roughness = L.rough;
    s.wi = bsdl_world(L.f, s.wi);
    return s;
}
// albedo_impl and filter_o (MTX/bsdf_dielectric_decl.h:146-157)
__device__ __forceinline__ void diel_albedo(const DielLobeDev& L, float* alb) {
    for (int c = 0; c < 3; ++c) alb[c] = !L.dorefr ? L.refl[c] * (1 - L.ems) : 1.0f;
}
__device__ __forceinline__ void diel_filter_o(const DielLobeDev& L, float* f) {
    for (int c = 0; c < 3; ++c) f[c] = !L.dorefr ? L.ems * L.wo_abs[c] : 0.0f;
}

}  // namespace dev
}  // namespace oslg
