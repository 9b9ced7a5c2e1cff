// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of testrender's BSDF sampling for the lobes of the
// wavefront workload, on top of oracle_shading.h:
//   * Diffuse<0>::sample (src/testrender/shading.cpp:301-320) with
//     Sampling::sample_cosine_hemisphere / to_unit_disk (sampling.h:70-100);
//   * Microfacet<GGXDist, Refract> for Refract 0, 1, 2 — eval and sample
//     (shading.cpp:571-760, GGXDist::sampleSlope :480-508), fresnel_refraction
//     (optics.h:34-66);
//   * the oren_nayar closure as testrender builds it: BSDL's
//     OrenNayarDiffuseLobe without energy compensation, albedo 1
//     (shading.cpp:1496-1502; libbsdl MTX/bsdf_oren_nayar_diffuse_impl.h:
//     41-113) in BSDL's Frame (tools.h:459-508) around the visible normal
//     (bsdf_impl.h:51-84), cosine hemisphere via the square-to-disc map with
//     Clarberg's quadrant polynomials (tools.h:196-275);
//   * CompositeBSDF::prepare / eval / sample (shading.h:319-402);
//   * emission adds the component weight to Le (shading.cpp:1485-1486).
// The reference's OIIO::fast_sincos in to_unit_disk is replaced by the
// executor's own sincos (oracle_fmath.h); OIIO's source is not in the tree.
#pragma once
#include <algorithm>
#include <cmath>
#include <new>

#include "oracle_fastmath.h"
#include "oracle_fmath.h"
#include "oracle_shading.h"

namespace oracle {

static const int kMaxLobes = 8;  // CompositeBSDF::MaxEntries

inline V3 frame_get(const TangentFrame& f, float x, float y, float z) { return f.u * x + f.v * y + f.w * z; }

// sampling.h:70-100
inline void to_unit_disk(float& x, float& y) {
    const float PI_OVER_4 = float(M_PI_4), PI_OVER_2 = float(M_PI_2);
    float phi, r;
    float a = 2 * x - 1, b = 2 * y - 1;
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
inline void sample_cosine_hemisphere(const V3& N, float rx, float ry, V3* out, float* pdf) {
    to_unit_disk(rx, ry);
    float cos_theta = std::sqrt(std::max(1 - rx * rx - ry * ry, 0.0f));
    *out = frame_get(TangentFrame::from_normal(N), rx, ry, cos_theta);
    *pdf = cos_theta * float(M_1_PI);
}

inline Sample diffuse_sample(const V3& N, float rx, float ry) {
    Sample s;
    V3 wi;
    float pdf;
    sample_cosine_hemisphere(N, rx, ry, &wi, &pdf);
    s.wi = wi;
    s.weight = V3(1.0f);
    s.pdf = pdf;
    s.roughness = 1.0f;
    return s;
}

// optics.h:34-66
inline float fresnel_refraction(const V3& I, const V3& N, float eta, V3* T) {
    float cosi = -dotv(I, N);
    V3 Nn;
    float neta;
    if (cosi > 0) {
        neta = 1 / eta;
        Nn = N;
    } else {
        cosi = -cosi;
        neta = eta;
        Nn = -N;
    }
    float arg = 1.0f - (neta * neta * (1.0f - cosi * cosi));
    if (arg >= 0) {
        float dnp = std::sqrt(arg);
        float nK = (neta * cosi) - dnp;
        *T = I * neta + Nn * nK;
        return 1 - fresnel_dielectric(cosi, eta);
    }
    *T = V3(0.0f);
    return 0;
}

// Microfacet<GGXDist, Refract>
struct MicrofacetGGX : MicrofacetGGXRefl {
    int refract;
    MicrofacetGGX(const V3& n, const V3& u, float ax, float ay, float e, int r)
        : MicrofacetGGXRefl(n, u, ax, ay, e), refract(r) {}
    V3 albedo(const V3& wo) const {
        if (refract == 2) return V3(1.0f);
        float fr = fresnel_dielectric(dotv(N, wo), eta);
        return V3(refract ? 1 - fr : fr);
    }
    Sample eval(const V3& wo, const V3& wi) const {
        const V3 wo_l = tf.tolocal(wo);
        const V3 wi_l = tf.tolocal(wi);
        Sample s;
        s.wi = wi;
        if (refract == 0 || refract == 2) {
            if (wo_l.z > 0 && wi_l.z > 0) {
                const V3 m = imath_normalize(wi_l + wo_l);
                const float D = evalD(m);
                const float Lo = evalLambda(wo_l), Li = evalLambda(wi_l);
                const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
                const float Fr = fresnel_dielectric(dotv(m, wo_l), eta);
                float pdf = (G1 * D * 0.25f) / wo_l.z;
                float out = G2 / G1;
                s.roughness = std::max(xalpha, yalpha);
                if (refract == 2) {
                    s.pdf = pdf * Fr;
                    s.weight = V3(out);
                } else {
                    s.pdf = pdf;
                    s.weight = V3(out * Fr);
                }
                return s;
            }
        }
        if (refract == 1 || refract == 2) {
            if (wi_l.z < 0 && wo_l.z > 0.0f) {
                V3 ht = -(wi_l * eta + wo_l);
                if (eta < 1.0f) ht = -ht;
                V3 Ht = imath_normalize(ht);
                const float cosHO = dotv(Ht, wo_l);
                const float Ft = 1.0f - fresnel_dielectric(cosHO, eta);
                if (Ft > 0) {
                    const float cosHI = dotv(Ht, wi_l);
                    const float cosThetaM = Ht.z;
                    if (cosThetaM <= 0.0f) return Sample();
                    const float Dt = evalD(Ht);
                    const float Lo = evalLambda(wo_l), Li = evalLambda(wi_l);
                    const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
                    float invHt2 = 1 / dotv(ht, ht);
                    float pdf = (std::fabs(cosHI * cosHO) * (eta * eta) * (G1 * Dt) * invHt2) / wo_l.z;
                    float out = G2 / G1;
                    s.roughness = std::max(xalpha, yalpha);
                    if (refract == 2) {
                        s.pdf = pdf * Ft;
                        s.weight = V3(out);
                    } else {
                        s.pdf = pdf;
                        s.weight = V3(out * Ft);
                    }
                    return s;
                }
            }
        }
        return Sample();
    }
    // GGXDist::sampleSlope (shading.cpp:480-508)
    static void sample_slope(float cos_theta, float randu, float randv, float* sx, float* sy) {
        float c = cos_theta < 1e-6f ? 1e-6f : cos_theta;
        float Q = (1 + c) * randu - c;
        float num = c * std::sqrt((1 - c) * (1 + c)) - Q * std::sqrt((1 - Q) * (1 + Q));
        float den = (Q - c) * (Q + c);
        float eps = 1.0f / 4294967296.0f;
        den = std::fabs(den) < eps ? std::copysign(eps, den) : den;
        *sx = num / den;
        float Ru = 1 - 2 * randv;
        float u2 = std::fabs(Ru);
        float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f))
                / (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.0f) + 0.597999f);
        *sy = std::copysign(1.0f, Ru) * z * std::sqrt(1.0f + *sx * *sx);
    }
    // Microfacet::sampleMicronormal (shading.cpp:754-787)
    V3 sample_micronormal(const V3& wo, float randu, float randv) const {
        V3 swo = wo;
        swo.x *= xalpha;
        swo.y *= yalpha;
        swo = imath_normalize(swo);
        float cos_theta = std::max(swo.z, 0.0f);
        float cos_phi = 1, sin_phi = 0;
        if (cos_theta < 0.99999f) {
            float invnorm = 1 / std::sqrt(SQR(swo.x) + SQR(swo.y));
            cos_phi = swo.x * invnorm;
            sin_phi = swo.y * invnorm;
        }
        float slx, sly;
        sample_slope(cos_theta, randu, randv, &slx, &sly);
        float sx = cos_phi * slx - sin_phi * sly;
        float sy = sin_phi * slx + cos_phi * sly;
        sx *= xalpha;
        sy *= yalpha;
        float mlen = std::sqrt(sx * sx + sy * sy + 1);
        return V3(std::fabs(sx) < mlen ? -sx / mlen : 1.0f, std::fabs(sy) < mlen ? -sy / mlen : 1.0f, 1.0f / mlen);
    }
    // Microfacet::sample (shading.cpp:628-700)
    Sample sample(const V3& wo, float rx, float ry, float rz) const {
        const V3 wo_l = tf.tolocal(wo);
        const float cosNO = wo_l.z;
        if (!(cosNO > 0)) return Sample();
        const V3 m = sample_micronormal(wo_l, rx, ry);
        const float cosMO = dotv(m, wo_l);
        const float F = fresnel_dielectric(cosMO, eta);
        Sample s;
        if (refract == 0 || (refract == 2 && rz < F)) {
            const V3 wi_l = m * (2.0f * cosMO) - wo_l;
            const float D = evalD(m);
            const float Lo = evalLambda(wo_l), Li = evalLambda(wi_l);
            const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
            s.wi = frame_get(tf, wi_l.x, wi_l.y, wi_l.z);
            float pdf = (G1 * D * 0.25f) / cosNO;
            float out = G2 / G1;
            s.roughness = std::max(xalpha, yalpha);
            if (refract == 2) {
                s.pdf = pdf * F;
                s.weight = V3(out);
            } else {
                s.pdf = pdf;
                s.weight = V3(F * out);
            }
            return s;
        }
        const V3 M = frame_get(tf, m.x, m.y, m.z);
        V3 wi;
        float Ft = fresnel_refraction(-wo, M, eta, &wi);
        const V3 wi_l = tf.tolocal(wi);
        const float cosHO = dotv(m, wo_l), cosHI = dotv(m, wi_l);
        const float D = evalD(m);
        const float Lo = evalLambda(wo_l), Li = evalLambda(wi_l);
        const float G2 = 1 / (Lo + Li + 1), G1 = 1 / (Lo + 1);
        const V3 ht = -(wi_l * eta + wo_l);
        const float invHt2 = 1.0f / dotv(ht, ht);
        float pdf = (std::fabs(cosHI * cosHO) * (eta * eta) * (G1 * D) * invHt2) / std::fabs(wo_l.z);
        float out = G2 / G1;
        s.wi = wi;
        s.roughness = std::max(xalpha, yalpha);
        if (refract == 2) {
            s.pdf = pdf * Ft;
            s.weight = V3(out);
        } else {
            s.pdf = pdf;
            s.weight = V3(Ft * out);
        }
        return s;
    }
};

// BSDL pieces (libbsdl/include/BSDL/tools.h)
inline float bsdl_cos_quadrant(float x) {
    float x2 = x * x;
    float cp = 0.01578646f + -0.00029826362f * x2;
    cp = -0.30837047f + cp * x2;
    cp = 0.99998736f + cp * x2;
    return cp;
}
inline float bsdl_sin_quadrant(float x) {
    float x2 = x * x;
    float sp = 0.0024843954015523195266723632812500f + -0.0000341485538228880614042282104492f * x2;
    sp = -0.0807407423853874206542968750000000f + sp * x2;
    sp = 0.7853975892066955566406250000000000f + sp * x2;
    return sp * x;
}
inline V3 bsdl_sample_cos_hemisphere(float randu, float randv) {
    const float a = 2 * randu - 1, qa = std::fabs(a);
    const float b = 2 * randv - 1, qb = std::fabs(b);
    const float rad = qa > qb ? qa : qb;
    const float phi = qa > qb ? qb / qa : ((qa == qb) ? 1.0f : 2 - qa / qb);
    const float x = std::copysign(rad * bsdl_cos_quadrant(phi), a);
    const float y = std::copysign(rad * bsdl_sin_quadrant(phi), b);
    return V3(x, y, std::sqrt(1 - rad * rad));
}
struct BsdlFrame {
    V3 X, Y, Z;
    BsdlFrame() = default;
    explicit BsdlFrame(const V3& z) : Z(z) {
        const float s = std::copysign(1.0f, z.z);
        const float a = -1.0f / (s + z.z);
        const float b = z.x * z.y * a;
        X = V3(1.0f + s * z.x * z.x * a, s * b, -s * z.x);
        Y = V3(b, s + z.y * z.y * a, -z.y);
    }
    // Frame(Z, X) (tools.h:483-495): X along x but orthogonal to Z
    BsdlFrame(const V3& z, const V3& x);
    V3 local(const V3& a) const { return V3(dotv(a, X), dotv(a, Y), dotv(a, Z)); }
    V3 world(const V3& a) const {
        return V3(X.x * a.x + Y.x * a.y + Z.x * a.z, X.y * a.x + Y.y * a.y + Z.y * a.z, X.z * a.x + Y.z * a.y + Z.z * a.z);
    }
};
inline float bsdl_max_abs(const V3& v) { return std::max(std::fabs(v.x), std::max(std::fabs(v.y), std::fabs(v.z))); }
inline BsdlFrame::BsdlFrame(const V3& z, const V3& x) : X(x), Z(z) {
    if (bsdl_max_abs(X) < 1e-4f || std::fabs(dotv(Z, imath_normalize(X))) > 0.999f) {
        *this = BsdlFrame(z);
    } else {
        Y = imath_normalize(crossv(Z, X));
        X = crossv(Y, Z);
    }
}
// BsdfGlobals::visible_normal (bsdf_impl.h:51-78)
inline V3 bsdl_visible_normal(const V3& wo, const V3& Ngf, const V3& N) {
    if (dotv(wo, N) > 0.0f) return N;
    V3 V = crossv(wo, N);
    if (bsdl_max_abs(V) < 1e-4f) {
        V = crossv(wo, Ngf);
        if (bsdl_max_abs(V) < 1e-4f) {
            const float s = std::copysign(1.0f, wo.z);
            const float a = -1.0f / (s + wo.z);
            V = V3(wo.x * wo.y * a, s + wo.y * wo.y * a, -wo.y);
        } else {
            V = imath_normalize(V);
        }
    } else {
        V = imath_normalize(V);
    }
    return imath_normalize(crossv(V, wo) + wo * 1e-4f);
}
inline float bsdl_clamp(float x, float a, float b) { return std::min(std::max(x, a), b); }

// oren_nayar as testrender builds it (energy compensation off, albedo 1)
// BSDL OrenNayarDiffuseLobe (libbsdl MTX/bsdf_oren_nayar_diffuse_impl.h):
// testrender's oren_nayar is the QON form with albedo 1;
// oren_nayar_diffuse_bsdf carries its albedo and, with
// energy_compensation, takes the energy preserving FON form (single
// scattering plus a multiple scattering term from the analytic directional
// albedo E_FON; acos in double precision, where BSDL calls its fast acos).
struct OrenNayarQON {
    BsdlFrame frame;
    float rough;
    V3 alb = V3(1.0f);
    bool energy = false;
    OrenNayarQON(const V3& N, float sigma, const V3& wo)
        : frame(bsdl_visible_normal(wo, N, N)), rough(bsdl_clamp(sigma, 0.0f, 1.0f)) {}
    OrenNayarQON(const V3& N, const V3& albedo, float sigma, bool ec, const V3& wo)
        : frame(bsdl_visible_normal(wo, N, N)), rough(bsdl_clamp(sigma, 0.0f, 1.0f)), alb(albedo), energy(ec) {}
    static constexpr float c1 = 0.5f - 2.0f / (3.0f * float(M_PI));
    static constexpr float c2 = 2.0f / 3.0f - 28.0f / (15.0f * float(M_PI));
    float E_fon(float mu) const {
        const float AF = 1.0f / (1.0f + c1 * rough);
        const float BF = rough * AF;
        const float Si = std::sqrt(std::max(0.0f, 1.0f - mu * mu));
        const float G = Si * ((float)std::acos((double)mu) - Si * mu)
                      + 2.0f * ((Si / std::max(mu, 1e-7f)) * (1.0f - Si * Si * Si) - Si) * (1.0f / 3.0f);
        return AF + (BF * (1 / float(M_PI))) * G;
    }
    Sample eval_local(const V3& wo, const V3& wi) const {
        if (energy) return eval_fon(wo, wi);
        Sample s = eval_qon(wo, wi);
        s.weight = V3(alb.x * s.weight.x, alb.y * s.weight.y, alb.z * s.weight.z);
        return s;
    }
    Sample eval_fon(const V3& wo, const V3& wi) const {
        Sample s;
        const float cosNI = bsdl_clamp(wi.z, 0.0f, 1.0f);
        const float cosNO = bsdl_clamp(wo.z, 0.0f, 1.0f);
        if (cosNI <= 0.0f || cosNO <= 0.0f) return s;
        const float cosIO = bsdl_clamp(dotv(wo, wi), -1.0f, 1.0f);
        const float sv = cosIO - cosNI * cosNO;
        const float pdf = cosNI * (1 / float(M_PI));
        const float AF = 1.0f / (1.0f + c1 * rough);
        const float stinv = sv > 0.0f ? sv / std::max(cosNI, cosNO) : sv;
        const float f_ss = AF * (1.0f + rough * stinv);
        const float EFo = E_fon(cosNO), EFi = E_fon(cosNI);
        const float avgEF = AF * (1.0f + c2 * rough);
        const float f_ms = std::max(1e-7f, 1.0f - EFo) * std::max(1e-7f, 1.0f - EFi) / std::max(1e-7f, 1.0f - avgEF);
        const float a[3] = { alb.x, alb.y, alb.z };
        float w[3];
        for (int c = 0; c < 3; ++c) {
            const float rho_ms = (a[c] * a[c]) * avgEF / (1 - a[c] * std::max(0.0f, 1.0f - avgEF));
            w[c] = a[c] * f_ss + rho_ms * f_ms;
        }
        s.wi = wi;
        s.weight = V3(w[0], w[1], w[2]);
        s.pdf = pdf;
        s.roughness = 1.0f;
        return s;
    }
    Sample eval_qon(const V3& wo, const V3& wi) const {
        Sample s;
        const float cosNI = bsdl_clamp(wi.z, 0.0f, 1.0f);
        const float cosNO = bsdl_clamp(wo.z, 0.0f, 1.0f);
        if (cosNI <= 0.0f || cosNO <= 0.0f) return s;
        const float cosIO = bsdl_clamp(dotv(wo, wi), -1.0f, 1.0f);
        const float sv = cosIO - cosNI * cosNO;
        const float pdf = cosNI * (1 / float(M_PI));
        const float s2 = rough * rough;
        const float A = 1.0f - 0.50f * s2 / (s2 + 0.33f);
        const float B = 0.45f * s2 / (s2 + 0.09f);
        const float stinv = sv > 0.0f ? sv / std::max(cosNI, cosNO) : 0.0f;
        const float f_ss = A + B * stinv;
        s.wi = wi;
        s.weight = V3(1.0f) * f_ss;
        s.pdf = pdf;
        s.roughness = 1.0f;
        return s;
    }
    Sample eval(const V3& wo, const V3& wi) const {
        Sample s = eval_local(frame.local(wo), frame.local(wi));
        s.wi = wi;
        return s;
    }
    Sample sample(const V3& wo, float rx, float ry) const {
        const V3 wo_l = frame.local(wo);
        if (wo_l.z <= 0.0f) return Sample();
        Sample s = eval_local(wo_l, bsdl_sample_cos_hemisphere(rx, ry));
        s.wi = frame.world(s.wi);
        return s;
    }
};

// sheen_bsdf as testrender builds it: BSDL mtx::SheenLobe, Conty-Kulla
// mode, MaterialX albedo fit, non-legacy visibility term
// (libbsdl MTX/bsdf_sheen_impl.h:19-110, :120-260). The power in the
// distribution is the executor's own float power (OIIO::fast_pow in the
// reference: parity unpinned there).
inline float sheen_albedo_fit(float c, float r) {
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
// Zeltner, Burley and Chiang 2022 sheen (BSDL ZeltnerBurleySheen with LTC
// sampling and LTC albedo, libbsdl MTX/bsdf_sheen_impl.h:267-357): the
// paper's 32 x 32 table of LTC coefficients (A, B, R) over roughness and
// cos theta_o, interpolated bilinearly (LERP clamps its factor).
static const float kZeltnerLtc[32 * 32 * 3] = {
#include "../openshadinglanguage_gb300/csrc/oslg_zeltner_ltc.inc"
};
inline V3 zeltner_fetch(float a, float cosNO) {
    const float almost_one = 0.999999940395355224609375f;
    const float row = bsdl_clamp(a, 0.0f, almost_one) * 31.0f, col = bsdl_clamp(cosNO, 0.0f, almost_one) * 31.0f;
    const float r = std::floor(row), c = std::floor(col);
    const float rf = bsdl_clamp(row - r, 0.0f, 1.0f), cf = bsdl_clamp(col - c, 0.0f, 1.0f);
    const int i0 = ((int)r * 32 + (int)c) * 3, i1 = i0 + 96;
    float o[3];
    for (int k = 0; k < 3; ++k) {
        const float lo = (1 - cf) * kZeltnerLtc[i0 + k] + cf * kZeltnerLtc[i0 + 3 + k];
        const float hi = (1 - cf) * kZeltnerLtc[i1 + k] + cf * kZeltnerLtc[i1 + 3 + k];
        o[k] = (1 - rf) * lo + rf * hi;
    }
    return V3(o[0], o[1], o[2]);
}
inline Sample zeltner_eval(float a, const V3& wi, const V3& ltc) {
    Sample s;
    const V3 o(ltc.x * wi.x + ltc.y * wi.z, ltc.x * wi.y, wi.z);
    const float len2 = o.x * o.x + o.y * o.y + o.z * o.z;
    const float j = ltc.x / len2;
    const float pdf = j * j * std::max(o.z, 0.0f) * (1 / float(M_PI));
    if (pdf > 1.17549435e-38f) {
        s.wi = wi;
        s.weight = V3(ltc.z);
        s.pdf = pdf;
        s.roughness = a;
    }
    return s;
}

// sheen_bsdf: mode 0 Conty-Kulla (above), mode 1 Zeltner-Burley
struct SheenConty {
    BsdlFrame frame;
    V3 tint;
    float rough, a, emiss;
    bool backfacing, zeltner = false;
    SheenConty(const V3& N, const V3& albedo, float roughness, const V3& wo, float path_roughness, bool bf,
               int mode = 0)
        : frame(bsdl_visible_normal(wo, N, N)), tint(albedo), backfacing(bf) {
        rough = 1.0f - (1.0f - bsdl_clamp(roughness, 0.0f, 1.0f)) * (1.0f - path_roughness);
        zeltner = mode == 1;
        a = zeltner ? bsdl_clamp(std::max(0.02f, std::sqrt(rough)), 0.02f, 1.0f)
                    : bsdl_clamp(std::max(0.06f, rough), 0.06f, 1.0f);
        const float cosNO = bsdl_clamp(dotv(frame.Z, wo), 0.0f, 1.0f);
        const float tmax = std::max(std::max(tint.x, tint.y), tint.z);
        const float alb = zeltner ? zeltner_fetch(a, cosNO).z : sheen_albedo_fit(cosNO, a);
        emiss = backfacing ? 1.0f : 1.0f - std::min(alb * tmax, 1.0f);
    }
    V3 albedo() const { return tint * (1 - emiss); }
    static Sample mf_eval(float a, const V3& wo, const V3& wi) {
        Sample s;
        const float cosNO = wo.z, cosNI = wi.z;
        if (cosNI <= 1e-5f || cosNO <= 1e-5f) return s;
        const V3 H = imath_normalize(wo + wi);
        const float ct = bsdl_clamp(H.z, 0.0f, 1.0f);
        const float st = std::sqrt(1.0f - ct * ct);
        const float pi = float(M_PI), one_over_pi = 1 / pi;
        const float D = own_pow_pos(st, 1 / a) * (2 + 1 / a) * 0.5f * one_over_pi;
        if (D < 1e-6f) return s;
        const float ci = std::min(1.0f, wi.z), co = std::min(1.0f, wo.z);
        const float G2 = (ci * co) / (ci + co - ci * co);
        s.wi = wi;
        s.weight = V3(D * G2 * 0.5f * pi / cosNO);
        s.pdf = 0.5f * one_over_pi;
        return s;
    }
    Sample eval(const V3& wo, const V3& wi) const {
        const V3 wo_l = frame.local(wo), wi_l = frame.local(wi);
        Sample s;
        if (!(wi_l.z > 0 && wo_l.z >= 0) || backfacing) {
            s.wi = wi;
            return s;
        }
        if (zeltner) {
            if (wo_l.z >= 0 && wi_l.z > 0) s = zeltner_eval(a, wi_l, zeltner_fetch(a, wo_l.z));
        } else {
            s = mf_eval(a, wo_l, wi_l);
        }
        s.weight = s.weight * tint;
        s.roughness = rough;
        s.wi = wi;
        return s;
    }
    Sample sample(const V3& wo, float rx, float ry) const {
        if (backfacing) return Sample();
        if (zeltner) {
            const V3 wo_l = frame.local(wo);
            if (wo_l.z < 0) return Sample();
            const V3 ltc = zeltner_fetch(a, wo_l.z);
            const V3 c = bsdl_sample_cos_hemisphere(rx, ry);
            Sample s = zeltner_eval(a, imath_normalize(V3(c.x - c.z * ltc.y, c.y, ltc.x * c.z)), ltc);
            s.weight = s.weight * tint;
            s.roughness = rough;
            s.wi = frame.world(s.wi);
            return s;
        }
        const float ua = 2 * rx - 1, qa = std::fabs(ua);
        const float ub = 2 * ry - 1, qb = std::fabs(ub);
        const float rad = qa > qb ? qa : qb;
        const float phi = qa > qb ? qb / qa : ((qa == qb) ? 1.0f : 2 - qa / qb);
        const float x = std::copysign(rad * bsdl_cos_quadrant(phi), ua);
        const float y = std::copysign(rad * bsdl_sin_quadrant(phi), ub);
        const float cos_theta = 1 - rad * rad;
        const float sin_theta = std::sqrt(2 - rad * rad);
        Sample s = mf_eval(a, frame.local(wo), V3(sin_theta * x, sin_theta * y, cos_theta));
        s.weight = s.weight * tint;
        s.roughness = rough;
        s.wi = frame.world(s.wi);
        return s;
    }
};

// ---- BSDL mtx::DielectricLobe (libbsdl MTX/bsdf_dielectric_{decl,impl}.h) ----
// as testrender wraps it (BSDL_WRAP, shading.cpp:73-115: Nf = Ngf = N,
// outer IOR 1, lambda_0 0). The energy tables are the build's baked
// tables (gen_bsdl_luts.cpp, BSDL genluts' method), shared as data.
#define OSLG_LUT_QUAL static const
#include "../openshadinglanguage_gb300/csrc/oslg_bsdl_luts.inc"
#undef OSLG_LUT_QUAL

namespace bsdl_mx {
template <class T> inline T MIN(T a, T b) { return a < b ? a : b; }
template <class T> inline T MAX(T a, T b) { return a > b ? a : b; }
inline float CLAMP(float x, float a, float b) { return MIN(MAX(x, a), b); }
inline float LERP(float f, float a, float b) {
    f = CLAMP(f, 0, 1);
    return (1 - f) * a + f * b;
}
inline float SQR(float x) { return x * x; }
const float PI = 3.14159265358979323846f;

// TabulatedEnergyCurve (microfacet_tools_impl.h:113-212) over a baked table
// [Nf][16][16]; squared: cosines (i/15)^2 (MiniMicrofacetGGX), else i/15
struct EnergyCurve {
    const float* E;
    int Nf;
    bool squared;
    float roughness, fresnel_index;
    float cosine(int i) const {
        const float t = float(i) * (1.0f / (16 - 1));
        return std::max(squared ? SQR(t) : t, 1e-6f);
    }
    float interpolate_emiss(int i) const {
        float rf = roughness * (16 - 1);
        int ra = std::min(std::max((int)rf, 0), 15);  // BSDL reads past the table above roughness 1
        int rb = std::min(ra + 1, 16 - 1);
        rf -= ra;
        if (Nf == 1) return LERP(rf, E[ra * 16 + i], E[rb * 16 + i]);
        float ff = fresnel_index * (Nf - 1);
        int fa = std::min(std::max((int)ff, 0), Nf - 1);
        int fb = std::min(fa + 1, Nf - 1);
        ff -= fa;
        return LERP(ff, LERP(rf, E[(fa * 16 + ra) * 16 + i], E[(fa * 16 + rb) * 16 + i]),
                    LERP(rf, E[(fb * 16 + ra) * 16 + i], E[(fb * 16 + rb) * 16 + i]));
    }
    float Emiss_eval(float c) const {
        float cos0 = cosine(0);
        if (c <= cos0) return interpolate_emiss(0);
        for (int i = 1; i < 16; i++) {
            const float cos1 = cosine(i);
            if (c < cos1) {
                float q = (c - cos0) / (cos1 - cos0);
                return LERP(q, interpolate_emiss(i - 1), interpolate_emiss(i));
            }
            cos0 = cos1;
        }
        return interpolate_emiss(16 - 1);
    }
};

// GGXDist (microfacet_tools_decl.h:13-47, microfacet_tools_impl.h:17-112)
struct GGXDist {
    float ax = 0, ay = 0;
    GGXDist() = default;
    GGXDist(float rough, float aniso, bool flip_aniso) : ax(SQR(rough)), ay(ax) {
        if (flip_aniso) aniso = -aniso;
        ax = std::max(ax * (1 + aniso), 1e-5f);
        ay = std::max(ay * (1 - aniso), 1e-5f);
    }
    float D(const V3& Hr) const {
        const float cosPhi2st2 = SQR(Hr.x / ax);
        const float sinPhi2st2 = SQR(Hr.y / ay);
        const float cosThetaM2 = SQR(Hr.z);
        const float sinThetaM2 = cosPhi2st2 + sinPhi2st2;
        return 1.0f / (PI * ax * ay * SQR(cosThetaM2 + sinThetaM2));
    }
    float G1(V3 w) const {
        w = V3(w.x * ax, w.y * ay, w.z);
        return 2.0f * w.z / (w.z + imath_len(w));
    }
    float G2_G1(V3 wi, V3 wo) const {
        wi = V3(wi.x * ax, wi.y * ay, wi.z);
        wo = V3(wo.x * ax, wo.y * ay, wo.z);
        const float nl = imath_len(wi);
        const float nv = imath_len(wo);
        return wi.z * (wo.z + nv) / (wo.z * nl + wi.z * nv);
    }
    // Eto & Tokuyoshi, bounded VNDF sampling for Smith-GGX reflections
    V3 sample_for_refl(const V3& wo, float randu, float randv) const {
        V3 i_std = imath_normalize(V3(wo.x * ax, wo.y * ay, wo.z));
        const float phi = 2.0f * PI * randu;
        const float a = CLAMP(std::min(ax, ay), 0.0f, 1.0f);
        const float s = 1 + std::sqrt(SQR(wo.x) + SQR(wo.y));
        const float a2 = SQR(a);
        const float s2 = SQR(s);
        const float k = (1 - a2) * s2 / (s2 + a2 * SQR(wo.z));
        const float b = k * i_std.z;
        const float z = (1 - randv) * (1 + b) - b;
        const float sinTheta = std::sqrt(CLAMP(1 - SQR(z), 0.0f, 1.0f));
        V3 o_std(sinTheta * oracle_fm::cosf_(phi), sinTheta * oracle_fm::sinf_(phi), z);
        V3 m_std = i_std + o_std;
        return imath_normalize(V3(m_std.x * ax, m_std.y * ay, m_std.z));
    }
    float D_refl_D(const V3& wo) const {
        const float aix = wo.x * ax, aiy = wo.y * ay;
        const float len2 = aix * aix + aiy * aiy;
        const float t = std::sqrt(len2 + SQR(wo.z));
        const float a = CLAMP(std::min(ax, ay), 0.0f, 1.0f);
        const float s = 1 + std::sqrt(SQR(wo.x) + SQR(wo.y));
        const float a2 = SQR(a);
        const float s2 = SQR(s);
        const float k = (1 - a2) * s2 / (s2 + a2 * SQR(wo.z));
        return 2 * wo.z / (k * wo.z + t);
    }
};

// DielectricFresnel (MTX/bsdf_dielectric_impl.h:21-64)
struct DielectricFresnel {
    float eta = 1.5f;
    DielectricFresnel() = default;
    DielectricFresnel(float e, bool backside) {
        if (backside) e = 1 / e;
        eta = e >= 1 ? CLAMP(e, 1.001f, 5.0f) : CLAMP(e, 1 / 5.0f, 1 / 1.001f);
    }
    float eval(float c) const {
        float g = (eta - 1.0f) * (eta + 1.0f) + c * c;
        if (g > 0) {
            g = std::sqrt(g);
            float A = (g - c) / (g + c);
            float B = (c * (g + c) - 1) / (c * (g - c) + 1);
            return 0.5f * A * A * (1 + B * B);
        }
        return 1.0f;
    }
    float table_index() const {
        const float seta = CLAMP(eta < 1 ? 1 / eta : eta, 1.001f, 5.0f);
        const float x = (seta - 1.001f) * (1 / (5.0f - 1.001f));
        return std::sqrt(x);
    }
};

// BSDL reflect / refract (tools.h:301-334)
inline V3 reflect(const V3& E, const V3& N) { return N * (2 * dotv(N, E)) - E; }
inline V3 refract(const V3& E, const V3& N, float eta) {
    V3 R(0.0f);
    if (eta == 0) return R;
    V3 Nn;
    float cosi = dotv(E, N), neta;
    if (cosi > 0) {
        neta = 1 / eta;
        Nn = N;
    } else {
        cosi = -cosi;
        neta = eta;
        Nn = -N;
    }
    float arg = 1 - (neta * neta * (1 - (cosi * cosi)));
    if (arg >= 0) {
        float dnp = std::sqrt(arg);
        float nK = (neta * cosi) - dnp;
        R = imath_normalize(E * (-neta) + Nn * nK);
    }
    return R;
}

// DielectricBSDF<DielectricFresnel> (MTX/bsdf_dielectric_impl.h:66-216)
struct DielectricBSDF {
    GGXDist d;
    DielectricFresnel f;
    float E_ms = 0.0f;
    bool dorefr = false;
    DielectricBSDF() = default;
    DielectricBSDF(const GGXDist& dist, const DielectricFresnel& fr, float cosNO, float roughness, bool refr)
        : d(dist), f(fr), dorefr(refr) {
        if (!dorefr) E_ms = EnergyCurve{ kLutMiniGGX, 1, true, roughness, 0.0f }.Emiss_eval(cosNO);
    }
    // eval_turquin_microms_reflection (microfacet_tools_impl.h:343-373)
    Sample turquin_eval(const V3& wo, const V3& wi) const {
        const float cosNO = wo.z, cosNI = wi.z;
        if (cosNI <= 0 || cosNO <= 0) return Sample();
        V3 m = imath_normalize(wo + wi);
        float cosMO = dotv(m, wo);
        const float D = d.D(m);
        float D_refl_D = d.D_refl_D(wo);
        float D_refl = D_refl_D * D;
        const float G1 = d.G1(wo);
        float pdf = D_refl / (4 * cosNO);
        const float out = d.G2_G1(wi, wo) * G1 / D_refl_D;
        const float F = f.eval(cosMO);
        const float msf = E_ms / std::max(0.01f, 1 - E_ms);
        Sample s;
        s.wi = wi;
        s.weight = V3(out * F * (1 + F * msf));
        s.pdf = pdf;
        return s;
    }
    Sample eval(const V3& wo, const V3& wi) const {
        if (!dorefr) return turquin_eval(wo, wi);
        const float cosNO = wo.z;
        const float cosNI = wi.z;
        Sample s;
        if (cosNI > 0) {
            const V3 m = imath_normalize(wo + wi);
            const float cosMO = dotv(m, wo);
            if (cosMO <= 0) return Sample();
            const float D = d.D(m);
            const float G1 = d.G1(wo);
            const float F = f.eval(cosMO);
            if (F <= 0) return Sample();
            const float D_refl_D = d.D_refl_D(wo);
            const float D_refl = D_refl_D * D;
            s.weight = V3(F * (d.G2_G1(wi, wo) * G1 / (D_refl_D * F)));
            s.pdf = D_refl / (4.0f * cosNO) * F;
            s.wi = wi;
            return s;
        } else if (cosNI < 0) {
            const V3 Ht = imath_normalize(f.eta * wi + wo) * ((f.eta > 1) ? -1.0f : 1.0f);
            const float cosHO = dotv(Ht, wo);
            const float cosHI = dotv(Ht, wi);
            if (cosHO <= 0 || cosHI >= 0) return Sample();
            const float Ft = 1.0f - f.eval(cosHO);
            if (Ht.z <= 0 || Ft <= 0) return Sample();
            const float D = d.D(Ht);
            const float G1 = d.G1(wo);
            float J = (-cosHI * cosHO * SQR(f.eta)) / (wo.z * SQR(cosHI * f.eta + cosHO));
            const float D_refl_D = d.D_refl_D(wo);
            const float D_refl = D_refl_D * D;
            s.pdf = D_refl * J * Ft;
            s.weight = V3(Ft * (d.G2_G1(V3(wi.x, wi.y, -wi.z), wo) * G1 / (D_refl_D * Ft)));
            s.wi = wi;
            return s;
        }
        return Sample();
    }
    Sample sample(const V3& wo, float randu, float randv, float randw) const {
        if (!dorefr) {  // sample_turquin_microms_reflection (:375-391)
            if (wo.z <= 0) return Sample();
            V3 m = d.sample_for_refl(wo, randu, randv);
            V3 wi = reflect(wo, m);
            if (wi.z <= 0) return Sample();
            return turquin_eval(wo, wi);
        }
        V3 m = d.sample_for_refl(wo, randu, randv);
        const float cosMO = dotv(wo, m);
        if (cosMO <= 0) return Sample();
        const float F = f.eval(cosMO);
        bool choose_reflect = randw < F;
        const V3 wi = choose_reflect ? reflect(wo, m) : refract(wo, m, f.eta);
        if ((choose_reflect && wi.z <= 0) || (!choose_reflect && wi.z >= 0)) return Sample();
        return eval(wo, wi);
    }
};
}  // namespace bsdl_mx

// DielectricLobe (MTX/bsdf_dielectric_impl.h:245-366) through BSDL_WRAP
struct MxDielectric {
    BsdlFrame frame;
    bsdl_mx::DielectricBSDF spec;
    V3 refl_tint, refr_tint, wo_absorption = V3(1.0f);
    float E_ms = 0.0f, rough = 0.0f;
    bool dorefl = false, dorefr = false;
    MxDielectric(const V3& N, const V3& U, const V3& refl, const V3& refr, float roughness_x, float roughness_y,
                 float ior, const V3& absorption, const V3& wo, float path_roughness, bool backfacing)
        : refl_tint(refl), refr_tint(refr) {
        using namespace bsdl_mx;
        frame = BsdlFrame(bsdl_visible_normal(wo, N, N), U);
        dorefl = MAX(refl.x, MAX(refl.y, refl.z)) > 0;
        dorefr = MAX(refr.x, MAX(refr.y, refr.z)) > 0;
        const float rx = CLAMP(roughness_x, 1e-4f, 2.0f);
        const float ry = CLAMP(roughness_y, 1e-4f, 2.0f);
        const float ax = std::max(rx, ry);
        const float ay = std::min(rx, ry);
        const float b = ay / ax;
        const float aniso = (1 - b) / (1 + b);
        const float roughness = 1.0f - (1.0f - std::sqrt(ax / (1 + aniso))) * (1.0f - path_roughness);
        const float cosNO = dotv(frame.Z, wo);
        const float IOR = CLAMP(ior, 1.001f, 5.0f);
        DielectricFresnel fresnel(IOR / 1.0f, backfacing);
        spec = DielectricBSDF(GGXDist(roughness, aniso, rx < ry), fresnel, cosNO, roughness, dorefr);
        if (dorefl && !dorefr)
            E_ms = EnergyCurve{ kLutDielReflFront, 32, false, roughness, fresnel.table_index() }.Emiss_eval(cosNO);
        else if (dorefr)
            E_ms = EnergyCurve{ backfacing ? kLutDielBothBack : kLutDielBothFront, 32, false, roughness,
                                fresnel.table_index() }
                       .Emiss_eval(cosNO);
        rough = roughness;
        if (MAX(absorption.x, MAX(absorption.y, absorption.z)) > 0 && dorefl && !dorefr) {
            const float sinNO2 = 1 - SQR(cosNO);
            const float inveta2 = SQR(1 / fresnel.eta);
            const float cos_p = std::sqrt(1 - std::min(1.0f, inveta2 * sinNO2));
            const float dist = 1 / std::max(cos_p, 1.17549435e-38f);
            for (int i = 0; i < 3; ++i) wo_absorption[i] = oracle_fm::expf_(-absorption[i] * dist);
        }
    }
    V3 tint(float cosNI) const { return cosNI > 0 ? refl_tint : refr_tint; }
    Sample eval(const V3& wo, const V3& wi) const {
        Sample r;
        r.wi = wi;
        if (!dorefl && !dorefr) return r;
        Sample s = spec.eval(frame.local(wo), frame.local(wi));
        if (dorefr) s.weight = s.weight * (1 / std::max(0.01f, 1 - E_ms));
        s.weight = s.weight * tint(s.wi.z);
        r.weight = s.weight;
        r.pdf = s.pdf;
        r.roughness = rough;
        return r;
    }
    Sample sample(const V3& wo, float rx, float ry, float rz) const {
        if (!dorefl && !dorefr) return Sample();
        Sample s = spec.sample(frame.local(wo), rx, ry, rz);
        if (dorefr) s.weight = s.weight * (1 / std::max(0.01f, 1 - E_ms));
        if (bsdl_max_abs(s.wi) < 1e-4f) return Sample();
        s.weight = s.weight * tint(s.wi.z);
        s.roughness = rough;
        s.wi = frame.world(s.wi);
        return s;
    }
    V3 albedo() const { return !dorefr ? refl_tint * (1 - E_ms) : V3(1.0f); }
    V3 filter_o() const { return !dorefr ? E_ms * wo_absorption : V3(0.0f); }
};

// The lobes testrender builds from a closure tree, with their weights.
struct CompositeLobes {
    enum Kind { DIFFUSE, GGX, OREN_NAYAR, SHEEN, MX_DIELECTRIC };
    int kind[kMaxLobes];
    V3 w[kMaxLobes];
    float pdfs[kMaxLobes];
    static constexpr size_t kStore = std::max(std::max(sizeof(MicrofacetGGX), sizeof(MxDielectric)),
                                              std::max(sizeof(OrenNayarQON), sizeof(SheenConty)));
    alignas(16) unsigned char storage[kMaxLobes][kStore];
    V3 N[kMaxLobes];
    int n = 0;
    V3 Le = V3(0.0f);

    OrenNayarQON& on(int i) { return *reinterpret_cast<OrenNayarQON*>(storage[i]); }
    const OrenNayarQON& on(int i) const { return *reinterpret_cast<const OrenNayarQON*>(storage[i]); }
    const MicrofacetGGX& mf(int i) const { return *reinterpret_cast<const MicrofacetGGX*>(storage[i]); }
    const SheenConty& sh(int i) const { return *reinterpret_cast<const SheenConty*>(storage[i]); }
    const MxDielectric& mxd(int i) const { return *reinterpret_cast<const MxDielectric*>(storage[i]); }

    void add_diffuse(const V3& cw, const V3& normal) {
        if (n_full()) return;
        kind[n] = DIFFUSE; w[n] = cw; N[n] = normal;
        ++n;
    }
    void add_ggx(const V3& cw, const MicrofacetGGX& m) {
        if (n_full()) return;
        kind[n] = GGX; w[n] = cw;
        new (storage[n]) MicrofacetGGX(m);
        ++n;
    }
    void add_on(const V3& cw, const OrenNayarQON& o) {
        if (n_full()) return;
        kind[n] = OREN_NAYAR; w[n] = cw;
        new (storage[n]) OrenNayarQON(o);
        ++n;
    }
    void add_sheen(const V3& cw, const SheenConty& o) {
        if (n_full()) return;
        kind[n] = SHEEN; w[n] = cw;
        new (storage[n]) SheenConty(o);
        ++n;
    }
    void add_mx_dielectric(const V3& cw, const MxDielectric& o) {
        if (n_full()) return;
        kind[n] = MX_DIELECTRIC; w[n] = cw;
        new (storage[n]) MxDielectric(o);
        ++n;
    }
    bool n_full() const { return n >= kMaxLobes; }

    V3 albedo(int i, const V3& wo) const {
        if (kind[i] == GGX) return mf(i).albedo(wo);
        if (kind[i] == SHEEN) return sh(i).albedo();
        if (kind[i] == OREN_NAYAR) return on(i).alb;
        if (kind[i] == MX_DIELECTRIC) return mxd(i).albedo();
        return V3(1.0f);
    }
    Sample eval_lobe(int i, const V3& wo, const V3& wi) const {
        if (kind[i] == DIFFUSE) {
            Sample s = diffuse_eval(N[i], wi);
            s.wi = wi;
            return s;
        }
        if (kind[i] == GGX) return mf(i).eval(wo, wi);
        if (kind[i] == SHEEN) return sh(i).eval(wo, wi);
        if (kind[i] == MX_DIELECTRIC) return mxd(i).eval(wo, wi);
        return on(i).eval(wo, wi);
    }
    Sample sample_lobe(int i, const V3& wo, float rx, float ry, float rz) const {
        if (kind[i] == DIFFUSE) return diffuse_sample(N[i], rx, ry);
        if (kind[i] == GGX) return mf(i).sample(wo, rx, ry, rz);
        if (kind[i] == SHEEN) return sh(i).sample(wo, rx, ry);
        if (kind[i] == MX_DIELECTRIC) return mxd(i).sample(wo, rx, ry, rz);
        return on(i).sample(wo, rx, ry);
    }
    // CompositeBSDF::prepare (shading.h:322-350)
    void prepare(const V3& wo, const V3& path_weight, bool absorb) {
        float total = 0;
        for (int i = 0; i < n; ++i) {
            pdfs[i] = dotv(w[i], path_weight * albedo(i, wo)) / (path_weight.x + path_weight.y + path_weight.z);
            total += pdfs[i];
        }
        if ((!absorb && total > 0) || total > 1)
            for (int i = 0; i < n; ++i) pdfs[i] /= total;
    }
    // CompositeBSDF::eval (shading.h:360-370)
    Sample eval(const V3& wo, const V3& wi) const {
        Sample s;
        for (int i = 0; i < n; ++i) {
            Sample b = eval_lobe(i, wo, wi);
            b.weight = b.weight * w[i];
            mis_update_eval(&s.weight, &s.pdf, b.weight, b.pdf, pdfs[i]);
            s.roughness += b.roughness * pdfs[i];
        }
        return s;
    }
    // CompositeBSDF::sample (shading.h:372-398)
    Sample sample(const V3& wo, float rx, float ry, float rz) const {
        float accum = 0;
        for (int i = 0; i < n; ++i) {
            if (rx < (pdfs[i] + accum)) {
                rx = (rx - accum) / pdfs[i];
                rx = std::min(rx, 0.99999994f);
                Sample s = sample_lobe(i, wo, rx, ry, rz);
                s.weight = s.weight * (w[i] * (1 / pdfs[i]));
                s.pdf *= pdfs[i];
                if (s.pdf == 0.0f) return Sample();
                for (int j = 0; j < n; ++j) {
                    if (i != j) {
                        Sample b = eval_lobe(j, wo, s.wi);
                        b.weight = b.weight * w[j];
                        mis_update_eval(&s.weight, &s.pdf, b.weight, b.pdf, pdfs[j]);
                    }
                }
                return s;
            }
            accum += pdfs[i];
        }
        return Sample();
    }
};

}  // namespace oracle
