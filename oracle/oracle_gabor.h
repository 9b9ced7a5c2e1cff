// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of OSL's Gabor sparse-convolution noise as the batched
// library runs it:
//   * uniform parameters       src/liboslnoise/sfm_gabornoise.h:99-131
//   * filter set-up            sfm_gabornoise.h:163-215 (make_orthonormals
//                              gabornoise.h:198-212)
//   * impulse sampling         sfm_gabornoise.h:218-297 (fast_rng :21-57)
//   * cell / 27-cell grid      sfm_gabornoise.h:300-470
//   * kernel, slice, filter    gabornoise.h:112-183
//   * entry points and scale   sfm_gabornoise.h:490-660; 1-D/2-D/4-D forms
//                              slice to 3-D (gabornoise.cpp:212-226,
//                              opnoise.cpp:484-560)
// The math policy M supplies exp and sincos: OwnMath is the executor's own
// single-precision pair (oracle_fmath.h, what the device computes);
// LibmMath is libm, what the reference calls. 2^bandwidth is taken in
// double precision (the reference's OIIO::fast_exp2 is exact for integer
// bandwidths) and the Poisson threshold exp(-mean) likewise.
#pragma once
#include <cfloat>
#include <cmath>

#include "oracle_dual.h"
#include "oracle_fmath.h"
#include "oracle_noise.h"

namespace oracle {

struct OwnMath {
    static float exp(float x) { return own_exp(x); }
    static void sincos(float x, float* s, float* c) { own_sincos(x, s, c); }
};
struct LibmMath {
    static float exp(float x) { return std::exp(x); }
    static void sincos(float x, float* s, float* c) { *s = std::sin(x); *c = std::cos(x); }
};

struct GaborOptions {
    int anisotropic = 0;
    int do_filter = 1;
    V3 direction = V3(1.0f, 0.0f, 0.0f);
    float bandwidth = 1.0f;
    float impulses = 16.0f;
};

struct M22 {
    float m[2][2];
};
inline M22 m22(float a, float b, float c, float d) { M22 r; r.m[0][0] = a; r.m[0][1] = b; r.m[1][0] = c; r.m[1][1] = d; return r; }
inline M22 m22_mul(const M22& A, const M22& B) {
    M22 r;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) r.m[i][j] = A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j];
    return r;
}
inline M22 m22_add(const M22& A, const M22& B) {
    return m22(A.m[0][0] + B.m[0][0], A.m[0][1] + B.m[0][1], A.m[1][0] + B.m[1][0], A.m[1][1] + B.m[1][1]);
}
inline M22 m22_scale(float s, const M22& A) {
    return m22(A.m[0][0] * s, A.m[0][1] * s, A.m[1][0] * s, A.m[1][1] * s);
}
// Imathx.h:90-94
inline float m22_det(const M22& M) { return M.m[0][0] * M.m[1][1] - M.m[0][1] * M.m[1][0]; }
// 2x2 inverse: adjugate divided by the determinant, identity when the
// determinant is too small to divide every cofactor by (Imath's singular
// matrix rule with exceptions off).
inline M22 m22_inverse(const M22& M) {
    M22 s = m22(M.m[1][1], -M.m[0][1], -M.m[1][0], M.m[0][0]);
    float r = M.m[0][0] * M.m[1][1] - M.m[1][0] * M.m[0][1];
    if (std::fabs(r) >= 1.0f) {
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) s.m[i][j] /= r;
    } else {
        float mr = std::fabs(r) / FLT_MIN;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) {
                if (mr > std::fabs(s.m[i][j])) s.m[i][j] /= r;
                else return m22(1.0f, 0.0f, 0.0f, 1.0f);
            }
    }
    return s;
}
// gabornoise.h:142-147
inline void m22_mul_v2(const M22& m, float vx, float vy, float* ox, float* oy) {
    *ox = vx * m.m[0][0] + vy * m.m[1][0];
    *oy = vx * m.m[0][1] + vy * m.m[1][1];
}

struct M33 {
    float m[3][3];
};
inline M33 m33_cols(const V3& a, const V3& b, const V3& c) {
    M33 r;
    r.m[0][0] = a.x; r.m[0][1] = b.x; r.m[0][2] = c.x;
    r.m[1][0] = a.y; r.m[1][1] = b.y; r.m[1][2] = c.y;
    r.m[2][0] = a.z; r.m[2][1] = b.z; r.m[2][2] = c.z;
    return r;
}
inline M33 m33_mul(const M33& A, const M33& B) {
    M33 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[i][j] = A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j] + A.m[i][2] * B.m[2][j];
    return r;
}
// Imathx.h:31-41 (row vector times matrix)
inline V3 m33_mul_v3(const M33& M, const V3& s) {
    return V3(s.x * M.m[0][0] + s.y * M.m[1][0] + s.z * M.m[2][0],
              s.x * M.m[0][1] + s.y * M.m[1][1] + s.z * M.m[2][1],
              s.x * M.m[0][2] + s.y * M.m[1][2] + s.z * M.m[2][2]);
}
// dual_vec.h:289-300
inline DV m33_mul_dv(const M33& M, const DV& s) {
    DF s0 = comp(s, 0), s1 = comp(s, 1), s2 = comp(s, 2);
    DF a = s0 * M.m[0][0] + s1 * M.m[1][0] + s2 * M.m[2][0];
    DF b = s0 * M.m[0][1] + s1 * M.m[1][1] + s2 * M.m[2][1];
    DF c = s0 * M.m[0][2] + s1 * M.m[1][2] + s2 * M.m[2][2];
    DV r;
    setcomp(r, 0, a); setcomp(r, 1, b); setcomp(r, 2, c);
    return r;
}

// Imath Vec3 length (with the tiny-vector rescale) and normalize
inline float v3_length(const V3& a) {
    float l2 = a.x * a.x + a.y * a.y + a.z * a.z;
    if (l2 < 2.0f * FLT_MIN) {
        float m = std::fmax(std::fabs(a.x), std::fmax(std::fabs(a.y), std::fabs(a.z)));
        if (m == 0.0f) return 0.0f;
        V3 b(a.x / m, a.y / m, a.z / m);
        return m * std::sqrt(b.x * b.x + b.y * b.y + b.z * b.z);
    }
    return std::sqrt(l2);
}
inline V3 v3_normalized(const V3& a) {
    float l = v3_length(a);
    if (l == 0.0f) return a;
    return V3(a.x / l, a.y / l, a.z / l);
}
inline V3 v3_cross(const V3& a, const V3& b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// dual_vec.h:411-423 / :441-445
inline DF ddot(const DV& a, const DV& b) {
    return comp(a, 0) * comp(b, 0) + comp(a, 1) * comp(b, 1) + comp(a, 2) * comp(b, 2);
}
inline DF ddot(const V3& a, const DV& b) {
    return comp(b, 0) * a.x + comp(b, 1) * a.y + comp(b, 2) * a.z;
}

// sfm_gabornoise.h:21-57
struct FastRng {
    uint32_t seed;
    FastRng(const V3& p, int s) {
        seed = inthash((uint32_t)ifloor(p.x), (uint32_t)ifloor(p.y), (uint32_t)ifloor(p.z), (uint32_t)s);
        if (!seed) seed = 1;
    }
    float operator()() {
        seed *= 3039177861u;
        return (float)seed * (1.0f / 4294967296.0f);
    }
    int poisson(float g) {  // g = exp(-mean)
        int em = 0;
        float t = (*this)();
        while (t > g && em < 1024) {  // same bound as the device loop
            ++em;
            t *= (*this)();
        }
        return em;
    }
};

inline float gabor_wrap(float s, float period) {
    period = std::floor(period);
    if (period < 1.0f) period = 1.0f;
    return s - period * std::floor(s / period);
}

template <class M> struct Gabor {
    // uniform (sfm_gabornoise.h:99-131)
    float a, lambda, sqrt_lambda_inv, radius, radius2, radius3, radius_inv, poisson_g;
    // per point (sfm_gabornoise.h:134-162)
    int anisotropic, do_filter;
    V3 omega, N, period;
    bool periodic;
    M22 filter;
    M33 local;
    // per-point filter constants of filter_gabor_kernel_2d that do not
    // depend on the impulse (gabornoise.h:160-171)
    float c_F, inv_c_GF_den;
    M22 SGSF_inv, Sigma_GF_Gi;
    float a_f;

    explicit Gabor(const GaborOptions& o) {
        float bw = o.bandwidth < 0.01f ? 0.01f : (o.bandwidth > 100.0f ? 100.0f : o.bandwidth);
        float two_bw = (float)std::exp2((double)bw);
        a = 2.0f * ((two_bw - 1.0f) / (two_bw + 1.0f)) * 2.128934e+00f;
        // sqrtf(-logf(0.02f) / float(M_PI)) == 1.115901231765747f
        radius = 1.115901231765747f / a;
        radius2 = radius * radius;
        radius3 = radius2 * radius;
        radius_inv = 1.0f / radius;
        float imp = o.impulses < 1.0f ? 1.0f : (o.impulses > 32.0f ? 32.0f : o.impulses);
        lambda = imp / (4.188779830932617f * radius3);
        sqrt_lambda_inv = 1.0f / std::sqrt(lambda);
        poisson_g = (float)std::exp(-(double)(lambda * radius3));
        anisotropic = o.anisotropic;
        do_filter = o.do_filter;
        omega = o.direction;
        periodic = false;
    }

    // sfm_gabornoise.h:163-215
    void setup_filter(const DV& P) {
        V3 n = v3_cross(P.dx, P.dy);
        if (n.x * n.x + n.y * n.y + n.z * n.z < 1.0e-6f) {
            do_filter = 0;
            return;
        }
        // make_orthonormals (gabornoise.h:198-212)
        n = v3_normalized(n);
        V3 t = std::fabs(n.x) < 0.9f ? V3(0.0f, n.z, -n.y) : V3(-n.z, 0.0f, n.x);
        t = v3_normalized(t);
        V3 b = v3_cross(n, t);
        M33 tex_to_tan = m33_cols(t, b, n);
        M33 scr_to_tex = m33_cols(P.dx, P.dy, V3(0.0f, 0.0f, 0.0f));
        M33 scr_to_tan = m33_mul(scr_to_tex, tex_to_tan);
        M22 Ms = m22(scr_to_tan.m[0][0], scr_to_tan.m[0][1], scr_to_tan.m[1][0], scr_to_tan.m[1][1]);
        M22 Sf = m22(0.5f * 0.5f, 0.0f, 0.0f, 0.5f * 0.5f);
        M22 Mst = m22(Ms.m[0][0], Ms.m[1][0], Ms.m[0][1], Ms.m[1][1]);
        M22 Sft = m22_mul(m22_mul(Mst, Sf), Ms);
        N = n;
        filter = Sft;
        local = tex_to_tan;
        if (m22_det(Sft) < 1.0e-18f) {
            do_filter = 0;
            return;
        }
        // impulse-independent part of filter_gabor_kernel_2d
        M22 Sigma_G = m22_scale(a * a / 6.2831854820251465f, m22(1.0f, 0.0f, 0.0f, 1.0f));
        c_F = 1.0f / (6.2831854820251465f * std::sqrt(m22_det(filter)));
        M22 Sigma_F = m22_scale(0.02533029578626156f, m22_inverse(filter));
        M22 SGSF = m22_add(Sigma_G, Sigma_F);
        inv_c_GF_den = 1.0f / (6.2831854820251465f * std::sqrt(m22_det(SGSF)));
        SGSF_inv = m22_inverse(SGSF);
        M22 Sigma_G_i = m22_inverse(Sigma_G);
        M22 Sigma_GF = m22_inverse(m22_add(m22_inverse(Sigma_F), Sigma_G_i));
        Sigma_GF_Gi = m22_mul(Sigma_GF, Sigma_G_i);
        a_f = std::sqrt((float)(6.283185307179586 * (double)std::sqrt(m22_det(Sigma_GF))));
    }

    // gabornoise.h:112-120
    static DF kernel(const DF& w, const V3& om, const DF& phi, float bw, const DV& x) {
        DF q = ddot(x, x) * (-3.1415927410125732f * (bw * bw));
        float e = M::exp(q.v);
        DF g(e, e * q.dx, e * q.dy);
        DF arg = ddot(om, x) * 6.2831854820251465f + phi;
        float s, c;
        M::sincos(arg.v, &s, &c);
        DF h(c, -s * arg.dx, -s * arg.dy);
        return w * g * h;
    }
    static DF kernel2(const DF& w, float omx, float omy, const DF& phi, float bw, const DF& x0, const DF& x1) {
        DF q = (x0 * x0 + x1 * x1) * (-3.1415927410125732f * (bw * bw));
        float e = M::exp(q.v);
        DF g(e, e * q.dx, e * q.dy);
        DF arg = (x0 * omx + x1 * omy) * 6.2831854820251465f + phi;
        float s, c;
        M::sincos(arg.v, &s, &c);
        DF h(c, -s * arg.dx, -s * arg.dy);
        return w * g * h;
    }

    // sfm_gabornoise.h:218-277
    void sample(FastRng& rng, V3* om, float* phi) const {
        if (anisotropic == 1) {
            *om = omega;
        } else if (anisotropic == 0) {
            float omega_t = 6.2831854820251465f * rng();
            float t = rng();
            float cos_p = (1.0f - t) * -1.0f + t * 1.0f;
            float sin_p = std::sqrt(std::fmax(0.0f, 1.0f - cos_p * cos_p));
            float st, ct;
            M::sincos(omega_t, &st, &ct);
            *om = v3_normalized(V3(ct * sin_p, st * sin_p, cos_p));
        } else {
            float omega_r = v3_length(omega);
            float omega_t = 6.2831854820251465f * rng();
            float st, ct;
            M::sincos(omega_t, &st, &ct);
            *om = V3(ct, st, 0.0f) * omega_r;
        }
        *phi = 6.2831854820251465f * rng();
    }
    void no_sample(FastRng& rng) const {
        if (anisotropic == 0) { rng(); rng(); }
        else if (anisotropic != 1) rng();
        rng();
    }

    // sfm_gabornoise.h:300-395
    DF cell(const V3& c_i, const DV& x_c_i, int seed) const {
        V3 key = periodic ? V3(gabor_wrap(c_i.x, period.x), gabor_wrap(c_i.y, period.y), gabor_wrap(c_i.z, period.z))
                          : c_i;
        FastRng rng(key, seed);
        int n = rng.poisson(poisson_g);
        DF sum(0.0f);
        for (int i = 0; i < n; ++i) {
            float z = rng(), y = rng(), x = rng();
            DV x_k_i = (x_c_i - V3(x, y, z)) * radius;
            const V3& kv = x_k_i.v;
            if (kv.x * kv.x + kv.y * kv.y + kv.z * kv.z < radius2) {
                V3 om;
                float phi;
                sample(rng, &om, &phi);
                if (do_filter == 1) {
                    V3 om_t = m33_mul_v3(local, om);
                    DF d = -ddot(N, x_k_i);
                    // slice_gabor_kernel_3d (gabornoise.h:123-138), weight 1
                    DF dd = (d * d) * (-3.1415927410125732f * (a * a));
                    float e = M::exp(dd.v);
                    DF w_s = DF(e, e * dd.dx, e * dd.dy) * 1.0f;
                    DF phi_s = phi - (d * 6.2831854820251465f) * om_t.z;
                    // filter_gabor_kernel_2d (gabornoise.h:150-183)
                    float mx, my;
                    m22_mul_v2(SGSF_inv, om_t.x, om_t.y, &mx, &my);
                    float ex = M::exp(-0.5f * (mx * om_t.x + my * om_t.y));
                    DF w_f = ((w_s * c_F) * inv_c_GF_den) * ex;
                    float ofx, ofy;
                    m22_mul_v2(Sigma_GF_Gi, om_t.x, om_t.y, &ofx, &ofy);
                    DV xkit = m33_mul_dv(local, x_k_i);
                    DF gk = kernel2(w_f, ofx, ofy, phi_s, a_f, comp(xkit, 0), comp(xkit, 1));
                    if (!std::isfinite(gk.v)) gk = kernel(DF(1.0f), om, DF(phi), a, x_k_i);
                    sum = sum + gk;
                } else {
                    sum = sum + kernel(DF(1.0f), om, DF(phi), a, x_k_i);
                }
            } else {
                no_sample(rng);
            }
        }
        return sum;
    }

    // sfm_gabornoise.h:399-485
    DF evaluate(const DV& x, int seed) const {
        DV x_g = x * radius_inv;
        V3 f(std::floor(x_g.v.x), std::floor(x_g.v.y), std::floor(x_g.v.z));
        DV x_c = x_g - f;
        DF sum(0.0f);
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    V3 c((float)i, (float)j, (float)k);
                    sum = sum + cell(f + c, x_c - c, seed);
                }
        return sum * sqrt_lambda_inv;
    }

    float scale() const {
        float var = 1.0f / (4.0f * 1.4142135381698608f * (a * a * a));
        float s = 1.0f / (3.0f * std::sqrt(var));
        return s * 0.5f;
    }
};

// gabor / gabor3 / pgabor / pgabor3 on a Dual2<Vec3> position; nc = 1 or 3.
template <class M>
inline void gabor_eval(const GaborOptions& o, const DV& P, bool periodic, const V3& period, int nc, DF* out) {
    Gabor<M> g(o);
    g.periodic = periodic;
    g.period = period;
    if (g.do_filter) g.setup_filter(P);
    float s = g.scale();
    for (int c = 0; c < nc; ++c) out[c] = g.evaluate(P, c) * s;
}

}  // namespace oracle
