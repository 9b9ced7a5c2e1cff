// Gabor sparse-convolution noise on the device, in the batched library's
// operation order:
//   * uniform parameters       src/liboslnoise/sfm_gabornoise.h:99-131
//   * filter set-up            sfm_gabornoise.h:163-215 (make_orthonormals
//                              gabornoise.h:198-212)
//   * impulse sampling         sfm_gabornoise.h:218-297 (fast_rng :21-57)
//   * cell / 27-cell grid      sfm_gabornoise.h:300-470
//   * kernel, slice, filter    gabornoise.h:112-183
//   * entry points and scale   sfm_gabornoise.h:490-660
// The per-impulse exp and sincos are the executor's own single-precision
// pair (oslg_fmath.cuh). The impulse-independent half of the 2-D kernel
// filter (gabornoise.h:160-171) is computed once per point instead of once
// per impulse; it is the same arithmetic on the same inputs. 2^bandwidth and
// the Poisson threshold exp(-mean) are taken in double precision.
#pragma once
#include "oslg_fmath.cuh"
#include "oslg_noise.cuh"
#include "oslg_shading.cuh"

namespace oslg {
namespace dev {

struct GOpts {
    int anisotropic;
    int do_filter;
    V3 direction;
    float bandwidth;
    float impulses;
};

struct DV3 {
    V3 v, dx, dy;
};
__device__ __forceinline__ D2 dcomp(const DV3& a, int c) {
    return c == 0 ? d2(a.v.x, a.dx.x, a.dy.x) : (c == 1 ? d2(a.v.y, a.dx.y, a.dy.y) : d2(a.v.z, a.dx.z, a.dy.z));
}
__device__ __forceinline__ DV3 dv3_scale(const DV3& a, float s) {
    DV3 r;
    r.v = vmul(a.v, s); r.dx = vmul(a.dx, s); r.dy = vmul(a.dy, s);
    return r;
}
__device__ __forceinline__ DV3 dv3_sub(const DV3& a, V3 b) {
    DV3 r = a;
    r.v = vsub(a.v, b);
    return r;
}
// dual_vec.h:411-423
__device__ __forceinline__ D2 ddot(const DV3& a, const DV3& b) {
    return dcomp(a, 0) * dcomp(b, 0) + dcomp(a, 1) * dcomp(b, 1) + dcomp(a, 2) * dcomp(b, 2);
}
// dual_vec.h:441-445 (dot(Vec3, Dual2<Vec3>) = dot(b, a))
__device__ __forceinline__ D2 ddot(V3 a, const DV3& b) {
    return dcomp(b, 0) * a.x + dcomp(b, 1) * a.y + dcomp(b, 2) * a.z;
}

struct M22 {
    float m00, m01, m10, m11;
};
__device__ __forceinline__ M22 m22(float a, float b, float c, float d) { M22 r; r.m00 = a; r.m01 = b; r.m10 = c; r.m11 = d; return r; }
__device__ __forceinline__ M22 m22_mul(const M22& A, const M22& B) {
    return m22(A.m00 * B.m00 + A.m01 * B.m10, A.m00 * B.m01 + A.m01 * B.m11,
               A.m10 * B.m00 + A.m11 * B.m10, A.m10 * B.m01 + A.m11 * B.m11);
}
__device__ __forceinline__ M22 m22_add(const M22& A, const M22& B) {
    return m22(A.m00 + B.m00, A.m01 + B.m01, A.m10 + B.m10, A.m11 + B.m11);
}
__device__ __forceinline__ M22 m22_scale(float s, const M22& A) { return m22(A.m00 * s, A.m01 * s, A.m10 * s, A.m11 * s); }
// Imathx.h:90-94
__device__ __forceinline__ float m22_det(const M22& M) { return M.m00 * M.m11 - M.m01 * M.m10; }
// adjugate over determinant; identity when the determinant is too small to
// divide every cofactor by (Imath's singular-matrix rule, exceptions off)
__device__ __forceinline__ M22 m22_inverse(const M22& M) {
    float s[4] = { M.m11, -M.m01, -M.m10, M.m00 };
    const float r = M.m00 * M.m11 - M.m10 * M.m01;
    if (fabsf(r) >= 1.0f) {
        for (int i = 0; i < 4; ++i) s[i] /= r;
    } else {
        const float mr = fabsf(r) / 1.17549435e-38f;
        for (int i = 0; i < 4; ++i) {
            if (mr > fabsf(s[i])) s[i] /= r;
            else return m22(1.0f, 0.0f, 0.0f, 1.0f);
        }
    }
    return m22(s[0], s[1], s[2], s[3]);
}

struct M33 {
    float m[3][3];
};
__device__ __forceinline__ M33 m33_cols(V3 a, V3 b, V3 c) {
    M33 r;
    r.m[0][0] = a.x; r.m[0][1] = b.x; r.m[0][2] = c.x;
    r.m[1][0] = a.y; r.m[1][1] = b.y; r.m[1][2] = c.y;
    r.m[2][0] = a.z; r.m[2][1] = b.z; r.m[2][2] = c.z;
    return r;
}
__device__ __forceinline__ M33 m33_mul(const M33& A, const M33& B) {
    M33 r;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) r.m[i][j] = A.m[i][0] * B.m[0][j] + A.m[i][1] * B.m[1][j] + A.m[i][2] * B.m[2][j];
    return r;
}
// Imathx.h:31-41
__device__ __forceinline__ V3 m33_mul_v3(const M33& M, V3 s) {
    return v3(s.x * M.m[0][0] + s.y * M.m[1][0] + s.z * M.m[2][0], s.x * M.m[0][1] + s.y * M.m[1][1] + s.z * M.m[2][1],
              s.x * M.m[0][2] + s.y * M.m[1][2] + s.z * M.m[2][2]);
}

// sfm_gabornoise.h:21-57
struct FastRng {
    uint32_t seed;
    __device__ __forceinline__ float next() {
        seed *= 3039177861u;
        return (float)seed * (1.0f / 4294967296.0f);
    }
};
// Poisson draws are bounded; the count only reaches the bound if the
// generator were stuck, which an odd-multiplier LCG cannot be.
static const int kGaborPoissonCap = 1024;

__device__ __forceinline__ float gabor_wrap(float s, float period) {
    period = floorf(period);
    if (period < 1.0f) period = 1.0f;
    return s - period * floorf(s / period);
}

struct GaborState {
    float a, sqrt_lambda_inv, radius, radius2, radius_inv, poisson_g;
    int anisotropic, do_filter;
    bool periodic;
    V3 omega, N, period;
    M33 local;
    float c_F, inv_c_GF_den, a_f;
    M22 SGSF_inv, Sigma_GF_Gi;
};

// gabornoise.h:112-120 (3-D) with weight 1
__device__ __forceinline__ D2 gabor_kernel3(V3 om, float phi, float bw, const DV3& x) {
    const D2 q = ddot(x, x) * (-3.1415927410125732f * (bw * bw));
    const float e = own_exp(q.v);
    const D2 g = d2(e, e * q.dx, e * q.dy);
    const D2 arg = ddot(om, x) * 6.2831854820251465f + d2c(phi);
    float s, c;
    own_sincos(arg.v, &s, &c);
    const D2 h = d2(c, -s * arg.dx, -s * arg.dy);
    return d2c(1.0f) * g * h;
}
// gabornoise.h:112-120 (2-D)
__device__ __forceinline__ D2 gabor_kernel2(D2 w, float omx, float omy, D2 phi, float bw, D2 x0, D2 x1) {
    const D2 q = (x0 * x0 + x1 * x1) * (-3.1415927410125732f * (bw * bw));
    const float e = own_exp(q.v);
    const D2 g = d2(e, e * q.dx, e * q.dy);
    const D2 arg = (x0 * omx + x1 * omy) * 6.2831854820251465f + phi;
    float s, c;
    own_sincos(arg.v, &s, &c);
    const D2 h = d2(c, -s * arg.dx, -s * arg.dy);
    return w * g * h;
}

// sfm_gabornoise.h:300-395
__device__ __forceinline__ D2 gabor_cell(const GaborState& G, V3 c_i, const DV3& x_c_i, int seed) {
    V3 key = c_i;
    if (G.periodic)
        key = v3(gabor_wrap(c_i.x, G.period.x), gabor_wrap(c_i.y, G.period.y), gabor_wrap(c_i.z, G.period.z));
    FastRng rng;
    rng.seed = inthash4((uint32_t)ifloor(key.x), (uint32_t)ifloor(key.y), (uint32_t)ifloor(key.z), (uint32_t)seed);
    if (!rng.seed) rng.seed = 1;
    int n = 0;
    {
        float t = rng.next();
        while (t > G.poisson_g && n < kGaborPoissonCap) {
            ++n;
            t *= rng.next();
        }
    }
    D2 sum = d2c(0.0f);
    for (int i = 0; i < n; ++i) {
        const float z = rng.next(), y = rng.next(), x = rng.next();
        const DV3 xk = dv3_scale(dv3_sub(x_c_i, v3(x, y, z)), G.radius);
        if (xk.v.x * xk.v.x + xk.v.y * xk.v.y + xk.v.z * xk.v.z < G.radius2) {
            // gabor_sample (sfm_gabornoise.h:218-277)
            V3 om;
            if (G.anisotropic == 1) {
                om = G.omega;
            } else if (G.anisotropic == 0) {
                const float omega_t = 6.2831854820251465f * rng.next();
                const float t = rng.next();
                const float cos_p = (1.0f - t) * -1.0f + t * 1.0f;
                const float sin_p = sqrtf(fmaxf(0.0f, 1.0f - cos_p * cos_p));
                float st, ct;
                own_sincos(omega_t, &st, &ct);
                om = vnormalize_imath(v3(ct * sin_p, st * sin_p, cos_p));
            } else {
                const float omega_r = vlen_imath(G.omega);
                const float omega_t = 6.2831854820251465f * rng.next();
                float st, ct;
                own_sincos(omega_t, &st, &ct);
                om = vmul(v3(ct, st, 0.0f), omega_r);
            }
            const float phi = 6.2831854820251465f * rng.next();
            if (G.do_filter == 1) {
                const V3 om_t = m33_mul_v3(G.local, om);
                const D2 d = -ddot(G.N, xk);
                // slice_gabor_kernel_3d (gabornoise.h:123-138)
                const D2 dd = (d * d) * (-3.1415927410125732f * (G.a * G.a));
                const float e = own_exp(dd.v);
                const D2 w_s = d2(e, e * dd.dx, e * dd.dy) * 1.0f;
                const D2 pd = (d * 6.2831854820251465f) * om_t.z;
                const D2 phi_s = d2(phi - pd.v, -pd.dx, -pd.dy);
                // filter_gabor_kernel_2d (gabornoise.h:150-183)
                const float mx = om_t.x * G.SGSF_inv.m00 + om_t.y * G.SGSF_inv.m10;
                const float my = om_t.x * G.SGSF_inv.m01 + om_t.y * G.SGSF_inv.m11;
                const float ex = own_exp(-0.5f * (mx * om_t.x + my * om_t.y));
                const D2 w_f = ((w_s * G.c_F) * G.inv_c_GF_den) * ex;
                const float ofx = om_t.x * G.Sigma_GF_Gi.m00 + om_t.y * G.Sigma_GF_Gi.m10;
                const float ofy = om_t.x * G.Sigma_GF_Gi.m01 + om_t.y * G.Sigma_GF_Gi.m11;
                // multMatrix(local, Dual2<Vec3>) (dual_vec.h:289-300), x and y
                const D2 s0 = dcomp(xk, 0), s1 = dcomp(xk, 1), s2 = dcomp(xk, 2);
                const D2 k0 = s0 * G.local.m[0][0] + s1 * G.local.m[1][0] + s2 * G.local.m[2][0];
                const D2 k1 = s0 * G.local.m[0][1] + s1 * G.local.m[1][1] + s2 * G.local.m[2][1];
                D2 gk = gabor_kernel2(w_f, ofx, ofy, phi_s, G.a_f, k0, k1);
                if (!isfinite(gk.v)) gk = gabor_kernel3(om, phi, G.a, xk);
                sum = sum + gk;
            } else {
                sum = sum + gabor_kernel3(om, phi, G.a, xk);
            }
        } else {
            // gabor_no_sample (sfm_gabornoise.h:283-297)
            if (G.anisotropic == 0) { rng.next(); rng.next(); }
            else if (G.anisotropic != 1) rng.next();
            rng.next();
        }
    }
    return sum;
}

// gabor / gabor3 / pgabor / pgabor3 of a Dual2<Vec3> position; nc = 1 or 3
static __device__ __noinline__ void gabor_eval(const GOpts& o, const DV3& P, bool periodic, V3 period, int nc, D2* out) {
    GaborState G;
    const float bw = o.bandwidth < 0.01f ? 0.01f : (o.bandwidth > 100.0f ? 100.0f : o.bandwidth);
    const float two_bw = (float)exp2((double)bw);
    G.a = 2.0f * ((two_bw - 1.0f) / (two_bw + 1.0f)) * 2.128934e+00f;
    // sqrtf(-logf(0.02f) / float(M_PI)) == 1.115901231765747f
    G.radius = 1.115901231765747f / G.a;
    G.radius2 = G.radius * G.radius;
    const float radius3 = G.radius2 * G.radius;
    G.radius_inv = 1.0f / G.radius;
    const float imp = o.impulses < 1.0f ? 1.0f : (o.impulses > 32.0f ? 32.0f : o.impulses);
    const float lambda = imp / (4.188779830932617f * radius3);
    G.sqrt_lambda_inv = 1.0f / sqrtf(lambda);
    G.poisson_g = (float)exp(-(double)(lambda * radius3));
    G.anisotropic = o.anisotropic;
    G.do_filter = o.do_filter;
    G.omega = o.direction;
    G.periodic = periodic;
    G.period = period;
    if (G.do_filter) {
        // gabor_setup_filter (sfm_gabornoise.h:163-215)
        V3 n = vcross(P.dx, P.dy);
        if (n.x * n.x + n.y * n.y + n.z * n.z < 1.0e-6f) {
            G.do_filter = 0;
        } else {
            n = vnormalize_imath(n);
            V3 t = fabsf(n.x) < 0.9f ? v3(0.0f, n.z, -n.y) : v3(-n.z, 0.0f, n.x);
            t = vnormalize_imath(t);
            const V3 b = vcross(n, t);
            const M33 tex_to_tan = m33_cols(t, b, n);
            const M33 scr_to_tan = m33_mul(m33_cols(P.dx, P.dy, v3(0.0f, 0.0f, 0.0f)), tex_to_tan);
            const M22 Ms = m22(scr_to_tan.m[0][0], scr_to_tan.m[0][1], scr_to_tan.m[1][0], scr_to_tan.m[1][1]);
            const M22 Sf = m22(0.5f * 0.5f, 0.0f, 0.0f, 0.5f * 0.5f);
            const M22 Mst = m22(Ms.m00, Ms.m10, Ms.m01, Ms.m11);
            const M22 filter = m22_mul(m22_mul(Mst, Sf), Ms);
            G.N = n;
            G.local = tex_to_tan;
            if (m22_det(filter) < 1.0e-18f) {
                G.do_filter = 0;
            } else {
                const M22 Sigma_G = m22_scale(G.a * G.a / 6.2831854820251465f, m22(1.0f, 0.0f, 0.0f, 1.0f));
                G.c_F = 1.0f / (6.2831854820251465f * sqrtf(m22_det(filter)));
                const M22 Sigma_F = m22_scale(0.02533029578626156f, m22_inverse(filter));
                const M22 SGSF = m22_add(Sigma_G, Sigma_F);
                G.inv_c_GF_den = 1.0f / (6.2831854820251465f * sqrtf(m22_det(SGSF)));
                G.SGSF_inv = m22_inverse(SGSF);
                const M22 Sigma_G_i = m22_inverse(Sigma_G);
                const M22 Sigma_GF = m22_inverse(m22_add(m22_inverse(Sigma_F), Sigma_G_i));
                G.Sigma_GF_Gi = m22_mul(Sigma_GF, Sigma_G_i);
                G.a_f = sqrtf((float)(6.283185307179586 * (double)sqrtf(m22_det(Sigma_GF))));
            }
        }
    }
    const float var = 1.0f / (4.0f * 1.4142135381698608f * (G.a * G.a * G.a));
    float scale = 1.0f / (3.0f * sqrtf(var));
    scale *= 0.5f;
    // gabor_evaluate / gabor_grid (sfm_gabornoise.h:399-485)
    const DV3 xg = dv3_scale(P, G.radius_inv);
    const V3 f = v3(floorf(xg.v.x), floorf(xg.v.y), floorf(xg.v.z));
    const DV3 xc = dv3_sub(xg, f);
    for (int ch = 0; ch < nc; ++ch) {
        D2 sum = d2c(0.0f);
        for (int k = -1; k <= 1; ++k)
            for (int j = -1; j <= 1; ++j)
                for (int i = -1; i <= 1; ++i) {
                    const V3 c = v3((float)i, (float)j, (float)k);
                    sum = sum + gabor_cell(G, vadd(f, c), dv3_sub(xc, c), ch);
                }
        out[ch] = (sum * G.sqrt_lambda_inv) * scale;
    }
}

}  // namespace dev
}  // namespace oslg
