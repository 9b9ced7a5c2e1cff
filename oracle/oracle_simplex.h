// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of OSL's simplex noise with analytic derivatives
// (src/liboslnoise/simplexnoise.cpp:58-128 scramble/LUTs, :166-200 1D,
// :204-300 2D, :331-480 3D, :522-740 4D). The batched shadeops call the
// SIMD-friendly form in src/include/OSL/sfm_simplex.h:565-1200, which
// evaluates every corner unconditionally and zeroes the contribution and
// gradient of corners with t<0; both forms give the same values, which is
// what this restatement computes. Wrappers: SimplexNoise / USimplexNoise
// (oslnoise.h:2765-3190): vector results use seeds 0,1,2; Dual2 results
// chain the analytic gradient with the input partials.
#pragma once
#include "oracle_noise.h"

namespace oracle {

inline uint32_t scramble(uint32_t v0, uint32_t v1 = 0, uint32_t v2 = 0) {
    return bjfinal(v0, v1, v2 ^ 0xdeadbeefu);
}

// simplexnoise.cpp:70-75
static const float kGrad2[8][2] = { { -1, -1 }, { 1, 0 }, { -1, 0 }, { 1, 1 },
                                    { -1, 1 },  { 0, -1 }, { 0, 1 }, { 1, -1 } };
// simplexnoise.cpp:82-91
static const float kGrad3[16][3] = { { 1, 0, 1 },  { 0, 1, 1 },   { -1, 0, 1 }, { 0, -1, 1 },
                                     { 1, 0, -1 }, { 0, 1, -1 },  { -1, 0, -1 }, { 0, -1, -1 },
                                     { 1, -1, 0 }, { 1, 1, 0 },   { -1, 1, 0 }, { -1, -1, 0 },
                                     { 1, 0, 1 },  { -1, 0, 1 },  { 0, 1, -1 }, { 0, -1, -1 } };
// simplexnoise.cpp:94-103: the 32 edges of a tesseract, in the order
// (0,+-1,+-1,+-1), (+-1,0,+-1,+-1), (+-1,+-1,0,+-1), (+-1,+-1,+-1,0)
// with the sign pattern counting +,+,+ ... -,-,- in binary.
struct Grad4Table {
    float g[32][4];
    Grad4Table() {
        for (int zeroax = 0; zeroax < 4; ++zeroax)
            for (int sgn = 0; sgn < 8; ++sgn) {
                int row = zeroax * 8 + sgn, bit = 2;
                for (int a = 0; a < 4; ++a) {
                    if (a == zeroax) { g[row][a] = 0.0f; continue; }
                    g[row][a] = ((sgn >> bit) & 1) ? -1.0f : 1.0f;
                    --bit;
                }
            }
    }
};
inline const float* grad4lut(int idx) { static const Grad4Table t; return t.g[idx]; }

// simplexnoise.cpp:108-126: 4D traversal order table. Entry c (built from
// six pairwise comparisons of the offsets) ranks each axis 0..3 by
// magnitude. Entries that no ordering can produce are {0,0,0,0}.
struct Simplex4Table {
    unsigned char t[64][4];
    Simplex4Table() {
        std::memset(t, 0, sizeof(t));
        int perm[4] = { 0, 1, 2, 3 };
        // Enumerate all orderings of 4 distinct magnitudes: rank r[a] is
        // the number of axes a beats.
        for (int p = 0; p < 24; ++p) {
            int r[4];
            int q = p, avail[4] = { 0, 1, 2, 3 }, n = 4;
            for (int a = 0; a < 4; ++a) {
                int f = 1;
                for (int k = 1; k < n; ++k) f *= k;
                int idx = q / f;
                q %= f;
                r[a] = avail[idx];
                for (int k = idx; k < n - 1; ++k) avail[k] = avail[k + 1];
                --n;
            }
            (void)perm;
            // axis a with rank r[a]; bigger rank = bigger coordinate
            int c = (r[0] > r[1] ? 32 : 0) | (r[0] > r[2] ? 16 : 0) | (r[1] > r[2] ? 8 : 0)
                  | (r[0] > r[3] ? 4 : 0) | (r[1] > r[3] ? 2 : 0) | (r[2] > r[3] ? 1 : 0);
            for (int a = 0; a < 4; ++a) t[c][a] = (unsigned char)r[a];
        }
    }
};
inline const unsigned char* simplex4lut(int c) { static const Simplex4Table t; return t.t[c]; }

inline float sgrad1(int i, int seed) {
    int h = (int)scramble((uint32_t)i, (uint32_t)seed);
    float g = 1.0f + (h & 7);
    if (h & 8) g = -g;
    return g;
}
inline const float* sgrad2(int i, int j, int seed) {
    return kGrad2[scramble((uint32_t)i, (uint32_t)j, (uint32_t)seed) & 7];
}
inline const float* sgrad3(int i, int j, int k, int seed) {
    return kGrad3[scramble((uint32_t)i, (uint32_t)j, scramble((uint32_t)k, (uint32_t)seed)) & 15];
}
inline const float* sgrad4(int i, int j, int k, int l, int seed) {
    return grad4lut(scramble((uint32_t)i, (uint32_t)j, scramble((uint32_t)k, (uint32_t)l, (uint32_t)seed)) & 31);
}

static const float kZero4[4] = { 0, 0, 0, 0 };

// simplexnoise.cpp:166-200
inline float simplex1(float x, int seed, float* dx) {
    int i0 = ifloor(x);
    int i1 = i0 + 1;
    float x0 = x - (float)i0;
    float x1 = x0 - 1.0f;
    float x20 = x0 * x0;
    float t0 = 1.0f - x20;
    float t20 = t0 * t0;
    float t40 = t20 * t20;
    float gx0 = sgrad1(i0, seed);
    float n0 = t40 * gx0 * x0;
    float x21 = x1 * x1;
    float t1 = 1.0f - x21;
    float t21 = t1 * t1;
    float t41 = t21 * t21;
    float gx1 = sgrad1(i1, seed);
    float n1 = t41 * gx1 * x1;
    const float scale = 0.36f;
    if (dx) {
        float d = t20 * t0 * gx0 * x20;
        d += t21 * t1 * gx1 * x21;
        d *= -8.0f;
        d += t40 * gx0 + t41 * gx1;
        d *= scale;
        *dx = d;
    }
    return scale * (n0 + n1);
}

// simplexnoise.cpp:204-300
inline float simplex2(float x, float y, int seed, float* ddx, float* ddy) {
    const float F2 = 0.366025403f;
    const float G2 = 0.211324865f;
    const float *g0 = kZero4, *g1 = kZero4, *g2 = kZero4;
    float s = (x + y) * F2;
    float xs = x + s, ys = y + s;
    int i = ifloor(xs), j = ifloor(ys);
    float t = (float)(i + j) * G2;
    float X0 = (float)i - t, Y0 = (float)j - t;
    float x0 = x - X0, y0 = y - Y0;
    int i1, j1;
    if (x0 > y0) { i1 = 1; j1 = 0; } else { i1 = 0; j1 = 1; }
    float x1 = x0 - (float)i1 + G2;
    float y1 = y0 - (float)j1 + G2;
    float x2 = x0 - 1.0f + 2.0f * G2;
    float y2 = y0 - 1.0f + 2.0f * G2;
    float t20 = 0, t40 = 0, t21 = 0, t41 = 0, t22 = 0, t42 = 0;
    float n0 = 0, n1 = 0, n2 = 0;
    float t0 = 0.5f - x0 * x0 - y0 * y0;
    if (t0 >= 0.0f) {
        g0 = sgrad2(i, j, seed);
        t20 = t0 * t0; t40 = t20 * t20;
        n0 = t40 * (g0[0] * x0 + g0[1] * y0);
    }
    float t1 = 0.5f - x1 * x1 - y1 * y1;
    if (t1 >= 0.0f) {
        g1 = sgrad2(i + i1, j + j1, seed);
        t21 = t1 * t1; t41 = t21 * t21;
        n1 = t41 * (g1[0] * x1 + g1[1] * y1);
    }
    float t2 = 0.5f - x2 * x2 - y2 * y2;
    if (t2 >= 0.0f) {
        g2 = sgrad2(i + 1, j + 1, seed);
        t22 = t2 * t2; t42 = t22 * t22;
        n2 = t42 * (g2[0] * x2 + g2[1] * y2);
    }
    const float scale = 64.0f;
    float noise = scale * (n0 + n1 + n2);
    if (ddx) {
        float temp0 = t20 * t0 * (g0[0] * x0 + g0[1] * y0);
        float dx = temp0 * x0, dy = temp0 * y0;
        float temp1 = t21 * t1 * (g1[0] * x1 + g1[1] * y1);
        dx += temp1 * x1; dy += temp1 * y1;
        float temp2 = t22 * t2 * (g2[0] * x2 + g2[1] * y2);
        dx += temp2 * x2; dy += temp2 * y2;
        dx *= -8.0f; dy *= -8.0f;
        dx += t40 * g0[0] + t41 * g1[0] + t42 * g2[0];
        dy += t40 * g0[1] + t41 * g1[1] + t42 * g2[1];
        dx *= scale; dy *= scale;
        *ddx = dx; *ddy = dy;
    }
    return noise;
}

// simplexnoise.cpp:331-480
inline float simplex3(float x, float y, float z, int seed, float* ddx, float* ddy, float* ddz) {
    const float F3 = 0.333333333f;
    const float G3 = 0.166666667f;
    const float *g0 = kZero4, *g1 = kZero4, *g2 = kZero4, *g3 = kZero4;
    float s = (x + y + z) * F3;
    float xs = x + s, ys = y + s, zs = z + s;
    int i = ifloor(xs), j = ifloor(ys), k = ifloor(zs);
    float t = (float)(i + j + k) * G3;
    float X0 = (float)i - t, Y0 = (float)j - t, Z0 = (float)k - t;
    float x0 = x - X0, y0 = y - Y0, z0 = z - Z0;
    int i1, j1, k1, i2, j2, k2;
    if (x0 >= y0) {
        if (y0 >= z0)      { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
        else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
        else               { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
    } else {
        if (y0 < z0)       { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
        else if (x0 < z0)  { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
        else               { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    }
    float x1 = x0 - (float)i1 + G3, y1 = y0 - (float)j1 + G3, z1 = z0 - (float)k1 + G3;
    float x2 = x0 - (float)i2 + 2.0f * G3, y2 = y0 - (float)j2 + 2.0f * G3, z2 = z0 - (float)k2 + 2.0f * G3;
    float x3 = x0 - 1.0f + 3.0f * G3, y3 = y0 - 1.0f + 3.0f * G3, z3 = z0 - 1.0f + 3.0f * G3;
    float t20 = 0, t40 = 0, t21 = 0, t41 = 0, t22 = 0, t42 = 0, t23 = 0, t43 = 0;
    float n0 = 0, n1 = 0, n2 = 0, n3 = 0;
    float t0 = 0.5f - x0 * x0 - y0 * y0 - z0 * z0;
    if (t0 >= 0.0f) {
        g0 = sgrad3(i, j, k, seed);
        t20 = t0 * t0; t40 = t20 * t20;
        n0 = t40 * (g0[0] * x0 + g0[1] * y0 + g0[2] * z0);
    }
    float t1 = 0.5f - x1 * x1 - y1 * y1 - z1 * z1;
    if (t1 >= 0.0f) {
        g1 = sgrad3(i + i1, j + j1, k + k1, seed);
        t21 = t1 * t1; t41 = t21 * t21;
        n1 = t41 * (g1[0] * x1 + g1[1] * y1 + g1[2] * z1);
    }
    float t2 = 0.5f - x2 * x2 - y2 * y2 - z2 * z2;
    if (t2 >= 0.0f) {
        g2 = sgrad3(i + i2, j + j2, k + k2, seed);
        t22 = t2 * t2; t42 = t22 * t22;
        n2 = t42 * (g2[0] * x2 + g2[1] * y2 + g2[2] * z2);
    }
    float t3 = 0.5f - x3 * x3 - y3 * y3 - z3 * z3;
    if (t3 >= 0.0f) {
        g3 = sgrad3(i + 1, j + 1, k + 1, seed);
        t23 = t3 * t3; t43 = t23 * t23;
        n3 = t43 * (g3[0] * x3 + g3[1] * y3 + g3[2] * z3);
    }
    const float scale = 68.0f;
    float noise = scale * (n0 + n1 + n2 + n3);
    if (ddx) {
        float temp0 = t20 * t0 * (g0[0] * x0 + g0[1] * y0 + g0[2] * z0);
        float dx = temp0 * x0, dy = temp0 * y0, dz = temp0 * z0;
        float temp1 = t21 * t1 * (g1[0] * x1 + g1[1] * y1 + g1[2] * z1);
        dx += temp1 * x1; dy += temp1 * y1; dz += temp1 * z1;
        float temp2 = t22 * t2 * (g2[0] * x2 + g2[1] * y2 + g2[2] * z2);
        dx += temp2 * x2; dy += temp2 * y2; dz += temp2 * z2;
        float temp3 = t23 * t3 * (g3[0] * x3 + g3[1] * y3 + g3[2] * z3);
        dx += temp3 * x3; dy += temp3 * y3; dz += temp3 * z3;
        dx *= -8.0f; dy *= -8.0f; dz *= -8.0f;
        dx += t40 * g0[0] + t41 * g1[0] + t42 * g2[0] + t43 * g3[0];
        dy += t40 * g0[1] + t41 * g1[1] + t42 * g2[1] + t43 * g3[1];
        dz += t40 * g0[2] + t41 * g1[2] + t42 * g2[2] + t43 * g3[2];
        dx *= scale; dy *= scale; dz *= scale;
        *ddx = dx; *ddy = dy; *ddz = dz;
    }
    return noise;
}

// simplexnoise.cpp:522-740
inline float simplex4(float x, float y, float z, float w, int seed, float* ddx, float* ddy,
                      float* ddz, float* ddw) {
    const float F4 = 0.309016994f;
    const float G4 = 0.138196601f;
    const float* g[5] = { kZero4, kZero4, kZero4, kZero4, kZero4 };
    float s = (x + y + z + w) * F4;
    int i = ifloor(x + s), j = ifloor(y + s), k = ifloor(z + s), l = ifloor(w + s);
    float t = (float)(i + j + k + l) * G4;
    float x0 = x - ((float)i - t), y0 = y - ((float)j - t);
    float z0 = z - ((float)k - t), w0 = w - ((float)l - t);
    int c = (x0 > y0 ? 32 : 0) | (x0 > z0 ? 16 : 0) | (y0 > z0 ? 8 : 0) | (x0 > w0 ? 4 : 0)
          | (y0 > w0 ? 2 : 0) | (z0 > w0 ? 1 : 0);
    const unsigned char* sc = simplex4lut(c);
    int o1[4], o2[4], o3[4];
    for (int a = 0; a < 4; ++a) {
        o1[a] = sc[a] >= 3 ? 1 : 0;
        o2[a] = sc[a] >= 2 ? 1 : 0;
        o3[a] = sc[a] >= 1 ? 1 : 0;
    }
    float cx[5], cy[5], cz[5], cw[5];
    cx[0] = x0; cy[0] = y0; cz[0] = z0; cw[0] = w0;
    cx[1] = x0 - (float)o1[0] + G4; cy[1] = y0 - (float)o1[1] + G4;
    cz[1] = z0 - (float)o1[2] + G4; cw[1] = w0 - (float)o1[3] + G4;
    cx[2] = x0 - (float)o2[0] + 2.0f * G4; cy[2] = y0 - (float)o2[1] + 2.0f * G4;
    cz[2] = z0 - (float)o2[2] + 2.0f * G4; cw[2] = w0 - (float)o2[3] + 2.0f * G4;
    cx[3] = x0 - (float)o3[0] + 3.0f * G4; cy[3] = y0 - (float)o3[1] + 3.0f * G4;
    cz[3] = z0 - (float)o3[2] + 3.0f * G4; cw[3] = w0 - (float)o3[3] + 3.0f * G4;
    cx[4] = x0 - 1.0f + 4.0f * G4; cy[4] = y0 - 1.0f + 4.0f * G4;
    cz[4] = z0 - 1.0f + 4.0f * G4; cw[4] = w0 - 1.0f + 4.0f * G4;
    int ci[5] = { i, i + o1[0], i + o2[0], i + o3[0], i + 1 };
    int cj[5] = { j, j + o1[1], j + o2[1], j + o3[1], j + 1 };
    int ck[5] = { k, k + o1[2], k + o2[2], k + o3[2], k + 1 };
    int cl[5] = { l, l + o1[3], l + o2[3], l + o3[3], l + 1 };
    float tt[5], t2[5] = { 0, 0, 0, 0, 0 }, t4[5] = { 0, 0, 0, 0, 0 }, n[5] = { 0, 0, 0, 0, 0 };
    for (int q = 0; q < 5; ++q) {
        tt[q] = 0.5f - cx[q] * cx[q] - cy[q] * cy[q] - cz[q] * cz[q] - cw[q] * cw[q];
        if (tt[q] >= 0.0f) {
            t2[q] = tt[q] * tt[q];
            t4[q] = t2[q] * t2[q];
            g[q] = sgrad4(ci[q], cj[q], ck[q], cl[q], seed);
            n[q] = t4[q] * (g[q][0] * cx[q] + g[q][1] * cy[q] + g[q][2] * cz[q] + g[q][3] * cw[q]);
        }
    }
    const float scale = 54.0f;
    float noise = scale * (n[0] + n[1] + n[2] + n[3] + n[4]);
    if (ddx) {
        float dx = 0, dy = 0, dz = 0, dw = 0;
        for (int q = 0; q < 5; ++q) {
            float temp = t2[q] * tt[q]
                       * (g[q][0] * cx[q] + g[q][1] * cy[q] + g[q][2] * cz[q] + g[q][3] * cw[q]);
            if (q == 0) {
                dx = temp * cx[q]; dy = temp * cy[q]; dz = temp * cz[q]; dw = temp * cw[q];
            } else {
                dx += temp * cx[q]; dy += temp * cy[q]; dz += temp * cz[q]; dw += temp * cw[q];
            }
        }
        dx *= -8.0f; dy *= -8.0f; dz *= -8.0f; dw *= -8.0f;
        dx += t4[0] * g[0][0] + t4[1] * g[1][0] + t4[2] * g[2][0] + t4[3] * g[3][0] + t4[4] * g[4][0];
        dy += t4[0] * g[0][1] + t4[1] * g[1][1] + t4[2] * g[2][1] + t4[3] * g[3][1] + t4[4] * g[4][1];
        dz += t4[0] * g[0][2] + t4[1] * g[1][2] + t4[2] * g[2][2] + t4[3] * g[3][2] + t4[4] * g[4][2];
        dw += t4[0] * g[0][3] + t4[1] * g[1][3] + t4[2] * g[2][3] + t4[3] * g[3][3] + t4[4] * g[4][3];
        dx *= scale; dy *= scale; dz *= scale; dw *= scale;
        *ddx = dx; *ddy = dy; *ddz = dz; *ddw = dw;
    }
    return noise;
}

// SimplexNoise Dual2 wrappers (oslnoise.h:2805-2840): value plus the
// analytic gradient chained with each input's partials.
inline DF simplex_dual(int dim, const DF* xs, int seed) {
    float d[4] = { 0, 0, 0, 0 };
    float r;
    switch (dim) {
    case 1:
        r = simplex1(xs[0].v, seed, &d[0]);
        return DF(r, d[0] * xs[0].dx, d[0] * xs[0].dy);
    case 2:
        r = simplex2(xs[0].v, xs[1].v, seed, &d[0], &d[1]);
        return DF(r, d[0] * xs[0].dx + d[1] * xs[1].dx, d[0] * xs[0].dy + d[1] * xs[1].dy);
    case 3:
        r = simplex3(xs[0].v, xs[1].v, xs[2].v, seed, &d[0], &d[1], &d[2]);
        return DF(r, d[0] * xs[0].dx + d[1] * xs[1].dx + d[2] * xs[2].dx,
                  d[0] * xs[0].dy + d[1] * xs[1].dy + d[2] * xs[2].dy);
    default:
        r = simplex4(xs[0].v, xs[1].v, xs[2].v, xs[3].v, seed, &d[0], &d[1], &d[2], &d[3]);
        return DF(r, d[0] * xs[0].dx + d[1] * xs[1].dx + d[2] * xs[2].dx + d[3] * xs[3].dx,
                  d[0] * xs[0].dy + d[1] * xs[1].dy + d[2] * xs[2].dy + d[3] * xs[3].dy);
    }
}
inline float simplex_val(int dim, const float* xs, int seed) {
    switch (dim) {
    case 1: return simplex1(xs[0], seed, nullptr);
    case 2: return simplex2(xs[0], xs[1], seed, nullptr, nullptr);
    case 3: return simplex3(xs[0], xs[1], xs[2], seed, nullptr, nullptr, nullptr);
    default: return simplex4(xs[0], xs[1], xs[2], xs[3], seed, nullptr, nullptr, nullptr, nullptr);
    }
}

}  // namespace oracle
