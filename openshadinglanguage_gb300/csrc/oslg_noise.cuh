// Device noise library for the sm_103a interpreter.
//
// Perlin ("perlin"/"uperlin" and periodic forms), cell, hash and simplex
// noise with Dual2 derivatives, computing the same IEEE operations in the
// same order as the reference's scalar (full-batch "CGScalar") code:
//   src/include/OSL/oslnoise.h:135-329 (hashes), :337-550 (cell/hash),
//   :847-1041 (floorfrac/fade/grad/scale), :1327-2280 (perlin),
//   :2284-2762 (wrappers); src/liboslnoise/simplexnoise.cpp (simplex).
// The translation unit is built with -fmad=false so no multiply-add is
// contracted: the results are bit-identical to a non-FMA build of that code.
//
// GPU organisation: the 8 (3D) or 16 (4D) lattice hashes are computed once
// per point and shared by the three channels of a vector noise; channel c
// reads its gradient selector from byte c of the hash (HashVector's
// sliceup). Rotations are single funnel shifts.
#pragma once
#include <stdint.h>

namespace oslg {
namespace dev {

struct D2 {
    float v, dx, dy;
};
__device__ __forceinline__ D2 d2(float v, float dx, float dy) { D2 r; r.v = v; r.dx = dx; r.dy = dy; return r; }
__device__ __forceinline__ D2 d2c(float v) { return d2(v, 0.0f, 0.0f); }

// Dual2 arithmetic, operand order as src/include/OSL/dual.h:403-620
__device__ __forceinline__ D2 operator+(D2 a, D2 b) { return d2(a.v + b.v, a.dx + b.dx, a.dy + b.dy); }
__device__ __forceinline__ D2 operator-(D2 a, D2 b) { return d2(a.v - b.v, a.dx - b.dx, a.dy - b.dy); }
__device__ __forceinline__ D2 operator-(D2 a, float b) { return d2(a.v - b, a.dx, a.dy); }
__device__ __forceinline__ D2 operator+(D2 a, float b) { return d2(a.v + b, a.dx, a.dy); }
__device__ __forceinline__ D2 operator-(D2 a) { return d2(-a.v, -a.dx, -a.dy); }
__device__ __forceinline__ D2 operator*(D2 a, D2 b) {
    return d2(a.v * b.v, a.v * b.dx + a.dx * b.v, a.v * b.dy + a.dy * b.v);
}
__device__ __forceinline__ D2 operator*(D2 a, float b) { return d2(a.v * b, a.dx * b, a.dy * b); }
__device__ __forceinline__ D2 operator*(float b, D2 a) { return d2(a.v * b, a.dx * b, a.dy * b); }
__device__ __forceinline__ D2 operator-(float a, D2 b) { return d2(a - b.v, -b.dx, -b.dy); }
__device__ __forceinline__ D2 operator+(float a, D2 b) { return d2(a + b.v, b.dx, b.dy); }
__device__ __forceinline__ D2 operator/(D2 a, D2 b) {
    const float binv = 1.0f / b.v, ab = a.v / b.v;
    return d2(ab, binv * (a.dx - ab * b.dx), binv * (a.dy - ab * b.dy));
}
__device__ __forceinline__ D2 operator/(float a, D2 b) {
    const float binv = 1.0f / b.v, ab = a / b.v;
    return d2(ab, binv * (-ab * b.dx), binv * (-ab * b.dy));
}
__device__ __forceinline__ D2 operator/(D2 a, float b) {
    const float binv = 1.0f / b;
    return d2(a.v / b, binv * a.dx, binv * a.dy);
}

__device__ __forceinline__ uint32_t rotl(uint32_t x, int k) { return __funnelshift_l(x, x, k); }

__device__ __forceinline__ void bjmix(uint32_t& a, uint32_t& b, uint32_t& c) {
    a -= c; a ^= rotl(c, 4);  c += b;
    b -= a; b ^= rotl(a, 6);  a += c;
    c -= b; c ^= rotl(b, 8);  b += a;
    a -= c; a ^= rotl(c, 16); c += b;
    b -= a; b ^= rotl(a, 19); a += c;
    c -= b; c ^= rotl(b, 4);  b += a;
}
__device__ __forceinline__ uint32_t bjfinal(uint32_t a, uint32_t b, uint32_t c) {
    c ^= b; c -= rotl(b, 14);
    a ^= c; a -= rotl(c, 11);
    b ^= a; b -= rotl(a, 25);
    c ^= b; c -= rotl(b, 16);
    a ^= c; a -= rotl(c, 4);
    b ^= a; b -= rotl(a, 14);
    c ^= b; c -= rotl(b, 24);
    return c;
}
__device__ __forceinline__ float bits_to_01(uint32_t bits) {
    return (float)bits * (float)(1.0 / 4294967295.0);
}
__device__ __forceinline__ uint32_t inthash1(uint32_t k0) {
    const uint32_t s = 0xdeadbeefu + (1u << 2) + 13u;
    return bjfinal(s + k0, s, s);
}
__device__ __forceinline__ uint32_t inthash2(uint32_t k0, uint32_t k1) {
    const uint32_t s = 0xdeadbeefu + (2u << 2) + 13u;
    return bjfinal(s + k0, s + k1, s);
}
__device__ __forceinline__ uint32_t inthash3(uint32_t k0, uint32_t k1, uint32_t k2) {
    const uint32_t s = 0xdeadbeefu + (3u << 2) + 13u;
    return bjfinal(s + k0, s + k1, s + k2);
}
__device__ __forceinline__ uint32_t inthash4(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3) {
    const uint32_t s = 0xdeadbeefu + (4u << 2) + 13u;
    uint32_t a = s + k0, b = s + k1, c = s + k2;
    bjmix(a, b, c);
    a += k3;
    return bjfinal(a, b, c);
}
__device__ __forceinline__ uint32_t inthash5(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3, uint32_t k4) {
    const uint32_t s = 0xdeadbeefu + (5u << 2) + 13u;
    uint32_t a = s + k0, b = s + k1, c = s + k2;
    bjmix(a, b, c);
    b += k4;
    a += k3;
    return bjfinal(a, b, c);
}

// floor + saturating conversion (NaN -> 0); cvt.rmi.s32.f32
__device__ __forceinline__ int ifloor(float x) { return __float2int_rd(x); }

__device__ __forceinline__ float floorfrac(float x, int& i) { i = ifloor(x); return x - (float)i; }
__device__ __forceinline__ D2 floorfrac(D2 x, int& i) { i = ifloor(x.v); return d2(x.v - (float)i, x.dx, x.dy); }

__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
// fade on a Dual2 with dual constants 6, 15, 10 (zero partials): the
// product rule terms against a zero partial vanish, so t*6 has partials
// t.dx*6 and the additions of the constants leave the partials unchanged.
__device__ __forceinline__ D2 fade(D2 t) {
    D2 t2 = t * t;
    D2 t3 = t2 * t;
    D2 a = d2(t.v * 6.0f, t.dx * 6.0f, t.dy * 6.0f);
    a = a - 15.0f;
    D2 b = t * a;
    b = b + 10.0f;
    return t3 * b;
}

__device__ __forceinline__ float one_minus(float t) { return 1.0f - t; }
__device__ __forceinline__ D2 one_minus(D2 t) { return d2(1.0f - t.v, -t.dx, -t.dy); }

__device__ __forceinline__ float negate_if(float v, bool c) { return c ? -v : v; }
__device__ __forceinline__ D2 negate_if(D2 v, bool c) { return c ? -v : v; }
__device__ __forceinline__ float sel(bool c, float a, float b) { return c ? a : b; }
__device__ __forceinline__ D2 sel(bool c, D2 a, D2 b) { return c ? a : b; }

__device__ __forceinline__ float grad1(int hash, float x) {
    int h = hash & 15;
    float g = (float)(1 + (h & 7));
    if (h & 8) g = -g;
    return g * x;
}
__device__ __forceinline__ D2 grad1(int hash, D2 x) {
    int h = hash & 15;
    float g = (float)(1 + (h & 7));
    if (h & 8) g = -g;
    return x * g;
}
template <class T> __device__ __forceinline__ T grad2(int hash, T x, T y) {
    int h = hash & 7;
    T u = sel(h < 4, x, y);
    T v = sel(h < 4, y, x) * 2.0f;
    return negate_if(u, h & 1) + negate_if(v, h & 2);
}
template <class T> __device__ __forceinline__ T grad3(int hash, T x, T y, T z) {
    int h = hash & 15;
    T u = sel(h < 8, x, y);
    T v = sel(h < 4, y, sel(h == 12 || h == 14, x, z));
    return negate_if(u, h & 1) + negate_if(v, h & 2);
}
template <class T> __device__ __forceinline__ T grad4(int hash, T x, T y, T z, T w) {
    int h = hash & 31;
    T u = sel(h < 24, x, y);
    T v = sel(h < 16, y, z);
    T s = sel(h < 8, z, w);
    return negate_if(u, h & 1) + negate_if(v, h & 2) + negate_if(s, h & 4);
}

// OIIO lerp/bilerp/trilerp forms: a*(1-t) + b*t etc.
template <class T> __device__ __forceinline__ T mulw(T a, T w);
template <> __device__ __forceinline__ float mulw(float a, float w) { return a * w; }
template <> __device__ __forceinline__ D2 mulw(D2 a, D2 w) { return a * w; }

template <class T> __device__ __forceinline__ T lerp(T a, T b, T t) {
    return mulw(a, one_minus(t)) + mulw(b, t);
}
template <class T> __device__ __forceinline__ T bilerp(T v0, T v1, T v2, T v3, T s, T t) {
    T s1 = one_minus(s);
    return mulw(one_minus(t), mulw(v0, s1) + mulw(v1, s)) + mulw(t, mulw(v2, s1) + mulw(v3, s));
}
template <class T>
__device__ __forceinline__ T trilerp(T v0, T v1, T v2, T v3, T v4, T v5, T v6, T v7, T s, T t, T r) {
    T s1 = one_minus(s), t1 = one_minus(t), r1 = one_minus(r);
    return mulw(r1, mulw(t1, mulw(v0, s1) + mulw(v1, s)) + mulw(t, mulw(v2, s1) + mulw(v3, s)))
         + mulw(r, mulw(t1, mulw(v4, s1) + mulw(v5, s)) + mulw(t, mulw(v6, s1) + mulw(v7, s)));
}

__device__ __forceinline__ int imod(int a, int b) {
    int r = a % b;
    if (r < 0) r += b;
    return r;
}

// Lattice hasher; periodic hashers wrap each coordinate first
// (oslnoise.h:1157-1310).
struct Hasher {
    int px, py, pz, pw;
    bool periodic;
    __device__ __forceinline__ uint32_t wx(int x) const { return (uint32_t)(periodic ? imod(x, px) : x); }
    __device__ __forceinline__ uint32_t wy(int y) const { return (uint32_t)(periodic ? imod(y, py) : y); }
    __device__ __forceinline__ uint32_t wz(int z) const { return (uint32_t)(periodic ? imod(z, pz) : z); }
    __device__ __forceinline__ uint32_t ww(int w) const { return (uint32_t)(periodic ? imod(w, pw) : w); }
    __device__ __forceinline__ int h1(int x) const { return (int)inthash1(wx(x)); }
    __device__ __forceinline__ int h2(int x, int y) const { return (int)inthash2(wx(x), wy(y)); }
    __device__ __forceinline__ int h3(int x, int y, int z) const { return (int)inthash3(wx(x), wy(y), wz(z)); }
    __device__ __forceinline__ int h4(int x, int y, int z, int w) const {
        return (int)inthash4(wx(x), wy(y), wz(z), ww(w));
    }
};
__device__ __forceinline__ int period_of(float p) {
    int i = ifloor(p);
    return i < 1 ? 1 : i;
}

__device__ __forceinline__ int chan(int h, int c) { return c == 0 ? h : ((h >> (8 * c)) & 0xFF); }

// Perlin, all channels of one lookup. T = float or D2. NC = 1 or 3.
template <class T, int NC>
__device__ __forceinline__ void perlin1(const Hasher& H, T x, T* out) {
    int X; T fx = floorfrac(x, X);
    T u = fade(fx);
    int h0 = H.h1(X), h1 = H.h1(X + 1);
    T fx1 = fx - 1.0f;
#pragma unroll
    for (int c = 0; c < NC; ++c) out[c] = lerp(grad1(chan(h0, c), fx), grad1(chan(h1, c), fx1), u) * 0.2500f;
}
template <class T, int NC>
__device__ __forceinline__ void perlin2(const Hasher& H, T x, T y, T* out) {
    int X; T fx = floorfrac(x, X);
    int Y; T fy = floorfrac(y, Y);
    T u = fade(fx), v = fade(fy);
    int h00 = H.h2(X, Y), h10 = H.h2(X + 1, Y), h01 = H.h2(X, Y + 1), h11 = H.h2(X + 1, Y + 1);
    T fx1 = fx - 1.0f, fy1 = fy - 1.0f;
#pragma unroll
    for (int c = 0; c < NC; ++c)
        out[c] = bilerp(grad2(chan(h00, c), fx, fy), grad2(chan(h10, c), fx1, fy), grad2(chan(h01, c), fx, fy1),
                        grad2(chan(h11, c), fx1, fy1), u, v)
               * 0.6616f;
}
template <class T, int NC>
__device__ __forceinline__ void perlin3(const Hasher& H, T x, T y, T z, T* out) {
    int X; T fx = floorfrac(x, X);
    int Y; T fy = floorfrac(y, Y);
    int Z; T fz = floorfrac(z, Z);
    T u = fade(fx), v = fade(fy), w = fade(fz);
    int h[8];
    h[0] = H.h3(X, Y, Z);         h[1] = H.h3(X + 1, Y, Z);
    h[2] = H.h3(X, Y + 1, Z);     h[3] = H.h3(X + 1, Y + 1, Z);
    h[4] = H.h3(X, Y, Z + 1);     h[5] = H.h3(X + 1, Y, Z + 1);
    h[6] = H.h3(X, Y + 1, Z + 1); h[7] = H.h3(X + 1, Y + 1, Z + 1);
    T fx1 = fx - 1.0f, fy1 = fy - 1.0f, fz1 = fz - 1.0f;
#pragma unroll
    for (int c = 0; c < NC; ++c)
        out[c] = trilerp(grad3(chan(h[0], c), fx, fy, fz), grad3(chan(h[1], c), fx1, fy, fz),
                         grad3(chan(h[2], c), fx, fy1, fz), grad3(chan(h[3], c), fx1, fy1, fz),
                         grad3(chan(h[4], c), fx, fy, fz1), grad3(chan(h[5], c), fx1, fy, fz1),
                         grad3(chan(h[6], c), fx, fy1, fz1), grad3(chan(h[7], c), fx1, fy1, fz1), u, v, w)
               * 0.9820f;
}
template <class T, int NC>
__device__ __forceinline__ void perlin4(const Hasher& H, T x, T y, T z, T w, T* out) {
    int X; T fx = floorfrac(x, X);
    int Y; T fy = floorfrac(y, Y);
    int Z; T fz = floorfrac(z, Z);
    int W; T fw = floorfrac(w, W);
    T u = fade(fx), v = fade(fy), t = fade(fz), s = fade(fw);
    int h[16];
#pragma unroll
    for (int i = 0; i < 16; ++i)
        h[i] = H.h4(X + (i & 1), Y + ((i >> 1) & 1), Z + ((i >> 2) & 1), W + ((i >> 3) & 1));
    T fx1 = fx - 1.0f, fy1 = fy - 1.0f, fz1 = fz - 1.0f, fw1 = fw - 1.0f;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        T a = trilerp(grad4(chan(h[0], c), fx, fy, fz, fw), grad4(chan(h[1], c), fx1, fy, fz, fw),
                      grad4(chan(h[2], c), fx, fy1, fz, fw), grad4(chan(h[3], c), fx1, fy1, fz, fw),
                      grad4(chan(h[4], c), fx, fy, fz1, fw), grad4(chan(h[5], c), fx1, fy, fz1, fw),
                      grad4(chan(h[6], c), fx, fy1, fz1, fw), grad4(chan(h[7], c), fx1, fy1, fz1, fw), u, v, t);
        T b = trilerp(grad4(chan(h[8], c), fx, fy, fz, fw1), grad4(chan(h[9], c), fx1, fy, fz, fw1),
                      grad4(chan(h[10], c), fx, fy1, fz, fw1), grad4(chan(h[11], c), fx1, fy1, fz, fw1),
                      grad4(chan(h[12], c), fx, fy, fz1, fw1), grad4(chan(h[13], c), fx1, fy, fz1, fw1),
                      grad4(chan(h[14], c), fx, fy1, fz1, fw1), grad4(chan(h[15], c), fx1, fy1, fz1, fw1), u,
                      v, t);
        out[c] = lerp(a, b, s) * 0.8344f;
    }
}

// ---- cell / hash noise ----------------------------------------------------------
__device__ __forceinline__ uint32_t fbits(float f) { return __float_as_uint(f); }

// keys: cell -> ifloor, hash -> bit pattern
__device__ __forceinline__ uint32_t ikey(float v, bool cell) { return cell ? (uint32_t)ifloor(v) : fbits(v); }

// out[c] for c < nc; dims 1..4
__device__ __forceinline__ void intnoise(bool cell, int dims, const float* x, int nc, float* out) {
    uint32_t k0 = ikey(x[0], cell);
    if (nc == 1) {
        uint32_t h;
        switch (dims) {
        case 1: h = inthash1(k0); break;
        case 2: h = inthash2(k0, ikey(x[1], cell)); break;
        case 3: h = inthash3(k0, ikey(x[1], cell), ikey(x[2], cell)); break;
        default: h = inthash4(k0, ikey(x[1], cell), ikey(x[2], cell), ikey(x[3], cell)); break;
        }
        out[0] = bits_to_01(h);
        return;
    }
    switch (dims) {
    case 1:
        for (int c = 0; c < 3; ++c) out[c] = bits_to_01(inthash2(k0, (uint32_t)c));
        break;
    case 2: {
        uint32_t k1 = ikey(x[1], cell);
        for (int c = 0; c < 3; ++c) out[c] = bits_to_01(inthash3(k0, k1, (uint32_t)c));
        break;
    }
    case 3: {
        // shared bjmix (oslnoise.h:416-435)
        const uint32_t s = 0xdeadbeefu + (4u << 2) + 13u;
        uint32_t a = s + k0, b = s + ikey(x[1], cell), cc = s + ikey(x[2], cell);
        bjmix(a, b, cc);
        for (int c = 0; c < 3; ++c) out[c] = bits_to_01(bjfinal(a + (uint32_t)c, b, cc));
        break;
    }
    default: {
        const uint32_t s = 0xdeadbeefu + (5u << 2) + 13u;
        uint32_t a = s + k0, b = s + ikey(x[1], cell), cc = s + ikey(x[2], cell);
        bjmix(a, b, cc);
        uint32_t a2 = a + ikey(x[3], cell);
        for (int c = 0; c < 3; ++c) out[c] = bits_to_01(bjfinal(a2, b + (uint32_t)c, cc));
        break;
    }
    }
}

__device__ __forceinline__ float pwrap(float s, float period) {
    period = floorf(period);
    if (period < 1.0f) period = 1.0f;
    return s - period * floorf(s / period);
}

// ---- simplex (simplexnoise.cpp) --------------------------------------------------
__device__ __forceinline__ uint32_t scramble(uint32_t v0, uint32_t v1, uint32_t v2) {
    return bjfinal(v0, v1, v2 ^ 0xdeadbeefu);
}
__device__ __forceinline__ float sgrad1(int i, int seed) {
    int h = (int)scramble((uint32_t)i, (uint32_t)seed, 0u);
    float g = 1.0f + (float)(h & 7);
    if (h & 8) g = -g;
    return g;
}
// grad2lut (simplexnoise.cpp:70-75) as bit masks: entry e has x=+1 if bit e
// of 0x8A (entries 1,3,7), x=-1 if bit e of 0x15 (0,2,4); y=+1 for 0x58
// (3,4,6), y=-1 for 0xA1 (0,5,7).
__device__ __forceinline__ void sgrad2(int i, int j, int seed, float& gx, float& gy) {
    uint32_t e = scramble((uint32_t)i, (uint32_t)j, (uint32_t)seed) & 7u;
    uint32_t b = 1u << e;
    gx = (b & 0x8Au) ? 1.0f : ((b & 0x15u) ? -1.0f : 0.0f);
    gy = (b & 0x58u) ? 1.0f : ((b & 0xA1u) ? -1.0f : 0.0f);
}
// grad3lut (simplexnoise.cpp:82-91) as bit masks over the 16 entries
__device__ __forceinline__ void sgrad3(int i, int j, int k, int seed, float& gx, float& gy, float& gz) {
    uint32_t e = scramble((uint32_t)i, (uint32_t)j, scramble((uint32_t)k, (uint32_t)seed, 0u)) & 15u;
    uint32_t b = 1u << e;
    gx = (b & 0x1311u) ? 1.0f : ((b & 0x2C44u) ? -1.0f : 0.0f);
    gy = (b & 0x4622u) ? 1.0f : ((b & 0x8988u) ? -1.0f : 0.0f);
    gz = (b & 0x300Fu) ? 1.0f : ((b & 0xC0F0u) ? -1.0f : 0.0f);
}
// grad4lut (simplexnoise.cpp:94-103): row r = 8*zero_axis + sign bits
__device__ __forceinline__ void sgrad4(int i, int j, int k, int l, int seed, float* g) {
    uint32_t e = scramble((uint32_t)i, (uint32_t)j, scramble((uint32_t)k, (uint32_t)l, (uint32_t)seed)) & 31u;
    int zero = (int)(e >> 3), sgn = (int)(e & 7u), bit = 2;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (a == zero) { g[a] = 0.0f; continue; }
        g[a] = ((sgn >> bit) & 1) ? -1.0f : 1.0f;
        --bit;
    }
}

__device__ __forceinline__ float simplex1(float x, int seed, float* ddx) {
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
    if (ddx) {
        float d = t20 * t0 * gx0 * x20;
        d += t21 * t1 * gx1 * x21;
        d *= -8.0f;
        d += t40 * gx0 + t41 * gx1;
        d *= scale;
        *ddx = d;
    }
    return scale * (n0 + n1);
}

__device__ __forceinline__ float simplex2(float x, float y, int seed, float* ddx, float* ddy) {
    const float F2 = 0.366025403f, G2 = 0.211324865f;
    float s = (x + y) * F2;
    int i = ifloor(x + s), j = ifloor(y + s);
    float t = (float)(i + j) * G2;
    float x0 = x - ((float)i - t), y0 = y - ((float)j - t);
    int i1 = x0 > y0 ? 1 : 0, j1 = 1 - i1;
    float x1 = x0 - (float)i1 + G2, y1 = y0 - (float)j1 + G2;
    float x2 = x0 - 1.0f + 2.0f * G2, y2 = y0 - 1.0f + 2.0f * G2;
    float cx[3] = { x0, x1, x2 }, cy[3] = { y0, y1, y2 };
    int ci[3] = { i, i + i1, i + 1 }, cj[3] = { j, j + j1, j + 1 };
    float tt[3], t2[3], t4[3], gx[3], gy[3], n[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        tt[q] = 0.5f - cx[q] * cx[q] - cy[q] * cy[q];
        t2[q] = 0.0f; t4[q] = 0.0f; gx[q] = 0.0f; gy[q] = 0.0f; n[q] = 0.0f;
        if (tt[q] >= 0.0f) {
            sgrad2(ci[q], cj[q], seed, gx[q], gy[q]);
            t2[q] = tt[q] * tt[q];
            t4[q] = t2[q] * t2[q];
            n[q] = t4[q] * (gx[q] * cx[q] + gy[q] * cy[q]);
        }
    }
    const float scale = 64.0f;
    float noise = scale * (n[0] + n[1] + n[2]);
    if (ddx) {
        float dx = 0.0f, dy = 0.0f;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            float temp = t2[q] * tt[q] * (gx[q] * cx[q] + gy[q] * cy[q]);
            if (q == 0) { dx = temp * cx[q]; dy = temp * cy[q]; }
            else { dx += temp * cx[q]; dy += temp * cy[q]; }
        }
        dx *= -8.0f; dy *= -8.0f;
        dx += t4[0] * gx[0] + t4[1] * gx[1] + t4[2] * gx[2];
        dy += t4[0] * gy[0] + t4[1] * gy[1] + t4[2] * gy[2];
        *ddx = dx * scale; *ddy = dy * scale;
    }
    return noise;
}

__device__ __forceinline__ float simplex3(float x, float y, float z, int seed, float* ddx, float* ddy,
                                          float* ddz) {
    const float F3 = 0.333333333f, G3 = 0.166666667f;
    float s = (x + y + z) * F3;
    int i = ifloor(x + s), j = ifloor(y + s), k = ifloor(z + s);
    float t = (float)(i + j + k) * G3;
    float x0 = x - ((float)i - t), y0 = y - ((float)j - t), z0 = z - ((float)k - t);
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
    float cx[4] = { x0, x0 - (float)i1 + G3, x0 - (float)i2 + 2.0f * G3, x0 - 1.0f + 3.0f * G3 };
    float cy[4] = { y0, y0 - (float)j1 + G3, y0 - (float)j2 + 2.0f * G3, y0 - 1.0f + 3.0f * G3 };
    float cz[4] = { z0, z0 - (float)k1 + G3, z0 - (float)k2 + 2.0f * G3, z0 - 1.0f + 3.0f * G3 };
    int ci[4] = { i, i + i1, i + i2, i + 1 }, cj[4] = { j, j + j1, j + j2, j + 1 },
        ck[4] = { k, k + k1, k + k2, k + 1 };
    float tt[4], t2[4], t4[4], gx[4], gy[4], gz[4], n[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        tt[q] = 0.5f - cx[q] * cx[q] - cy[q] * cy[q] - cz[q] * cz[q];
        t2[q] = 0.0f; t4[q] = 0.0f; gx[q] = 0.0f; gy[q] = 0.0f; gz[q] = 0.0f; n[q] = 0.0f;
        if (tt[q] >= 0.0f) {
            sgrad3(ci[q], cj[q], ck[q], seed, gx[q], gy[q], gz[q]);
            t2[q] = tt[q] * tt[q];
            t4[q] = t2[q] * t2[q];
            n[q] = t4[q] * (gx[q] * cx[q] + gy[q] * cy[q] + gz[q] * cz[q]);
        }
    }
    const float scale = 68.0f;
    float noise = scale * (n[0] + n[1] + n[2] + n[3]);
    if (ddx) {
        float dx = 0.0f, dy = 0.0f, dz = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            float temp = t2[q] * tt[q] * (gx[q] * cx[q] + gy[q] * cy[q] + gz[q] * cz[q]);
            if (q == 0) { dx = temp * cx[q]; dy = temp * cy[q]; dz = temp * cz[q]; }
            else { dx += temp * cx[q]; dy += temp * cy[q]; dz += temp * cz[q]; }
        }
        dx *= -8.0f; dy *= -8.0f; dz *= -8.0f;
        dx += t4[0] * gx[0] + t4[1] * gx[1] + t4[2] * gx[2] + t4[3] * gx[3];
        dy += t4[0] * gy[0] + t4[1] * gy[1] + t4[2] * gy[2] + t4[3] * gy[3];
        dz += t4[0] * gz[0] + t4[1] * gz[1] + t4[2] * gz[2] + t4[3] * gz[3];
        *ddx = dx * scale; *ddy = dy * scale; *ddz = dz * scale;
    }
    return noise;
}

__device__ __forceinline__ float simplex4(float x, float y, float z, float w, int seed, float* dd) {
    const float F4 = 0.309016994f, G4 = 0.138196601f;
    float s = (x + y + z + w) * F4;
    int i = ifloor(x + s), j = ifloor(y + s), k = ifloor(z + s), l = ifloor(w + s);
    float t = (float)(i + j + k + l) * G4;
    float x0 = x - ((float)i - t), y0 = y - ((float)j - t), z0 = z - ((float)k - t), w0 = w - ((float)l - t);
    // simplexnoise.cpp:108-126 looks the axis ranks up in a table indexed by
    // six pairwise comparisons; with strict '>' every comparison pattern is
    // that of a strict order (ties favour the later axis), and each entry is
    // the number of axes that axis beats, counted here directly.
    const int c1 = x0 > y0, c2 = x0 > z0, c3 = y0 > z0, c4 = x0 > w0, c5 = y0 > w0, c6 = z0 > w0;
    int sc[4] = { c1 + c2 + c4, (1 - c1) + c3 + c5, (1 - c2) + (1 - c3) + c6, (1 - c4) + (1 - c5) + (1 - c6) };
    float cx[5], cy[5], cz[5], cw[5];
    int ci[5], cj[5], ck[5], cl[5];
    cx[0] = x0; cy[0] = y0; cz[0] = z0; cw[0] = w0;
    ci[0] = i; cj[0] = j; ck[0] = k; cl[0] = l;
#pragma unroll
    for (int q = 1; q <= 3; ++q) {
        int th = 4 - q;  // corner q uses offsets sc >= 3, 2, 1
        int oi = sc[0] >= th, oj = sc[1] >= th, ok = sc[2] >= th, ol = sc[3] >= th;
        float gq = (float)q * G4;
        if (q == 1) gq = G4;
        cx[q] = x0 - (float)oi + gq; cy[q] = y0 - (float)oj + gq;
        cz[q] = z0 - (float)ok + gq; cw[q] = w0 - (float)ol + gq;
        ci[q] = i + oi; cj[q] = j + oj; ck[q] = k + ok; cl[q] = l + ol;
    }
    cx[4] = x0 - 1.0f + 4.0f * G4; cy[4] = y0 - 1.0f + 4.0f * G4;
    cz[4] = z0 - 1.0f + 4.0f * G4; cw[4] = w0 - 1.0f + 4.0f * G4;
    ci[4] = i + 1; cj[4] = j + 1; ck[4] = k + 1; cl[4] = l + 1;
    float tt[5], t2[5], t4[5], g[5][4], n[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        tt[q] = 0.5f - cx[q] * cx[q] - cy[q] * cy[q] - cz[q] * cz[q] - cw[q] * cw[q];
        t2[q] = 0.0f; t4[q] = 0.0f; n[q] = 0.0f;
        g[q][0] = g[q][1] = g[q][2] = g[q][3] = 0.0f;
        if (tt[q] >= 0.0f) {
            t2[q] = tt[q] * tt[q];
            t4[q] = t2[q] * t2[q];
            sgrad4(ci[q], cj[q], ck[q], cl[q], seed, g[q]);
            n[q] = t4[q] * (g[q][0] * cx[q] + g[q][1] * cy[q] + g[q][2] * cz[q] + g[q][3] * cw[q]);
        }
    }
    const float scale = 54.0f;
    float noise = scale * (n[0] + n[1] + n[2] + n[3] + n[4]);
    if (dd) {
        float dx = 0.0f, dy = 0.0f, dz = 0.0f, dw = 0.0f;
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            float temp = t2[q] * tt[q] * (g[q][0] * cx[q] + g[q][1] * cy[q] + g[q][2] * cz[q] + g[q][3] * cw[q]);
            if (q == 0) { dx = temp * cx[q]; dy = temp * cy[q]; dz = temp * cz[q]; dw = temp * cw[q]; }
            else { dx += temp * cx[q]; dy += temp * cy[q]; dz += temp * cz[q]; dw += temp * cw[q]; }
        }
        dx *= -8.0f; dy *= -8.0f; dz *= -8.0f; dw *= -8.0f;
        dx += t4[0] * g[0][0] + t4[1] * g[1][0] + t4[2] * g[2][0] + t4[3] * g[3][0] + t4[4] * g[4][0];
        dy += t4[0] * g[0][1] + t4[1] * g[1][1] + t4[2] * g[2][1] + t4[3] * g[3][1] + t4[4] * g[4][1];
        dz += t4[0] * g[0][2] + t4[1] * g[1][2] + t4[2] * g[2][2] + t4[3] * g[3][2] + t4[4] * g[4][2];
        dw += t4[0] * g[0][3] + t4[1] * g[1][3] + t4[2] * g[2][3] + t4[3] * g[3][3] + t4[4] * g[4][3];
        dd[0] = dx * scale; dd[1] = dy * scale; dd[2] = dz * scale; dd[3] = dw * scale;
    }
    return noise;
}

}  // namespace dev
}  // namespace oslg
