// ORACLE — test infrastructure only. Not part of the shipped library.
//
// CPU restatement of OSL's Perlin / cell / hash noise in the reference's
// scalar ("CGScalar", full-batch) operation order:
//   src/include/OSL/oslnoise.h  hashes :135-329, cell/hash noise :337-480,
//   periodic adapter :486-550, floorfrac/fade/grad/scale :847-1041,
//   hashers :1044-1310, perlin non-SIMD branches :1327-2280,
//   Noise/SNoise/PeriodicNoise/PeriodicSNoise wrappers :2284-2762.
//
// Third-party arithmetic the reference calls but does not vendor
// (OpenImageIO >= 3.0, no lockfile pin; the algorithms below are restated
// from OIIO's published headers):
//   * bjhash::bjmix / bjfinal: Bob Jenkins' lookup3 mix and final mix.
//     The reference states the same rotation schedule in-tree for its SIMD
//     form (oslnoise.h:154-180).
//   * ifloor(x) = (int)floorf(x). Out-of-range and NaN inputs are defined
//     here as saturating (NaN -> 0), which is what CUDA's cvt.rzi and
//     AArch64's fcvtzs do; x86's cvttss2si returns INT_MIN instead.
//   * lerp(a,b,t) = a*(1-t) + b*t;
//     bilerp = (1-t)*(v0*s1 + v1*s) + t*(v2*s1 + v3*s), s1 = 1-s;
//     trilerp = r1*(t1*(v0*s1+v1*s) + t*(v2*s1+v3*s))
//             + r *(t1*(v4*s1+v5*s) + t*(v6*s1+v7*s)).
#pragma once
#include "oracle_dual.h"
#include <climits>

namespace oracle {

inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

inline void bjmix(uint32_t& a, uint32_t& b, uint32_t& c) {
    a -= c; a ^= rotl32(c, 4);  c += b;
    b -= a; b ^= rotl32(a, 6);  a += c;
    c -= b; c ^= rotl32(b, 8);  b += a;
    a -= c; a ^= rotl32(c, 16); c += b;
    b -= a; b ^= rotl32(a, 19); a += c;
    c -= b; c ^= rotl32(b, 4);  b += a;
}

inline uint32_t bjfinal(uint32_t a, uint32_t b, uint32_t c) {
    c ^= b; c -= rotl32(b, 14);
    a ^= c; a -= rotl32(c, 11);
    b ^= a; b -= rotl32(a, 25);
    c ^= b; c -= rotl32(b, 16);
    a ^= c; a -= rotl32(c, 4);
    b ^= a; b -= rotl32(a, 14);
    c ^= b; c -= rotl32(b, 24);
    return c;
}

// oslnoise.h:135-141
inline float bits_to_01(uint32_t bits) {
    const float k = (float)(1.0 / 4294967295.0);
    return (float)bits * k;
}

// oslnoise.h:224-289 hand-unrolled lookup3 for 1..5 keys
inline uint32_t inthash(uint32_t k0) {
    uint32_t s = 0xdeadbeefu + (1u << 2) + 13u;
    return bjfinal(s + k0, s, s);
}
inline uint32_t inthash(uint32_t k0, uint32_t k1) {
    uint32_t s = 0xdeadbeefu + (2u << 2) + 13u;
    return bjfinal(s + k0, s + k1, s);
}
inline uint32_t inthash(uint32_t k0, uint32_t k1, uint32_t k2) {
    uint32_t s = 0xdeadbeefu + (3u << 2) + 13u;
    return bjfinal(s + k0, s + k1, s + k2);
}
inline uint32_t inthash(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3) {
    uint32_t s = 0xdeadbeefu + (4u << 2) + 13u;
    uint32_t a = s + k0, b = s + k1, c = s + k2;
    bjmix(a, b, c);
    a += k3;
    return bjfinal(a, b, c);
}
inline uint32_t inthash(uint32_t k0, uint32_t k1, uint32_t k2, uint32_t k3, uint32_t k4) {
    uint32_t s = 0xdeadbeefu + (5u << 2) + 13u;
    uint32_t a = s + k0, b = s + k1, c = s + k2;
    bjmix(a, b, c);
    b += k4;
    a += k3;
    return bjfinal(a, b, c);
}

inline int ifloor(float x) {
    float f = std::floor(x);
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

// ---- cell / hash noise (oslnoise.h:337-480) --------------------------------
// Both hash their (transformed) inputs with inthash; the Vec3 results append
// a 0/1/2 key (oslnoise.h:410-414). CellNoise keys are ifloor(x)
// (:462-470); HashNoise keys are the float bit patterns (:472-480).
struct CellKey { static uint32_t k(float v) { return (uint32_t)ifloor(v); } };
struct HashKey { static uint32_t k(float v) { return fbits(v); } };

template <class K> inline float intnoise1(float x) { return bits_to_01(inthash(K::k(x))); }
template <class K> inline float intnoise2(float x, float y) { return bits_to_01(inthash(K::k(x), K::k(y))); }
template <class K> inline float intnoise3(float x, float y, float z) {
    return bits_to_01(inthash(K::k(x), K::k(y), K::k(z)));
}
template <class K> inline float intnoise4(float x, float y, float z, float w) {
    return bits_to_01(inthash(K::k(x), K::k(y), K::k(z), K::k(w)));
}
template <class K> inline V3 vintnoise1(float x) {
    uint32_t a = K::k(x);
    return V3(bits_to_01(inthash(a, 0u)), bits_to_01(inthash(a, 1u)), bits_to_01(inthash(a, 2u)));
}
template <class K> inline V3 vintnoise2(float x, float y) {
    uint32_t a = K::k(x), b = K::k(y);
    return V3(bits_to_01(inthash(a, b, 0u)), bits_to_01(inthash(a, b, 1u)), bits_to_01(inthash(a, b, 2u)));
}
// oslnoise.h:416-435 (three keys + channel: shares the bjmix)
template <class K> inline V3 vintnoise3(float x, float y, float z) {
    uint32_t k0 = K::k(x), k1 = K::k(y), k2 = K::k(z);
    return V3(bits_to_01(inthash(k0, k1, k2, 0u)), bits_to_01(inthash(k0, k1, k2, 1u)),
              bits_to_01(inthash(k0, k1, k2, 2u)));
}
// oslnoise.h:437-457
template <class K> inline V3 vintnoise4(float x, float y, float z, float w) {
    uint32_t k0 = K::k(x), k1 = K::k(y), k2 = K::k(z), k3 = K::k(w);
    return V3(bits_to_01(inthash(k0, k1, k2, k3, 0u)), bits_to_01(inthash(k0, k1, k2, k3, 1u)),
              bits_to_01(inthash(k0, k1, k2, k3, 2u)));
}

// Periodic wrap (oslnoise.h:532-540)
inline float pwrap(float s, float period) {
    period = std::floor(period);
    if (period < 1.0f) period = 1.0f;
    return s - period * std::floor(s / period);
}

// inthashi / inthashf (oslnoise.h:555-605): the `hash` shadeop
inline int hash_i(int x) { return (int)inthash((uint32_t)x); }
inline int hash_f(float x) { return (int)inthash(fbits(x)); }
inline int hash_ff(float x, float y) { return (int)inthash(fbits(x), fbits(y)); }
inline int hash_v(const V3& p) { return (int)inthash(fbits(p.x), fbits(p.y), fbits(p.z)); }
inline int hash_vf(const V3& p, float t) {
    return (int)inthash(fbits(p.x), fbits(p.y), fbits(p.z), fbits(t));
}

// ---- Perlin helpers ---------------------------------------------------------
// imod (oslnoise.h:847-859)
inline int imod(int a, int b) {
    int r = a % b;
    if (r < 0) r += b;
    return r;
}
// floorfrac (oslnoise.h:872-882): the slope passes through unchanged
inline float floorfrac(float x, int* i) { *i = ifloor(x); return x - (float)*i; }
inline DF floorfrac(const DF& x, int* i) { float f = floorfrac(x.v, i); return DF(f, x.dx, x.dy); }

// fade (oslnoise.h:909-912): t*t*t*(t*(t*6-15)+10), with T(6) etc. promoted
// to T (so a Dual2 multiplies by a dual constant whose partials are zero).
inline float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
inline DF fade(const DF& t) {
    DF six(6.0f), fifteen(15.0f), ten(10.0f);
    return t * t * t * (t * (t * six - fifteen) + ten);
}

// OIIO-style negate_if / select on float and Dual2 (oslnoise.h:611-760)
inline float negate_if(float v, bool c) { return c ? -v : v; }
inline DF negate_if(const DF& v, bool c) { return c ? DF(-v.v, -v.dx, -v.dy) : v; }

// grad (oslnoise.h:926-990). 1D: g*x with g in +-1..8.
inline float grad(int hash, float x) {
    int h = hash & 15;
    float g = 1 + (h & 7);
    if (h & 8) g = -g;
    return g * x;
}
inline DF grad(int hash, const DF& x) {
    int h = hash & 15;
    float g = 1 + (h & 7);
    if (h & 8) g = -g;
    return g * x;
}
template <class T> inline T grad(int hash, const T& x, const T& y) {
    int h = hash & 7;
    T u = h < 4 ? x : y;
    T v = 2.0f * (h < 4 ? y : x);
    return negate_if(u, h & 1) + negate_if(v, h & 2);
}
template <class T> inline T grad(int hash, const T& x, const T& y, const T& z) {
    int h = hash & 15;
    T u = h < 8 ? x : y;
    T v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
    return negate_if(u, h & 1) + negate_if(v, h & 2);
}
template <class T> inline T grad(int hash, const T& x, const T& y, const T& z, const T& w) {
    int h = hash & 31;
    T u = h < 24 ? x : y;
    T v = h < 16 ? y : z;
    T s = h < 8 ? z : w;
    return negate_if(u, h & 1) + negate_if(v, h & 2) + negate_if(s, h & 4);
}

// OIIO lerp / bilerp / trilerp (see file header)
inline float one_minus(float t) { return 1.0f - t; }
inline DF one_minus(const DF& t) { return DF(1.0f) - t; }
template <class T, class Q> inline T lerp(const T& a, const T& b, const Q& t) {
    return a * one_minus(t) + b * t;
}
template <class T, class Q>
inline T bilerp(const T& v0, const T& v1, const T& v2, const T& v3, const Q& s, const Q& t) {
    Q s1 = one_minus(s);
    return one_minus(t) * (v0 * s1 + v1 * s) + t * (v2 * s1 + v3 * s);
}
template <class T, class Q>
inline T trilerp(const T& v0, const T& v1, const T& v2, const T& v3, const T& v4, const T& v5,
                 const T& v6, const T& v7, const Q& s, const Q& t, const Q& r) {
    Q s1 = one_minus(s);
    Q t1 = one_minus(t);
    Q r1 = one_minus(r);
    return r1 * (t1 * (v0 * s1 + v1 * s) + t * (v2 * s1 + v3 * s))
         + r * (t1 * (v4 * s1 + v5 * s) + t * (v6 * s1 + v7 * s));
}

// scale1..4 (oslnoise.h:1034-1041)
template <class T> inline T scale1(const T& r) { return 0.2500f * r; }
template <class T> inline T scale2(const T& r) { return 0.6616f * r; }
template <class T> inline T scale3(const T& r) { return 0.9820f * r; }
template <class T> inline T scale4(const T& r) { return 0.8344f * r; }

// Lattice hashers. HashScalar (oslnoise.h:1044-1093) returns the 32-bit
// hash; HashVector (:1105-1128) slices it into three bytes, one per output
// channel (sliceup, :1096-1103), so channel c of a vector noise is the
// scalar noise with gradient selector (h >> 8c) & 0xFF. The periodic
// hashers (:1157-1310) wrap each lattice coordinate with imod first.
struct Hasher {
    bool periodic = false;
    int px = 1, py = 1, pz = 1, pw = 1;
    static int per(float p) { int i = ifloor(p); return i < 1 ? 1 : i; }
    int wx(int x) const { return periodic ? imod(x, px) : x; }
    int wy(int y) const { return periodic ? imod(y, py) : y; }
    int wz(int z) const { return periodic ? imod(z, pz) : z; }
    int ww(int w) const { return periodic ? imod(w, pw) : w; }
    int operator()(int x) const { return (int)inthash((uint32_t)wx(x)); }
    int operator()(int x, int y) const { return (int)inthash((uint32_t)wx(x), (uint32_t)wy(y)); }
    int operator()(int x, int y, int z) const {
        return (int)inthash((uint32_t)wx(x), (uint32_t)wy(y), (uint32_t)wz(z));
    }
    int operator()(int x, int y, int z, int w) const {
        return (int)inthash((uint32_t)wx(x), (uint32_t)wy(y), (uint32_t)wz(z), (uint32_t)ww(w));
    }
};

inline int chan(int h, int c) { return c == 0 ? h : ((h >> (8 * c)) & 0xFF); }

// perlin, CGScalar branches (oslnoise.h:1327-1335 1D, :1364-1377 2D,
// :1420-1438 3D, :1489-1520 4D and the Dual2 / Vec3 twins at :1600-1616,
// :1680-1700, :1707-1740, :1780-1795, :1920-1985, :2000-2033, :2083-2096,
// :2157-2171, :2245-2277). T is float or Dual2<float>; `c` picks the output
// channel of a vector noise (0 for float noise).
template <class T> inline T perlin1(const Hasher& hash, int c, const T& x) {
    int X; T fx = floorfrac(x, &X);
    T u = fade(fx);
    T r = lerp(grad(chan(hash(X), c), fx), grad(chan(hash(X + 1), c), fx - 1.0f), u);
    return scale1(r);
}
template <class T> inline T perlin2(const Hasher& hash, int c, const T& x, const T& y) {
    int X; T fx = floorfrac(x, &X);
    int Y; T fy = floorfrac(y, &Y);
    T u = fade(fx), v = fade(fy);
    T r = bilerp(grad(chan(hash(X, Y), c), fx, fy),
                 grad(chan(hash(X + 1, Y), c), fx - 1.0f, fy),
                 grad(chan(hash(X, Y + 1), c), fx, fy - 1.0f),
                 grad(chan(hash(X + 1, Y + 1), c), fx - 1.0f, fy - 1.0f), u, v);
    return scale2(r);
}
template <class T> inline T perlin3(const Hasher& hash, int c, const T& x, const T& y, const T& z) {
    int X; T fx = floorfrac(x, &X);
    int Y; T fy = floorfrac(y, &Y);
    int Z; T fz = floorfrac(z, &Z);
    T u = fade(fx), v = fade(fy), w = fade(fz);
    T r = trilerp(grad(chan(hash(X, Y, Z), c), fx, fy, fz),
                  grad(chan(hash(X + 1, Y, Z), c), fx - 1.0f, fy, fz),
                  grad(chan(hash(X, Y + 1, Z), c), fx, fy - 1.0f, fz),
                  grad(chan(hash(X + 1, Y + 1, Z), c), fx - 1.0f, fy - 1.0f, fz),
                  grad(chan(hash(X, Y, Z + 1), c), fx, fy, fz - 1.0f),
                  grad(chan(hash(X + 1, Y, Z + 1), c), fx - 1.0f, fy, fz - 1.0f),
                  grad(chan(hash(X, Y + 1, Z + 1), c), fx, fy - 1.0f, fz - 1.0f),
                  grad(chan(hash(X + 1, Y + 1, Z + 1), c), fx - 1.0f, fy - 1.0f, fz - 1.0f), u, v, w);
    return scale3(r);
}
template <class T>
inline T perlin4(const Hasher& hash, int c, const T& x, const T& y, const T& z, const T& w) {
    int X; T fx = floorfrac(x, &X);
    int Y; T fy = floorfrac(y, &Y);
    int Z; T fz = floorfrac(z, &Z);
    int W; T fw = floorfrac(w, &W);
    T u = fade(fx), v = fade(fy), t = fade(fz), s = fade(fw);
    T a = trilerp(grad(chan(hash(X, Y, Z, W), c), fx, fy, fz, fw),
                  grad(chan(hash(X + 1, Y, Z, W), c), fx - 1.0f, fy, fz, fw),
                  grad(chan(hash(X, Y + 1, Z, W), c), fx, fy - 1.0f, fz, fw),
                  grad(chan(hash(X + 1, Y + 1, Z, W), c), fx - 1.0f, fy - 1.0f, fz, fw),
                  grad(chan(hash(X, Y, Z + 1, W), c), fx, fy, fz - 1.0f, fw),
                  grad(chan(hash(X + 1, Y, Z + 1, W), c), fx - 1.0f, fy, fz - 1.0f, fw),
                  grad(chan(hash(X, Y + 1, Z + 1, W), c), fx, fy - 1.0f, fz - 1.0f, fw),
                  grad(chan(hash(X + 1, Y + 1, Z + 1, W), c), fx - 1.0f, fy - 1.0f, fz - 1.0f, fw),
                  u, v, t);
    T b = trilerp(grad(chan(hash(X, Y, Z, W + 1), c), fx, fy, fz, fw - 1.0f),
                  grad(chan(hash(X + 1, Y, Z, W + 1), c), fx - 1.0f, fy, fz, fw - 1.0f),
                  grad(chan(hash(X, Y + 1, Z, W + 1), c), fx, fy - 1.0f, fz, fw - 1.0f),
                  grad(chan(hash(X + 1, Y + 1, Z, W + 1), c), fx - 1.0f, fy - 1.0f, fz, fw - 1.0f),
                  grad(chan(hash(X, Y, Z + 1, W + 1), c), fx, fy, fz - 1.0f, fw - 1.0f),
                  grad(chan(hash(X + 1, Y, Z + 1, W + 1), c), fx - 1.0f, fy, fz - 1.0f, fw - 1.0f),
                  grad(chan(hash(X, Y + 1, Z + 1, W + 1), c), fx, fy - 1.0f, fz - 1.0f, fw - 1.0f),
                  grad(chan(hash(X + 1, Y + 1, Z + 1, W + 1), c), fx - 1.0f, fy - 1.0f, fz - 1.0f, fw - 1.0f),
                  u, v, t);
    return scale4(lerp(a, b, s));
}

// Dimension dispatch over up to 4 coordinates.
template <class T> inline T perlin_n(const Hasher& h, int c, int dim, const T* xs) {
    switch (dim) {
    case 1: return perlin1(h, c, xs[0]);
    case 2: return perlin2(h, c, xs[0], xs[1]);
    case 3: return perlin3(h, c, xs[0], xs[1], xs[2]);
    default: return perlin4(h, c, xs[0], xs[1], xs[2], xs[3]);
    }
}

// Unsigned wrapper (NoiseImpl, oslnoise.h:2284-2414): 0.5*(r+1), with the
// Dual2<Vec3> form written Vec3(0.5)*(r+Vec3(1)), which is the same
// per-channel arithmetic.
inline float unsigned_of(float r) { return 0.5f * (r + 1.0f); }
inline DF unsigned_of(const DF& r) { return 0.5f * (r + 1.0f); }

}  // namespace oracle
