// sm_103a interpreter for lowered OSL shader groups (device code). Included
// by the tier translation units (oslg_tier.cu), each of which instantiates
// interp_kernel<heap_in_smem, TIER> for one feature tier.
//
// One thread shades one point. All lanes of a warp walk the same op index
// (the program counter is warp-uniform), so the big dispatch switch never
// diverges; varying control flow is carried by a per-lane `act` flag and
// per-depth bit stacks, the same masked-SIMD model the reference's batched
// backend uses (src/liboslexec/batched_llvm_gen.cpp:1068 if, :3806-4250
// loops, break/continue), with __any_sync skipping blocks no lane enters.
//
// Memory: the op stream and the constant pool are staged once per CTA in
// shared memory (warp-uniform broadcast reads). Per-point symbol values
// live in a slot-major heap, either in shared memory (heap_smem=1) or in a
// per-CTA slice of an HBM scratch buffer sized to the resident grid, which
// stays L2-resident (heap_smem=0). Grid-stride tiles keep the grid at the
// resident CTA count.
//
// Built with -fmad=false: every float result equals the non-FMA reference
// arithmetic bit for bit (see oslg_noise.cuh).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <mutex>
#include <string>

#include "oslg_exec.h"
#include "oslg_fastmath.cuh"
#include "oslg_gabor.cuh"
#include "oslg_noise.cuh"
#include "oslg_shading.cuh"

namespace oslg {
namespace dev {


// blackbody / closure helpers live further down
static const unsigned FULL = 0xFFFFFFFFu;

// Capacities of the closure walk stack and of the BSDF lobe list. A
// specialized kernel whose program has no loops defines smaller bounds that
// its closure ops cannot exceed (walk depth <= ADD ops, lobes <= 2^ADD ops),
// and indexes these arrays with compile-time indices (OSLG_FIXED_INDEX) so
// that they stay in registers; results are the same as with the defaults.
// Component loops whose trip count is a per-op constant: a specialized
// kernel unrolls them so that symbol indices are compile-time constants
// (its symbol array then stays in registers).
#ifdef OSLG_SPEC
#define OSLG_SPEC_UNROLL _Pragma("unroll")
#else
#define OSLG_SPEC_UNROLL
#endif
#ifndef OSLG_WALK_STACK
#define OSLG_WALK_STACK kClosureWalkStack
#endif
#ifndef OSLG_LOBES_MAX
#define OSLG_LOBES_MAX kBsdfMaxLobes
#endif

// KArgs: see oslg_exec.h

struct Lane {
    float* heap;
    const uint32_t* pool;
    int hs;      // heap stride (points per CTA tile)
    int li;      // lane index within the tile
    int64_t pt;  // global point index
    const int32_t* si = nullptr;  // arena record of each point (null: the point index)
#ifdef OSLG_SPEC
    // A specialized kernel keeps symbol slots in a thread-local array (hs 1,
    // li 0, constant offsets: registers) and the closure node pools, which
    // are indexed at run time, in a separate slot-major heap.
    float* cheap;
    int chs, cli;
    uint32_t cbase;
#endif
};

// Output-arena stores. A specialized kernel that stages a tile's output
// records in shared memory (OSLG_STAGE_STRIDE = record bytes) marks each
// written word, so that only written words are copied out.
#ifdef OSLG_STAGE_STRIDE
extern __shared__ __align__(16) unsigned char oslg_smem[];
__device__ __forceinline__ void ostore32(void* p, uint32_t w) {
    *reinterpret_cast<uint32_t*>(p) = w;
    const size_t word = (size_t)(reinterpret_cast<unsigned char*>(p) - oslg_smem) >> 2;
    oslg_smem[(size_t)blockDim.x * OSLG_STAGE_STRIDE + word] = 1;
}
#else
__device__ __forceinline__ void ostore32(void* p, uint32_t w) { *reinterpret_cast<uint32_t*>(p) = w; }
#endif
__device__ __forceinline__ void ostoref(void* p, float v) { ostore32(p, __float_as_uint(v)); }

// The point's record in the userdata and output arenas: the caller's
// shadeindex when given (base + shadeindex * stride, as
// batched_llvm_instance.cpp:1219-1229 addresses them), else the point. A
// kernel that stages its output records in shared memory writes them by
// point and scatters them by shadeindex when it copies the tile out.
__device__ __forceinline__ int64_t urec(const Lane& L) { return L.si ? (int64_t)__ldg(L.si + L.pt) : L.pt; }
#ifdef OSLG_STAGE_STRIDE
__device__ __forceinline__ int64_t orec(const Lane& L) { return L.pt; }
#else
__device__ __forceinline__ int64_t orec(const Lane& L) { return urec(L); }
#endif

__device__ __forceinline__ uint32_t aoff(uint32_t a) { return a & kArgOffsetMask; }
__device__ __forceinline__ bool aconst(uint32_t a) { return (a & kArgConst) != 0; }
__device__ __forceinline__ bool ader(uint32_t a) { return (a & kArgDerivs) != 0; }
__device__ __forceinline__ uint32_t atc(uint32_t a) { return (a >> kArgTCShift) & 7u; }
__device__ __forceinline__ int anc(uint32_t a) {
    uint32_t t = atc(a);
    return t == TC_TRIPLE ? 3 : (t == TC_MATRIX ? 16 : 1);
}

__device__ __forceinline__ uint32_t ldw(const Lane& L, uint32_t a, int idx) {
    uint32_t o = aoff(a) + (uint32_t)idx;
    if (aconst(a)) return L.pool[o];
    return __float_as_uint(L.heap[(size_t)o * L.hs + L.li]);
}
__device__ __forceinline__ void stw(const Lane& L, uint32_t a, int idx, uint32_t v) {
    L.heap[(size_t)(aoff(a) + (uint32_t)idx) * L.hs + L.li] = __uint_as_float(v);
}
__device__ __forceinline__ void stf(const Lane& L, uint32_t a, int idx, float v) { stw(L, a, idx, __float_as_uint(v)); }

// value (d=0) or x/y partial (d=1,2) of component c; scalars broadcast,
// ints convert, missing partials read as zero
__device__ __forceinline__ float ldf(const Lane& L, uint32_t a, int c, int d) {
    int nc = anc(a);
    if (d && !ader(a)) return 0.0f;
    uint32_t w = ldw(L, a, d * nc + (nc == 1 ? 0 : c));
    return atc(a) == TC_INT ? (float)(int)w : __uint_as_float(w);
}
__device__ __forceinline__ D2 ldd(const Lane& L, uint32_t a, int c) {
    return d2(ldf(L, a, c, 0), ldf(L, a, c, 1), ldf(L, a, c, 2));
}
__device__ __forceinline__ int ldi(const Lane& L, uint32_t a, int c) {
    uint32_t t = atc(a);
    uint32_t w = ldw(L, a, t == TC_TRIPLE ? c : 0);
    if (t == TC_FLOAT || t == TC_TRIPLE) return (int)__uint_as_float(w);
    return (int)w;
}
// store a Dual2 into component c of r (partials only if r carries them)
__device__ __forceinline__ void std2(const Lane& L, uint32_t r, int c, D2 v) {
    int nc = anc(r);
    if (atc(r) == TC_INT) { stw(L, r, c, (uint32_t)(int)v.v); return; }
    stf(L, r, c, v.v);
    if (ader(r)) {
        stf(L, r, nc + c, v.dx);
        stf(L, r, 2 * nc + c, v.dy);
    }
}
__device__ __forceinline__ void stval(const Lane& L, uint32_t r, int c, float v) {
    if (atc(r) == TC_INT) { stw(L, r, c, (uint32_t)(int)v); return; }
    int nc = anc(r);
    stf(L, r, c, v);
    if (ader(r)) {
        stf(L, r, nc + c, 0.0f);
        stf(L, r, 2 * nc + c, 0.0f);
    }
}
__device__ __forceinline__ void raise_status(uint32_t* st, uint32_t bit) { atomicOr(st, bit); }

// ---- math helpers (values through double precision: correctly rounded
// float results, identical on every platform that rounds double libm
// results correctly to float) --------------------------------------------------
__device__ __forceinline__ float fsin(float x) { return (float)sin((double)x); }
__device__ __forceinline__ float fcos(float x) { return (float)cos((double)x); }
__device__ __forceinline__ float ftan(float x) { return (float)tan((double)x); }
__device__ __forceinline__ float fasin(float x) { return (float)asin((double)x); }
__device__ __forceinline__ float facos(float x) { return (float)acos((double)x); }
__device__ __forceinline__ float fatan(float x) { return (float)atan((double)x); }
__device__ __forceinline__ float fatan2(float y, float x) { return (float)atan2((double)y, (double)x); }
__device__ __forceinline__ float fsinh(float x) { return (float)sinh((double)x); }
__device__ __forceinline__ float fcosh(float x) { return (float)cosh((double)x); }
__device__ __forceinline__ float ftanh(float x) { return (float)tanh((double)x); }
__device__ __forceinline__ float fexp(float x) { return (float)exp((double)x); }
__device__ __forceinline__ float fexp2(float x) { return (float)exp2((double)x); }
__device__ __forceinline__ float fexpm1(float x) { return (float)expm1((double)x); }
__device__ __forceinline__ float fcbrt(float x) { return (float)cbrt((double)x); }
__device__ __forceinline__ float flog_raw(float x) { return (float)log((double)x); }
__device__ __forceinline__ float flog2_raw(float x) { return (float)log2((double)x); }
__device__ __forceinline__ float flog10_raw(float x) { return (float)log10((double)x); }
__device__ __forceinline__ float fpow_raw(float x, float y) { return (float)pow((double)x, (double)y); }
static const float kFltMin = 1.17549435e-38f;
static const float kFltMax = 3.40282347e+38f;
// logb as OpenImageIO's fast_logb (fmath.h, the host path the reference's
// logb op calls, llvm_ops.cpp:542-545): the unbiased exponent of |x|
// clamped to the normal range, so 0 gives -126 and infinity 127
__device__ __forceinline__ float logb_fast(float x) {
    x = fabsf(x);
    if (x < kFltMin) x = kFltMin;
    if (x > kFltMax) x = kFltMax;
    return (float)((int)(__float_as_uint(x) >> 23) - 127);
}
// OIIO safe_log/log2/log10: clamp the argument to the smallest normal
__device__ __forceinline__ float safe_log(float x) { return flog_raw(x < kFltMin ? kFltMin : x); }
__device__ __forceinline__ float safe_log2(float x) { return flog2_raw(x < kFltMin ? kFltMin : x); }
__device__ __forceinline__ float safe_log10(float x) { return flog10_raw(x < kFltMin ? kFltMin : x); }
// OIIO safe_pow: integer powers only for negative bases; no infinities
__device__ __forceinline__ float safe_pow(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return 0.0f;
    if (x < 0.0f && y != floorf(y)) return 0.0f;
    float r = fpow_raw(x, y);
    return fminf(fmaxf(r, -kFltMax), kFltMax);
}
__device__ __forceinline__ float safe_fmod(float a, float b) {
    if (b != 0.0f) {
        int N = (int)(a / b);
        return a - (float)N * b;
    }
    return 0.0f;
}

// ---- handlers -------------------------------------------------------------------
static __device__ void h_assign(const Lane& L, const uint32_t* a, uint32_t* st) {
    uint32_t r = a[0], s = a[1];
    uint32_t tr = atc(r), ts = atc(s);
    int count = (int)a[2];
    if (tr == TC_CLOSURE) {
        stw(L, r, 0, ts == TC_CLOSURE ? ldw(L, s, 0) : 0u);
        return;
    }
    if (tr == TC_STRING) { stw(L, r, 0, ldw(L, s, 0)); return; }
    if (tr == TC_MATRIX) {
        if (ts == TC_MATRIX) {
            for (int i = 0; i < 16; ++i) stw(L, r, i, ldw(L, s, i));
        } else {
            float v = ldf(L, s, 0, 0);
            for (int i = 0; i < 16; ++i) stf(L, r, i, (i % 5 == 0) ? v : 0.0f);
        }
        return;
    }
    int ralen = (int)a[3], salen = (int)a[4];
    if (ralen < 1) ralen = 1;
    if (salen < 1) salen = 1;
    int nr = anc(r), ns = anc(s);
    OSLG_SPEC_UNROLL
    for (int e = 0; e < count; ++e) {
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nr; ++c) {
            int sc = ns == 1 ? 0 : c;
            uint32_t sw = ldw(L, s, e * ns + sc);
            if (tr == TC_INT) {
                int iv = ts == TC_INT ? (int)sw : (int)__uint_as_float(sw);
                stw(L, r, e * nr + c, (uint32_t)iv);
                continue;
            }
            float v = ts == TC_INT ? (float)(int)sw : __uint_as_float(sw);
            stf(L, r, e * nr + c, v);
            if (ader(r)) {
                float dx = 0.0f, dy = 0.0f;
                if (ader(s)) {
                    dx = __uint_as_float(ldw(L, s, salen * ns + e * ns + sc));
                    dy = __uint_as_float(ldw(L, s, 2 * salen * ns + e * ns + sc));
                }
                stf(L, r, ralen * nr + e * nr + c, dx);
                stf(L, r, 2 * ralen * nr + e * nr + c, dy);
            }
        }
    }
}

// ---- decoded operands ------------------------------------------------------------------
// A float-based operand decoded once per op: component c, partial d (1 = x,
// 2 = y) lives at p[c*cs + d*ds]; scalars broadcast (cs = 0); operands
// without partials read zero partials.
struct Opd {
    float* p;
    int cs, ds;
    bool hasd;
};
__device__ __forceinline__ Opd dec(const Lane& L, uint32_t a) {
    Opd o;
    int nc = anc(a);
    int unit;
    if (aconst(a)) {
        o.p = const_cast<float*>(reinterpret_cast<const float*>(L.pool)) + aoff(a);
        unit = 1;
    } else {
        o.p = L.heap + (size_t)aoff(a) * L.hs + L.li;
        unit = L.hs;
    }
    o.cs = nc == 1 ? 0 : unit;
    o.ds = nc * unit;
    o.hasd = ader(a);
    return o;
}
__device__ __forceinline__ float gv(const Opd& o, int c) { return o.p[c * o.cs]; }
__device__ __forceinline__ float gd(const Opd& o, int c, int d) { return o.hasd ? o.p[c * o.cs + d * o.ds] : 0.0f; }
__device__ __forceinline__ void sv(const Opd& o, int c, float v) { o.p[c * o.cs] = v; }
__device__ __forceinline__ void sd(const Opd& o, int c, int d, float v) { o.p[c * o.cs + d * o.ds] = v; }
__device__ __forceinline__ bool no_ints(uint32_t a, uint32_t b, uint32_t c) {
    return atc(a) != TC_INT && atc(b) != TC_INT && atc(c) != TC_INT;
}

// add/sub/mul/div over NC components of float-based operands (same Dual2
// rules as h_arith below, with the operand decode hoisted out of the loop)
template <int K, int NC>
__device__ __forceinline__ void arith_fast_n(const Opd& R, const Opd& X, const Opd& Y, bool rd) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        float xv = gv(X, c), yv = gv(Y, c);
        float v;
        if (K == 0) v = xv + yv;
        else if (K == 1) v = xv - yv;
        else if (K == 2) v = xv * yv;
        else v = (yv == 0.0f) ? 0.0f : xv / yv;
        sv(R, c, v);
        if (!rd) continue;
        float dx, dy;
        if (K == 0 || K == 1) {
            if (X.hasd && Y.hasd) {
                float xdx = gd(X, c, 1), xdy = gd(X, c, 2), ydx = gd(Y, c, 1), ydy = gd(Y, c, 2);
                dx = K == 0 ? xdx + ydx : xdx - ydx;
                dy = K == 0 ? xdy + ydy : xdy - ydy;
            } else if (X.hasd) {
                dx = gd(X, c, 1); dy = gd(X, c, 2);
            } else if (Y.hasd) {
                dx = K == 0 ? gd(Y, c, 1) : -gd(Y, c, 1);
                dy = K == 0 ? gd(Y, c, 2) : -gd(Y, c, 2);
            } else { dx = 0.0f; dy = 0.0f; }
        } else if (K == 2) {
            if (X.hasd && Y.hasd) {
                dx = xv * gd(Y, c, 1) + gd(X, c, 1) * yv;
                dy = xv * gd(Y, c, 2) + gd(X, c, 2) * yv;
            } else if (X.hasd) {
                dx = gd(X, c, 1) * yv; dy = gd(X, c, 2) * yv;
            } else if (Y.hasd) {
                dx = gd(Y, c, 1) * xv; dy = gd(Y, c, 2) * xv;
            } else { dx = 0.0f; dy = 0.0f; }
        } else {
            if (yv == 0.0f) { dx = 0.0f; dy = 0.0f; }
            else {
                float binv = 1.0f / yv, q = xv / yv;
                if (X.hasd && Y.hasd) {
                    dx = binv * (gd(X, c, 1) - q * gd(Y, c, 1));
                    dy = binv * (gd(X, c, 2) - q * gd(Y, c, 2));
                } else if (X.hasd) {
                    dx = binv * gd(X, c, 1); dy = binv * gd(X, c, 2);
                } else if (Y.hasd) {
                    dx = binv * (-q * gd(Y, c, 1)); dy = binv * (-q * gd(Y, c, 2));
                } else { dx = 0.0f; dy = 0.0f; }
            }
        }
        sd(R, c, 1, dx);
        sd(R, c, 2, dy);
    }
}

template <int K>
static __device__ void h_arith(const Lane& L, const uint32_t* a);

template <int K>
__device__ __forceinline__ void h_arith_fast(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], x = a[1], y = a[2];
    if (!no_ints(r, x, y)) { h_arith<K>(L, a); return; }
    Opd R = dec(L, r), X = dec(L, x), Y = dec(L, y);
    bool rd = ader(r);
    int nc = anc(r);
    if (nc == 3) arith_fast_n<K, 3>(R, X, Y, rd);
    else if (nc == 1) arith_fast_n<K, 1>(R, X, Y, rd);
    else h_arith<K>(L, a);
}

// assign of a non-array float-based value (broadcasting scalars)
static __device__ void h_assign(const Lane& L, const uint32_t* a, uint32_t* st);
__device__ __forceinline__ void h_assign_fast(const Lane& L, const uint32_t* a, uint32_t* st) {
    uint32_t r = a[0], s = a[1];
    uint32_t tr = atc(r), ts = atc(s);
    if ((tr != TC_FLOAT && tr != TC_TRIPLE) || (ts != TC_FLOAT && ts != TC_TRIPLE) || a[3] > 1u || a[4] > 1u) {
        h_assign(L, a, st);
        return;
    }
    Opd R = dec(L, r), S = dec(L, s);
    int nc = anc(r);
    bool rd = ader(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        sv(R, c, gv(S, c));
        if (rd) { sd(R, c, 1, gd(S, c, 1)); sd(R, c, 2, gd(S, c, 2)); }
    }
}

// add/sub/mul/div/mod on float-based values, componentwise with scalar
// broadcast; derivatives follow src/include/OSL/dual.h:403-620
template <int K>
static __device__ void h_arith(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], x = a[1], y = a[2];
    int nc = anc(r);
    bool rd = ader(r), xd = ader(x), yd = ader(y);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        float xv = ldf(L, x, c, 0), yv = ldf(L, y, c, 0);
        float v;
        if (K == 0) v = xv + yv;
        else if (K == 1) v = xv - yv;
        else if (K == 2) v = xv * yv;
        else if (K == 3) v = (yv == 0.0f) ? 0.0f : xv / yv;
        else v = (yv == 0.0f) ? 0.0f : fmodf(xv, yv);
        if (atc(r) == TC_INT) { stw(L, r, c, (uint32_t)(int)v); continue; }
        stf(L, r, c, v);
        if (!rd) continue;
        float dx, dy;
        if (K == 0 || K == 1) {
            float xdx = ldf(L, x, c, 1), xdy = ldf(L, x, c, 2), ydx = ldf(L, y, c, 1), ydy = ldf(L, y, c, 2);
            if (K == 0) { dx = xdx + ydx; dy = xdy + ydy; }
            else { dx = xdx - ydx; dy = xdy - ydy; }
            if (!yd) { dx = xdx; dy = xdy; if (K == 1 && !xd) { dx = 0.0f; dy = 0.0f; } }
            if (!xd && yd) { dx = K == 0 ? ydx : -ydx; dy = K == 0 ? ydy : -ydy; }
        } else if (K == 2) {
            if (xd && yd) {
                dx = xv * ldf(L, y, c, 1) + ldf(L, x, c, 1) * yv;
                dy = xv * ldf(L, y, c, 2) + ldf(L, x, c, 2) * yv;
            } else if (xd) {
                dx = ldf(L, x, c, 1) * yv; dy = ldf(L, x, c, 2) * yv;
            } else if (yd) {
                dx = ldf(L, y, c, 1) * xv; dy = ldf(L, y, c, 2) * xv;
            } else { dx = 0.0f; dy = 0.0f; }
        } else if (K == 3) {
            if (yv == 0.0f) { dx = 0.0f; dy = 0.0f; }
            else {
                float binv = 1.0f / yv, q = xv / yv;
                if (xd && yd) {
                    dx = binv * (ldf(L, x, c, 1) - q * ldf(L, y, c, 1));
                    dy = binv * (ldf(L, x, c, 2) - q * ldf(L, y, c, 2));
                } else if (xd) {
                    dx = binv * ldf(L, x, c, 1); dy = binv * ldf(L, x, c, 2);
                } else if (yd) {
                    dx = binv * (-q * ldf(L, y, c, 1)); dy = binv * (-q * ldf(L, y, c, 2));
                } else { dx = 0.0f; dy = 0.0f; }
            }
        } else {
            dx = ldf(L, x, c, 1); dy = ldf(L, x, c, 2);
        }
        stf(L, r, nc + c, dx);
        stf(L, r, 2 * nc + c, dy);
    }
}

template <int K>
static __device__ void h_iarith(const Lane& L, const uint32_t* a) {
    int x = ldi(L, a[1], 0), y = ldi(L, a[2], 0), v;
    if (K == 0) v = (int)((uint32_t)x + (uint32_t)y);
    else if (K == 1) v = (int)((uint32_t)x - (uint32_t)y);
    else if (K == 2) v = (int)((uint32_t)x * (uint32_t)y);
    else if (K == 3) v = (y == 0 || (x == INT_MIN && y == -1)) ? 0 : x / y;
    else v = (y == 0 || (x == INT_MIN && y == -1)) ? 0 : x % y;
    stw(L, a[0], 0, (uint32_t)v);
}

static __device__ void h_mmul(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], x = a[1], y = a[2];
    float out[16];
    if (atc(x) == TC_MATRIX && atc(y) == TC_MATRIX) {
        float A[16], B[16];
        for (int i = 0; i < 16; ++i) { A[i] = __uint_as_float(ldw(L, x, i)); B[i] = __uint_as_float(ldw(L, y, i)); }
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                out[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j]
                               + A[i * 4 + 2] * B[2 * 4 + j] + A[i * 4 + 3] * B[3 * 4 + j];
    } else {
        uint32_t m = atc(x) == TC_MATRIX ? x : y, s = atc(x) == TC_MATRIX ? y : x;
        float f = ldf(L, s, 0, 0);
        for (int i = 0; i < 16; ++i) out[i] = __uint_as_float(ldw(L, m, i)) * f;
    }
    for (int i = 0; i < 16; ++i) stf(L, r, i, out[i]);
}

// comparisons: float compare unless both operands are ints (or strings)
template <int K>
static __device__ void h_cmp(const Lane& L, const uint32_t* a) {
    uint32_t x = a[1], y = a[2];
    bool ints = (atc(x) == TC_INT || atc(x) == TC_STRING) && (atc(y) == TC_INT || atc(y) == TC_STRING);
    int n = anc(x) > anc(y) ? anc(x) : anc(y);
    bool res;
    if (ints) {
        int xi = (int)ldw(L, x, 0), yi = (int)ldw(L, y, 0);
        if (K == 0) res = xi == yi; else if (K == 1) res = xi != yi; else if (K == 2) res = xi < yi;
        else if (K == 3) res = xi > yi; else if (K == 4) res = xi <= yi; else res = xi >= yi;
    } else if (K == 0 || K == 1) {
        bool eq = true;
        OSLG_SPEC_UNROLL
        for (int c = 0; c < n; ++c) eq = eq && (ldf(L, x, c, 0) == ldf(L, y, c, 0));
        res = K == 0 ? eq : !eq;
    } else {
        float xv = ldf(L, x, 0, 0), yv = ldf(L, y, 0, 0);
        if (K == 2) res = xv < yv; else if (K == 3) res = xv > yv; else if (K == 4) res = xv <= yv; else res = xv >= yv;
    }
    stw(L, a[0], 0, res ? 1u : 0u);
}

__device__ __forceinline__ bool truth(const Lane& L, uint32_t a) {
    uint32_t t = atc(a);
    if (t == TC_FLOAT) return ldf(L, a, 0, 0) != 0.0f;
    if (t == TC_TRIPLE) return ldf(L, a, 0, 0) != 0.0f || ldf(L, a, 1, 0) != 0.0f || ldf(L, a, 2, 0) != 0.0f;
    return ldw(L, a, 0) != 0u;
}

// OpenImageIO fast_* forms of the transcendental ops with dual.h's fast_*
// derivative rules (dual.h:836-1262); false when OPC has none
template <int OPC>
__device__ __forceinline__ bool unary_fast(float v, float& f, float& df, bool& zero_derivs) {
    switch (OPC) {
    case OP_SIN: fm::sincos(v, &f, &df); return true;
    case OP_COS: { float sv; fm::sincos(v, &sv, &f); df = -sv; return true; }
    case OP_TAN: { f = fm::tan(v); const float cs = fm::cos(v); df = 1.0f / (cs * cs); return true; }
    case OP_ASIN:
        f = fm::asin(v);
        df = fabsf(v) < 1.0f ? 1.0f / sqrtf(1.0f - v * v) : 0.0f;
        return true;
    case OP_ACOS:
        f = fm::acos(v);
        df = fabsf(v) < 1.0f ? -1.0f / sqrtf(1.0f - v * v) : 0.0f;
        return true;
    case OP_ATAN: f = fm::atan(v); df = 1.0f / (1.0f + v * v); return true;
    case OP_SINH: f = fm::sinh(v); df = fm::cosh(v); return true;
    case OP_COSH: f = fm::cosh(v); df = fm::sinh(v); return true;
    case OP_TANH: { f = fm::tanh(v); const float ch = fm::cosh(v); df = 1.0f / (ch * ch); return true; }
    case OP_EXP: f = fm::exp(v); df = f; return true;
    case OP_EXP2: f = fm::exp2(v); df = f * 0.693147180559945309417f; return true;
    case OP_EXPM1: f = fm::expm1(v); df = fm::exp(v); return true;
    case OP_LOG: f = fm::log(v); df = v < kFltMin ? 0.0f : 1.0f / v; return true;
    case OP_LOG2: {
        f = fm::log2(v);
        const float aln2 = v * 0.693147180559945309417f;
        df = aln2 < kFltMin ? 0.0f : 1.0f / aln2;
        return true;
    }
    case OP_LOG10: {
        f = fm::log10(v);
        const float aln10 = v * 2.30258509299404568402f;
        df = aln10 < kFltMin ? 0.0f : 1.0f / aln10;
        return true;
    }
    case OP_ERF: f = fm::erf(v); df = fm::exp(-v * v) * 1.12837916709551257390f; return true;
    case OP_ERFC: f = fm::erfc(v); df = fm::exp(-v * v) * -1.12837916709551257390f; return true;
    case OP_CBRT:
        if (v != 0.0f) { f = fm::cbrt(v); df = 1.0f / (3.0f * f * f); }
        else { f = 0.0f; zero_derivs = true; }
        return true;
    default: return false;
    }
}

// componentwise unary math with dual.h derivative rules; a2 = 1 selects
// the fast forms
template <int OPC>
static __device__ void h_unary(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], x = a[1];
    int nc = anc(r);
    bool rd = ader(r);
    const bool fast = a[2] == 1u;
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        float v = ldf(L, x, c, 0);
        float f, df = 0.0f;
        bool zero_derivs = false;
        if (!(fast && unary_fast<OPC>(v, f, df, zero_derivs)))
        switch (OPC) {
        case OP_ABS: f = fabsf(v); df = v >= 0.0f ? 1.0f : -1.0f; break;
        case OP_FLOOR: f = floorf(v); zero_derivs = true; break;
        case OP_CEIL: f = ceilf(v); zero_derivs = true; break;
        case OP_ROUND: f = roundf(v); zero_derivs = true; break;
        case OP_TRUNC: f = truncf(v); zero_derivs = true; break;
        case OP_SIGN: f = v < 0.0f ? -1.0f : (v == 0.0f ? 0.0f : 1.0f); zero_derivs = true; break;
        case OP_SQRT:
            if (v > 0.0f) { f = sqrtf(v); df = 0.5f / f; } else { f = 0.0f; zero_derivs = true; }
            break;
        case OP_INVSQRT:
            if (v > 0.0f) { f = 1.0f / sqrtf(v); df = -0.5f * f / v; } else { f = 0.0f; zero_derivs = true; }
            break;
        case OP_CBRT:
            if (v != 0.0f) { f = fcbrt(v); df = 1.0f / (3.0f * f * f); } else { f = 0.0f; zero_derivs = true; }
            break;
        case OP_SIN: f = fsin(v); df = fcos(v); break;
        case OP_COS: f = fcos(v); df = -fsin(v); break;
        case OP_TAN: { f = ftan(v); float cs = fcos(v); df = 1.0f / (cs * cs); break; }
        case OP_ASIN:
            if (v >= 1.0f) { f = 1.57079632679489661923f; zero_derivs = true; }
            else if (v <= -1.0f) { f = -1.57079632679489661923f; zero_derivs = true; }
            else { f = fasin(v); df = 1.0f / sqrtf(1.0f - v * v); }
            break;
        case OP_ACOS:
            if (v >= 1.0f) { f = 0.0f; zero_derivs = true; }
            else if (v <= -1.0f) { f = 3.14159265358979323846f; zero_derivs = true; }
            else { f = facos(v); df = -1.0f / sqrtf(1.0f - v * v); }
            break;
        case OP_ATAN: f = fatan(v); df = 1.0f / (1.0f + v * v); break;
        case OP_SINH: f = fsinh(v); df = fcosh(v); break;
        case OP_COSH: f = fcosh(v); df = fsinh(v); break;
        case OP_TANH: { f = ftanh(v); float ch = fcosh(v); df = 1.0f / (ch * ch); break; }
        case OP_EXP: f = fexp(v); df = f; break;
        case OP_EXP2: f = fexp2(v); df = f * 0.693147180559945309417f; break;
        case OP_EXPM1: f = fexpm1(v); df = fexp(v); break;
        case OP_LOG: f = safe_log(v); df = v < kFltMin ? 0.0f : 1.0f / v; break;
        case OP_LOG2: f = safe_log2(v); df = v < kFltMin ? 0.0f : 1.0f / (v * 0.693147180559945309417f); break;
        case OP_LOG10: f = safe_log10(v); df = v < kFltMin ? 0.0f : 1.0f / (v * 2.30258509299404568402f); break;
        case OP_LOGB: f = logb_fast(v); zero_derivs = true; break;
        case OP_ERF: f = (float)erf((double)v); df = 1.12837916709551257390f * fexp(-v * v); break;
        case OP_ERFC: f = (float)erfc((double)v); df = -1.12837916709551257390f * fexp(-v * v); break;
        case OP_RADIANS: f = v * (3.14159265358979323846f / 180.0f); df = 3.14159265358979323846f / 180.0f; break;
        case OP_DEGREES: f = v * (180.0f / 3.14159265358979323846f); df = 180.0f / 3.14159265358979323846f; break;
        case OP_NEG: f = -v; df = -1.0f; break;
        default: f = v; break;
        }
        if (atc(r) == TC_INT) { stw(L, r, c, (uint32_t)(int)f); continue; }
        stf(L, r, c, f);
        if (!rd) continue;
        float dx = 0.0f, dy = 0.0f;
        if (!zero_derivs && ader(x)) {
            if (OPC == OP_NEG) { dx = -ldf(L, x, c, 1); dy = -ldf(L, x, c, 2); }
            else if (OPC == OP_ABS) {
                // fabs of a dual negates the whole dual when val < 0
                dx = v >= 0.0f ? ldf(L, x, c, 1) : -ldf(L, x, c, 1);
                dy = v >= 0.0f ? ldf(L, x, c, 2) : -ldf(L, x, c, 2);
            } else if (OPC == OP_RADIANS || OPC == OP_DEGREES) {
                dx = ldf(L, x, c, 1) * df; dy = ldf(L, x, c, 2) * df;
            } else { dx = df * ldf(L, x, c, 1); dy = df * ldf(L, x, c, 2); }
        }
        stf(L, r, nc + c, dx);
        stf(L, r, 2 * nc + c, dy);
    }
}

template <int OPC>
static __device__ void h_binary(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], x = a[1], y = a[2];
    int nc = anc(r);
    bool rd = ader(r);
    const bool fast = a[3] == 1u;  // pow, atan2: the fast forms
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        D2 u = ldd(L, x, c), v = ldd(L, y, c);
        D2 res;
        if (OPC == OP_POW) {
            if (rd && (ader(x) || ader(y))) {
                float powuvm1 = fast ? fm::safe_pow(u.v, v.v - 1.0f) : safe_pow(u.v, v.v - 1.0f);
                float powuv = powuvm1 * u.v;
                float logu = u.v > 0.0f ? (fast ? fm::log(u.v) : safe_log(u.v)) : 0.0f;
                float du = v.v * powuvm1, dv = logu * powuv;
                res = d2(powuv, du * u.dx + dv * v.dx, du * u.dy + dv * v.dy);
            } else {
                res = d2c(fast ? fm::safe_pow(u.v, v.v) : safe_pow(u.v, v.v));
            }
        } else if (OPC == OP_ATAN2) {
            float f = fast ? fm::atan2(u.v, v.v) : fatan2(u.v, v.v);
            float denom = (v.v == 0.0f && u.v == 0.0f) ? 0.0f : 1.0f / (v.v * v.v + u.v * u.v);
            float dfdy = -v.v * denom, dfdx = u.v * denom;
            res = d2(f, dfdy * u.dx + dfdx * v.dx, dfdy * u.dy + dfdx * v.dy);
        } else if (OPC == OP_FMOD) {
            res = d2(safe_fmod(u.v, v.v), u.dx, u.dy);
        } else if (OPC == OP_MIN) {
            res = u.v <= v.v ? u : v;
        } else if (OPC == OP_MAX) {
            res = u.v > v.v ? u : v;
        } else {  // OP_STEP: step(edge, x)
            res = d2c(v.v < u.v ? 0.0f : 1.0f);
        }
        if (!rd) { stval(L, r, c, res.v); continue; }
        std2(L, r, c, res);
    }
}

static __device__ void h_clamp(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0];
    int nc = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        D2 x = ldd(L, a[1], c), lo = ldd(L, a[2], c), hi = ldd(L, a[3], c);
        if (atc(r) == TC_INT) {
            int xi = ldi(L, a[1], c), li = ldi(L, a[2], c), hiv = ldi(L, a[3], c);
            xi = xi < li ? li : xi;
            xi = xi > hiv ? hiv : xi;
            stw(L, r, c, (uint32_t)xi);
            continue;
        }
        D2 v = x.v < lo.v ? lo : x;
        v = v.v > hi.v ? hi : v;
        std2(L, r, c, v);
    }
}

static __device__ void h_mix(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0];
    int nc = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        D2 x = ldd(L, a[1], c), y = ldd(L, a[2], c), t = ldd(L, a[3], c);
        float one_t = 1.0f - t.v;
        float v = x.v * one_t + y.v * t.v;
        float ymx = y.v - x.v;
        D2 res = d2(v, one_t * x.dx + t.v * y.dx + ymx * t.dx, one_t * x.dy + t.v * y.dy + ymx * t.dy);
        std2(L, r, c, res);
    }
}

static __device__ void h_smoothstep(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0];
    int nc = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        D2 e0 = ldd(L, a[1], c), e1 = ldd(L, a[2], c), x = ldd(L, a[3], c);
        D2 res;
        if (x.v < e0.v) res = d2c(0.0f);
        else if (x.v >= e1.v) res = d2c(1.0f);
        else if (!ader(r)) {
            float t = (x.v - e0.v) / (e1.v - e0.v);
            res = d2c((3.0f - 2.0f * t) * (t * t));
        } else {
            // Dual2: t = (x-e0)/(e1-e0); (3 - 2t)*t*t
            D2 num = x - e0, den = e1 - e0;
            float binv = 1.0f / den.v, q = num.v / den.v;
            D2 t = d2(q, binv * (num.dx - q * den.dx), binv * (num.dy - q * den.dy));
            D2 k = d2(3.0f - 2.0f * t.v, -(t.dx * 2.0f), -(t.dy * 2.0f));
            res = (k * t) * t;
        }
        std2(L, r, c, res);
    }
}

static __device__ void h_select(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0];
    int nc = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        bool cond = atc(a[3]) == TC_TRIPLE ? ldf(L, a[3], c, 0) != 0.0f : truth(L, a[3]);
        D2 v = cond ? ldd(L, a[2], c) : ldd(L, a[1], c);
        if (atc(r) == TC_INT) { stw(L, r, c, (uint32_t)ldi(L, cond ? a[2] : a[1], c)); continue; }
        std2(L, r, c, v);
    }
}

// ---- vector ops (dual_vec.h) ----------------------------------------------------
static __device__ void h_dot(const Lane& L, const uint32_t* a) {
    D2 ax = ldd(L, a[1], 0), ay = ldd(L, a[1], 1), az = ldd(L, a[1], 2);
    D2 bx = ldd(L, a[2], 0), by = ldd(L, a[2], 1), bz = ldd(L, a[2], 2);
    if (!ader(a[0])) { stval(L, a[0], 0, ax.v * bx.v + ay.v * by.v + az.v * bz.v); return; }
    std2(L, a[0], 0, ax * bx + ay * by + az * bz);
}
static __device__ void h_cross(const Lane& L, const uint32_t* a) {
    D2 ax = ldd(L, a[1], 0), ay = ldd(L, a[1], 1), az = ldd(L, a[1], 2);
    D2 bx = ldd(L, a[2], 0), by = ldd(L, a[2], 1), bz = ldd(L, a[2], 2);
    if (!ader(a[0])) {
        stval(L, a[0], 0, ay.v * bz.v - az.v * by.v);
        stval(L, a[0], 1, az.v * bx.v - ax.v * bz.v);
        stval(L, a[0], 2, ax.v * by.v - ay.v * bx.v);
        return;
    }
    std2(L, a[0], 0, ay * bz - az * by);
    std2(L, a[0], 1, az * bx - ax * bz);
    std2(L, a[0], 2, ax * by - ay * bx);
}
__device__ __forceinline__ D2 dsqrt(D2 a) {
    if (a.v > 0.0f) { float f = sqrtf(a.v), df = 0.5f / f; return d2(f, df * a.dx, df * a.dy); }
    return d2c(0.0f);
}
// Imath Vec3::length() for the value-only path
__device__ __forceinline__ float vlength(float x, float y, float z) {
    float l2 = x * x + y * y + z * z;
    if (l2 < 2.0f * kFltMin) {
        // lengthTiny: rescale by the largest component
        float m = fmaxf(fabsf(x), fmaxf(fabsf(y), fabsf(z)));
        if (m == 0.0f) return 0.0f;
        x /= m; y /= m; z /= m;
        return m * sqrtf(x * x + y * y + z * z);
    }
    return sqrtf(l2);
}
static __device__ void h_length(const Lane& L, const uint32_t* a, bool distance) {
    D2 x = ldd(L, a[1], 0), y = ldd(L, a[1], 1), z = ldd(L, a[1], 2);
    if (distance) { x = x - ldd(L, a[2], 0); y = y - ldd(L, a[2], 1); z = z - ldd(L, a[2], 2); }
    if (!ader(a[0])) {
        float v = distance ? sqrtf(x.v * x.v + y.v * y.v + z.v * z.v) : vlength(x.v, y.v, z.v);
        stval(L, a[0], 0, v);
        return;
    }
    std2(L, a[0], 0, dsqrt(x * x + y * y + z * z));
}
static __device__ void h_normalize(const Lane& L, const uint32_t* a) {
    D2 x = ldd(L, a[1], 0), y = ldd(L, a[1], 1), z = ldd(L, a[1], 2);
    if (!ader(a[0])) {
        float len = sqrtf(x.v * x.v + y.v * y.v + z.v * z.v);
        if (len > 0.0f) {
            float inv = 1.0f / len;
            stval(L, a[0], 0, x.v * inv); stval(L, a[0], 1, y.v * inv); stval(L, a[0], 2, z.v * inv);
        } else {
            stval(L, a[0], 0, 0.0f); stval(L, a[0], 1, 0.0f); stval(L, a[0], 2, 0.0f);
        }
        return;
    }
    D2 len = dsqrt(x * x + y * y + z * z);
    if (len.v > 0.0f) {
        float binv = 1.0f / len.v, q = 1.0f / len.v;
        D2 inv = d2(q, binv * (-q * len.dx), binv * (-q * len.dy));
        std2(L, a[0], 0, x * inv); std2(L, a[0], 1, y * inv); std2(L, a[0], 2, z * inv);
    } else {
        for (int c = 0; c < 3; ++c) std2(L, a[0], c, d2c(0.0f));
    }
}

// ---- transforms (dual_vec.h:336-400, opmatrix.cpp:86-131) ---------------------
static __device__ void h_transform(const Lane& L, const uint32_t* a) {
    uint32_t r = a[0], p = a[1], m = a[2];
    int kind = (int)a[3];
    float M[16];
    for (int i = 0; i < 16; ++i) M[i] = __uint_as_float(ldw(L, m, i));
    D2 x = ldd(L, p, 0), y = ldd(L, p, 1), z = ldd(L, p, 2);
    if (kind == 0) {
        // robust_multVecMatrix: homogeneous point, divide by w unless w == 0
        if (!ader(r)) {
            float A = x.v * M[0] + y.v * M[4] + z.v * M[8] + M[12];
            float B = x.v * M[1] + y.v * M[5] + z.v * M[9] + M[13];
            float C = x.v * M[2] + y.v * M[6] + z.v * M[10] + M[14];
            float W = x.v * M[3] + y.v * M[7] + z.v * M[11] + M[15];
            if (W != 0.0f) { stval(L, r, 0, A / W); stval(L, r, 1, B / W); stval(L, r, 2, C / W); }
            else { stval(L, r, 0, 0.0f); stval(L, r, 1, 0.0f); stval(L, r, 2, 0.0f); }
            return;
        }
        D2 A = x * M[0] + y * M[4] + z * M[8] + M[12];
        D2 B = x * M[1] + y * M[5] + z * M[9] + M[13];
        D2 C = x * M[2] + y * M[6] + z * M[10] + M[14];
        D2 W = x * M[3] + y * M[7] + z * M[11] + M[15];
        if (W.v != 0.0f) {
            float binv = 1.0f / W.v;
            D2 o[3] = { A, B, C };
            for (int c = 0; c < 3; ++c) {
                float q = o[c].v / W.v;
                std2(L, r, c, d2(q, binv * (o[c].dx - q * W.dx), binv * (o[c].dy - q * W.dy)));
            }
        } else {
            for (int c = 0; c < 3; ++c) std2(L, r, c, d2c(0.0f));
        }
        return;
    }
    // vector (multDirMatrix on value and each partial)
    float in[3][3] = { { x.v, y.v, z.v }, { x.dx, y.dx, z.dx }, { x.dy, y.dy, z.dy } };
    int nd = ader(r) ? 3 : 1;
    OSLG_SPEC_UNROLL
    for (int d = 0; d < nd; ++d) {
        float X = in[d][0], Y = in[d][1], Z = in[d][2];
        float o0 = X * M[0] + Y * M[4] + Z * M[8];
        float o1 = X * M[1] + Y * M[5] + Z * M[9];
        float o2 = X * M[2] + Y * M[6] + Z * M[10];
        stf(L, r, d * 3 + 0, o0); stf(L, r, d * 3 + 1, o1); stf(L, r, d * 3 + 2, o2);
    }
}

// ---- matrix extras ---------------------------------------------------------------
// 4x4 inverse by Gauss-Jordan elimination with partial pivoting; a singular
// matrix gives the identity (Imath's inverse() with exceptions off returns
// identity). Same steps as the host statement in the oracle.
__device__ __forceinline__ void m44_inverse(const float* A, float* out) {
    float t[16], s[16];
    for (int i = 0; i < 16; ++i) { t[i] = A[i]; s[i] = (i % 5 == 0) ? 1.0f : 0.0f; }
    for (int i = 0; i < 4; ++i) {
        int piv = i;
        float pmax = fabsf(t[i * 4 + i]);
        for (int j = i + 1; j < 4; ++j)
            if (fabsf(t[j * 4 + i]) > pmax) { pmax = fabsf(t[j * 4 + i]); piv = j; }
        if (pmax == 0.0f) {
            for (int k = 0; k < 16; ++k) out[k] = (k % 5 == 0) ? 1.0f : 0.0f;
            return;
        }
        if (piv != i)
            for (int k = 0; k < 4; ++k) {
                float u = t[i * 4 + k]; t[i * 4 + k] = t[piv * 4 + k]; t[piv * 4 + k] = u;
                u = s[i * 4 + k]; s[i * 4 + k] = s[piv * 4 + k]; s[piv * 4 + k] = u;
            }
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            const float f = t[j * 4 + i] / t[i * 4 + i];
            for (int k = 0; k < 4; ++k) {
                t[j * 4 + k] = t[j * 4 + k] - f * t[i * 4 + k];
                s[j * 4 + k] = s[j * 4 + k] - f * s[i * 4 + k];
            }
        }
    }
    for (int i = 0; i < 4; ++i) {
        const float f = t[i * 4 + i];
        for (int k = 0; k < 4; ++k) out[i * 4 + k] = s[i * 4 + k] / f;
    }
}
__device__ __forceinline__ void m44_mul(const float* A, const float* B, float* out) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            out[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j] + A[i * 4 + 2] * B[2 * 4 + j]
                           + A[i * 4 + 3] * B[3 * 4 + j];
}
// Imathx.h:456-492
__device__ __forceinline__ float det2(float a, float b, float c, float d) { return a * d - b * c; }
__device__ __forceinline__ float det3(float a1, float a2, float a3, float b1, float b2, float b3, float c1, float c2,
                                      float c3) {
    return a1 * det2(b2, b3, c2, c3) - b1 * det2(a2, a3, c2, c3) + c1 * det2(a2, a3, b2, b3);
}
__device__ __forceinline__ float det4(const float* m) {
    const float a1 = m[0], b1 = m[1], c1 = m[2], d1 = m[3];
    const float a2 = m[4], b2 = m[5], c2 = m[6], d2_ = m[7];
    const float a3 = m[8], b3 = m[9], c3 = m[10], d3 = m[11];
    const float a4 = m[12], b4 = m[13], c4 = m[14], d4 = m[15];
    return a1 * det3(b2, b3, b4, c2, c3, c4, d2_, d3, d4) - b1 * det3(a2, a3, a4, c2, c3, c4, d2_, d3, d4)
         + c1 * det3(a2, a3, a4, b2, b3, b4, d2_, d3, d4) - d1 * det3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
}

// matrix division (src/liboslexec/opmatrix.cpp:49-73)
static __device__ void h_mdiv(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0], x = a[1], y = a[2];
    float out[16];
    const bool mx = atc(x) == TC_MATRIX, my = atc(y) == TC_MATRIX;
    if (mx && my) {
        float A[16], B[16], Bi[16];
        for (int i = 0; i < 16; ++i) { A[i] = __uint_as_float(ldw(L, x, i)); B[i] = __uint_as_float(ldw(L, y, i)); }
        m44_inverse(B, Bi);
        m44_mul(A, Bi, out);
    } else if (mx) {
        const float f = 1.0f / ldf(L, y, 0, 0);
        for (int i = 0; i < 16; ++i) out[i] = __uint_as_float(ldw(L, x, i)) * f;
    } else if (my) {
        float B[16], Bi[16];
        for (int i = 0; i < 16; ++i) B[i] = __uint_as_float(ldw(L, y, i));
        m44_inverse(B, Bi);
        const float f = ldf(L, x, 0, 0);
        for (int i = 0; i < 16; ++i) out[i] = Bi[i] * f;
    } else {
        const float av = ldf(L, x, 0, 0), bv = ldf(L, y, 0, 0);
        const float f = (bv == 0.0f) ? 0.0f : (av / bv);
        for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? f : 0.0f;
    }
    for (int i = 0; i < 16; ++i) stf(L, r, i, out[i]);
}

// transformn: multDirMatrix by the transposed inverse (opmatrix.cpp:122-137)
static __device__ void h_transformn(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0], p = a[1], m = a[2];
    float M[16], Mi[16], T[16];
    for (int i = 0; i < 16; ++i) M[i] = __uint_as_float(ldw(L, m, i));
    m44_inverse(M, Mi);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) T[i * 4 + j] = Mi[j * 4 + i];
    const int nd = ader(r) ? 3 : 1;
    OSLG_SPEC_UNROLL
    for (int d = 0; d < nd; ++d) {
        const float X = ldf(L, p, 0, d), Y = ldf(L, p, 1, d), Z = ldf(L, p, 2, d);
        stf(L, r, d * 3 + 0, X * T[0] + Y * T[4] + Z * T[8]);
        stf(L, r, d * 3 + 1, X * T[1] + Y * T[5] + Z * T[9]);
        stf(L, r, d * 3 + 2, X * T[2] + Y * T[6] + Z * T[10]);
    }
}

static __device__ void h_matrix_misc(const Lane& L, uint32_t code, const uint32_t* a) {
    const uint32_t r = a[0], x = a[1];
    if (code == OP_TRANSPOSE) {
        float M[16];
        for (int i = 0; i < 16; ++i) M[i] = __uint_as_float(ldw(L, x, i));
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) stf(L, r, i * 4 + j, M[j * 4 + i]);
    } else {  // OP_DETERMINANT
        float M[16];
        for (int i = 0; i < 16; ++i) M[i] = __uint_as_float(ldw(L, x, i));
        stval(L, r, 0, det4(M));
    }
}

// area (llvm_ops.cpp:915-941) and filterwidth (:944-965): value-only results
static __device__ void h_deriv_misc(const Lane& L, uint32_t code, const uint32_t* a) {
    const uint32_t r = a[0], x = a[1];
    if (code == OP_AREA) {
        const V3 dx = v3(ldf(L, x, 0, 1), ldf(L, x, 1, 1), ldf(L, x, 2, 1));
        const V3 dy = v3(ldf(L, x, 0, 2), ldf(L, x, 1, 2), ldf(L, x, 2, 2));
        stval(L, r, 0, vlen_imath(vcross(dx, dy)));
    } else {
        const int n = anc(x);
        OSLG_SPEC_UNROLL
        for (int c = 0; c < n; ++c) {
            const float dx = ldf(L, x, c, 1), dy = ldf(L, x, c, 2);
            stval(L, r, c, sqrtf(dx * dx + dy * dy));
        }
    }
}

// sincos (llvm_ops.cpp:298-430): sine and cosine of each component; each
// result carries the derivatives its symbol asks for; a3 = 1: fast forms
static __device__ void h_sincos(const Lane& L, const uint32_t* a) {
    const uint32_t x = a[0], rs = a[1], rc = a[2];
    const int nc = anc(x);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        const float v = ldf(L, x, c, 0), xdx = ldf(L, x, c, 1), xdy = ldf(L, x, c, 2);  // x may alias a result
        float sv, cv;
        if (a[3] == 1u) fm::sincos(v, &sv, &cv);
        else { sv = fsin(v); cv = fcos(v); }
        stf(L, rs, c, sv);
        stf(L, rc, c, cv);
        if (ader(rs)) { stf(L, rs, nc + c, cv * xdx); stf(L, rs, 2 * nc + c, cv * xdy); }
        if (ader(rc)) { stf(L, rc, nc + c, -sv * xdx); stf(L, rc, 2 * nc + c, -sv * xdy); }
    }
}

// calculatenormal (llvm_ops.cpp:915-934): dP/dx x dP/dy, operands swapped
// when flipHandedness is set; not normalized, no derivatives
static __device__ void h_calcnormal(const Lane& L, const uint32_t* a, const oslg_shaderglobals& G);
// raytype (batched_llvm_gen.cpp:8520-8560): the raytype bits of the rays
// being shaded against the name's bit, ShadingSystemImpl::raytype_bit
// (shadingsys.cpp:3823-3829) looked up at run time for a varying name
static __device__ void h_raytype(const Lane& L, const uint32_t* a, const oslg_shaderglobals& G) {
    uint32_t bit = a[2];
    if (a[1] != kNoArg) {
        const uint32_t h = ldw(L, a[1], 0);
        bit = 0;
        for (int i = 0; i < (int)a[4]; ++i)
            if (ldw(L, a[3], i) == h) { bit = 1u << i; break; }
    }
    stw(L, a[0], 0, ((uint32_t)G.raytype & bit) != 0u ? 1u : 0u);
}

// luminance: dot with the colour system's luminance scale (a2, a constant
// triple the lowering computes; opcolor.cpp:461-476)
static __device__ void h_luminance(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0], c = a[1], s = a[2];
    const float sx = ldf(L, s, 0, 0), sy = ldf(L, s, 1, 0), sz = ldf(L, s, 2, 0);
    const int nd = ader(r) ? 3 : 1;
    OSLG_SPEC_UNROLL
    for (int d = 0; d < nd; ++d)
        stf(L, r, d, ldf(L, c, 0, d) * sx + ldf(L, c, 1, d) * sy + ldf(L, c, 2, d) * sz);
}

// ---- colour spaces (src/liboslexec/opcolor.cpp:270-380 ColorSystem::transformc,
// opcolor_impl.h:240-490 the conversions; Foley & van Dam) on float or Dual2
// components: comparisons and branches on values, arithmetic as dual.h ----
__device__ __forceinline__ float cval(float x) { return x; }
__device__ __forceinline__ float cval(D2 x) { return x.v; }
template <class S> __device__ __forceinline__ S ck(float v);
template <> __device__ __forceinline__ float ck<float>(float v) { return v; }
template <> __device__ __forceinline__ D2 ck<D2>(float v) { return d2c(v); }
template <class S> __device__ __forceinline__ S cmin(S a, S b) { return cval(a) < cval(b) ? a : b; }
template <class S> __device__ __forceinline__ S cmax(S a, S b) { return cval(a) > cval(b) ? a : b; }
template <class S> struct C3 { S x, y, z; };
template <class S>
__device__ __forceinline__ C3<S> hsv_to_rgb(C3<S> c) {
    S h = c.x;
    const S s = c.y, v = c.z;
    if (cval(s) < 0.0001f) return { v, v, v };
    h = 6.0f * (h - floorf(cval(h)));
    const float fh = floorf(cval(h));
    const int hi = fh != fh ? 0 : (int)fh;
    const S f = h - (float)hi;
    const S p = v * (1.0f - s);
    const S q = v * (1.0f - s * f);
    const S t = v * (1.0f - s * (1.0f - f));
    if (hi == 0) return { v, t, p };
    if (hi == 1) return { q, v, p };
    if (hi == 2) return { p, v, t };
    if (hi == 3) return { p, q, v };
    if (hi == 4) return { t, p, v };
    return { v, p, q };
}
template <class S>
__device__ __forceinline__ C3<S> rgb_to_hsv(C3<S> c) {
    const S mn = cmin(c.x, cmin(c.y, c.z)), mx = cmax(c.x, cmax(c.y, c.z));
    const S delta = mx - mn;
    const S v = mx;
    S s = ck<S>(0.0f), h = ck<S>(0.0f);
    if (cval(mx) > 0.0f) s = delta / mx;
    if (cval(s) > 0.0f) {
        float k;
        S x, y;
        if (cval(c.x) >= cval(mx)) { k = 0.0f / 6.0f; x = c.y; y = c.z; }
        else if (cval(c.y) >= cval(mx)) { k = 2.0f / 6.0f; x = c.z; y = c.x; }
        else { k = 4.0f / 6.0f; x = c.x; y = c.y; }
        h = k + (x - y) / (6.0f * delta);
        if (cval(h) < 0.0f) h = h + 1.0f;
    }
    return { h, s, v };
}
template <class S>
__device__ __forceinline__ C3<S> hsl_to_rgb(C3<S> c) {
    const S h = c.x, l = c.z;
    S s = c.y;
    const S v = cval(l) <= 0.5f ? l * (1.0f + s) : l * (1.0f - s) + s;
    if (cval(v) <= 0.0f) return { ck<S>(0.0f), ck<S>(0.0f), ck<S>(0.0f) };
    const S mn = 2.0f * l - v;
    s = (v - mn) / v;
    return hsv_to_rgb<S>({ h, s, v });
}
template <class S>
__device__ __forceinline__ C3<S> rgb_to_hsl(C3<S> c) {
    const S minval = cmin(c.x, cmin(c.y, c.z));
    const C3<S> hsv = rgb_to_hsv(c);
    const S maxval = hsv.z;
    const S h = hsv.x, l = (minval + maxval) / 2.0f;
    S s;
    if (cval(minval) == cval(maxval)) {
        s = ck<S>(0.0f);
    } else {
        const S m2m = maxval - minval;
        const S divisor = cval(l) <= 0.5f ? maxval + minval : (2.0f - maxval) - minval;
        s = m2m / divisor;
    }
    return { h, s, l };
}
// row vector times a 3x3 matrix m (rows of 3)
template <class S>
__device__ __forceinline__ C3<S> cmul33(C3<S> c, const float* m) {
    return { c.x * m[0] + c.y * m[3] + c.z * m[6], c.x * m[1] + c.y * m[4] + c.z * m[7],
             c.x * m[2] + c.y * m[5] + c.z * m[8] };
}
__device__ __constant__ const float c_yiq_to_rgb[9] = { 1.0000f, 1.0000f, 1.0000f, 0.9557f, -0.2716f, -1.1082f,
                                                        0.6199f, -0.6469f, 1.7051f };
__device__ __constant__ const float c_rgb_to_yiq[9] = { 0.299f, 0.596f, 0.212f, 0.587f, -0.275f, -0.523f,
                                                        0.114f, -0.321f, 0.311f };
template <class S>
__device__ __forceinline__ C3<S> xyz_to_xyy(C3<S> c) {
    const S n = (c.x + c.y) + c.z;
    const S ninv = cval(n) >= 1.0e-6f ? 1.0f / n : ck<S>(0.0f);
    return { c.x * ninv, c.y * ninv, c.y };
}
template <class S>
__device__ __forceinline__ C3<S> xyy_to_xyz(C3<S> c) {
    const S Y = c.z;
    const S Y_y = cval(c.y) > 1.0e-6f ? Y / c.y : ck<S>(0.0f);
    return { Y_y * c.x, Y, Y_y * ((1.0f - c.x) - c.y) };
}
__device__ __forceinline__ float cpow(float x, float y) { return safe_pow(x, y); }
__device__ __forceinline__ D2 cpow(D2 u, float y) {  // dual.h safe_pow, the exponent a constant Dual2
    const float powuvm1 = safe_pow(u.v, y - 1.0f);
    const float powuv = powuvm1 * u.v;
    const float logu = u.v > 0.0f ? safe_log(u.v) : 0.0f;
    const float du = y * powuvm1, dv = logu * powuv;
    return d2(powuv, du * u.dx + dv * 0.0f, du * u.dy + dv * 0.0f);
}
template <class S>
__device__ __forceinline__ S srgb_to_linear1(S x) {
    return cval(x) <= 0.04045f ? x * (1.0f / 12.92f) : cpow((x + 0.055f) * (1.0f / 1.055f), 2.4f);
}
template <class S>
__device__ __forceinline__ S linear_to_srgb1(S x) {
    return cval(x) <= 0.0031308f ? 12.92f * x : 1.055f * cpow(x, 1.f / 2.4f) - 0.055f;
}
template <class S>
__device__ __forceinline__ C3<S> transformc_any(C3<S> c, uint32_t from, uint32_t to, const float* xyz2rgb,
                                                const float* rgb2xyz) {
    C3<S> rgb;
    switch (from) {
    case CS_HSV: rgb = hsv_to_rgb(c); break;
    case CS_HSL: rgb = hsl_to_rgb(c); break;
    case CS_YIQ: rgb = cmul33(c, c_yiq_to_rgb); break;
    case CS_XYZ: rgb = cmul33(c, xyz2rgb); break;
    case CS_XYY: rgb = cmul33(xyy_to_xyz(c), xyz2rgb); break;
    case CS_SRGB: rgb = { srgb_to_linear1(c.x), srgb_to_linear1(c.y), srgb_to_linear1(c.z) }; break;
    default: rgb = c; break;
    }
    switch (to) {
    case CS_HSV: return rgb_to_hsv(rgb);
    case CS_HSL: return rgb_to_hsl(rgb);
    case CS_YIQ: return cmul33(rgb, c_rgb_to_yiq);
    case CS_XYZ: return cmul33(rgb, rgb2xyz);
    case CS_XYY: return xyz_to_xyy(cmul33(rgb, rgb2xyz));
    case CS_SRGB: return { linear_to_srgb1(rgb.x), linear_to_srgb1(rgb.y), linear_to_srgb1(rgb.z) };
    default: return rgb;
    }
}
static __device__ void h_transformc(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0], c = a[1];
    float m[18];
    OSLG_SPEC_UNROLL
    for (int k = 0; k < 18; ++k) m[k] = __uint_as_float(ldw(L, a[3], k));
    const uint32_t from = a[2] & 0xFFu, to = (a[2] >> 8) & 0xFFu;
    if (ader(r)) {
        const C3<D2> o = transformc_any<D2>({ ldd(L, c, 0), ldd(L, c, 1), ldd(L, c, 2) }, from, to, m, m + 9);
        std2(L, r, 0, o.x);
        std2(L, r, 1, o.y);
        std2(L, r, 2, o.z);
    } else {
        const C3<float> o = transformc_any<float>({ ldf(L, c, 0, 0), ldf(L, c, 1, 0), ldf(L, c, 2, 0) }, from, to, m,
                                                  m + 9);
        stf(L, r, 0, o.x);
        stf(L, r, 1, o.y);
        stf(L, r, 2, o.z);
    }
}
// osl_wavelength_color_vf (opcolor.cpp:446-456): the CIE matching functions
// lerped at (lambda - 380) / 5 (zero outside 380..775 nm), to RGB, scaled
// by 1 / 2.52 and clamped at zero; no derivatives.
static __device__ void h_wavelength(const Lane& L, const uint32_t* a) {
    const float lambda = ldf(L, a[1], 0, 0);
    const float ii = (lambda - 380.0f) / 5.0f;
    const int i = (int)ii;
    float xyz[3] = { 0.0f, 0.0f, 0.0f };
    if (!((i < 0) | (i >= 80))) {
        const float rem = ii - (float)i;
        for (int k = 0; k < 3; ++k) {
            const float c0 = __uint_as_float(ldw(L, a[2], 9 + 3 * i + k));
            const float c1 = __uint_as_float(ldw(L, a[2], 9 + 3 * i + 3 + k));
            xyz[k] = c0 * (1.0f - rem) + c1 * rem;
        }
    }
    float m[9];
    for (int k = 0; k < 9; ++k) m[k] = __uint_as_float(ldw(L, a[2], k));
    const C3<float> rgb = cmul33<float>({ xyz[0], xyz[1], xyz[2] }, m);
    const float sc = (float)(1.0 / 2.52);
    const float o[3] = { rgb.x * sc, rgb.y * sc, rgb.z * sc };
    const uint32_t r = a[0];
    for (int k = 0; k < 3; ++k) stf(L, r, k, o[k] < 0.0f ? 0.0f : o[k]);
    if (ader(r))
        for (int k = 0; k < 6; ++k) stf(L, r, 3 + k, 0.0f);
}

// ---- texture (src/liboslexec/optexture.cpp:54-111 osl_texture; the
// filtering itself is OIIO's TextureSystem, which is not in the tree) ----
// A mipmapped bilinear lookup: the footprint of (s, t)'s x/y derivatives in
// level-0 texels (times "width") picks a level of detail log2(footprint),
// the two nearest levels are sampled bilinearly at texel centres and
// blended. Every step is single float operations (own_log for the level),
// so the oracle's statement of the same steps gives the same bits.
__device__ __forceinline__ int tex_wrap(int i, int n, uint32_t mode, bool* inside) {
    *inside = true;
    if (mode == TW_PERIODIC) {
        int m = i % n;
        return m < 0 ? m + n : m;
    }
    if (mode == TW_MIRROR) {
        const int p = 2 * n;
        int m = i % p;
        if (m < 0) m += p;
        return m < n ? m : p - 1 - m;
    }
    if (i < 0 || i >= n) {
        *inside = mode != TW_BLACK;
        return i < 0 ? 0 : n - 1;
    }
    return i;
}
__device__ __forceinline__ float tex_coord(float x) {
    // finite and bounded before the float->int conversions (NaN -> 0)
    return x == x ? fminf(fmaxf(x, -1.0e7f), 1.0e7f) : 0.0f;
}
__device__ __forceinline__ void tex_bilinear(const TexDesc& T, int lev, float s, float t, uint32_t sw, uint32_t tw,
                                             int first, int nc, float* out) {
    const int W = T.w[lev], H = T.h[lev];
    const float* base = T.data + T.off[lev];
    const float x = tex_coord(s * (float)W - 0.5f), y = tex_coord(t * (float)H - 0.5f);
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    bool in_x0, in_x1, in_y0, in_y1;
    const int cx0 = tex_wrap(ix, W, sw, &in_x0), cx1 = tex_wrap(ix + 1, W, sw, &in_x1);
    const int cy0 = tex_wrap(iy, H, tw, &in_y0), cy1 = tex_wrap(iy + 1, H, tw, &in_y1);
    for (int c = 0; c < nc; ++c) {
        const int ch = first + c < T.nch ? first + c : (T.nch == 1 ? 0 : -1);
        float v00 = 0.0f, v10 = 0.0f, v01 = 0.0f, v11 = 0.0f;
        if (ch >= 0) {
            if (in_x0 && in_y0) v00 = __ldg(base + ((int64_t)cy0 * W + cx0) * T.nch + ch);
            if (in_x1 && in_y0) v10 = __ldg(base + ((int64_t)cy0 * W + cx1) * T.nch + ch);
            if (in_x0 && in_y1) v01 = __ldg(base + ((int64_t)cy1 * W + cx0) * T.nch + ch);
            if (in_x1 && in_y1) v11 = __ldg(base + ((int64_t)cy1 * W + cx1) * T.nch + ch);
        }
        const float top = (1.0f - fx) * v00 + fx * v10;
        const float bot = (1.0f - fx) * v01 + fx * v11;
        out[c] = (1.0f - fy) * top + fy * bot;
    }
}
// Mipmapped bilinear lookup: the footprint (level-0 texels along x and y,
// times width) picks the level of detail; the two nearest levels blend.
__device__ __forceinline__ void tex_filtered(const TexDesc& T, float s, float t, float dsx, float dtx, float dsy,
                                             float dty, float width, uint32_t sw, uint32_t tw, int first, int nc,
                                             float* res) {
    const float len = fmaxf(sqrtf(dsx * dsx + dtx * dtx), sqrtf(dsy * dsy + dty * dty)) * width;
    float lod = len > 1.0f ? own_log(len) * 1.44269504f : 0.0f;
    lod = fminf(lod, (float)(T.nlevels - 1));
    const int l0 = (int)lod;
    const float f = lod - (float)l0;
    tex_bilinear(T, l0, s, t, sw, tw, first, nc, res);
    if (f > 0.0f && l0 + 1 < T.nlevels) {
        float hi[3];
        tex_bilinear(T, l0 + 1, s, t, sw, tw, first, nc, hi);
        for (int c = 0; c < nc; ++c) res[c] = (1.0f - f) * res[c] + f * hi[c];
    }
}
static __device__ void h_texture(const Lane& L, const uint32_t* a, const TexDesc* tex, int ntex, uint32_t* st) {
    const uint32_t r = a[0];
    const int nc = anc(r) == 3 ? 3 : 1;
    const int id = (int)(a[3] & 0xFFu);
    float res[3] = { 0.0f, 0.0f, 0.0f };
    if (id < ntex) {
        const TexDesc& T = tex[id];
        const uint32_t sw = (a[3] >> 8) & 15u, tw = (a[3] >> 12) & 15u;
        const int first = (int)((a[3] >> 16) & 0xFFu);
        const D2 s = ldd(L, a[1], 0), t = ldd(L, a[2], 0);
        const float width = ldf(L, a[4], 0, 0);
        const float w0 = (float)T.w[0], h0 = (float)T.h[0];
        tex_filtered(T, s.v, t.v, s.dx * w0, t.dx * h0, s.dy * w0, t.dy * h0, width, sw, tw, first, nc, res);
    } else {
        raise_status(st, ST_ARRAY_BOUNDS);
    }
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) std2(L, r, c, d2c(res[c]));
}

// environment (osl_environment, src/liboslexec/optexture.cpp): a
// latitude-longitude image looked up by direction, z up:
// s = atan2(y, x) / 2pi + 0.5 (periodic), t = 0.5 - atan2(z, hypot(x, y)) / pi
// (clamped). The footprint maps R + dR/dx and R + dR/dy the same way, the
// s differences wrapped into [-0.5, 0.5] across the seam.
__device__ __forceinline__ void env_st(float x, float y, float z, float* s, float* t) {
    const float h = sqrtf(x * x + y * y);
    *s = fatan2(y, x) * 0.159154943f + 0.5f;
    *t = 0.5f - fatan2(z, h) * 0.318309886f;
}
__device__ __forceinline__ float env_wrap_ds(float d) { return d > 0.5f ? d - 1.0f : (d < -0.5f ? d + 1.0f : d); }
static __device__ void h_environment(const Lane& L, const uint32_t* a, const TexDesc* tex, int ntex, uint32_t* st) {
    const uint32_t r = a[0];
    const int nc = anc(r) == 3 ? 3 : 1;
    const int id = (int)(a[3] & 0xFFu);
    float res[3] = { 0.0f, 0.0f, 0.0f };
    if (id < ntex) {
        const TexDesc& T = tex[id];
        const int first = (int)((a[3] >> 16) & 0xFFu);
        const D2 x = ldd(L, a[1], 0), y = ldd(L, a[1], 1), z = ldd(L, a[1], 2);
        const float width = ldf(L, a[4], 0, 0);
        float s, t, sx, tx, sy, ty;
        env_st(x.v, y.v, z.v, &s, &t);
        env_st(x.v + x.dx, y.v + y.dx, z.v + z.dx, &sx, &tx);
        env_st(x.v + x.dy, y.v + y.dy, z.v + z.dy, &sy, &ty);
        const float w0 = (float)T.w[0], h0 = (float)T.h[0];
        tex_filtered(T, s, t, env_wrap_ds(sx - s) * w0, (tx - t) * h0, env_wrap_ds(sy - s) * w0, (ty - t) * h0,
                     width, TW_PERIODIC, TW_CLAMP, first, nc, res);
    } else {
        raise_status(st, ST_ARRAY_BOUNDS);
    }
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) std2(L, r, c, d2c(res[c]));
}

// setmessage / getmessage between the layers of one point
// (src/liboslexec/opmessage.cpp:19-138): a message name has one state word
// per point (0 unset, 1 + type id once set, kMsgQueried after a strict query
// that found nothing) and one store per type it is used with. Setting a
// message twice, setting it after a failed strict query, or reading it as
// another type is an error (status bit) that leaves the values unchanged.
// Stored values carry no derivatives; a found message zeroes the
// destination's.
static __device__ void h_setmessage(const Lane& L, const uint32_t* a, uint32_t* st) {
    const uint32_t state = a[0], store = a[1], src = a[2];
    const int nw = (int)(a[3] & 0xFFFFu);
    if (ldw(L, state, 0) != 0u) {
        raise_status(st, ST_MESSAGE);
        return;
    }
    stw(L, state, 0, 1u + (a[3] >> 16));
    OSLG_SPEC_UNROLL
    for (int i = 0; i < nw; ++i) stw(L, store, i, ldw(L, src, i));
}
static __device__ void h_getmessage(const Lane& L, const uint32_t* a, uint32_t* st) {
    const uint32_t state = a[1], store = a[2], dst = a[3];
    const int nw = (int)(a[4] & 0xFFFFu);
    const uint32_t tid = (a[4] >> 16) & 0x7FFFu;
    const uint32_t s = ldw(L, state, 0);
    uint32_t found = 0u;
    if (s == 0u) {
        if (a[4] >> 31) stw(L, state, 0, kMsgQueried);
    } else if (s != kMsgQueried) {
        if (s != 1u + tid) {
            raise_status(st, ST_MESSAGE);
        } else {
            OSLG_SPEC_UNROLL
            for (int i = 0; i < nw; ++i) stw(L, dst, i, ldw(L, store, i));
            if (ader(dst)) {
                OSLG_SPEC_UNROLL
                for (int i = nw; i < 3 * nw; ++i) stw(L, dst, i, 0u);
            }
            found = 1u;
        }
    }
    stw(L, a[0], 0, found);
}

// blackbody (src/liboslexec/opcolor_impl.h:510-575): a2 = constant table
// of N RGB^(1/5) entries, then the XYZ->RGB matrix and the CIE table; a3 = N
static __device__ void h_blackbody(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0];
    const float T = ldf(L, a[1], 0, 0);
    const uint32_t tb = a[2];
    const int N = (int)a[3];
    float rgb[3];
    if (T < 800.0f) {
        rgb[0] = 1.0e-6f; rgb[1] = 0.0f; rgb[2] = 0.0f;
    } else if (T < 12000.0f) {
        const float ic = (float)cbrt((double)((T - 800.0f) / 2.0f));
        const float t = ic * ic;
        int ti = (int)t;
        if (ti > N - 2) ti = N - 2;
        const float rem = t - (float)ti;
        for (int c = 0; c < 3; ++c) {
            const float x0 = __uint_as_float(ldw(L, tb, ti * 3 + c)), x1 = __uint_as_float(ldw(L, tb, ti * 3 + 3 + c));
            const float v = x0 * (1.0f - rem) + x1 * rem;
            const float v2 = v * v, v4 = v2 * v2;
            rgb[c] = v4 * v;
        }
    } else {
        float X = 0.0f, Y = 0.0f, Z = 0.0f;
        const float dlambda = (float)(5.0f * 1e-9);
        const int cie = N * 3 + 9;
        for (int i = 0; i < 81; ++i) {
            const float lambda = 380.0f + 5.0f * (float)i;
            const float wlm = lambda * 1e-9f;
            const float wlm2 = wlm * wlm, wlm4 = wlm2 * wlm2, wlm5 = wlm4 * wlm;
            const float inv5 = 1.0f / wlm5;
            const float e = (float)expm1((double)(1.4388e-2f / (wlm * T)));
            const float Me = ((3.74183e-16f * inv5) / e) * dlambda;
            X += Me * __uint_as_float(ldw(L, tb, cie + i * 3 + 0));
            Y += Me * __uint_as_float(ldw(L, tb, cie + i * 3 + 1));
            Z += Me * __uint_as_float(ldw(L, tb, cie + i * 3 + 2));
        }
        const int mx = N * 3;
        for (int c = 0; c < 3; ++c) {
            const float v = X * __uint_as_float(ldw(L, tb, mx + c)) + Y * __uint_as_float(ldw(L, tb, mx + 3 + c))
                          + Z * __uint_as_float(ldw(L, tb, mx + 6 + c));
            rgb[c] = v < 0.0f ? 0.0f : v;
        }
    }
    for (int c = 0; c < 3; ++c) stval(L, r, c, rgb[c]);
}

// ---- noise ---------------------------------------------------------------------
// gabor / pgabor: a = r, S, T, kind word, anisotropic, direction,
// bandwidth; b (the carrier op that follows) = impulses, do_filter,
// Speriod, Tperiod. 1-D and 2-D positions slice to 3-D and the 4-D forms
// drop t (src/liboslexec/opnoise.cpp:484-640).
static __device__ void h_gabor(const Lane& L, const uint32_t* a, const uint32_t* b) {
    const uint32_t r = a[0], S = a[1], kw = a[3];
    const bool periodic = (kw & 16u) != 0;
    const int dims = (int)((kw >> 5) & 7u);
    const int nc = (kw & 256u) ? 3 : 1;
    const int ns = anc(S);
    GOpts o;
    o.anisotropic = ldi(L, a[4], 0);
    o.direction = v3(ldf(L, a[5], 0, 0), ldf(L, a[5], 1, 0), ldf(L, a[5], 2, 0));
    o.bandwidth = ldf(L, a[6], 0, 0);
    o.impulses = ldf(L, b[0], 0, 0);
    o.do_filter = ldi(L, b[1], 0);
    DV3 X;
    X.v = X.dx = X.dy = v3(0.0f, 0.0f, 0.0f);
    {
        const D2 x0 = ldd(L, S, 0);
        X.v.x = x0.v; X.dx.x = x0.dx; X.dy.x = x0.dy;
        if (ns == 3) {
            const D2 x1 = ldd(L, S, 1), x2 = ldd(L, S, 2);
            X.v.y = x1.v; X.dx.y = x1.dx; X.dy.y = x1.dy;
            X.v.z = x2.v; X.dx.z = x2.dx; X.dy.z = x2.dy;
        } else if (dims == 2) {
            const D2 x1 = ldd(L, a[2], 0);
            X.v.y = x1.v; X.dx.y = x1.dx; X.dy.y = x1.dy;
        }
    }
    V3 period = v3(0.0f, 0.0f, 0.0f);
    if (periodic) {
        if (ns == 3) {
            period = v3(ldf(L, b[2], 0, 0), ldf(L, b[2], 1, 0), ldf(L, b[2], 2, 0));
        } else {
            period.x = ldf(L, b[2], 0, 0);
            if (dims == 2) period.y = ldf(L, b[3], 0, 0);
        }
    }
    D2 res[3];
    gabor_eval(o, X, periodic, period, nc, res);
    const int rn = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < rn; ++c) {
        const D2 v = res[nc == 1 ? 0 : c];
        stf(L, r, c, v.v);
        if (ader(r)) {
            stf(L, r, rn + c, v.dx);
            stf(L, r, 2 * rn + c, v.dy);
        }
    }
}

// Operands of one noise evaluation, by value: the inputs as Dual2 (zero
// derivatives when the op takes none), the raw period operands, results.
struct NoiseIO {
    D2 xs[4];
    float per[4];
    float res[3], rdx[3], rdy[3];
};

// The evaluation proper. A kernel specialized to many programs (the
// persistent batch kernels) compiles it once, out of line, for every noise
// kind at run time; elsewhere it is inlined and the kind word is a constant.
#ifdef OSLG_SPEC_BATCH
static __device__ __noinline__
#else
static __device__ __forceinline__
#endif
void noise_eval(uint32_t kw, int ns, bool has_t, NoiseIO& io) {
    int kind = (int)(kw & 15u);
    bool periodic = (kw & 16u) != 0;
    int dims = (int)((kw >> 5) & 7u);
    bool vec = (kw & 256u) != 0;
    bool derivs = (kw & 512u) != 0;
    int nc = vec ? 3 : 1;
    float* res = io.res;
    float* rdx = io.rdx;
    float* rdy = io.rdy;
    OSLG_SPEC_UNROLL
    for (int c = 0; c < 3; ++c) rdx[c] = rdy[c] = 0.0f;
    Hasher H;
    H.periodic = periodic;
    H.px = H.py = H.pz = H.pw = 1;
    if (periodic) {
        if (ns == 3) {
            H.px = period_of(io.per[0]); H.py = period_of(io.per[1]); H.pz = period_of(io.per[2]);
            if (dims == 4) H.pw = period_of(io.per[3]);
        } else {
            H.px = period_of(io.per[0]);
            if (dims == 2) H.py = period_of(io.per[1]);
        }
    }
    (void)has_t;
    if (kind == NK_CELL || kind == NK_HASH) {
        float xs[4];
        OSLG_SPEC_UNROLL
        for (int i = 0; i < 4; ++i) xs[i] = io.xs[i].v;
        if (periodic) {
            if (ns == 3) {
                xs[0] = pwrap(xs[0], io.per[0]); xs[1] = pwrap(xs[1], io.per[1]);
                xs[2] = pwrap(xs[2], io.per[2]);
                if (dims == 4) xs[3] = pwrap(xs[3], io.per[3]);
            } else {
                xs[0] = pwrap(xs[0], io.per[0]);
                if (dims == 2) xs[1] = pwrap(xs[1], io.per[1]);
            }
        }
        intnoise(kind == NK_CELL, dims, xs, nc, res);
    } else if (kind == NK_PERLIN || kind == NK_UPERLIN) {
        if (derivs) {
            const D2* xs = io.xs;
            D2 o[3];
            if (vec) {
                switch (dims) {
                case 1: perlin1<D2, 3>(H, xs[0], o); break;
                case 2: perlin2<D2, 3>(H, xs[0], xs[1], o); break;
                case 3: perlin3<D2, 3>(H, xs[0], xs[1], xs[2], o); break;
                default: perlin4<D2, 3>(H, xs[0], xs[1], xs[2], xs[3], o); break;
                }
            } else {
                switch (dims) {
                case 1: perlin1<D2, 1>(H, xs[0], o); break;
                case 2: perlin2<D2, 1>(H, xs[0], xs[1], o); break;
                case 3: perlin3<D2, 1>(H, xs[0], xs[1], xs[2], o); break;
                default: perlin4<D2, 1>(H, xs[0], xs[1], xs[2], xs[3], o); break;
                }
            }
            OSLG_SPEC_UNROLL
            for (int c = 0; c < nc; ++c) {
                if (kind == NK_UPERLIN) o[c] = (o[c] + 1.0f) * 0.5f;
                res[c] = o[c].v; rdx[c] = o[c].dx; rdy[c] = o[c].dy;
            }
        } else {
            float xs[4];
            OSLG_SPEC_UNROLL
            for (int i = 0; i < 4; ++i) xs[i] = io.xs[i].v;
            if (vec) {
                switch (dims) {
                case 1: perlin1<float, 3>(H, xs[0], res); break;
                case 2: perlin2<float, 3>(H, xs[0], xs[1], res); break;
                case 3: perlin3<float, 3>(H, xs[0], xs[1], xs[2], res); break;
                default: perlin4<float, 3>(H, xs[0], xs[1], xs[2], xs[3], res); break;
                }
            } else {
                switch (dims) {
                case 1: perlin1<float, 1>(H, xs[0], res); break;
                case 2: perlin2<float, 1>(H, xs[0], xs[1], res); break;
                case 3: perlin3<float, 1>(H, xs[0], xs[1], xs[2], res); break;
                default: perlin4<float, 1>(H, xs[0], xs[1], xs[2], xs[3], res); break;
                }
            }
            if (kind == NK_UPERLIN)
                OSLG_SPEC_UNROLL
                for (int c = 0; c < nc; ++c) res[c] = 0.5f * (res[c] + 1.0f);
        }
    } else if (kind == NK_SIMPLEX || kind == NK_USIMPLEX) {
        const D2* xs = io.xs;
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) {
            float g[4] = { 0, 0, 0, 0 };
            float v;
            switch (dims) {
            case 1: v = simplex1(xs[0].v, c, derivs ? &g[0] : nullptr); break;
            case 2: v = simplex2(xs[0].v, xs[1].v, c, derivs ? &g[0] : nullptr, &g[1]); break;
            case 3: v = simplex3(xs[0].v, xs[1].v, xs[2].v, c, derivs ? &g[0] : nullptr, &g[1], &g[2]); break;
            default: v = simplex4(xs[0].v, xs[1].v, xs[2].v, xs[3].v, c, derivs ? g : nullptr); break;
            }
            D2 o = d2c(v);
            if (derivs) {
                float dx = g[0] * xs[0].dx, dy = g[0] * xs[0].dy;
                for (int i = 1; i < dims; ++i) { dx = dx + g[i] * xs[i].dx; dy = dy + g[i] * xs[i].dy; }
                o = d2(v, dx, dy);
            }
            if (kind == NK_USIMPLEX) o = (o + 1.0f) * 0.5f;
            res[c] = o.v; rdx[c] = o.dx; rdy[c] = o.dy;
        }
    } else if (kind == NK_NULL || kind == NK_UNULL) {
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) res[c] = kind == NK_UNULL ? 0.5f : 0.0f;
    } else {
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) res[c] = 0.0f;
    }
}

static __device__ void h_noise(const Lane& L, const uint32_t* a) {
    const uint32_t r = a[0], S = a[1], T = a[2], kw = a[3];
    const bool periodic = (kw & 16u) != 0;
    const int dims = (int)((kw >> 5) & 7u);
    const bool vec = (kw & 256u) != 0;
    const bool derivs = (kw & 512u) != 0;
    const int ns = anc(S);
    const int nc = vec ? 3 : 1;
    NoiseIO io;
    OSLG_SPEC_UNROLL
    for (int i = 0; i < 4; ++i) { io.xs[i] = d2c(0.0f); io.per[i] = 1.0f; }
    OSLG_SPEC_UNROLL
    for (int i = 0; i < ns; ++i) io.xs[i] = derivs ? ldd(L, S, i) : d2c(ldf(L, S, i, 0));
    if (T != kNoArg) io.xs[ns] = derivs ? ldd(L, T, 0) : d2c(ldf(L, T, 0, 0));
    if (periodic) {
        const uint32_t SP = a[4], TP = a[5];
        if (ns == 3) {
            io.per[0] = ldf(L, SP, 0, 0); io.per[1] = ldf(L, SP, 1, 0); io.per[2] = ldf(L, SP, 2, 0);
            if (dims == 4) io.per[3] = ldf(L, TP, 0, 0);
        } else {
            io.per[0] = ldf(L, SP, 0, 0);
            if (dims == 2) io.per[1] = ldf(L, TP, 0, 0);
        }
    }
    noise_eval(kw, ns, T != kNoArg, io);
    // float result from triple request or vice versa is handled by lowering;
    // scalar noise into a triple symbol broadcasts
    int rn = anc(r);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < rn; ++c) {
        int sc = nc == 1 ? 0 : c;
        stf(L, r, c, io.res[sc]);
        if (ader(r)) {
            stf(L, r, rn + c, io.rdx[sc]);
            stf(L, r, 2 * rn + c, io.rdy[sc]);
        }
    }
}

static __device__ void h_hash(const Lane& L, const uint32_t* a) {
    uint32_t x = a[1], y = a[2];
    uint32_t h;
    uint32_t tx = atc(x);
    if (tx == TC_INT) h = inthash1(ldw(L, x, 0));
    else if (tx == TC_STRING) h = ldw(L, x, 0);
    else if (tx == TC_TRIPLE) {
        if (y == kNoArg) h = inthash3(ldw(L, x, 0), ldw(L, x, 1), ldw(L, x, 2));
        else h = inthash4(ldw(L, x, 0), ldw(L, x, 1), ldw(L, x, 2), __float_as_uint(ldf(L, y, 0, 0)));
    } else {
        if (y == kNoArg) h = inthash1(__float_as_uint(ldf(L, x, 0, 0)));
        else h = inthash2(__float_as_uint(ldf(L, x, 0, 0)), __float_as_uint(ldf(L, y, 0, 0)));
    }
    stw(L, a[0], 0, h);
}

// ---- globals / arenas -------------------------------------------------------------
__device__ __forceinline__ const oslg_field& gfield(const oslg_shaderglobals& G, int id) {
    switch (id) {
    case G_P: return G.P; case G_DPDX: return G.dPdx; case G_DPDY: return G.dPdy; case G_DPDZ: return G.dPdz;
    case G_I: return G.I; case G_DIDX: return G.dIdx; case G_DIDY: return G.dIdy;
    case G_N: return G.N; case G_NG: return G.Ng;
    case G_U: return G.u; case G_DUDX: return G.dudx; case G_DUDY: return G.dudy;
    case G_V: return G.v; case G_DVDX: return G.dvdx; case G_DVDY: return G.dvdy;
    case G_DPDU: return G.dPdu; case G_DPDV: return G.dPdv;
    case G_TIME: return G.time; case G_DTIME: return G.dtime; case G_DPDTIME: return G.dPdtime;
    case G_PS: return G.Ps; case G_DPSDX: return G.dPsdx; case G_DPSDY: return G.dPsdy;
    case G_FLIPHANDEDNESS: return G.flipHandedness; case G_BACKFACING: return G.backfacing;
    default: return G.surfacearea;
    }
}
__device__ __forceinline__ float fld(const oslg_field& f, int c, int64_t pt) {
    return f.data ? __ldg(f.data + c * f.plane_stride + pt) : f.value[c];
}
// an int flag field: int32 per point, or value[0] != 0 for all
__device__ __forceinline__ bool gflag(const oslg_field& f, int64_t pt) {
    return f.data ? __ldg(reinterpret_cast<const int*>(f.data) + pt) != 0 : f.value[0] != 0.0f;
}

static __device__ void h_load_global(const Lane& L, const uint32_t* a, const oslg_shaderglobals& G) {
    uint32_t r = a[0];
    int id = (int)a[1];
    if (global_is_int((uint32_t)id)) {  // flipHandedness, backfacing: 0 or 1
        stw(L, r, 0, gflag(gfield(G, id), L.pt) ? 1u : 0u);
        return;
    }
    int nc = anc(r);
    const oslg_field& f = gfield(G, id);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) stf(L, r, c, fld(f, c, L.pt));
    if (ader(r)) {
        int dxid = -1, dyid = -1;
        if (id == G_P) { dxid = G_DPDX; dyid = G_DPDY; }
        else if (id == G_I) { dxid = G_DIDX; dyid = G_DIDY; }
        else if (id == G_U) { dxid = G_DUDX; dyid = G_DUDY; }
        else if (id == G_V) { dxid = G_DVDX; dyid = G_DVDY; }
        else if (id == G_PS) { dxid = G_DPSDX; dyid = G_DPSDY; }
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) {
            stf(L, r, nc + c, dxid >= 0 ? fld(gfield(G, dxid), c, L.pt) : 0.0f);
            stf(L, r, 2 * nc + c, dyid >= 0 ? fld(gfield(G, dyid), c, L.pt) : 0.0f);
        }
    }
}

static __device__ void h_calcnormal(const Lane& L, const uint32_t* a, const oslg_shaderglobals& G) {
    const uint32_t r = a[0], p = a[1];
    const V3 dx = v3(ldf(L, p, 0, 1), ldf(L, p, 1, 1), ldf(L, p, 2, 1));
    const V3 dy = v3(ldf(L, p, 0, 2), ldf(L, p, 1, 2), ldf(L, p, 2, 2));
    const V3 n = gflag(G.flipHandedness, L.pt) ? vcross(dy, dx) : vcross(dx, dy);
    stval(L, r, 0, n.x);
    stval(L, r, 1, n.y);
    stval(L, r, 2, n.z);
}

// a3 bit 1: the record carries [val][dx][dy]; a destination with
// derivatives reads them, or gets zeros when the record has none
static __device__ void h_load_userdata(const Lane& L, const uint32_t* a, char* base) {
    uint32_t r = a[0];
    int nc = anc(r);
    const char* p = base + (int64_t)a[1] + urec(L) * (int64_t)(int32_t)a[2];
    const bool src_d = (a[3] & 2u) != 0u;
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
    for (int i = 0; i < nc; ++i) stw(L, r, i, q[i]);
    if (ader(r))
        for (int i = nc; i < 3 * nc; ++i) stw(L, r, i, src_d ? q[i] : 0u);
}

static __device__ void h_store_output(const Lane& L, const uint32_t* a, char* base) {
    uint32_t s = a[0];
    int nc = anc(s);
    uint32_t flags = a[3];
    int elems = (int)a[4];
    if (elems < 1) elems = 1;
    char* p = base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2];
    int total = nc * elems;
    int nd = (flags & 1u) ? 3 : 1;
    OSLG_SPEC_UNROLL
    for (int d = 0; d < nd; ++d)
        OSLG_SPEC_UNROLL
        for (int i = 0; i < total; ++i) {
            uint32_t w;
            if (d > 0 && !ader(s)) w = 0u;
            else if (flags & 2u) w = atc(s) == TC_INT ? ldw(L, s, i) : (uint32_t)ldi(L, s, i);  // int arrays: element i
            else w = ldw(L, s, d * total + i);
            if (!(flags & 2u) && atc(s) == TC_INT) w = __float_as_uint((float)(int)w);
            ostore32(reinterpret_cast<uint32_t*>(p) + d * total + i, w);
        }
}

static __device__ void h_compref(const Lane& L, const uint32_t* a, uint32_t* st) {
    int i = ldi(L, a[2], 0);
    if (i < 0 || i > 2) { raise_status(st, ST_ARRAY_BOUNDS); i = i < 0 ? 0 : 2; }
    std2(L, a[0], 0, ader(a[1]) ? ldd(L, a[1], i) : d2c(ldf(L, a[1], i, 0)));
}
static __device__ void h_compassign(const Lane& L, const uint32_t* a, uint32_t* st) {
    int i = ldi(L, a[1], 0);
    if (i < 0 || i > 2) { raise_status(st, ST_ARRAY_BOUNDS); i = i < 0 ? 0 : 2; }
    std2(L, a[0], i, ldd(L, a[2], 0));
}
static __device__ void h_construct3(const Lane& L, const uint32_t* a) {
    for (int c = 0; c < 3; ++c) std2(L, a[0], c, ldd(L, a[1 + c], 0));
}
static __device__ void h_aref(const Lane& L, const uint32_t* a, uint32_t* st) {
    uint32_t r = a[0], arr = a[1];
    int alen = (int)a[3];
    int i = ldi(L, a[2], 0);
    if (i < 0 || i >= alen) { raise_status(st, ST_ARRAY_BOUNDS); i = i < 0 ? 0 : alen - 1; }
    int nc = anc(arr);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        uint32_t w = ldw(L, arr, i * nc + c);
        if (atc(r) == TC_INT || atc(r) == TC_STRING || atc(r) == TC_CLOSURE) { stw(L, r, c, w); continue; }
        float v = atc(arr) == TC_INT ? (float)(int)w : __uint_as_float(w);
        stf(L, r, c, v);
        if (ader(r)) {
            float dx = 0.0f, dy = 0.0f;
            if (ader(arr)) {
                dx = __uint_as_float(ldw(L, arr, alen * nc + i * nc + c));
                dy = __uint_as_float(ldw(L, arr, 2 * alen * nc + i * nc + c));
            }
            stf(L, r, nc + c, dx);
            stf(L, r, 2 * nc + c, dy);
        }
    }
}
static __device__ void h_aassign(const Lane& L, const uint32_t* a, uint32_t* st) {
    uint32_t arr = a[0], v = a[2];
    int alen = (int)a[3];
    int i = ldi(L, a[1], 0);
    if (i < 0 || i >= alen) { raise_status(st, ST_ARRAY_BOUNDS); i = i < 0 ? 0 : alen - 1; }
    int nc = anc(arr);
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        int vc = anc(v) == 1 ? 0 : c;
        if (atc(arr) == TC_INT || atc(arr) == TC_STRING || atc(arr) == TC_CLOSURE) {
            stw(L, arr, i * nc + c, atc(arr) == TC_INT ? (uint32_t)ldi(L, v, vc) : ldw(L, v, vc));
            continue;
        }
        stf(L, arr, i * nc + c, ldf(L, v, vc, 0));
        if (ader(arr)) {
            stf(L, arr, alen * nc + i * nc + c, ldf(L, v, vc, 1));
            stf(L, arr, 2 * alen * nc + i * nc + c, ldf(L, v, vc, 2));
        }
    }
}

// ---- closures (reference closure tree, node pool in the heap) -------------------------
struct ClosurePools {
    uint32_t base, max_nodes;
    uint32_t nf = kRecordFloats;  // floats per node (ProgramHeader::node_floats)
};
// closure node pool access (slots at and above the program's closure base)
#ifdef OSLG_SPEC
__device__ __forceinline__ float hget(const Lane& L, uint32_t slot) { return L.cheap[(size_t)(slot - L.cbase) * L.chs + L.cli]; }
__device__ __forceinline__ void hset(const Lane& L, uint32_t slot, float v) { L.cheap[(size_t)(slot - L.cbase) * L.chs + L.cli] = v; }
#else
__device__ __forceinline__ float hget(const Lane& L, uint32_t slot) { return L.heap[(size_t)slot * L.hs + L.li]; }
__device__ __forceinline__ void hset(const Lane& L, uint32_t slot, float v) { L.heap[(size_t)slot * L.hs + L.li] = v; }
#endif
__device__ __forceinline__ uint32_t hgetu(const Lane& L, uint32_t slot) { return __float_as_uint(hget(L, slot)); }
__device__ __forceinline__ void hsetu(const Lane& L, uint32_t slot, uint32_t v) { hset(L, slot, __uint_as_float(v)); }
// symbol-heap words (static closure nodes live among the symbols: registers
// in a specialized kernel)
__device__ __forceinline__ float sget(const Lane& L, uint32_t slot) { return L.heap[(size_t)slot * L.hs + L.li]; }
__device__ __forceinline__ void sset(const Lane& L, uint32_t slot, float v) { L.heap[(size_t)slot * L.hs + L.li] = v; }
__device__ __forceinline__ uint32_t sgetu(const Lane& L, uint32_t slot) { return __float_as_uint(sget(L, slot)); }
__device__ __forceinline__ void ssetu(const Lane& L, uint32_t slot, uint32_t v) { sset(L, slot, __uint_as_float(v)); }
// Where a lobe's node parameters are read: the closure node pool (trees
// built at run time) or the symbol heap (static closures).
struct PoolNodes {
    static __device__ __forceinline__ float f(const Lane& L, uint32_t s) { return hget(L, s); }
    static __device__ __forceinline__ uint32_t u(const Lane& L, uint32_t s) { return hgetu(L, s); }
};
struct SymNodes {
    static __device__ __forceinline__ float f(const Lane& L, uint32_t s) { return sget(L, s); }
    static __device__ __forceinline__ uint32_t u(const Lane& L, uint32_t s) { return sgetu(L, s); }
};
__device__ __forceinline__ uint32_t node_slot(const ClosurePools& P, uint32_t node) {
    return P.base + 1 + node * P.nf;
}
// returns node index + 1, or 0 when the pool is full
__device__ __forceinline__ uint32_t cl_alloc(const Lane& L, const ClosurePools& P, uint32_t* st) {
    uint32_t n = hgetu(L, P.base);
    if (n >= P.max_nodes) { raise_status(st, ST_CLOSURE_OVERFLOW); return 0u; }
    hsetu(L, P.base, n + 1);
    return n + 1;
}

// A component node [id][w.rgb][parameter words] at slot ns: the closure
// op's parameters in order, int and string operands as their words, floats
// as values, zero-padded to kRecordParams words, or to kClosureParamFloats
// when more are filled (the lowering sizes every node for what its closure
// op fills).
template <class NODES>
__device__ __forceinline__ void closure_fill(const Lane& L, uint32_t ns, const uint32_t* a, const uint32_t* extra,
                                             const float* w) {
    auto setu = [&](uint32_t s, uint32_t v) {
        if constexpr (std::is_same<NODES, SymNodes>::value) ssetu(L, s, v);
        else hsetu(L, s, v);
    };
    setu(ns, a[1]);
    for (int c = 0; c < 3; ++c) setu(ns + 1 + c, __float_as_uint(w[c]));
    uint32_t params[11];
    int np = 0;
    for (int i = 3; i < 7; ++i) params[np++] = a[i];
    if (extra)
        for (int i = 0; i < 7; ++i) params[np++] = extra[i];
    int k = 0;
    // fixed trip counts with early exits (a specialized kernel unrolls them
    // into constant operand indices)
    OSLG_SPEC_UNROLL
    for (int i = 0; i < 11; ++i) {
        if (i >= np || k >= kClosureParamFloats) break;
        uint32_t p = params[i];
        if (p == kNoArg) break;
        int nc = anc(p);
        uint32_t t = atc(p);
        OSLG_SPEC_UNROLL
        for (int c = 0; c < 16; ++c) {
            if (c >= nc || k >= kClosureParamFloats) break;
            setu(ns + 4 + k++, (t == TC_INT || t == TC_STRING || t == TC_CLOSURE) ? ldw(L, p, c)
                                                                               : __float_as_uint(ldf(L, p, c, 0)));
        }
    }
    const int kpad = k <= kRecordParams ? kRecordParams : kClosureParamFloats;
    OSLG_SPEC_UNROLL
    for (int j = 0; j < kClosureParamFloats; ++j)
        if (j >= k && j < kpad) setu(ns + 4 + j, 0u);
}

// osl_allocate_(weighted_)closure_component (opclosure.cpp:83-117)
static __device__ void h_closure(const Lane& L, const uint32_t* a, const uint32_t* extra, const ClosurePools& P,
                          uint32_t* st) {
    float w[3] = { 1.0f, 1.0f, 1.0f };
    if (a[2] != kNoArg) {
        for (int c = 0; c < 3; ++c) w[c] = ldf(L, a[2], c, 0);
        if (w[0] == 0.0f && w[1] == 0.0f && w[2] == 0.0f) { stw(L, a[0], 0, 0u); return; }
    }
    uint32_t h = cl_alloc(L, P, st);
    if (!h) { stw(L, a[0], 0, 0u); return; }
    closure_fill<PoolNodes>(L, node_slot(P, h - 1), a, extra, w);
    stw(L, a[0], 0, h);
}

// The static form: the node sits at the symbol-heap slot of operand a0; a
// zero weight marks it absent (the reference returns a null closure).
static __device__ void h_closure_node(const Lane& L, const uint32_t* a, const uint32_t* extra) {
    const uint32_t ns = a[0] & kArgOffsetMask;
    float w[3] = { 1.0f, 1.0f, 1.0f };
    if (a[2] != kNoArg) {
        for (int c = 0; c < 3; ++c) w[c] = ldf(L, a[2], c, 0);
        if (w[0] == 0.0f && w[1] == 0.0f && w[2] == 0.0f) { ssetu(L, ns, (uint32_t)kClosureAbsent); return; }
    }
    closure_fill<SymNodes>(L, ns, a, extra, w);
}

// osl_mul_closure_color / osl_mul_closure_float (opclosure.cpp:35-80)
static __device__ void h_closure_mul(const Lane& L, const uint32_t* a, const ClosurePools& P, uint32_t* st) {
    uint32_t c = ldw(L, a[1], 0);
    float w[3] = { ldf(L, a[2], 0, 0), ldf(L, a[2], 1, 0), ldf(L, a[2], 2, 0) };
    if (c == 0u || (w[0] == 0.0f && w[1] == 0.0f && w[2] == 0.0f)) { stw(L, a[0], 0, 0u); return; }
    if (w[0] == 1.0f && w[1] == 1.0f && w[2] == 1.0f) { stw(L, a[0], 0, c); return; }
    uint32_t h = cl_alloc(L, P, st);
    if (!h) { stw(L, a[0], 0, 0u); return; }
    uint32_t ns = node_slot(P, h - 1);
    hsetu(L, ns, (uint32_t)kClosureMul);
    for (int k = 0; k < 3; ++k) hset(L, ns + 1 + k, w[k]);
    hsetu(L, ns + 4, c);
    stw(L, a[0], 0, h);
}

// osl_add_closure_closure (opclosure.cpp:15-33)
static __device__ void h_closure_add(const Lane& L, const uint32_t* a, const ClosurePools& P, uint32_t* st) {
    uint32_t x = ldw(L, a[1], 0), y = ldw(L, a[2], 0);
    if (x == 0u) { stw(L, a[0], 0, y); return; }
    if (y == 0u) { stw(L, a[0], 0, x); return; }
    uint32_t h = cl_alloc(L, P, st);
    if (!h) { stw(L, a[0], 0, 0u); return; }
    uint32_t ns = node_slot(P, h - 1);
    hsetu(L, ns, (uint32_t)kClosureAdd);
    hsetu(L, ns + 4, x);
    hsetu(L, ns + 5, y);
    stw(L, a[0], 0, h);
}

// testrender's non-recursive walk (shading.cpp:1450-1500): visits the
// components in order with the accumulated weight weight*comp.w.
// With LAYERS, a layer(top, base) component (MaterialX layering as testrender
// walks it, shading.cpp:1666-1681) continues into top with the layer's
// weight and pushes base with the walk weight times (1 - clamp(opacity of
// top)); `opacity(top, out)` gives that opacity.
struct NoOpacity {
    __device__ void operator()(uint32_t, float* o) const { o[0] = o[1] = o[2] = 0.0f; }
};
template <bool LAYERS = false, class F, class O = NoOpacity>
__device__ void closure_walk(const Lane& L, const ClosurePools& P, uint32_t root, uint32_t* st, F&& visit,
                             O&& opacity = O()) {
    uint32_t stack_node[OSLG_WALK_STACK];
    float stack_w[OSLG_WALK_STACK][3];
    int sp = 0;
    float w[3] = { 1.0f, 1.0f, 1.0f };
    uint32_t cur = root;
    int guard = 0;
    while (cur != 0u && cur <= P.max_nodes) {
        if (++guard > 4 * (int)P.max_nodes + 8) break;
        uint32_t ns = node_slot(P, cur - 1);
        int id = (int)hgetu(L, ns);
        if (id == kClosureMul) {
            for (int k = 0; k < 3; ++k) w[k] = w[k] * hget(L, ns + 1 + k);
            cur = hgetu(L, ns + 4);
        } else if (id == kClosureAdd) {
            if (sp < OSLG_WALK_STACK) {
                const uint32_t right = hgetu(L, ns + 5);
#ifdef OSLG_FIXED_INDEX
#pragma unroll
                for (int j = 0; j < OSLG_WALK_STACK; ++j)
                    if (j == sp) {
                        stack_node[j] = right;
                        for (int k = 0; k < 3; ++k) stack_w[j][k] = w[k];
                    }
#else
                stack_node[sp] = right;
                for (int k = 0; k < 3; ++k) stack_w[sp][k] = w[k];
#endif
                ++sp;
            } else {
                raise_status(st, ST_CLOSURE_OVERFLOW);
            }
            cur = hgetu(L, ns + 4);
        } else {
            float cw[3];
            for (int k = 0; k < 3; ++k) cw[k] = w[k] * hget(L, ns + 1 + k);
            cur = 0u;
            if (LAYERS && id == kIdMxLayer) {
                float op[3], bw[3];
                opacity(hgetu(L, ns + 4), op);
                for (int k = 0; k < 3; ++k) bw[k] = w[k] * (1.0f - bsdl_clamp(op[k], 0.0f, 1.0f));
                if (bw[0] != 0.0f || bw[1] != 0.0f || bw[2] != 0.0f) {
                    if (sp < OSLG_WALK_STACK) {
                        const uint32_t base = hgetu(L, ns + 5);
#ifdef OSLG_FIXED_INDEX
#pragma unroll
                        for (int j = 0; j < OSLG_WALK_STACK; ++j)
                            if (j == sp) {
                                stack_node[j] = base;
                                for (int k = 0; k < 3; ++k) stack_w[j][k] = bw[k];
                            }
#else
                        stack_node[sp] = base;
                        for (int k = 0; k < 3; ++k) stack_w[sp][k] = bw[k];
#endif
                        ++sp;
                    } else {
                        raise_status(st, ST_CLOSURE_OVERFLOW);
                    }
                }
                for (int k = 0; k < 3; ++k) w[k] = cw[k];
                cur = hgetu(L, ns + 4);
            } else {
                visit(id, cw, ns + 4);
            }
        }
        if (cur == 0u && sp > 0) {
            --sp;
#ifdef OSLG_FIXED_INDEX
#pragma unroll
            for (int j = 0; j < OSLG_WALK_STACK; ++j)
                if (j == sp) {
                    cur = stack_node[j];
                    for (int k = 0; k < 3; ++k) w[k] = stack_w[j][k];
                }
#else
            cur = stack_node[sp];
            for (int k = 0; k < 3; ++k) w[k] = stack_w[sp][k];
#endif
        }
    }
}

// Output record per point: [count][per component: id, w.rgb, the first
// kRecordParams parameter words]
static __device__ void h_store_closure(const Lane& L, const uint32_t* a, char* base, const ClosurePools& P, uint32_t* st) {
    uint32_t root = ldw(L, a[0], 0), maxc = a[3];
    uint32_t* o = reinterpret_cast<uint32_t*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    uint32_t n = 0;
    closure_walk(L, P, root, st, [&](int id, const float* cw, uint32_t params) {
        if (n >= maxc) return;
        uint32_t* q = o + 1 + n * kRecordFloats;
        ostore32(q, (uint32_t)id);
        for (int k = 0; k < 3; ++k) ostore32(q + 1 + k, __float_as_uint(cw[k]));
        for (int k = 0; k < kRecordParams; ++k) ostore32(q + 4 + k, hgetu(L, params + k));
        ++n;
    });
    ostore32(o, n);
}

// CompositeBSDF::prepare + eval (shading.h:322-374) over the lobes the walk
// finds: diffuse, and microfacet "ggx" reflection; other ids add nothing.
// The lobes testrender's process_closure builds from a closure tree
// (shading.cpp:1481-1530): emission accumulates Le; diffuse, oren_nayar and
// GGX microfacet (refract 0/1/2) become lobes in walk order. Lobe
// parameters stay in the heap (node params) and are read when used.
// Lobe kinds this build compiles (bit k: LobeKind k); a specialized kernel
// defines the kinds its program's closures make.
#ifndef OSLG_LOBE_KINDS
#define OSLG_LOBE_KINDS 0xFFu
#endif
__device__ __forceinline__ constexpr bool lobe_on(int k) { return ((OSLG_LOBE_KINDS) >> k) & 1u; }
// the lobe kind of a component (testrender's process_closure), -1 for none
template <class NODES>
__device__ __forceinline__ int lobe_kind_of(const Lane& L, int id, uint32_t params, uint32_t ggx) {
    int k = -1;
    if (id == kIdDiffuse) k = LK_DIFFUSE;
    else if (id == kIdOrenNayar) k = LK_OREN_NAYAR;
    else if (id == kIdMxOrenNayarDiffuse) k = LK_MX_OREN_NAYAR;
    else if (id == kIdMxSheen) k = LK_SHEEN;
    else if (id == kIdMxDielectric) k = LK_MX_DIELECTRIC;
    else if (id == kIdMicrofacet && lobe_on(LK_GGX) && NODES::u(L, params + 0) == ggx) {  // "ggx"
        const int r = (int)NODES::u(L, params + 10);
        if (r >= 0 && r <= 2) k = LK_GGX;
    }
    return k >= 0 && lobe_on(k) ? k : -1;
}
struct Lobes {
    int n;
    int kind[OSLG_LOBES_MAX];  // LobeKind (oslg_program.h), -1 no lobe
    float w[OSLG_LOBES_MAX][3];
    float pdf[OSLG_LOBES_MAX];
    uint32_t p[OSLG_LOBES_MAX];
    float Le[3];
    float path_rough;  // roughness of the incoming ray (BSDL regularization)
    bool backfacing;
};
// Loops over the lobe list: unrolled over the capacity (constant indices)
// in a fixed-index build, a plain loop over n otherwise.
// A lobe position with kind < 0 holds no lobe (static term tables keep
// one position per term).
#ifdef OSLG_FIXED_INDEX
#define OSLG_FOR_LOBES(i, B) _Pragma("unroll") for (int i = 0; i < OSLG_LOBES_MAX; ++i) if (i < (B).n && (B).kind[i] >= 0)
#else
#define OSLG_FOR_LOBES(i, B) for (int i = 0; i < (B).n; ++i) if ((B).kind[i] >= 0)
#endif
// process_closure's lobes (shading.cpp:1481-1530) from the components a walk
// visits: `walk(visit)` calls visit(id, weight, parameter slot) for each
// component in the walk's order.
template <class NODES, class W>
__device__ __forceinline__ void lobes_collect(const Lane& L, W&& walk, uint32_t ggx, Lobes& B, float path_rough,
                                              bool backfacing) {
    B.n = 0;
    B.Le[0] = B.Le[1] = B.Le[2] = 0.0f;
    B.path_rough = path_rough;
    B.backfacing = backfacing;
    walk([&](int id, const float* cw, uint32_t params) {
        if (id == kIdEmission) {
            for (int c = 0; c < 3; ++c) B.Le[c] = B.Le[c] + cw[c];
            return;
        }
        const int k = lobe_kind_of<NODES>(L, id, params, ggx);
        if (k < 0 || B.n >= OSLG_LOBES_MAX) return;
#ifdef OSLG_FIXED_INDEX
#pragma unroll
        for (int j = 0; j < OSLG_LOBES_MAX; ++j)
            if (j == B.n) {
                B.kind[j] = k;
                for (int c = 0; c < 3; ++c) B.w[j][c] = cw[c];
                B.p[j] = params;
            }
#else
        B.kind[B.n] = k;
        for (int c = 0; c < 3; ++c) B.w[B.n][c] = cw[c];
        B.p[B.n] = params;
#endif
        ++B.n;
    });
}
// The opacity of a layer's top (testrender's evaluate_layer_opacity,
// shading.cpp:1199-1281): its own walk, a nested layer continuing into its
// top and pushing its base with weight * w, a sheen component scaling the
// weight by w * (1 - E) with E the part of the light the sheen lets through,
// any other component opaque. The walk's last weight is the opacity.
__device__ __forceinline__ void layer_opacity(const Lane& L, const ClosurePools& P, uint32_t top, uint32_t* st, V3 wo,
                                              float path_rough, bool backfacing, float* out);
// the lobes of a tree in the node pool, visited by testrender's walk
__device__ __forceinline__ void lobes_build(const Lane& L, const ClosurePools& P, uint32_t root, uint32_t ggx,
                                            uint32_t* st, Lobes& B, float path_rough = 0.0f, bool backfacing = false,
                                            V3 wo = V3{ 0.0f, 0.0f, 1.0f }) {
    lobes_collect<PoolNodes>(
        L,
        [&](auto&& visit) {
            closure_walk<true>(L, P, root, st, visit, [&](uint32_t top, float* o) {
                layer_opacity(L, P, top, st, wo, path_rough, backfacing, o);
            });
        },
        ggx, B, path_rough, backfacing);
}
template <class NODES = PoolNodes>
__device__ __forceinline__ GGXLobe lobe_ggx(const Lane& L, uint32_t p) {
    GGXLobe g;
    const V3 N = v3(NODES::f(L, p + 1), NODES::f(L, p + 2), NODES::f(L, p + 3));
    const V3 U = v3(NODES::f(L, p + 4), NODES::f(L, p + 5), NODES::f(L, p + 6));
    g.tf = frame_from_normal_and_tangent(N, U);
    g.ax = NODES::f(L, p + 7);
    g.ay = NODES::f(L, p + 8);
    g.eta = NODES::f(L, p + 9);
    g.refract = (int)NODES::u(L, p + 10);
    return g;
}
// An int keyword parameter of a component (name hash, then the value) after
// its fixed parameters; dflt when absent. The scan stops at the first zero
// name word, which the zero padding of a node's unfilled words places
// inside the node.
template <class NODES>
__device__ __forceinline__ int closure_keyword_int(const Lane& L, uint32_t params, int first, uint32_t key, int dflt) {
    int v = dflt;
    bool done = false;
    OSLG_SPEC_UNROLL
    for (int k = first; k + 1 < kClosureParamFloats; k += 2) {
        if (done) continue;  // no read past the first zero name (a 16-float node ends there)
        const uint32_t w = NODES::u(L, params + k);
        if (w == 0u) {
            done = true;
            continue;
        }
        if (w == key) {
            v = (int)NODES::u(L, params + k + 1);
            done = true;
        }
    }
    return v;
}
template <class NODES = PoolNodes>
__device__ __forceinline__ SheenLobeDev lobe_sheen(const Lane& L, const Lobes& B, uint32_t p, V3 wo) {
    const float albedo[3] = { NODES::f(L, p + 3), NODES::f(L, p + 4), NODES::f(L, p + 5) };
    return sheen_make(v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2)), albedo, NODES::f(L, p + 6), wo, B.path_rough,
                      B.backfacing, closure_keyword_int<NODES>(L, p, 7, string_hash_const("mode"), 0));
}
// oren_nayar_diffuse_bsdf(N, albedo, roughness, "energy_compensation", int)
template <class NODES>
__device__ __forceinline__ BsdfSample lobe_mxon(const Lane& L, uint32_t p, V3 wo, V3 wi, bool sample, float rx,
                                                float ry) {
    const V3 N = v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2));
    const float albedo[3] = { NODES::f(L, p + 3), NODES::f(L, p + 4), NODES::f(L, p + 5) };
    const float rough = bsdl_clamp(NODES::f(L, p + 6), 0.0f, 1.0f);
    const bool energy = closure_keyword_int<NODES>(L, p, 7, string_hash_const("energy_compensation"), 0) != 0;
    const Frame f = bsdl_frame(bsdl_visible_normal(wo, N, N));
    const V3 wo_l = tolocal(f, wo);
    if (sample) {
        if (wo_l.z <= 0.0f) return bsdf_zero();
        BsdfSample s = on_mx_eval_local(rough, albedo, energy, wo_l, bsdl_sample_cos_hemisphere(rx, ry));
        s.wi = bsdl_world(f, s.wi);
        return s;
    }
    BsdfSample s = on_mx_eval_local(rough, albedo, energy, wo_l, tolocal(f, wi));
    s.wi = wi;
    return s;
}
// dielectric_bsdf(N, U, reflection_tint, transmission_tint, roughness_x,
// roughness_y, ior, distribution [, "absorption", color]): parameter words
// 0-15, then the keyword words 16-19 (absorption only when it comes first:
// its colour fills the four)
template <class NODES = PoolNodes>
__device__ __forceinline__ DielLobeDev lobe_diel(const Lane& L, uint32_t p, V3 wo, float path_rough, bool backfacing) {
    const float refl[3] = { NODES::f(L, p + 6), NODES::f(L, p + 7), NODES::f(L, p + 8) };
    const float refr[3] = { NODES::f(L, p + 9), NODES::f(L, p + 10), NODES::f(L, p + 11) };
    const bool ab = NODES::u(L, p + 16) == string_hash_const("absorption");
    const float absorption[3] = { ab ? NODES::f(L, p + 17) : 0.0f, ab ? NODES::f(L, p + 18) : 0.0f,
                                  ab ? NODES::f(L, p + 19) : 0.0f };
    return diel_make(v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2)),
                     v3(NODES::f(L, p + 3), NODES::f(L, p + 4), NODES::f(L, p + 5)), refl, refr, NODES::f(L, p + 12),
                     NODES::f(L, p + 13), NODES::f(L, p + 14), absorption, wo, path_rough, backfacing);
}
template <class NODES = PoolNodes>
__device__ __forceinline__ BsdfSample lobe_eval(const Lane& L, const Lobes& B, int i, V3 wo, V3 wi) {
    const uint32_t p = B.p[i];
    const int kind = B.kind[i];
    if (lobe_on(LK_SHEEN) && kind == LK_SHEEN) return sheen_eval(lobe_sheen<NODES>(L, B, p, wo), wo, wi);
    if (lobe_on(LK_DIFFUSE) && kind == LK_DIFFUSE) {
        BsdfSample s = diffuse_eval(v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2)), wi);
        s.wi = wi;
        return s;
    }
    if (lobe_on(LK_GGX) && kind == LK_GGX) return ggx_eval(lobe_ggx<NODES>(L, p), wo, wi);
    if (lobe_on(LK_MX_OREN_NAYAR) && kind == LK_MX_OREN_NAYAR)
        return lobe_mxon<NODES>(L, p, wo, wi, false, 0.0f, 0.0f);
    if (lobe_on(LK_MX_DIELECTRIC) && kind == LK_MX_DIELECTRIC)
        return diel_eval(lobe_diel<NODES>(L, p, wo, B.path_rough, B.backfacing), wo, wi);
    if (!lobe_on(LK_OREN_NAYAR)) return bsdf_zero();
    const V3 N = v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2));
    const Frame f = bsdl_frame(bsdl_visible_normal(wo, N, N));
    BsdfSample s = on_eval_local(bsdl_clamp(NODES::f(L, p + 3), 0.0f, 1.0f), tolocal(f, wo), tolocal(f, wi));
    s.wi = wi;
    return s;
}
template <class NODES = PoolNodes>
__device__ __forceinline__ BsdfSample lobe_sample(const Lane& L, const Lobes& B, int i, V3 wo, float rx, float ry,
                                                  float rz) {
    const uint32_t p = B.p[i];
    const int kind = B.kind[i];
    if (lobe_on(LK_SHEEN) && kind == LK_SHEEN) return sheen_sample(lobe_sheen<NODES>(L, B, p, wo), wo, rx, ry);
    if (lobe_on(LK_DIFFUSE) && kind == LK_DIFFUSE)
        return diffuse_sample(v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2)), rx, ry);
    if (lobe_on(LK_GGX) && kind == LK_GGX) return ggx_sample(lobe_ggx<NODES>(L, p), wo, rx, ry, rz);
    if (lobe_on(LK_MX_OREN_NAYAR) && kind == LK_MX_OREN_NAYAR) return lobe_mxon<NODES>(L, p, wo, wo, true, rx, ry);
    if (lobe_on(LK_MX_DIELECTRIC) && kind == LK_MX_DIELECTRIC)
        return diel_sample(lobe_diel<NODES>(L, p, wo, B.path_rough, B.backfacing), wo, rx, ry, rz);
    if (!lobe_on(LK_OREN_NAYAR)) return bsdf_zero();
    const V3 N = v3(NODES::f(L, p + 0), NODES::f(L, p + 1), NODES::f(L, p + 2));
    const Frame f = bsdl_frame(bsdl_visible_normal(wo, N, N));
    const V3 wo_l = tolocal(f, wo);
    if (wo_l.z <= 0.0f) return bsdf_zero();
    BsdfSample s = on_eval_local(bsdl_clamp(NODES::f(L, p + 3), 0.0f, 1.0f), wo_l, bsdl_sample_cos_hemisphere(rx, ry));
    s.wi = bsdl_world(f, s.wi);
    return s;
}
// CompositeBSDF::prepare (shading.h:322-350)
template <class NODES = PoolNodes>
__device__ __forceinline__ void lobes_prepare(const Lane& L, Lobes& B, V3 wo, const float* pw, bool absorb) {
    float total = 0.0f;
    OSLG_FOR_LOBES(i, B) {
        float alb[3] = { 1.0f, 1.0f, 1.0f };
        if (lobe_on(LK_GGX) && B.kind[i] == LK_GGX) {
            const uint32_t p = B.p[i];
            const GGXLobe g = lobe_ggx<NODES>(L, p);
            alb[0] = alb[1] = alb[2] = ggx_albedo(g, v3(NODES::f(L, p + 1), NODES::f(L, p + 2), NODES::f(L, p + 3)), wo);
        } else if (lobe_on(LK_SHEEN) && B.kind[i] == LK_SHEEN) {
            const SheenLobeDev sh = lobe_sheen<NODES>(L, B, B.p[i], wo);
            for (int c = 0; c < 3; ++c) alb[c] = sh.tint[c] * (1 - sh.emiss);
        } else if (lobe_on(LK_MX_OREN_NAYAR) && B.kind[i] == LK_MX_OREN_NAYAR) {
            // BSDL albedo_impl: the closure's albedo
            for (int c = 0; c < 3; ++c) alb[c] = NODES::f(L, B.p[i] + 3 + c);
        } else if (lobe_on(LK_MX_DIELECTRIC) && B.kind[i] == LK_MX_DIELECTRIC) {
            diel_albedo(lobe_diel<NODES>(L, B.p[i], wo, B.path_rough, B.backfacing), alb);
        }
        B.pdf[i] = (B.w[i][0] * (pw[0] * alb[0]) + B.w[i][1] * (pw[1] * alb[1]) + B.w[i][2] * (pw[2] * alb[2]))
                 / (pw[0] + pw[1] + pw[2]);
        total += B.pdf[i];
    }
    if ((!absorb && total > 0.0f) || total > 1.0f)
        OSLG_FOR_LOBES(i, B) B.pdf[i] /= total;
}
// CompositeBSDF::eval (shading.h:360-370)
template <class NODES = PoolNodes>
__device__ __forceinline__ BsdfSample lobes_eval(const Lane& L, const Lobes& B, V3 wo, V3 wi) {
    BsdfSample r = bsdf_zero();
    OSLG_FOR_LOBES(i, B) {
        BsdfSample b = lobe_eval<NODES>(L, B, i, wo, wi);
        for (int c = 0; c < 3; ++c) b.w[c] *= B.w[i][c];
        mis_update_eval(r.w, &r.pdf, b.w, b.pdf, B.pdf[i]);
        r.roughness += b.roughness * B.pdf[i];
    }
    return r;
}
// CompositeBSDF::sample (shading.h:372-398)
template <class NODES = PoolNodes>
__device__ __forceinline__ BsdfSample lobes_sample(const Lane& L, const Lobes& B, V3 wo, float rx, float ry, float rz) {
    float accum = 0.0f;
    OSLG_FOR_LOBES(i, B) {
        if (rx < (B.pdf[i] + accum)) {
            rx = (rx - accum) / B.pdf[i];
            rx = fminf(rx, 0.99999994f);
            BsdfSample s = lobe_sample<NODES>(L, B, i, wo, rx, ry, rz);
            const float inv = 1 / B.pdf[i];
            for (int c = 0; c < 3; ++c) s.w[c] *= B.w[i][c] * inv;
            s.pdf *= B.pdf[i];
            if (s.pdf == 0.0f) return bsdf_zero();
            OSLG_FOR_LOBES(j, B) {
                if (i != j) {
                    BsdfSample b = lobe_eval<NODES>(L, B, j, wo, s.wi);
                    for (int c = 0; c < 3; ++c) b.w[c] *= B.w[j][c];
                    mis_update_eval(s.w, &s.pdf, b.w, b.pdf, B.pdf[j]);
                }
            }
            return s;
        }
        accum += B.pdf[i];
    }
    return bsdf_zero();
}

__device__ __forceinline__ void layer_opacity(const Lane& L, const ClosurePools& P, uint32_t top, uint32_t* st, V3 wo,
                                              float path_rough, bool backfacing, float* out) {
    float w[3] = { 1.0f, 1.0f, 1.0f };
    if (top == 0u) {  // a null top lets everything through
        out[0] = out[1] = out[2] = 0.0f;
        return;
    }
    uint32_t stack_node[kClosureWalkStack];
    float stack_w[kClosureWalkStack][3];
    int sp = 0, guard = 0;
    uint32_t cur = top;
    auto push = [&](uint32_t node, const float* pw) {
        if (sp >= kClosureWalkStack) {
            raise_status(st, ST_CLOSURE_OVERFLOW);
            return;
        }
        stack_node[sp] = node;
        for (int k = 0; k < 3; ++k) stack_w[sp][k] = pw[k];
        ++sp;
    };
    while (cur != 0u && cur <= P.max_nodes) {
        if (++guard > 4 * (int)P.max_nodes + 8) break;
        const uint32_t ns = node_slot(P, cur - 1);
        const int id = (int)hgetu(L, ns);
        if (id == kClosureMul) {
            for (int k = 0; k < 3; ++k) w[k] = w[k] * hget(L, ns + 1 + k);
            cur = hgetu(L, ns + 4);
        } else if (id == kClosureAdd) {
            push(hgetu(L, ns + 5), w);
            cur = hgetu(L, ns + 4);
        } else {
            const float cw[3] = { hget(L, ns + 1), hget(L, ns + 2), hget(L, ns + 3) };
            const uint32_t p = ns + 4;
            cur = 0u;
            if (id == kIdMxLayer) {
                float bw[3];
                for (int k = 0; k < 3; ++k) bw[k] = w[k] * cw[k];
                push(hgetu(L, p + 1), bw);
                cur = hgetu(L, p);
            } else if (lobe_on(LK_SHEEN) && id == kIdMxSheen) {
                const float albedo[3] = { hget(L, p + 3), hget(L, p + 4), hget(L, p + 5) };
                const SheenLobeDev sh =
                    sheen_make(v3(hget(L, p + 0), hget(L, p + 1), hget(L, p + 2)), albedo, hget(L, p + 6), wo,
                               path_rough, backfacing,
                               closure_keyword_int<PoolNodes>(L, p, 7, string_hash_const("mode"), 0));
                for (int k = 0; k < 3; ++k) w[k] = w[k] * (cw[k] * (1.0f - sh.emiss));
            } else if (lobe_on(LK_MX_DIELECTRIC) && id == kIdMxDielectric) {
                float fo[3];
                diel_filter_o(lobe_diel<PoolNodes>(L, p, wo, path_rough, backfacing), fo);
                for (int k = 0; k < 3; ++k) w[k] = w[k] * (cw[k] * (1.0f - fo[k]));
            }
        }
        if (cur == 0u && sp > 0) {
            --sp;
            cur = stack_node[sp];
            for (int k = 0; k < 3; ++k) w[k] = stack_w[sp][k];
        }
    }
    for (int k = 0; k < 3; ++k) out[k] = w[k];
}

// Renderer-side BSDF evaluation of a closure output at a light direction:
// prepare(wo, path_weight 1, absorb false) and eval (shading.h:322-374).
static __device__ void h_bsdf_eval(const Lane& L, const uint32_t* a, char* base, const ClosurePools& P, uint32_t* st) {
    const uint32_t root = ldw(L, a[0], 0);
    const V3 wi = v3(ldf(L, a[3], 0, 0), ldf(L, a[3], 1, 0), ldf(L, a[3], 2, 0));
    const V3 wo = v3(-ldf(L, a[4], 0, 0), -ldf(L, a[4], 1, 0), -ldf(L, a[4], 2, 0));
    Lobes B;
    lobes_build(L, P, root, a[5], st, B, 0.0f, false, wo);
    const float one[3] = { 1.0f, 1.0f, 1.0f };
    lobes_prepare(L, B, wo, one, false);
    const BsdfSample r = lobes_eval(L, B, wo, wi);
    float* o = reinterpret_cast<float*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    ostoref(o + 0, r.w[0]);
    ostoref(o + 1, r.w[1]);
    ostoref(o + 2, r.w[2]);
    ostoref(o + 3, r.pdf);
}

// Renderer-side sampling of a closure output, the per-hit step of
// testrender's path loop (simpleraytracer.cpp:1038-1079): userdata record
// {rx, ry, rz, path weight rgb, absorb, ray roughness, backfacing};
// output {wi, weight, pdf, Le, roughness}.
static __device__ void h_bsdf_sample(const Lane& L, const uint32_t* a, char* base, const char* ud,
                                     const ClosurePools& P, uint32_t* st) {
    const uint32_t root = ldw(L, a[0], 0);
    const V3 wo = v3(-ldf(L, a[3], 0, 0), -ldf(L, a[3], 1, 0), -ldf(L, a[3], 2, 0));
    const float* in = reinterpret_cast<const float*>(ud + (int64_t)a[5] + urec(L) * (int64_t)(int32_t)a[6]);
    Lobes B;
    lobes_build(L, P, root, a[4], st, B, in[7], in[8] != 0.0f, wo);
    const float pw[3] = { in[3], in[4], in[5] };
    lobes_prepare(L, B, wo, pw, in[6] != 0.0f);
    const BsdfSample r = lobes_sample(L, B, wo, in[0], in[1], in[2]);
    float* o = reinterpret_cast<float*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    const float vals[11] = { r.wi.x, r.wi.y, r.wi.z, r.w[0], r.w[1], r.w[2], r.pdf, B.Le[0], B.Le[1], B.Le[2],
                             r.roughness };
#pragma unroll
    for (int k = 0; k < 11; ++k) ostoref(o + k, vals[k]);
}

// ---- static closures: consumers over a term table ---------------------------------
// Term j of a static consumer is words 3*(j%2).. of the (j/2)-th carrier op
// after it: {node slot, weight operand or kNoArg, presence operand or kNoArg}
// (see kClosureAbsent). Visiting the present terms in table order is the
// reference walk of the tree the lowering knew.
__device__ __forceinline__ uint32_t term_word(const Op* tab, int j, int w) { return tab[j >> 1].a[3 * (j & 1) + w]; }
template <class F>
__device__ __forceinline__ void closure_walk_static(const Lane& L, const Op* tab, uint32_t nterms, F&& visit) {
    OSLG_SPEC_UNROLL
    for (int j = 0; j < kMaxStaticTerms; ++j) {
        if (j >= (int)nterms) break;
        const uint32_t ns = term_word(tab, j, 0), cwop = term_word(tab, j, 1), pop = term_word(tab, j, 2);
        const int id = (int)sgetu(L, ns);
        if (id == kClosureAbsent) continue;
        if (pop != kNoArg && ldw(L, pop, 0) == 0u) continue;
        float cw[3];
        for (int k = 0; k < 3; ++k) cw[k] = cwop == kNoArg ? sget(L, ns + 1 + k) : ldf(L, cwop, k, 0);
        visit(id, cw, ns + 4);
    }
}
// The lobes of a term table, one position per term (kind -1 where the term
// is absent, is no lobe, or comes after CompositeBSDF's capacity is full),
// so that every lobe's parameter slots stay compile-time constants in a
// specialized kernel. Lobes in position order are the walk's lobes.
__device__ __forceinline__ void lobes_collect_static(const Lane& L, const Op* tab, uint32_t nterms, uint32_t ggx,
                                                     Lobes& B, float path_rough, bool backfacing) {
    B.n = (int)nterms;
    B.Le[0] = B.Le[1] = B.Le[2] = 0.0f;
    B.path_rough = path_rough;
    B.backfacing = backfacing;
    int count = 0;
    OSLG_SPEC_UNROLL
    for (int j = 0; j < OSLG_LOBES_MAX; ++j) {
        if (j >= (int)nterms) break;
        B.kind[j] = -1;
        const uint32_t ns = term_word(tab, j, 0), cwop = term_word(tab, j, 1), pop = term_word(tab, j, 2);
        const int id = (int)sgetu(L, ns);
        if (id == kClosureAbsent) continue;
        if (pop != kNoArg && ldw(L, pop, 0) == 0u) continue;
        float cw[3];
        for (int k = 0; k < 3; ++k) cw[k] = cwop == kNoArg ? sget(L, ns + 1 + k) : ldf(L, cwop, k, 0);
        const uint32_t params = ns + 4;
        if (id == kIdEmission) {
            for (int c = 0; c < 3; ++c) B.Le[c] = B.Le[c] + cw[c];
            continue;
        }
        const int k = lobe_kind_of<SymNodes>(L, id, params, ggx);
        if (k < 0 || count >= kBsdfMaxLobes) continue;
        B.kind[j] = k;
        for (int c = 0; c < 3; ++c) B.w[j][c] = cw[c];
        B.p[j] = params;
        ++count;
    }
}
// records as h_store_closure writes them
static __device__ void h_cl_store(const Lane& L, const uint32_t* a, const Op* tab, char* base) {
    const uint32_t maxc = a[3];
    uint32_t* o = reinterpret_cast<uint32_t*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    uint32_t n = 0;
    closure_walk_static(L, tab, a[0], [&](int id, const float* cw, uint32_t params) {
        if (n >= maxc) return;
        uint32_t* q = o + 1 + n * kRecordFloats;
        ostore32(q, (uint32_t)id);
        for (int k = 0; k < 3; ++k) ostore32(q + 1 + k, __float_as_uint(cw[k]));
        for (int k = 0; k < kRecordParams; ++k) ostore32(q + 4 + k, sgetu(L, params + k));
        ++n;
    });
    ostore32(o, n);
}
// as h_bsdf_eval
static __device__ void h_cl_bsdf_eval(const Lane& L, const uint32_t* a, const Op* tab, char* base) {
    const V3 wi = v3(ldf(L, a[3], 0, 0), ldf(L, a[3], 1, 0), ldf(L, a[3], 2, 0));
    const V3 wo = v3(-ldf(L, a[4], 0, 0), -ldf(L, a[4], 1, 0), -ldf(L, a[4], 2, 0));
    Lobes B;
    lobes_collect_static(L, tab, a[0], a[5], B, 0.0f, false);
    const float one[3] = { 1.0f, 1.0f, 1.0f };
    lobes_prepare<SymNodes>(L, B, wo, one, false);
    const BsdfSample r = lobes_eval<SymNodes>(L, B, wo, wi);
    float* o = reinterpret_cast<float*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    ostoref(o + 0, r.w[0]);
    ostoref(o + 1, r.w[1]);
    ostoref(o + 2, r.w[2]);
    ostoref(o + 3, r.pdf);
}
// as h_bsdf_sample
static __device__ void h_cl_bsdf_sample(const Lane& L, const uint32_t* a, const Op* tab, char* base, const char* ud) {
    const V3 wo = v3(-ldf(L, a[3], 0, 0), -ldf(L, a[3], 1, 0), -ldf(L, a[3], 2, 0));
    const float* in = reinterpret_cast<const float*>(ud + (int64_t)a[5] + urec(L) * (int64_t)(int32_t)a[6]);
    Lobes B;
    lobes_collect_static(L, tab, a[0], a[4], B, in[7], in[8] != 0.0f);
    const float pw[3] = { in[3], in[4], in[5] };
    lobes_prepare<SymNodes>(L, B, wo, pw, in[6] != 0.0f);
    const BsdfSample r = lobes_sample<SymNodes>(L, B, wo, in[0], in[1], in[2]);
    float* o = reinterpret_cast<float*>(base + (int64_t)a[1] + orec(L) * (int64_t)(int32_t)a[2]);
    const float vals[11] = { r.wi.x, r.wi.y, r.wi.z, r.w[0], r.w[1], r.w[2], r.pdf, B.Le[0], B.Le[1], B.Le[2],
                             r.roughness };
#pragma unroll
    for (int k = 0; k < 11; ++k) ostoref(o + k, vals[k]);
}

// ---- splineinverse (splineimpl.h:241-296) ------------------------------------------------
// The spline of float knots at a Dual2 position (SplineInterp::evaluate with
// float knots): the root finder's function.
struct SplineFn {
    const Lane* L;
    uint32_t kn;
    int basis, count;
    __device__ float knot(int k) const { return __uint_as_float(ldw(*L, kn, k)); }
    __device__ D2 operator()(D2 xval) const {
        const SplineBasisDev& B = c_spline_basis[basis];
        D2 x = xval;
        if (!(0.0f <= x.v)) x = d2c(0.0f);
        if (x.v > 1.0f) x = d2c(1.0f);
        const int nsegs = ((count - 4) / B.step) + 1;
        x = x * (float)nsegs;
        int segnum = (int)x.v;
        if (segnum < 0) segnum = 0;
        if (segnum > nsegs - 1) segnum = nsegs - 1;
        if (basis == 5) return d2c(knot(segnum + 1));
        x = x - (float)segnum;
        const int s = segnum * B.step;
        float tk[4];
        for (int k = 0; k < 4; ++k)
            tk[k] = ((knot(s) * B.m[k][0] + knot(s + 1) * B.m[k][1]) + knot(s + 2) * B.m[k][2]) + knot(s + 3) * B.m[k][3];
        D2 t = x * tk[0];
        t = t + tk[1];
        t = t * x;
        t = t + tk[2];
        t = t * x;
        t = t + tk[3];
        return t;
    }
};
__device__ __forceinline__ D2 d2_div(D2 a, D2 b) {
    const float binv = 1.0f / b.v, ab = a.v / b.v;
    return d2(ab, binv * (a.dx - ab * b.dx), binv * (a.dy - ab * b.dy));
}
// root of f(x) = y on [xmin, xmax]: regula falsi for the first three
// quarters of the iterations (bisecting when the interpolant leaves the
// bracket), then bisection; stops when the bracket or the residual is below
// eps. Unbracketed: the end of the interval toward y. (OpenImageIO's
// invert(), which the reference calls; the published method.)
static __device__ D2 spline_root(const SplineFn& f, D2 y, D2 xmin, D2 xmax, int maxiters, float eps, bool* brack) {
    D2 v0 = f(xmin), v1 = f(xmax);
    D2 x = xmin, v = v0;
    const bool increasing = v0.v < v1.v;
    const float vmin = increasing ? v0.v : v1.v, vmax = increasing ? v1.v : v0.v;
    const bool bracketed = y.v >= vmin && y.v <= vmax;
    *brack = bracketed;
    if (!bracketed) return ((y.v < vmin) == increasing) ? xmin : xmax;
    if (fabsf(v0.v - v1.v) < eps) return x;
    const int rfiters = (3 * maxiters) / 4;
    for (int it = 0; it < maxiters; ++it) {
        D2 t = d2c(0.5f);
        if (it < rfiters) {
            t = d2_div(y - v0, v1 - v0);
            if (t.v <= 0.0f || t.v >= 1.0f) t = d2c(0.5f);
        }
        const D2 omt = d2(1.0f - t.v, -t.dx, -t.dy);
        x = xmin * omt + xmax * t;
        v = f(x);
        if ((v.v < y.v) == increasing) {
            xmin = x;
            v0 = v;
        } else {
            xmax = x;
            v1 = v;
        }
        if (fabsf(xmax.v - xmin.v) < eps || fabsf(v.v - y.v) < eps) return x;
    }
    return x;
}
static __device__ void h_splineinverse(const Lane& L, const uint32_t* a, uint32_t* st) {
    const uint32_t r = a[0];
    SplineFn f;
    f.L = &L;
    f.kn = a[2];
    f.basis = a[3] < 6u ? (int)a[3] : 0;
    const int alen = (int)a[5];
    f.count = a[4] != kNoArg ? ldi(L, a[4], 0) : alen;
    if (f.count > alen) f.count = alen;
    if (f.count < 4) {  // a spline needs four knots
        raise_status(st, ST_ARRAY_BOUNDS);
        std2(L, r, 0, d2c(0.0f));
        return;
    }
    const D2 y = ldd(L, a[1], 0);
    const SplineBasisDev& B = c_spline_basis[f.basis];
    const int lo = B.step == 1 ? 1 : 0, hi = B.step == 1 ? f.count - 2 : f.count - 1;
    const bool increasing = f.knot(1) < f.knot(f.count - 2);
    D2 x = d2c(0.0f);
    bool done = false;
    if (increasing) {
        if (y.v <= f.knot(lo)) { x = d2c(0.0f); done = true; }
        else if (y.v >= f.knot(hi)) { x = d2c(1.0f); done = true; }
    } else {
        if (y.v >= f.knot(lo)) { x = d2c(0.0f); done = true; }
        else if (y.v <= f.knot(hi)) { x = d2c(1.0f); done = true; }
    }
    if (!done) {
        const int nsegs = (f.count - 4) / B.step + 1;
        const float nseginv = 1.0f / (float)nsegs;
        D2 r0 = d2c(0.0f);
        for (int s = 0; s < nsegs; ++s) {
            const D2 r1 = d2c(nseginv * (float)(s + 1));
            bool brack;
            x = spline_root(f, y, r0, r1, 32, 1.0e-6f, &brack);
            if (brack) break;
            r0 = r1;
        }
    }
    std2(L, r, 0, x);
}

// ---- spline (splineimpl.h:191-239) -----------------------------------------------------
static __device__ void h_spline(const Lane& L, const uint32_t* a, uint32_t* st) {
    uint32_t r = a[0], xa = a[1], kn = a[2];
    const SplineBasisDev& B = c_spline_basis[a[3] < 6u ? a[3] : 0u];
    int alen = (int)a[5];
    int knot_count = a[4] != kNoArg ? ldi(L, a[4], 0) : alen;
    if (knot_count > alen) knot_count = alen;
    int nc = anc(r);
    if (knot_count < 4) {  // a spline needs four knots
        raise_status(st, ST_ARRAY_BOUNDS);
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) std2(L, r, c, d2c(0.0f));
        return;
    }
    int kc = anc(kn);
    bool xd = ader(xa), kd = ader(kn), rd = ader(r);
    D2 x = ldd(L, xa, 0);
    if (!(0.0f <= x.v)) x = d2c(0.0f);
    if (x.v > 1.0f) x = d2c(1.0f);
    int nsegs = ((knot_count - 4) / B.step) + 1;
    x = x * (float)nsegs;
    int segnum = (int)x.v;
    if (segnum < 0) segnum = 0;
    if (segnum > nsegs - 1) segnum = nsegs - 1;
    if (a[3] == 5u) {  // constant basis
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) stval(L, r, c, __uint_as_float(ldw(L, kn, (segnum + 1) * kc + (kc == 1 ? 0 : c))));
        return;
    }
    x = x - (float)segnum;
    int s = segnum * B.step;
    OSLG_SPEC_UNROLL
    for (int c = 0; c < nc; ++c) {
        int cc = kc == 1 ? 0 : c;
        D2 P[4];
        for (int k = 0; k < 4; ++k) {
            float v = __uint_as_float(ldw(L, kn, (s + k) * kc + cc));
            float dx = kd ? __uint_as_float(ldw(L, kn, alen * kc + (s + k) * kc + cc)) : 0.0f;
            float dy = kd ? __uint_as_float(ldw(L, kn, 2 * alen * kc + (s + k) * kc + cc)) : 0.0f;
            P[k] = d2(v, dx, dy);
        }
        D2 tk[4];
        for (int k = 0; k < 4; ++k) {
            // basis[k][j] * P[j], summed left to right (float * CTYPE)
            D2 t0 = P[0] * B.m[k][0], t1 = P[1] * B.m[k][1], t2 = P[2] * B.m[k][2], t3 = P[3] * B.m[k][3];
            tk[k] = ((t0 + t1) + t2) + t3;
        }
        D2 res;
        if (!xd && !kd) {
            float xv = x.v;
            float t = tk[0].v * xv + tk[1].v;
            t = t * xv + tk[2].v;
            t = t * xv + tk[3].v;
            res = d2c(t);
        } else if (!kd) {
            // CTYPE without partials times a Dual2 x: tk*x scales every element
            D2 t = x * tk[0].v;
            t = t + tk[1].v;
            t = t * x;
            t = t + tk[2].v;
            t = t * x;
            t = t + tk[3].v;
            res = t;
        } else {
            D2 t = tk[0] * x + tk[1];
            t = t * x + tk[2];
            t = t * x + tk[3];
            res = t;
        }
        if (!rd) stval(L, r, c, res.v);
        else std2(L, r, c, res);
    }
}

// ---- the interpreter -----------------------------------------------------------------
__device__ __forceinline__ bool bit(uint32_t m, int d) { return (m >> d) & 1u; }
__device__ __forceinline__ uint32_t setbit(uint32_t m, int d, bool v) { return v ? (m | (1u << d)) : (m & ~(1u << d)); }


// Feature tiers: a program only pays (in code size and instruction-cache
// footprint) for the op families it uses. TIER bits: 1 noise/hash, 2
// closures/BSDF/spline, 4 transcendental math, vectors, matrices, transforms.
#define OSLG_TIER_CASE(bit, stmt)                 \
    if constexpr ((TIER & (bit)) != 0) {          \
        stmt;                                     \
    } else {                                      \
        raise_status(R.status, ST_BAD_OPCODE);    \
    }

// Everything a program run needs besides the lane: the staged op stream,
// closure pools and the caller's arenas.
struct RunCtx {
    const Op* sops;
    int nops;
    const TexDesc* textures = nullptr;
    int ntextures = 0;
    ClosurePools CP;
    bool uses_closures;
    const oslg_shaderglobals* G;
    char* userdata;
    char* outputs;
    uint32_t* status;
    uint32_t max_iters = kDefaultMaxLoopIterations;  // loop back edges per point
    float* symheap = nullptr;  // retained symbols (KArgs::symheap)
    int64_t symheap_stride = 0;
};

// Control state of the masked walk: per thread, PPT points with their
// active / valid / exited / returned bits, per-depth if and loop stacks and
// the loop back edges each point has taken.
template <int PPT>
struct Ctl {
    uint32_t validm, actm, extm, lretm;
    uint32_t extm0;  // points that exited before the current layer
    uint32_t stk[PPT], cnd[PPT], brk[PPT], cnt[PPT], iters[PPT];
    uint32_t fret[PPT];  // bit (tag - 1): the point returned from that user function
};

template <int PPT>
__device__ __forceinline__ void ctl_init(Ctl<PPT>& C, const RunCtx& R, Lane& L, int64_t npoints) {
    const uint32_t li0 = L.li;
    const int64_t pt0 = L.pt;
    C.validm = 0;
    C.extm = 0;
    C.extm0 = 0;
    C.lretm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        C.stk[j] = C.cnd[j] = C.brk[j] = C.cnt[j] = C.iters[j] = C.fret[j] = 0;
        if (pt0 + (int64_t)j * blockDim.x < npoints) C.validm |= 1u << j;
    }
    C.actm = C.validm;
    if (R.uses_closures) {
#pragma unroll
        for (int j = 0; j < PPT; ++j)
            if (C.validm & (1u << j)) {
                L.li = li0 + j * blockDim.x;
                hsetu(L, R.CP.base, 0u);
            }
        L.li = li0;
    }
}

// The mask ops. Those that can skip a block return true when no lane of the
// warp stays active (the caller then jumps to a[2]).
template <int PPT>
__device__ __forceinline__ bool ctl_if(Ctl<PPT>& C, Lane& L, uint32_t li0, const uint32_t* a) {
    const int d = (int)a[1];
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const bool aj = (C.actm >> j) & 1u;
        L.li = li0 + j * blockDim.x;
        const bool c = aj && truth(L, a[0]);
        C.stk[j] = setbit(C.stk[j], d, aj);
        C.cnd[j] = setbit(C.cnd[j], d, c);
        if (c) nm |= 1u << j;
    }
    L.li = li0;
    C.actm = nm;
    return !__any_sync(FULL, C.actm != 0);
}
template <int PPT>
__device__ __forceinline__ bool ctl_else(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int ll = (int)a[3];
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const bool off = ((C.extm | C.lretm) >> j & 1u) || C.fret[j] != 0u ||
                         (ll && (bit(C.brk[j], ll - 1) || bit(C.cnt[j], ll - 1)));
        if (bit(C.stk[j], d) && !bit(C.cnd[j], d) && !off) nm |= 1u << j;
    }
    C.actm = nm;
    return !__any_sync(FULL, C.actm != 0);
}
template <int PPT>
__device__ __forceinline__ void ctl_endif(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int ll = (int)a[3];
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const bool off = ((C.extm | C.lretm) >> j & 1u) || C.fret[j] != 0u ||
                         (ll && (bit(C.brk[j], ll - 1) || bit(C.cnt[j], ll - 1)));
        if (bit(C.stk[j], d) && !off) nm |= 1u << j;
    }
    C.actm = nm;
}
template <int PPT>
__device__ __forceinline__ void ctl_loop_begin(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int ll = (int)a[3];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        C.stk[j] = setbit(C.stk[j], d, (C.actm >> j) & 1u);
        C.brk[j] = setbit(C.brk[j], ll - 1, false);
        C.cnt[j] = setbit(C.cnt[j], ll - 1, false);
    }
}
template <int PPT>
__device__ __forceinline__ bool ctl_loop_test(Ctl<PPT>& C, Lane& L, uint32_t li0, const uint32_t* a) {
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        L.li = li0 + j * blockDim.x;
        if (((C.actm >> j) & 1u) && truth(L, a[0])) nm |= 1u << j;
    }
    L.li = li0;
    C.actm = nm;
    return !__any_sync(FULL, C.actm != 0);
}
template <int PPT>
__device__ __forceinline__ void ctl_loop_step(Ctl<PPT>& C, const uint32_t* a) {
    const int ll = (int)a[3];
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        if ((((C.actm >> j) & 1u) || bit(C.cnt[j], ll - 1)) && !bit(C.brk[j], ll - 1) && !((C.extm | C.lretm) >> j & 1u)
            && C.fret[j] == 0u)
            nm |= 1u << j;
        C.cnt[j] = setbit(C.cnt[j], ll - 1, false);
    }
    C.actm = nm;
}
template <int PPT>
__device__ __forceinline__ void ctl_loop_end(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int ll = (int)a[3];
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        C.brk[j] = setbit(C.brk[j], ll - 1, false);
        C.cnt[j] = setbit(C.cnt[j], ll - 1, false);
        // lanes that broke out of an enclosing loop stay off via the
        // enclosing ENDIF/LOOP_STEP recomputation
        if (bit(C.stk[j], d) && !((C.extm | C.lretm) >> j & 1u) && C.fret[j] == 0u) nm |= 1u << j;
    }
    C.actm = nm;
}
// user-function bodies (oslc wraps each call in a functioncall op,
// codegen.cpp:1890-1905): the points active at the call enter; a return
// inside marks the point off until the body ends (other points go on, e.g.
// into an else branch). Begin skips the body when no point of the warp
// enters it.
template <int PPT>
__device__ __forceinline__ bool ctl_func_begin(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int f = (int)a[3] - 1;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        C.stk[j] = setbit(C.stk[j], d, (C.actm >> j) & 1u);
        C.fret[j] = setbit(C.fret[j], f, false);
    }
    return !__any_sync(FULL, C.actm != 0);
}
template <int PPT>
__device__ __forceinline__ void ctl_func_return(Ctl<PPT>& C, const uint32_t* a) {
    const int f = (int)a[3] - 1;
#pragma unroll
    for (int j = 0; j < PPT; ++j)
        if ((C.actm >> j) & 1u) C.fret[j] = setbit(C.fret[j], f, true);
    C.actm = 0;
}
template <int PPT>
__device__ __forceinline__ void ctl_func_end(Ctl<PPT>& C, const uint32_t* a) {
    const int d = (int)a[1];
    const int f = (int)a[3] - 1;
    uint32_t nm = 0;
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        C.fret[j] = setbit(C.fret[j], f, false);
        if (bit(C.stk[j], d) && !((C.extm | C.lretm) >> j & 1u) && C.fret[j] == 0u) nm |= 1u << j;
    }
    C.actm = nm;
}
template <int PPT>
__device__ __forceinline__ void ctl_break(Ctl<PPT>& C, const uint32_t* a) {
    const int ll = (int)a[3];
#pragma unroll
    for (int j = 0; j < PPT; ++j)
        if (((C.actm >> j) & 1u) && ll) C.brk[j] = setbit(C.brk[j], ll - 1, true);
    C.actm = 0;
}
template <int PPT>
__device__ __forceinline__ void ctl_continue(Ctl<PPT>& C, const uint32_t* a) {
    const int ll = (int)a[3];
#pragma unroll
    for (int j = 0; j < PPT; ++j)
        if (((C.actm >> j) & 1u) && ll) C.cnt[j] = setbit(C.cnt[j], ll - 1, true);
    C.actm = 0;
}
// A loop's back edge: each point still iterating counts one. When a point
// passes `cap`, it raises ST_TIMEOUT and the whole warp stops its walk (the
// decision is warp-uniform, as the program counter is); returns true then.
template <int PPT>
__device__ __forceinline__ bool ctl_back_edge(Ctl<PPT>& C, const RunCtx& R, uint32_t cap) {
    bool over = false;
#pragma unroll
    for (int j = 0; j < PPT; ++j)
        if (((C.actm >> j) & 1u) && ++C.iters[j] > cap) over = true;
    if (!__any_sync(FULL, over)) return false;
    if (over) raise_status(R.status, ST_TIMEOUT);
    return true;
}

template <int PPT>
__device__ __forceinline__ void ctl_return(Ctl<PPT>& C) { C.lretm |= C.actm; C.actm = 0; }
template <int PPT>
__device__ __forceinline__ void ctl_exit(Ctl<PPT>& C) { C.extm |= C.actm; C.actm = 0; }
template <int PPT>
__device__ __forceinline__ void ctl_layer_end(Ctl<PPT>& C) {
    // the layer's output stores follow: they run for every point that ran
    // the layer, also one that exited inside it (what it wrote before
    // exit() is its result, as the reference's symloc outputs keep it)
    C.lretm = 0;
    C.actm = C.validm & ~C.extm0;
}
template <int PPT>
__device__ __forceinline__ void ctl_stores_end(Ctl<PPT>& C, const uint32_t* a) {
    C.extm0 = C.extm;
    C.actm = a[0] ? C.validm : C.validm & ~C.extm;
}

// One data op for the point L addresses. next() gives the following op
// (the closure and Gabor ops carry extra operands there) or null at the end;
// it is called only by those ops.
template <int TIER, class NextOp>
__device__ __forceinline__ void exec_op(const RunCtx& R, Lane& L, uint32_t code, const uint32_t* a, NextOp next_op) {
    switch (code) {
    case OP_LOAD_GLOBAL: h_load_global(L, a, (*R.G)); break;
    case OP_LOAD_USERDATA: h_load_userdata(L, a, R.userdata); break;
    case OP_STORE_OUTPUT: h_store_output(L, a, R.outputs); break;
    case OP_ASSIGN: h_assign_fast(L, a, R.status); break;
    case OP_COMPREF: h_compref(L, a, R.status); break;
    case OP_COMPASSIGN: h_compassign(L, a, R.status); break;
    case OP_MXCOMPREF: {
        int r = ldi(L, a[2], 0), c = ldi(L, a[3], 0);
        r = r < 0 ? 0 : (r > 3 ? 3 : r); c = c < 0 ? 0 : (c > 3 ? 3 : c);
        stval(L, a[0], 0, __uint_as_float(ldw(L, a[1], r * 4 + c)));
        break;
    }
    case OP_MXCOMPASSIGN: {
        int r = ldi(L, a[1], 0), c = ldi(L, a[2], 0);
        r = r < 0 ? 0 : (r > 3 ? 3 : r); c = c < 0 ? 0 : (c > 3 ? 3 : c);
        stf(L, a[0], r * 4 + c, ldf(L, a[3], 0, 0));
        break;
    }
    case OP_CONSTRUCT3: h_construct3(L, a); break;
    case OP_AREF: OSLG_TIER_CASE(4, h_aref(L, a, R.status)) break;
    case OP_AASSIGN: OSLG_TIER_CASE(4, h_aassign(L, a, R.status)) break;
    case OP_MATRIX_DIAG: {
        float v = ldf(L, a[1], 0, 0);
        for (int i = 0; i < 16; ++i) stf(L, a[0], i, (i % 5 == 0) ? v : 0.0f);
        break;
    }
    case OP_ADD: h_arith_fast<0>(L, a); break;
    case OP_SUB: h_arith_fast<1>(L, a); break;
    case OP_MUL: h_arith_fast<2>(L, a); break;
    case OP_DIV: h_arith_fast<3>(L, a); break;
    case OP_MOD: h_arith<4>(L, a); break;
    case OP_NEG: h_unary<OP_NEG>(L, a); break;
    case OP_IADD: h_iarith<0>(L, a); break;
    case OP_ISUB: h_iarith<1>(L, a); break;
    case OP_IMUL: h_iarith<2>(L, a); break;
    case OP_IDIV: h_iarith<3>(L, a); break;
    case OP_IMOD: h_iarith<4>(L, a); break;
    case OP_INEG: stw(L, a[0], 0, (uint32_t)(-ldi(L, a[1], 0))); break;
    case OP_MMUL: OSLG_TIER_CASE(4, h_mmul(L, a)) break;
    case OP_EQ: h_cmp<0>(L, a); break;
    case OP_NEQ: h_cmp<1>(L, a); break;
    case OP_LT: h_cmp<2>(L, a); break;
    case OP_GT: h_cmp<3>(L, a); break;
    case OP_LE: h_cmp<4>(L, a); break;
    case OP_GE: h_cmp<5>(L, a); break;
    case OP_AND: stw(L, a[0], 0, (truth(L, a[1]) && truth(L, a[2])) ? 1u : 0u); break;
    case OP_OR: stw(L, a[0], 0, (truth(L, a[1]) || truth(L, a[2])) ? 1u : 0u); break;
    case OP_BITAND: stw(L, a[0], 0, (uint32_t)(ldi(L, a[1], 0) & ldi(L, a[2], 0))); break;
    case OP_BITOR: stw(L, a[0], 0, (uint32_t)(ldi(L, a[1], 0) | ldi(L, a[2], 0))); break;
    case OP_XOR: stw(L, a[0], 0, (uint32_t)(ldi(L, a[1], 0) ^ ldi(L, a[2], 0))); break;
    case OP_SHL: stw(L, a[0], 0, (uint32_t)ldi(L, a[1], 0) << (ldi(L, a[2], 0) & 31)); break;
    case OP_SHR: stw(L, a[0], 0, (uint32_t)(ldi(L, a[1], 0) >> (ldi(L, a[2], 0) & 31))); break;
    case OP_COMPL: stw(L, a[0], 0, ~(uint32_t)ldi(L, a[1], 0)); break;
    case OP_ABS: h_unary<OP_ABS>(L, a); break;
    case OP_IABS: { int v = ldi(L, a[1], 0); stw(L, a[0], 0, (uint32_t)(v < 0 ? -v : v)); break; }
    case OP_FLOOR: h_unary<OP_FLOOR>(L, a); break;
    case OP_CEIL: h_unary<OP_CEIL>(L, a); break;
    case OP_ROUND: h_unary<OP_ROUND>(L, a); break;
    case OP_TRUNC: h_unary<OP_TRUNC>(L, a); break;
    case OP_SIGN: h_unary<OP_SIGN>(L, a); break;
    case OP_SQRT: h_unary<OP_SQRT>(L, a); break;
    case OP_INVSQRT: h_unary<OP_INVSQRT>(L, a); break;
    case OP_CBRT: OSLG_TIER_CASE(4, h_unary<OP_CBRT>(L, a)) break;
    case OP_SIN: OSLG_TIER_CASE(4, h_unary<OP_SIN>(L, a)) break;
    case OP_COS: OSLG_TIER_CASE(4, h_unary<OP_COS>(L, a)) break;
    case OP_TAN: OSLG_TIER_CASE(4, h_unary<OP_TAN>(L, a)) break;
    case OP_ASIN: OSLG_TIER_CASE(4, h_unary<OP_ASIN>(L, a)) break;
    case OP_ACOS: OSLG_TIER_CASE(4, h_unary<OP_ACOS>(L, a)) break;
    case OP_ATAN: OSLG_TIER_CASE(4, h_unary<OP_ATAN>(L, a)) break;
    case OP_SINH: OSLG_TIER_CASE(4, h_unary<OP_SINH>(L, a)) break;
    case OP_COSH: OSLG_TIER_CASE(4, h_unary<OP_COSH>(L, a)) break;
    case OP_TANH: OSLG_TIER_CASE(4, h_unary<OP_TANH>(L, a)) break;
    case OP_EXP: OSLG_TIER_CASE(4, h_unary<OP_EXP>(L, a)) break;
    case OP_EXP2: OSLG_TIER_CASE(4, h_unary<OP_EXP2>(L, a)) break;
    case OP_EXPM1: OSLG_TIER_CASE(4, h_unary<OP_EXPM1>(L, a)) break;
    case OP_LOG: OSLG_TIER_CASE(4, h_unary<OP_LOG>(L, a)) break;
    case OP_LOG2: OSLG_TIER_CASE(4, h_unary<OP_LOG2>(L, a)) break;
    case OP_LOG10: OSLG_TIER_CASE(4, h_unary<OP_LOG10>(L, a)) break;
    case OP_LOGB: OSLG_TIER_CASE(4, h_unary<OP_LOGB>(L, a)) break;
    case OP_ERF: OSLG_TIER_CASE(4, h_unary<OP_ERF>(L, a)) break;
    case OP_ERFC: OSLG_TIER_CASE(4, h_unary<OP_ERFC>(L, a)) break;
    case OP_SINCOS: OSLG_TIER_CASE(4, h_sincos(L, a)) break;
    case OP_CALCNORMAL: OSLG_TIER_CASE(4, h_calcnormal(L, a, *R.G)) break;
    case OP_RAYTYPE: OSLG_TIER_CASE(4, h_raytype(L, a, *R.G)) break;
    case OP_STORE_HEAP:
        // a retained symbol's words into its planes (values, by point)
        if (R.symheap)
            for (uint32_t c = 0; c < a[2]; ++c)
                R.symheap[(int64_t)(a[1] + c) * R.symheap_stride + L.pt] = __uint_as_float(ldw(L, a[0], (int)c));
        break;
    case OP_RADIANS: h_unary<OP_RADIANS>(L, a); break;
    case OP_DEGREES: h_unary<OP_DEGREES>(L, a); break;
    case OP_ISNAN: stw(L, a[0], 0, isnan(ldf(L, a[1], 0, 0)) ? 1u : 0u); break;
    case OP_ISINF: stw(L, a[0], 0, isinf(ldf(L, a[1], 0, 0)) ? 1u : 0u); break;
    case OP_ISFINITE: stw(L, a[0], 0, isfinite(ldf(L, a[1], 0, 0)) ? 1u : 0u); break;
    case OP_POW: OSLG_TIER_CASE(4, h_binary<OP_POW>(L, a)) break;
    case OP_ATAN2: OSLG_TIER_CASE(4, h_binary<OP_ATAN2>(L, a)) break;
    case OP_FMOD: OSLG_TIER_CASE(4, h_binary<OP_FMOD>(L, a)) break;
    case OP_MIN: h_binary<OP_MIN>(L, a); break;
    case OP_MAX: h_binary<OP_MAX>(L, a); break;
    case OP_STEP: h_binary<OP_STEP>(L, a); break;
    case OP_IMIN: { int x = ldi(L, a[1], 0), y = ldi(L, a[2], 0); stw(L, a[0], 0, (uint32_t)(x <= y ? x : y)); break; }
    case OP_IMAX: { int x = ldi(L, a[1], 0), y = ldi(L, a[2], 0); stw(L, a[0], 0, (uint32_t)(x > y ? x : y)); break; }
    case OP_CLAMP: OSLG_TIER_CASE(4, h_clamp(L, a)) break;
    case OP_MIX: OSLG_TIER_CASE(4, h_mix(L, a)) break;
    case OP_SMOOTHSTEP: OSLG_TIER_CASE(4, h_smoothstep(L, a)) break;
    case OP_SELECT: OSLG_TIER_CASE(4, h_select(L, a)) break;
    case OP_DOT: OSLG_TIER_CASE(4, h_dot(L, a)) break;
    case OP_CROSS: OSLG_TIER_CASE(4, h_cross(L, a)) break;
    case OP_LENGTH: OSLG_TIER_CASE(4, h_length(L, a, false)) break;
    case OP_DISTANCE: OSLG_TIER_CASE(4, h_length(L, a, true)) break;
    case OP_NORMALIZE: OSLG_TIER_CASE(4, h_normalize(L, a)) break;
    case OP_DX:
    case OP_DY: {
        int d = code == OP_DX ? 1 : 2;
        int nc = anc(a[0]);
        OSLG_SPEC_UNROLL
        for (int c = 0; c < nc; ++c) stval(L, a[0], c, ldf(L, a[1], c, d));
        break;
    }
    case OP_TRANSFORM:
        if (a[3] == 2u) { OSLG_TIER_CASE(4, h_transformn(L, a)) }
        else { OSLG_TIER_CASE(4, h_transform(L, a)) }
        break;
    case OP_MDIV: OSLG_TIER_CASE(4, h_mdiv(L, a)) break;
    case OP_TRANSPOSE:
    case OP_DETERMINANT: OSLG_TIER_CASE(4, h_matrix_misc(L, code, a)) break;
    case OP_AREA:
    case OP_FILTERWIDTH: OSLG_TIER_CASE(4, h_deriv_misc(L, code, a)) break;
    case OP_LUMINANCE: OSLG_TIER_CASE(4, h_luminance(L, a)) break;
    case OP_TRANSFORMC: OSLG_TIER_CASE(4, h_transformc(L, a)) break;
    case OP_WAVELENGTH: OSLG_TIER_CASE(4, h_wavelength(L, a)) break;
    case OP_BLACKBODY: OSLG_TIER_CASE(4, h_blackbody(L, a)) break;
    case OP_TEXTURE: OSLG_TIER_CASE(4, h_texture(L, a, R.textures, R.ntextures, R.status)) break;
    case OP_ENVIRONMENT: OSLG_TIER_CASE(4, h_environment(L, a, R.textures, R.ntextures, R.status)) break;
    case OP_SETMESSAGE: OSLG_TIER_CASE(4, h_setmessage(L, a, R.status)) break;
    case OP_GETMESSAGE: OSLG_TIER_CASE(4, h_getmessage(L, a, R.status)) break;
    case OP_NOISE: OSLG_TIER_CASE(1, h_noise(L, a)) break;
    case OP_GABOR: {
        if constexpr ((TIER & 1) != 0) {
            const Op* next = next_op();
            if (next) h_gabor(L, a, next->a);
            else raise_status(R.status, ST_BAD_OPCODE);
        } else {
            raise_status(R.status, ST_BAD_OPCODE);
        }
        break;
    }
    case OP_HASH: OSLG_TIER_CASE(1, h_hash(L, a)) break;
    case OP_CLOSURE: {
        if constexpr ((TIER & 2) != 0) {
            const uint32_t* extra = nullptr;
            const Op* next = next_op();
            if (next && next->code == OP_NOP && next->nargs == 7) extra = next->a;
            h_closure(L, a, extra, R.CP, R.status);
        } else {
            raise_status(R.status, ST_BAD_OPCODE);
        }
        break;
    }
    case OP_CLOSURE_NODE: {
        if constexpr ((TIER & 2) != 0) {
            const uint32_t* extra = nullptr;
            const Op* next = next_op();
            if (next && next->code == OP_NOP && next->nargs == 7) extra = next->a;
            h_closure_node(L, a, extra);
        } else {
            raise_status(R.status, ST_BAD_OPCODE);
        }
        break;
    }
    case OP_CL_STORE: OSLG_TIER_CASE(2, h_cl_store(L, a, next_op(), R.outputs)) break;
    case OP_CL_BSDF_EVAL: OSLG_TIER_CASE(2, h_cl_bsdf_eval(L, a, next_op(), R.outputs)) break;
    case OP_CL_BSDF_SAMPLE: OSLG_TIER_CASE(2, h_cl_bsdf_sample(L, a, next_op(), R.outputs, R.userdata)) break;
    case OP_CLOSURE_MUL: OSLG_TIER_CASE(2, h_closure_mul(L, a, R.CP, R.status)) break;
    case OP_CLOSURE_ADD: OSLG_TIER_CASE(2, h_closure_add(L, a, R.CP, R.status)) break;
    case OP_STORE_CLOSURE: OSLG_TIER_CASE(2, h_store_closure(L, a, R.outputs, R.CP, R.status)) break;
    case OP_BSDF_EVAL: OSLG_TIER_CASE(2, h_bsdf_eval(L, a, R.outputs, R.CP, R.status)) break;
    case OP_BSDF_SAMPLE: OSLG_TIER_CASE(2, h_bsdf_sample(L, a, R.outputs, R.userdata, R.CP, R.status)) break;
    case OP_SPLINE: OSLG_TIER_CASE(2, h_spline(L, a, R.status)) break;
    case OP_SPLINEINV: OSLG_TIER_CASE(2, h_splineinverse(L, a, R.status)) break;
    default: raise_status(R.status, ST_BAD_OPCODE); break;
    }
}

// One op whose code is known at compile time (specialized kernels): one
// instantiation per opcode, in which the dispatch is already resolved, so
// a program's call sites inline only their own handler. `nx` is the
// following operand carrier (or null).
template <int TIER, uint32_t CODE>
__device__ __forceinline__ void exec_op_c(const RunCtx& R, Lane& L, const uint32_t* a, const Op* nx) {
    exec_op<TIER>(R, L, CODE, a, [nx]() -> const Op* { return nx; });
}

// Run the whole program for one point per thread (L.pt; lanes past npoints
// take part in the warp-uniform walk with no active bits). The mask ops
// here are the ctl_* functions above written out over plain locals (the
// struct form costs the interpreter registers); a specialized kernel calls
// ctl_* and exec_op directly.
template <int TIER, int PPT = 1>
__device__ __forceinline__ void run_tile(const RunCtx& R, Lane& L, int64_t npoints) {
    // Each thread carries PPT points of the tile: lane slot li0 + j*blockDim
    // (heap column) and point pt0 + j*blockDim. Ops are decoded once and run
    // for every active point of the thread; control state is per point.
    const uint32_t li0 = L.li;
    const int64_t pt0 = L.pt;
    uint32_t validm = 0, actm, extm = 0, lretm = 0, extm0 = 0;
    uint32_t stk[PPT], cnd[PPT], brk[PPT], cnt[PPT], iters[PPT], fret[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        stk[j] = cnd[j] = brk[j] = cnt[j] = iters[j] = fret[j] = 0;
        if (pt0 + (int64_t)j * blockDim.x < npoints) validm |= 1u << j;
    }
    actm = validm;
    if (R.uses_closures) {
#pragma unroll
        for (int j = 0; j < PPT; ++j)
            if (validm & (1u << j)) {
                L.li = li0 + j * blockDim.x;
                hsetu(L, R.CP.base, 0u);
            }
        L.li = li0;
    }
    int pc = 0;
    while (pc < R.nops) {
        const uint4* ow = reinterpret_cast<const uint4*>(R.sops + pc);
        const uint4 w0 = ow[0], w1 = ow[1];
        const uint32_t code = w0.x & 0xFFFFu;
        const uint32_t a[7] = { w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w };
        switch (code) {
        case OP_NOP: break;
        case OP_IF: {
            const int d = (int)a[1];
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                const bool aj = (actm >> j) & 1u;
                L.li = li0 + j * blockDim.x;
                const bool c = aj && truth(L, a[0]);
                stk[j] = setbit(stk[j], d, aj);
                cnd[j] = setbit(cnd[j], d, c);
                if (c) nm |= 1u << j;
            }
            L.li = li0;
            actm = nm;
            if (!__any_sync(FULL, actm != 0)) { pc = (int)a[2]; continue; }
            break;
        }
        case OP_ELSE: {
            const int d = (int)a[1];
            const int ll = (int)a[3];
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                const bool off = ((extm | lretm) >> j & 1u) || fret[j] != 0u ||
                                 (ll && (bit(brk[j], ll - 1) || bit(cnt[j], ll - 1)));
                if (bit(stk[j], d) && !bit(cnd[j], d) && !off) nm |= 1u << j;
            }
            actm = nm;
            if (!__any_sync(FULL, actm != 0)) { pc = (int)a[2]; continue; }
            break;
        }
        case OP_ENDIF: {
            const int d = (int)a[1];
            const int ll = (int)a[3];
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                const bool off = ((extm | lretm) >> j & 1u) || fret[j] != 0u ||
                                 (ll && (bit(brk[j], ll - 1) || bit(cnt[j], ll - 1)));
                if (bit(stk[j], d) && !off) nm |= 1u << j;
            }
            actm = nm;
            break;
        }
        case OP_LOOP_BEGIN: {
            const int d = (int)a[1];
            const int ll = (int)a[3];
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                stk[j] = setbit(stk[j], d, (actm >> j) & 1u);
                brk[j] = setbit(brk[j], ll - 1, false);
                cnt[j] = setbit(cnt[j], ll - 1, false);
            }
            break;
        }
        case OP_LOOP_TEST: {
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                L.li = li0 + j * blockDim.x;
                if (((actm >> j) & 1u) && truth(L, a[0])) nm |= 1u << j;
            }
            L.li = li0;
            actm = nm;
            if (!__any_sync(FULL, actm != 0)) { pc = (int)a[2]; continue; }
            break;
        }
        case OP_LOOP_STEP: {
            const int ll = (int)a[3];
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                if ((((actm >> j) & 1u) || bit(cnt[j], ll - 1)) && !bit(brk[j], ll - 1) && !((extm | lretm) >> j & 1u)
                    && fret[j] == 0u)
                    nm |= 1u << j;
                cnt[j] = setbit(cnt[j], ll - 1, false);
            }
            actm = nm;
            break;
        }
        case OP_JUMP: {
            if (a[2] <= (uint32_t)pc) {  // a loop's back edge (as ctl_back_edge)
                bool over = false;
#pragma unroll
                for (int j = 0; j < PPT; ++j)
                    if (((actm >> j) & 1u) && ++iters[j] > R.max_iters) over = true;
                if (__any_sync(FULL, over)) {
                    if (over) raise_status(R.status, ST_TIMEOUT);
                    pc = R.nops;
                    continue;
                }
            }
            pc = (int)a[2];
            continue;
        }
        case OP_LOOP_END: {
            const int d = (int)a[1];
            const int ll = (int)a[3];
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                brk[j] = setbit(brk[j], ll - 1, false);
                cnt[j] = setbit(cnt[j], ll - 1, false);
                // lanes that broke out of an enclosing loop stay off via the
                // enclosing ENDIF/LOOP_STEP recomputation
                if (bit(stk[j], d) && !((extm | lretm) >> j & 1u) && fret[j] == 0u) nm |= 1u << j;
            }
            actm = nm;
            break;
        }
        case OP_FUNC_BEGIN: {  // as ctl_func_begin
            const int d = (int)a[1], f = (int)a[3] - 1;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                stk[j] = setbit(stk[j], d, (actm >> j) & 1u);
                fret[j] = setbit(fret[j], f, false);
            }
            if (!__any_sync(FULL, actm != 0)) { pc = (int)a[2]; continue; }
            break;
        }
        case OP_FUNC_RETURN: {
            const int f = (int)a[3] - 1;
#pragma unroll
            for (int j = 0; j < PPT; ++j)
                if ((actm >> j) & 1u) fret[j] = setbit(fret[j], f, true);
            actm = 0;
            break;
        }
        case OP_FUNC_END: {
            const int d = (int)a[1], f = (int)a[3] - 1;
            uint32_t nm = 0;
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                fret[j] = setbit(fret[j], f, false);
                if (bit(stk[j], d) && !((extm | lretm) >> j & 1u) && fret[j] == 0u) nm |= 1u << j;
            }
            actm = nm;
            break;
        }
        case OP_BREAK: {
            const int ll = (int)a[3];
#pragma unroll
            for (int j = 0; j < PPT; ++j)
                if (((actm >> j) & 1u) && ll) brk[j] = setbit(brk[j], ll - 1, true);
            actm = 0;
            break;
        }
        case OP_CONTINUE: {
            const int ll = (int)a[3];
#pragma unroll
            for (int j = 0; j < PPT; ++j)
                if (((actm >> j) & 1u) && ll) cnt[j] = setbit(cnt[j], ll - 1, true);
            actm = 0;
            break;
        }
        case OP_RETURN: lretm |= actm; actm = 0; break;
        case OP_EXIT: extm |= actm; actm = 0; break;
        case OP_LAYER_END: lretm = 0; actm = validm & ~extm0; break;  // as ctl_layer_end
        case OP_STORES_END: extm0 = extm; actm = a[0] ? validm : validm & ~extm; break;
        default: {
            auto next = [&]() -> const Op* { return pc + 1 < R.nops ? R.sops + pc + 1 : nullptr; };
            uint32_t todo = actm;
#pragma unroll 1
            for (int j = 0; todo; ++j, todo >>= 1) {
                if (!(todo & 1u)) continue;
                L.li = li0 + j * blockDim.x;
                L.pt = pt0 + (int64_t)j * blockDim.x;
                exec_op<TIER>(R, L, code, a, next);
            }
            L.li = li0;
            L.pt = pt0;
            break;
        }
        }
        ++pc;
    }
}


template <bool SMEM, int TIER>
// at least two CTAs of 256 per SM: the register budget is 128 per thread
__global__ void __launch_bounds__(256, 2) interp_kernel(const __grid_constant__ KArgs k) {
    extern __shared__ __align__(16) unsigned char smem[];
    const ProgramHeader* H = reinterpret_cast<const ProgramHeader*>(k.blob);
    const int nops = (int)H->nops, nconst = (int)H->nconst, slots = (int)H->heap_slots;
    Op* sops = reinterpret_cast<Op*>(smem);
    uint32_t* spool = reinterpret_cast<uint32_t*>(smem + (size_t)nops * sizeof(Op));
    float* sheap = reinterpret_cast<float*>(spool + ((nconst + 3) & ~3));
    {
        const uint4* gops = reinterpret_cast<const uint4*>(k.blob + sizeof(ProgramHeader));
        uint4* so = reinterpret_cast<uint4*>(sops);
        for (int i = threadIdx.x; i < nops * 2; i += blockDim.x) so[i] = gops[i];
        const uint32_t* gpool = reinterpret_cast<const uint32_t*>(k.blob + sizeof(ProgramHeader) + (size_t)nops * sizeof(Op));
        for (int i = threadIdx.x; i < nconst; i += blockDim.x) spool[i] = gpool[i];
    }
    __syncthreads();
    RunCtx R;
    R.sops = sops;
    R.nops = nops;
    R.CP.base = H->closure_base;
    R.CP.max_nodes = H->max_comps;
    R.CP.nf = node_floats(*H);
    R.uses_closures = (H->flags & 1u) != 0;
    R.G = &k.G;
    R.userdata = k.userdata;
    R.outputs = k.outputs;
    R.status = k.status;
    R.textures = k.textures;
    R.ntextures = k.ntextures;
    R.max_iters = max_loop_iterations(*H);
    R.symheap = k.symheap;
    R.symheap_stride = k.symheap_stride;

    Lane L;
    L.pool = spool;
    L.hs = blockDim.x;
    L.li = threadIdx.x;
    L.si = k.shadeindex;
    L.heap = SMEM ? sheap : (k.gheap + (size_t)blockIdx.x * (size_t)slots * blockDim.x);

    const int64_t ntiles = (k.npoints + blockDim.x - 1) / blockDim.x;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        L.pt = tile * blockDim.x + threadIdx.x;
        run_tile<TIER>(R, L, k.npoints);
    }
}

// Persistent batch kernel: CTAs take work items (job, tile) from a device
// counter until the list is exhausted, staging each job's program into
// shared memory when the job changes. One launch runs every group of the
// batch; items are ordered so that a CTA mostly stays on one job. A tile is
// blockDim * PPT points; each thread interleaves PPT of them.
template <bool SMEM, int TIER, int MAXT, int PPT>
__global__ void __launch_bounds__(MAXT, 512 / MAXT) batch_kernel(const __grid_constant__ BatchArgs b) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_item;
    Op* sops = reinterpret_cast<Op*>(smem);
    float* sheap = reinterpret_cast<float*>(smem + (size_t)b.prog_bytes);
    const uint32_t tile_pts = blockDim.x * PPT;
    Lane L;
    L.hs = tile_pts;
    L.li = threadIdx.x;
    L.heap = SMEM ? sheap : (b.gheap + (size_t)blockIdx.x * (size_t)b.heap_slots * tile_pts);
    L.pool = nullptr;
    RunCtx R;
    R.sops = sops;
    int cur = -1;
    const uint32_t nitems = b.nitems_dev ? *b.nitems_dev : b.nitems;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        __syncthreads();
        if (it >= nitems) break;
        const uint2 w = b.items[it];
        const BatchJob* J = b.jobs + w.x;
        if ((int)w.x != cur) {
            const ProgramHeader* H = reinterpret_cast<const ProgramHeader*>(J->blob);
            const int nops = (int)H->nops, nconst = (int)H->nconst;
            uint32_t* spool = reinterpret_cast<uint32_t*>(smem + (size_t)nops * sizeof(Op));
            const uint4* gops = reinterpret_cast<const uint4*>(J->blob + sizeof(ProgramHeader));
            uint4* so = reinterpret_cast<uint4*>(sops);
            for (int i = threadIdx.x; i < nops * 2; i += blockDim.x) so[i] = gops[i];
            const uint32_t* gpool = reinterpret_cast<const uint32_t*>(J->blob + sizeof(ProgramHeader) + (size_t)nops * sizeof(Op));
            for (int i = threadIdx.x; i < nconst; i += blockDim.x) spool[i] = gpool[i];
            __syncthreads();
            R.nops = nops;
            R.CP.base = H->closure_base;
            R.CP.max_nodes = H->max_comps;
            R.CP.nf = node_floats(*H);
            R.uses_closures = (H->flags & 1u) != 0;
            R.G = &J->G;
            R.userdata = J->userdata;
            R.outputs = J->outputs;
            R.status = J->status ? J->status : b.status;
            R.textures = b.textures;
            R.ntextures = b.ntextures;
            R.max_iters = max_loop_iterations(*H);
            L.pool = spool;
            cur = (int)w.x;
        }
        L.li = threadIdx.x;
        L.pt = (int64_t)w.y * tile_pts + threadIdx.x;
        run_tile<TIER, PPT>(R, L, J->npoints);
    }
}

}  // namespace dev
}  // namespace oslg
