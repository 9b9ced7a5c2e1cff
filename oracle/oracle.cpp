// ORACLE — test infrastructure only. Not part of the shipped library; only
// the tests, the smoke check and the CPU-baseline leg of bench.py load it.
//
// CPU restatement of OSL's batched execution semantics for one lowered
// shader group, used to check the GPU interpreter point for point:
//   * control flow runs per point with a real program counter (jumps), the
//     scalar reading of what the batched backend does with lane masks
//     (src/liboslexec/batched_llvm_gen.cpp:1068 if, :3806-4250 loops and
//     break/continue; src/liboslexec/llvm_gen.cpp for the scalar ops);
//   * op results follow the reference's shadeops: Dual2 arithmetic
//     (src/include/OSL/dual.h), vector ops (dual_vec.h), noise
//     (oslnoise.h, simplexnoise.cpp), min/max/clamp selection
//     (llvm_gen.cpp:1345-1380, :1170-1210), normalize/length/distance
//     (llvm_ops.cpp:850-915), transforms (dual_vec.h:336-400).
// Transcendental functions are evaluated in double precision and rounded to
// float (correctly rounded results), the same definition the device uses.
// It reads the op-program format (openshadinglanguage_gb300/csrc/
// oslg_program.h) as a file format; it shares no code with the executor.
//
// Build: oracle/build.py (g++ -O2 -ffp-contract=off -fopenmp).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../include/oslg.h"
#include "../openshadinglanguage_gb300/csrc/oslg_program.h"
#include "oracle_bsdf.h"
#include "oracle_fastmath.h"
#include "oracle_gabor.h"
#include "oracle_shading.h"
#include "oracle_simplex.h"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace oracle;
using oslg::Op;

namespace {

struct Prog {
    const oslg::ProgramHeader* h;
    const Op* ops;
    const uint32_t* pool;
    // control-flow partners, resolved once
    std::vector<int> loop_end_of_level;  // per op: for BREAK/CONTINUE
    std::vector<int> partner;            // IF->ELSE, ELSE->ENDIF, LOOP_TEST->LOOP_END
    std::vector<int> break_target, continue_target;
    std::vector<int> layer_end_after;    // RETURN, EXIT -> the layer's LAYER_END
    int final_section = 0;               // the STORES_END that opens the renderer-side section
};

struct Point {
    std::vector<uint32_t> heap;
    const uint32_t* pool;
    int64_t pt;
    uint32_t status = 0;
};

inline uint32_t aoff(uint32_t a) { return a & oslg::kArgOffsetMask; }
inline bool aconst(uint32_t a) { return (a & oslg::kArgConst) != 0; }
inline bool ader(uint32_t a) { return (a & oslg::kArgDerivs) != 0; }
inline uint32_t atc(uint32_t a) { return (a >> oslg::kArgTCShift) & 7u; }
inline int anc(uint32_t a) {
    uint32_t t = atc(a);
    return t == oslg::TC_TRIPLE ? 3 : (t == oslg::TC_MATRIX ? 16 : 1);
}

inline uint32_t word(const Point& P, uint32_t a, int idx) {
    uint32_t o = aoff(a) + (uint32_t)idx;
    return aconst(a) ? P.pool[o] : P.heap[o];
}
inline void setw(Point& P, uint32_t a, int idx, uint32_t v) { P.heap[aoff(a) + (uint32_t)idx] = v; }
inline void setf(Point& P, uint32_t a, int idx, float v) { setw(P, a, idx, fbits(v)); }

// component c (scalars broadcast) of value / x / y partial; ints convert
inline float getf(const Point& P, uint32_t a, int c, int d) {
    int nc = anc(a);
    if (d && !ader(a)) return 0.0f;
    uint32_t w = word(P, a, d * nc + (nc == 1 ? 0 : c));
    return atc(a) == oslg::TC_INT ? (float)(int32_t)w : bitsf(w);
}
inline DF getd(const Point& P, uint32_t a, int c) { return DF(getf(P, a, c, 0), getf(P, a, c, 1), getf(P, a, c, 2)); }
inline int geti(const Point& P, uint32_t a, int c) {
    uint32_t t = atc(a);
    uint32_t w = word(P, a, t == oslg::TC_TRIPLE ? c : 0);
    if (t == oslg::TC_FLOAT || t == oslg::TC_TRIPLE) return (int)bitsf(w);
    return (int32_t)w;
}
// store a dual into component c of r; only the value if r has no partials
inline void putd(Point& P, uint32_t r, int c, const DF& v) {
    if (atc(r) == oslg::TC_INT) { setw(P, r, c, (uint32_t)(int)v.v); return; }
    int nc = anc(r);
    setf(P, r, c, v.v);
    if (ader(r)) { setf(P, r, nc + c, v.dx); setf(P, r, 2 * nc + c, v.dy); }
}
inline void putv(Point& P, uint32_t r, int c, float v) { putd(P, r, c, DF(v)); }

// ---- math: correctly rounded through double --------------------------------
inline float f_sin(float x) { return (float)std::sin((double)x); }
inline float f_cos(float x) { return (float)std::cos((double)x); }
const float kMin = FLT_MIN;
// OpenImageIO fast_logb (fmath.h; OpenImageIO 2.5, the host branch the
// reference's logb calls, llvm_ops.cpp:542-545): exponent of |x| clamped
// to the normal float range
inline float fast_logb(float x) {
    x = std::fabs(x);
    if (x < FLT_MIN) x = FLT_MIN;
    if (x > FLT_MAX) x = FLT_MAX;
    uint32_t bits;
    std::memcpy(&bits, &x, 4);
    return (float)((int)(bits >> 23) - 127);
}
// OIIO safe_log / safe_pow / safe_fmod
inline float safe_log(float x) { return (float)std::log((double)(x < kMin ? kMin : x)); }
inline float safe_log2(float x) { return (float)std::log2((double)(x < kMin ? kMin : x)); }
inline float safe_log10(float x) { return (float)std::log10((double)(x < kMin ? kMin : x)); }
inline float safe_pow(float x, float y) {
    if (y == 0.0f) return 1.0f;
    if (x == 0.0f) return 0.0f;
    if (x < 0.0f && y != std::floor(y)) return 0.0f;
    float r = (float)std::pow((double)x, (double)y);
    return std::min(std::max(r, -FLT_MAX), FLT_MAX);
}
inline float safe_fmod(float a, float b) {
    if (b != 0.0f) {
        int N = (int)(a / b);
        return a - (float)N * b;
    }
    return 0.0f;
}

// dualfunc (dual.h:760-775)
inline DF dualfunc(const DF& u, float f, float df) { return DF(f, df * u.dx, df * u.dy); }

// ---- ops -------------------------------------------------------------------------
void op_assign(Point& P, const uint32_t* a) {
    uint32_t r = a[0], s = a[1];
    uint32_t tr = atc(r), ts = atc(s);
    if (tr == oslg::TC_CLOSURE) { setw(P, r, 0, ts == oslg::TC_CLOSURE ? word(P, s, 0) : 0u); return; }
    if (tr == oslg::TC_STRING) { setw(P, r, 0, word(P, s, 0)); return; }
    if (tr == oslg::TC_MATRIX) {
        if (ts == oslg::TC_MATRIX) for (int i = 0; i < 16; ++i) setw(P, r, i, word(P, s, i));
        else {
            float v = getf(P, s, 0, 0);
            for (int i = 0; i < 16; ++i) setf(P, r, i, i % 5 == 0 ? v : 0.0f);
        }
        return;
    }
    int count = (int)a[2], ralen = std::max(1, (int)a[3]), salen = std::max(1, (int)a[4]);
    int nr = anc(r), ns = anc(s);
    for (int e = 0; e < count; ++e)
        for (int c = 0; c < nr; ++c) {
            int sc = ns == 1 ? 0 : c;
            uint32_t sw = word(P, s, e * ns + sc);
            if (tr == oslg::TC_INT) {
                setw(P, r, e * nr + c, (uint32_t)(ts == oslg::TC_INT ? (int32_t)sw : (int)bitsf(sw)));
                continue;
            }
            setf(P, r, e * nr + c, ts == oslg::TC_INT ? (float)(int32_t)sw : bitsf(sw));
            if (ader(r)) {
                float dx = 0, dy = 0;
                if (ader(s)) {
                    dx = bitsf(word(P, s, salen * ns + e * ns + sc));
                    dy = bitsf(word(P, s, 2 * salen * ns + e * ns + sc));
                }
                setf(P, r, ralen * nr + e * nr + c, dx);
                setf(P, r, 2 * ralen * nr + e * nr + c, dy);
            }
        }
}

// add / sub / mul / div / mod with dual.h semantics per operand kind
void op_arith(Point& P, const uint32_t* a, int K) {
    uint32_t r = a[0], x = a[1], y = a[2];
    int nc = anc(r);
    for (int c = 0; c < nc; ++c) {
        float xv = getf(P, x, c, 0), yv = getf(P, y, c, 0);
        DF X(xv, getf(P, x, c, 1), getf(P, x, c, 2)), Y(yv, getf(P, y, c, 1), getf(P, y, c, 2));
        bool xd = ader(x), yd = ader(y);
        DF res;
        switch (K) {
        case 0:
            if (xd && yd) res = X + Y;
            else if (xd) res = X + yv;
            else if (yd) res = xv + Y;
            else res = DF(xv + yv);
            break;
        case 1:
            if (xd && yd) res = X - Y;
            else if (xd) res = X - yv;
            else if (yd) res = xv - Y;
            else res = DF(xv - yv);
            break;
        case 2:
            if (xd && yd) res = X * Y;
            else if (xd) res = X * yv;
            else if (yd) res = Y * xv;
            else res = DF(xv * yv);
            break;
        case 3:
            // safe division (the reference's div codegen returns 0 for x/0)
            if (yv == 0.0f) res = DF(0.0f);
            else if (xd && yd) res = X / Y;
            else if (xd) res = X / yv;
            else if (yd) res = xv / Y;
            else res = DF(xv / yv);
            break;
        default:
            res = DF(yv == 0.0f ? 0.0f : std::fmod(xv, yv), X.dx, X.dy);
            break;
        }
        if (atc(r) == oslg::TC_INT) { setw(P, r, c, (uint32_t)(int)res.v); continue; }
        putd(P, r, c, res);
    }
}

void op_iarith(Point& P, const uint32_t* a, int K) {
    int x = geti(P, a[1], 0), y = geti(P, a[2], 0), v;
    switch (K) {
    case 0: v = (int)((uint32_t)x + (uint32_t)y); break;
    case 1: v = (int)((uint32_t)x - (uint32_t)y); break;
    case 2: v = (int)((uint32_t)x * (uint32_t)y); break;
    case 3: v = (y == 0 || (x == INT32_MIN && y == -1)) ? 0 : x / y; break;
    default: v = (y == 0 || (x == INT32_MIN && y == -1)) ? 0 : x % y; break;
    }
    setw(P, a[0], 0, (uint32_t)v);
}

bool truth(const Point& P, uint32_t a) {
    uint32_t t = atc(a);
    if (t == oslg::TC_FLOAT) return getf(P, a, 0, 0) != 0.0f;
    if (t == oslg::TC_TRIPLE) return getf(P, a, 0, 0) != 0.0f || getf(P, a, 1, 0) != 0.0f || getf(P, a, 2, 0) != 0.0f;
    return word(P, a, 0) != 0u;
}

void op_cmp(Point& P, const uint32_t* a, int K) {
    uint32_t x = a[1], y = a[2];
    bool ints = (atc(x) == oslg::TC_INT || atc(x) == oslg::TC_STRING)
             && (atc(y) == oslg::TC_INT || atc(y) == oslg::TC_STRING);
    bool res;
    if (ints) {
        int32_t xi = (int32_t)word(P, x, 0), yi = (int32_t)word(P, y, 0);
        const bool rs[6] = { xi == yi, xi != yi, xi < yi, xi > yi, xi <= yi, xi >= yi };
        res = rs[K];
    } else if (K <= 1) {
        int n = std::max(anc(x), anc(y));
        bool eq = true;
        for (int c = 0; c < n; ++c) eq = eq && getf(P, x, c, 0) == getf(P, y, c, 0);
        res = K == 0 ? eq : !eq;
    } else {
        float xv = getf(P, x, 0, 0), yv = getf(P, y, 0, 0);
        const bool rs[6] = { false, false, xv < yv, xv > yv, xv <= yv, xv >= yv };
        res = rs[K];
    }
    setw(P, a[0], 0, res ? 1u : 0u);
}

// unary math per component (dual.h:829-1260 derivative rules)
// OpenImageIO fast_* forms with dual.h's fast_* derivative rules
// (dual.h:836-1262); false when the op has none
bool unary_fast(uint16_t code, const DF& X, DF& res) {
    namespace F = oracle_fm;
    const float v = X.v;
    switch (code) {
    case oslg::OP_SIN: { float s, c; F::sincosf_(v, s, c); res = dualfunc(X, s, c); return true; }
    case oslg::OP_COS: { float s, c; F::sincosf_(v, s, c); res = dualfunc(X, c, -s); return true; }
    case oslg::OP_TAN: { float cs = F::cosf_(v); res = dualfunc(X, F::tanf_(v), 1.0f / (cs * cs)); return true; }
    case oslg::OP_ASIN:
        res = dualfunc(X, F::asinf_(v), std::fabs(v) < 1.0f ? 1.0f / std::sqrt(1.0f - v * v) : 0.0f);
        return true;
    case oslg::OP_ACOS:
        res = dualfunc(X, F::acosf_(v), std::fabs(v) < 1.0f ? -1.0f / std::sqrt(1.0f - v * v) : 0.0f);
        return true;
    case oslg::OP_ATAN: res = dualfunc(X, F::atanf_(v), 1.0f / (1.0f + v * v)); return true;
    case oslg::OP_SINH: res = dualfunc(X, F::sinhf_(v), F::coshf_(v)); return true;
    case oslg::OP_COSH: res = dualfunc(X, F::coshf_(v), F::sinhf_(v)); return true;
    case oslg::OP_TANH: { float ch = F::coshf_(v); res = dualfunc(X, F::tanhf_(v), 1.0f / (ch * ch)); return true; }
    case oslg::OP_EXP: { float f = F::expf_(v); res = dualfunc(X, f, f); return true; }
    case oslg::OP_EXP2: { float f = F::exp2f_(v); res = dualfunc(X, f, f * 0.693147180559945309417f); return true; }
    case oslg::OP_EXPM1: res = dualfunc(X, F::expm1f_(v), F::expf_(v)); return true;
    case oslg::OP_LOG: res = dualfunc(X, F::logf_(v), v < kMin ? 0.0f : 1.0f / v); return true;
    case oslg::OP_LOG2: {
        float aln2 = v * 0.693147180559945309417f;
        res = dualfunc(X, F::log2f_(v), aln2 < kMin ? 0.0f : 1.0f / aln2);
        return true;
    }
    case oslg::OP_LOG10: {
        float aln10 = v * 2.30258509299404568402f;
        res = dualfunc(X, F::log10f_(v), aln10 < kMin ? 0.0f : 1.0f / aln10);
        return true;
    }
    case oslg::OP_ERF: res = dualfunc(X, F::erff_(v), F::expf_(-v * v) * 1.12837916709551257390f); return true;
    case oslg::OP_ERFC: res = dualfunc(X, F::erfcf_(v), F::expf_(-v * v) * -1.12837916709551257390f); return true;
    case oslg::OP_CBRT:
        if (v != 0.0f) { float f = F::cbrtf_(v); res = dualfunc(X, f, 1.0f / (3.0f * f * f)); }
        else res = DF(0.0f);
        return true;
    default: return false;
    }
}

void op_unary(Point& P, const uint32_t* a, uint16_t code) {
    uint32_t r = a[0], x = a[1];
    int nc = anc(r);
    for (int c = 0; c < nc; ++c) {
        DF X = getd(P, x, c);
        float v = X.v;
        DF res;
        bool has = ader(x);
        if (!(a[2] == 1u && unary_fast(code, X, res)))
        switch (code) {
        case oslg::OP_NEG: res = -X; break;
        case oslg::OP_ABS: res = v >= 0.0f ? DF(std::fabs(v), X.dx, X.dy) : -X; break;
        case oslg::OP_FLOOR: res = DF(std::floor(v)); break;
        case oslg::OP_CEIL: res = DF(std::ceil(v)); break;
        case oslg::OP_ROUND: res = DF(std::round(v)); break;
        case oslg::OP_TRUNC: res = DF(std::trunc(v)); break;
        case oslg::OP_SIGN: res = DF(v < 0.0f ? -1.0f : (v == 0.0f ? 0.0f : 1.0f)); break;
        case oslg::OP_SQRT:
            if (v > 0.0f) { float f = std::sqrt(v); res = dualfunc(X, f, 0.5f / f); } else res = DF(0.0f);
            break;
        case oslg::OP_INVSQRT:
            if (v > 0.0f) { float f = 1.0f / std::sqrt(v); res = dualfunc(X, f, -0.5f * f / v); } else res = DF(0.0f);
            break;
        case oslg::OP_CBRT:
            if (v != 0.0f) { float f = (float)std::cbrt((double)v); res = dualfunc(X, f, 1.0f / (3.0f * f * f)); }
            else res = DF(0.0f);
            break;
        case oslg::OP_SIN: res = dualfunc(X, f_sin(v), f_cos(v)); break;
        case oslg::OP_COS: res = dualfunc(X, f_cos(v), -f_sin(v)); break;
        case oslg::OP_TAN: { float cs = f_cos(v); res = dualfunc(X, (float)std::tan((double)v), 1.0f / (cs * cs)); break; }
        case oslg::OP_ASIN:
            if (v >= 1.0f) res = DF(1.57079632679489661923f);
            else if (v <= -1.0f) res = DF(-1.57079632679489661923f);
            else res = dualfunc(X, (float)std::asin((double)v), 1.0f / std::sqrt(1.0f - v * v));
            break;
        case oslg::OP_ACOS:
            if (v >= 1.0f) res = DF(0.0f);
            else if (v <= -1.0f) res = DF(3.14159265358979323846f);
            else res = dualfunc(X, (float)std::acos((double)v), -1.0f / std::sqrt(1.0f - v * v));
            break;
        case oslg::OP_ATAN: res = dualfunc(X, (float)std::atan((double)v), 1.0f / (1.0f + v * v)); break;
        case oslg::OP_SINH: res = dualfunc(X, (float)std::sinh((double)v), (float)std::cosh((double)v)); break;
        case oslg::OP_COSH: res = dualfunc(X, (float)std::cosh((double)v), (float)std::sinh((double)v)); break;
        case oslg::OP_TANH: {
            float ch = (float)std::cosh((double)v);
            res = dualfunc(X, (float)std::tanh((double)v), 1.0f / (ch * ch));
            break;
        }
        case oslg::OP_EXP: { float f = (float)std::exp((double)v); res = dualfunc(X, f, f); break; }
        case oslg::OP_EXP2: { float f = (float)std::exp2((double)v); res = dualfunc(X, f, f * 0.693147180559945309417f); break; }
        case oslg::OP_EXPM1: res = dualfunc(X, (float)std::expm1((double)v), (float)std::exp((double)v)); break;
        case oslg::OP_LOG: res = dualfunc(X, safe_log(v), v < kMin ? 0.0f : 1.0f / v); break;
        case oslg::OP_LOG2: res = dualfunc(X, safe_log2(v), v < kMin ? 0.0f : 1.0f / (v * 0.693147180559945309417f)); break;
        case oslg::OP_LOG10: res = dualfunc(X, safe_log10(v), v < kMin ? 0.0f : 1.0f / (v * 2.30258509299404568402f)); break;
        case oslg::OP_LOGB: res = DF(fast_logb(v)); break;
        case oslg::OP_ERF:  // dual.h:1170-1179
            res = dualfunc(X, (float)std::erf((double)v), (float)std::exp((double)(-v * v)) * 1.12837916709551257390f);
            break;
        case oslg::OP_ERFC:  // dual.h:1190-1199
            res = dualfunc(X, (float)std::erfc((double)v), -1.12837916709551257390f * (float)std::exp((double)(-v * v)));
            break;
        case oslg::OP_RADIANS: res = X * (3.14159265358979323846f / 180.0f); break;
        case oslg::OP_DEGREES: res = X * (180.0f / 3.14159265358979323846f); break;
        default: res = X; break;
        }
        if (!has && res.dx != 0.0f) res.dx = 0.0f;
        if (!has && res.dy != 0.0f) res.dy = 0.0f;
        if (atc(r) == oslg::TC_INT) { setw(P, r, c, (uint32_t)(int)res.v); continue; }
        putd(P, r, c, res);
    }
}

void op_binary(Point& P, const uint32_t* a, uint16_t code) {
    uint32_t r = a[0], x = a[1], y = a[2];
    int nc = anc(r);
    bool rd = ader(r);
    const bool fast = a[3] == 1u;  // pow, atan2
    for (int c = 0; c < nc; ++c) {
        DF u = getd(P, x, c), v = getd(P, y, c);
        DF res;
        switch (code) {
        case oslg::OP_POW:
            if (rd && (ader(x) || ader(y))) {
                // dual.h:1059-1067, fast form 1072-1080
                float powuvm1 = fast ? oracle_fm::safe_powf_(u.v, v.v - 1.0f) : safe_pow(u.v, v.v - 1.0f);
                float powuv = powuvm1 * u.v;
                float logu = u.v > 0.0f ? (fast ? oracle_fm::logf_(u.v) : safe_log(u.v)) : 0.0f;
                float du = v.v * powuvm1, dv = logu * powuv;
                res = DF(powuv, du * u.dx + dv * v.dx, du * u.dy + dv * v.dy);
            } else {
                res = DF(fast ? oracle_fm::safe_powf_(u.v, v.v) : safe_pow(u.v, v.v));
            }
            break;
        case oslg::OP_ATAN2: {
            // dual.h:1018-1023 (y = first operand), fast form 1025-1031
            float f = fast ? oracle_fm::atan2f_(u.v, v.v) : (float)std::atan2((double)u.v, (double)v.v);
            float denom = (v.v == 0.0f && u.v == 0.0f) ? 0.0f : 1.0f / (v.v * v.v + u.v * u.v);
            float dfdy = -v.v * denom, dfdx = u.v * denom;
            res = DF(f, dfdy * u.dx + dfdx * v.dx, dfdy * u.dy + dfdx * v.dy);
            break;
        }
        case oslg::OP_FMOD: res = DF(safe_fmod(u.v, v.v), u.dx, u.dy); break;
        case oslg::OP_MIN: res = u.v <= v.v ? u : v; break;
        case oslg::OP_MAX: res = u.v > v.v ? u : v; break;
        default: res = DF(v.v < u.v ? 0.0f : 1.0f); break;  // step(edge, x)
        }
        if (!rd) { putv(P, r, c, res.v); continue; }
        putd(P, r, c, res);
    }
}

void op_dot(Point& P, const uint32_t* a) {
    DF ax = getd(P, a[1], 0), ay = getd(P, a[1], 1), az = getd(P, a[1], 2);
    DF bx = getd(P, a[2], 0), by = getd(P, a[2], 1), bz = getd(P, a[2], 2);
    if (!ader(a[0])) { putv(P, a[0], 0, ax.v * bx.v + ay.v * by.v + az.v * bz.v); return; }
    putd(P, a[0], 0, ax * bx + ay * by + az * bz);
}
void op_cross(Point& P, const uint32_t* a) {
    DF ax = getd(P, a[1], 0), ay = getd(P, a[1], 1), az = getd(P, a[1], 2);
    DF bx = getd(P, a[2], 0), by = getd(P, a[2], 1), bz = getd(P, a[2], 2);
    if (!ader(a[0])) {
        putv(P, a[0], 0, ay.v * bz.v - az.v * by.v);
        putv(P, a[0], 1, az.v * bx.v - ax.v * bz.v);
        putv(P, a[0], 2, ax.v * by.v - ay.v * bx.v);
        return;
    }
    putd(P, a[0], 0, ay * bz - az * by);
    putd(P, a[0], 1, az * bx - ax * bz);
    putd(P, a[0], 2, ax * by - ay * bx);
}
inline DF dsqrt(const DF& a) {
    if (a.v > 0.0f) { float f = std::sqrt(a.v); return dualfunc(a, f, 0.5f / f); }
    return DF(0.0f);
}
// Imath Vec3<float>::length()
float imath_length(float x, float y, float z) {
    float l2 = x * x + y * y + z * z;
    if (l2 < 2.0f * FLT_MIN) {
        float m = std::max(std::fabs(x), std::max(std::fabs(y), std::fabs(z)));
        if (m == 0.0f) return 0.0f;
        x /= m; y /= m; z /= m;
        return m * std::sqrt(x * x + y * y + z * z);
    }
    return std::sqrt(l2);
}
void op_length(Point& P, const uint32_t* a, bool distance) {
    DF x = getd(P, a[1], 0), y = getd(P, a[1], 1), z = getd(P, a[1], 2);
    if (distance) { x = x - getd(P, a[2], 0); y = y - getd(P, a[2], 1); z = z - getd(P, a[2], 2); }
    if (!ader(a[0])) {
        putv(P, a[0], 0, distance ? std::sqrt(x.v * x.v + y.v * y.v + z.v * z.v) : imath_length(x.v, y.v, z.v));
        return;
    }
    putd(P, a[0], 0, dsqrt(x * x + y * y + z * z));
}
void op_normalize(Point& P, const uint32_t* a) {
    DF x = getd(P, a[1], 0), y = getd(P, a[1], 1), z = getd(P, a[1], 2);
    if (!ader(a[0])) {
        float len = std::sqrt(x.v * x.v + y.v * y.v + z.v * z.v);
        float inv = len > 0.0f ? 1.0f / len : 0.0f;
        if (len > 0.0f) { putv(P, a[0], 0, x.v * inv); putv(P, a[0], 1, y.v * inv); putv(P, a[0], 2, z.v * inv); }
        else for (int c = 0; c < 3; ++c) putv(P, a[0], c, 0.0f);
        return;
    }
    DF len = dsqrt(x * x + y * y + z * z);
    if (len.v > 0.0f) {
        DF inv = 1.0f / len;
        putd(P, a[0], 0, x * inv); putd(P, a[0], 1, y * inv); putd(P, a[0], 2, z * inv);
    } else {
        for (int c = 0; c < 3; ++c) putd(P, a[0], c, DF(0.0f));
    }
}
void op_transform(Point& P, const uint32_t* a) {
    uint32_t r = a[0], p = a[1], m = a[2];
    float M[4][4];
    for (int i = 0; i < 16; ++i) M[i / 4][i % 4] = bitsf(word(P, m, i));
    DF x = getd(P, p, 0), y = getd(P, p, 1), z = getd(P, p, 2);
    if (a[3] == 0) {
        if (!ader(r)) {
            float A = x.v * M[0][0] + y.v * M[1][0] + z.v * M[2][0] + M[3][0];
            float B = x.v * M[0][1] + y.v * M[1][1] + z.v * M[2][1] + M[3][1];
            float C = x.v * M[0][2] + y.v * M[1][2] + z.v * M[2][2] + M[3][2];
            float W = x.v * M[0][3] + y.v * M[1][3] + z.v * M[2][3] + M[3][3];
            if (W != 0.0f) { putv(P, r, 0, A / W); putv(P, r, 1, B / W); putv(P, r, 2, C / W); }
            else for (int c = 0; c < 3; ++c) putv(P, r, c, 0.0f);
            return;
        }
        DF A = x * M[0][0] + y * M[1][0] + z * M[2][0] + M[3][0];
        DF B = x * M[0][1] + y * M[1][1] + z * M[2][1] + M[3][1];
        DF C = x * M[0][2] + y * M[1][2] + z * M[2][2] + M[3][2];
        DF W = x * M[0][3] + y * M[1][3] + z * M[2][3] + M[3][3];
        if (W.v != 0.0f) { putd(P, r, 0, A / W); putd(P, r, 1, B / W); putd(P, r, 2, C / W); }
        else for (int c = 0; c < 3; ++c) putd(P, r, c, DF(0.0f));
        return;
    }
    float in[3][3] = { { x.v, y.v, z.v }, { x.dx, y.dx, z.dx }, { x.dy, y.dy, z.dy } };
    int nd = ader(r) ? 3 : 1;
    for (int d = 0; d < nd; ++d) {
        float X = in[d][0], Y = in[d][1], Z = in[d][2];
        setf(P, r, d * 3 + 0, X * M[0][0] + Y * M[1][0] + Z * M[2][0]);
        setf(P, r, d * 3 + 1, X * M[0][1] + Y * M[1][1] + Z * M[2][1]);
        setf(P, r, d * 3 + 2, X * M[0][2] + Y * M[1][2] + Z * M[2][2]);
    }
}

// 4x4 inverse by Gauss-Jordan elimination with partial pivoting; singular
// gives the identity (Imath's inverse() with exceptions off). Imath is not
// in the reference tree, so inverse-dependent results (matrix division,
// transformn) are pinned to this algorithm, not to Imath's bits.
void m44_inverse(const float* A, float* out) {
    float t[16], s[16];
    for (int i = 0; i < 16; ++i) { t[i] = A[i]; s[i] = (i % 5 == 0) ? 1.0f : 0.0f; }
    for (int i = 0; i < 4; ++i) {
        int piv = i;
        float pmax = std::fabs(t[i * 4 + i]);
        for (int j = i + 1; j < 4; ++j)
            if (std::fabs(t[j * 4 + i]) > pmax) { pmax = std::fabs(t[j * 4 + i]); piv = j; }
        if (pmax == 0.0f) {
            for (int k = 0; k < 16; ++k) out[k] = (k % 5 == 0) ? 1.0f : 0.0f;
            return;
        }
        if (piv != i)
            for (int k = 0; k < 4; ++k) {
                std::swap(t[i * 4 + k], t[piv * 4 + k]);
                std::swap(s[i * 4 + k], s[piv * 4 + k]);
            }
        for (int j = 0; j < 4; ++j) {
            if (j == i) continue;
            float f = t[j * 4 + i] / t[i * 4 + i];
            for (int k = 0; k < 4; ++k) {
                t[j * 4 + k] = t[j * 4 + k] - f * t[i * 4 + k];
                s[j * 4 + k] = s[j * 4 + k] - f * s[i * 4 + k];
            }
        }
    }
    for (int i = 0; i < 4; ++i) {
        float f = t[i * 4 + i];
        for (int k = 0; k < 4; ++k) out[i * 4 + k] = s[i * 4 + k] / f;
    }
}
void m44_mul(const float* A, const float* B, float* out) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
            out[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j] + A[i * 4 + 2] * B[2 * 4 + j]
                           + A[i * 4 + 3] * B[3 * 4 + j];
}
// Imathx.h:456-492
inline float det2(float a, float b, float c, float d) { return a * d - b * c; }
inline float det3(float a1, float a2, float a3, float b1, float b2, float b3, float c1, float c2, float c3) {
    return a1 * det2(b2, b3, c2, c3) - b1 * det2(a2, a3, c2, c3) + c1 * det2(a2, a3, b2, b3);
}
float det4(const float* m) {
    float a1 = m[0], b1 = m[1], c1 = m[2], d1 = m[3];
    float a2 = m[4], b2 = m[5], c2 = m[6], d2 = m[7];
    float a3 = m[8], b3 = m[9], c3 = m[10], d3 = m[11];
    float a4 = m[12], b4 = m[13], c4 = m[14], d4 = m[15];
    return a1 * det3(b2, b3, b4, c2, c3, c4, d2, d3, d4) - b1 * det3(a2, a3, a4, c2, c3, c4, d2, d3, d4)
         + c1 * det3(a2, a3, a4, b2, b3, b4, d2, d3, d4) - d1 * det3(a2, a3, a4, b2, b3, b4, c2, c3, c4);
}

// matrix division (src/liboslexec/opmatrix.cpp:49-73)
void op_mdiv(Point& P, const uint32_t* a) {
    uint32_t r = a[0], x = a[1], y = a[2];
    float out[16];
    bool mx = atc(x) == oslg::TC_MATRIX, my = atc(y) == oslg::TC_MATRIX;
    if (mx && my) {
        float A[16], B[16], Bi[16];
        for (int i = 0; i < 16; ++i) { A[i] = bitsf(word(P, x, i)); B[i] = bitsf(word(P, y, i)); }
        m44_inverse(B, Bi);
        m44_mul(A, Bi, out);
    } else if (mx) {
        float f = 1.0f / getf(P, y, 0, 0);
        for (int i = 0; i < 16; ++i) out[i] = bitsf(word(P, x, i)) * f;
    } else if (my) {
        float B[16], Bi[16];
        for (int i = 0; i < 16; ++i) B[i] = bitsf(word(P, y, i));
        m44_inverse(B, Bi);
        float f = getf(P, x, 0, 0);
        for (int i = 0; i < 16; ++i) out[i] = Bi[i] * f;
    } else {
        float av = getf(P, x, 0, 0), bv = getf(P, y, 0, 0);
        float f = (bv == 0.0f) ? 0.0f : (av / bv);
        for (int i = 0; i < 16; ++i) out[i] = (i % 5 == 0) ? f : 0.0f;
    }
    for (int i = 0; i < 16; ++i) setf(P, r, i, out[i]);
}

// transformn: multDirMatrix by the transposed inverse (opmatrix.cpp:122-137)
void op_transformn(Point& P, const uint32_t* a) {
    uint32_t r = a[0], p = a[1], m = a[2];
    float M[16], Mi[16], T[16];
    for (int i = 0; i < 16; ++i) M[i] = bitsf(word(P, m, i));
    m44_inverse(M, Mi);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) T[i * 4 + j] = Mi[j * 4 + i];
    int nd = ader(r) ? 3 : 1;
    for (int d = 0; d < nd; ++d) {
        float X = getf(P, p, 0, d), Y = getf(P, p, 1, d), Z = getf(P, p, 2, d);
        setf(P, r, d * 3 + 0, X * T[0] + Y * T[4] + Z * T[8]);
        setf(P, r, d * 3 + 1, X * T[1] + Y * T[5] + Z * T[9]);
        setf(P, r, d * 3 + 2, X * T[2] + Y * T[6] + Z * T[10]);
    }
}

// area (llvm_ops.cpp:915-941): length of cross(dPdx, dPdy); filterwidth
// (:944-965): sqrt(dx*dx + dy*dy) per component
void op_area(Point& P, const uint32_t* a) {
    V3 dx(getf(P, a[1], 0, 1), getf(P, a[1], 1, 1), getf(P, a[1], 2, 1));
    V3 dy(getf(P, a[1], 0, 2), getf(P, a[1], 1, 2), getf(P, a[1], 2, 2));
    putv(P, a[0], 0, v3_length(v3_cross(dx, dy)));
}
// sincos (llvm_ops.cpp:298-430): a0 = x, a1 = sine, a2 = cosine
void op_sincos(Point& P, const uint32_t* a) {
    const uint32_t x = a[0], rs = a[1], rc = a[2];
    const int nc = anc(x);
    for (int c = 0; c < nc; ++c) {
        const float v = getf(P, x, c, 0), xdx = getf(P, x, c, 1), xdy = getf(P, x, c, 2);
        float sv, cv;
        if (a[3] == 1u) oracle_fm::sincosf_(v, sv, cv);
        else { sv = f_sin(v); cv = f_cos(v); }
        setf(P, rs, c, sv);
        setf(P, rc, c, cv);
        if (ader(rs)) { setf(P, rs, nc + c, cv * xdx); setf(P, rs, 2 * nc + c, cv * xdy); }
        if (ader(rc)) { setf(P, rc, nc + c, -sv * xdx); setf(P, rc, 2 * nc + c, -sv * xdy); }
    }
}
void op_filterwidth(Point& P, const uint32_t* a) {
    for (int c = 0; c < anc(a[1]); ++c) {
        float dx = getf(P, a[1], c, 1), dy = getf(P, a[1], c, 2);
        putv(P, a[0], c, std::sqrt(dx * dx + dy * dy));
    }
}
// luminance (opcolor.cpp:461-476, opcolor.h:59-62); a2 = scale triple
void op_luminance(Point& P, const uint32_t* a) {
    float sx = getf(P, a[2], 0, 0), sy = getf(P, a[2], 1, 0), sz = getf(P, a[2], 2, 0);
    int nd = ader(a[0]) ? 3 : 1;
    for (int d = 0; d < nd; ++d) setf(P, a[0], d, getf(P, a[1], 0, d) * sx + getf(P, a[1], 1, d) * sy + getf(P, a[1], 2, d) * sz);
}

// ---- colour spaces: ColorSystem::transformc (opcolor.cpp:324-380) and the
// Foley & van Dam conversions of opcolor_impl.h:240-490, for float and
// Dual2 components (branches on values, Dual2 arithmetic of dual.h) ----
namespace colorsp {
inline float val(float x) { return x; }
inline float val(const DF& x) { return x.v; }
template <class S> S k(float v) { return S(v); }
template <class S> S mn(const S& a, const S& b) { return val(a) < val(b) ? a : b; }
template <class S> S mx(const S& a, const S& b) { return val(a) > val(b) ? a : b; }
template <class S> struct C { S x, y, z; };
template <class S> C<S> hsv2rgb(C<S> c) {
    S h = c.x;
    const S s = c.y, v = c.z;
    if (val(s) < 0.0001f) return { v, v, v };
    h = 6.0f * (h - std::floor(val(h)));
    const float fh = std::floor(val(h));
    const int hi = fh != fh ? 0 : (int)fh;
    const S f = h - (float)hi;
    const S p = v * (1.0f - s), q = v * (1.0f - s * f), t = v * (1.0f - s * (1.0f - f));
    switch (hi) {
    case 0: return { v, t, p };
    case 1: return { q, v, p };
    case 2: return { p, v, t };
    case 3: return { p, q, v };
    case 4: return { t, p, v };
    default: return { v, p, q };
    }
}
template <class S> C<S> rgb2hsv(C<S> c) {
    const S lo = mn(c.x, mn(c.y, c.z)), hi = mx(c.x, mx(c.y, c.z));
    const S delta = hi - lo;
    S s = k<S>(0.0f), h = k<S>(0.0f);
    if (val(hi) > 0.0f) s = delta / hi;
    if (val(s) > 0.0f) {
        float kk;
        S a, b;
        if (val(c.x) >= val(hi)) { kk = 0.0f / 6.0f; a = c.y; b = c.z; }
        else if (val(c.y) >= val(hi)) { kk = 2.0f / 6.0f; a = c.z; b = c.x; }
        else { kk = 4.0f / 6.0f; a = c.x; b = c.y; }
        h = kk + (a - b) / (6.0f * delta);
        if (val(h) < 0.0f) h = h + 1.0f;
    }
    return { h, s, hi };
}
template <class S> C<S> hsl2rgb(C<S> c) {
    const S h = c.x, l = c.z;
    S s = c.y;
    const S v = val(l) <= 0.5f ? l * (1.0f + s) : l * (1.0f - s) + s;
    if (val(v) <= 0.0f) return { k<S>(0.0f), k<S>(0.0f), k<S>(0.0f) };
    const S lo = 2.0f * l - v;
    s = (v - lo) / v;
    return hsv2rgb<S>({ h, s, v });
}
template <class S> C<S> rgb2hsl(C<S> c) {
    const S lo = mn(c.x, mn(c.y, c.z));
    const C<S> hsv = rgb2hsv(c);
    const S hi = hsv.z, l = (lo + hi) / 2.0f;
    S s;
    if (val(lo) == val(hi)) s = k<S>(0.0f);
    else s = (hi - lo) / (val(l) <= 0.5f ? hi + lo : (2.0f - hi) - lo);
    return { hsv.x, s, l };
}
template <class S> C<S> mul33(C<S> c, const float* m) {
    return { c.x * m[0] + c.y * m[3] + c.z * m[6], c.x * m[1] + c.y * m[4] + c.z * m[7],
             c.x * m[2] + c.y * m[5] + c.z * m[8] };
}
const float kYiq2Rgb[9] = { 1.0000f, 1.0000f, 1.0000f, 0.9557f, -0.2716f, -1.1082f, 0.6199f, -0.6469f, 1.7051f };
const float kRgb2Yiq[9] = { 0.299f, 0.596f, 0.212f, 0.587f, -0.275f, -0.523f, 0.114f, -0.321f, 0.311f };
template <class S> C<S> xyz2xyy(C<S> c) {
    const S n = (c.x + c.y) + c.z;
    const S ninv = val(n) >= 1.0e-6f ? 1.0f / n : k<S>(0.0f);
    return { c.x * ninv, c.y * ninv, c.y };
}
template <class S> C<S> xyy2xyz(C<S> c) {
    const S Yy = val(c.y) > 1.0e-6f ? c.z / c.y : k<S>(0.0f);
    return { Yy * c.x, c.z, Yy * ((1.0f - c.x) - c.y) };
}
inline float pw(float x, float y) { return safe_pow(x, y); }
inline DF pw(const DF& u, float y) {  // dual.h safe_pow, constant exponent
    const float powuvm1 = safe_pow(u.v, y - 1.0f), powuv = powuvm1 * u.v;
    const float logu = u.v > 0.0f ? safe_log(u.v) : 0.0f;
    const float du = y * powuvm1, dv = logu * powuv;
    return DF(powuv, du * u.dx + dv * 0.0f, du * u.dy + dv * 0.0f);
}
template <class S> S s2l(S x) { return val(x) <= 0.04045f ? x * (1.0f / 12.92f) : pw((x + 0.055f) * (1.0f / 1.055f), 2.4f); }
template <class S> S l2s(S x) { return val(x) <= 0.0031308f ? 12.92f * x : 1.055f * pw(x, 1.f / 2.4f) - 0.055f; }
template <class S> C<S> convert(C<S> c, uint32_t from, uint32_t to, const float* xyz2rgb, const float* rgb2xyz) {
    C<S> rgb;
    switch (from) {
    case oslg::CS_HSV: rgb = hsv2rgb(c); break;
    case oslg::CS_HSL: rgb = hsl2rgb(c); break;
    case oslg::CS_YIQ: rgb = mul33(c, kYiq2Rgb); break;
    case oslg::CS_XYZ: rgb = mul33(c, xyz2rgb); break;
    case oslg::CS_XYY: rgb = mul33(xyy2xyz(c), xyz2rgb); break;
    case oslg::CS_SRGB: rgb = { s2l(c.x), s2l(c.y), s2l(c.z) }; break;
    default: rgb = c; break;
    }
    switch (to) {
    case oslg::CS_HSV: return rgb2hsv(rgb);
    case oslg::CS_HSL: return rgb2hsl(rgb);
    case oslg::CS_YIQ: return mul33(rgb, kRgb2Yiq);
    case oslg::CS_XYZ: return mul33(rgb, rgb2xyz);
    case oslg::CS_XYY: return xyz2xyy(mul33(rgb, rgb2xyz));
    case oslg::CS_SRGB: return { l2s(rgb.x), l2s(rgb.y), l2s(rgb.z) };
    default: return rgb;
    }
}
}  // namespace colorsp

void op_transformc(Point& P, const uint32_t* a) {
    float m[18];
    for (int i = 0; i < 18; ++i) m[i] = bitsf(word(P, a[3], i));
    const uint32_t from = a[2] & 0xFFu, to = (a[2] >> 8) & 0xFFu;
    if (ader(a[0])) {
        const colorsp::C<DF> o = colorsp::convert<DF>({ getd(P, a[1], 0), getd(P, a[1], 1), getd(P, a[1], 2) }, from,
                                                      to, m, m + 9);
        putd(P, a[0], 0, o.x);
        putd(P, a[0], 1, o.y);
        putd(P, a[0], 2, o.z);
    } else {
        const colorsp::C<float> o = colorsp::convert<float>(
            { getf(P, a[1], 0, 0), getf(P, a[1], 1, 0), getf(P, a[1], 2, 0) }, from, to, m, m + 9);
        setf(P, a[0], 0, o.x);
        setf(P, a[0], 1, o.y);
        setf(P, a[0], 2, o.z);
    }
}
// osl_wavelength_color_vf (opcolor.cpp:446-456)
void op_wavelength(Point& P, const uint32_t* a) {
    const float lambda = getf(P, a[1], 0, 0);
    const float ii = (lambda - 380.0f) / 5.0f;
    const int i = (int)ii;
    float xyz[3] = { 0.0f, 0.0f, 0.0f };
    if (!((i < 0) | (i >= 80))) {
        const float rem = ii - (float)i;
        for (int c = 0; c < 3; ++c)
            xyz[c] = bitsf(word(P, a[2], 9 + 3 * i + c)) * (1.0f - rem) + bitsf(word(P, a[2], 9 + 3 * i + 3 + c)) * rem;
    }
    float m[9];
    for (int i2 = 0; i2 < 9; ++i2) m[i2] = bitsf(word(P, a[2], i2));
    const colorsp::C<float> rgb = colorsp::mul33<float>({ xyz[0], xyz[1], xyz[2] }, m);
    const float sc = (float)(1.0 / 2.52);
    const float o[3] = { rgb.x * sc, rgb.y * sc, rgb.z * sc };
    for (int c = 0; c < 3; ++c) setf(P, a[0], c, o[c] < 0.0f ? 0.0f : o[c]);
    if (ader(a[0]))
        for (int c = 0; c < 6; ++c) setf(P, a[0], 3 + c, 0.0f);
}

// ---- texture: mipmapped bilinear lookup (osl_texture, optexture.cpp:54-111;
// the filter stands in for OIIO's TextureSystem, which is not in the tree) --
struct OTexture {
    int nch = 0, nlevels = 0;
    int w[oslg::kTexMaxLevels] = {}, h[oslg::kTexMaxLevels] = {};
    std::vector<std::vector<float>> level;
};
std::vector<OTexture>& otextures() {
    static std::vector<OTexture> t;
    return t;
}
// level 0 the image; each next level the 2x2 box average of the previous
// (coordinates clamped at odd edges) down to 1x1 or 16 levels
void otex_build(OTexture& T, int w, int h, int nch, const float* src) {
    T.nch = nch;
    T.level.clear();
    T.level.emplace_back(src, src + (size_t)w * h * nch);
    T.nlevels = 0;
    int lw = w, lh = h;
    for (;;) {
        T.w[T.nlevels] = lw;
        T.h[T.nlevels] = lh;
        ++T.nlevels;
        if ((lw == 1 && lh == 1) || T.nlevels == oslg::kTexMaxLevels) break;
        const int nw = std::max(1, lw / 2), nh = std::max(1, lh / 2);
        std::vector<float> next((size_t)nw * nh * nch);
        const std::vector<float>& prev = T.level.back();
        for (int y = 0; y < nh; ++y)
            for (int x = 0; x < nw; ++x)
                for (int c = 0; c < nch; ++c) {
                    const int x0 = std::min(2 * x, lw - 1), x1 = std::min(2 * x + 1, lw - 1);
                    const int y0 = std::min(2 * y, lh - 1), y1 = std::min(2 * y + 1, lh - 1);
                    const float p00 = prev[((size_t)y0 * lw + x0) * nch + c];
                    const float p10 = prev[((size_t)y0 * lw + x1) * nch + c];
                    const float p01 = prev[((size_t)y1 * lw + x0) * nch + c];
                    const float p11 = prev[((size_t)y1 * lw + x1) * nch + c];
                    next[((size_t)y * nw + x) * nch + c] = (((p00 + p10) + p01) + p11) * 0.25f;
                }
        T.level.push_back(std::move(next));
        lw = nw;
        lh = nh;
    }
}
// texel index under the wrap mode; `inside` false for black outside the image
int otex_wrap(int i, int n, uint32_t mode, bool* inside) {
    *inside = true;
    if (mode == oslg::TW_PERIODIC) {
        const int m = i % n;
        return m < 0 ? m + n : m;
    }
    if (mode == oslg::TW_MIRROR) {
        const int p = 2 * n;
        int m = i % p;
        if (m < 0) m += p;
        return m < n ? m : p - 1 - m;
    }
    if (i < 0 || i >= n) {
        *inside = mode != oslg::TW_BLACK;
        return i < 0 ? 0 : n - 1;
    }
    return i;
}
float otex_coord(float x) { return x == x ? std::min(std::max(x, -1.0e7f), 1.0e7f) : 0.0f; }
void otex_bilinear(const OTexture& T, int lev, float s, float t, uint32_t sw, uint32_t tw, int first, int nc,
                   float* out) {
    const int W = T.w[lev], H = T.h[lev];
    const std::vector<float>& L = T.level[lev];
    const float x = otex_coord(s * (float)W - 0.5f), y = otex_coord(t * (float)H - 0.5f);
    const float x0 = std::floor(x), y0 = std::floor(y);
    const float fx = x - x0, fy = y - y0;
    const int ix = (int)x0, iy = (int)y0;
    bool ix0, ix1, iy0, iy1;
    const int cx0 = otex_wrap(ix, W, sw, &ix0), cx1 = otex_wrap(ix + 1, W, sw, &ix1);
    const int cy0 = otex_wrap(iy, H, tw, &iy0), cy1 = otex_wrap(iy + 1, H, tw, &iy1);
    for (int c = 0; c < nc; ++c) {
        const int ch = first + c < T.nch ? first + c : (T.nch == 1 ? 0 : -1);
        float v00 = 0.0f, v10 = 0.0f, v01 = 0.0f, v11 = 0.0f;
        if (ch >= 0) {
            if (ix0 && iy0) v00 = L[((size_t)cy0 * W + cx0) * T.nch + ch];
            if (ix1 && iy0) v10 = L[((size_t)cy0 * W + cx1) * T.nch + ch];
            if (ix0 && iy1) v01 = L[((size_t)cy1 * W + cx0) * T.nch + ch];
            if (ix1 && iy1) v11 = L[((size_t)cy1 * W + cx1) * T.nch + ch];
        }
        const float top = (1.0f - fx) * v00 + fx * v10;
        const float bot = (1.0f - fx) * v01 + fx * v11;
        out[c] = (1.0f - fy) * top + fy * bot;
    }
}
// mipmapped bilinear: level of detail from the footprint in level-0
// texels (times width), the two nearest levels blended
void otex_filtered(const OTexture& T, float s, float t, float dsx, float dtx, float dsy, float dty, float width,
                   uint32_t sw, uint32_t tw, int first, int nc, float* res) {
    const float len = std::max(std::sqrt(dsx * dsx + dtx * dtx), std::sqrt(dsy * dsy + dty * dty)) * width;
    float lod = len > 1.0f ? oracle::own_log(len) * 1.44269504f : 0.0f;
    lod = std::min(lod, (float)(T.nlevels - 1));
    const int l0 = (int)lod;
    const float f = lod - (float)l0;
    otex_bilinear(T, l0, s, t, sw, tw, first, nc, res);
    if (f > 0.0f && l0 + 1 < T.nlevels) {
        float hi[3];
        otex_bilinear(T, l0 + 1, s, t, sw, tw, first, nc, hi);
        for (int c = 0; c < nc; ++c) res[c] = (1.0f - f) * res[c] + f * hi[c];
    }
}
void op_texture(Point& P, const uint32_t* a) {
    const uint32_t r = a[0];
    const int nc = anc(r) == 3 ? 3 : 1;
    const int id = (int)(a[3] & 0xFFu);
    float res[3] = { 0.0f, 0.0f, 0.0f };
    const std::vector<OTexture>& tex = otextures();
    if (id < (int)tex.size() && tex[id].nlevels > 0) {
        const OTexture& T = tex[id];
        const uint32_t sw = (a[3] >> 8) & 15u, tw = (a[3] >> 12) & 15u;
        const int first = (int)((a[3] >> 16) & 0xFFu);
        const DF s = getd(P, a[1], 0), t = getd(P, a[2], 0);
        const float width = getf(P, a[4], 0, 0);
        const float w0 = (float)T.w[0], h0 = (float)T.h[0];
        otex_filtered(T, s.v, t.v, s.dx * w0, t.dx * h0, s.dy * w0, t.dy * h0, width, sw, tw, first, nc, res);
    } else {
        P.status |= oslg::ST_ARRAY_BOUNDS;
    }
    for (int c = 0; c < nc; ++c) putd(P, r, c, DF(res[c]));
}

// environment (osl_environment, src/liboslexec/optexture.cpp): a
// latitude-longitude image by direction, z up: s = atan2(y, x) / 2pi + 0.5
// (periodic), t = 0.5 - atan2(z, hypot(x, y)) / pi (clamped); the footprint
// maps R + dR/dx, R + dR/dy the same way (s differences wrapped into
// [-0.5, 0.5]).
void oenv_st(float x, float y, float z, float* s, float* t) {
    const float h = std::sqrt(x * x + y * y);
    *s = (float)std::atan2((double)y, (double)x) * 0.159154943f + 0.5f;
    *t = 0.5f - (float)std::atan2((double)z, (double)h) * 0.318309886f;
}
float oenv_wrap_ds(float d) { return d > 0.5f ? d - 1.0f : (d < -0.5f ? d + 1.0f : d); }
void op_environment(Point& P, const uint32_t* a) {
    const uint32_t r = a[0];
    const int nc = anc(r) == 3 ? 3 : 1;
    const int id = (int)(a[3] & 0xFFu);
    float res[3] = { 0.0f, 0.0f, 0.0f };
    const std::vector<OTexture>& tex = otextures();
    if (id < (int)tex.size() && tex[id].nlevels > 0) {
        const OTexture& T = tex[id];
        const int first = (int)((a[3] >> 16) & 0xFFu);
        const DF x = getd(P, a[1], 0), y = getd(P, a[1], 1), z = getd(P, a[1], 2);
        const float width = getf(P, a[4], 0, 0);
        float s, t, sx, tx, sy, ty;
        oenv_st(x.v, y.v, z.v, &s, &t);
        oenv_st(x.v + x.dx, y.v + y.dx, z.v + z.dx, &sx, &tx);
        oenv_st(x.v + x.dy, y.v + y.dy, z.v + z.dy, &sy, &ty);
        const float w0 = (float)T.w[0], h0 = (float)T.h[0];
        otex_filtered(T, s, t, oenv_wrap_ds(sx - s) * w0, (tx - t) * h0, oenv_wrap_ds(sy - s) * w0, (ty - t) * h0,
                      width, oslg::TW_PERIODIC, oslg::TW_CLAMP, first, nc, res);
    } else {
        P.status |= oslg::ST_ARRAY_BOUNDS;
    }
    for (int c = 0; c < nc; ++c) putd(P, r, c, DF(res[c]));
}

// splineinverse (src/liboslexec/splineimpl.h:241-296): clamp outside the
// knots' range, else search each segment for f(x) = y with OpenImageIO's
// invert() (the reference calls it; restated from the published method:
// regula falsi for three quarters of the iterations, bisecting when the
// interpolant leaves the bracket, then bisection; stop when the bracket or
// the residual is below eps; unbracketed -> the end toward y). Dual2
// throughout, so the result carries derivatives as the reference's does.
struct OSplineFn {
    const Point* P;
    uint32_t kn;
    int basis, count;
    float knot(int k) const { return bitsf(word(*P, kn, k)); }
    DF operator()(DF xval) const {
        const SplineBasis& B = spline_basis(basis);
        DF x = xval;
        if (!(0.0f <= x.v)) x = DF(0.0f);
        if (x.v > 1.0f) x = DF(1.0f);
        const int nsegs = ((count - 4) / B.step) + 1;
        x = x * (float)nsegs;
        int segnum = (int)x.v;
        if (segnum < 0) segnum = 0;
        if (segnum > nsegs - 1) segnum = nsegs - 1;
        if (basis == 5) return DF(knot(segnum + 1));
        x = x - (float)segnum;
        const int s = segnum * B.step;
        float tk[4];
        for (int k = 0; k < 4; ++k)
            tk[k] = ((knot(s) * B.m[k][0] + knot(s + 1) * B.m[k][1]) + knot(s + 2) * B.m[k][2]) + knot(s + 3) * B.m[k][3];
        DF t = x * tk[0];
        t = t + tk[1];
        t = t * x;
        t = t + tk[2];
        t = t * x;
        t = t + tk[3];
        return t;
    }
};
DF ospline_root(const OSplineFn& f, DF y, DF xmin, DF xmax, int maxiters, float eps, bool* brack) {
    DF v0 = f(xmin), v1 = f(xmax);
    DF x = xmin, v = v0;
    const bool increasing = v0.v < v1.v;
    const float vmin = increasing ? v0.v : v1.v, vmax = increasing ? v1.v : v0.v;
    const bool bracketed = y.v >= vmin && y.v <= vmax;
    *brack = bracketed;
    if (!bracketed) return ((y.v < vmin) == increasing) ? xmin : xmax;
    if (std::fabs(v0.v - v1.v) < eps) return x;
    const int rfiters = (3 * maxiters) / 4;
    for (int it = 0; it < maxiters; ++it) {
        DF t = DF(0.5f);
        if (it < rfiters) {
            t = (y - v0) / (v1 - v0);
            if (t.v <= 0.0f || t.v >= 1.0f) t = DF(0.5f);
        }
        const DF omt = 1.0f - t;
        x = xmin * omt + xmax * t;
        v = f(x);
        if ((v.v < y.v) == increasing) {
            xmin = x;
            v0 = v;
        } else {
            xmax = x;
            v1 = v;
        }
        if (std::fabs(xmax.v - xmin.v) < eps || std::fabs(v.v - y.v) < eps) return x;
    }
    return x;
}
void op_splineinverse(Point& P, const uint32_t* a) {
    OSplineFn f;
    f.P = &P;
    f.kn = a[2];
    f.basis = a[3] < 6u ? (int)a[3] : 0;
    const int alen = (int)a[5];
    f.count = a[4] != oslg::kNoArg ? geti(P, a[4], 0) : alen;
    if (f.count > alen) f.count = alen;
    if (f.count < 4) {
        P.status |= oslg::ST_ARRAY_BOUNDS;
        putd(P, a[0], 0, DF(0.0f));
        return;
    }
    const DF y = getd(P, a[1], 0);
    const SplineBasis& B = spline_basis(f.basis);
    const int lo = B.step == 1 ? 1 : 0, hi = B.step == 1 ? f.count - 2 : f.count - 1;
    const bool increasing = f.knot(1) < f.knot(f.count - 2);
    DF x(0.0f);
    bool done = false;
    if (increasing) {
        if (y.v <= f.knot(lo)) { x = DF(0.0f); done = true; }
        else if (y.v >= f.knot(hi)) { x = DF(1.0f); done = true; }
    } else {
        if (y.v >= f.knot(lo)) { x = DF(0.0f); done = true; }
        else if (y.v <= f.knot(hi)) { x = DF(1.0f); done = true; }
    }
    if (!done) {
        const int nsegs = (f.count - 4) / B.step + 1;
        const float nseginv = 1.0f / (float)nsegs;
        DF r0(0.0f);
        for (int s = 0; s < nsegs; ++s) {
            const DF r1(nseginv * (float)(s + 1));
            bool brack;
            x = ospline_root(f, y, r0, r1, 32, 1.0e-6f, &brack);
            if (brack) break;
            r0 = r1;
        }
    }
    putd(P, a[0], 0, x);
}

// setmessage / getmessage (src/liboslexec/opmessage.cpp:19-138): per point
// and message name a state word (0 unset, 1 + type id once set, kMsgQueried
// after a strict query that found nothing) and a store per type. Double
// sets, sets after a failed strict query and reads as another type are
// errors: status bit, values unchanged.
void op_setmessage(Point& P, const uint32_t* a) {
    const int nw = (int)(a[3] & 0xFFFFu);
    if (word(P, a[0], 0) != 0u) {
        P.status |= oslg::ST_MESSAGE;
        return;
    }
    setw(P, a[0], 0, 1u + (a[3] >> 16));
    for (int i = 0; i < nw; ++i) setw(P, a[1], i, word(P, a[2], i));
}
void op_getmessage(Point& P, const uint32_t* a) {
    const int nw = (int)(a[4] & 0xFFFFu);
    const uint32_t tid = (a[4] >> 16) & 0x7FFFu;
    const bool strict = (a[4] >> 31) != 0u;
    const uint32_t s = word(P, a[1], 0);
    uint32_t found = 0u;
    if (s == 0u) {
        if (strict) setw(P, a[1], 0, oslg::kMsgQueried);
    } else if (s == oslg::kMsgQueried) {
        // queried before and not found: still not found
    } else if (s != 1u + tid) {
        P.status |= oslg::ST_MESSAGE;
    } else {
        for (int i = 0; i < nw; ++i) setw(P, a[3], i, word(P, a[2], i));
        if (ader(a[3]))
            for (int i = nw; i < 3 * nw; ++i) setw(P, a[3], i, 0u);
        found = 1u;
    }
    setw(P, a[0], 0, found);
}

// blackbody (src/liboslexec/opcolor_impl.h:510-575, opcolor.cpp:438-442):
// a2 = constant table (N entries of RGB^(1/5), XYZ->RGB matrix, CIE table)
void op_blackbody(Point& P, const uint32_t* a) {
    float T = getf(P, a[1], 0, 0);
    uint32_t tb = a[2];
    int N = (int)a[3];
    auto tab = [&](int i) { return bitsf(word(P, tb, i)); };
    float rgb[3];
    if (T < 800.0f) {
        rgb[0] = 1.0e-6f; rgb[1] = 0.0f; rgb[2] = 0.0f;
    } else if (T < 12000.0f) {
        float ic = (float)std::cbrt((double)((T - 800.0f) / 2.0f));
        float t = ic * ic;
        int ti = (int)t;
        if (ti > N - 2) ti = N - 2;
        float rem = t - (float)ti;
        for (int c = 0; c < 3; ++c) {
            float v = tab(ti * 3 + c) * (1.0f - rem) + tab(ti * 3 + 3 + c) * rem;
            float v2 = v * v, v4 = v2 * v2;
            rgb[c] = v4 * v;
        }
    } else {
        float X = 0.0f, Y = 0.0f, Z = 0.0f;
        const float dlambda = (float)(5.0f * 1e-9);
        int cie = N * 3 + 9;
        for (int i = 0; i < 81; ++i) {
            float lambda = 380.0f + 5.0f * (float)i;
            float wlm = lambda * 1e-9f;
            float wlm2 = wlm * wlm, wlm4 = wlm2 * wlm2, wlm5 = wlm4 * wlm;
            float inv5 = 1.0f / wlm5;
            float e = (float)std::expm1((double)(1.4388e-2f / (wlm * T)));
            float Me = ((3.74183e-16f * inv5) / e) * dlambda;
            X += Me * tab(cie + i * 3 + 0);
            Y += Me * tab(cie + i * 3 + 1);
            Z += Me * tab(cie + i * 3 + 2);
        }
        int mx = N * 3;
        for (int c = 0; c < 3; ++c) {
            float v = X * tab(mx + c) + Y * tab(mx + 3 + c) + Z * tab(mx + 6 + c);
            rgb[c] = v < 0.0f ? 0.0f : v;
        }
    }
    for (int c = 0; c < 3; ++c) putv(P, a[0], c, rgb[c]);
}

// noise (batched_llvm_gen.cpp:6032-6190 kinds; oslnoise.h wrappers)
void op_noise(Point& P, const uint32_t* a) {
    uint32_t r = a[0], S = a[1], T = a[2], kw = a[3];
    int kind = (int)(kw & 15u);
    bool periodic = (kw & 16u) != 0;
    int dims = (int)((kw >> 5) & 7u);
    bool vec = (kw & 256u) != 0;
    bool derivs = (kw & 512u) != 0;
    int ns = anc(S), nc = vec ? 3 : 1;
    DF res[3];
    Hasher H;
    if (periodic) {
        H.periodic = true;
        if (ns == 3) {
            H.px = Hasher::per(getf(P, a[4], 0, 0)); H.py = Hasher::per(getf(P, a[4], 1, 0));
            H.pz = Hasher::per(getf(P, a[4], 2, 0));
            if (dims == 4) H.pw = Hasher::per(getf(P, a[5], 0, 0));
        } else {
            H.px = Hasher::per(getf(P, a[4], 0, 0));
            if (dims == 2) H.py = Hasher::per(getf(P, a[5], 0, 0));
        }
    }
    DF xs[4];
    for (int i = 0; i < ns; ++i) xs[i] = getd(P, S, i);
    if (T != oslg::kNoArg) xs[ns] = getd(P, T, 0);
    if (kind == oslg::NK_CELL || kind == oslg::NK_HASH) {
        float v[4];
        for (int i = 0; i < dims; ++i) v[i] = xs[i].v;
        if (periodic) {
            if (ns == 3) {
                for (int i = 0; i < 3; ++i) v[i] = pwrap(v[i], getf(P, a[4], i, 0));
                if (dims == 4) v[3] = pwrap(v[3], getf(P, a[5], 0, 0));
            } else {
                v[0] = pwrap(v[0], getf(P, a[4], 0, 0));
                if (dims == 2) v[1] = pwrap(v[1], getf(P, a[5], 0, 0));
            }
        }
        bool cell = kind == oslg::NK_CELL;
        if (!vec) {
            float f;
            if (cell) f = dims == 1 ? intnoise1<CellKey>(v[0]) : dims == 2 ? intnoise2<CellKey>(v[0], v[1])
                        : dims == 3 ? intnoise3<CellKey>(v[0], v[1], v[2]) : intnoise4<CellKey>(v[0], v[1], v[2], v[3]);
            else f = dims == 1 ? intnoise1<HashKey>(v[0]) : dims == 2 ? intnoise2<HashKey>(v[0], v[1])
                   : dims == 3 ? intnoise3<HashKey>(v[0], v[1], v[2]) : intnoise4<HashKey>(v[0], v[1], v[2], v[3]);
            res[0] = DF(f);
        } else {
            V3 f;
            if (cell) f = dims == 1 ? vintnoise1<CellKey>(v[0]) : dims == 2 ? vintnoise2<CellKey>(v[0], v[1])
                        : dims == 3 ? vintnoise3<CellKey>(v[0], v[1], v[2]) : vintnoise4<CellKey>(v[0], v[1], v[2], v[3]);
            else f = dims == 1 ? vintnoise1<HashKey>(v[0]) : dims == 2 ? vintnoise2<HashKey>(v[0], v[1])
                   : dims == 3 ? vintnoise3<HashKey>(v[0], v[1], v[2]) : vintnoise4<HashKey>(v[0], v[1], v[2], v[3]);
            for (int c = 0; c < 3; ++c) res[c] = DF(f[c]);
        }
    } else if (kind == oslg::NK_PERLIN || kind == oslg::NK_UPERLIN) {
        for (int c = 0; c < nc; ++c) {
            if (derivs) {
                DF o = perlin_n<DF>(H, c, dims, xs);
                res[c] = kind == oslg::NK_UPERLIN ? unsigned_of(o) : o;
            } else {
                float v[4];
                for (int i = 0; i < dims; ++i) v[i] = xs[i].v;
                float o = perlin_n<float>(H, c, dims, v);
                res[c] = DF(kind == oslg::NK_UPERLIN ? unsigned_of(o) : o);
            }
        }
    } else if (kind == oslg::NK_SIMPLEX || kind == oslg::NK_USIMPLEX) {
        for (int c = 0; c < nc; ++c) {
            DF o;
            if (derivs) o = simplex_dual(dims, xs, c);
            else {
                float v[4];
                for (int i = 0; i < dims; ++i) v[i] = xs[i].v;
                o = DF(simplex_val(dims, v, c));
            }
            if (kind == oslg::NK_USIMPLEX) o = 0.5f * (o + 1.0f);
            res[c] = o;
        }
    } else if (kind == oslg::NK_UNULL) {
        for (int c = 0; c < nc; ++c) res[c] = DF(0.5f);
    } else {
        for (int c = 0; c < nc; ++c) res[c] = DF(0.0f);
    }
    int rn = anc(r);
    for (int c = 0; c < rn; ++c) putd(P, r, c, res[nc == 1 ? 0 : c]);
}

// gabor / pgabor (opnoise.cpp:484-640 forms; sfm_gabornoise.h:490-660).
// a: r, S, T, kind word, anisotropic, direction, bandwidth; the carrier op
// that follows holds impulses, do_filter, Speriod, Tperiod.
void op_gabor(Point& P, const uint32_t* a, const uint32_t* b) {
    uint32_t r = a[0], S = a[1], kw = a[3];
    bool periodic = (kw & 16u) != 0;
    int dims = (int)((kw >> 5) & 7u);
    bool vec = (kw & 256u) != 0;
    int ns = anc(S), nc = vec ? 3 : 1;
    GaborOptions o;
    o.anisotropic = geti(P, a[4], 0);
    o.direction = V3(getf(P, a[5], 0, 0), getf(P, a[5], 1, 0), getf(P, a[5], 2, 0));
    o.bandwidth = getf(P, a[6], 0, 0);
    o.impulses = getf(P, b[0], 0, 0);
    o.do_filter = geti(P, b[1], 0);
    // position as Dual2<Vec3>: 1-D and 2-D slice to 3-D, the 4-D forms drop t
    DV X;
    if (ns == 3) {
        for (int c = 0; c < 3; ++c) setcomp(X, c, getd(P, S, c));
    } else {
        setcomp(X, 0, getd(P, S, 0));
        if (dims == 2) setcomp(X, 1, getd(P, a[2], 0));
    }
    V3 period(0.0f);
    if (periodic) {
        if (ns == 3) period = V3(getf(P, b[2], 0, 0), getf(P, b[2], 1, 0), getf(P, b[2], 2, 0));
        else {
            period.x = getf(P, b[2], 0, 0);
            if (dims == 2) period.y = getf(P, b[3], 0, 0);
        }
    }
    DF res[3];
    gabor_eval<OwnMath>(o, X, periodic, period, nc, res);
    int rn = anc(r);
    for (int c = 0; c < rn; ++c) putd(P, r, c, res[nc == 1 ? 0 : c]);
}

void op_hash(Point& P, const uint32_t* a) {
    uint32_t x = a[1], y = a[2];
    int h;
    uint32_t tx = atc(x);
    if (tx == oslg::TC_INT) h = hash_i((int32_t)word(P, x, 0));
    else if (tx == oslg::TC_STRING) h = (int)word(P, x, 0);
    else if (tx == oslg::TC_TRIPLE) {
        V3 p(bitsf(word(P, x, 0)), bitsf(word(P, x, 1)), bitsf(word(P, x, 2)));
        h = y == oslg::kNoArg ? hash_v(p) : hash_vf(p, getf(P, y, 0, 0));
    } else {
        h = y == oslg::kNoArg ? hash_f(getf(P, x, 0, 0)) : hash_ff(getf(P, x, 0, 0), getf(P, y, 0, 0));
    }
    setw(P, a[0], 0, (uint32_t)h);
}

const oslg_field& gfield(const oslg_shaderglobals& G, int id) {
    const oslg_field* f = &G.P;  // fields are laid out in GlobalId order
    return f[id];
}
float fld(const oslg_field& f, int c, int64_t pt) { return f.data ? f.data[c * f.plane_stride + pt] : f.value[c]; }
bool gflag(const oslg_field& f, int64_t pt) {
    return f.data ? reinterpret_cast<const int32_t*>(f.data)[pt] != 0 : f.value[0] != 0.0f;
}
// calculatenormal (llvm_ops.cpp:915-934): cross(dPdx, dPdy), operands
// swapped under flipHandedness
void op_calcnormal(Point& P, const uint32_t* a, const oslg_shaderglobals& G) {
    V3 dx(getf(P, a[1], 0, 1), getf(P, a[1], 1, 1), getf(P, a[1], 2, 1));
    V3 dy(getf(P, a[1], 0, 2), getf(P, a[1], 1, 2), getf(P, a[1], 2, 2));
    V3 n = gflag(G.flipHandedness, P.pt) ? v3_cross(dy, dx) : v3_cross(dx, dy);
    putv(P, a[0], 0, n.x);
    putv(P, a[0], 1, n.y);
    putv(P, a[0], 2, n.z);
}

void op_load_global(Point& P, const uint32_t* a, const oslg_shaderglobals& G) {
    uint32_t r = a[0];
    int id = (int)a[1];
    if (oslg::global_is_int((uint32_t)id)) {  // flipHandedness, backfacing: 0 or 1
        setw(P, r, 0, gflag(gfield(G, id), P.pt) ? 1u : 0u);
        return;
    }
    int nc = anc(r);
    for (int c = 0; c < nc; ++c) setf(P, r, c, fld(gfield(G, id), c, P.pt));
    if (ader(r)) {
        int dxid = -1, dyid = -1;
        if (id == oslg::G_P) { dxid = oslg::G_DPDX; dyid = oslg::G_DPDY; }
        else if (id == oslg::G_I) { dxid = oslg::G_DIDX; dyid = oslg::G_DIDY; }
        else if (id == oslg::G_U) { dxid = oslg::G_DUDX; dyid = oslg::G_DUDY; }
        else if (id == oslg::G_V) { dxid = oslg::G_DVDX; dyid = oslg::G_DVDY; }
        else if (id == oslg::G_PS) { dxid = oslg::G_DPSDX; dyid = oslg::G_DPSDY; }
        for (int c = 0; c < nc; ++c) {
            setf(P, r, nc + c, dxid >= 0 ? fld(gfield(G, dxid), c, P.pt) : 0.0f);
            setf(P, r, 2 * nc + c, dyid >= 0 ? fld(gfield(G, dyid), c, P.pt) : 0.0f);
        }
    }
}

// Closure tree (src/include/OSL/oslclosure.h:65-147) in a per-point node
// pool: [count][nodes of nf words (ProgramHeader::node_floats)]; a closure
// value is node index + 1.
struct CPools { uint32_t base, maxn, nf; };
inline uint32_t nslot(const CPools& C, uint32_t node) { return C.base + 1 + node * C.nf; }
inline uint32_t cl_alloc(Point& P, const CPools& C) {
    uint32_t n = P.heap[C.base];
    if (n >= C.maxn) { P.status |= oslg::ST_CLOSURE_OVERFLOW; return 0u; }
    P.heap[C.base] = n + 1;
    return n + 1;
}

// testrender's traversal (src/testrender/shading.cpp:1450-1500): MUL scales
// the running weight, ADD pushes its B branch with the current weight and
// follows A, a component is visited with weight * comp.w.
// With an opacity function, a layer(top, base) component continues into
// top with the layer's weight and pushes base with weight * (1 -
// clamp(opacity(top))) (testrender's MX_LAYER_ID, shading.cpp:1666-1681).
struct NoLayers {};
template <class F, class O = NoLayers> void closure_walk(Point& P, const CPools& C, uint32_t root, F&& visit,
                                                        O&& opacity = O()) {
    uint32_t stack_node[oslg::kClosureWalkStack];
    V3 stack_w[oslg::kClosureWalkStack];
    int sp = 0;
    V3 w(1.0f);
    uint32_t cur = root;
    int guard = 0;
    while (cur != 0u && cur <= C.maxn) {
        if (++guard > 4 * (int)C.maxn + 8) break;
        uint32_t ns = nslot(C, cur - 1);
        int id = (int32_t)P.heap[ns];
        if (id == oslg::kClosureMul) {
            w = w * V3(bitsf(P.heap[ns + 1]), bitsf(P.heap[ns + 2]), bitsf(P.heap[ns + 3]));
            cur = P.heap[ns + 4];
        } else if (id == oslg::kClosureAdd) {
            if (sp < oslg::kClosureWalkStack) {
                stack_node[sp] = P.heap[ns + 5];
                stack_w[sp] = w;
                ++sp;
            } else {
                P.status |= oslg::ST_CLOSURE_OVERFLOW;
            }
            cur = P.heap[ns + 4];
        } else {
            V3 cw = w * V3(bitsf(P.heap[ns + 1]), bitsf(P.heap[ns + 2]), bitsf(P.heap[ns + 3]));
            cur = 0u;
            if constexpr (!std::is_same<std::decay_t<O>, NoLayers>::value) {
                if (id == oslg::kIdMxLayer) {
                    const V3 op = opacity(P.heap[ns + 4]);
                    const V3 bw = w * V3(1.0f - bsdl_clamp(op.x, 0.0f, 1.0f), 1.0f - bsdl_clamp(op.y, 0.0f, 1.0f),
                                         1.0f - bsdl_clamp(op.z, 0.0f, 1.0f));
                    if (bw.x != 0.0f || bw.y != 0.0f || bw.z != 0.0f) {
                        if (sp < oslg::kClosureWalkStack) {
                            stack_node[sp] = P.heap[ns + 5];
                            stack_w[sp] = bw;
                            ++sp;
                        } else {
                            P.status |= oslg::ST_CLOSURE_OVERFLOW;
                        }
                    }
                    w = cw;
                    cur = P.heap[ns + 4];
                    goto next;
                }
            }
            visit(id, cw, ns + 4);
        }
    next:
        if (cur == 0u && sp > 0) {
            --sp;
            cur = stack_node[sp];
            w = stack_w[sp];
        }
    }
}

// process_closure's lobe construction for the lobes the executor shades
// (src/testrender/shading.cpp:1481-1530): emission accumulates Le,
// diffuse / oren_nayar / GGX microfacet (params: dist, N, U, xalpha,
// yalpha, eta, refract) become lobes in walk order; ggx_hash names "ggx".
// An int keyword parameter of a component (name hash, then the value) after
// its fixed parameters; dflt when absent.
inline int keyword_int(const Point& P, uint32_t p, int first, const char* name, int dflt) {
    const uint32_t key = oslg::string_hash_const(name);
    for (int k = first; k + 1 < oslg::kClosureParamFloats; k += 2) {
        const uint32_t w = P.heap[p + k];
        if (w == 0u) break;
        if (w == key) return (int32_t)P.heap[p + k + 1];
    }
    return dflt;
}

// dielectric_bsdf(N, U, reflection_tint, transmission_tint, roughness_x,
// roughness_y, ior, distribution): words 0-15; a leading "absorption"
// keyword fills words 16-19 with its name and colour
inline MxDielectric mx_dielectric(const Point& P, uint32_t p, const V3& wo, float path_roughness, bool backfacing) {
    auto f = [&](uint32_t s) { return bitsf(P.heap[s]); };
    V3 absorption(0.0f);
    if (P.heap[p + 16] == oslg::string_hash_const("absorption")) absorption = V3(f(p + 17), f(p + 18), f(p + 19));
    return MxDielectric(V3(f(p + 0), f(p + 1), f(p + 2)), V3(f(p + 3), f(p + 4), f(p + 5)),
                        V3(f(p + 6), f(p + 7), f(p + 8)), V3(f(p + 9), f(p + 10), f(p + 11)), f(p + 12), f(p + 13),
                        f(p + 14), absorption, wo, path_roughness, backfacing);
}

template <class WALK>
void collect_lobes(Point& P, WALK&& walk, const V3& wo, uint32_t ggx_hash, CompositeLobes* L, float path_roughness,
                   bool backfacing) {
    auto f = [&](uint32_t s) { return bitsf(P.heap[s]); };
    walk([&](int id, const V3& cw, uint32_t p) {
        if (id == 1) {  // EMISSION_ID
            L->Le = L->Le + cw;
        } else if (id == 3) {  // DIFFUSE_ID
            L->add_diffuse(cw, V3(f(p + 0), f(p + 1), f(p + 2)));
        } else if (id == 4) {  // OREN_NAYAR_ID
            L->add_on(cw, OrenNayarQON(V3(f(p + 0), f(p + 1), f(p + 2)), f(p + 3), wo));
        } else if (id == oslg::kIdMxOrenNayarDiffuse) {
            // oren_nayar_diffuse_bsdf(N, albedo, roughness, "energy_compensation", int)
            int ec = 0;
            for (int k = 7; k + 1 < oslg::kClosureParamFloats; k += 2) {
                const uint32_t w = P.heap[p + k];
                if (w == 0u) break;
                if (w == oslg::string_hash_const("energy_compensation")) {
                    ec = (int32_t)P.heap[p + k + 1];
                    break;
                }
            }
            L->add_on(cw, OrenNayarQON(V3(f(p + 0), f(p + 1), f(p + 2)), V3(f(p + 3), f(p + 4), f(p + 5)), f(p + 6),
                                       ec != 0, wo));
        } else if (id == oslg::kIdMxSheen) {  // sheen_bsdf(N, albedo, roughness, "mode", int)
            L->add_sheen(cw, SheenConty(V3(f(p + 0), f(p + 1), f(p + 2)), V3(f(p + 3), f(p + 4), f(p + 5)), f(p + 6), wo,
                                        path_roughness, backfacing, keyword_int(P, p, 7, "mode", 0)));
        } else if (id == oslg::kIdMxDielectric) {
            L->add_mx_dielectric(cw, mx_dielectric(P, p, wo, path_roughness, backfacing));
        } else if (id == 8 && P.heap[p] == ggx_hash) {  // MICROFACET_ID, "ggx"
            int refract = (int32_t)P.heap[p + 10];
            if (refract < 0 || refract > 2) return;
            L->add_ggx(cw, MicrofacetGGX(V3(f(p + 1), f(p + 2), f(p + 3)), V3(f(p + 4), f(p + 5), f(p + 6)), f(p + 7),
                                         f(p + 8), f(p + 9), refract));
        }
    });
}
// testrender's evaluate_layer_opacity (shading.cpp:1199-1281): a walk of
// the layer's top in which a nested layer continues into its top (pushing
// its base with weight * w), sheen scales the weight by w * (1 - E) (E the
// part of the light the sheen lets through) and other components are
// opaque; the walk's last weight is the opacity.
V3 layer_opacity(Point& P, const CPools& C, uint32_t top, const V3& wo, float path_roughness, bool backfacing) {
    if (top == 0u) return V3(0.0f);
    uint32_t stack_node[oslg::kClosureWalkStack];
    V3 stack_w[oslg::kClosureWalkStack];
    int sp = 0, guard = 0;
    V3 w(1.0f);
    uint32_t cur = top;
    auto push = [&](uint32_t node, const V3& pw) {
        if (sp >= oslg::kClosureWalkStack) {
            P.status |= oslg::ST_CLOSURE_OVERFLOW;
            return;
        }
        stack_node[sp] = node;
        stack_w[sp] = pw;
        ++sp;
    };
    auto f = [&](uint32_t s) { return bitsf(P.heap[s]); };
    while (cur != 0u && cur <= C.maxn) {
        if (++guard > 4 * (int)C.maxn + 8) break;
        const uint32_t ns = nslot(C, cur - 1);
        const int id = (int32_t)P.heap[ns];
        if (id == oslg::kClosureMul) {
            w = w * V3(f(ns + 1), f(ns + 2), f(ns + 3));
            cur = P.heap[ns + 4];
        } else if (id == oslg::kClosureAdd) {
            push(P.heap[ns + 5], w);
            cur = P.heap[ns + 4];
        } else {
            const V3 cw(f(ns + 1), f(ns + 2), f(ns + 3));
            const uint32_t p = ns + 4;
            cur = 0u;
            if (id == oslg::kIdMxLayer) {
                push(P.heap[p + 1], w * cw);
                cur = P.heap[p];
            } else if (id == oslg::kIdMxSheen) {
                const SheenConty sh(V3(f(p + 0), f(p + 1), f(p + 2)), V3(f(p + 3), f(p + 4), f(p + 5)), f(p + 6), wo,
                                    path_roughness, backfacing, keyword_int(P, p, 7, "mode", 0));
                w = w * (cw * V3(1.0f - sh.emiss));
            } else if (id == oslg::kIdMxDielectric) {  // testrender shading.cpp:1242-1248
                w = w * (cw * (V3(1.0f) - mx_dielectric(P, p, wo, path_roughness, backfacing).filter_o()));
            }
        }
        if (cur == 0u && sp > 0) {
            --sp;
            cur = stack_node[sp];
            w = stack_w[sp];
        }
    }
    return w;
}

void build_lobes(Point& P, const CPools& C, uint32_t root, const V3& wo, uint32_t ggx_hash, CompositeLobes* L,
                 float path_roughness = 0.0f, bool backfacing = false) {
    collect_lobes(
        P,
        [&](auto&& visit) {
            closure_walk(P, C, root, visit,
                         [&](uint32_t top) { return layer_opacity(P, C, top, wo, path_roughness, backfacing); });
        },
        wo, ggx_hash, L, path_roughness, backfacing);
}

// Static closures (oslg_program.h kClosureAbsent): the components of a
// known tree, visited in the walk's order from a consumer's term table
// (term j in words 3*(j%2).. of the (j/2)-th carrier op after it:
// node slot, weight operand or kNoArg, presence operand or kNoArg).
template <class F>
void closure_walk_static(Point& P, const oslg::Op* tab, uint32_t nterms, F&& visit) {
    for (uint32_t j = 0; j < nterms; ++j) {
        const uint32_t* t = tab[j / 2].a + 3 * (j % 2);
        const uint32_t ns = t[0];
        const int id = (int32_t)P.heap[ns];
        if (id == oslg::kClosureAbsent) continue;
        if (t[2] != oslg::kNoArg && word(P, t[2], 0) == 0u) continue;
        V3 cw = t[1] == oslg::kNoArg ? V3(bitsf(P.heap[ns + 1]), bitsf(P.heap[ns + 2]), bitsf(P.heap[ns + 3]))
                                     : V3(getf(P, t[1], 0, 0), getf(P, t[1], 1, 0), getf(P, t[1], 2, 0));
        visit(id, cw, ns + 4);
    }
}

struct Runner {
    const Prog& prog;
    const oslg_shaderglobals& G;
    char* userdata;
    char* outputs;

    void run_point(Point& P) {
        const oslg::ProgramHeader& h = *prog.h;
        CPools C{ h.closure_base, h.max_comps, oslg::node_floats(h) };
        if (h.flags & 1u) P.heap[C.base] = 0u;
        int nops = (int)h.nops;
        // the loop limit: back edges this point takes, summed over every loop
        const uint32_t cap = oslg::max_loop_iterations(h);
        uint32_t iters = 0;
        bool exited = false;
        for (int pc = 0; pc < nops;) {
            const Op& op = prog.ops[pc];
            const uint32_t* a = op.a;
            switch (op.code) {
            case oslg::OP_IF:
                pc = truth(P, a[0]) ? pc + 1 : prog.partner[pc] + 1;
                continue;
            case oslg::OP_ELSE:  // reached at the end of the then-block
                pc = prog.partner[pc];
                continue;
            case oslg::OP_LOOP_TEST:
                pc = truth(P, a[0]) ? pc + 1 : prog.partner[pc];
                continue;
            case oslg::OP_JUMP:
                if ((int)a[2] <= pc && ++iters > cap) { P.status |= oslg::ST_TIMEOUT; return; }
                pc = (int)a[2];
                continue;
            case oslg::OP_BREAK: pc = prog.break_target[pc]; continue;
            case oslg::OP_CONTINUE: pc = prog.continue_target[pc]; continue;
            case oslg::OP_RETURN: pc = prog.layer_end_after[pc]; continue;
            // exit: the rest of the group is skipped, but the layer's output
            // stores run (what the point wrote stays its result), then the
            // renderer-side section
            case oslg::OP_EXIT: exited = true; pc = prog.layer_end_after[pc]; continue;
            case oslg::OP_STORES_END:
                if (exited && a[0] == 0u) { pc = prog.final_section; continue; }
                break;
            // a return inside a user function's body ends the body (a2 = its end)
            case oslg::OP_FUNC_RETURN: pc = (int)a[2]; continue;
            case oslg::OP_NOP: case oslg::OP_ENDIF: case oslg::OP_LOOP_BEGIN: case oslg::OP_LOOP_STEP:
            case oslg::OP_LOOP_END: case oslg::OP_LAYER_END: case oslg::OP_FUNC_BEGIN: case oslg::OP_FUNC_END:
            case oslg::OP_STORE_HEAP:  // retained symbols are the executor's bookkeeping
                break;
            case oslg::OP_LOAD_GLOBAL: op_load_global(P, a, G); break;
            case oslg::OP_LOAD_USERDATA: {
                const uint32_t* q = reinterpret_cast<const uint32_t*>(userdata + (int64_t)a[1] + P.pt * (int64_t)(int32_t)a[2]);
                const int nc = anc(a[0]);
                const bool src_d = (a[3] & 2u) != 0u;  // the record carries derivatives
                for (int i = 0; i < nc; ++i) setw(P, a[0], i, q[i]);
                if (ader(a[0]))
                    for (int i = nc; i < 3 * nc; ++i) setw(P, a[0], i, src_d ? q[i] : 0u);
                break;
            }
            case oslg::OP_STORE_OUTPUT: {
                uint32_t s = a[0], flags = a[3];
                int elems = std::max(1, (int)a[4]);
                int total = anc(s) * elems;
                uint32_t* q = reinterpret_cast<uint32_t*>(outputs + (int64_t)a[1] + P.pt * (int64_t)(int32_t)a[2]);
                int nd = (flags & 1u) ? 3 : 1;
                for (int d = 0; d < nd; ++d)
                    for (int i = 0; i < total; ++i) {
                        uint32_t w;
                        if (d > 0 && !ader(s)) w = 0u;
                        else if (flags & 2u) w = atc(s) == oslg::TC_INT ? word(P, s, i) : (uint32_t)geti(P, s, i);
                        else w = word(P, s, d * total + i);
                        if (!(flags & 2u) && atc(s) == oslg::TC_INT) w = fbits((float)(int32_t)w);
                        q[d * total + i] = w;
                    }
                break;
            }
            case oslg::OP_ASSIGN: op_assign(P, a); break;
            case oslg::OP_COMPREF: {
                int i = geti(P, a[2], 0);
                if (i < 0 || i > 2) { P.status |= oslg::ST_ARRAY_BOUNDS; i = std::min(std::max(i, 0), 2); }
                putd(P, a[0], 0, ader(a[1]) ? getd(P, a[1], i) : DF(getf(P, a[1], i, 0)));
                break;
            }
            case oslg::OP_COMPASSIGN: {
                int i = geti(P, a[1], 0);
                if (i < 0 || i > 2) { P.status |= oslg::ST_ARRAY_BOUNDS; i = std::min(std::max(i, 0), 2); }
                putd(P, a[0], i, getd(P, a[2], 0));
                break;
            }
            case oslg::OP_MXCOMPREF: {
                int rr = std::min(std::max(geti(P, a[2], 0), 0), 3), cc = std::min(std::max(geti(P, a[3], 0), 0), 3);
                putv(P, a[0], 0, bitsf(word(P, a[1], rr * 4 + cc)));
                break;
            }
            case oslg::OP_MXCOMPASSIGN: {
                int rr = std::min(std::max(geti(P, a[1], 0), 0), 3), cc = std::min(std::max(geti(P, a[2], 0), 0), 3);
                setf(P, a[0], rr * 4 + cc, getf(P, a[3], 0, 0));
                break;
            }
            case oslg::OP_CONSTRUCT3:
                for (int c = 0; c < 3; ++c) putd(P, a[0], c, getd(P, a[1 + c], 0));
                break;
            case oslg::OP_AREF: {
                uint32_t r = a[0], arr = a[1];
                int alen = (int)a[3], i = geti(P, a[2], 0);
                if (i < 0 || i >= alen) { P.status |= oslg::ST_ARRAY_BOUNDS; i = std::min(std::max(i, 0), alen - 1); }
                int nc = anc(arr);
                for (int c = 0; c < nc; ++c) {
                    uint32_t w = word(P, arr, i * nc + c);
                    uint32_t tr = atc(r);
                    if (tr == oslg::TC_INT || tr == oslg::TC_STRING || tr == oslg::TC_CLOSURE) { setw(P, r, c, w); continue; }
                    float dx = 0, dy = 0;
                    if (ader(arr)) {
                        dx = bitsf(word(P, arr, alen * nc + i * nc + c));
                        dy = bitsf(word(P, arr, 2 * alen * nc + i * nc + c));
                    }
                    putd(P, r, c, DF(atc(arr) == oslg::TC_INT ? (float)(int32_t)w : bitsf(w), dx, dy));
                }
                break;
            }
            case oslg::OP_AASSIGN: {
                uint32_t arr = a[0], v = a[2];
                int alen = (int)a[3], i = geti(P, a[1], 0);
                if (i < 0 || i >= alen) { P.status |= oslg::ST_ARRAY_BOUNDS; i = std::min(std::max(i, 0), alen - 1); }
                int nc = anc(arr);
                for (int c = 0; c < nc; ++c) {
                    int vc = anc(v) == 1 ? 0 : c;
                    uint32_t ta = atc(arr);
                    if (ta == oslg::TC_INT || ta == oslg::TC_STRING || ta == oslg::TC_CLOSURE) {
                        setw(P, arr, i * nc + c, ta == oslg::TC_INT ? (uint32_t)geti(P, v, vc) : word(P, v, vc));
                        continue;
                    }
                    setf(P, arr, i * nc + c, getf(P, v, vc, 0));
                    if (ader(arr)) {
                        setf(P, arr, alen * nc + i * nc + c, getf(P, v, vc, 1));
                        setf(P, arr, 2 * alen * nc + i * nc + c, getf(P, v, vc, 2));
                    }
                }
                break;
            }
            case oslg::OP_MATRIX_DIAG: {
                float v = getf(P, a[1], 0, 0);
                for (int i = 0; i < 16; ++i) setf(P, a[0], i, i % 5 == 0 ? v : 0.0f);
                break;
            }
            case oslg::OP_ADD: op_arith(P, a, 0); break;
            case oslg::OP_SUB: op_arith(P, a, 1); break;
            case oslg::OP_MUL: op_arith(P, a, 2); break;
            case oslg::OP_DIV: op_arith(P, a, 3); break;
            case oslg::OP_MOD: op_arith(P, a, 4); break;
            case oslg::OP_IADD: op_iarith(P, a, 0); break;
            case oslg::OP_ISUB: op_iarith(P, a, 1); break;
            case oslg::OP_IMUL: op_iarith(P, a, 2); break;
            case oslg::OP_IDIV: op_iarith(P, a, 3); break;
            case oslg::OP_IMOD: op_iarith(P, a, 4); break;
            case oslg::OP_INEG: setw(P, a[0], 0, (uint32_t)(-geti(P, a[1], 0))); break;
            case oslg::OP_MMUL: {
                float out[16];
                if (atc(a[1]) == oslg::TC_MATRIX && atc(a[2]) == oslg::TC_MATRIX) {
                    float A[16], B[16];
                    for (int i = 0; i < 16; ++i) { A[i] = bitsf(word(P, a[1], i)); B[i] = bitsf(word(P, a[2], i)); }
                    for (int i = 0; i < 4; ++i)
                        for (int j = 0; j < 4; ++j)
                            out[i * 4 + j] = A[i * 4 + 0] * B[0 * 4 + j] + A[i * 4 + 1] * B[1 * 4 + j]
                                           + A[i * 4 + 2] * B[2 * 4 + j] + A[i * 4 + 3] * B[3 * 4 + j];
                } else {
                    uint32_t m = atc(a[1]) == oslg::TC_MATRIX ? a[1] : a[2], s = atc(a[1]) == oslg::TC_MATRIX ? a[2] : a[1];
                    float f = getf(P, s, 0, 0);
                    for (int i = 0; i < 16; ++i) out[i] = bitsf(word(P, m, i)) * f;
                }
                for (int i = 0; i < 16; ++i) setf(P, a[0], i, out[i]);
                break;
            }
            case oslg::OP_EQ: op_cmp(P, a, 0); break;
            case oslg::OP_NEQ: op_cmp(P, a, 1); break;
            case oslg::OP_LT: op_cmp(P, a, 2); break;
            case oslg::OP_GT: op_cmp(P, a, 3); break;
            case oslg::OP_LE: op_cmp(P, a, 4); break;
            case oslg::OP_GE: op_cmp(P, a, 5); break;
            case oslg::OP_AND: setw(P, a[0], 0, truth(P, a[1]) && truth(P, a[2]) ? 1u : 0u); break;
            case oslg::OP_OR: setw(P, a[0], 0, truth(P, a[1]) || truth(P, a[2]) ? 1u : 0u); break;
            case oslg::OP_BITAND: setw(P, a[0], 0, (uint32_t)(geti(P, a[1], 0) & geti(P, a[2], 0))); break;
            case oslg::OP_BITOR: setw(P, a[0], 0, (uint32_t)(geti(P, a[1], 0) | geti(P, a[2], 0))); break;
            case oslg::OP_XOR: setw(P, a[0], 0, (uint32_t)(geti(P, a[1], 0) ^ geti(P, a[2], 0))); break;
            case oslg::OP_SHL: setw(P, a[0], 0, (uint32_t)geti(P, a[1], 0) << (geti(P, a[2], 0) & 31)); break;
            case oslg::OP_SHR: setw(P, a[0], 0, (uint32_t)(geti(P, a[1], 0) >> (geti(P, a[2], 0) & 31))); break;
            case oslg::OP_COMPL: setw(P, a[0], 0, ~(uint32_t)geti(P, a[1], 0)); break;
            case oslg::OP_IABS: { int v = geti(P, a[1], 0); setw(P, a[0], 0, (uint32_t)(v < 0 ? -v : v)); break; }
            case oslg::OP_NEG: case oslg::OP_ABS: case oslg::OP_FLOOR: case oslg::OP_CEIL: case oslg::OP_ROUND:
            case oslg::OP_TRUNC: case oslg::OP_SIGN: case oslg::OP_SQRT: case oslg::OP_INVSQRT: case oslg::OP_CBRT:
            case oslg::OP_SIN: case oslg::OP_COS: case oslg::OP_TAN: case oslg::OP_ASIN: case oslg::OP_ACOS:
            case oslg::OP_ATAN: case oslg::OP_SINH: case oslg::OP_COSH: case oslg::OP_TANH: case oslg::OP_EXP:
            case oslg::OP_EXP2: case oslg::OP_EXPM1: case oslg::OP_LOG: case oslg::OP_LOG2: case oslg::OP_LOG10:
            case oslg::OP_RADIANS: case oslg::OP_DEGREES: case oslg::OP_LOGB: case oslg::OP_ERF: case oslg::OP_ERFC:
                op_unary(P, a, op.code);
                break;
            case oslg::OP_SINCOS: op_sincos(P, a); break;
            case oslg::OP_CALCNORMAL: op_calcnormal(P, a, G); break;
            case oslg::OP_RAYTYPE: {  // batched_llvm_gen.cpp:8520-8560, shadingsys.cpp:3823-3829
                uint32_t bit = a[2];
                if (a[1] != oslg::kNoArg) {
                    const uint32_t h = word(P, a[1], 0);
                    bit = 0;
                    for (uint32_t i = 0; i < a[4]; ++i)
                        if (word(P, a[3], (int)i) == h) { bit = 1u << i; break; }
                }
                setw(P, a[0], 0, ((uint32_t)G.raytype & bit) != 0u ? 1u : 0u);
                break;
            }
            case oslg::OP_ISNAN: setw(P, a[0], 0, std::isnan(getf(P, a[1], 0, 0)) ? 1u : 0u); break;
            case oslg::OP_ISINF: setw(P, a[0], 0, std::isinf(getf(P, a[1], 0, 0)) ? 1u : 0u); break;
            case oslg::OP_ISFINITE: setw(P, a[0], 0, std::isfinite(getf(P, a[1], 0, 0)) ? 1u : 0u); break;
            case oslg::OP_POW: case oslg::OP_ATAN2: case oslg::OP_FMOD: case oslg::OP_MIN: case oslg::OP_MAX:
            case oslg::OP_STEP:
                op_binary(P, a, op.code);
                break;
            case oslg::OP_IMIN: { int x = geti(P, a[1], 0), y = geti(P, a[2], 0); setw(P, a[0], 0, (uint32_t)(x <= y ? x : y)); break; }
            case oslg::OP_IMAX: { int x = geti(P, a[1], 0), y = geti(P, a[2], 0); setw(P, a[0], 0, (uint32_t)(x > y ? x : y)); break; }
            case oslg::OP_CLAMP: {
                int nc = anc(a[0]);
                for (int c = 0; c < nc; ++c) {
                    if (atc(a[0]) == oslg::TC_INT) {
                        int x = geti(P, a[1], c), lo = geti(P, a[2], c), hi = geti(P, a[3], c);
                        x = x < lo ? lo : x;
                        x = x > hi ? hi : x;
                        setw(P, a[0], c, (uint32_t)x);
                        continue;
                    }
                    DF x = getd(P, a[1], c), lo = getd(P, a[2], c), hi = getd(P, a[3], c);
                    DF v = x.v < lo.v ? lo : x;
                    v = v.v > hi.v ? hi : v;
                    putd(P, a[0], c, v);
                }
                break;
            }
            case oslg::OP_MIX: {
                int nc = anc(a[0]);
                for (int c = 0; c < nc; ++c) {
                    DF x = getd(P, a[1], c), y = getd(P, a[2], c), t = getd(P, a[3], c);
                    // dual.h:1267-1272 via dualfunc of three variables
                    float one_t = 1.0f - t.v;
                    float v = x.v * one_t + y.v * t.v;
                    float ymx = y.v - x.v;
                    putd(P, a[0], c, DF(v, one_t * x.dx + t.v * y.dx + ymx * t.dx, one_t * x.dy + t.v * y.dy + ymx * t.dy));
                }
                break;
            }
            case oslg::OP_SMOOTHSTEP: {
                int nc = anc(a[0]);
                for (int c = 0; c < nc; ++c) {
                    DF e0 = getd(P, a[1], c), e1 = getd(P, a[2], c), x = getd(P, a[3], c);
                    DF res;
                    if (x.v < e0.v) res = DF(0.0f);
                    else if (x.v >= e1.v) res = DF(1.0f);
                    else if (!ader(a[0])) {
                        float t = (x.v - e0.v) / (e1.v - e0.v);
                        res = DF((3.0f - 2.0f * t) * (t * t));
                    } else {
                        // dual.h:1325-1336
                        DF t = (x - e0) / (e1 - e0);
                        res = (3.0f - 2.0f * t) * t * t;
                    }
                    putd(P, a[0], c, res);
                }
                break;
            }
            case oslg::OP_SELECT: {
                int nc = anc(a[0]);
                for (int c = 0; c < nc; ++c) {
                    bool cond = atc(a[3]) == oslg::TC_TRIPLE ? getf(P, a[3], c, 0) != 0.0f : truth(P, a[3]);
                    if (atc(a[0]) == oslg::TC_INT) { setw(P, a[0], c, (uint32_t)geti(P, cond ? a[2] : a[1], c)); continue; }
                    putd(P, a[0], c, getd(P, cond ? a[2] : a[1], c));
                }
                break;
            }
            case oslg::OP_DOT: op_dot(P, a); break;
            case oslg::OP_CROSS: op_cross(P, a); break;
            case oslg::OP_LENGTH: op_length(P, a, false); break;
            case oslg::OP_DISTANCE: op_length(P, a, true); break;
            case oslg::OP_NORMALIZE: op_normalize(P, a); break;
            case oslg::OP_DX: case oslg::OP_DY: {
                int d = op.code == oslg::OP_DX ? 1 : 2;
                for (int c = 0; c < anc(a[0]); ++c) putv(P, a[0], c, getf(P, a[1], c, d));
                break;
            }
            case oslg::OP_TRANSFORM:
                if (a[3] == 2u) op_transformn(P, a);
                else op_transform(P, a);
                break;
            case oslg::OP_MDIV: op_mdiv(P, a); break;
            case oslg::OP_TRANSPOSE: {
                float M[16];
                for (int i = 0; i < 16; ++i) M[i] = bitsf(word(P, a[1], i));
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) setf(P, a[0], i * 4 + j, M[j * 4 + i]);
                break;
            }
            case oslg::OP_DETERMINANT: {
                float M[16];
                for (int i = 0; i < 16; ++i) M[i] = bitsf(word(P, a[1], i));
                putv(P, a[0], 0, det4(M));
                break;
            }
            case oslg::OP_AREA: op_area(P, a); break;
            case oslg::OP_FILTERWIDTH: op_filterwidth(P, a); break;
            case oslg::OP_LUMINANCE: op_luminance(P, a); break;
            case oslg::OP_TRANSFORMC: op_transformc(P, a); break;
            case oslg::OP_WAVELENGTH: op_wavelength(P, a); break;
            case oslg::OP_BLACKBODY: op_blackbody(P, a); break;
            case oslg::OP_TEXTURE: op_texture(P, a); break;
            case oslg::OP_ENVIRONMENT: op_environment(P, a); break;
            case oslg::OP_SETMESSAGE: op_setmessage(P, a); break;
            case oslg::OP_GETMESSAGE: op_getmessage(P, a); break;
            case oslg::OP_NOISE: op_noise(P, a); break;
            case oslg::OP_GABOR: op_gabor(P, a, prog.ops[pc + 1].a); break;
            case oslg::OP_HASH: op_hash(P, a); break;
            case oslg::OP_CLOSURE:
            case oslg::OP_CLOSURE_NODE: {
                // osl_allocate_(weighted_)closure_component (opclosure.cpp:83-117);
                // the static form writes its node at the slot of a0 and marks
                // a zero-weight component absent instead of returning null
                const bool stat = op.code == oslg::OP_CLOSURE_NODE;
                V3 w(1.0f);
                if (a[2] != oslg::kNoArg) {
                    w = V3(getf(P, a[2], 0, 0), getf(P, a[2], 1, 0), getf(P, a[2], 2, 0));
                    if (w.x == 0.0f && w.y == 0.0f && w.z == 0.0f) {
                        if (stat) P.heap[aoff(a[0])] = (uint32_t)oslg::kClosureAbsent;
                        else setw(P, a[0], 0, 0u);
                        break;
                    }
                }
                uint32_t h = 0, ns;
                if (stat) {
                    ns = aoff(a[0]);
                } else {
                    h = cl_alloc(P, C);
                    if (!h) { setw(P, a[0], 0, 0u); break; }
                    ns = nslot(C, h - 1);
                }
                P.heap[ns] = a[1];
                P.heap[ns + 1] = fbits(w.x); P.heap[ns + 2] = fbits(w.y); P.heap[ns + 3] = fbits(w.z);
                uint32_t params[11];
                int np = 0;
                for (int i = 3; i < 7; ++i) params[np++] = a[i];
                if (pc + 1 < nops && prog.ops[pc + 1].code == oslg::OP_NOP && prog.ops[pc + 1].nargs == 7)
                    for (int i = 0; i < 7; ++i) params[np++] = prog.ops[pc + 1].a[i];
                int k = 0;
                for (int i = 0; i < np && k < oslg::kClosureParamFloats; ++i) {
                    if (params[i] == oslg::kNoArg) break;
                    uint32_t t = atc(params[i]);
                    for (int c = 0; c < anc(params[i]) && k < oslg::kClosureParamFloats; ++c)
                        P.heap[ns + 4 + k++] = (t == oslg::TC_INT || t == oslg::TC_STRING || t == oslg::TC_CLOSURE)
                                                   ? word(P, params[i], c)
                                                   : fbits(getf(P, params[i], c, 0));
                }
                // zero padding to the node's capacity: 12 words, 20 when more are filled
                const int kpad = k <= oslg::kRecordParams ? oslg::kRecordParams : oslg::kClosureParamFloats;
                for (; k < kpad; ++k) P.heap[ns + 4 + k] = fbits(0.0f);
                if (!stat) setw(P, a[0], 0, h);
                break;
            }
            case oslg::OP_CLOSURE_MUL: {
                // osl_mul_closure_color / _float (opclosure.cpp:35-80)
                uint32_t c = word(P, a[1], 0);
                V3 w(getf(P, a[2], 0, 0), getf(P, a[2], 1, 0), getf(P, a[2], 2, 0));
                if (c == 0u || (w.x == 0.0f && w.y == 0.0f && w.z == 0.0f)) { setw(P, a[0], 0, 0u); break; }
                if (w.x == 1.0f && w.y == 1.0f && w.z == 1.0f) { setw(P, a[0], 0, c); break; }
                uint32_t h = cl_alloc(P, C);
                if (!h) { setw(P, a[0], 0, 0u); break; }
                uint32_t ns = nslot(C, h - 1);
                P.heap[ns] = (uint32_t)oslg::kClosureMul;
                P.heap[ns + 1] = fbits(w.x); P.heap[ns + 2] = fbits(w.y); P.heap[ns + 3] = fbits(w.z);
                P.heap[ns + 4] = c;
                setw(P, a[0], 0, h);
                break;
            }
            case oslg::OP_CLOSURE_ADD: {
                // osl_add_closure_closure (opclosure.cpp:15-33)
                uint32_t x = word(P, a[1], 0), y = word(P, a[2], 0);
                if (x == 0u) { setw(P, a[0], 0, y); break; }
                if (y == 0u) { setw(P, a[0], 0, x); break; }
                uint32_t h = cl_alloc(P, C);
                if (!h) { setw(P, a[0], 0, 0u); break; }
                uint32_t ns = nslot(C, h - 1);
                P.heap[ns] = (uint32_t)oslg::kClosureAdd;
                P.heap[ns + 4] = x;
                P.heap[ns + 5] = y;
                setw(P, a[0], 0, h);
                break;
            }
            case oslg::OP_STORE_CLOSURE:
            case oslg::OP_CL_STORE: {
                uint32_t maxc = a[3];
                uint32_t* q = reinterpret_cast<uint32_t*>(outputs + (int64_t)a[1] + P.pt * (int64_t)(int32_t)a[2]);
                uint32_t n = 0;
                auto walk = [&](auto&& visit) {
                    if (op.code == oslg::OP_CL_STORE) closure_walk_static(P, &prog.ops[pc + 1], a[0], visit);
                    else closure_walk(P, C, word(P, a[0], 0), visit);
                };
                walk([&](int id, const V3& cw, uint32_t params) {
                    if (n >= maxc) return;
                    uint32_t* rec = q + 1 + n * oslg::kRecordFloats;
                    rec[0] = (uint32_t)id;
                    rec[1] = fbits(cw.x); rec[2] = fbits(cw.y); rec[3] = fbits(cw.z);
                    for (int k = 0; k < oslg::kRecordParams; ++k) rec[4 + k] = P.heap[params + k];
                    ++n;
                });
                q[0] = n;
                break;
            }
            case oslg::OP_BSDF_EVAL:
            case oslg::OP_CL_BSDF_EVAL: {
                // testrender CompositeBSDF built by the closure walk, then
                // prepare(wo, 1, absorb=false) and eval(wo, wi) (shading.h:322-374)
                V3 wi(getf(P, a[3], 0, 0), getf(P, a[3], 1, 0), getf(P, a[3], 2, 0));
                V3 wo(-getf(P, a[4], 0, 0), -getf(P, a[4], 1, 0), -getf(P, a[4], 2, 0));
                CompositeLobes L;
                if (op.code == oslg::OP_CL_BSDF_EVAL)
                    collect_lobes(
                        P, [&](auto&& visit) { closure_walk_static(P, &prog.ops[pc + 1], a[0], visit); }, wo, a[5],
                        &L, 0.0f, false);
                else
                    build_lobes(P, C, word(P, a[0], 0), wo, a[5], &L);
                L.prepare(wo, V3(1.0f), false);
                Sample sres = L.eval(wo, wi);
                float* o = reinterpret_cast<float*>(outputs + (int64_t)a[1] + P.pt * (int64_t)(int32_t)a[2]);
                o[0] = sres.weight.x; o[1] = sres.weight.y; o[2] = sres.weight.z; o[3] = sres.pdf;
                break;
            }
            case oslg::OP_BSDF_SAMPLE:
            case oslg::OP_CL_BSDF_SAMPLE: {
                // process_closure + prepare(wo, path_weight, absorb) + sample
                // (simpleraytracer.cpp:1038-1079, shading.h:322-398). Userdata
                // record: rx ry rz, path weight rgb, absorb, ray roughness,
                // backfacing; output record: wi xyz, weight rgb, pdf, Le rgb,
                // roughness.
                V3 wo(-getf(P, a[3], 0, 0), -getf(P, a[3], 1, 0), -getf(P, a[3], 2, 0));
                const float* in = reinterpret_cast<const float*>(userdata + (int64_t)a[5] + P.pt * (int64_t)(int32_t)a[6]);
                CompositeLobes L;
                if (op.code == oslg::OP_CL_BSDF_SAMPLE)
                    collect_lobes(
                        P, [&](auto&& visit) { closure_walk_static(P, &prog.ops[pc + 1], a[0], visit); }, wo, a[4],
                        &L, in[7], in[8] != 0.0f);
                else
                    build_lobes(P, C, word(P, a[0], 0), wo, a[4], &L, in[7], in[8] != 0.0f);
                L.prepare(wo, V3(in[3], in[4], in[5]), in[6] != 0.0f);
                Sample sres = L.sample(wo, in[0], in[1], in[2]);
                float* o = reinterpret_cast<float*>(outputs + (int64_t)a[1] + P.pt * (int64_t)(int32_t)a[2]);
                o[0] = sres.wi.x; o[1] = sres.wi.y; o[2] = sres.wi.z;
                o[3] = sres.weight.x; o[4] = sres.weight.y; o[5] = sres.weight.z;
                o[6] = sres.pdf;
                o[7] = L.Le.x; o[8] = L.Le.y; o[9] = L.Le.z;
                o[10] = sres.roughness;
                break;
            }
            case oslg::OP_SPLINEINV: op_splineinverse(P, a); break;
            case oslg::OP_SPLINE: {
                uint32_t r = a[0], xa = a[1], kn = a[2];
                int alen = (int)a[5];
                int kcount = a[4] != oslg::kNoArg ? geti(P, a[4], 0) : alen;
                if (kcount > alen) kcount = alen;
                int nc = anc(r), kc = anc(kn);
                if (kcount < 4) {  // a spline needs four knots
                    P.status |= oslg::ST_ARRAY_BOUNDS;
                    for (int c = 0; c < nc; ++c) putd(P, r, c, DF(0.0f));
                    break;
                }
                bool kd = ader(kn);
                for (int c = 0; c < nc; ++c) {
                    int cc = kc == 1 ? 0 : c;
                    auto knot = [&](int k) {
                        float v = bitsf(word(P, kn, k * kc + cc));
                        if (!kd) return DF(v);
                        return DF(v, bitsf(word(P, kn, alen * kc + k * kc + cc)),
                                  bitsf(word(P, kn, 2 * alen * kc + k * kc + cc)));
                    };
                    DF res = spline_channel((int)a[3], getd(P, xa, 0), ader(xa), kd, kcount, knot);
                    if (!ader(r)) putv(P, r, c, res.v);
                    else putd(P, r, c, res);
                }
                break;
            }
            default:
                P.status |= oslg::ST_BAD_OPCODE;
                break;
            }
            ++pc;
        }
    }
};

bool resolve(Prog& p, const void* blob, size_t bytes) {
    if (bytes < sizeof(oslg::ProgramHeader)) return false;
    p.h = static_cast<const oslg::ProgramHeader*>(blob);
    if (p.h->magic != oslg::kProgramMagic) return false;
    size_t need = sizeof(oslg::ProgramHeader) + (size_t)p.h->nops * sizeof(Op) + (size_t)p.h->nconst * 4;
    if (bytes < need) return false;
    p.ops = reinterpret_cast<const Op*>(static_cast<const uint8_t*>(blob) + sizeof(oslg::ProgramHeader));
    p.pool = reinterpret_cast<const uint32_t*>(p.ops + p.h->nops);
    int n = (int)p.h->nops;
    p.partner.assign(n, n);
    p.break_target.assign(n, n);
    p.continue_target.assign(n, n);
    p.layer_end_after.assign(n, n);
    for (int i = 0; i < n; ++i) {
        const Op& o = p.ops[i];
        if (o.code == oslg::OP_IF || o.code == oslg::OP_ELSE || o.code == oslg::OP_LOOP_TEST) p.partner[i] = (int)o.a[2];
    }
    // BREAK/CONTINUE: the enclosing loop's LOOP_END / LOOP_STEP with the same level tag
    for (int i = 0; i < n; ++i) {
        const Op& o = p.ops[i];
        if (o.code == oslg::OP_BREAK || o.code == oslg::OP_CONTINUE) {
            for (int j = i + 1; j < n; ++j) {
                const Op& q = p.ops[j];
                if (q.a[3] != o.a[3]) continue;
                if (o.code == oslg::OP_BREAK && q.code == oslg::OP_LOOP_END) { p.break_target[i] = j; break; }
                if (o.code == oslg::OP_CONTINUE && q.code == oslg::OP_LOOP_STEP) { p.continue_target[i] = j; break; }
            }
        }
        if (o.code == oslg::OP_RETURN || o.code == oslg::OP_EXIT)
            for (int j = i + 1; j < n; ++j)
                if (p.ops[j].code == oslg::OP_LAYER_END) { p.layer_end_after[i] = j; break; }
    }
    p.final_section = n;
    for (int j = 0; j < n; ++j)
        if (p.ops[j].code == oslg::OP_STORES_END && p.ops[j].a[0] == 1u) { p.final_section = j; break; }
    return true;
}

}  // namespace

extern "C" {

// Register texture `id` (the same index the executor assigned) for the
// oracle's texture lookups.
int oracle_texture_create(int id, int width, int height, int nchannels, const float* texels) {
    if (id < 0 || id > 255 || width < 1 || height < 1 || nchannels < 1) return -1;
    std::vector<OTexture>& t = otextures();
    if ((int)t.size() <= id) t.resize(id + 1);
    otex_build(t[id], width, height, nchannels, texels);
    return 0;
}

// Run a lowered program over points [begin, end) on the host. Globals,
// userdata and outputs are host memory with the device layout.
int oracle_run(const void* blob, size_t bytes, int64_t begin, int64_t end, const oslg_shaderglobals* G,
               void* userdata, void* outputs, int nthreads, uint32_t* status_out) {
    Prog p;
    if (!resolve(p, blob, bytes)) return 1;
    uint32_t status = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : status)
#endif
    {
        Runner R{ p, *G, static_cast<char*>(userdata), static_cast<char*>(outputs) };
        Point P;
        P.heap.assign(p.h->heap_slots + 1, 0u);
        P.pool = p.pool;
#ifdef _OPENMP
#pragma omp for schedule(static, 16)
#endif
        for (int64_t i = begin; i < end; ++i) {
            P.pt = i;
            P.status = 0;
            R.run_point(P);
            status |= P.status;
        }
    }
    if (status_out) *status_out = status;
    return 0;
}

// Scalar noise entry for known-answer tests: kind as NoiseKind, `in` holds
// up to 4 Dual2 inputs (val,dx,dy each), out 3 Dual2 results.
void oracle_noise(int kind, int dims, int vec, int derivs, int periodic, const float* in, const float* periods,
                  float* out) {
    Point P;
    // lay the operands out in a tiny heap: S (3 comps + derivs) at 0, T at 9,
    // result at 12, periods at 21..24
    P.heap.assign(32, 0u);
    P.pool = nullptr;
    P.pt = 0;
    int ns = dims >= 3 ? 3 : 1;
    for (int c = 0; c < ns; ++c)
        for (int d = 0; d < 3; ++d) P.heap[d * ns + c] = fbits(in[c * 3 + d]);
    if (dims == 2 || dims == 4)
        for (int d = 0; d < 3; ++d) P.heap[9 + d] = fbits(in[ns * 3 + d]);
    for (int i = 0; i < 4; ++i) P.heap[21 + i] = fbits(periods ? periods[i] : 1.0f);
    uint32_t a[7];
    a[0] = oslg::arg_make(12, false, true, vec ? oslg::TC_TRIPLE : oslg::TC_FLOAT);
    a[1] = oslg::arg_make(0, false, true, ns == 3 ? oslg::TC_TRIPLE : oslg::TC_FLOAT);
    a[2] = (dims == 2 || dims == 4) ? oslg::arg_make(9, false, true, oslg::TC_FLOAT) : oslg::kNoArg;
    a[3] = oslg::noise_word((uint32_t)kind, periodic != 0, dims, vec != 0, derivs != 0);
    a[4] = oslg::arg_make(21, false, false, ns == 3 ? oslg::TC_TRIPLE : oslg::TC_FLOAT);
    a[5] = oslg::arg_make(24, false, false, oslg::TC_FLOAT);
    a[6] = 0;
    if (!periodic && ns == 1 && dims == 2) a[4] = oslg::kNoArg;
    op_noise(P, a);
    int nr = vec ? 3 : 1;
    for (int c = 0; c < nr; ++c)
        for (int d = 0; d < 3; ++d) out[c * 3 + d] = bitsf(P.heap[12 + d * nr + c]);
}

// Gabor of one Dual2<Vec3> position (in: val xyz, dx xyz, dy xyz) with the
// executor's own exp/sincos (libm = 0) or libm's (libm = 1); out: nc x
// (val, dx, dy).
void oracle_gabor(int anisotropic, int do_filter, const float* direction, float bandwidth, float impulses,
                  const float* in, int periodic, const float* period, int nc, int libm, float* out) {
    GaborOptions o;
    o.anisotropic = anisotropic;
    o.do_filter = do_filter;
    o.direction = V3(direction[0], direction[1], direction[2]);
    o.bandwidth = bandwidth;
    o.impulses = impulses;
    DV X(V3(in[0], in[1], in[2]), V3(in[3], in[4], in[5]), V3(in[6], in[7], in[8]));
    V3 per = period ? V3(period[0], period[1], period[2]) : V3(0.0f);
    DF res[3];
    if (libm) gabor_eval<LibmMath>(o, X, periodic != 0, per, nc, res);
    else gabor_eval<OwnMath>(o, X, periodic != 0, per, nc, res);
    for (int c = 0; c < nc; ++c) { out[c * 3] = res[c].v; out[c * 3 + 1] = res[c].dx; out[c * 3 + 2] = res[c].dy; }
}
// the executor's own exp and sincos over an array (accuracy tests)
void oracle_own_exp(const float* x, int n, float* y) { for (int i = 0; i < n; ++i) y[i] = own_exp(x[i]); }
void oracle_own_sincos(const float* x, int n, float* s, float* c) {
    for (int i = 0; i < n; ++i) own_sincos(x[i], &s[i], &c[i]);
}

int oracle_hash_f(float x) { return hash_f(x); }
uint32_t oracle_inthash(const uint32_t* k, int n) {
    switch (n) {
    case 1: return inthash(k[0]);
    case 2: return inthash(k[0], k[1]);
    case 3: return inthash(k[0], k[1], k[2]);
    case 4: return inthash(k[0], k[1], k[2], k[3]);
    default: return inthash(k[0], k[1], k[2], k[3], k[4]);
    }
}

}  // extern "C"
