// Device op-program format: what the host lowering produces from an
// optimized ShaderGroup and what the sm_103a interpreter executes.
//
// A program is one flat op stream for the whole group: global loads, every
// layer's parameter initialisation and body in layer order, and the stores
// of the renderer outputs (the reference runs the same layers, see
// src/liboslexec/context.cpp:360-396 and batched_llvm_instance.cpp:2060+).
// Structured control flow of the .oso form (if / for / while / dowhile with
// jump targets, src/liboslexec/batched_llvm_gen.cpp:1068, :3806) is
// rewritten into explicit mask ops so that every lane of a warp walks the
// same op index and varying branches become lane masks.
//
// Per-point values live in a slot heap: slot s of point p is
// heap[s * stride + p] (slot-major, point-minor, so a warp touching one slot
// touches consecutive words). Uniform values live in a constant pool that
// every CTA stages into shared memory.
#pragma once
#include <stdint.h>

namespace oslg {

static const uint32_t kProgramMagic = 0x4f534c47u;  // "OSLG"
static const uint32_t kProgramVersion = 8;

// ---- operand words ----------------------------------------------------------
// bits 0..19  slot offset (heap) or index (constant pool)
// bit  20     operand lives in the constant pool
// bit  21     operand carries derivatives ([val][dx][dy] blocks)
// bits 22..24 type class
// bits 25..31 unused
enum TypeClass : uint32_t {
    TC_FLOAT = 0,
    TC_INT = 1,
    TC_TRIPLE = 2,
    TC_MATRIX = 3,
    TC_CLOSURE = 4,
    TC_STRING = 5,
};
static const uint32_t kArgOffsetMask = 0xFFFFFu;
static const uint32_t kArgConst = 1u << 20;
static const uint32_t kArgDerivs = 1u << 21;
static const uint32_t kArgTCShift = 22;

inline uint32_t arg_make(uint32_t off, bool is_const, bool derivs, uint32_t tc) {
    return (off & kArgOffsetMask) | (is_const ? kArgConst : 0u) | (derivs ? kArgDerivs : 0u)
         | (tc << kArgTCShift);
}

// ---- opcodes ------------------------------------------------------------------
// Grouped by handler family; the reference op each implements is named in
// the lowering (oslg_lower.cpp) next to the name table.
enum OpCode : uint16_t {
    OP_NOP = 0,
    // control (mask) ops; a[] holds immediates
    OP_IF,          // a0=cond  a1=depth  a2=pc_else    (else marker index)
    OP_ELSE,        // a1=depth a2=pc_endif a3=loop level+1 (0 = none)
    OP_ENDIF,       // a1=depth a3=loop level+1
    OP_LOOP_BEGIN,  // a1=depth a3=loop level+1
    OP_LOOP_TEST,   // a0=cond a1=depth a2=pc_loop_end a3=loop level+1
    OP_LOOP_STEP,   // a3=loop level+1
    OP_JUMP,        // a2=pc
    OP_LOOP_END,    // a1=depth a3=loop level+1
    OP_BREAK,       // a3=loop level+1
    OP_CONTINUE,    // a3=loop level+1
    OP_RETURN,      // ends the current layer for the active lanes
    OP_EXIT,        // ends the whole group for the active lanes
    OP_LAYER_END,   // re-enables lanes that returned from this layer and those that
                    // exited in it, for the layer's output stores that follow
    // data movement
    OP_LOAD_GLOBAL,   // a0=dst a1=global id
    OP_LOAD_USERDATA, // a0=dst a1=byte offset a2=byte stride a3=bit 0 int, bit 1 the
                      // record carries derivatives
    OP_STORE_OUTPUT,  // a0=src a1=byte offset a2=byte stride a3=flags(bit0 derivs, bit1 int)
    OP_ASSIGN,        // a0=r a1=src
    OP_ZERO_DERIVS,   // a0=r
    OP_COMPREF,       // a0=r a1=triple a2=index
    OP_COMPASSIGN,    // a0=r a1=index a2=value
    OP_MXCOMPREF,     // a0=r a1=matrix a2=row a3=col
    OP_MXCOMPASSIGN,  // a0=r a1=row a2=col a3=value
    OP_CONSTRUCT3,    // a0=r a1=x a2=y a3=z
    OP_AREF,          // a0=r a1=array a2=index a3=arraylen
    OP_AASSIGN,       // a0=array a1=index a2=value a3=arraylen
    OP_MATRIX_DIAG,   // a0=r a1=scalar
    OP_MATRIX16,      // a0=r a1..: first of 16 consecutive scalar operands stored in a[1] as base list (see lowering)
    // arithmetic (float/triple with scalar broadcast; int when every operand is int)
    OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_NEG,
    OP_IADD, OP_ISUB, OP_IMUL, OP_IDIV, OP_IMOD, OP_INEG,
    OP_MMUL,          // matrix * matrix / matrix*scalar
    OP_MDIV,          // matrix / matrix (a*inverse(b))
    OP_TRANSPOSE, OP_DETERMINANT,
    // compare / logic (result int)
    OP_EQ, OP_NEQ, OP_LT, OP_GT, OP_LE, OP_GE,
    OP_AND, OP_OR,
    OP_BITAND, OP_BITOR, OP_XOR, OP_SHL, OP_SHR, OP_COMPL,
    // unary math on float/triple (componentwise, Dual2-aware)
    OP_ABS, OP_FLOOR, OP_CEIL, OP_ROUND, OP_TRUNC, OP_SIGN,
    OP_SQRT, OP_INVSQRT, OP_CBRT,
    OP_SIN, OP_COS, OP_TAN, OP_ASIN, OP_ACOS, OP_ATAN, OP_SINH, OP_COSH, OP_TANH,
    OP_EXP, OP_EXP2, OP_EXPM1, OP_LOG, OP_LOG2, OP_LOG10,
    OP_RADIANS, OP_DEGREES,
    OP_ISNAN, OP_ISINF, OP_ISFINITE,
    OP_IABS,
    // binary / ternary math
    OP_POW, OP_ATAN2, OP_FMOD, OP_MIN, OP_MAX, OP_IMIN, OP_IMAX,
    OP_CLAMP, OP_MIX, OP_STEP, OP_SMOOTHSTEP, OP_SELECT,
    // vector
    OP_DOT, OP_CROSS, OP_LENGTH, OP_NORMALIZE, OP_DISTANCE,
    // derivatives
    OP_DX, OP_DY, OP_AREA, OP_FILTERWIDTH,
    // matrix / transforms (a2 = matrix operand, a3 = kind: 0 point, 1 vector, 2 normal)
    OP_TRANSFORM,
    // noise family (a3 = NoiseKind | flags, see below)
    OP_NOISE,        // a0=r a1=S a2=T (or 0xFFFFFFFF) a3=kind word a4=Speriod a5=Tperiod
    OP_GABOR,        // a0=r a1=S a2=T a3=kind word a4..a6 option operands
    OP_HASH,         // a0=r(int) a1=x a2=y (or none)
    // spline: a0=r a1=x a2=knots (array) a3=basis id a4=nknots
    OP_SPLINE,
    // color
    OP_BLACKBODY, OP_LUMINANCE,
    // closures: a0=r a1=closure id a2.. params (see lowering)
    OP_CLOSURE,      // a0=r a1=closure id a2=weight (or kNoArg) a3..a6 first params;
                     // an OP_NOP carrier with 7 operands may follow with more params
    OP_CLOSURE_MUL,  // a0=r a1=closure a2=weight (float or color)
    OP_CLOSURE_ADD,  // a0=r a1=a a2=b
    OP_STORE_CLOSURE,// a0=src a1=byte offset a2=byte stride a3=max components
    OP_BSDF_EVAL,    // a0=closure a1=byte offset a2=byte stride a3=wi (triple)
                     // a4=I (triple global) a5=hash("ggx")
    OP_BSDF_SAMPLE,  // a0=closure a1=out byte offset a2=out byte stride a3=I (triple
                     // global) a4=hash("ggx") a5=userdata byte offset a6=userdata stride
    OP_TEXTURE,      // a0=r (float or triple) a1=s a2=t (Dual2: the footprint) a3=texture
                     // index | swrap << 8 | twrap << 12 | firstchannel << 16 a4=width
    OP_SETMESSAGE,   // a0=state (int) a1=store a2=value a3=words | type id << 16
    OP_GETMESSAGE,   // a0=r (int) a1=state a2=store a3=dest a4=words | type id << 16
                     // | strict << 31
    OP_ENVIRONMENT,  // a0=r (float or triple) a1=R (triple, Dual2: the footprint)
                     // a3=texture index | firstchannel << 16 a4=width
    OP_SPLINEINV,    // a0=r (float) a1=y (float) a2=knots (float array) a3=basis id
                     // a4=knot count operand or kNoArg a5=array length
    // static closures (see kClosureAbsent): a closure tree whose shape the
    // lowering knows is kept as one component node per closure op at a
    // fixed heap slot; consumers visit a term table instead of walking
    OP_CLOSURE_NODE, // as OP_CLOSURE, but a0 = the node's first heap slot (an int
                     // operand) and no result handle
    OP_CL_STORE,     // a0=terms a1=byte offset a2=byte stride a3=max components;
                     // term table in the OP_NOP carriers that follow
    OP_CL_BSDF_EVAL, // a0=terms a1..a5 as OP_BSDF_EVAL; term table follows
    OP_CL_BSDF_SAMPLE,// a0=terms a1..a6 as OP_BSDF_SAMPLE; term table follows
    // colour spaces (ColorSystem, src/liboslexec/opcolor.cpp:270-380)
    OP_TRANSFORMC,   // a0=r (triple) a1=C (triple) a2=from space | to space << 8
                     // a3=colour system table (9 XYZ->RGB then 9 RGB->XYZ floats)
    OP_WAVELENGTH,   // a0=r (triple) a1=lambda (float) a2=table (9 XYZ->RGB then 81 x 3 CIE)
    // more componentwise unary math (as OP_ABS..): logb has no derivatives
    OP_LOGB, OP_ERF, OP_ERFC,
    OP_SINCOS,       // a0=x a1=sine result a2=cosine result (float or triple)
    OP_CALCNORMAL,   // a0=r (triple) a1=P (triple with derivatives); reads flipHandedness
    OP_RAYTYPE,      // a0=r (int) a1=name (string) or kNoArg a2=the name's bit (when a1 is
                     // kNoArg) a3=raytype name hashes (ints) a4=count: r = raytype & bit != 0
    // user-function bodies with early returns (oslc's functioncall op): a
    // return inside ends the body for the point; tag a3 = depth + 1
    OP_FUNC_BEGIN,   // a1=depth a2=pc of the OP_FUNC_END a3=tag
    OP_FUNC_RETURN,  // a2=pc of the OP_FUNC_END a3=tag
    OP_FUNC_END,     // a1=depth a3=tag
    OP_STORES_END,   // after a layer's output stores: lanes that exited stay off from
                     // here; a0 = 1: the renderer-side section, every point
    OP_STORE_HEAP,   // a0=symbol a1=first plane a2=words: a retained symbol's values
                     // (find_symbol / symbol_address) into the launch's symbol planes
    OP_COUNT
};

// noise kind word (OP_NOISE a3): bits 0..3 kind, bit 4 periodic, bits 5..7 dims,
// bit 8 result is a triple, bit 9 compute derivatives
enum NoiseKind : uint32_t {
    NK_PERLIN = 0,   // signed ("perlin" / "snoise")
    NK_UPERLIN = 1,  // unsigned ("uperlin" / "noise")
    NK_CELL = 2,
    NK_HASH = 3,
    NK_SIMPLEX = 4,
    NK_USIMPLEX = 5,
    NK_GABOR = 6,
    NK_NULL = 7,
    NK_UNULL = 8,
};
inline uint32_t noise_word(uint32_t kind, bool periodic, int dims, bool vec, bool derivs) {
    return kind | (periodic ? 16u : 0u) | ((uint32_t)dims << 5) | (vec ? 256u : 0u)
         | (derivs ? 512u : 0u);
}

static const uint32_t kNoArg = 0xFFFFFFFFu;

// Ops that write the point's output record at a1 (byte offset), a2 (stride),
// and the sampling ops that read its userdata record at a5, a6.
#ifdef __CUDACC__
__host__ __device__
#endif
inline bool writes_output_record(uint32_t c) {
    return c == OP_STORE_OUTPUT || c == OP_STORE_CLOSURE || c == OP_BSDF_EVAL || c == OP_BSDF_SAMPLE ||
           c == OP_CL_STORE || c == OP_CL_BSDF_EVAL || c == OP_CL_BSDF_SAMPLE;
}
#ifdef __CUDACC__
__host__ __device__
#endif
inline bool reads_sample_record(uint32_t c) { return c == OP_BSDF_SAMPLE || c == OP_CL_BSDF_SAMPLE; }

// Colour spaces of OP_TRANSFORMC (rgb is the colour system's own space)
enum ColorSpace : uint32_t { CS_RGB = 0, CS_HSV, CS_HSL, CS_YIQ, CS_XYZ, CS_XYY, CS_SRGB };

// The string hash the lowering stores for string operands (FNV-1a, 32 bit),
// usable in constant expressions (keyword names of closure parameters).
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr uint32_t string_hash_const(const char* s, uint32_t h = 2166136261u) {
    return *s ? string_hash_const(s + 1, (h ^ (uint32_t)(unsigned char)*s) * 16777619u) : h;
}
// testrender's closure ids (src/testrender/shading.h:25-61) the BSDF code reads
static const int kIdEmission = 1, kIdDiffuse = 3, kIdOrenNayar = 4, kIdMicrofacet = 8,
                 kIdMxOrenNayarDiffuse = 15, kIdMxDielectric = 17, kIdMxSheen = 23, kIdMxLayer = 27;
// Lobe kinds of the BSDF code (bit k of a lobe-kind mask): the closure id
// each comes from; a specialized kernel compiles only the kinds its
// program's closures can make.
enum LobeKind : int { LK_DIFFUSE = 0, LK_GGX = 1, LK_OREN_NAYAR = 2, LK_SHEEN = 3, LK_MX_OREN_NAYAR = 4,
                      LK_MX_DIELECTRIC = 5 };
#ifdef __CUDACC__
__host__ __device__
#endif
inline uint32_t lobe_kind_bits(int closure_id) {
    return closure_id == kIdDiffuse              ? 1u << LK_DIFFUSE
         : closure_id == kIdMicrofacet           ? 1u << LK_GGX
         : closure_id == kIdOrenNayar            ? 1u << LK_OREN_NAYAR
         : closure_id == kIdMxSheen              ? 1u << LK_SHEEN
         : closure_id == kIdMxOrenNayarDiffuse   ? 1u << LK_MX_OREN_NAYAR
         : closure_id == kIdMxDielectric         ? 1u << LK_MX_DIELECTRIC
                                                 : 0u;
}

// Shader-globals the program can load (OP_LOAD_GLOBAL a1). Each triple
// global with derivatives names its dx / dy fields so the loader can fill
// a Dual2 in one op. Matches the varying members of BatchedShaderGlobals
// (src/include/OSL/batched_shaderglobals.h:77-197).
enum GlobalId : uint32_t {
    G_P = 0, G_DPDX, G_DPDY, G_DPDZ,
    G_I, G_DIDX, G_DIDY,
    G_N, G_NG,
    G_U, G_DUDX, G_DUDY,
    G_V, G_DVDX, G_DVDY,
    G_DPDU, G_DPDV,
    G_TIME, G_DTIME, G_DPDTIME,
    G_PS, G_DPSDX, G_DPSDY,
    G_SURFACEAREA,
    G_FLIPHANDEDNESS, G_BACKFACING,  // int fields
    G_COUNT
};
#ifdef __CUDACC__
__host__ __device__
#endif
inline bool global_is_int(uint32_t id) { return id == G_FLIPHANDEDNESS || id == G_BACKFACING; }

struct Op {
    uint16_t code;
    uint8_t nargs;
    uint8_t flags;
    uint32_t a[7];
};
static_assert(sizeof(Op) == 32, "Op must be 32 bytes");

// Closure storage inside the heap (per point): a node pool holding the
// reference's closure tree (src/include/OSL/oslclosure.h:65-147):
//   component  [id >= 0][w.r w.g w.b][params x 12 or x 20]
//   MUL        [-1][w.r w.g w.b][child]
//   ADD        [-2][.  .  .  ][A][B]
// The pool starts with its node count. A closure value (one heap slot, int
// bits) is node index + 1; 0 is the null closure. A node holds
// kClosureParamFloats parameter words when some closure of the program
// needs more than kRecordParams of them (dielectric_bsdf: N, U, two tints,
// two roughnesses, IOR and distribution are 16 words before its keyword
// parameters), else kRecordParams; the header's node_floats says which.
// Parameter words a component does not fill are zero up to its capacity.
static const int kClosureParamFloats = 20;
static const int kNodeFloats = 4 + kClosureParamFloats;
// Closure output records (OP_STORE_CLOSURE / OP_CL_STORE): per component
// [id][w.rgb][the first kRecordParams parameter words].
static const int kRecordParams = 12;
static const int kRecordFloats = 4 + kRecordParams;
static const int kClosureMul = -1;
static const int kClosureAdd = -2;
static const int kClosureWalkStack = 16;  // testrender's traversal stack
// Static closures. When no closure value depends on control flow (no
// closure write under an if or loop, no return or exit), the lowering knows
// every closure's tree: each closure op gets a node at a fixed heap slot
// ([id][w.rgb][12 params], id kClosureAbsent when its weight is zero), and
// a consumer (record store, BSDF eval or sample) gets the walk of its tree
// unrolled into a term table: per visited component, in the walk's order,
// {node slot, weight operand, presence operand}. The weight operand is the
// product of the MUL weights down to the component times its own weight,
// computed by ordinary ops in the walk's order (kNoArg: the node's own
// weight); the presence operand is an int that is 0 when some MUL weight
// on the way is zero (kNoArg: always present). Two terms per carrier op.
static const int kClosureAbsent = -3;
static const int kMaxStaticTerms = 16;
static const int kBsdfMaxLobes = 8;       // CompositeBSDF::MaxEntries

struct ProgramHeader {
    uint32_t magic;
    uint32_t version;
    uint32_t nops;
    uint32_t nconst;        // floats in the constant pool
    uint32_t heap_slots;    // floats per point
    uint32_t flags;         // bit0 uses closures, bit1 uses derivatives
    uint32_t closure_base;  // heap slot of the closure pools (if bit0)
    uint32_t max_comps;     // closure node pool capacity
    uint32_t max_terms;     // unused
    uint32_t max_depth;     // deepest if/loop nesting (<= 32)
    uint32_t max_loop_iterations;  // loop back edges one point may take (0: kDefaultMaxLoopIterations)
    uint32_t node_floats;   // floats per closure pool node (0: kRecordFloats)
    uint32_t reserved[4];
};
static_assert(sizeof(ProgramHeader) == 64, "header must be 64 bytes");

// A point that takes more loop back edges than this (summed over every loop
// of the program) ends with ST_TIMEOUT instead of running on: the device
// and the oracle count the same thing, one per iteration a point starts
// again. The reference has no such limit (a shader that never leaves a
// loop hangs the renderer); the system attribute "max_loop_iterations"
// overrides the default per lowered program.
static const uint32_t kDefaultMaxLoopIterations = 1u << 24;
#ifdef __CUDACC__
__host__ __device__
#endif
inline uint32_t max_loop_iterations(const ProgramHeader& h) {
    return h.max_loop_iterations ? h.max_loop_iterations : kDefaultMaxLoopIterations;
}
#ifdef __CUDACC__
__host__ __device__
#endif
inline uint32_t node_floats(const ProgramHeader& h) { return h.node_floats ? h.node_floats : (uint32_t)kRecordFloats; }

// Texture wrap modes (OP_TEXTURE), the names of OIIO's TextureOpt::Wrap.
enum TexWrap : uint32_t { TW_PERIODIC = 0, TW_CLAMP = 1, TW_BLACK = 2, TW_MIRROR = 3 };
static const int kTexMaxLevels = 16;

// A registered texture: a mip pyramid of float texels (level 0 the image,
// each next level a 2x2 box reduction), channels interleaved, rows from the
// top (t = 0).
struct TexDesc {
    const float* data;  // device address of the whole pyramid
    int32_t nch, nlevels;
    int32_t w[kTexMaxLevels], h[kTexMaxLevels];
    int64_t off[kTexMaxLevels];  // float offset of each level
};

// Status bits a kernel reports back (OR-ed across points).
enum StatusBits : uint32_t {
    ST_CLOSURE_OVERFLOW = 1u,
    ST_BAD_OPCODE = 2u,
    ST_ARRAY_BOUNDS = 4u,
    ST_TIMEOUT = 8u,
    ST_MESSAGE = 16u,  // message set twice, set after a failed query, or read as another type
};

// Per-point message state word (OP_SETMESSAGE / OP_GETMESSAGE): 0 never
// set, 1 + type id once set, kMsgQueried after a query that found nothing.
static const uint32_t kMsgQueried = 0xFFFFFFFFu;

}  // namespace oslg
