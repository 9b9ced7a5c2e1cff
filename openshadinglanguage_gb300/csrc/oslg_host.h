// Host-side model of OSL shader masters, groups and the shading system,
// kept to the shape of the reference API so a renderer written against
// ShadingSystem / ShaderGroup can drive this executor:
//   ShadingSystem        src/include/OSL/oslexec.h:170
//   ShaderGroupBegin/End, Parameter, Shader, ConnectShaders  oslexec.h:634-771
//   SymLocationDesc / add_symlocs                            oslexec.h:69-105, :1075
//   BatchedExecutor<W>::execute                              oslexec.h:982-1033
// Masters are read from .oso text (the oslc output format; see
// src/liboslexec/osogram.y and testsuite/*/test.oso).
#pragma once
#include <cstdint>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "oslg_program.h"

namespace oslg {

enum BaseType { BT_INT, BT_FLOAT, BT_TRIPLE, BT_MATRIX, BT_STRING, BT_CLOSURE, BT_VOID };
enum VecSem { VS_NONE, VS_POINT, VS_VECTOR, VS_NORMAL, VS_COLOR };

struct TypeSpec {
    BaseType base = BT_FLOAT;
    VecSem vecsem = VS_NONE;
    int arraylen = 0;  // 0: scalar, >0 fixed array, -1 unsized
    bool is_array() const { return arraylen != 0; }
    int ncomp() const {
        switch (base) {
        case BT_TRIPLE: return 3;
        case BT_MATRIX: return 16;
        case BT_VOID: return 0;
        default: return 1;
        }
    }
    int elems() const { return arraylen > 0 ? arraylen : 1; }
    bool is_float_based() const { return base == BT_FLOAT || base == BT_TRIPLE || base == BT_MATRIX; }
    bool derivable() const { return base == BT_FLOAT || base == BT_TRIPLE; }
    uint32_t tclass() const {
        switch (base) {
        case BT_INT: return TC_INT;
        case BT_TRIPLE: return TC_TRIPLE;
        case BT_MATRIX: return TC_MATRIX;
        case BT_CLOSURE: return TC_CLOSURE;
        case BT_STRING: return TC_STRING;
        default: return TC_FLOAT;
        }
    }
    std::string str() const;
};
bool parse_typespec(const std::string& tok1, const std::string& tok2, TypeSpec& ts, int& consumed);

enum SymKind { SK_PARAM, SK_OPARAM, SK_GLOBAL, SK_LOCAL, SK_TEMP, SK_CONST };

// Symbol (src/liboslexec/osl_pvt.h:474)
struct Symbol {
    std::string name;
    SymKind kind = SK_LOCAL;
    TypeSpec type;
    std::vector<float> fdefault;       // numeric defaults (ints stored as values)
    std::vector<std::string> sdefault; // string defaults
    bool lockgeom = true;              // [[ int lockgeom = 0 ]] makes it varying
    bool has_init_ops = false;
    int initbegin = 0, initend = 0;    // op range of the default-value code
};

// Opcode (src/liboslexec/osl_pvt.h:955)
struct OsoOp {
    std::string name;
    std::vector<int> args;   // symbol indices
    std::vector<int> jumps;  // absolute op indices
    std::string argrw;
    int line = 0;
};

// ShaderMaster (src/liboslexec/oslexec_pvt.h:409)
struct ShaderMaster {
    std::string name;
    std::string shadertype;
    std::vector<Symbol> symbols;
    std::vector<OsoOp> ops;
    int maincodebegin = 0, maincodeend = 0;
    int find_symbol(const std::string& n) const;
};
bool parse_oso(const std::string& text, ShaderMaster& m, std::string& err);

struct InstanceParam {
    std::string name;
    TypeSpec type;
    std::vector<float> fvals;
    std::vector<std::string> svals;
    bool lockgeom = true;
};

struct Connection {
    int srclayer;
    std::string srcparam;
    std::string dstparam;
};

// ShaderInstance (oslexec_pvt.h:1231)
struct Layer {
    std::string layername;
    std::string usage;
    std::shared_ptr<ShaderMaster> master;
    std::vector<InstanceParam> params;
    std::vector<Connection> connections;  // inbound connections to this layer
};

// SymLocationDesc (oslexec.h:69-105)
enum SymArena { ARENA_UNKNOWN = 0, ARENA_HEAP = 1, ARENA_OUTPUTS = 2, ARENA_USERDATA = 3 };
struct SymLoc {
    std::string name;   // "layer.sym" or "sym"
    TypeSpec type;
    bool derivs = false;
    SymArena arena = ARENA_OUTPUTS;
    int64_t offset = 0;
    int64_t stride = 0;
};

// Renderer-side evaluation of a closure output at one light direction
// (testrender's CompositeBSDF::eval): weight rgb + pdf per point.
struct BsdfEvalRequest {
    std::string closure;  // "layer.sym" or "sym"
    float wi[3] = { 0, 0, 1 };
    int64_t offset = 0;
    int64_t stride = 16;
};

// Renderer-side sampling of a closure output (testrender's
// CompositeBSDF::prepare + sample): random numbers, path weight and the
// absorb flag per point from the userdata arena; direction, weight, pdf,
// emission and roughness per point into the output arena.
struct BsdfSampleRequest {
    std::string closure;
    int64_t offset = 0, stride = 44;        // outputs
    int64_t in_offset = 0, in_stride = 36;  // userdata
};

struct SpecKernel;  // oslg_spec.h

// A lowered group ready to run: the op program plus a serialized blob the
// device (or a checker) consumes.
struct CompiledGroup {
    std::vector<uint8_t> blob;   // ProgramHeader + ops + const pool
    ProgramHeader header{};
    std::vector<std::string> op_names;  // reference op each device op came from
    void* d_blob = nullptr;             // device copy (owned by the executor)
    int device = -1;
    std::shared_ptr<SpecKernel> spec;   // specialized kernel, when built
    int retained_words = 0;             // symbol planes its OP_STORE_HEAP ops fill
};

// ShaderGroup (oslexec_pvt.h:1777)
struct ShaderGroup {
    std::string name;
    std::vector<Layer> layers;
    std::vector<std::string> renderer_outputs;
    std::vector<SymLoc> symlocs;
    std::vector<BsdfEvalRequest> bsdf_evals;
    std::vector<BsdfSampleRequest> bsdf_samples;
    bool ended = false;
    std::mutex mutex;  // lowering happens once, under this lock
    std::unique_ptr<CompiledGroup> compiled;
    std::map<int, std::unique_ptr<CompiledGroup>> layer_compiled;  // programs ending at a layer
    // symbols find_symbol retained: each execution keeps their values in
    // `words` planes from `plane` on (ShadingSystem::symbol_address)
    struct Retained {
        int layer;
        std::string name;
        TypeSpec type;
        int plane, words;
    };
    std::vector<std::unique_ptr<Retained>> retained;
    int find_layer(const std::string& n) const;
};

// The OSL release whose behaviour this executor follows (1.16.0), as
// OSL_LIBRARY_VERSION_CODE: 10000 * major + 100 * minor + patch; what
// getattribute("osl:version") answers.
static const int kOslVersionCode = 11600;

// A uniform attribute the renderer answers getattribute with
// (RendererServices::get_attribute for one object, or scene-wide under the
// empty object name); values as device words (strings hashed).
struct RendererAttribute {
    TypeSpec type;
    std::vector<uint32_t> words;
    std::vector<std::string> strings;
};

struct SystemOptions {
    int debug = 0;
    int strict_messages = 1;  // ShadingSystem attribute "strict_messages" (shadingsys.cpp:1078)
    int opt_constant_fold = 1;       // "opt_constant_fold" (shadingsys.cpp:1641)
    int opt_elide_useless_ops = 1;   // "opt_elide_useless_ops" (shadingsys.cpp:1643)
    int opt_static_closures = 1;     // closure trees the lowering knows become term tables
    std::string colorspace = "Rec709";  // "colorspace" (shadingsys.cpp:1613): the colour system's primaries
    int max_closure_components = 16;  // closure tree nodes per point when closures are made inside loops
    int max_closure_terms = 16;
    int max_loop_iterations = 0;  // loop back edges per point (0: the program format's default)
    // transcendental ops in OpenImageIO's fast_* forms, as the reference's
    // default build (USE_FAST_MATH=ON, CMakeLists.txt:145-150); 0: the
    // math-library forms of a USE_FAST_MATH=OFF build
    int fast_math = 1;
    int userdata_isconnected = 0;  // "userdata_isconnected" (shadingsys.cpp:1073): lockgeom=0 params count as connected
    // "raytypes" (shadingsys.cpp:1256-1265): raytype(name) tests bit 1 << position
    std::vector<std::string> raytypes = { "camera", "shadow", "reflection", "refraction",
                                          "diffuse", "glossy", "subsurface", "displacement" };
    int heap_in_smem = -1;  // -1 auto
    int threads_per_block = 256;
    int points_per_thread = 1;
};

// What gettextureinfo reports about a registered texture (the queries of
// RendererServices::get_texture_info over OpenImageIO's image info)
struct TextureInfo {
    int width = 0, height = 0, nchannels = 0;
    std::vector<float> average;  // per channel, over the base level
    bool constant = false;       // every texel the same (average == the texel)
};

class ShadingSystem {
public:
    std::map<std::string, std::shared_ptr<ShaderMaster>> masters;
    std::map<std::string, int> closure_ids;  // registered closure name -> id
    std::map<std::string, int> texture_ids;  // registered texture name -> index
    std::map<std::string, TextureInfo> texture_info;
    std::map<std::pair<std::string, std::string>, RendererAttribute> attributes;  // (object, name)
    std::map<std::string, std::array<float, 16>> named_matrices;  // space -> space-to-common matrix
    SystemOptions opts;
    std::string last_error;
    std::mutex mutex;

    ShadingSystem();
    bool load_memory_compiled_shader(const std::string& name, const std::string& oso);
    std::shared_ptr<ShaderMaster> find_master(const std::string& name);
    bool error(const std::string& msg) { last_error = msg; return false; }
};

// Lowering entry point: group -> device op program (oslg_lower.cpp).
// stop_layer >= 0 lowers the layers [0, stop_layer] only, with the outputs
// those layers write (execute_layer).
bool lower_group(ShadingSystem& ss, ShaderGroup& g, CompiledGroup& out, std::string& err, int stop_layer = -1);

}  // namespace oslg
