// C ABI over the host model (oslg_host.h), the lowering (oslg_lower.cpp) and
// the device interpreter (oslg_kernels.cu). Every entry point returns an int
// status and leaves a message in oslg_last_error(); no C++ exception crosses
// the boundary (the reference reports through bool returns and an
// ErrorHandler, src/liboslexec/context.cpp:443-451).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <new>

#include "../../include/oslg.h"
#include "oslg_batch.h"
#include "oslg_serve.h"
#include "oslg_exec.h"
#include "oslg_host.h"
#include "oslg_spec.h"
#include "oslg_wavefront.h"

#include <dlfcn.h>

// One pipeline slot of oslg_execute_batch_host: a stream, device copies of
// a chunk's inputs and outputs, and its own scratch heap (slots run
// concurrently).
struct HostSlot {
    cudaStream_t stream = nullptr;
    float* d_glob = nullptr;
    char* d_ud = nullptr;
    char* d_out = nullptr;
    size_t glob_bytes = 0, ud_bytes = 0, out_bytes = 0;
    float* gheap = nullptr;
    size_t gheap_bytes = 0;
};

struct oslg_system {
    oslg::ShadingSystem ss;
    oslg::DeviceState dev;
    std::vector<HostSlot> host_slots;
    // registered textures: host pyramids, uploaded with the descriptor table
    // before the next launch that may read them
    struct Tex {
        std::vector<float> pyramid;
        oslg::TexDesc desc;
        bool stale = true;  // pyramid not (or no longer) in device memory
    };
    std::vector<Tex> textures;
    bool textures_dirty = false;
    oslg::LaunchConfig launch;
    int jit = 0;  // build a specialized kernel per group at optimize time
    int jit_block = 0;       // specialized launch: threads per CTA (0: 256)
    int jit_pool_smem = -1;  // closure pools: 1 shared memory, 0 HBM, -1 shared when it fits
    int jit_min_blocks = 0;  // register cap of specialized kernels (256-thread CTAs per SM; 0: automatic)
    int host_direct_outputs = 1;  // host-buffer execution: kernels write pinned output records directly
    std::string err;
    std::vector<oslg::InstanceParam> pending_params;  // Parameter() before Shader()
};

struct oslg_group {
    oslg::ShaderGroup g;
    // retained symbols' planes of the last device execution
    float* d_symheap = nullptr;
    size_t symheap_bytes = 0;
    int64_t symheap_points = -1;
    int symheap_words = 0;
    ~oslg_group() { if (d_symheap) cudaFree(d_symheap); }
};

struct oslg_batch {
    oslg_system* sys;
    oslg::BatchExecutor ex;
    int jit = 0;  // the system's "jit" attribute when the batch was created
};

struct oslg_server {
    oslg_system* sys;
    std::unique_ptr<oslg::ShadingServer> srv;
};

struct oslg_wavefront {
    oslg_system* sys;
    std::unique_ptr<oslg::Wavefront> wf;
};

namespace oslg {

ShadingSystem::ShadingSystem() {
    // closure ids follow testrender's ClosureIDs (src/testrender/shading.h:25-61)
    static const char* names[] = { "emission", "background", "diffuse", "oren_nayar", "translucent",
                                   "phong", "ward", "microfacet", "reflection", "fresnel_reflection",
                                   "refraction", "transparent", "debug", "holdout",
                                   "oren_nayar_diffuse_bsdf", "burley_diffuse_bsdf", "dielectric_bsdf",
                                   "conductor_bsdf", "generalized_schlick_bsdf", "translucent_bsdf",
                                   "transparent_bsdf", "subsurface_bssrdf", "sheen_bsdf", "uniform_edf",
                                   "anisotropic_vdf", "medium_vdf", "layer" };
    for (int i = 0; i < (int)(sizeof(names) / sizeof(names[0])); ++i) closure_ids[names[i]] = i + 1;
}

bool ShadingSystem::load_memory_compiled_shader(const std::string& name, const std::string& oso) {
    auto m = std::make_shared<ShaderMaster>();
    std::string err;
    if (!parse_oso(oso, *m, err)) return error("parse of " + name + " failed: " + err);
    std::lock_guard<std::mutex> lock(mutex);
    masters[name] = m;
    return true;
}

std::shared_ptr<ShaderMaster> ShadingSystem::find_master(const std::string& name) {
    std::lock_guard<std::mutex> lock(mutex);
    auto it = masters.find(name);
    return it == masters.end() ? nullptr : it->second;
}

int ShaderGroup::find_layer(const std::string& n) const {
    for (size_t i = 0; i < layers.size(); ++i)
        if (layers[i].layername == n) return (int)i;
    return -1;
}

}  // namespace oslg

namespace {

using namespace oslg;

int fail(oslg_system* sys, int code, const std::string& msg) {
    if (sys) sys->err = msg;
    return code;
}

bool typedesc_to_spec(const oslg_typedesc& t, TypeSpec& ts) {
    ts = TypeSpec();
    ts.arraylen = t.arraylen;
    if (t.basetype == OSLG_BASE_INT32) ts.base = BT_INT;
    else if (t.basetype == OSLG_BASE_STRING) ts.base = BT_STRING;
    else if (t.basetype == OSLG_BASE_FLOAT) {
        if (t.aggregate == OSLG_AGG_VEC3) {
            ts.base = BT_TRIPLE;
            ts.vecsem = t.vecsemantics == OSLG_VEC_COLOR ? VS_COLOR
                      : t.vecsemantics == OSLG_VEC_POINT ? VS_POINT
                      : t.vecsemantics == OSLG_VEC_NORMAL ? VS_NORMAL : VS_VECTOR;
        } else if (t.aggregate == OSLG_AGG_MATRIX44) {
            ts.base = BT_MATRIX;
        } else {
            ts.base = BT_FLOAT;
        }
    } else {
        return false;
    }
    return true;
}

oslg_typedesc spec_to_typedesc(const TypeSpec& ts) {
    oslg_typedesc t;
    std::memset(&t, 0, sizeof(t));
    t.arraylen = ts.arraylen;
    t.aggregate = OSLG_AGG_SCALAR;
    t.vecsemantics = OSLG_VEC_NOXFORM;
    if (ts.base == BT_INT) t.basetype = OSLG_BASE_INT32;
    else if (ts.base == BT_STRING) t.basetype = OSLG_BASE_STRING;
    else {
        t.basetype = OSLG_BASE_FLOAT;
        if (ts.base == BT_MATRIX) t.aggregate = OSLG_AGG_MATRIX44;
        if (ts.base == BT_TRIPLE) {
            t.aggregate = OSLG_AGG_VEC3;
            t.vecsemantics = ts.vecsem == VS_COLOR ? OSLG_VEC_COLOR
                           : ts.vecsem == VS_POINT ? OSLG_VEC_POINT
                           : ts.vecsem == VS_NORMAL ? OSLG_VEC_NORMAL : OSLG_VEC_VECTOR;
        }
    }
    return t;
}

template <class F> int guarded(oslg_system* sys, F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return fail(sys, OSLG_ERR_ARG, "out of host memory");
    } catch (const std::exception& e) {
        return fail(sys, OSLG_ERR_ARG, e.what());
    } catch (...) {
        return fail(sys, OSLG_ERR_ARG, "unknown C++ exception");
    }
}

}  // namespace

extern "C" {

int oslg_create_system(oslg_system** out) {
    if (!out) return OSLG_ERR_ARG;
    try {
        *out = new oslg_system();
    } catch (...) {
        return OSLG_ERR_ARG;
    }
    return OSLG_OK;
}

int oslg_destroy_system(oslg_system* sys) {
    if (!sys) return OSLG_ERR_ARG;
    if (sys->dev.gheap) device_free(sys->dev.gheap);
    if (sys->dev.d_status) device_free(sys->dev.d_status);
    for (const auto& t : sys->textures) cudaFree(const_cast<float*>(t.desc.data));
    cudaFree(sys->dev.d_textures);
    for (HostSlot& S : sys->host_slots) {
        if (S.stream) cudaStreamDestroy(S.stream);
        cudaFree(S.d_glob);
        cudaFree(S.d_ud);
        cudaFree(S.d_out);
        cudaFree(S.gheap);
    }
    delete sys;
    return OSLG_OK;
}

int oslg_attribute_int(oslg_system* sys, const char* name, int value) {
    if (!sys || !name) return OSLG_ERR_ARG;
    std::string n(name);
    if (n == "max_closure_components") sys->ss.opts.max_closure_components = value;
    else if (n == "max_closure_terms") sys->ss.opts.max_closure_terms = value;
    else if (n == "max_loop_iterations") {
        if (value < 0) return fail(sys, OSLG_ERR_ARG, "max_loop_iterations must be >= 0");
        sys->ss.opts.max_loop_iterations = value;
    }
    else if (n == "gpu_block") sys->launch.block = value;
    else if (n == "gpu_points_per_thread") sys->launch.points_per_thread = value;
    else if (n == "gpu_heap_placement") sys->launch.heap_smem = value;
    else if (n == "gpu_grid") sys->launch.grid = value;
    else if (n == "debug") sys->ss.opts.debug = value;
    else if (n == "strict_messages") sys->ss.opts.strict_messages = value != 0;
    else if (n == "opt_constant_fold") sys->ss.opts.opt_constant_fold = value != 0;
    else if (n == "opt_elide_useless_ops") sys->ss.opts.opt_elide_useless_ops = value != 0;
    else if (n == "opt_static_closures") sys->ss.opts.opt_static_closures = value != 0;
    else if (n == "userdata_isconnected") sys->ss.opts.userdata_isconnected = value != 0;
    else if (n == "fast_math") sys->ss.opts.fast_math = value != 0;
    else if (n == "jit") sys->jit = value;
    else if (n == "jit_block") sys->jit_block = value;
    else if (n == "jit_pool_smem") sys->jit_pool_smem = value;
    else if (n == "jit_min_blocks") sys->jit_min_blocks = value;
    else if (n == "host_direct_outputs") sys->host_direct_outputs = value;
    else return fail(sys, OSLG_ERR_ARG, "unknown attribute '" + n + "'");
    if (sys->ss.opts.max_closure_terms > 0xFFFF || sys->ss.opts.max_closure_components > 0xFFFF)
        return fail(sys, OSLG_ERR_ARG, "closure pool capacity must stay below 65536");
    return OSLG_OK;
}

int oslg_attribute_string(oslg_system* sys, const char* name, const char* value) {
    if (!sys || !name || !value) return OSLG_ERR_ARG;
    std::string n(name), v(value);
    if (n == "colorspace") {
        static const char* known[] = { "Rec709", "sRGB", "NTSC", "EBU", "PAL", "SECAM", "SMPTE", "HDTV", "CIE",
                                       "AdobeRGB", "XYZ", "ACES2065-1", "ACEScg" };
        for (const char* k : known)
            if (v == k) {
                sys->ss.opts.colorspace = v;
                return OSLG_OK;
            }
        return fail(sys, OSLG_ERR_ARG, "unknown colour space '" + v + "'");
    }
    return fail(sys, OSLG_ERR_ARG, "unknown string attribute '" + n + "'");
}

int oslg_attribute_strings(oslg_system* sys, const char* name, const char* const* values, int n) {
    if (!sys || !name || n < 0 || (n > 0 && !values)) return OSLG_ERR_ARG;
    std::string nm(name);
    if (nm == "raytypes") {
        if (n > 32) return fail(sys, OSLG_ERR_ARG, "at most 32 raytypes");
        std::vector<std::string> v;
        for (int i = 0; i < n; ++i) {
            if (!values[i]) return OSLG_ERR_ARG;
            v.push_back(values[i]);
        }
        sys->ss.opts.raytypes = v;
        return OSLG_OK;
    }
    return fail(sys, OSLG_ERR_ARG, "unknown string-array attribute '" + nm + "'");
}

int oslg_register_closure(oslg_system* sys, const char* name, int id) {
    if (!sys || !name) return OSLG_ERR_ARG;
    sys->ss.closure_ids[name] = id;
    return OSLG_OK;
}

int oslg_load_memory_compiled_shader(oslg_system* sys, const char* shadername, const char* oso_text) {
    if (!sys || !shadername || !oso_text) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        if (!sys->ss.load_memory_compiled_shader(shadername, oso_text))
            return fail(sys, OSLG_ERR_PARSE, sys->ss.last_error);
        return OSLG_OK;
    });
}

const char* oslg_last_error(oslg_system* sys) { return sys ? sys->err.c_str() : "null system"; }

int oslg_shader_group_begin(oslg_system* sys, const char* groupname, oslg_group** out) {
    if (!sys || !out) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        oslg_group* g = new oslg_group();
        g->g.name = groupname ? groupname : "";
        sys->pending_params.clear();
        *out = g;
        return OSLG_OK;
    });
}

int oslg_parameter(oslg_system* sys, oslg_group* group, const char* name, oslg_typedesc type,
                   const void* value, int lockgeom) {
    if (!sys || !group || !name || !value) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        if (group->g.ended) return fail(sys, OSLG_ERR_STATE, "Parameter() after ShaderGroupEnd");
        InstanceParam p;
        p.name = name;
        p.lockgeom = lockgeom != 0;
        if (!typedesc_to_spec(type, p.type)) return fail(sys, OSLG_ERR_ARG, "unsupported parameter type");
        int elems = type.arraylen > 0 ? type.arraylen : 1;
        if (p.type.base == BT_STRING) {
            const char* const* sv = static_cast<const char* const*>(value);
            for (int i = 0; i < elems; ++i) p.svals.push_back(sv[i] ? sv[i] : "");
        } else if (p.type.base == BT_INT) {
            const int* iv = static_cast<const int*>(value);
            for (int i = 0; i < elems; ++i) p.fvals.push_back((float)iv[i]);
        } else {
            const float* fv = static_cast<const float*>(value);
            int n = elems * p.type.ncomp();
            for (int i = 0; i < n; ++i) p.fvals.push_back(fv[i]);
        }
        sys->pending_params.push_back(p);
        return OSLG_OK;
    });
}

int oslg_shader(oslg_system* sys, oslg_group* group, const char* shaderusage, const char* shadername,
                const char* layername) {
    if (!sys || !group || !shadername) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        if (group->g.ended) return fail(sys, OSLG_ERR_STATE, "Shader() after ShaderGroupEnd");
        auto m = sys->ss.find_master(shadername);
        if (!m) return fail(sys, OSLG_ERR_ARG, std::string("shader '") + shadername + "' is not loaded");
        Layer L;
        L.master = m;
        L.usage = shaderusage ? shaderusage : "surface";
        L.layername = (layername && *layername) ? layername : m->name;
        for (const InstanceParam& p : sys->pending_params) {
            int si = m->find_symbol(p.name);
            if (si < 0 || (m->symbols[si].kind != SK_PARAM && m->symbols[si].kind != SK_OPARAM)) {
                sys->pending_params.clear();
                return fail(sys, OSLG_ERR_ARG, "shader '" + m->name + "' has no parameter '" + p.name + "'");
            }
            InstanceParam q = p;
            // keep the declared type (e.g. a float value for a color param broadcasts)
            const TypeSpec& decl = m->symbols[si].type;
            if (q.type.base == BT_FLOAT && decl.base == BT_TRIPLE && q.fvals.size() == 1)
                q.fvals = { q.fvals[0], q.fvals[0], q.fvals[0] };
            q.type = decl;
            L.params.push_back(q);
        }
        sys->pending_params.clear();
        group->g.layers.push_back(L);
        return OSLG_OK;
    });
}

int oslg_connect_shaders(oslg_system* sys, oslg_group* group, const char* srclayer, const char* srcparam,
                         const char* dstlayer, const char* dstparam) {
    if (!sys || !group || !srclayer || !srcparam || !dstlayer || !dstparam) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        ShaderGroup& g = group->g;
        int s = g.find_layer(srclayer), d = g.find_layer(dstlayer);
        if (s < 0 || d < 0) return fail(sys, OSLG_ERR_ARG, "ConnectShaders: unknown layer");
        if (s >= d) return fail(sys, OSLG_ERR_ARG, "ConnectShaders: source layer must precede destination");
        if (g.layers[s].master->find_symbol(srcparam) < 0)
            return fail(sys, OSLG_ERR_ARG, std::string("ConnectShaders: no source param ") + srcparam);
        int di = g.layers[d].master->find_symbol(dstparam);
        if (di < 0 || g.layers[d].master->symbols[di].kind != SK_PARAM)
            return fail(sys, OSLG_ERR_ARG, std::string("ConnectShaders: no input param ") + dstparam);
        g.layers[d].connections.push_back({ s, srcparam, dstparam });
        return OSLG_OK;
    });
}

int oslg_shader_group_end(oslg_system* sys, oslg_group* group) {
    if (!sys || !group) return OSLG_ERR_ARG;
    if (group->g.layers.empty()) return fail(sys, OSLG_ERR_STATE, "ShaderGroupEnd on an empty group");
    group->g.ended = true;
    return OSLG_OK;
}

int oslg_group_renderer_outputs(oslg_system* sys, oslg_group* group, const char** names, int n) {
    if (!sys || !group || (n > 0 && !names)) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        group->g.renderer_outputs.clear();
        for (int i = 0; i < n; ++i) group->g.renderer_outputs.push_back(names[i]);
        return OSLG_OK;
    });
}

int oslg_add_symlocs(oslg_system* sys, oslg_group* group, const oslg_symloc* locs, int n) {
    if (!sys || !group || (n > 0 && !locs)) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        for (int i = 0; i < n; ++i) {
            SymLoc sl;
            if (!locs[i].name) return fail(sys, OSLG_ERR_ARG, "symloc without a name");
            sl.name = locs[i].name;
            if (!typedesc_to_spec(locs[i].type, sl.type)) {
                if (locs[i].type.basetype != 0) return fail(sys, OSLG_ERR_ARG, "symloc type not supported");
                sl.type = TypeSpec();
                sl.type.base = BT_CLOSURE;  // basetype 0: a closure output record
                sl.type.arraylen = locs[i].type.arraylen;
            }
            sl.derivs = locs[i].derivs != 0;
            sl.arena = (SymArena)locs[i].arena;
            sl.offset = locs[i].offset;
            sl.stride = locs[i].stride;
            if (sl.offset < 0 || (sl.offset & 3) || (sl.stride & 3))
                return fail(sys, OSLG_ERR_ARG, "symloc offset and stride must be non-negative multiples of 4 bytes");
            group->g.symlocs.push_back(sl);
        }
        std::lock_guard<std::mutex> lock(group->g.mutex);
        group->g.compiled.reset();  // placement changed: lower again
        return OSLG_OK;
    });
}

int oslg_group_bsdf_eval(oslg_system* sys, oslg_group* group, const char* closure, const float wi[3],
                         int64_t offset, int64_t stride) {
    if (!sys || !group || !closure || !wi) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        if (offset < 0 || (offset & 3) || (stride & 3))
            return fail(sys, OSLG_ERR_ARG, "bsdf eval offset and stride must be non-negative multiples of 4 bytes");
        BsdfEvalRequest r;
        r.closure = closure;
        for (int i = 0; i < 3; ++i) r.wi[i] = wi[i];
        r.offset = offset;
        r.stride = stride;
        std::lock_guard<std::mutex> lock(group->g.mutex);
        group->g.bsdf_evals.push_back(r);
        group->g.compiled.reset();
        return OSLG_OK;
    });
}

int oslg_group_bsdf_sample(oslg_system* sys, oslg_group* group, const char* closure, int64_t offset, int64_t stride,
                           int64_t in_offset, int64_t in_stride) {
    if (!sys || !group || !closure) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        if (offset < 0 || in_offset < 0 || ((offset | stride | in_offset | in_stride) & 3))
            return fail(sys, OSLG_ERR_ARG, "bsdf sample offsets and strides must be non-negative multiples of 4 bytes");
        BsdfSampleRequest r;
        r.closure = closure;
        r.offset = offset;
        r.stride = stride;
        r.in_offset = in_offset;
        r.in_stride = in_stride;
        std::lock_guard<std::mutex> lock(group->g.mutex);
        group->g.bsdf_samples.push_back(r);
        group->g.compiled.reset();
        return OSLG_OK;
    });
}

// Folder of this library (the interpreter headers live in its csrc/).
static std::string library_dir() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&oslg_create_system), &info) && info.dli_fname) {
        std::string p = info.dli_fname;
        size_t k = p.rfind('/');
        if (k != std::string::npos) return p.substr(0, k);
    }
    return ".";
}

static int upload_textures(oslg_system* sys);

static int ensure_compiled(oslg_system* sys, oslg_group* group, bool upload, bool allow_spec = true) {
    ShaderGroup& g = group->g;
    if (!g.ended) return fail(sys, OSLG_ERR_STATE, "group used before ShaderGroupEnd");
    if (upload && sys->textures_dirty) {
        int rc = upload_textures(sys);
        if (rc != OSLG_OK) return rc;
    }
    std::lock_guard<std::mutex> lock(g.mutex);
    if (!g.compiled) {
        auto cg = std::make_unique<CompiledGroup>();
        std::string err;
        if (!lower_group(sys->ss, g, *cg, err)) return fail(sys, OSLG_ERR_LOWER, "group '" + g.name + "': " + err);
        g.compiled = std::move(cg);
    }
    if (upload && !g.compiled->d_blob) {
        std::string err;
        int rc = device_init(sys->dev, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        rc = device_upload_program(g.compiled->blob.data(), g.compiled->blob.size(), &g.compiled->d_blob, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        g.compiled->device = sys->dev.device;
    }
    if (upload && allow_spec && sys->jit && !g.compiled->spec) {
        auto sk = std::make_shared<SpecKernel>();
        std::string err;
        const std::string dir = library_dir();
        int rc = spec_build(*g.compiled, dir + "/csrc", dir + "/_build/jit", sk.get(), &err, sys->jit_min_blocks);
        if (rc != OSLG_OK) return fail(sys, rc, "group '" + g.name + "': " + err);
        g.compiled->spec = sk;
    }
    return OSLG_OK;
}

int oslg_jit_groups(oslg_system* sys, oslg_group* const* groups, int ngroups, int nthreads) {
    if (!sys || ngroups < 0 || (ngroups > 0 && !groups)) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        // lower and upload every group here, then compile the specialized
        // kernels on worker threads (each build is one nvcc process)
        for (int i = 0; i < ngroups; ++i) {
            if (!groups[i]) return fail(sys, OSLG_ERR_ARG, "null group");
            int rc = ensure_compiled(sys, groups[i], true, false);
            if (rc != OSLG_OK) return rc;
        }
        if (!sys->jit) return OSLG_OK;
        const std::string dir = library_dir();
        std::atomic<int> next{ 0 };
        std::mutex emu;
        std::string first_err;
        auto work = [&]() {
            for (int i = next++; i < ngroups; i = next++) {
                ShaderGroup& g = groups[i]->g;
                std::lock_guard<std::mutex> lock(g.mutex);
                if (!g.compiled || g.compiled->spec) continue;
                auto sk = std::make_shared<SpecKernel>();
                std::string err;
                if (spec_build(*g.compiled, dir + "/csrc", dir + "/_build/jit", sk.get(), &err, sys->jit_min_blocks) !=
                    OSLG_OK) {
                    std::lock_guard<std::mutex> el(emu);
                    if (first_err.empty()) first_err = "group '" + g.name + "': " + err;
                    continue;
                }
                g.compiled->spec = sk;
            }
        };
        int nt = nthreads > 0 ? nthreads : (int)std::max(1u, std::thread::hardware_concurrency());
        nt = std::min(nt, std::max(1, ngroups));
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (std::thread& t : pool) t.join();
        if (!first_err.empty()) return fail(sys, OSLG_ERR_LOWER, first_err);
        return OSLG_OK;
    });
}

int oslg_optimize_group(oslg_system* sys, oslg_group* group) {
    if (!sys || !group) return OSLG_ERR_ARG;
    return guarded(sys, [&]() { return ensure_compiled(sys, group, false); });
}

int oslg_release_group(oslg_system* sys, oslg_group* group) {
    if (!group) return OSLG_ERR_ARG;
    if (group->g.compiled && group->g.compiled->d_blob) device_free(group->g.compiled->d_blob);
    for (auto& kv : group->g.layer_compiled)
        if (kv.second && kv.second->d_blob) device_free(kv.second->d_blob);
    delete group;
    (void)sys;
    return OSLG_OK;
}

int oslg_group_program(oslg_system* sys, oslg_group* group, void* buf, size_t cap, size_t* size) {
    if (!sys || !group) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, false);
        if (rc != OSLG_OK) return rc;
        const std::vector<uint8_t>& b = group->g.compiled->blob;
        if (size) *size = b.size();
        if (buf) std::memcpy(buf, b.data(), std::min(cap, b.size()));
        return OSLG_OK;
    });
}

namespace {
int execute_batch_impl(oslg_system* sys, oslg_group* group, int64_t npoints, const oslg_shaderglobals* globals,
                       const int32_t* shadeindex, void* userdata_base, void* output_base, void* stream) {
    if (!sys || !group || !globals || npoints < 0) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, true);
        if (rc != OSLG_OK) return rc;
        std::string err;
        const CompiledGroup& cg = *group->g.compiled;
        LaunchExtras ex;
        ex.shadeindex = shadeindex;
        if (cg.retained_words > 0 && npoints > 0) {  // planes for find_symbol's symbols
            const size_t need = (size_t)cg.retained_words * (size_t)npoints * sizeof(float);
            if (need > group->symheap_bytes) {
                if (group->d_symheap) cudaFree(group->d_symheap);
                group->d_symheap = nullptr;
                group->symheap_bytes = 0;
                if (cudaMalloc(&group->d_symheap, need) != cudaSuccess)
                    return fail(sys, OSLG_ERR_CUDA, "cudaMalloc of the retained-symbol planes");
                group->symheap_bytes = need;
            }
            ex.symheap = group->d_symheap;
            ex.symheap_stride = npoints;
        }
        if (cg.spec)
            rc = spec_launch(sys->dev, *cg.spec, cg, npoints, *globals, userdata_base, output_base, stream, &err,
                             sys->jit_block, sys->jit_pool_smem, false, &ex);
        else
            rc = device_execute(sys->dev, cg.header, cg.d_blob, npoints, *globals, userdata_base, output_base,
                                stream, sys->launch, &err, &ex);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        group->symheap_points = cg.retained_words > 0 ? npoints : -1;
        group->symheap_words = cg.retained_words;
        return OSLG_OK;
    });
}
}  // namespace

int oslg_find_symbol(oslg_system* sys, oslg_group* group, const char* layername, const char* symbolname,
                     const oslg_symbol** out) {
    if (!sys || !group || !symbolname || !out) return OSLG_ERR_ARG;
    *out = nullptr;
    return guarded(sys, [&]() {
        ShaderGroup& g = group->g;
        std::string lname = layername ? layername : "", sname = symbolname;
        if (lname.empty()) {  // "layer.symbol"
            const size_t dot = sname.find('.');
            if (dot != std::string::npos && g.find_layer(sname.substr(0, dot)) >= 0) {
                lname = sname.substr(0, dot);
                sname = sname.substr(dot + 1);
            }
        }
        int li = -1, msi = -1;
        for (int k = (int)g.layers.size() - 1; k >= 0 && msi < 0; --k) {  // last to first
            if (!lname.empty() && g.layers[(size_t)k].layername != lname) continue;
            const int m = g.layers[(size_t)k].master->find_symbol(sname);
            if (m >= 0) { li = k; msi = m; }
        }
        if (msi < 0) return fail(sys, OSLG_ERR_ARG, "no symbol '" + sname + "' in the group");
        const Symbol& ms = g.layers[(size_t)li].master->symbols[(size_t)msi];
        if (ms.type.base == BT_CLOSURE || ms.kind == SK_GLOBAL)
            return fail(sys, OSLG_ERR_ARG, "symbol '" + sname + "': closures and globals have no address here");
        for (const auto& r : g.retained)
            if (r->layer == li && r->name == sname) {
                *out = reinterpret_cast<const oslg_symbol*>(r.get());
                return OSLG_OK;
            }
        auto r = std::make_unique<ShaderGroup::Retained>();
        r->layer = li;
        r->name = sname;
        r->type = ms.type;
        r->plane = g.retained.empty() ? 0 : g.retained.back()->plane + g.retained.back()->words;
        r->words = ms.type.ncomp() * ms.type.elems();
        *out = reinterpret_cast<const oslg_symbol*>(r.get());
        std::lock_guard<std::mutex> lock(g.mutex);
        g.retained.push_back(std::move(r));
        g.compiled.reset();  // its values must now be kept: lower again
        g.layer_compiled.clear();
        return OSLG_OK;
    });
}

int oslg_symbol_typedesc(const oslg_symbol* sym, oslg_typedesc* out) {
    if (!sym || !out) return OSLG_ERR_ARG;
    const auto* r = reinterpret_cast<const ShaderGroup::Retained*>(sym);
    *out = spec_to_typedesc(r->type);
    return OSLG_OK;
}

int oslg_symbol_address(oslg_system* sys, oslg_group* group, const oslg_symbol* sym, const void** address,
                        int64_t* plane_stride) {
    if (!sys || !group || !sym || !address || !plane_stride) return OSLG_ERR_ARG;
    const auto* r = reinterpret_cast<const ShaderGroup::Retained*>(sym);
    bool mine = false;
    for (const auto& q : group->g.retained) mine = mine || q.get() == r;
    if (!mine) return fail(sys, OSLG_ERR_ARG, "the symbol was found in another group");
    if (group->symheap_points < 0 || r->plane + r->words > group->symheap_words)
        return fail(sys, OSLG_ERR_STATE, "symbol_address: execute the group after find_symbol");
    *address = group->d_symheap + (size_t)r->plane * (size_t)group->symheap_points;
    *plane_stride = group->symheap_points;
    return OSLG_OK;
}

int oslg_execute_batch(oslg_system* sys, oslg_group* group, int64_t npoints, const oslg_shaderglobals* globals,
                       void* userdata_base, void* output_base, void* stream) {
    return execute_batch_impl(sys, group, npoints, globals, nullptr, userdata_base, output_base, stream);
}

int oslg_execute_batch_indexed(oslg_system* sys, oslg_group* group, int64_t npoints,
                               const oslg_shaderglobals* globals, const int32_t* shadeindex, void* userdata_base,
                               void* output_base, void* stream) {
    if (!shadeindex && npoints > 0) return OSLG_ERR_ARG;
    return execute_batch_impl(sys, group, npoints, globals, shadeindex, userdata_base, output_base, stream);
}

// ---- textures ---------------------------------------------------------------------
namespace {
// Mip pyramid: level 0 the image, each next level a 2x2 box average of the
// one before (texel coordinates clamped at odd edges), down to 1x1 or
// kTexMaxLevels levels.
void build_pyramid(int w, int h, int nch, const float* src, std::vector<float>& out, TexDesc& d) {
    d.nch = nch;
    d.nlevels = 0;
    out.assign(src, src + (size_t)w * h * nch);
    int lw = w, lh = h;
    size_t off = 0;
    for (;;) {
        const int lev = d.nlevels++;
        d.w[lev] = lw;
        d.h[lev] = lh;
        d.off[lev] = (int64_t)off;
        if ((lw == 1 && lh == 1) || d.nlevels == kTexMaxLevels) break;
        const int nw = std::max(1, lw / 2), nh = std::max(1, lh / 2);
        const size_t noff = out.size();
        out.resize(noff + (size_t)nw * nh * nch);
        const float* prev = out.data() + off;
        float* next = out.data() + noff;
        for (int y = 0; y < nh; ++y)
            for (int x = 0; x < nw; ++x) {
                const int x0 = std::min(2 * x, lw - 1), x1 = std::min(2 * x + 1, lw - 1);
                const int y0 = std::min(2 * y, lh - 1), y1 = std::min(2 * y + 1, lh - 1);
                for (int c = 0; c < nch; ++c) {
                    const float a = prev[((size_t)y0 * lw + x0) * nch + c], b = prev[((size_t)y0 * lw + x1) * nch + c];
                    const float e = prev[((size_t)y1 * lw + x0) * nch + c], f = prev[((size_t)y1 * lw + x1) * nch + c];
                    next[((size_t)y * nw + x) * nch + c] = (((a + b) + e) + f) * 0.25f;
                }
            }
        off = noff;
        lw = nw;
        lh = nh;
    }
}
}  // namespace

int oslg_texture_create(oslg_system* sys, const char* name, int width, int height, int nchannels,
                        const float* texels, int* index) {
    if (!sys || !name || !texels || width < 1 || height < 1 || nchannels < 1 || nchannels > 64) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        oslg_system::Tex t;
        std::memset(&t.desc, 0, sizeof(t.desc));
        build_pyramid(width, height, nchannels, texels, t.pyramid, t.desc);
        int id;
        auto it = sys->ss.texture_ids.find(name);
        if (it != sys->ss.texture_ids.end()) {  // replace in place: lowered programs keep the index
            id = it->second;
            t.desc.data = sys->textures[id].desc.data;  // the old pyramid, freed at the next upload
            sys->textures[id] = std::move(t);
        } else {
            if (sys->textures.size() >= 256) return fail(sys, OSLG_ERR_ARG, "at most 256 textures");
            id = (int)sys->textures.size();
            sys->textures.push_back(std::move(t));
            sys->ss.texture_ids[name] = id;
        }
        sys->textures_dirty = true;
        TextureInfo info;
        info.width = width;
        info.height = height;
        info.nchannels = nchannels;
        info.constant = true;
        const size_t ntex = (size_t)width * height;
        for (int c = 0; c < nchannels; ++c) {
            double sum = 0.0;
            for (size_t i = 0; i < ntex; ++i) {
                const float v = texels[i * nchannels + c];
                sum += v;
                info.constant = info.constant && v == texels[c];
            }
            info.average.push_back((float)(sum / (double)ntex));
        }
        sys->ss.texture_info[name] = info;
        if (index) *index = id;
        return OSLG_OK;
    });
}

int oslg_renderer_attribute(oslg_system* sys, const char* object, const char* name, oslg_typedesc type,
                            const void* data) {
    if (!sys || !name || !data) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        RendererAttribute a;
        if (!typedesc_to_spec(type, a.type) || a.type.arraylen < 0)
            return fail(sys, OSLG_ERR_ARG, "unsupported attribute type");
        const int elems = a.type.elems();
        if (a.type.base == BT_STRING) {
            const char* const* sv = static_cast<const char* const*>(data);
            for (int i = 0; i < elems; ++i) a.strings.push_back(sv[i] ? sv[i] : "");
        } else {
            const uint32_t* w = static_cast<const uint32_t*>(data);
            a.words.assign(w, w + (size_t)elems * a.type.ncomp());
        }
        sys->ss.attributes[{ object ? object : "", name }] = std::move(a);
        return OSLG_OK;
    });
}

int oslg_renderer_matrix(oslg_system* sys, const char* name, const float* matrix16) {
    if (!sys || !name || !matrix16) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        std::array<float, 16> m;
        std::memcpy(m.data(), matrix16, sizeof(m));
        sys->ss.named_matrices[name] = m;
        return OSLG_OK;
    });
}

// Upload new or replaced texture pyramids and the descriptor table.
static int upload_textures(oslg_system* sys) {
    if (!sys->textures_dirty) return OSLG_OK;
    std::string err;
    int rc = device_init(sys->dev, &err);
    if (rc != OSLG_OK) return fail(sys, rc, err);
    cudaDeviceSynchronize();  // no launch may still read the old table
    std::vector<TexDesc> table;
    for (auto& t : sys->textures) {
        if (t.stale) {
            cudaFree(const_cast<float*>(t.desc.data));
            t.desc.data = nullptr;
            float* dp = nullptr;
            if (cudaMalloc(&dp, t.pyramid.size() * sizeof(float)) != cudaSuccess ||
                cudaMemcpy(dp, t.pyramid.data(), t.pyramid.size() * sizeof(float), cudaMemcpyHostToDevice) !=
                    cudaSuccess) {
                cudaFree(dp);
                return fail(sys, OSLG_ERR_CUDA, "texture upload failed");
            }
            t.desc.data = dp;
            t.stale = false;
        }
        table.push_back(t.desc);
    }
    cudaFree(sys->dev.d_textures);
    sys->dev.d_textures = nullptr;
    if (!table.empty() &&
        (cudaMalloc(&sys->dev.d_textures, table.size() * sizeof(TexDesc)) != cudaSuccess ||
         cudaMemcpy(sys->dev.d_textures, table.data(), table.size() * sizeof(TexDesc), cudaMemcpyHostToDevice) !=
             cudaSuccess))
        return fail(sys, OSLG_ERR_CUDA, "texture table upload failed");
    sys->dev.ntextures = (int32_t)table.size();
    sys->textures_dirty = false;
    return OSLG_OK;
}

// ---- execution over host buffers --------------------------------------------------
namespace {
// components per shader-global field (GlobalId order)
const int kGlobalComps[G_COUNT] = { 3, 3, 3, 3, 3, 3, 3, 3, 3, 1, 1, 1, 1, 1, 1, 3, 3, 1, 1, 3, 3, 3, 3, 1, 1, 1 };

bool cu_ok(oslg_system* sys, cudaError_t e, const char* what, int* rc) {
    if (e == cudaSuccess) return true;
    fail(sys, OSLG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    *rc = OSLG_ERR_CUDA;
    return false;
}

bool grow(void** p, size_t* have, size_t need) {
    if (*have >= need) return true;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    if (cudaMalloc(p, need) != cudaSuccess) return false;
    *have = need;
    return true;
}
}  // namespace

int oslg_execute_batch_host(oslg_system* sys, oslg_group* group, int64_t npoints,
                            const oslg_shaderglobals* host_globals, const void* host_userdata,
                            int64_t userdata_stride, void* host_outputs, int64_t output_stride, int flags) {
    if (!sys || !group || !host_globals || npoints < 0 || userdata_stride < 0 || output_stride < 0 ||
        (npoints > 0 && output_stride > 0 && !host_outputs) || (userdata_stride > 0 && !host_userdata))
        return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, true);
        if (rc != OSLG_OK) return rc;
        const CompiledGroup& cg = *group->g.compiled;
        if (npoints == 0) return OSLG_OK;
        // every arena access of the program must fall inside its point's record
        const Op* ops = reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader));
        for (uint32_t i = 0; i < cg.header.nops; ++i) {
            const Op& op = ops[i];
            const bool out = writes_output_record(op.code);
            if (out && (int64_t)(int32_t)op.a[2] != output_stride)
                return fail(sys, OSLG_ERR_ARG, "output_stride differs from the group's output record stride");
            if (op.code == OP_LOAD_USERDATA && (int64_t)(int32_t)op.a[2] != userdata_stride)
                return fail(sys, OSLG_ERR_ARG, "userdata_stride differs from the group's userdata record stride");
            if (reads_sample_record(op.code) && (int64_t)(int32_t)op.a[6] != userdata_stride)
                return fail(sys, OSLG_ERR_ARG, "userdata_stride differs from the group's sampling record stride");
        }
        // chunks of at most an eighth of the points (>= 64K), three slots in flight
        const int nslots = 3;
        const int64_t chunk = std::min<int64_t>(npoints, std::max<int64_t>(65536, ((npoints + 7) / 8 + 255) / 256 * 256));
        int planes = 0;
        const oslg_field* hf = reinterpret_cast<const oslg_field*>(host_globals);
        for (int f = 0; f < (int)G_COUNT; ++f)
            if (hf[f].data) planes += kGlobalComps[f];
        if ((int)sys->host_slots.size() < nslots) sys->host_slots.resize(nslots);
        for (int k = 0; k < nslots; ++k) {
            HostSlot& S = sys->host_slots[k];
            if (!S.stream && !cu_ok(sys, cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking), "stream", &rc))
                return rc;
            if (!grow(reinterpret_cast<void**>(&S.d_glob), &S.glob_bytes, (size_t)std::max(1, planes) * chunk * 4) ||
                !grow(reinterpret_cast<void**>(&S.d_ud), &S.ud_bytes, (size_t)std::max<int64_t>(4, userdata_stride * chunk)) ||
                !grow(reinterpret_cast<void**>(&S.d_out), &S.out_bytes, (size_t)std::max<int64_t>(4, output_stride * chunk)))
                return fail(sys, OSLG_ERR_CUDA, "cudaMalloc of the host-execution buffers failed");
        }
        const bool preserve = (flags & OSLG_HOST_PRESERVE_OUTPUTS) != 0;
        // Pinned, device-mapped output records and a specialized kernel that
        // stages whole records: the kernel writes the records straight into
        // host memory (over the CPU-GPU link, overlapped with the shading;
        // unwritten words are zeroed in the same pass, or kept when
        // preserving). Otherwise device buffers and copies.
        char* out_direct = nullptr;
        if (sys->host_direct_outputs && output_stride > 0 && cg.spec && cg.spec->stage_stride == (uint32_t)output_stride) {
            cudaPointerAttributes pa;
            if (cudaPointerGetAttributes(&pa, host_outputs) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                pa.devicePointer)
                out_direct = static_cast<char*>(pa.devicePointer);
            else
                cudaGetLastError();
        }
        const int64_t nchunks = (npoints + chunk - 1) / chunk;
        for (int64_t c = 0; c < nchunks; ++c) {
            HostSlot& S = sys->host_slots[c % nslots];
            const int64_t start = c * chunk, n = std::min(chunk, npoints - start);
            oslg_shaderglobals dg = *host_globals;
            oslg_field* df = reinterpret_cast<oslg_field*>(&dg);
            int plane = 0;
            for (int f = 0; f < (int)G_COUNT; ++f) {
                if (!hf[f].data) continue;
                float* base = S.d_glob + (size_t)plane * chunk;
                for (int comp = 0; comp < kGlobalComps[f]; ++comp)
                    if (!cu_ok(sys, cudaMemcpyAsync(base + (size_t)comp * chunk,
                                                    hf[f].data + comp * hf[f].plane_stride + start, (size_t)n * 4,
                                                    cudaMemcpyHostToDevice, S.stream),
                               "input copy", &rc))
                        return rc;
                df[f].data = base;
                df[f].plane_stride = chunk;
                plane += kGlobalComps[f];
            }
            if (userdata_stride > 0 &&
                !cu_ok(sys, cudaMemcpyAsync(S.d_ud, static_cast<const char*>(host_userdata) + start * userdata_stride,
                                            (size_t)(n * userdata_stride), cudaMemcpyHostToDevice, S.stream),
                       "userdata copy", &rc))
                return rc;
            if (output_stride > 0 && !out_direct) {
                char* hout = static_cast<char*>(host_outputs) + start * output_stride;
                const cudaError_t e = preserve ? cudaMemcpyAsync(S.d_out, hout, (size_t)(n * output_stride),
                                                                 cudaMemcpyHostToDevice, S.stream)
                                               : cudaMemsetAsync(S.d_out, 0, (size_t)(n * output_stride), S.stream);
                if (!cu_ok(sys, e, "output preparation", &rc)) return rc;
            }
            DeviceState ds = sys->dev;
            ds.gheap = S.gheap;
            ds.gheap_bytes = S.gheap_bytes;
            std::string err;
            if (cg.spec)
                rc = spec_launch(ds, *cg.spec, cg, n, dg, S.d_ud,
                                 out_direct ? static_cast<void*>(out_direct + start * output_stride) : S.d_out,
                                 S.stream, &err, sys->jit_block, sys->jit_pool_smem, out_direct && !preserve);
            else
                rc = device_execute(ds, cg.header, cg.d_blob, n, dg, S.d_ud, S.d_out, S.stream, sys->launch, &err);
            S.gheap = ds.gheap;
            S.gheap_bytes = ds.gheap_bytes;
            if (rc != OSLG_OK) return fail(sys, rc, err);
            if (output_stride > 0 && !out_direct &&
                !cu_ok(sys, cudaMemcpyAsync(static_cast<char*>(host_outputs) + start * output_stride, S.d_out,
                                            (size_t)(n * output_stride), cudaMemcpyDeviceToHost, S.stream),
                       "output copy", &rc))
                return rc;
        }
        for (int k = 0; k < nslots; ++k)
            if (!cu_ok(sys, cudaStreamSynchronize(sys->host_slots[k].stream), "synchronize", &rc)) return rc;
        uint32_t bits = 0;
        std::string err;
        rc = device_read_status(sys->dev, nullptr, &bits, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        if (bits) return fail(sys, OSLG_ERR_DEVICE, "kernel status bits " + std::to_string(bits));
        return OSLG_OK;
    });
}

// The program that runs layers [0, layer] of the group, lowered and
// uploaded on first use.
static int ensure_layer_compiled(oslg_system* sys, oslg_group* group, int layer, const CompiledGroup** out) {
    ShaderGroup& g = group->g;
    if (!g.ended) return fail(sys, OSLG_ERR_STATE, "group used before ShaderGroupEnd");
    if (sys->textures_dirty) {
        int rc = upload_textures(sys);
        if (rc != OSLG_OK) return rc;
    }
    std::lock_guard<std::mutex> lock(g.mutex);
    std::unique_ptr<CompiledGroup>& slot = g.layer_compiled[layer];
    if (!slot) {
        auto cg = std::make_unique<CompiledGroup>();
        std::string err;
        if (!lower_group(sys->ss, g, *cg, err, layer))
            return fail(sys, OSLG_ERR_LOWER, "group '" + g.name + "' up to layer " + std::to_string(layer) + ": " + err);
        slot = std::move(cg);
    }
    if (!slot->d_blob) {
        std::string err;
        int rc = device_init(sys->dev, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        rc = device_upload_program(slot->blob.data(), slot->blob.size(), &slot->d_blob, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        slot->device = sys->dev.device;
    }
    *out = slot.get();
    return OSLG_OK;
}

int oslg_execute_layer(oslg_system* sys, oslg_group* group, const char* layername, int64_t npoints,
                       const oslg_shaderglobals* globals, void* userdata_base, void* output_base, void* stream) {
    if (!sys || !group || !layername || !globals || npoints < 0) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        const int layer = group->g.find_layer(layername);
        if (layer < 0) return fail(sys, OSLG_ERR_ARG, std::string("no layer '") + layername + "' in the group");
        if (layer == (int)group->g.layers.size() - 1)
            return oslg_execute_batch(sys, group, npoints, globals, userdata_base, output_base, stream);
        const CompiledGroup* cg = nullptr;
        int rc = ensure_layer_compiled(sys, group, layer, &cg);
        if (rc != OSLG_OK) return rc;
        std::string err;
        rc = device_execute(sys->dev, cg->header, cg->d_blob, npoints, *globals, userdata_base, output_base, stream,
                            sys->launch, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        return OSLG_OK;
    });
}

int oslg_group_layer_program(oslg_system* sys, oslg_group* group, const char* layername, void* buf, size_t cap,
                             size_t* size) {
    if (!sys || !group || !layername) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        const int layer = group->g.find_layer(layername);
        if (layer < 0) return fail(sys, OSLG_ERR_ARG, std::string("no layer '") + layername + "' in the group");
        std::lock_guard<std::mutex> lock(group->g.mutex);
        std::unique_ptr<CompiledGroup>& slot = group->g.layer_compiled[layer];
        if (!slot) {
            auto cg = std::make_unique<CompiledGroup>();
            std::string err;
            if (!lower_group(sys->ss, group->g, *cg, err, layer))
                return fail(sys, OSLG_ERR_LOWER, "group '" + group->g.name + "': " + err);
            slot = std::move(cg);
        }
        if (size) *size = slot->blob.size();
        if (buf) std::memcpy(buf, slot->blob.data(), std::min(cap, slot->blob.size()));
        return OSLG_OK;
    });
}

int oslg_group_record_strides(oslg_system* sys, oslg_group* group, int64_t* output_stride, int64_t* userdata_stride) {
    if (!sys || !group || !output_stride || !userdata_stride) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, false);
        if (rc != OSLG_OK) return rc;
        const CompiledGroup& cg = *group->g.compiled;
        const Op* ops = reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader));
        *output_stride = 0;
        *userdata_stride = 0;
        for (uint32_t i = 0; i < cg.header.nops; ++i) {
            const Op& op = ops[i];
            if (writes_output_record(op.code)) *output_stride = (int64_t)(int32_t)op.a[2];
            if (op.code == OP_LOAD_USERDATA) *userdata_stride = (int64_t)(int32_t)op.a[2];
            if (reads_sample_record(op.code)) *userdata_stride = (int64_t)(int32_t)op.a[6];
        }
        return OSLG_OK;
    });
}

int oslg_group_specialized_source(oslg_system* sys, oslg_group* group, char* buf, size_t cap, size_t* size) {
    if (!sys || !group) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, false);
        if (rc != OSLG_OK) return rc;
        const std::string src = spec_source(*group->g.compiled, sys->jit_min_blocks);
        if (size) *size = src.size() + 1;
        if (buf && cap) {
            const size_t n = std::min(cap - 1, src.size());
            std::memcpy(buf, src.data(), n);
            buf[n] = 0;
        }
        return OSLG_OK;
    });
}

int oslg_groups_specialized_batch_source(oslg_system* sys, oslg_group* const* groups, int ngroups, char* buf,
                                         size_t cap, size_t* size) {
    if (!sys || !groups || ngroups < 1) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        std::vector<const CompiledGroup*> cgs;
        for (int i = 0; i < ngroups; ++i) {
            if (!groups[i]) return fail(sys, OSLG_ERR_ARG, "null group");
            int rc = ensure_compiled(sys, groups[i], false);
            if (rc != OSLG_OK) return rc;
            cgs.push_back(groups[i]->g.compiled.get());
        }
        const std::string src = spec_batch_source(cgs);
        if (size) *size = src.size() + 1;
        if (buf && cap) {
            const size_t n = std::min(cap - 1, src.size());
            std::memcpy(buf, src.data(), n);
            buf[n] = 0;
        }
        return OSLG_OK;
    });
}

int oslg_group_is_specialized(oslg_system* sys, oslg_group* group, int* out) {
    if (!sys || !group || !out) return OSLG_ERR_ARG;
    *out = group->g.compiled && group->g.compiled->spec ? 1 : 0;
    return OSLG_OK;
}

int oslg_execute_batch_sync(oslg_system* sys, oslg_group* group, int64_t npoints,
                            const oslg_shaderglobals* globals, void* userdata_base, void* output_base,
                            void* stream) {
    int rc = oslg_execute_batch(sys, group, npoints, globals, userdata_base, output_base, stream);
    if (rc != OSLG_OK) return rc;
    uint32_t bits = 0;
    std::string err;
    rc = device_read_status(sys->dev, stream, &bits, &err);
    if (rc != OSLG_OK) return fail(sys, rc, err);
    if (bits) {
        std::string m = "kernel status:";
        if (bits & ST_CLOSURE_OVERFLOW) m += " closure-arena-overflow";
        if (bits & ST_BAD_OPCODE) m += " bad-opcode";
        if (bits & ST_ARRAY_BOUNDS) m += " index-out-of-range";
        if (bits & ST_TIMEOUT) m += " loop-iteration-limit";
        if (bits & ST_MESSAGE) m += " message-error";
        return fail(sys, OSLG_ERR_DEVICE, m);
    }
    return OSLG_OK;
}

int oslg_device_status(oslg_system* sys, uint32_t* bits) {
    if (!sys || !bits) return OSLG_ERR_ARG;
    std::string err;
    int rc = device_read_status(sys->dev, nullptr, bits, &err);
    if (rc != OSLG_OK) return fail(sys, rc, err);
    // bits the allocation-free entry left when its caller did not ask for them
    uint32_t na = 0;
    rc = noalloc_read_status(nullptr, &na, &err);
    if (rc != OSLG_OK) return fail(sys, rc, err);
    *bits |= na;
    return OSLG_OK;
}

int oslg_set_launch(oslg_system* sys, int block, int points_per_thread, int heap_smem) {
    if (!sys) return OSLG_ERR_ARG;
    if (block > 0) sys->launch.block = block;
    if (points_per_thread > 0) sys->launch.points_per_thread = points_per_thread;
    sys->launch.heap_smem = heap_smem;
    return OSLG_OK;
}

// Allocation-free execute (see include/oslg.h): no lowering, no upload, no
// device allocation; everything the kernel needs goes to a static array.
int oslg_execute_batch_noalloc(oslg_system* sys, oslg_group* group, int64_t npoints,
                               const oslg_shaderglobals* globals, void* userdata_base, void* output_base,
                               void* stream, uint32_t* status_out) {
    if (!sys || !group || !globals || npoints < 0) return OSLG_ERR_ARG;
    ShaderGroup& g = group->g;
    std::lock_guard<std::mutex> lock(g.mutex);
    if (!g.compiled) return fail(sys, OSLG_ERR_STATE, "group must be lowered with oslg_optimize_group first");
    // texture() and environment() read the system's descriptor table, which
    // only the allocating entries upload (it takes device memory)
    int max_tex = -1;
    {
        const CompiledGroup& cg = *g.compiled;
        const Op* ops = reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader));
        for (uint32_t i = 0; i < cg.header.nops; ++i)
            if (ops[i].code == OP_TEXTURE || ops[i].code == OP_ENVIRONMENT)
                max_tex = std::max(max_tex, (int)(ops[i].a[3] & 0xFFu));
    }
    if (max_tex >= 0 && (sys->textures_dirty || !sys->dev.d_textures || max_tex >= sys->dev.ntextures))
        return fail(sys, OSLG_ERR_STATE,
                    "group looks up textures that are not in device memory yet: run a group of this system through "
                    "oslg_execute_batch once after registering them");
    std::string err;
    uint32_t bits = 0;
    int rc = device_execute_noalloc(g.compiled->blob.data(), g.compiled->blob.size(), g.compiled->header, npoints,
                                    *globals, userdata_base, output_base, stream, sys->launch,
                                    max_tex >= 0 ? sys->dev.d_textures : nullptr,
                                    max_tex >= 0 ? sys->dev.ntextures : 0, status_out ? &bits : nullptr, &err);
    if (rc != OSLG_OK) return fail(sys, rc, err);
    if (status_out) {
        *status_out = bits;
        if (bits) return fail(sys, OSLG_ERR_DEVICE, "kernel status bits " + std::to_string(bits));
    }
    return OSLG_OK;
}

}  // extern "C"

// ---- persistent batch executor ----------------------------------------------------
int oslg_batch_create(oslg_system* sys, oslg_batch** out) {
    if (!sys || !out) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        oslg_batch* b = new oslg_batch;
        b->sys = sys;
        b->jit = sys->jit ? 1 : 0;
        if (b->jit) {
            const std::string dir = library_dir();
            b->ex.set_jit_dirs(dir + "/csrc", dir + "/_build/jit");
            BatchLaunch l;
            l.jit = 1;
            b->ex.set_launch(l);
        }
        *out = b;
        return OSLG_OK;
    });
}

int oslg_batch_destroy(oslg_batch* batch) {
    delete batch;
    return OSLG_OK;
}

int oslg_batch_clear(oslg_batch* batch) {
    if (!batch) return OSLG_ERR_ARG;
    batch->ex.clear();
    return OSLG_OK;
}

int oslg_batch_add(oslg_batch* batch, oslg_group* group, int64_t npoints, const oslg_shaderglobals* globals,
                   void* userdata_base, void* output_base) {
    if (!batch || !group || !globals || npoints < 0) return OSLG_ERR_ARG;
    oslg_system* sys = batch->sys;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, true);
        if (rc != OSLG_OK) return rc;
        if (npoints == 0) return OSLG_OK;
        batch->ex.add(*group->g.compiled, npoints, *globals, userdata_base, output_base);
        return OSLG_OK;
    });
}

int oslg_batch_set_launch(oslg_batch* batch, int block, int points_per_thread, int heap_smem, int use_graph) {
    if (!batch || block < 0 || block > 512 || heap_smem < -1 || heap_smem > 1) return OSLG_ERR_ARG;
    if (points_per_thread != 0 && points_per_thread != 1 && points_per_thread != 2 && points_per_thread != 4)
        return OSLG_ERR_ARG;
    BatchLaunch l;
    BatchTuneResult cur;
    batch->ex.last_launch(&cur);
    l.block = block > 0 ? block : (cur.block > 0 ? cur.block : 256);
    l.points_per_thread = points_per_thread > 0 ? points_per_thread : (cur.points_per_thread > 0 ? cur.points_per_thread : 1);
    l.heap_smem = heap_smem;
    l.use_graph = use_graph ? 1 : 0;
    l.jit = batch->jit;
    batch->ex.set_launch(l);
    return OSLG_OK;
}

int oslg_batch_execute(oslg_batch* batch, void* stream) {
    if (!batch) return OSLG_ERR_ARG;
    oslg_system* sys = batch->sys;
    return guarded(sys, [&]() {
        std::string err;
        int rc = device_init(sys->dev, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        rc = batch->ex.execute(sys->dev, stream, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        return OSLG_OK;
    });
}

static void to_c(const BatchTuneResult& r, oslg_batch_tuning* o) {
    o->block = r.block;
    o->points_per_thread = r.points_per_thread;
    o->heap_smem = r.heap_smem;
    o->grid = r.grid;
    o->ctas_per_sm = r.ctas_per_sm;
    o->ms = r.ms;
}

int oslg_batch_autotune(oslg_batch* batch, void* stream, int reps, oslg_batch_tuning* results, int cap, int* n,
                        oslg_batch_tuning* best) {
    if (!batch || cap < 0) return OSLG_ERR_ARG;
    oslg_system* sys = batch->sys;
    return guarded(sys, [&]() {
        std::string err;
        int rc = device_init(sys->dev, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        std::vector<BatchTuneResult> res((size_t)std::max(cap, 32));
        int cnt = 0;
        BatchLaunch bl;
        rc = batch->ex.autotune(sys->dev, stream, reps, res.data(), (int)res.size(), &cnt, &bl, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        if (n) *n = std::min(cnt, cap);
        for (int i = 0; i < std::min(cnt, cap) && results; ++i) to_c(res[i], &results[i]);
        if (best) {
            float bm = 1e30f;
            for (int i = 0; i < std::min(cnt, (int)res.size()); ++i)
                if (res[i].ms < bm) { bm = res[i].ms; to_c(res[i], best); }
        }
        return OSLG_OK;
    });
}

int oslg_batch_last_launch(oslg_batch* batch, oslg_batch_tuning* out) {
    if (!batch || !out) return OSLG_ERR_ARG;
    BatchTuneResult r;
    batch->ex.last_launch(&r);
    to_c(r, out);
    return OSLG_OK;
}

// ---- shading server ---------------------------------------------------------------
int oslg_server_create(oslg_system* sys, const oslg_server_options* opts, oslg_server** out) {
    if (!sys || !out) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        std::string err;
        int rc = device_init(sys->dev, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        ServerOptions o;
        if (opts) {
            if (opts->budget_bytes) o.budget_bytes = opts->budget_bytes;
            if (opts->streams) o.streams = opts->streams;
            if (opts->block) o.block = opts->block;
            if (opts->points_per_thread) o.points_per_thread = opts->points_per_thread;
            if (opts->max_wave_points) o.max_wave_points = opts->max_wave_points;
            if (opts->max_wave_requests) o.max_wave_requests = opts->max_wave_requests;
            o.arena_bytes = opts->arena_bytes;
        }
        if (o.points_per_thread != 1 && o.points_per_thread != 2 && o.points_per_thread != 4)
            return fail(sys, OSLG_ERR_ARG, "points_per_thread must be 1, 2 or 4");
        if (sys->jit) {  // waves run a kernel specialized to the resident programs
            o.jit_csrc = library_dir() + "/csrc";
            o.jit_cache = library_dir() + "/_build/jit";
        }
        std::unique_ptr<oslg_server> s(new oslg_server);
        s->sys = sys;
        s->srv.reset(new ShadingServer(sys->dev, o));
        rc = s->srv->start(&err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        *out = s.release();
        return OSLG_OK;
    });
}

int oslg_server_destroy(oslg_server* server) {
    if (!server) return OSLG_ERR_ARG;
    server->srv->stop();
    delete server;
    return OSLG_OK;
}

int oslg_server_register(oslg_server* server, oslg_group* group) {
    if (!server || !group) return OSLG_ERR_ARG;
    oslg_system* sys = server->sys;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, true);
        if (rc != OSLG_OK) return rc;
        std::string err;
        rc = server->srv->register_program(*group->g.compiled, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        return OSLG_OK;
    });
}

int oslg_server_submit(oslg_server* server, oslg_group* group, int64_t npoints, const oslg_shaderglobals* host_globals,
                       void* host_output, size_t output_bytes, uint64_t* ticket) {
    if (!server || !group || !host_globals || !ticket || npoints < 0) return OSLG_ERR_ARG;
    oslg_system* sys = server->sys;
    return guarded(sys, [&]() {
        int rc = ensure_compiled(sys, group, true);
        if (rc != OSLG_OK) return rc;
        std::string err;
        rc = server->srv->submit(*group->g.compiled, npoints, *host_globals, host_output, output_bytes, ticket, &err);
        if (rc != OSLG_OK) return fail(sys, rc, err);
        return OSLG_OK;
    });
}

static void to_c(const RequestStats& r, oslg_request_stats* o) {
    o->submit_ns = r.submit_ns;
    o->admit_ns = r.admit_ns;
    o->done_ns = r.done_ns;
    o->wave = r.wave;
    o->status = r.status;
}

int oslg_server_wait(oslg_server* server, uint64_t ticket, int timeout_ms, oslg_request_stats* stats) {
    if (!server) return OSLG_ERR_ARG;
    RequestStats st;
    std::string err;
    int rc = server->srv->wait(ticket, timeout_ms, &st, &err);
    if (stats) to_c(st, stats);
    if (rc != OSLG_OK) return fail(server->sys, rc, err);
    return OSLG_OK;
}

int oslg_server_poll(oslg_server* server, uint64_t ticket, int* done, oslg_request_stats* stats) {
    if (!server || !done) return OSLG_ERR_ARG;
    RequestStats st;
    std::string err;
    bool d = false;
    int rc = server->srv->poll(ticket, &d, &st, &err);
    *done = d ? 1 : 0;
    if (d && stats) to_c(st, stats);
    if (rc != OSLG_OK) return fail(server->sys, rc, err);
    return OSLG_OK;
}

int oslg_server_get_stats(oslg_server* server, oslg_server_stats* out) {
    if (!server || !out) return OSLG_ERR_ARG;
    ServerStats s;
    server->srv->stats(&s);
    out->submitted = s.submitted;
    out->completed = s.completed;
    out->failed = s.failed;
    out->waves = s.waves;
    out->points_done = s.points_done;
    out->arena_capacity = s.arena_capacity;
    out->arena_high_water = s.arena_high_water;
    out->program_bytes = s.program_bytes;
    out->scratch_bytes = s.scratch_bytes;
    out->in_flight_waves = s.in_flight_waves;
    out->pending = s.pending;
    return OSLG_OK;
}

// ---- wavefront path tracing ---------------------------------------------------------
static bool wf_check_options(const oslg_wavefront_options& o, std::string* why) {
    if (o.width < 1 || o.height < 1 || o.spp < 1) return *why = "width, height and spp must be positive", false;
    if ((int64_t)o.width * o.height * o.spp > (int64_t)1 << 30) return *why = "more than 2^30 paths", false;
    if (o.max_hits < 1 || o.max_hits > oslg::kWfMaxHits) return *why = "max_hits must be in [1, 16]", false;
    if (!(o.rr_survival > 0.0f && o.rr_survival <= 1.0f)) return *why = "rr_survival must be in (0, 1]", false;
    if (!(o.fov_deg > 0.0f && o.fov_deg < 180.0f)) return *why = "fov_deg must be in (0, 180)", false;
    if (o.block < 0 || o.block > 512) return *why = "block must be in [0, 512]", false;
    return true;
}

static bool wf_check_prim(const oslg_primitive& q, int nmat, std::string* why) {
    if (q.material < 0 || q.material >= nmat) return *why = "material index out of range", false;
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(q.p[k]) || !std::isfinite(q.ex[k]) || !std::isfinite(q.ey[k]))
            return *why = "non-finite coordinate", false;
    if (q.kind == OSLG_PRIM_SPHERE) {
        if (!(q.radius > 0.0f) || !std::isfinite(q.radius)) return *why = "sphere radius must be positive", false;
        return true;
    }
    if (q.kind != OSLG_PRIM_QUAD) return *why = "unknown primitive kind", false;
    const double lx = (double)q.ex[0] * q.ex[0] + (double)q.ex[1] * q.ex[1] + (double)q.ex[2] * q.ex[2];
    const double ly = (double)q.ey[0] * q.ey[0] + (double)q.ey[1] * q.ey[1] + (double)q.ey[2] * q.ey[2];
    const double dxy = (double)q.ex[0] * q.ey[0] + (double)q.ex[1] * q.ey[1] + (double)q.ex[2] * q.ey[2];
    if (!(lx > 0.0 && ly > 0.0)) return *why = "rectangle edge of zero length", false;
    if (std::fabs(dxy) > 1e-5 * std::sqrt(lx * ly)) return *why = "rectangle edges are not orthogonal", false;
    return true;
}

int oslg_wavefront_create(oslg_system* sys, const oslg_wavefront_options* opts, const oslg_primitive* prims,
                          int nprims, oslg_group* const* materials, int nmaterials, oslg_wavefront** out) {
    if (!sys || !opts || !out || nprims < 0 || (nprims > 0 && !prims) || !materials) return OSLG_ERR_ARG;
    return guarded(sys, [&]() {
        std::string why;
        if (!wf_check_options(*opts, &why)) return fail(sys, OSLG_ERR_ARG, "wavefront: " + why);
        if (nmaterials < 1 || nmaterials > oslg::kWfMaxMaterials)
            return fail(sys, OSLG_ERR_ARG, "wavefront: 1 to 64 materials");
        for (int i = 0; i < nprims; ++i)
            if (!wf_check_prim(prims[i], nmaterials, &why))
                return fail(sys, OSLG_ERR_ARG, "wavefront: primitive " + std::to_string(i) + ": " + why);
        std::vector<const CompiledGroup*> mats;
        for (int m = 0; m < nmaterials; ++m) {
            oslg_group* g = materials[m];
            if (!g) return fail(sys, OSLG_ERR_ARG, "wavefront: null material group");
            bool found = false;
            for (const BsdfSampleRequest& r : g->g.bsdf_samples)
                found = found || (r.offset == 0 && r.stride == 4 * oslg::kWfOutFloats && r.in_offset == 0 &&
                                  r.in_stride == 4 * oslg::kWfInFloats);
            if (!found)
                return fail(sys, OSLG_ERR_ARG,
                            "wavefront: material group '" + g->g.name +
                                "' has no bsdf_sample output at offset 0, stride 44, in_offset 0, in_stride 36");
            int rc = ensure_compiled(sys, g, true);
            if (rc != OSLG_OK) return rc;
            mats.push_back(g->g.compiled.get());
        }
        auto w = std::make_unique<oslg_wavefront>();
        w->sys = sys;
        w->wf = std::make_unique<oslg::Wavefront>();
        std::string err;
        const std::string dir = library_dir();
        const std::string jit_dirs[2] = { dir + "/csrc", dir + "/_build/jit" };
        int rc = w->wf->init(sys->dev, *opts, prims, nprims, mats, sys->jit ? jit_dirs : nullptr, &err);
        if (rc != OSLG_OK) return fail(sys, rc, "wavefront: " + err);
        *out = w.release();
        return OSLG_OK;
    });
}

int oslg_wavefront_destroy(oslg_wavefront* wf) {
    delete wf;
    return OSLG_OK;
}

static int wf_render(oslg_wavefront* wf, float* d_path_radiance, float* d_image, void* stream, bool profile) {
    if (!wf) return OSLG_ERR_ARG;
    oslg_system* sys = wf->sys;
    return guarded(sys, [&]() {
        std::string err;
        int rc = wf->wf->render(d_path_radiance, d_image, stream, profile, &err);
        if (rc != OSLG_OK) return fail(sys, rc, "wavefront: " + err);
        return OSLG_OK;
    });
}

int oslg_wavefront_render(oslg_wavefront* wf, float* d_path_radiance, float* d_image, void* stream) {
    return wf_render(wf, d_path_radiance, d_image, stream, false);
}

int oslg_wavefront_render_profiled(oslg_wavefront* wf, float* d_path_radiance, float* d_image, void* stream) {
    return wf_render(wf, d_path_radiance, d_image, stream, true);
}

int oslg_wavefront_get_stats(oslg_wavefront* wf, oslg_wavefront_stats* out) {
    if (!wf || !out) return OSLG_ERR_ARG;
    oslg_system* sys = wf->sys;
    return guarded(sys, [&]() {
        oslg::WavefrontStats s;
        std::string err;
        int rc = wf->wf->stats(&s, &err);
        if (rc != OSLG_OK) return fail(sys, rc, "wavefront: " + err);
        out->paths = s.paths;
        for (int b = 0; b < 16; ++b) out->hits[b] = s.hits[b];
        out->total_hits = s.total_hits;
        out->bounces = s.bounces;
        out->ms_total = s.ms_total;
        for (int k = 0; k < 5; ++k) out->ms_stage[k] = s.ms_stage[k];
        return OSLG_OK;
    });
}
