/* C++ facade over the C ABI in oslg.h with the reference's batched API
 * shape: ShadingSystem::batched<W>().execute(group, batch_size, globals,
 * userdata, outputs) over a W-lane BatchedShaderGlobals
 * (src/include/OSL/oslexec.h:990-1030, batched_shaderglobals.h:77-197,
 * wide.h:439-444 for the Block<Vec3, W> layout), plus an N-point overload
 * over device-resident SoA globals, the executor's native form. Calls return
 * bool and keep the message for geterror(), as the reference's
 * ShadingSystem does. Header only; link liboslg_gb300.so. */
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "oslg.h"

namespace oslg {

struct Vec3 {
    float x, y, z;
};

/* Block<T, W>: one value per lane. Block<Vec3, W> keeps the components as
 * three lane arrays (x[W], y[W], z[W]), i.e. SoA planes W floats apart. */
template <typename T, int W> struct Block {
    T data[W];
    void set(int lane, T v) { data[lane] = v; }
    T get(int lane) const { return data[lane]; }
};
template <int W> struct Block<Vec3, W> {
    float x[W];
    float y[W];
    float z[W];
    void set(int lane, const Vec3& v) {
        x[lane] = v.x;
        y[lane] = v.y;
        z[lane] = v.z;
    }
    Vec3 get(int lane) const { return Vec3{ x[lane], y[lane], z[lane] }; }
};

struct UniformShaderGlobals {
    void* renderstate = nullptr;
    void* tracedata = nullptr;
    void* objdata = nullptr;
    int raytype = 0;
};

/* The varying members the executor reads, in the reference's order. */
template <int W> struct VaryingShaderGlobals {
    Block<Vec3, W> P, dPdx, dPdy, dPdz;
    Block<Vec3, W> I, dIdx, dIdy;
    Block<Vec3, W> N, Ng;
    Block<float, W> u, dudx, dudy;
    Block<float, W> v, dvdx, dvdy;
    Block<Vec3, W> dPdu, dPdv;
    Block<float, W> time, dtime;
    Block<Vec3, W> dPdtime;
    Block<Vec3, W> Ps, dPsdx, dPsdy;
    Block<float, W> surfacearea;
    Block<int, W> flipHandedness;
    Block<int, W> backfacing;
};

template <int W> struct BatchedShaderGlobals {
    UniformShaderGlobals uniform;
    VaryingShaderGlobals<W> varying;
};

using ShaderGroupRef = oslg_group*;

class ShadingSystem {
public:
    ShadingSystem() { ok(oslg_create_system(&sys_)); }
    ~ShadingSystem() {
        if (sys_) oslg_destroy_system(sys_);
    }
    ShadingSystem(const ShadingSystem&) = delete;
    ShadingSystem& operator=(const ShadingSystem&) = delete;

    oslg_system* handle() const { return sys_; }
    /* the message of the last failed call (ShadingSystem::geterror) */
    std::string geterror() const { return error_; }

    bool attribute(const std::string& name, int value) { return ok(oslg_attribute_int(sys_, name.c_str(), value)); }
    bool LoadMemoryCompiledShader(const std::string& name, const std::string& oso) {
        return ok(oslg_load_memory_compiled_shader(sys_, name.c_str(), oso.c_str()));
    }
    ShaderGroupRef ShaderGroupBegin(const std::string& name = std::string()) {
        oslg_group* g = nullptr;
        return ok(oslg_shader_group_begin(sys_, name.c_str(), &g)) ? g : nullptr;
    }
    bool Parameter(ShaderGroupRef g, const std::string& name, oslg_typedesc type, const void* value,
                   bool lockgeom = true) {
        return ok(oslg_parameter(sys_, g, name.c_str(), type, value, lockgeom ? 1 : 0));
    }
    bool Shader(ShaderGroupRef g, const std::string& usage, const std::string& shadername,
                const std::string& layername) {
        return ok(oslg_shader(sys_, g, usage.c_str(), shadername.c_str(), layername.c_str()));
    }
    bool ConnectShaders(ShaderGroupRef g, const std::string& srclayer, const std::string& srcparam,
                        const std::string& dstlayer, const std::string& dstparam) {
        return ok(oslg_connect_shaders(sys_, g, srclayer.c_str(), srcparam.c_str(), dstlayer.c_str(),
                                       dstparam.c_str()));
    }
    bool ShaderGroupEnd(ShaderGroupRef g) { return ok(oslg_shader_group_end(sys_, g)); }
    /* add_symlocs with SymLocationDesc records (oslexec.h:1075-1076) */
    bool add_symlocs(ShaderGroupRef g, const std::vector<oslg_symloc>& locs) {
        return ok(oslg_add_symlocs(sys_, g, locs.data(), (int)locs.size()));
    }
    bool optimize_group(ShaderGroupRef g) { return ok(oslg_optimize_group(sys_, g)); }
    bool renderer_attribute(const std::string& object, const std::string& name, oslg_typedesc type,
                            const void* data) {
        return ok(oslg_renderer_attribute(sys_, object.c_str(), name.c_str(), type, data));
    }
    bool renderer_matrix(const std::string& name, const float* m16) {
        return ok(oslg_renderer_matrix(sys_, name.c_str(), m16));
    }

    /* ShadingContext (oslexec.h:819-824 get_context / release_context): the
     * per-thread scratch of a caller. Here it holds the host staging of the
     * records a shadeindex scatters. */
    class ShadingContext {
        friend class ShadingSystem;
        std::vector<unsigned char> userdata, outputs;
    };
    ShadingContext* get_context() { return new ShadingContext(); }
    void release_context(ShadingContext* ctx) { delete ctx; }

    /* BatchedExecutor<W> (oslexec.h:990-1030) */
    template <int W> class BatchedExecutor {
    public:
        explicit BatchedExecutor(ShadingSystem& ss) : ss_(ss) {}
        /* The reference's signature (oslexec.h:1000-1004): lane i reads its
         * userdata from, and writes its outputs to, record wide_shadeindex[i]
         * of the arenas (batched_llvm_instance.cpp:1219-1229). */
        bool execute(ShadingContext& ctx, ShaderGroupRef group, int batch_size, const Block<int, W>& wide_shadeindex,
                     BatchedShaderGlobals<W>& bsg, void* userdata_base_ptr, void* output_base_ptr, bool run = true) {
            if (batch_size < 0 || batch_size > W) return ss_.fail("batch_size must be in [0, W]");
            int64_t out_stride = 0, ud_stride = 0;
            if (!ss_.ok(oslg_group_record_strides(ss_.sys_, group, &out_stride, &ud_stride))) return false;
            if (!run || batch_size == 0) return true;
            for (int i = 0; i < batch_size; ++i)
                if (wide_shadeindex.data[i] < 0) return ss_.fail("shadeindex must be >= 0");
            // gather the lanes' records, shade them contiguously, scatter back
            ctx.userdata.resize((size_t)batch_size * (size_t)ud_stride);
            ctx.outputs.resize((size_t)batch_size * (size_t)out_stride);
            unsigned char* ud = static_cast<unsigned char*>(userdata_base_ptr);
            unsigned char* out = static_cast<unsigned char*>(output_base_ptr);
            for (int i = 0; i < batch_size; ++i) {
                const size_t rec = (size_t)wide_shadeindex.data[i];
                if (ud_stride > 0)
                    std::memcpy(ctx.userdata.data() + i * ud_stride, ud + rec * ud_stride, (size_t)ud_stride);
                if (out_stride > 0)
                    std::memcpy(ctx.outputs.data() + i * out_stride, out + rec * out_stride, (size_t)out_stride);
            }
            oslg_shaderglobals sg = view(bsg);
            if (!ss_.ok(oslg_execute_batch_host(ss_.sys_, group, batch_size, &sg,
                                                ud_stride > 0 ? ctx.userdata.data() : nullptr, ud_stride,
                                                out_stride > 0 ? ctx.outputs.data() : nullptr, out_stride,
                                                OSLG_HOST_PRESERVE_OUTPUTS)))
                return false;
            for (int i = 0; i < batch_size && out_stride > 0; ++i)
                std::memcpy(out + (size_t)wide_shadeindex.data[i] * out_stride, ctx.outputs.data() + i * out_stride,
                            (size_t)out_stride);
            return true;
        }
        /* N device points whose records are d_shadeindex[i] (device int32). */
        bool execute(ShaderGroupRef group, int64_t npoints, const oslg_shaderglobals& device_globals,
                     const int32_t* d_shadeindex, void* d_userdata, void* d_outputs, void* stream) {
            return ss_.ok(oslg_execute_batch_indexed(ss_.sys_, group, npoints, &device_globals, d_shadeindex,
                                                     d_userdata, d_outputs, stream));
        }
        /* Shade lanes [0, batch_size) of a W-lane batch: inputs from the
         * batch's varying blocks, outputs and userdata in the arenas the
         * group's symlocs address. Output bytes the group does not write
         * keep their values. run = false only prepares the group. */
        bool execute(ShaderGroupRef group, int batch_size, BatchedShaderGlobals<W>& bsg, void* userdata_base_ptr,
                     void* output_base_ptr, bool run = true) {
            if (batch_size < 0 || batch_size > W) return ss_.fail("batch_size must be in [0, W]");
            int64_t out_stride = 0, ud_stride = 0;
            if (!ss_.ok(oslg_group_record_strides(ss_.sys_, group, &out_stride, &ud_stride))) return false;
            if (!run || batch_size == 0) return true;
            oslg_shaderglobals sg = view(bsg);
            return ss_.ok(oslg_execute_batch_host(ss_.sys_, group, batch_size, &sg, userdata_base_ptr, ud_stride,
                                                  output_base_ptr, out_stride, OSLG_HOST_PRESERVE_OUTPUTS));
        }
        /* N points already in device memory (SoA planes), one launch. */
        bool execute(ShaderGroupRef group, int64_t npoints, const oslg_shaderglobals& device_globals,
                     void* d_userdata, void* d_outputs, void* stream = nullptr) {
            return ss_.ok(oslg_execute_batch_sync(ss_.sys_, group, npoints, &device_globals, d_userdata, d_outputs,
                                                  stream));
        }

    private:
        static void put(oslg_field& f, const Block<Vec3, W>& b) {
            f.data = b.x;
            f.plane_stride = W;
        }
        static void put(oslg_field& f, const Block<float, W>& b) {
            f.data = b.data;
            f.plane_stride = W;
        }
        static void put(oslg_field& f, const Block<int, W>& b) {  // int32 lanes
            f.data = reinterpret_cast<const float*>(b.data);
            f.plane_stride = W;
        }
        static oslg_shaderglobals view(const BatchedShaderGlobals<W>& bsg) {
            const VaryingShaderGlobals<W>& v = bsg.varying;
            oslg_shaderglobals g = {};
            g.raytype = bsg.uniform.raytype;
            put(g.P, v.P); put(g.dPdx, v.dPdx); put(g.dPdy, v.dPdy); put(g.dPdz, v.dPdz);
            put(g.I, v.I); put(g.dIdx, v.dIdx); put(g.dIdy, v.dIdy);
            put(g.N, v.N); put(g.Ng, v.Ng);
            put(g.u, v.u); put(g.dudx, v.dudx); put(g.dudy, v.dudy);
            put(g.v, v.v); put(g.dvdx, v.dvdx); put(g.dvdy, v.dvdy);
            put(g.dPdu, v.dPdu); put(g.dPdv, v.dPdv);
            put(g.time, v.time); put(g.dtime, v.dtime); put(g.dPdtime, v.dPdtime);
            put(g.Ps, v.Ps); put(g.dPsdx, v.dPsdx); put(g.dPsdy, v.dPsdy);
            put(g.surfacearea, v.surfacearea);
            put(g.flipHandedness, v.flipHandedness);
            put(g.backfacing, v.backfacing);
            return g;
        }
        ShadingSystem& ss_;
    };
    template <int W> BatchedExecutor<W> batched() {
        static_assert(W == 4 || W == 8 || W == 16, "batch widths are 4, 8 or 16");
        return BatchedExecutor<W>(*this);
    }

private:
    bool ok(int rc) {
        if (rc == OSLG_OK) return true;
        const char* m = sys_ ? oslg_last_error(sys_) : nullptr;
        error_ = m ? m : "error " + std::to_string(rc);
        return false;
    }
    bool fail(const std::string& m) {
        error_ = m;
        return false;
    }
    oslg_system* sys_ = nullptr;
    std::string error_;
};

}  // namespace oslg
