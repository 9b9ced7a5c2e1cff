/*
 * osl-gb300: C ABI of the GB300 batched shading executor.
 *
 * This is the drop-in boundary for OSL's data-parallel hot path: running an
 * optimized ShaderGroup over many shading points. Each entry point replaces
 * one member of the reference's C++ API (paths relative to the
 * OpenShadingLanguage source tree); the C++ facade (oslg.hpp) and the
 * Python ctypes binding bind to exactly these symbols.
 *
 * Conventions: plain pointers and sizes only; every call returns an int
 * status (OSLG_OK == 0) and the message of the last failure is available
 * from oslg_last_error(). No C++ exception crosses this boundary.
 * Device pointers are CUDA device addresses on the current device;
 * `stream` is a cudaStream_t (NULL = legacy default stream).
 */
#ifndef OSLG_H
#define OSLG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OSLG_OK 0
#define OSLG_ERR_ARG 1        /* bad argument or unknown name */
#define OSLG_ERR_PARSE 2      /* .oso text could not be read */
#define OSLG_ERR_LOWER 3      /* group uses something the executor lacks */
#define OSLG_ERR_CUDA 4       /* a CUDA call failed */
#define OSLG_ERR_STATE 5      /* call out of order (e.g. execute before end) */
#define OSLG_ERR_DEVICE 6     /* the kernel reported a status bit */

typedef struct oslg_system oslg_system;
typedef struct oslg_group oslg_group;
typedef struct oslg_symbol oslg_symbol;

/* OIIO TypeDesc numbering (basetype / aggregate / vecsemantics), so a
 * caller holding an OIIO::TypeDesc can pass its fields straight through. */
#define OSLG_BASE_INT32 7
#define OSLG_BASE_FLOAT 11
#define OSLG_BASE_STRING 13
#define OSLG_AGG_SCALAR 1
#define OSLG_AGG_VEC3 3
#define OSLG_AGG_MATRIX44 16
#define OSLG_VEC_NOXFORM 0
#define OSLG_VEC_COLOR 1
#define OSLG_VEC_POINT 2
#define OSLG_VEC_VECTOR 3
#define OSLG_VEC_NORMAL 4

typedef struct oslg_typedesc {
    int32_t basetype;
    int32_t aggregate;
    int32_t vecsemantics;
    int32_t arraylen;
} oslg_typedesc;

/* SymArena (src/include/OSL/oslexec.h:57-63) */
#define OSLG_ARENA_HEAP 1
#define OSLG_ARENA_OUTPUTS 2
#define OSLG_ARENA_USERDATA 3

/* SymLocationDesc (src/include/OSL/oslexec.h:69-105): point i of symbol
 * `name` lives at base + offset + i * stride; with derivs the value is
 * followed by its x and y derivatives. */
typedef struct oslg_symloc {
    const char* name;
    oslg_typedesc type;
    int32_t derivs;
    int32_t arena;
    int64_t offset;
    int64_t stride;
} oslg_symloc;

/* One shader-global field. `data` == NULL means every point uses `value`;
 * otherwise data points to SoA planes on the device: component c of point
 * i is data[c * plane_stride + i]. */
typedef struct oslg_field {
    const float* data;
    int64_t plane_stride;
    float value[3];
    float pad;
} oslg_field;

/* Device-side BatchedShaderGlobals: the varying members of
 * src/include/OSL/batched_shaderglobals.h:77-197 over N points. Fields the
 * group does not read may be left zeroed. */
typedef struct oslg_shaderglobals {
    oslg_field P, dPdx, dPdy, dPdz;
    oslg_field I, dIdx, dIdy;
    oslg_field N, Ng;
    oslg_field u, dudx, dudy;
    oslg_field v, dvdx, dvdy;
    oslg_field dPdu, dPdv;
    oslg_field time, dtime, dPdtime;
    oslg_field Ps, dPsdx, dPsdy;
    oslg_field surfacearea;
    /* Block<int> flipHandedness and backfacing (batched_shaderglobals.h:
     * 136-140): with data, one int32 per point (data[i], nonzero = true);
     * without, value[0] != 0 holds for every point. flipHandedness flips
     * calculatenormal(); backfacing() returns backfacing. */
    oslg_field flipHandedness;
    oslg_field backfacing;
    /* UniformShaderGlobals::raytype (batched_shaderglobals.h:47): the
     * raytype bits of the rays being shaded; raytype(name) tests the bit
     * of name's position in the system's "raytypes" list. */
    int32_t raytype;
    int32_t reserved[3];
} oslg_shaderglobals;

/* ---- ShadingSystem ------------------------------------------------------ */

/* ShadingSystem::ShadingSystem (src/include/OSL/oslexec.h:170) */
int oslg_create_system(oslg_system** out);
/* ShadingSystem::~ShadingSystem */
int oslg_destroy_system(oslg_system* sys);
/* ShadingSystem::attribute(name, TypeDesc, const void*) (oslexec.h:324).
 * Integer options: "max_closure_components", "max_closure_terms",
 * "gpu_block", "gpu_points_per_thread", "gpu_heap_placement" (0 HBM, 1 smem,
 * -1 auto), "debug", "jit" (1: optimize builds a kernel specialized to the
 * group, see oslg_group_specialized_source; the counterpart of the
 * reference's per-group JIT), "jit_block" (64/128/256 threads per CTA of a
 * specialized launch), "jit_pool_smem" (closure pools in shared memory 1,
 * HBM scratch 0, automatic -1), "jit_min_blocks" (register cap of
 * specialized kernels: 256-thread CTAs per SM that must fit, 2..8),
 * "strict_messages", "opt_constant_fold", "opt_elide_useless_ops" (as the
 * reference's ShadingSystem attributes of those names, shadingsys.cpp:1639-1684),
 * "userdata_isconnected" (isconnected() counts lockgeom=0 parameters as
 * connected, shadingsys.cpp:1073), "fast_math" (1, the default: sin, cos,
 * tan, asin, acos, atan, atan2, sinh, cosh, tanh, exp, exp2, expm1, log,
 * log2, log10, pow, erf, erfc, cbrt and sincos use OpenImageIO's fast_*
 * approximations as the reference's default USE_FAST_MATH build; 0: the
 * correctly rounded forms), "max_loop_iterations" (loop back edges one point may take, summed over
 * the group's loops, before the launch ends with the loop-limit status
 * bit; 0 keeps the default 2^24; the reference has no such limit),
 * "host_direct_outputs" (host-buffer execution writes pinned output records
 * from the kernel, 1 by default). */
int oslg_attribute_int(oslg_system* sys, const char* name, int value);
/* ShadingSystem::attribute(name, TypeString, &value) (oslexec.h:324).
 * String options: "colorspace" (the colour system whose primaries rgb
 * means: Rec709 (default), sRGB, NTSC, EBU, PAL, SECAM, SMPTE, HDTV, CIE,
 * AdobeRGB, XYZ, ACES2065-1, ACEScg; src/liboslexec/opcolor.cpp:31-85,
 * shadingsys.cpp:1613). Groups lowered afterwards use it for luminance,
 * blackbody, wavelength_color and transformc. */
int oslg_attribute_string(oslg_system* sys, const char* name, const char* value);
/* ShadingSystem::attribute(name, TypeDesc(TypeString, n), values)
 * (oslexec.h:324). String-array options: "raytypes" (at most 32 names;
 * raytype(name) tests bit 1 << position; default camera, shadow,
 * reflection, refraction, diffuse, glossy, subsurface, displacement as
 * shadingsys.cpp:1256-1265). Groups lowered afterwards use it. */
int oslg_attribute_strings(oslg_system* sys, const char* name, const char* const* values, int n);
/* ShadingSystem::register_closure (oslexec.h:1041). Parameters are taken
 * positionally from the `closure` op's arguments. */
int oslg_register_closure(oslg_system* sys, const char* name, int id);
/* ShadingSystem::LoadMemoryCompiledShader (oslexec.h:608) */
int oslg_load_memory_compiled_shader(oslg_system* sys, const char* shadername,
                                     const char* oso_text);
/* Message of the last failed call on this system (ShadingSystem errors are
 * reported through an ErrorHandler in the reference). */
const char* oslg_last_error(oslg_system* sys);

/* ---- group construction (oslexec.h:634-771) ---------------------------- */

/* ShadingSystem::ShaderGroupBegin (oslexec.h:634) */
int oslg_shader_group_begin(oslg_system* sys, const char* groupname, oslg_group** out);
/* ShadingSystem::Parameter (oslexec.h:656): applies to the next Shader()
 * call, as in the reference. `value` holds arraylen (or 1) elements of the
 * type; strings are passed as an array of const char*. */
int oslg_parameter(oslg_system* sys, oslg_group* group, const char* name,
                   oslg_typedesc type, const void* value, int lockgeom);
/* ShadingSystem::Shader (oslexec.h:723) */
int oslg_shader(oslg_system* sys, oslg_group* group, const char* shaderusage,
                const char* shadername, const char* layername);
/* ShadingSystem::ConnectShaders (oslexec.h:740) */
int oslg_connect_shaders(oslg_system* sys, oslg_group* group, const char* srclayer,
                         const char* srcparam, const char* dstlayer, const char* dstparam);
/* ShadingSystem::ShaderGroupEnd (oslexec.h:650) */
int oslg_shader_group_end(oslg_system* sys, oslg_group* group);
/* ShadingSystem::attribute(group, "renderer_outputs", ...) (oslexec.h:360) */
int oslg_group_renderer_outputs(oslg_system* sys, oslg_group* group, const char** names, int n);
/* ShadingSystem::add_symlocs(group, symlocs) (oslexec.h:1076) */
int oslg_add_symlocs(oslg_system* sys, oslg_group* group, const oslg_symloc* locs, int n);
/* Renderer-side evaluation of a closure output: after the group runs, the
 * closure symbol `closure` ("layer.sym" or "sym") is walked and evaluated
 * as testrender's CompositeBSDF at wo = -I and the light direction wi
 * (src/testrender/shading.cpp:1450-1500 walk, shading.h:322-374 prepare and
 * eval). Writes {weight.r, weight.g, weight.b, pdf} (4 floats) at
 * output_base + offset + i*stride. Lobes: diffuse, oren_nayar, microfacet
 * "ggx" (refract 0/1/2), oren_nayar_diffuse_bsdf, sheen_bsdf and
 * dielectric_bsdf, under layer() as testrender layers them; other closure
 * ids contribute nothing. */
int oslg_group_bsdf_eval(oslg_system* sys, oslg_group* group, const char* closure,
                         const float wi[3], int64_t offset, int64_t stride);
/* Renderer-side sampling of a closure output, the per-hit step of
 * testrender's path loop (src/testrender/simpleraytracer.cpp:1038-1079):
 * the closure tree is walked (emission adds to Le; diffuse, oren_nayar,
 * microfacet "ggx" with refract 0/1/2, oren_nayar_diffuse_bsdf, sheen_bsdf
 * and dielectric_bsdf become lobes),
 * prepared with the path weight and sampled (src/testrender/shading.h:322-398).
 * Reads {rx, ry, rz, path_weight.rgb, absorb, ray_roughness, backfacing}
 * (9 floats; the last two feed BSDL's roughness regularization and
 * backfacing rule) per point at
 * userdata_base + in_offset + i*in_stride; writes {wi.xyz, weight.rgb,
 * pdf, Le.rgb, roughness} (11 floats) at output_base + offset + i*stride.
 * No counterpart as one call in the reference, which does these steps in
 * the renderer. */
int oslg_group_bsdf_sample(oslg_system* sys, oslg_group* group, const char* closure, int64_t offset,
                           int64_t stride, int64_t in_offset, int64_t in_stride);
/* ShadingSystem::optimize_group (oslexec.h:1093) + BatchedExecutor::jit_group
 * (oslexec.h:993): lowers the group to a device op program and uploads it. */
int oslg_optimize_group(oslg_system* sys, oslg_group* group);
/* BatchedExecutor<W>::jit_group / jit_all_groups (oslexec.h:986-992): lower
 * and upload `groups` and, with attribute "jit", build their specialized
 * kernels on `nthreads` threads (0: every hardware thread), so that first
 * launches do not wait for compiles. */
int oslg_jit_groups(oslg_system* sys, oslg_group* const* groups, int ngroups, int nthreads);
/* BatchedExecutor::execute over HOST buffers (the reference's execute reads
 * and writes host memory). Shader-global fields with data != NULL are host
 * SoA planes (plane_stride apart); host_userdata and host_outputs hold one
 * record per point, userdata_stride / output_stride bytes apart (the
 * strides the group's symlocs use; 0 when the group has none). The points
 * run in chunks whose input copies, launches and output copies overlap on
 * three internal streams; returns when the outputs are in host memory.
 * Output bytes the group does not write are zero, or keep their host values
 * with OSLG_HOST_PRESERVE_OUTPUTS (which copies the records in first). Host
 * memory should be pinned for the copies to run asynchronously. */
#define OSLG_HOST_PRESERVE_OUTPUTS 1
int oslg_execute_batch_host(oslg_system* sys, oslg_group* group, int64_t npoints,
                            const oslg_shaderglobals* host_globals, const void* host_userdata,
                            int64_t userdata_stride, void* host_outputs, int64_t output_stride, int flags);
/* The CUDA source of the kernel specialized to this group (each op a call
 * of the interpreter's handler with constant operands, control flow as
 * gotos, constants in constant memory). With attribute "jit" = 1 it is
 * compiled for sm_103a when the group is first uploaded (cubins cached by
 * content hash) and oslg_execute_batch launches it instead of the
 * interpreter. Replaces BatchedBackendLLVM code generation
 * (src/liboslexec/batched_backendllvm.cpp). `size` gets the length + 1. */
int oslg_group_specialized_source(oslg_system* sys, oslg_group* group, char* buf, size_t cap, size_t* size);
/* The CUDA source of a persistent batch kernel specialized to several
 * groups (job i of a batch runs groups[i]'s body); with attribute "jit" the
 * wavefront driver shades its materials with such a kernel. */
int oslg_groups_specialized_batch_source(oslg_system* sys, oslg_group* const* groups, int ngroups, char* buf,
                                         size_t cap, size_t* size);
/* BatchedExecutor::execute_init + execute_layer(layername)
 * (src/include/OSL/oslexec.h:1006-1027): run the group's layers up to and
 * including `layername` over N device points and store the outputs those
 * layers write (outputs of later layers are left untouched). Each call is a
 * complete launch; no per-point state is kept between calls. */
int oslg_execute_layer(oslg_system* sys, oslg_group* group, const char* layername, int64_t npoints,
                       const oslg_shaderglobals* globals, void* userdata_base, void* output_base, void* stream);
/* The serialized program that runs layers [0, layername] (as
 * oslg_group_program for the whole group). */
int oslg_group_layer_program(oslg_system* sys, oslg_group* group, const char* layername, void* buf, size_t cap,
                             size_t* size);
/* The byte strides of the group's output and userdata records (0 when it
 * has none), as its symlocs and BSDF requests place them; the group is
 * optimized first. oslg_execute_batch_host takes these strides. */
int oslg_group_record_strides(oslg_system* sys, oslg_group* group, int64_t* output_stride,
                              int64_t* userdata_stride);
/* 1 when the group runs its specialized kernel. */
int oslg_group_is_specialized(oslg_system* sys, oslg_group* group, int* out);
/* Register (or replace) the image that texture(name, s, t, ...) looks up:
 * width x height texels of nchannels floats, channels interleaved, rows
 * from the top (t = 0). A mip pyramid (2x2 box reductions) is built and kept
 * in device memory; lookups are mipmapped bilinear with the level chosen
 * from the s, t derivatives, wrap modes black/clamp/periodic/mirror. Stands
 * in for OIIO's TextureSystem behind RendererServices::texture
 * (src/include/OSL/rendererservices.h:361-383; the reference reads files).
 * Groups naming the texture must be lowered after it is registered. */
int oslg_texture_create(oslg_system* sys, const char* name, int width, int height, int nchannels,
                        const float* texels, int* index);
/* Answer getattribute([object,] name, [index,] value) in shaders with a
 * uniform value: the renderer side of RendererServices::get_attribute /
 * get_array_attribute (src/include/OSL/rendererservices.h:278-288) and
 * BatchedRendererServices::get_attribute_uniform
 * (src/include/OSL/batched_rendererservices.h:143-156). object NULL or ""
 * is the scene-wide name space that a lookup without an object name reads.
 * data: max(1, arraylen) elements of the type (floats, int32, or
 * const char* for strings). Lookups fold to constants when a group is
 * lowered, as the reference's constant folder does
 * (src/liboslexec/constfold.cpp:2262-2360); a name with no value makes
 * getattribute return 0 and leave its destination unchanged. */
int oslg_renderer_attribute(oslg_system* sys, const char* object, const char* name, oslg_typedesc type,
                            const void* data);
/* The matrix from the named coordinate system to "common" (16 floats, row
 * major, points as row vectors like Imath): the renderer side of
 * RendererServices::get_matrix / get_inverse_matrix by name
 * (src/include/OSL/rendererservices.h:96-145), and of the object and
 * shader transforms when name is "object" or "shader". transform(),
 * matrix(), getmatrix() with constant space names fold these (and inverses)
 * into constant matrices when a group is lowered. */
int oslg_renderer_matrix(oslg_system* sys, const char* name, const float* matrix16);
/* ShaderGroupRef release */
int oslg_release_group(oslg_system* sys, oslg_group* group);

/* The lowered op program (no reference counterpart: it replaces the JIT'd
 * LLVM module). Copies up to `cap` bytes into `buf` and returns the size
 * through `size`. Lets a caller cache or inspect what will run. */
int oslg_group_program(oslg_system* sys, oslg_group* group, void* buf, size_t cap, size_t* size);

/* ---- execution ------------------------------------------------------------ */

/* BatchedExecutor<W>::execute (oslexec.h:1000-1004, shadingsys.cpp:329),
 * over npoints device-resident points instead of one W-lane batch:
 * globals as above, userdata/outputs arenas addressed by the symlocs.
 * Stream-ordered; returns once the launch is enqueued. */
int oslg_execute_batch(oslg_system* sys, oslg_group* group, int64_t npoints,
                       const oslg_shaderglobals* globals, void* userdata_base,
                       void* output_base, void* stream);
/* BatchedExecutor<W>::execute with its wide_shadeindex (oslexec.h:1000-1004):
 * point i reads its globals from element i of the SoA fields, and its
 * userdata and output records at base + shadeindex[i] * stride
 * (batched_llvm_instance.cpp:1219-1229), so a renderer that shades sorted or
 * compacted hits scatters the results back to their pixels. `shadeindex`
 * is a device array of npoints int32; every index must address a record
 * inside both arenas, and two points with the same index write the same
 * record in an unspecified order. */
int oslg_execute_batch_indexed(oslg_system* sys, oslg_group* group, int64_t npoints,
                               const oslg_shaderglobals* globals, const int32_t* shadeindex, void* userdata_base,
                               void* output_base, void* stream);

/* ShadingSystem::find_symbol (oslexec.h:950-959): symbol `symbolname` of
 * layer `layername`, or with layername NULL of the last layer that has one
 * ("layer.symbol" names both). Finding a symbol retains it: the group is
 * lowered again so that every device execution (oslg_execute_batch,
 * _sync, _indexed) keeps the symbol's final values. Closures and shader
 * globals are refused. The handle lives as long as the group. */
int oslg_find_symbol(oslg_system* sys, oslg_group* group, const char* layername, const char* symbolname,
                     const oslg_symbol** out);
/* ShadingSystem::symbol_typedesc (oslexec.h:961-963) */
int oslg_symbol_typedesc(const oslg_symbol* sym, oslg_typedesc* out);
/* ShadingSystem::symbol_address (oslexec.h:965-971) for a batch: the device
 * SoA view of the symbol's values after the group's most recent device
 * execution. Word c of point i (c < components x array length; floats, or
 * int32 for int symbols) is at ((float*)*address)[c * *plane_stride + i],
 * point i being the launch's i-th point. OSLG_ERR_STATE when the group has
 * not run since the symbol was found. */
int oslg_symbol_address(oslg_system* sys, oslg_group* group, const oslg_symbol* sym, const void** address,
                        int64_t* plane_stride);

/* Same as oslg_execute_batch, then waits for the stream and reports any
 * status bit the kernel raised (closure arena overflow, bad opcode, array
 * bounds) as OSLG_ERR_DEVICE (context.cpp:443-451 flushes errors the same
 * way at execute_cleanup). */
int oslg_execute_batch_sync(oslg_system* sys, oslg_group* group, int64_t npoints,
                            const oslg_shaderglobals* globals, void* userdata_base,
                            void* output_base, void* stream);

/* Status bits raised by kernels since the last call (and clears them),
 * including those of allocation-free calls that did not collect theirs. */
int oslg_device_status(oslg_system* sys, uint32_t* bits);

/* Launch shape the next execute uses: threads per block, points per
 * thread, heap placement (0 HBM scratch, 1 shared memory, -1 auto). */
int oslg_set_launch(oslg_system* sys, int block, int points_per_thread, int heap_smem);

/* Allocation-free variant of oslg_execute_batch. It has no counterpart in
 * the reference. It is for callers that cannot allocate device memory: a
 * renderer that hands out all HBM from its own pool under a fixed budget,
 * or code that must not pay the implicit device synchronisation of
 * cudaMalloc/cudaFree. It calls no allocation routine: the lowered program,
 * the symbol heap and the status word live in one static device array of
 * 32 MiB that every GPU loading the library holds until exit. Limits: the
 * lowered program must be at most 64 KiB and one CTA's symbol heap must fit
 * the rest of the array (otherwise OSLG_ERR_ARG with a message). The group
 * must already be lowered (oslg_optimize_group), else OSLG_ERR_STATE.
 * A group that calls texture() or environment() reads the system's texture
 * table, which only the allocating entries upload: it runs here once a
 * group of this system has gone through oslg_execute_batch after the
 * textures were registered, and is refused with OSLG_ERR_STATE before.
 * The first call on a device does a one-time set-up (resolves the array's
 * device address and sets the kernels' shared-memory limit); make that
 * first call before any stream capture. Calls share the array and leave
 * their contents in it: the status word is cleared at the start of each
 * call and the program is copied in only when it differs from the one the
 * last call on the same stream left there. Calls that overlap on the GPU
 * race. With status_out == NULL the call only enqueues work and the status
 * bits stay in the array, where oslg_device_status reads (and clears)
 * them; otherwise it waits for the stream, stores the kernel status bits
 * and returns OSLG_ERR_DEVICE if any is set. */
int oslg_execute_batch_noalloc(oslg_system* sys, oslg_group* group, int64_t npoints,
                               const oslg_shaderglobals* globals, void* userdata_base,
                               void* output_base, void* stream, uint32_t* status_out);

/* ---- persistent batch executor --------------------------------------------
 * No counterpart in the reference: its renderers call execute() once per
 * group and batch (src/liboslexec/shadingsys.cpp:329-394, the loop in
 * src/testshade/testshade.cpp:1864-1881). A batch collects requests of many
 * groups (each with the same arguments as oslg_execute_batch) and runs them
 * all in one persistent kernel launch that takes (group, tile) work items
 * from a device counter, heaviest groups first. The step is captured as a
 * CUDA graph on first execute and replayed while the batch is unchanged.
 * Results are identical to one oslg_execute_batch call per request. The
 * caller keeps every globals/userdata/output buffer alive and in place until
 * the batch is cleared or destroyed; requests must not overlap in output. */
typedef struct oslg_batch oslg_batch;

typedef struct oslg_batch_tuning {
    int block;       /* threads per CTA */
    int points_per_thread; /* 1, 2 or 4: a work item is block * points_per_thread points */
    int heap_smem;   /* 1 symbol heap in shared memory, 0 in HBM */
    int grid;        /* persistent CTAs */
    int ctas_per_sm; /* resident CTAs per SM for this shape */
    float ms;        /* measured milliseconds per launch (autotune only) */
} oslg_batch_tuning;

/* With the system attribute "jit" set when the batch is created, the batch
 * runs one persistent kernel specialized to its distinct programs (each a
 * specialized body, see oslg_group_specialized_source; built once per set
 * of programs and cached), with the same results. */
int oslg_batch_create(oslg_system* sys, oslg_batch** out);
int oslg_batch_destroy(oslg_batch* batch);
/* Drop all requests (device tables are kept for reuse). */
int oslg_batch_clear(oslg_batch* batch);
/* Append one request; lowers and uploads the group on first use. */
int oslg_batch_add(oslg_batch* batch, oslg_group* group, int64_t npoints, const oslg_shaderglobals* globals,
                   void* userdata_base, void* output_base);
/* block 0 keeps the current size; points_per_thread 1/2/4 (0 keeps);
 * heap_smem -1 auto; use_graph 0/1. */
int oslg_batch_set_launch(oslg_batch* batch, int block, int points_per_thread, int heap_smem, int use_graph);
/* Enqueue every request on `stream` (asynchronous). */
int oslg_batch_execute(oslg_batch* batch, void* stream);
/* Time `reps` launches of each points-per-thread {1, 2, 4} x block size
 * {128, 256, 512} x heap placement {shared, HBM} that fits, keep the
 * fastest for later executes. Writes up
 * to `cap` measured candidates to `results` and their count to `n`. */
int oslg_batch_autotune(oslg_batch* batch, void* stream, int reps, oslg_batch_tuning* results, int cap, int* n,
                        oslg_batch_tuning* best);
/* Launch shape of the last built batch. */
int oslg_batch_last_launch(oslg_batch* batch, oslg_batch_tuning* out);

/* ---- shading server ---------------------------------------------------------
 * No counterpart in the reference (renderers call execute() per batch). A
 * server keeps programs resident and runs requests submitted from any host
 * thread with continuous batching: a worker admits waiting requests, in
 * arrival order, into "waves" while device memory (an arena sized from
 * budget_bytes) and stream slots allow, copies their inputs from host
 * memory, runs each wave as one persistent batch launch and copies the
 * outputs back; several waves are in flight at once. Inputs are the host
 * fields of `host_globals` (data != NULL: SoA planes of npoints floats,
 * plane_stride apart); they and `host_output` must stay valid until the
 * request completes (pinned memory makes the copies asynchronous).
 * Outputs are written as oslg_execute_batch would write them into a zeroed
 * buffer of output_bytes. Userdata is not supported in served requests. */
typedef struct oslg_server oslg_server;

typedef struct oslg_server_options {
    size_t budget_bytes;    /* device memory for arena + scratch heaps (default 40 GiB) */
    int streams;            /* waves in flight (default 3) */
    int block;              /* threads per CTA of a wave (default 512) */
    int points_per_thread;  /* 1, 2 or 4 (default 1) */
    int64_t max_wave_points;
    int max_wave_requests;
    size_t arena_bytes;     /* request memory (0: what the budget leaves) */
} oslg_server_options;

typedef struct oslg_request_stats {
    int64_t submit_ns, admit_ns, done_ns;  /* host steady clock */
    int wave;
    int status;
} oslg_request_stats;

typedef struct oslg_server_stats {
    uint64_t submitted, completed, failed, waves;
    int64_t points_done;
    size_t arena_capacity, arena_high_water, program_bytes, scratch_bytes;
    int in_flight_waves, pending;
} oslg_server_stats;

/* opts NULL: defaults. Starts the worker thread. With the system's
 * attribute "jit" set, waves run one persistent kernel specialized to the
 * resident programs (built by the worker when that set changes; the same
 * set gives the same kernel as a jit batch); otherwise the interpreter. */
int oslg_server_create(oslg_system* sys, const oslg_server_options* opts, oslg_server** out);
/* Finishes every submitted request, then stops. */
int oslg_server_destroy(oslg_server* server);
/* Lower, upload and keep a group resident ahead of its first request. */
int oslg_server_register(oslg_server* server, oslg_group* group);
int oslg_server_submit(oslg_server* server, oslg_group* group, int64_t npoints, const oslg_shaderglobals* host_globals,
                       void* host_output, size_t output_bytes, uint64_t* ticket);
/* timeout_ms < 0 waits forever; a finished request's ticket is released. */
int oslg_server_wait(oslg_server* server, uint64_t ticket, int timeout_ms, oslg_request_stats* stats);
int oslg_server_poll(oslg_server* server, uint64_t ticket, int* done, oslg_request_stats* stats);
int oslg_server_get_stats(oslg_server* server, oslg_server_stats* out);

/* ---- wavefront path tracing -------------------------------------------------
 * testrender's per-sample path loop (src/testrender/simpleraytracer.cpp:
 * 960-1184: trace, globals_from_hit, execute, process_closure, add
 * emission, prepare + sample, continue) run for every path of a frame at
 * once, one bounce per wavefront, with the hits of each bounce sorted by
 * material and shaded by the persistent batch kernel. The scene is analytic
 * spheres and rectangles (testrender tessellates its spheres and quads,
 * src/testrender/scene.cpp; here they are intersected exactly). Material k
 * is a group whose closure output is sampled with
 * oslg_group_bsdf_sample(..., offset 0, stride 44, in_offset 0, in_stride
 * 36). Differences from testrender, by design: no light sampling (emission
 * is gathered by BSDF sampling, MIS weight 1), no background importance
 * sampling or media, and Russian roulette with a fixed survival
 * probability after every hit. */
typedef struct oslg_wavefront oslg_wavefront;

#define OSLG_PRIM_SPHERE 0
#define OSLG_PRIM_QUAD 1 /* rectangle p + s*ex + t*ey, s,t in [0,1], ex orthogonal to ey */

typedef struct oslg_primitive {
    int32_t kind;      /* OSLG_PRIM_SPHERE or OSLG_PRIM_QUAD */
    int32_t material;  /* index into the materials array */
    float p[3];        /* sphere centre or rectangle corner */
    float ex[3];       /* rectangle edges */
    float ey[3];
    float radius;      /* sphere radius */
} oslg_primitive;

typedef struct oslg_wavefront_options {
    int32_t width, height, spp;  /* paths = width * height * spp */
    int32_t max_hits;            /* shading points per path at most (<= 16) */
    float rr_survival;           /* Russian roulette survival probability per hit */
    float eye[3], look[3], up[3];
    float fov_deg;               /* vertical field of view */
    float background[3];         /* radiance of rays that leave the scene */
    uint32_t seed;
    int32_t block;               /* shading launch: threads per CTA (0: 256) */
    int32_t points_per_thread;   /* 1, 2 or 4 (0: 1) */
    int32_t heap_smem;           /* 1 shared memory, 2 HBM, 0: shared memory when it fits */
    int32_t use_graph;           /* replay the frame as a CUDA graph (default 1; pass -1 for 0) */
} oslg_wavefront_options;

typedef struct oslg_wavefront_stats {
    int64_t paths;
    int64_t hits[16];      /* shading points per bounce of the last frame */
    int64_t total_hits;
    int32_t bounces;       /* bounces with at least one hit */
    float ms_total;        /* last frame, CUDA events on the render stream */
    float ms_stage[5];     /* trace, plan, scatter, shade, update (profiled frames) */
} oslg_wavefront_stats;

int oslg_wavefront_create(oslg_system* sys, const oslg_wavefront_options* opts, const oslg_primitive* prims,
                          int nprims, oslg_group* const* materials, int nmaterials, oslg_wavefront** out);
int oslg_wavefront_destroy(oslg_wavefront* wf);
/* One frame. d_path_radiance (3 planes of paths floats; path index
 * (y * width + x) * spp + s) and d_image (width * height * 3, the mean of
 * the pixel's samples) are device buffers; either may be NULL. */
int oslg_wavefront_render(oslg_wavefront* wf, float* d_path_radiance, float* d_image, void* stream);
/* One frame launched stage by stage with CUDA events between the stages
 * (no graph); ms_stage of the stats holds the sums over bounces. */
int oslg_wavefront_render_profiled(oslg_wavefront* wf, float* d_path_radiance, float* d_image, void* stream);
/* Synchronises with the last frame. */
int oslg_wavefront_get_stats(oslg_wavefront* wf, oslg_wavefront_stats* out);

#ifdef __cplusplus
}
#endif
#endif /* OSLG_H */
