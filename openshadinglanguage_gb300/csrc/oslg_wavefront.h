// Wavefront path tracing over the batch executor (oslg_wavefront.cu).
//
// testrender traces one path per pixel sample at a time and shades every
// hit with one execute() call (src/testrender/simpleraytracer.cpp:960-1184).
// Here every path of a frame advances one bounce per wavefront:
//   trace    BVH traversal of the analytic spheres and quads, misses gather
//            the background, hits counted per material
//   plan     one CTA: per-material slot ranges (tile aligned), the batch
//            job table and the (job, tile) work list, all on the device
//   scatter  hit globals (P, I, N, Ng, u, v, dPdu, dPdv) and the sampling
//            record written material-sorted
//   shade    the persistent batch kernel over every material at once; each
//            material group ends in a BSDF sample (oslg_group_bsdf_sample)
//   update   emission, path weight, Russian roulette, next ray, compaction
// Counts never leave the device, so a frame is one fixed sequence of
// launches, captured once as a CUDA graph and replayed.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "oslg_batch.h"
#include "oslg_exec.h"
#include "oslg_host.h"
#include "oslg_spec.h"

namespace oslg {

static const int kWfMaxMaterials = 64;
static const int kWfMaxHits = 16;
static const int kWfInFloats = 9;    // rx ry rz, path weight rgb, absorb, ray roughness, backfacing
static const int kWfOutFloats = 11;  // wi xyz, weight rgb, pdf, Le rgb, roughness

namespace dev {
// Primitive after set-up: six float4 (96 B).
//   r0 p.xyz, radius      r1 ex.xyz, 0           r2 ey.xyz, kind (int bits)
//   r3 n.xyz, material    r4 ux.xyz, id          r5 uy.xyz, 0
// n = normalize(cross(ex, ey)), ux = ex / |ex|^2, uy = ey / |ey|^2.
struct WfPrim {
    float4 r[6];
};
// BVH node (64 B): the boxes of both children, so that one visit tests
// both. A child reference >= 0 is an inner node; < 0 is a leaf ~(first << 4
// | count): records [first, first + count), count <= 15.
struct WfNode {
    float4 a;  // left lo.xyz, left hi.x
    float4 b;  // left hi.yz, right lo.xy
    float4 c;  // right lo.z, right hi.xyz
    int4 d;    // left ref, right ref, 0, 0
};
static const int kWfStack = 32;  // traversal stack; the build keeps the depth below it
}  // namespace dev

struct WavefrontStats {
    int64_t paths = 0;
    int64_t hits[kWfMaxHits] = {};
    int64_t total_hits = 0;
    int bounces = 0;
    float ms_total = 0;
    float ms_stage[5] = {};  // trace, plan, scatter, shade, update (profiled frames only)
};

class Wavefront {
public:
    ~Wavefront();
    // prims/materials validated by the caller (oslg_capi.cpp)
    // jit_dirs: {interpreter headers, cubin cache} to shade with a batch
    // kernel specialized to the materials, or null for the interpreter
    int init(DeviceState& ds, const oslg_wavefront_options& o, const oslg_primitive* prims, int nprims,
             const std::vector<const CompiledGroup*>& materials, const std::string* jit_dirs, std::string* err);
    bool specialized() const { return spec_.kernel != nullptr; }
    int render(float* d_path_radiance, float* d_image, void* stream, bool profile, std::string* err);
    int stats(WavefrontStats* s, std::string* err);
    int64_t paths() const { return npaths_; }

private:
    int enqueue_frame(void* stream, bool profile, std::string* err);
    void release();

    DeviceState* ds_ = nullptr;
    oslg_wavefront_options opt_{};
    int64_t npaths_ = 0, cap_ = 0;
    int nprims_ = 0, nmat_ = 0, tile_ = 0, block_ = 256, ppt_ = 1, maxt_ = 256;
    bool smem_heap_ = false;
    size_t shmem_ = 0;
    int grid_shade_ = 0, grid_stream_ = 0, grid_trace_ = 0;
    float cam_[12] = {};  // eye, dir, right*tan*aspect, up*tan
    dev::BatchArgs bargs_{};
    SpecBatchKernel spec_;         // specialized shading kernel (when built)
    dev::BatchArgs sbargs_{};
    int grid_spec_ = 0, spec_pool_smem_ = 0;
    size_t spec_shmem_ = 0;
    float* d_spec_heap_ = nullptr;

    // device memory
    dev::WfPrim* d_prims_ = nullptr;
    dev::WfNode* d_nodes_ = nullptr;
    int nnodes_ = 0;
    float* d_state_ = nullptr;       // 14 planes of npaths: o, d, tp, L, skip, ray roughness
    uint32_t* d_active_ = nullptr;   // 2 x npaths path lists
    int32_t* d_hit_rec_ = nullptr;   // per active index: record or -1
    float* d_hit_t_ = nullptr;
    uint32_t* d_hit_slot_ = nullptr;
    float* d_globals_ = nullptr;     // 20 planes of cap: P I N Ng u v dPdu dPdv
    float* d_ud_ = nullptr;          // cap x 9
    float* d_out_ = nullptr;         // cap x 11
    uint32_t* d_ctl_ = nullptr;      // counters (see oslg_wavefront.cu)
    dev::BatchJob* d_jobs_ = nullptr;      // nmat live jobs
    dev::BatchJob* d_templ_ = nullptr;     // nmat templates (offset 0)
    uint2* d_items_ = nullptr;
    int32_t* d_order_ = nullptr;     // materials, heaviest first
    float* d_heap_ = nullptr;
    float* d_radiance_out_ = nullptr;  // last user pointers the graph was captured with
    float* d_image_out_ = nullptr;

    void* graph_ = nullptr;
    void* gexec_ = nullptr;
    void* ev_[12] = {};
    WavefrontStats last_{};
};

}  // namespace oslg
