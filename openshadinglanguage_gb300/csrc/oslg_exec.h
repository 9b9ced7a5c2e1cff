// Host-callable launch interface of the device interpreter (oslg_kernels.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <vector_types.h>

#include "../../include/oslg.h"
#include "oslg_program.h"

namespace oslg {

namespace dev {
// Kernel arguments of the interpreter (oslg_interp.cuh).
struct KArgs {
    const uint8_t* blob;
    int64_t npoints;
    char* userdata;
    char* outputs;
    float* gheap;
    uint32_t* status;
    oslg_shaderglobals G;
    const TexDesc* textures = nullptr;  // the system's registered textures
    int32_t ntextures = 0;
    // record of point i in the userdata and output arenas: shadeindex[i]
    // (BatchedExecutor::execute's wide_shadeindex); null: i
    const int32_t* shadeindex = nullptr;
    // retained symbols (find_symbol): word c of a retained symbol's plane
    // block at symheap[(plane + c) * symheap_stride + point]; null: none
    float* symheap = nullptr;
    int64_t symheap_stride = 0;
};


// One group's request inside a persistent batch launch.
struct BatchJob {
    const uint8_t* blob;  // lowered program (device)
    int64_t npoints;
    char* userdata;
    char* outputs;
    oslg_shaderglobals G;
    int32_t spec_case;    // program index inside a specialized batch kernel
    int32_t pad_;
    uint32_t* status;     // this job's status word (null: the launch's BatchArgs::status)
};
// Arguments of the persistent batch kernel: items are (job, tile) pairs,
// taken in order through *counter (reset to 0 before every launch).
struct BatchArgs {
    const BatchJob* jobs;
    const uint2* items;
    uint32_t nitems;
    uint32_t* counter;
    float* gheap;          // HBM heap: heap_slots x block floats per CTA
    uint32_t* status;
    uint32_t prog_bytes;   // shared-memory bytes reserved for the largest program
    uint32_t heap_slots;   // largest heap of any job (floats per point)
    // When set, the item count is read from device memory at kernel start
    // (work lists planned on the device, e.g. by the wavefront driver).
    const uint32_t* nitems_dev = nullptr;
    const TexDesc* textures = nullptr;
    int32_t ntextures = 0;
};
}  // namespace dev

// Per-launch options beyond the program and its arenas.
struct LaunchExtras {
    const int32_t* shadeindex = nullptr;
    float* symheap = nullptr;
    int64_t symheap_stride = 0;
};

// One interpreter instantiation per feature tier (oslg_tier.cu compiled with
// -DOSLG_TIER=N): TIER bits 1 noise/hash, 2 closures/BSDF/spline, 4 math.
static const int kNumTiers = 8;
struct TierFns {
    int (*launch)(bool smem_heap, unsigned grid, unsigned block, size_t shmem, void* stream, const dev::KArgs& k);
    int (*occupancy)(bool smem_heap, int block, size_t shmem, int* per_sm);
    int (*set_smem_limit)(int bytes);
};
const TierFns& tier_fns(int tier);

// Persistent batch kernels (oslg_batch.cu): every op family, heap in shared
// memory or HBM, launch bounds of 256 or 512 threads.
struct BatchFns {
    int (*launch)(bool smem_heap, int maxt, unsigned grid, unsigned block, size_t shmem, void* stream,
                  const dev::BatchArgs& b);
    int (*occupancy)(bool smem_heap, int maxt, int block, size_t shmem, int* per_sm);
    int (*set_smem_limit)(int bytes);
};
const BatchFns& batch_fns();

struct LaunchConfig {
    int block = 0;             // threads per CTA (0: chosen from the heap size)
    int points_per_thread = 1; // points each thread interleaves
    int heap_smem = -1;        // 1 shared-memory heap, 0 HBM scratch heap, -1 auto
    int grid = 0;              // 0: as many CTAs as the point count needs
};

// Per-device executor state: scratch heap, status word.
struct DeviceState {
    int device = -1;
    int sm_count = 0;
    size_t smem_optin = 0;
    float* gheap = nullptr;
    size_t gheap_bytes = 0;
    uint32_t* d_status = nullptr;
    TexDesc* d_textures = nullptr;  // descriptor table of the registered textures
    int32_t ntextures = 0;
};

// Upload a program blob to the device (returns device pointer).
int device_upload_program(const void* blob, size_t bytes, void** d_blob, std::string* err);
void device_free(void* p);

// Enqueue one plain per-group launch over [0, npoints).
int device_execute(DeviceState& ds, const ProgramHeader& hdr, const void* d_blob, int64_t npoints,
                   const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream,
                   const LaunchConfig& cfg, std::string* err, const LaunchExtras* ex = nullptr);

// Read-and-clear the device status word (synchronises the stream).
int device_read_status(DeviceState& ds, void* stream, uint32_t* bits, std::string* err);

int device_init(DeviceState& ds, std::string* err);

// Allocation-free launch: the program, heap and status word live in a
// fixed-size static device array (see oslg_kernels.cu). Copies the host
// program blob into it, launches, and optionally waits and reports status.
static const size_t kNoAllocScratchBytes = 32u << 20;  // whole static array
static const size_t kNoAllocProgramBytes = 64u << 10;  // program area
// Texture lookups read `textures` (a descriptor table already in device
// memory, or null when the program looks up none).
int device_execute_noalloc(const void* blob, size_t blob_bytes, const ProgramHeader& hdr, int64_t npoints,
                           const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream,
                           const LaunchConfig& cfg, const TexDesc* textures, int32_t ntextures,
                           uint32_t* status_out, std::string* err);
// Read and clear the allocation-free entry's status word on the current
// device (0 when that entry never ran there); synchronises the stream.
int noalloc_read_status(void* stream, uint32_t* bits, std::string* err);

}  // namespace oslg
