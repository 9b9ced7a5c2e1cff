// Host side of the sm_103a interpreter: device set-up, launch-shape choice,
// the per-group launch (oslg_execute_batch) and the allocation-free launch.
// The kernels themselves live in the tier translation units (oslg_tier.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "oslg_exec.h"

namespace oslg {

const TierFns& tier_fns_0();
const TierFns& tier_fns_1();
const TierFns& tier_fns_2();
const TierFns& tier_fns_3();
const TierFns& tier_fns_4();
const TierFns& tier_fns_5();
const TierFns& tier_fns_6();
const TierFns& tier_fns_7();

const TierFns& tier_fns(int tier) {
    switch (tier & 7) {
    case 0: return tier_fns_0();
    case 1: return tier_fns_1();
    case 2: return tier_fns_2();
    case 3: return tier_fns_3();
    case 4: return tier_fns_4();
    case 5: return tier_fns_5();
    case 6: return tier_fns_6();
    default: return tier_fns_7();
    }
}

namespace {
bool cuda_ok(cudaError_t e, std::string* err, const char* what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

}  // namespace

int device_init(DeviceState& ds, std::string* err) {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), err, "cudaGetDevice")) return OSLG_ERR_CUDA;
    if (ds.device == dev && ds.d_status) return OSLG_OK;
    ds.device = dev;
    if (!cuda_ok(cudaDeviceGetAttribute(&ds.sm_count, cudaDevAttrMultiProcessorCount, dev), err, "sm count"))
        return OSLG_ERR_CUDA;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    ds.smem_optin = (size_t)optin;
    if (!cuda_ok(cudaMalloc(&ds.d_status, sizeof(uint32_t)), err, "cudaMalloc status")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaMemset(ds.d_status, 0, sizeof(uint32_t)), err, "cudaMemset status")) return OSLG_ERR_CUDA;
    // the kernels may use up to the opt-in shared memory size
    for (int t = 0; t < kNumTiers; ++t) tier_fns(t).set_smem_limit(optin);
    return OSLG_OK;
}

int device_upload_program(const void* blob, size_t bytes, void** d_blob, std::string* err) {
    void* p = nullptr;
    if (!cuda_ok(cudaMalloc(&p, bytes), err, "cudaMalloc program")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaMemcpy(p, blob, bytes, cudaMemcpyHostToDevice), err, "upload program")) {
        cudaFree(p);
        return OSLG_ERR_CUDA;
    }
    *d_blob = p;
    return OSLG_OK;
}

void device_free(void* p) {
    if (p) cudaFree(p);
}

int device_execute(DeviceState& ds, const ProgramHeader& hdr, const void* d_blob, int64_t npoints,
                   const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream,
                   const LaunchConfig& cfg, std::string* err, const LaunchExtras* ex) {
    if (npoints <= 0) return OSLG_OK;
    int rc = device_init(ds, err);
    if (rc != OSLG_OK) return rc;
    size_t static_bytes = (size_t)hdr.nops * sizeof(Op) + (size_t)((hdr.nconst + 3) & ~3u) * 4;
    // Launch shape: an explicit block/heap placement is honoured; otherwise
    // 256 threads, with the symbol heap in shared memory when that keeps as
    // many CTAs resident per SM as the HBM-heap kernel gets (its registers
    // allow two), else in HBM (measured faster than shrinking the block to
    // fit shared memory).
    const TierFns& fns = tier_fns((int)((hdr.flags >> 8) & 7u));
    int block = cfg.block > 0 ? cfg.block : 256;
    if (block > 256) block = 256;
    block = (block + 31) & ~31;
    bool smem = cfg.heap_smem == 1;
    if (cfg.heap_smem < 0) {
        size_t hb = (size_t)hdr.heap_slots * block * sizeof(float);
        if (static_bytes + hb <= ds.smem_optin) {
            int occ_s = 0, occ_h = 0;
            if (!cuda_ok((cudaError_t)fns.occupancy(true, block, static_bytes + hb, &occ_s), err, "occupancy") ||
                !cuda_ok((cudaError_t)fns.occupancy(false, block, static_bytes, &occ_h), err, "occupancy"))
                return OSLG_ERR_CUDA;
            smem = occ_s >= 1 && occ_s >= std::min(occ_h, 2);
        }
    }
    size_t heap_bytes = (size_t)hdr.heap_slots * block * sizeof(float);
    if (smem && static_bytes + heap_bytes > ds.smem_optin) smem = false;
    size_t shmem = static_bytes + (smem ? heap_bytes : 0);
    if (shmem > ds.smem_optin) {
        if (err) *err = "program does not fit in shared memory";
        return OSLG_ERR_LOWER;
    }
    int per_sm = 0;
    if (!cuda_ok((cudaError_t)fns.occupancy(smem, block, shmem, &per_sm), err, "occupancy")) return OSLG_ERR_CUDA;
    if (per_sm < 1) per_sm = 1;
    // With the heap in shared memory: one CTA per tile, so the hardware
    // scheduler balances tiles of uneven cost (data-dependent loops). With
    // the HBM heap each resident CTA owns one heap slice, so the grid is
    // the resident CTA count and CTAs stride over the tiles. An explicit
    // grid always strides.
    int64_t tiles = (npoints + block - 1) / block;
    int64_t grid = smem ? std::min<int64_t>(tiles, 0x7FFFFFFF) : (int64_t)ds.sm_count * per_sm;
    if (cfg.grid > 0) grid = cfg.grid;
    if (grid > tiles) grid = tiles;
    dev::KArgs k;
    k.blob = static_cast<const uint8_t*>(d_blob);
    k.npoints = npoints;
    k.userdata = static_cast<char*>(userdata);
    k.outputs = static_cast<char*>(outputs);
    if (ex) {
        k.shadeindex = ex->shadeindex;
        k.symheap = ex->symheap;
        k.symheap_stride = ex->symheap_stride;
    }
    k.status = ds.d_status;
    k.G = G;
    k.textures = ds.d_textures;
    k.ntextures = ds.ntextures;
    k.gheap = nullptr;
    if (!smem) {
        size_t need = (size_t)grid * heap_bytes;
        if (need > ds.gheap_bytes) {
            if (ds.gheap) cudaFree(ds.gheap);
            ds.gheap = nullptr;
            ds.gheap_bytes = 0;
            if (!cuda_ok(cudaMalloc(&ds.gheap, need), err, "cudaMalloc heap")) return OSLG_ERR_CUDA;
            ds.gheap_bytes = need;
        }
        k.gheap = ds.gheap;
    }
    if (!cuda_ok((cudaError_t)fns.launch(smem, (unsigned)grid, (unsigned)block, shmem, stream, k), err, "launch"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

int device_read_status(DeviceState& ds, void* stream, uint32_t* bits, std::string* err) {
    *bits = 0;
    if (!ds.d_status) return OSLG_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t v = 0;
    if (!cuda_ok(cudaMemcpyAsync(&v, ds.d_status, 4, cudaMemcpyDeviceToHost, s), err, "status copy")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaMemsetAsync(ds.d_status, 0, 4, s), err, "status clear")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return OSLG_ERR_CUDA;
    *bits = v;
    return OSLG_OK;
}

// ---- allocation-free entry ------------------------------------------------------------
// For callers that cannot allocate device memory: a renderer that hands out
// all HBM from its own pool under a fixed budget, or code that must not pay
// the implicit device synchronisation of cudaMalloc/cudaFree between
// launches. The HBM-heap interpreter runs with every piece of scratch it
// needs inside one file-scope array of kNoAllocScratchBytes (32 MiB), held
// by every GPU that loads this library until the process exits:
//   [0, 256)                      status word
//   [256, 256 + 64 KiB)           copy of the lowered program
//   [256 + 64 KiB, 32 MiB)        symbol heap, one slice per resident CTA
// Every call shares the array and leaves its contents behind; the status
// word is cleared at the start of each call, and the program is copied in
// only when it differs from the one the last call on that stream left
// there. Calls that overlap on the GPU (different streams, or the same
// group from two host threads) race on it.
namespace dev {
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
}

namespace {
struct NoAllocDevice {
    bool ready = false;
    unsigned char* base = nullptr;
    int sm_count = 0;
    int smem_optin = 0;
    std::vector<unsigned char> resident;  // host copy of the program in the array
    void* resident_stream = nullptr;      // the stream that copied it
};
std::mutex g_noalloc_mutex;
NoAllocDevice g_noalloc_dev[128];

// One-time set-up per device, with that device current: resolve the
// array's device address (the host-side symbol is only a stand-in) and
// allow the kernels their shared memory. Runs on the first call on a device.
int noalloc_setup(int dev, NoAllocDevice& d, std::string* err) {
    if (d.ready) return OSLG_OK;
    void* p = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&p, dev::g_noalloc_scratch), err, "cudaGetSymbolAddress(scratch)"))
        return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev), err, "sm count"))
        return OSLG_ERR_CUDA;
    cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    for (int t = 0; t < kNumTiers; ++t)
        if (!cuda_ok((cudaError_t)tier_fns(t).set_smem_limit(d.smem_optin), err, "kernel attribute"))
            return OSLG_ERR_CUDA;
    d.base = static_cast<unsigned char*>(p);
    d.ready = true;
    return OSLG_OK;
}
}  // namespace

int device_execute_noalloc(const void* blob, size_t blob_bytes, const ProgramHeader& hdr, int64_t npoints,
                           const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream,
                           const LaunchConfig& cfg, const TexDesc* textures, int32_t ntextures,
                           uint32_t* status_out, std::string* err) {
    if (status_out) *status_out = 0;
    if (blob_bytes > kNoAllocProgramBytes) {
        if (err) *err = "program is " + std::to_string(blob_bytes) + " bytes; the allocation-free entry holds at most "
                      + std::to_string(kNoAllocProgramBytes);
        return OSLG_ERR_ARG;
    }
    int block = cfg.block > 0 ? cfg.block : 256;
    if (block > 256) block = 256;
    block = (block + 31) & ~31;
    const size_t heap_area = kNoAllocScratchBytes - 256 - kNoAllocProgramBytes;
    const size_t heap_per_cta = (size_t)hdr.heap_slots * block * sizeof(float);
    if (heap_per_cta > heap_area) {
        if (err) *err = "symbol heap of one CTA (" + std::to_string(heap_per_cta) + " bytes) exceeds the "
                      + std::to_string(heap_area) + "-byte heap area of the allocation-free entry";
        return OSLG_ERR_ARG;
    }
    int devid = 0;
    if (!cuda_ok(cudaGetDevice(&devid), err, "cudaGetDevice")) return OSLG_ERR_CUDA;
    if (devid < 0 || devid >= 128) {
        if (err) *err = "device ordinal out of range";
        return OSLG_ERR_ARG;
    }
    NoAllocDevice* d;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        int rc = noalloc_setup(devid, g_noalloc_dev[devid], err);
        if (rc != OSLG_OK) return rc;
        d = &g_noalloc_dev[devid];
    }
    size_t static_bytes = (size_t)hdr.nops * sizeof(Op) + (size_t)((hdr.nconst + 3) & ~3u) * 4;
    if (static_bytes > (size_t)d->smem_optin) {
        if (err) *err = "program does not fit in shared memory";
        return OSLG_ERR_LOWER;
    }
    const TierFns& fns = tier_fns((int)((hdr.flags >> 8) & 7u));
    int per_sm = 0;
    if (!cuda_ok((cudaError_t)fns.occupancy(false, block, static_bytes, &per_sm), err, "occupancy"))
        return OSLG_ERR_CUDA;
    if (per_sm < 1) per_sm = 1;
    int64_t tiles = (npoints + block - 1) / block;
    int64_t grid = (int64_t)d->sm_count * per_sm;
    int64_t fit = (int64_t)(heap_area / heap_per_cta);
    if (grid > fit) grid = fit;
    if (grid > tiles) grid = tiles;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* status = reinterpret_cast<uint32_t*>(d->base);
    unsigned char* prog = d->base + 256;
    float* heap = reinterpret_cast<float*>(d->base + 256 + kNoAllocProgramBytes);
    if (!cuda_ok(cudaMemsetAsync(status, 0, sizeof(uint32_t), s), err, "clear status")) return OSLG_ERR_CUDA;
    if (npoints > 0) {
        {
            std::lock_guard<std::mutex> lock(g_noalloc_mutex);
            const unsigned char* b = static_cast<const unsigned char*>(blob);
            if (d->resident_stream != stream || d->resident.size() != blob_bytes ||
                std::memcmp(d->resident.data(), b, blob_bytes) != 0) {
                if (!cuda_ok(cudaMemcpyAsync(prog, blob, blob_bytes, cudaMemcpyHostToDevice, s), err, "program copy"))
                    return OSLG_ERR_CUDA;
                d->resident.assign(b, b + blob_bytes);
                d->resident_stream = stream;
            }
        }
        dev::KArgs k;
        k.blob = prog;
        k.npoints = npoints;
        k.userdata = static_cast<char*>(userdata);
        k.outputs = static_cast<char*>(outputs);
        k.gheap = heap;
        k.status = status;
        k.G = G;
        k.textures = textures;
        k.ntextures = ntextures;
        if (!cuda_ok((cudaError_t)fns.launch(false, (unsigned)grid, (unsigned)block, static_bytes, stream, k), err,
                     "launch"))
            return OSLG_ERR_CUDA;
    }
    if (status_out) {
        uint32_t v = 0;
        if (!cuda_ok(cudaMemcpyAsync(&v, status, sizeof(v), cudaMemcpyDeviceToHost, s), err, "status copy"))
            return OSLG_ERR_CUDA;
        if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return OSLG_ERR_CUDA;
        *status_out = v;
    }
    return OSLG_OK;
}

int noalloc_read_status(void* stream, uint32_t* bits, std::string* err) {
    *bits = 0;
    int devid = 0;
    if (!cuda_ok(cudaGetDevice(&devid), err, "cudaGetDevice")) return OSLG_ERR_CUDA;
    if (devid < 0 || devid >= 128) return OSLG_OK;
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (g_noalloc_dev[devid].ready) base = g_noalloc_dev[devid].base;
    }
    if (!base) return OSLG_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t v = 0;
    if (!cuda_ok(cudaMemcpyAsync(&v, base, 4, cudaMemcpyDeviceToHost, s), err, "status copy")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaMemsetAsync(base, 0, 4, s), err, "status clear")) return OSLG_ERR_CUDA;
    if (!cuda_ok(cudaStreamSynchronize(s), err, "sync")) return OSLG_ERR_CUDA;
    *bits = v;
    return OSLG_OK;
}

}  // namespace oslg
