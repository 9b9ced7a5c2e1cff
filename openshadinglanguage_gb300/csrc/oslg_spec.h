// Per-group kernel specialization (oslg_spec.cpp).
//
// The reference JIT-compiles every optimized group to native code
// (BatchedBackendLLVM, src/liboslexec/batched_backendllvm.cpp; jit_group,
// src/liboslexec/shadingsys.cpp:4111-4181). The executor's counterpart
// writes CUDA source for one lowered program — each op becomes a call of the
// interpreter's own handler with its operand words as constants, control
// flow becomes gotos between op labels, the constant pool becomes constant
// memory — compiles it for sm_103a with nvcc, caches the cubin by content
// hash and loads it with the CUDA library API. Symbol slots then live in a
// thread-local array with constant indices (registers); only the closure
// node pools, indexed at run time, keep a slot-major heap.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "oslg_exec.h"
#include "oslg_host.h"

namespace oslg {

struct SpecKernel {
    void* library = nullptr;  // cudaLibrary_t
    void* kernel = nullptr;   // cudaKernel_t
    std::string key;          // content hash of the source
    uint32_t sym_slots = 0;   // thread-local floats
    uint32_t pool_slots = 0;  // closure-pool floats per point (slot-major heap)
    uint32_t stage_stride = 0;  // output record bytes staged in shared memory (0: none)
    ~SpecKernel();
};

// CUDA source of the specialized kernel for one lowered program.
// min_blocks: resident 256-thread CTAs the register budget must allow
// (2: up to 128 registers per thread, 4: 64; 0: chosen from the program).
std::string spec_source(const CompiledGroup& cg, int min_blocks = 0);

// A persistent batch kernel specialized to a list of programs: the
// interpreter's batch_kernel work loop (items (job, tile) from a device
// counter) with a switch over BatchJob::spec_case into each program's
// specialized body. Closure pools live in BatchArgs::gheap (heap_slots =
// the largest pool) or in shared memory.
struct SpecBatchKernel {
    void* library = nullptr;
    void* kernel = nullptr;
    std::string key;
    uint32_t pool_slots = 0;  // largest closure pool (floats per point)
    int cases = 0;
    ~SpecBatchKernel();
};
std::string spec_batch_source(const std::vector<const CompiledGroup*>& cases);
// Distinct programs in a canonical order (by program content), so that the
// same set of programs gives the same batch kernel source, and cubin, in
// every executor.
void canonical_cases(std::vector<const CompiledGroup*>& cases);
int spec_batch_build(const std::vector<const CompiledGroup*>& cases, const std::string& csrc_dir,
                     const std::string& cache_dir, SpecBatchKernel* out, std::string* err);

// Build (or take from the cache) and load the kernel. `csrc_dir` holds the
// interpreter headers, `cache_dir` the generated sources and cubins.
int spec_build(const CompiledGroup& cg, const std::string& csrc_dir, const std::string& cache_dir,
               SpecKernel* out, std::string* err, int min_blocks = 0);

// Launch over [0, npoints): one CTA of 256 points per tile, closure pools in
// shared memory when they fit, else in the executor's HBM scratch.
// `block` 0 and `pool_smem` -1 choose automatically. With staged output
// records, `fill_unwritten` writes zeros to the record words no output op
// wrote (otherwise they keep what the buffer held).
int spec_launch(DeviceState& ds, const SpecKernel& k, const CompiledGroup& cg, int64_t npoints,
                const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream, std::string* err,
                int block = 0, int pool_smem = -1, bool fill_unwritten = false, const LaunchExtras* ex = nullptr);

}  // namespace oslg
