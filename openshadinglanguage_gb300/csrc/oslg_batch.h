// Persistent batch executor (oslg_batch_host.cu): many groups, one launch.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <memory>

#include "oslg_exec.h"
#include "oslg_host.h"
#include "oslg_spec.h"

namespace oslg {

struct BatchLaunch {
    int block = 256;     // threads per CTA
    int points_per_thread = 1;  // 1, 2 or 4: a tile is block * points_per_thread points
    int heap_smem = -1;  // 1 shared memory, 0 HBM, -1 shared memory when it fits 100 KiB
    int grid = 0;        // 0: SMs x resident CTAs per SM
    int use_graph = 1;   // replay a captured CUDA graph
    int jit = 0;         // run the groups' specialized bodies (one kernel built for the batch's programs)
};

struct BatchTuneResult {
    int block;
    int points_per_thread;
    int heap_smem;
    int grid;
    int ctas_per_sm;
    float ms;
};

double program_cost(const ProgramHeader& hdr, const Op* ops);

// Launch one variant of the batch kernel (maxt 256/512, ppt 1/2/4).
int batch_variant_launch(int maxt, int ppt, bool smem, unsigned grid, unsigned block, size_t shmem, void* stream,
                         const dev::BatchArgs& b);
int batch_variant_occupancy(int maxt, int ppt, bool smem, int block, size_t shmem, int* per_sm);
// Allow every variant its dynamic shared memory (once per device).
int batch_variants_prepare(const DeviceState& ds);
size_t batch_static_smem();

class BatchExecutor {
public:
    ~BatchExecutor();
    void clear();
    void add(const CompiledGroup& cg, int64_t npoints, const oslg_shaderglobals& G, void* userdata, void* outputs);
    void set_launch(const BatchLaunch& l);
    // Where specialized kernels are generated from and cached (jit launches).
    void set_jit_dirs(const std::string& csrc, const std::string& cache) {
        jit_csrc_ = csrc;
        jit_cache_ = cache;
    }
    int execute(DeviceState& ds, void* stream, std::string* err);
    int autotune(DeviceState& ds, void* stream, int reps, BatchTuneResult* results, int cap, int* n,
                 BatchLaunch* best, std::string* err);
    void last_launch(BatchTuneResult* r) const;
    size_t size() const { return entries_.size(); }

private:
    struct BatchEntry {
        const CompiledGroup* cg;
        int64_t npoints;
        oslg_shaderglobals G;
        void* userdata;
        void* outputs;
        double cost;
    };
    int ensure_ready(DeviceState& ds, std::string* err);
    int build(DeviceState& ds, std::string* err);
    int enqueue(void* stream, std::string* err);
    void release();

    std::vector<BatchEntry> entries_;
    BatchLaunch want_, cur_;
    bool dirty_ = true;
    bool ds_ready_ = false;
    dev::BatchArgs args_{};
    size_t shmem_ = 0;
    int maxt_ = 256;
    int per_sm_ = 0;
    dev::BatchJob* d_jobs_ = nullptr;
    uint2* d_items_ = nullptr;
    uint32_t* d_counter_ = nullptr;
    float* d_heap_ = nullptr;
    size_t jobs_cap_ = 0, items_cap_ = 0, heap_bytes_ = 0;
    void* graph_ = nullptr;
    void* gexec_ = nullptr;
    void* cap_stream_ = nullptr;
    // specialized persistent kernel (jit): one body per distinct program
    std::string jit_csrc_, jit_cache_;
    std::unique_ptr<SpecBatchKernel> spec_;
    std::vector<const CompiledGroup*> spec_cases_;
    int spec_pool_smem_ = 0;
    float* d_spec_heap_ = nullptr;
    size_t spec_heap_bytes_ = 0;
    int build_jit(DeviceState& ds, std::string* err);
};

}  // namespace oslg
