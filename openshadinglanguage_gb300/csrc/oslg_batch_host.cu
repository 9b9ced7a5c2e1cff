// Host side of the persistent batch executor: job table and work list,
// launch-shape choice, CUDA-graph capture and replay, and the autotuner.
//
// A batch holds requests (group, point count, globals, arenas) of many
// different groups. One launch of batch_kernel runs all of them: the work
// list has one item per (job, tile of `block` points), jobs ordered by
// their estimated cost per point, heaviest first, so that long tiles start
// early and short ones fill the tail. The whole step (counter reset +
// launch) is captured once as a CUDA graph and replayed while the batch is
// unchanged. The reference runs groups one execute() call at a time
// (src/liboslexec/shadingsys.cpp:329-394); nothing in it corresponds to
// this layer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "oslg_batch.h"

namespace oslg {

#define OSLG_BATCH_VARIANT(M, P)                                                                     \
    int batch_launch_##M##_##P(bool, unsigned, unsigned, size_t, void*, const dev::BatchArgs&);          \
    int batch_occupancy_##M##_##P(bool, int, size_t, int*);                                              \
    int batch_smem_limit_##M##_##P(int);
OSLG_BATCH_VARIANT(256, 1)
OSLG_BATCH_VARIANT(256, 2)
OSLG_BATCH_VARIANT(256, 4)
OSLG_BATCH_VARIANT(512, 1)
OSLG_BATCH_VARIANT(512, 2)
OSLG_BATCH_VARIANT(512, 4)
#undef OSLG_BATCH_VARIANT

namespace {
const size_t kBatchStaticSmem = 256;
bool ok(cudaError_t e, std::string* err, const char* what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}
struct VariantFns {
    int (*launch)(bool, unsigned, unsigned, size_t, void*, const dev::BatchArgs&);
    int (*occupancy)(bool, int, size_t, int*);
    int (*smem_limit)(int);
};
// indexed [maxt == 512][log2(ppt)]
const VariantFns kVariants[2][3] = {
    { { batch_launch_256_1, batch_occupancy_256_1, batch_smem_limit_256_1 },
      { batch_launch_256_2, batch_occupancy_256_2, batch_smem_limit_256_2 },
      { batch_launch_256_4, batch_occupancy_256_4, batch_smem_limit_256_4 } },
    { { batch_launch_512_1, batch_occupancy_512_1, batch_smem_limit_512_1 },
      { batch_launch_512_2, batch_occupancy_512_2, batch_smem_limit_512_2 },
      { batch_launch_512_4, batch_occupancy_512_4, batch_smem_limit_512_4 } } };
const VariantFns& variant(int maxt, int ppt) {
    return kVariants[maxt > 256 ? 1 : 0][ppt >= 4 ? 2 : (ppt == 2 ? 1 : 0)];
}
int norm_ppt(int p) { return p >= 4 ? 4 : (p == 2 || p == 3 ? 2 : 1); }
}  // namespace

// Shared entry points for other launchers of the batch kernel (the server).
int batch_variant_launch(int maxt, int ppt, bool smem, unsigned grid, unsigned block, size_t shmem, void* stream,
                         const dev::BatchArgs& b) {
    return variant(maxt, norm_ppt(ppt)).launch(smem, grid, block, shmem, stream, b);
}
int batch_variant_occupancy(int maxt, int ppt, bool smem, int block, size_t shmem, int* per_sm) {
    return variant(maxt, norm_ppt(ppt)).occupancy(smem, block, shmem, per_sm);
}
int batch_variants_prepare(const DeviceState& ds) {
    int dyn = (int)ds.smem_optin - (int)kBatchStaticSmem;
    for (int m = 0; m < 2; ++m)
        for (int q = 0; q < 3; ++q) {
            int e = kVariants[m][q].smem_limit(dyn);
            if (e != 0) return e;
        }
    return 0;
}
size_t batch_static_smem() { return kBatchStaticSmem; }

// Estimated cost of one point of a program: one unit per op, noise and
// transcendental ops weighted by their measured relative cost, ops inside
// loops by an expected trip count of 8 per nesting level.
double program_cost(const ProgramHeader& hdr, const Op* ops) {
    double cost = 0.0, mult = 1.0;
    for (uint32_t i = 0; i < hdr.nops; ++i) {
        const Op& o = ops[i];
        double w = 1.0;
        switch (o.code) {
        case OP_LOOP_BEGIN: mult *= 8.0; break;
        case OP_LOOP_END: mult = std::max(1.0, mult / 8.0); break;
        case OP_GABOR: w = (o.a[3] & 256u) ? 600.0 : 200.0; break;
        case OP_NOISE: {
            uint32_t kind = o.a[3] & 15u;
            bool vec = (o.a[3] & 256u) != 0, der = (o.a[3] & 512u) != 0;
            w = (kind == NK_CELL || kind == NK_HASH) ? 3.0 : (kind == NK_SIMPLEX || kind == NK_USIMPLEX) ? 6.0 : 7.0;
            if (vec) w *= 2.5;
            if (der) w *= 2.0;
            break;
        }
        case OP_SIN: case OP_COS: case OP_TAN: case OP_EXP: case OP_LOG: case OP_POW: case OP_ATAN2:
            w = 12.0;
            break;
        case OP_TRANSFORM: case OP_MDIV: w = 3.0; break;
        default: break;
        }
        cost += w * mult;
    }
    return cost;
}

BatchExecutor::~BatchExecutor() { release(); }

void BatchExecutor::release() {
    if (gexec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(gexec_));
    if (graph_) cudaGraphDestroy(static_cast<cudaGraph_t>(graph_));
    if (cap_stream_) cudaStreamDestroy(static_cast<cudaStream_t>(cap_stream_));
    gexec_ = graph_ = cap_stream_ = nullptr;
    cudaFree(d_jobs_);
    cudaFree(d_items_);
    cudaFree(d_counter_);
    cudaFree(d_heap_);
    cudaFree(d_spec_heap_);
    d_jobs_ = nullptr;
    d_items_ = nullptr;
    d_counter_ = nullptr;
    d_heap_ = nullptr;
    d_spec_heap_ = nullptr;
    jobs_cap_ = items_cap_ = heap_bytes_ = spec_heap_bytes_ = 0;
    spec_.reset();
    spec_cases_.clear();
}

void BatchExecutor::clear() {
    entries_.clear();
    dirty_ = true;
}

void BatchExecutor::add(const CompiledGroup& cg, int64_t npoints, const oslg_shaderglobals& G, void* userdata,
                        void* outputs) {
    BatchEntry e;
    e.cg = &cg;
    e.npoints = npoints;
    e.G = G;
    e.userdata = userdata;
    e.outputs = outputs;
    e.cost = program_cost(cg.header, reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader)));
    entries_.push_back(e);
    dirty_ = true;
}

void BatchExecutor::set_launch(const BatchLaunch& l) {
    want_ = l;
    dirty_ = true;
}

int BatchExecutor::ensure_ready(DeviceState& ds, std::string* err) {
    if (!ds_ready_) {
        // dynamic shared memory may use the opt-in size less the kernel's
        // static work-item slot (kBatchStaticSmem covers it)
        int dyn = (int)ds.smem_optin - (int)kBatchStaticSmem;
        for (int m = 0; m < 2; ++m)
            for (int q = 0; q < 3; ++q)
                if (!ok((cudaError_t)kVariants[m][q].smem_limit(dyn), err, "batch kernel attribute"))
                    return OSLG_ERR_CUDA;
        if (!ok(cudaMalloc(&d_counter_, sizeof(uint32_t)), err, "cudaMalloc counter")) return OSLG_ERR_CUDA;
        ds_ready_ = true;
    }
    return OSLG_OK;
}

// Upload the job table and work list (items (job, tile), heaviest jobs first).
static int upload_tables(std::vector<dev::BatchJob>& jobs, std::vector<uint2>& items, dev::BatchJob** d_jobs,
                         size_t* jobs_cap, uint2** d_items, size_t* items_cap, std::string* err) {
    if (jobs.size() > *jobs_cap) {
        cudaFree(*d_jobs);
        *d_jobs = nullptr;
        if (!ok(cudaMalloc(d_jobs, jobs.size() * sizeof(dev::BatchJob)), err, "cudaMalloc jobs")) return OSLG_ERR_CUDA;
        *jobs_cap = jobs.size();
    }
    if (items.size() > *items_cap) {
        cudaFree(*d_items);
        *d_items = nullptr;
        if (!ok(cudaMalloc(d_items, items.size() * sizeof(uint2)), err, "cudaMalloc items")) return OSLG_ERR_CUDA;
        *items_cap = items.size();
    }
    if (!jobs.empty() &&
        !ok(cudaMemcpy(*d_jobs, jobs.data(), jobs.size() * sizeof(dev::BatchJob), cudaMemcpyHostToDevice), err,
            "upload jobs"))
        return OSLG_ERR_CUDA;
    if (!items.empty() &&
        !ok(cudaMemcpy(*d_items, items.data(), items.size() * sizeof(uint2), cudaMemcpyHostToDevice), err,
            "upload items"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

// The jit launch: a persistent kernel whose cases are the batch's distinct
// programs, each a specialized body (the reference JITs each group, then
// renderers call it per batch; here one launch runs them all). Tiles are
// one point per thread; closure pools in shared memory when they fit.
int BatchExecutor::build_jit(DeviceState& ds, std::string* err) {
    std::vector<int> order(entries_.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return entries_[a].cost > entries_[b].cost; });
    std::vector<const CompiledGroup*> cases;
    for (const BatchEntry& e : entries_) cases.push_back(e.cg);
    canonical_cases(cases);
    std::vector<int> case_of(entries_.size(), 0);
    for (size_t i = 0; i < entries_.size(); ++i)
        case_of[i] = (int)(std::find(cases.begin(), cases.end(), entries_[i].cg) - cases.begin());
    if (!spec_ || cases != spec_cases_) {
        if (jit_csrc_.empty()) {
            if (err) *err = "batch: no source directory for specialized kernels";
            return OSLG_ERR_STATE;
        }
        auto k = std::make_unique<SpecBatchKernel>();
        int rc = spec_batch_build(cases, jit_csrc_, jit_cache_, k.get(), err);
        if (rc != OSLG_OK) return rc;
        spec_ = std::move(k);
        spec_cases_ = cases;
    }
    int block = want_.block > 0 ? want_.block : 256;
    block = std::max(32, std::min(256, (block + 31) & ~31));
    const void* fn = spec_->kernel;
    const size_t pool_b = (size_t)spec_->pool_slots * block * sizeof(float);
    const bool smem = pool_b > 0 && pool_b <= 100 * 1024 && want_.heap_smem != 0;
    const size_t shmem = smem ? pool_b : 0;
    if (shmem > 48 * 1024 &&
        !ok(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem), err,
            "specialized kernel attribute"))
        return OSLG_ERR_CUDA;
    int per_sm = 0;
    if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, shmem), err, "occupancy"))
        return OSLG_ERR_CUDA;
    if (per_sm < 1) {
        if (err) *err = "specialized batch launch does not fit on an SM";
        return OSLG_ERR_LOWER;
    }
    int grid = ds.sm_count * per_sm;
    if (want_.grid > 0) grid = want_.grid;
    std::vector<dev::BatchJob> jobs(entries_.size());
    std::vector<uint2> items;
    for (size_t j = 0; j < order.size(); ++j) {
        const BatchEntry& e = entries_[order[j]];
        dev::BatchJob& J = jobs[j];
        J.blob = static_cast<const uint8_t*>(e.cg->d_blob);
        J.npoints = e.npoints;
        J.userdata = static_cast<char*>(e.userdata);
        J.outputs = static_cast<char*>(e.outputs);
        J.G = e.G;
        J.spec_case = case_of[order[j]];
        const int64_t tiles = (e.npoints + block - 1) / block;
        for (int64_t t = 0; t < tiles; ++t) items.push_back(make_uint2((unsigned)j, (unsigned)t));
    }
    int rc = upload_tables(jobs, items, &d_jobs_, &jobs_cap_, &d_items_, &items_cap_, err);
    if (rc != OSLG_OK) return rc;
    if (!smem && pool_b > 0 && (size_t)grid * pool_b > spec_heap_bytes_) {
        cudaFree(d_spec_heap_);
        d_spec_heap_ = nullptr;
        spec_heap_bytes_ = 0;
        if (!ok(cudaMalloc(&d_spec_heap_, (size_t)grid * pool_b), err, "cudaMalloc closure pools"))
            return OSLG_ERR_CUDA;
        spec_heap_bytes_ = (size_t)grid * pool_b;
    }
    args_ = dev::BatchArgs{};
    args_.jobs = d_jobs_;
    args_.items = d_items_;
    args_.nitems = (uint32_t)items.size();
    args_.counter = d_counter_;
    args_.gheap = smem ? nullptr : d_spec_heap_;
    args_.status = ds.d_status;
    args_.textures = ds.d_textures;
    args_.ntextures = ds.ntextures;
    args_.heap_slots = spec_->pool_slots;
    spec_pool_smem_ = smem ? 1 : 0;
    cur_.block = block;
    cur_.points_per_thread = 1;
    cur_.heap_smem = smem ? 1 : 0;
    cur_.grid = grid;
    cur_.use_graph = want_.use_graph;
    cur_.jit = 1;
    shmem_ = shmem;
    per_sm_ = per_sm;
    if (gexec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(gexec_));
    if (graph_) cudaGraphDestroy(static_cast<cudaGraph_t>(graph_));
    gexec_ = graph_ = nullptr;
    dirty_ = false;
    return OSLG_OK;
}

// Work list, job table, heap and launch shape for the requested launch.
int BatchExecutor::build(DeviceState& ds, std::string* err) {
    int rc = ensure_ready(ds, err);
    if (rc != OSLG_OK) return rc;
    if (want_.jit) return build_jit(ds, err);
    BatchLaunch L = want_;
    int block = L.block > 0 ? L.block : 256;
    block = std::max(32, std::min(512, (block + 31) & ~31));
    const int maxt = block > 256 ? 512 : 256;
    const int ppt = norm_ppt(L.points_per_thread);
    const int tile = block * ppt;
    uint32_t prog_bytes = 0, slots = 0;
    for (const BatchEntry& e : entries_) {
        const ProgramHeader& h = e.cg->header;
        uint32_t pb = h.nops * (uint32_t)sizeof(Op) + ((h.nconst + 3u) & ~3u) * 4u;
        prog_bytes = std::max(prog_bytes, pb);
        slots = std::max(slots, h.heap_slots);
    }
    prog_bytes = (prog_bytes + 15u) & ~15u;
    const size_t heap_b = (size_t)slots * tile * sizeof(float);
    bool smem = L.heap_smem == 1 || (L.heap_smem < 0 && prog_bytes + heap_b <= 100 * 1024);
    if (smem && prog_bytes + heap_b + kBatchStaticSmem > ds.smem_optin) smem = false;
    const size_t shmem = prog_bytes + (smem ? heap_b : 0);
    if (shmem + kBatchStaticSmem > ds.smem_optin) {
        if (err) *err = "batch programs do not fit in shared memory";
        return OSLG_ERR_LOWER;
    }
    int per_sm = 0;
    if (!ok((cudaError_t)variant(maxt, ppt).occupancy(smem, block, shmem, &per_sm), err, "occupancy"))
        return OSLG_ERR_CUDA;
    if (per_sm < 1) {
        if (err) *err = "batch launch shape does not fit on an SM";
        return OSLG_ERR_LOWER;
    }
    int grid = ds.sm_count * per_sm;
    if (L.grid > 0) grid = L.grid;

    // jobs by estimated cost per point, heaviest first; ties keep insertion order
    std::vector<int> order(entries_.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return entries_[a].cost > entries_[b].cost; });
    std::vector<dev::BatchJob> jobs(entries_.size());
    std::vector<uint2> items;
    for (size_t j = 0; j < order.size(); ++j) {
        const BatchEntry& e = entries_[order[j]];
        dev::BatchJob& J = jobs[j];
        J.blob = static_cast<const uint8_t*>(e.cg->d_blob);
        J.npoints = e.npoints;
        J.userdata = static_cast<char*>(e.userdata);
        J.outputs = static_cast<char*>(e.outputs);
        J.G = e.G;
        const int64_t tiles = (e.npoints + tile - 1) / tile;
        for (int64_t t = 0; t < tiles; ++t) items.push_back(make_uint2((unsigned)j, (unsigned)t));
    }
    rc = upload_tables(jobs, items, &d_jobs_, &jobs_cap_, &d_items_, &items_cap_, err);
    if (rc != OSLG_OK) return rc;
    if (!smem) {
        size_t need = (size_t)grid * heap_b;
        if (need > heap_bytes_) {
            cudaFree(d_heap_);
            d_heap_ = nullptr;
            heap_bytes_ = 0;
            if (!ok(cudaMalloc(&d_heap_, need), err, "cudaMalloc batch heap")) return OSLG_ERR_CUDA;
            heap_bytes_ = need;
        }
    }
    args_.jobs = d_jobs_;
    args_.items = d_items_;
    args_.nitems = (uint32_t)items.size();
    args_.counter = d_counter_;
    args_.gheap = smem ? nullptr : d_heap_;
    args_.status = ds.d_status;
    args_.textures = ds.d_textures;
    args_.ntextures = ds.ntextures;
    args_.prog_bytes = prog_bytes;
    args_.heap_slots = slots;
    cur_.block = block;
    cur_.points_per_thread = ppt;
    cur_.heap_smem = smem ? 1 : 0;
    cur_.grid = grid;
    cur_.use_graph = L.use_graph;
    cur_.jit = 0;
    shmem_ = shmem;
    maxt_ = maxt;
    per_sm_ = per_sm;
    // any captured graph refers to the old tables
    if (gexec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(gexec_));
    if (graph_) cudaGraphDestroy(static_cast<cudaGraph_t>(graph_));
    gexec_ = graph_ = nullptr;
    dirty_ = false;
    return OSLG_OK;
}

int BatchExecutor::enqueue(void* stream, std::string* err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!ok(cudaMemsetAsync(d_counter_, 0, sizeof(uint32_t), s), err, "counter reset")) return OSLG_ERR_CUDA;
    if (args_.nitems == 0) return OSLG_OK;
    if (cur_.jit) {
        int pool_smem = spec_pool_smem_;
        void* kargs[] = { &args_, &pool_smem };
        if (!ok(cudaLaunchKernel(spec_->kernel, dim3((unsigned)cur_.grid), dim3((unsigned)cur_.block), kargs, shmem_,
                                 s),
                err, "specialized batch launch"))
            return OSLG_ERR_CUDA;
        return OSLG_OK;
    }
    if (!ok((cudaError_t)variant(maxt_, cur_.points_per_thread)
                .launch(cur_.heap_smem == 1, (unsigned)cur_.grid, (unsigned)cur_.block, shmem_, stream, args_),
            err, "batch launch"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

int BatchExecutor::execute(DeviceState& ds, void* stream, std::string* err) {
    if (dirty_) {
        int rc = build(ds, err);
        if (rc != OSLG_OK) return rc;
    }
    if (!cur_.use_graph) return enqueue(stream, err);
    if (!gexec_) {
        // capture on a private stream (the caller's may be the legacy default
        // stream, which cannot be captured); the graph replays on any stream
        if (!cap_stream_) {
            cudaStream_t cs;
            if (!ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), err, "capture stream")) return OSLG_ERR_CUDA;
            cap_stream_ = cs;
        }
        cudaStream_t cs = static_cast<cudaStream_t>(cap_stream_);
        if (!ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), err, "begin capture")) return OSLG_ERR_CUDA;
        std::string e2;
        int rc = enqueue(cs, &e2);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(cs, &g);
        if (rc != OSLG_OK) {
            if (g) cudaGraphDestroy(g);
            if (err) *err = e2;
            return rc;
        }
        if (!ok(ce, err, "end capture")) return OSLG_ERR_CUDA;
        cudaGraphExec_t ge = nullptr;
        if (!ok(cudaGraphInstantiate(&ge, g, 0), err, "graph instantiate")) {
            cudaGraphDestroy(g);
            return OSLG_ERR_CUDA;
        }
        graph_ = g;
        gexec_ = ge;
    }
    if (!ok(cudaGraphLaunch(static_cast<cudaGraphExec_t>(gexec_), static_cast<cudaStream_t>(stream)), err,
            "graph launch"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

// Sweep points per thread x block size x heap placement, timing `reps` launches of each with
// CUDA events on the caller's stream; keep the fastest. Candidates whose
// shared-memory heap does not fit are skipped.
int BatchExecutor::autotune(DeviceState& ds, void* stream, int reps, BatchTuneResult* results, int cap, int* n,
                            BatchLaunch* best, std::string* err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const BatchLaunch keep = want_;
    float best_ms = 1e30f;
    BatchLaunch best_l = keep;
    int count = 0;
    cudaEvent_t e0, e1;
    if (!ok(cudaEventCreate(&e0), err, "event")) return OSLG_ERR_CUDA;
    if (!ok(cudaEventCreate(&e1), err, "event")) {
        cudaEventDestroy(e0);
        return OSLG_ERR_CUDA;
    }
    int rc = OSLG_OK;
    // a jit batch has one kernel: only its block size (128 or 256) is swept
    const bool jit = keep.jit != 0;
    for (int ppt : { 1, 2, 4 }) {
    if (jit && ppt != 1) break;
    for (int block : { 128, 256, 512 }) {
        if (jit && block > 256) break;
        for (int heap : { 1, 0 }) {
            BatchLaunch l = keep;
            l.block = block;
            l.points_per_thread = ppt;
            l.heap_smem = heap;
            l.use_graph = 0;
            if (jit && heap == 0) continue;  // pools placed automatically
            want_ = l;
            dirty_ = true;
            std::string e2;
            int r2 = build(ds, &e2);
            if (r2 != OSLG_OK || (!jit && cur_.heap_smem != heap)) continue;  // does not fit: skip
            if ((rc = enqueue(stream, err)) != OSLG_OK) break;      // warm-up
            if (!ok(cudaEventRecord(e0, s), err, "event record")) { rc = OSLG_ERR_CUDA; break; }
            for (int r = 0; r < std::max(1, reps) && rc == OSLG_OK; ++r) rc = enqueue(stream, err);
            if (rc != OSLG_OK) break;
            if (!ok(cudaEventRecord(e1, s), err, "event record") || !ok(cudaEventSynchronize(e1), err, "event sync")) {
                rc = OSLG_ERR_CUDA;
                break;
            }
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            ms /= (float)std::max(1, reps);
            if (results && count < cap) {
                results[count].block = cur_.block;
                results[count].points_per_thread = cur_.points_per_thread;
                results[count].heap_smem = cur_.heap_smem;
                results[count].grid = cur_.grid;
                results[count].ctas_per_sm = per_sm_;
                results[count].ms = ms;
            }
            ++count;
            if (ms < best_ms) {
                best_ms = ms;
                best_l = l;
            }
        }
        if (rc != OSLG_OK) break;
    }
    if (rc != OSLG_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (n) *n = count;
    best_l.use_graph = keep.use_graph;
    want_ = best_l;
    dirty_ = true;
    if (best) *best = best_l;
    return rc;
}

void BatchExecutor::last_launch(BatchTuneResult* r) const {
    r->block = cur_.block;
    r->points_per_thread = cur_.points_per_thread;
    r->heap_smem = cur_.heap_smem;
    r->grid = cur_.grid;
    r->ctas_per_sm = per_sm_;
    r->ms = 0.0f;
}

}  // namespace oslg
