// Shading server (oslg_serve.h): admission against an HBM budget, waves of
// requests run by the persistent batch kernel, several waves in flight.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>

#include "oslg_serve.h"

namespace oslg {

namespace {
bool ok(cudaError_t e, std::string* err, const char* what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}
int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
// components of each shader-global field (GlobalId order)
int field_components(int gid) {
    switch (gid) {
    case G_U: case G_DUDX: case G_DUDY: case G_V: case G_DVDX: case G_DVDY: case G_TIME: case G_DTIME:
    case G_SURFACEAREA: case G_FLIPHANDEDNESS: case G_BACKFACING:
        return 1;
    default: return 3;
    }
}
oslg_field* fields(oslg_shaderglobals& G) { return &G.P; }
const oslg_field* fields(const oslg_shaderglobals& G) { return &G.P; }
// heap slots need at most this many per program in the worst case the
// scratch reserve is sized for (larger programs grow the reserve on use)
const uint32_t kReserveSlots = 256;
// threads per CTA of a specialized wave (one point per thread)
const int kSpecWaveBlock = 256;
}  // namespace

// ---- arena ---------------------------------------------------------------------------
int DeviceArena::init(size_t bytes, std::string* err) {
    bytes = bytes & ~size_t(255);
    if (bytes == 0) {
        if (err) *err = "device arena of zero bytes";
        return OSLG_ERR_ARG;
    }
    if (!ok(cudaMalloc(&base_, bytes), err, "cudaMalloc arena")) return OSLG_ERR_CUDA;
    cap_ = bytes;
    used_ = 0;
    free_.clear();
    free_[0] = bytes;
    return OSLG_OK;
}

void DeviceArena::release() {
    if (base_) cudaFree(base_);
    base_ = nullptr;
    cap_ = used_ = 0;
    free_.clear();
}

bool DeviceArena::alloc(size_t bytes, size_t* off) {
    bytes = round(std::max<size_t>(bytes, 1));
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second < bytes) continue;
        *off = it->first;
        size_t rest = it->second - bytes;
        size_t noff = it->first + bytes;
        free_.erase(it);
        if (rest) free_[noff] = rest;
        used_ += bytes;
        return true;
    }
    return false;
}

void DeviceArena::free(size_t off, size_t bytes) {
    bytes = round(std::max<size_t>(bytes, 1));
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
    }
    if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_.erase(it);
        }
    }
}

// ---- server --------------------------------------------------------------------------
ShadingServer::~ShadingServer() { stop(); }

int ShadingServer::start(std::string* err) {
    if (running_) return OSLG_OK;
    int rc = start_resources(err);
    if (rc != OSLG_OK) {
        release_resources();
        return rc;
    }
    running_ = true;
    stopping_ = false;
    thread_ = std::thread([this]() { worker(); });
    return OSLG_OK;
}

int ShadingServer::start_resources(std::string* err) {
    if (opt_.streams < 1 || opt_.streams > 16 || opt_.block < 32 || opt_.block > 512 || opt_.max_wave_requests < 1 ||
        opt_.max_wave_points < 1) {
        if (err) *err = "server options out of range";
        return OSLG_ERR_ARG;
    }
    int rc = batch_variants_prepare(ds_);
    if (rc != 0) {
        if (err) *err = std::string("batch kernel attribute: ") + cudaGetErrorString((cudaError_t)rc);
        return OSLG_ERR_CUDA;
    }
    const int tile = opt_.block * opt_.points_per_thread;
    int per_sm = 0;
    const int maxt = opt_.block > 256 ? 512 : 256;
    if (!ok((cudaError_t)batch_variant_occupancy(maxt, opt_.points_per_thread, false, opt_.block, 64 * 1024, &per_sm),
            err, "occupancy"))
        return OSLG_ERR_CUDA;
    per_sm_ = std::max(1, per_sm);
    grid_ = ds_.sm_count * per_sm_;
    const size_t items_cap = (size_t)(opt_.max_wave_points / tile) + (size_t)opt_.max_wave_requests + 1;
    const size_t scratch_each = (size_t)grid_ * kReserveSlots * tile * sizeof(float);
    const size_t reserve = scratch_each * opt_.streams + (size_t(64) << 20);  // + programs and tables
    if (opt_.budget_bytes <= reserve + (size_t(16) << 20)) {
        if (err) *err = "HBM budget too small for the server's scratch heaps";
        return OSLG_ERR_ARG;
    }
    size_t arena = opt_.budget_bytes - reserve;
    if (opt_.arena_bytes) {
        if (opt_.arena_bytes > arena) {
            if (err) *err = "arena_bytes does not fit in the HBM budget next to the scratch heaps";
            return OSLG_ERR_ARG;
        }
        arena = opt_.arena_bytes;
    }
    rc = arena_.init(arena, err);
    if (rc != OSLG_OK) return rc;
    slots_.resize(opt_.streams);
    for (Slot& s : slots_) {
        s.owner = this;
        cudaStream_t st;
        if (!ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), err, "stream")) return OSLG_ERR_CUDA;
        s.stream = st;
        if (!ok(cudaMalloc(&s.d_jobs, opt_.max_wave_requests * sizeof(dev::BatchJob)), err, "cudaMalloc jobs") ||
            !ok(cudaMalloc(&s.d_items, items_cap * sizeof(uint2)), err, "cudaMalloc items") ||
            !ok(cudaMalloc(&s.d_counter, sizeof(uint32_t)), err, "cudaMalloc counter") ||
            !ok(cudaMallocHost(&s.h_jobs, opt_.max_wave_requests * sizeof(dev::BatchJob)), err, "pinned jobs") ||
            !ok(cudaMallocHost(&s.h_items, items_cap * sizeof(uint2)), err, "pinned items") ||
            !ok(cudaMalloc(&s.d_status, opt_.max_wave_requests * sizeof(uint32_t)), err, "cudaMalloc status") ||
            !ok(cudaMallocHost(&s.h_status, opt_.max_wave_requests * sizeof(uint32_t)), err, "pinned status"))
            return OSLG_ERR_CUDA;
        s.items_cap = items_cap;
        s.heap_bytes = scratch_each;
        if (!ok(cudaMalloc(&s.d_heap, s.heap_bytes), err, "cudaMalloc scratch heap")) return OSLG_ERR_CUDA;
        stats_.scratch_bytes += s.heap_bytes;
    }
    stats_.arena_capacity = arena_.capacity();
    return OSLG_OK;
}

void ShadingServer::stop() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (!running_) return;
        stopping_ = true;
    }
    cv_.notify_all();
    if (thread_.joinable()) thread_.join();
    release_resources();
    running_ = false;
}

void ShadingServer::release_resources() {
    for (Slot& s : slots_) {
        if (s.stream) cudaStreamSynchronize(static_cast<cudaStream_t>(s.stream));
        cudaFree(s.d_jobs);
        cudaFree(s.d_items);
        cudaFree(s.d_counter);
        cudaFree(s.d_heap);
        cudaFreeHost(s.h_jobs);
        cudaFreeHost(s.h_items);
        cudaFree(s.d_status);
        cudaFreeHost(s.h_status);
        if (s.stream) cudaStreamDestroy(static_cast<cudaStream_t>(s.stream));
    }
    slots_.clear();
    arena_.release();
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& kv : reqs_) delete kv.second;
    reqs_.clear();
    pending_.clear();
}

int ShadingServer::register_program(const CompiledGroup& cg, std::string* err) {
    if (!cg.d_blob) {
        if (err) *err = "program is not on the device";
        return OSLG_ERR_STATE;
    }
    std::lock_guard<std::mutex> lk(mu_);
    if (programs_.count(&cg)) return OSLG_OK;
    programs_[&cg] = cg.header.heap_slots;
    heap_slots_ = std::max(heap_slots_, cg.header.heap_slots);
    uint32_t pb = cg.header.nops * (uint32_t)sizeof(Op) + ((cg.header.nconst + 3u) & ~3u) * 4u;
    prog_bytes_ = std::max(prog_bytes_, (pb + 15u) & ~15u);
    stats_.program_bytes += cg.blob.size();
    return OSLG_OK;
}

size_t ShadingServer::request_device_bytes(const Request& r) const {
    return DeviceArena::round(r.in_bytes) + DeviceArena::round(r.out_bytes);
}

int ShadingServer::submit(const CompiledGroup& cg, int64_t npoints, const oslg_shaderglobals& hG, void* host_out,
                          size_t out_bytes, uint64_t* ticket, std::string* err) {
    if (npoints < 0 || (npoints > 0 && (!host_out || out_bytes == 0))) {
        if (err) *err = "bad request";
        return OSLG_ERR_ARG;
    }
    int rc = register_program(cg, err);
    if (rc != OSLG_OK) return rc;
    Request* r = new Request;
    r->cg = &cg;
    r->n = npoints;
    r->hG = hG;
    r->host_out = host_out;
    r->out_bytes = out_bytes;
    const oslg_field* f = fields(hG);
    for (int g = 0; g < G_COUNT; ++g)
        if (f[g].data) r->in_bytes += DeviceArena::round((size_t)field_components(g) * npoints * sizeof(float));
    r->dev_bytes = request_device_bytes(*r);
    r->st.submit_ns = now_ns();
    std::lock_guard<std::mutex> lk(mu_);
    if (!running_ || stopping_) {
        delete r;
        if (err) *err = "server is not running";
        return OSLG_ERR_STATE;
    }
    if (r->dev_bytes > arena_.capacity()) {
        delete r;
        if (err) *err = "request needs more device memory than the HBM budget allows";
        return OSLG_ERR_ARG;
    }
    r->id = next_id_++;
    reqs_[r->id] = r;
    stats_.submitted++;
    if (npoints == 0) {
        r->st.admit_ns = r->st.done_ns = r->st.submit_ns;
        r->done = true;
        stats_.completed++;
    } else {
        pending_.push_back(r);
    }
    *ticket = r->id;
    cv_.notify_all();
    return OSLG_OK;
}

void ShadingServer::on_wave_done(void* p) {
    Slot* s = static_cast<Slot*>(p);
    ShadingServer* self = s->owner;
    int64_t t = now_ns();
    std::lock_guard<std::mutex> lk(self->mu_);
    for (Request* r : s->reqs) {
        r->st.done_ns = t;
        // a job that raised a status bit (closure overflow, index bounds,
        // loop limit) fails its own request only
        r->bits = s->h_status[r->job];
        if (r->bits) r->st.status = OSLG_ERR_DEVICE;
    }
    s->complete = true;
    self->cv_.notify_all();
}

// The specialized wave kernel for the resident programs (canonical order:
// the same set gives the same kernel as the batch executor's).
int ShadingServer::ensure_spec(std::string* err) {
    std::vector<const CompiledGroup*> cases;
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (auto& kv : programs_) cases.push_back(kv.first);
    }
    canonical_cases(cases);
    if (!spec_kernels_.empty() && cases == spec_cases_) return OSLG_OK;
    auto k = std::make_unique<SpecBatchKernel>();
    int rc = spec_batch_build(cases, opt_.jit_csrc, opt_.jit_cache, k.get(), err);
    if (rc != OSLG_OK) return rc;
    int per_sm = 0;
    if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k->kernel, kSpecWaveBlock, 0), err, "occupancy"))
        return OSLG_ERR_CUDA;
    spec_grid_ = ds_.sm_count * std::max(1, per_sm);
    spec_kernels_.push_back(std::move(k));
    spec_cases_ = cases;
    return OSLG_OK;
}

int ShadingServer::launch_wave(Slot& s, std::vector<Request*>& wave, std::string* err) {
    cudaStream_t st = static_cast<cudaStream_t>(s.stream);
    const bool jit = !opt_.jit_csrc.empty();
    if (jit) {
        int rc = ensure_spec(err);
        if (rc != OSLG_OK) return rc;
    }
    // specialized waves: one point per thread, closure pools in the slot's scratch
    const int tile = jit ? kSpecWaveBlock : opt_.block * opt_.points_per_thread;
    const int maxt = opt_.block > 256 ? 512 : 256;
    uint32_t slots = 0, pbytes = 0;
    for (Request* r : wave) {
        slots = std::max(slots, r->cg->header.heap_slots);
        uint32_t pb = r->cg->header.nops * (uint32_t)sizeof(Op) + ((r->cg->header.nconst + 3u) & ~3u) * 4u;
        pbytes = std::max(pbytes, (pb + 15u) & ~15u);
    }
    const size_t heap_need = jit ? (size_t)spec_grid_ * spec_kernels_.back()->pool_slots * tile * sizeof(float)
                                 : (size_t)grid_ * slots * tile * sizeof(float);
    if (heap_need > s.heap_bytes) {
        // a program larger than the reserve: grow this slot's scratch heap
        if (!ok(cudaStreamSynchronize(st), err, "sync")) return OSLG_ERR_CUDA;
        cudaFree(s.d_heap);
        s.d_heap = nullptr;
        if (!ok(cudaMalloc(&s.d_heap, heap_need), err, "cudaMalloc scratch heap")) return OSLG_ERR_CUDA;
        s.heap_bytes = heap_need;
    }
    // jobs heaviest first, then their tiles
    std::vector<std::pair<double, Request*>> order;
    for (Request* r : wave)
        order.push_back({ program_cost(r->cg->header,
                                       reinterpret_cast<const Op*>(r->cg->blob.data() + sizeof(ProgramHeader))),
                          r });
    std::stable_sort(order.begin(), order.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
    size_t total_tiles = 0;
    for (Request* r : wave) total_tiles += (size_t)((r->n + tile - 1) / tile);
    if (total_tiles > s.items_cap) {
        // one request larger than a wave: grow this slot's work list (the
        // slot is idle, its staging buffers are free)
        cudaFree(s.d_items);
        cudaFreeHost(s.h_items);
        s.d_items = nullptr;
        s.h_items = nullptr;
        s.items_cap = 0;
        if (!ok(cudaMalloc(&s.d_items, total_tiles * sizeof(uint2)), err, "cudaMalloc items") ||
            !ok(cudaMallocHost(&s.h_items, total_tiles * sizeof(uint2)), err, "pinned items"))
            return OSLG_ERR_CUDA;
        s.items_cap = total_tiles;
    }
    size_t nitems = 0;
    for (size_t j = 0; j < order.size(); ++j) {
        Request* r = order[j].second;
        char* base = arena_.base() + r->dev_off;
        size_t o = 0;
        r->dG = r->hG;
        oslg_field* df = fields(r->dG);
        const oslg_field* hf = fields(r->hG);
        for (int g = 0; g < G_COUNT; ++g) {
            if (!hf[g].data) continue;
            const int nc = field_components(g);
            float* d = reinterpret_cast<float*>(base + o);
            const size_t plane = (size_t)r->n * sizeof(float);
            if (nc == 1 || hf[g].plane_stride == r->n) {
                if (!ok(cudaMemcpyAsync(d, hf[g].data, plane * nc, cudaMemcpyHostToDevice, st), err, "input copy"))
                    return OSLG_ERR_CUDA;
            } else {
                for (int c = 0; c < nc; ++c)
                    if (!ok(cudaMemcpyAsync(d + (size_t)c * r->n, hf[g].data + (size_t)c * hf[g].plane_stride, plane,
                                            cudaMemcpyHostToDevice, st),
                            err, "input copy"))
                        return OSLG_ERR_CUDA;
            }
            df[g].data = d;
            df[g].plane_stride = r->n;
            o += DeviceArena::round(plane * nc);
        }
        char* d_out = base + DeviceArena::round(r->in_bytes);
        // outputs start zeroed so that bytes the program does not write are
        // the same in every mix
        if (!ok(cudaMemsetAsync(d_out, 0, r->out_bytes, st), err, "output clear")) return OSLG_ERR_CUDA;
        dev::BatchJob& J = s.h_jobs[j];
        r->job = (int)j;
        J.status = s.d_status + j;
        J.blob = static_cast<const uint8_t*>(r->cg->d_blob);
        J.npoints = r->n;
        J.userdata = nullptr;
        J.outputs = d_out;
        J.G = r->dG;
        J.spec_case = jit ? (int)(std::find(spec_cases_.begin(), spec_cases_.end(), r->cg) - spec_cases_.begin()) : 0;
        const int64_t tiles = (r->n + tile - 1) / tile;
        for (int64_t t = 0; t < tiles; ++t) s.h_items[nitems++] = make_uint2((unsigned)j, (unsigned)t);
    }
    if (!ok(cudaMemcpyAsync(s.d_jobs, s.h_jobs, order.size() * sizeof(dev::BatchJob), cudaMemcpyHostToDevice, st), err,
            "jobs copy") ||
        !ok(cudaMemcpyAsync(s.d_items, s.h_items, nitems * sizeof(uint2), cudaMemcpyHostToDevice, st), err,
            "items copy") ||
        !ok(cudaMemsetAsync(s.d_counter, 0, sizeof(uint32_t), st), err, "counter reset") ||
        !ok(cudaMemsetAsync(s.d_status, 0, order.size() * sizeof(uint32_t), st), err, "status clear"))
        return OSLG_ERR_CUDA;
    dev::BatchArgs a;
    a.jobs = s.d_jobs;
    a.items = s.d_items;
    a.nitems = (uint32_t)nitems;
    a.counter = s.d_counter;
    a.gheap = s.d_heap;
    a.status = ds_.d_status;
    a.textures = ds_.d_textures;
    a.ntextures = ds_.ntextures;
    a.prog_bytes = pbytes;
    a.heap_slots = slots;
    if (jit) {
        a.heap_slots = spec_kernels_.back()->pool_slots;
        int pool_smem = 0;
        void* kargs[] = { &a, &pool_smem };
        if (!ok(cudaLaunchKernel(spec_kernels_.back()->kernel, dim3((unsigned)spec_grid_), dim3(kSpecWaveBlock), kargs,
                                 0, st),
                err, "specialized wave launch"))
            return OSLG_ERR_CUDA;
    } else if (!ok((cudaError_t)batch_variant_launch(maxt, opt_.points_per_thread, false, (unsigned)grid_,
                                                     (unsigned)opt_.block, pbytes, st, a),
                   err, "wave launch"))
        return OSLG_ERR_CUDA;
    for (auto& pr : order) {
        Request* r = pr.second;
        char* d_out = arena_.base() + r->dev_off + DeviceArena::round(r->in_bytes);
        if (!ok(cudaMemcpyAsync(r->host_out, d_out, r->out_bytes, cudaMemcpyDeviceToHost, st), err, "output copy"))
            return OSLG_ERR_CUDA;
    }
    if (!ok(cudaMemcpyAsync(s.h_status, s.d_status, order.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st), err,
            "status copy"))
        return OSLG_ERR_CUDA;
    if (!ok(cudaLaunchHostFunc(st, &ShadingServer::on_wave_done, &s), err, "completion callback"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

void ShadingServer::worker() {
    if (ds_.device >= 0) cudaSetDevice(ds_.device);
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        // retire finished waves: free their device memory, report their requests
        bool busy = false;
        for (Slot& s : slots_) {
            if (s.busy && s.complete) {
                for (Request* r : s.reqs) {
                    arena_.free(r->dev_off, r->dev_bytes);
                    r->done = true;
                    if (r->st.status != OSLG_OK) {
                        stats_.failed++;
                    } else {
                        stats_.completed++;
                        stats_.points_done += r->n;
                    }
                }
                s.reqs.clear();
                s.busy = false;
                s.complete = false;
                stats_.in_flight_waves--;
                done_cv_.notify_all();
            }
            busy = busy || s.busy;
        }
        if (stopping_ && pending_.empty() && !busy) break;
        Slot* slot = nullptr;
        for (Slot& s : slots_)
            if (!s.busy) { slot = &s; break; }
        if (!slot || pending_.empty()) {
            cv_.wait(lk);
            continue;
        }
        // admit in arrival order while device memory and the wave limits allow
        std::vector<Request*> wave;
        int64_t pts = 0;
        while (!pending_.empty() && (int)wave.size() < opt_.max_wave_requests) {
            Request* r = pending_.front();
            if (!wave.empty() && pts + r->n > opt_.max_wave_points) break;
            size_t off = 0;
            if (!arena_.alloc(r->dev_bytes, &off)) break;
            r->dev_off = off;
            r->st.admit_ns = now_ns();
            pending_.pop_front();
            wave.push_back(r);
            pts += r->n;
        }
        if (wave.empty()) {  // memory full: wait for a wave to finish
            cv_.wait(lk);
            continue;
        }
        stats_.arena_high_water = std::max(stats_.arena_high_water, arena_.used());
        slot->busy = true;
        slot->complete = false;
        slot->reqs = wave;
        slot->wave = next_wave_++;
        for (Request* r : wave) r->st.wave = slot->wave;
        stats_.waves++;
        stats_.in_flight_waves++;
        lk.unlock();
        std::string e;
        int rc = launch_wave(*slot, wave, &e);
        lk.lock();
        if (rc != OSLG_OK) {
            // nothing of this wave reaches the callback: fail its requests
            cudaStreamSynchronize(static_cast<cudaStream_t>(slot->stream));
            for (Request* r : wave) {
                arena_.free(r->dev_off, r->dev_bytes);
                r->st.status = rc;
                r->st.done_ns = now_ns();
                r->done = true;
                stats_.failed++;
            }
            worker_error_ = e;
            slot->reqs.clear();
            slot->busy = false;
            stats_.in_flight_waves--;
            done_cv_.notify_all();
        }
    }
}

int ShadingServer::wait(uint64_t ticket, int timeout_ms, RequestStats* st, std::string* err) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = reqs_.find(ticket);
    if (it == reqs_.end()) {
        if (err) *err = "unknown request ticket";
        return OSLG_ERR_ARG;
    }
    Request* r = it->second;
    auto pred = [&]() { return r->done; };
    if (timeout_ms < 0) done_cv_.wait(lk, pred);
    else if (!done_cv_.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) {
        if (err) *err = "timed out";
        return OSLG_ERR_STATE;
    }
    if (st) *st = r->st;
    int status = r->st.status;
    const uint32_t bits = r->bits;
    reqs_.erase(it);
    delete r;
    if (status != OSLG_OK && err)
        *err = bits ? "request failed: kernel status bits " + std::to_string(bits) : "request failed: " + worker_error_;
    return status;
}

int ShadingServer::poll(uint64_t ticket, bool* done, RequestStats* st, std::string* err) {
    std::lock_guard<std::mutex> lk(mu_);
    auto it = reqs_.find(ticket);
    if (it == reqs_.end()) {
        if (err) *err = "unknown request ticket";
        return OSLG_ERR_ARG;
    }
    Request* r = it->second;
    *done = r->done;
    if (!r->done) return OSLG_OK;
    if (st) *st = r->st;
    int status = r->st.status;
    const uint32_t bits = r->bits;
    reqs_.erase(it);
    delete r;
    if (status != OSLG_OK && err)
        *err = bits ? "request failed: kernel status bits " + std::to_string(bits) : "request failed: " + worker_error_;
    return status;
}

void ShadingServer::stats(ServerStats* s) {
    std::lock_guard<std::mutex> lk(mu_);
    *s = stats_;
    s->pending = (int)pending_.size();
}

}  // namespace oslg
