// Shading server: continuous batching of shading requests on one GPU.
//
// Requests (group, point count, host-side BatchedShaderGlobals, host output
// buffer) arrive from any thread. A worker thread admits waiting requests
// into "waves" as device memory and stream slots free up: it copies each
// request's inputs into a device arena (admission is against an HBM
// budget), runs the whole wave in one persistent batch-kernel launch and
// copies the outputs back; a host callback stamps completion. Several
// waves are in flight on separate streams, so requests that arrive while
// others run are admitted and overlap on the device. Compiled programs stay
// resident. The reference has no serving layer: renderers call execute()
// per batch (src/liboslexec/shadingsys.cpp:329-394).
#pragma once
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "oslg_batch.h"
#include "oslg_spec.h"

#include <memory>

namespace oslg {

// First-fit allocator over one device allocation, 256-byte granules,
// neighbouring free ranges merged on release.
class DeviceArena {
public:
    int init(size_t bytes, std::string* err);
    void release();
    bool alloc(size_t bytes, size_t* off);
    void free(size_t off, size_t bytes);
    char* base() const { return base_; }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }
    static size_t round(size_t b) { return (b + 255) & ~size_t(255); }

private:
    char* base_ = nullptr;
    size_t cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;  // offset -> size
};

struct ServerOptions {
    size_t budget_bytes = size_t(40) << 30;  // programs + arena + scratch heaps
    int streams = 3;                        // waves in flight
    int block = 512;
    int points_per_thread = 1;
    int64_t max_wave_points = 8 << 20;
    int max_wave_requests = 512;
    size_t arena_bytes = 0;  // request memory; 0: what the budget leaves after the scratch heaps
    // waves run one persistent kernel specialized to the resident programs
    // (built when the set of programs changes) when these name the
    // interpreter headers and the kernel cache; empty: the interpreter
    std::string jit_csrc, jit_cache;
};

struct RequestStats {
    int64_t submit_ns = 0, admit_ns = 0, done_ns = 0;
    int wave = -1;
    int status = 0;  // 0 ok, else an OSLG_ERR_* code
};

struct ServerStats {
    uint64_t submitted = 0, completed = 0, failed = 0, waves = 0;
    int64_t points_done = 0;
    size_t arena_capacity = 0, arena_high_water = 0, program_bytes = 0, scratch_bytes = 0;
    int in_flight_waves = 0, pending = 0;
};

class ShadingServer {
public:
    ShadingServer(DeviceState& ds, const ServerOptions& o) : ds_(ds), opt_(o) {}
    ~ShadingServer();
    int start(std::string* err);
    // Make a lowered, uploaded program resident (counts against the budget).
    int register_program(const CompiledGroup& cg, std::string* err);
    int submit(const CompiledGroup& cg, int64_t npoints, const oslg_shaderglobals& host_globals, void* host_output,
               size_t output_bytes, uint64_t* ticket, std::string* err);
    // Wait (timeout_ms < 0: forever) for a request; a finished request's
    // record is released when wait or poll reports it done.
    int wait(uint64_t ticket, int timeout_ms, RequestStats* st, std::string* err);
    int poll(uint64_t ticket, bool* done, RequestStats* st, std::string* err);
    void stats(ServerStats* s);
    void stop();

private:
    struct Request {
        uint64_t id = 0;
        const CompiledGroup* cg = nullptr;
        int64_t n = 0;
        oslg_shaderglobals hG{}, dG{};
        void* host_out = nullptr;
        size_t out_bytes = 0, in_bytes = 0;
        size_t dev_off = 0, dev_bytes = 0;
        RequestStats st;
        bool done = false;
        int job = 0;          // index of its job in the wave's launch
        uint32_t bits = 0;    // kernel status bits its job raised
    };
    struct Slot {
        void* stream = nullptr;
        dev::BatchJob* d_jobs = nullptr;
        uint2* d_items = nullptr;
        uint32_t* d_counter = nullptr;
        float* d_heap = nullptr;
        size_t heap_bytes = 0;
        dev::BatchJob* h_jobs = nullptr;  // pinned staging
        uint2* h_items = nullptr;
        uint32_t* d_status = nullptr;  // one status word per job of the wave
        uint32_t* h_status = nullptr;  // pinned copy, read by the completion callback
        size_t items_cap = 0;
        std::vector<Request*> reqs;
        bool busy = false;
        bool complete = false;
        int wave = -1;
        ShadingServer* owner = nullptr;
    };
    static void on_wave_done(void* slot);
    int start_resources(std::string* err);
    void release_resources();
    void worker();
    int launch_wave(Slot& s, std::vector<Request*>& wave, std::string* err);
    size_t request_device_bytes(const Request& r) const;

    DeviceState& ds_;
    ServerOptions opt_;
    DeviceArena arena_;
    std::vector<Slot> slots_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<Request*> pending_;
    std::unordered_map<uint64_t, Request*> reqs_;
    std::unordered_map<const CompiledGroup*, uint32_t> programs_;  // resident program -> heap slots
    std::thread thread_;
    bool running_ = false, stopping_ = false;
    uint64_t next_id_ = 1;
    int next_wave_ = 0;
    uint32_t heap_slots_ = 0;     // largest heap of any resident program
    uint32_t prog_bytes_ = 0;     // largest program (shared-memory staging)
    int grid_ = 0, per_sm_ = 0;
    size_t shmem_ = 0;
    // specialized waves: the kernel for spec_cases_ (every kernel built stays
    // loaded until the server stops: waves in flight may use an older one)
    int ensure_spec(std::string* err);
    std::vector<std::unique_ptr<SpecBatchKernel>> spec_kernels_;
    std::vector<const CompiledGroup*> spec_cases_;
    int spec_grid_ = 0;
    ServerStats stats_{};
    std::string worker_error_;
};

}  // namespace oslg
