// Per-group kernel specialization: source generation, nvcc build with a
// content-addressed cubin cache, loading and launch (see oslg_spec.h).
#include "oslg_spec.h"

#include <cuda_runtime.h>
#include <dirent.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <vector>

namespace oslg {

namespace {

bool ok(cudaError_t e, std::string* err, const char* what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ull) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string read_file(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// Hash of every header the generated source includes (so that a changed
// interpreter never reuses a stale cubin).
uint64_t headers_hash(const std::string& csrc) {
    static std::mutex mu;
    static std::string dir;
    static uint64_t h = 0;
    std::lock_guard<std::mutex> lock(mu);
    if (dir == csrc && h) return h;
    std::vector<std::string> names;
    if (DIR* d = opendir(csrc.c_str())) {
        while (dirent* e = readdir(d)) {
            std::string n = e->d_name;
            if (n.size() > 3 && (n.compare(n.size() - 4, 4, ".cuh") == 0 || n.compare(n.size() - 2, 2, ".h") == 0
                                 || n.compare(n.size() - 4, 4, ".inc") == 0))
                names.push_back(n);
        }
        closedir(d);
    }
    std::sort(names.begin(), names.end());
    uint64_t x = 1469598103934665603ull;
    for (const std::string& n : names) x = fnv1a(n + "\n" + read_file(csrc + "/" + n), x);
    x = fnv1a(read_file(csrc + "/../../include/oslg.h"), x);
    dir = csrc;
    h = x;
    return h;
}

const char* kKernelName = "oslg_spec_kernel";
const char* kFlags = "-cubin -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3 -fmad=false";
const char* kBatchFlags = "--split-compile=0";

bool jump_op(uint16_t c) {
    return c == OP_IF || c == OP_ELSE || c == OP_LOOP_TEST || c == OP_JUMP || c == OP_FUNC_BEGIN;
}

uint32_t arg_ncomp(uint32_t a) {
    const uint32_t t = (a >> kArgTCShift) & 7u;
    return t == TC_TRIPLE ? 3u : (t == TC_MATRIX ? 16u : 1u);
}

// Record stride of the output arena when every output op writes inside
// records of one common stride (then a tile's records can be staged in
// shared memory and copied out whole); 0 otherwise.
uint32_t staging_stride(const Op* ops, int n) {
    int64_t stride = -1;
    for (int i = 0; i < n; ++i) {
        const Op& op = ops[i];
        int64_t off, st, size;
        switch (op.code) {
        case OP_STORE_OUTPUT:
            off = op.a[1];
            st = (int32_t)op.a[2];
            size = 4ll * arg_ncomp(op.a[0]) * std::max<uint32_t>(1u, op.a[4]) * ((op.a[3] & 1u) ? 3 : 1);
            break;
        case OP_STORE_CLOSURE:
        case OP_CL_STORE:
            off = op.a[1];
            st = (int32_t)op.a[2];
            size = 4ll * (1 + (int64_t)op.a[3] * kRecordFloats);
            break;
        case OP_BSDF_EVAL:
        case OP_CL_BSDF_EVAL: off = op.a[1]; st = (int32_t)op.a[2]; size = 16; break;
        case OP_BSDF_SAMPLE:
        case OP_CL_BSDF_SAMPLE: off = op.a[1]; st = (int32_t)op.a[2]; size = 44; break;
        default: continue;
        }
        if (st <= 0 || st % 4 || off % 4 || off + size > st || (stride >= 0 && st != stride)) return 0;
        stride = st;
    }
    return stride > 0 && stride <= 512 ? (uint32_t)stride : 0;
}

void put_args(std::ostringstream& o, const uint32_t* a) {
    o << "{";
    for (int i = 0; i < 7; ++i) o << (i ? ", " : "") << a[i] << "u";
    o << "}";
}

}  // namespace

SpecKernel::~SpecKernel() {
    if (library) cudaLibraryUnload(static_cast<cudaLibrary_t>(library));
}

namespace {

struct ProgView {
    const ProgramHeader* h;
    const Op* ops;
    const uint32_t* pool;
    int n;
    bool uses_cl;
    uint32_t sym, cpool;
};

// The lobe kinds (LobeKind bits) the closures of a program can make.
uint32_t lobe_kinds(const ProgView& v) {
    uint32_t m = 0;
    for (int i = 0; i < v.n; ++i)
        if (v.ops[i].code == OP_CLOSURE || v.ops[i].code == OP_CLOSURE_NODE) m |= lobe_kind_bits((int)v.ops[i].a[1]);
    return m;
}

ProgView view(const CompiledGroup& cg) {
    ProgView v;
    v.h = &cg.header;
    v.ops = reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader));
    v.pool = reinterpret_cast<const uint32_t*>(cg.blob.data() + sizeof(ProgramHeader) + (size_t)cg.header.nops * sizeof(Op));
    v.n = (int)cg.header.nops;
    v.uses_cl = (cg.header.flags & 1u) != 0;
    v.sym = v.uses_cl ? cg.header.closure_base : cg.header.heap_slots;
    v.cpool = v.uses_cl ? cg.header.heap_slots - cg.header.closure_base : 0;
    return v;
}

// Loop-free programs execute each closure op at most once per point, so
// the closure walk is at most (ADD ops) deep and finds at most 2^(ADD ops)
// leaves: those bounds replace the reference capacities (16, 8). A static
// consumer finds at most its term count of lobes.
struct Bounds {
    bool fixed = true, any = false;
    int walk = 1, lobes = 1;
};
void add_bounds(Bounds& B, const ProgView& v) {
    bool loops = false;
    int adds = 0;
    for (int i = 0; i < v.n; ++i) {
        loops = loops || v.ops[i].code == OP_LOOP_BEGIN || v.ops[i].code == OP_JUMP;
        // a layer(top, base) closure branches like an ADD: the walk pushes its
        // base, and top and base both hold lobes
        adds += v.ops[i].code == OP_CLOSURE_ADD ||
                (v.ops[i].code == OP_CLOSURE && (int)v.ops[i].a[1] == kIdMxLayer);
        if (v.ops[i].code == OP_CL_BSDF_EVAL || v.ops[i].code == OP_CL_BSDF_SAMPLE || v.ops[i].code == OP_CL_STORE) {
            B.any = true;
            B.lobes = std::max(B.lobes, std::min((int)kBsdfMaxLobes, std::max(1, (int)v.ops[i].a[0])));
        }
    }
    if (!v.uses_cl) return;
    B.any = true;
    if (loops) B.fixed = false;
    B.walk = std::max(B.walk, std::max(1, std::min(adds, (int)kClosureWalkStack)));
    B.lobes = std::max(B.lobes, std::min((int)kBsdfMaxLobes, 1 << std::min(adds, 3)));
}
void emit_bounds(std::ostringstream& o, const Bounds& B) {
    if (!B.any || !B.fixed) return;
    o << "#define OSLG_FIXED_INDEX 1\n";
    o << "#define OSLG_WALK_STACK " << B.walk << "\n";
    o << "#define OSLG_LOBES_MAX " << B.lobes << "\n";
}

// The constant pool and the op sequence of one program as
// spec_body<sfx>(R, L, npoints).
void emit_body(std::ostringstream& o, const ProgView& v, const std::string& sfx) {
    const int n = v.n;
    const Op* ops = v.ops;
    std::vector<char> target(n + 1, 0);
    for (int i = 0; i < n; ++i)
        if (jump_op(ops[i].code) && ops[i].a[2] <= (uint32_t)n) target[ops[i].a[2]] = 1;
    o << "__constant__ const uint32_t kPool" << sfx << "[" << std::max(1u, v.h->nconst) << "] = {";
    for (uint32_t i = 0; i < v.h->nconst; ++i) o << (i ? ", " : "") << v.pool[i] << "u";
    if (!v.h->nconst) o << "0u";
    o << "};\n\n";
    o << "__device__ __forceinline__ void spec_body" << sfx << "(const RunCtx& R, Lane& L, int64_t npoints) {\n";
    o << "    Ctl<1> C;\n    ctl_init<1>(C, R, L, npoints);\n";
    o << "    const uint32_t li0 = L.li;\n    (void)li0;\n";
    for (int i = 0; i < n; ++i) {
        const Op& op = ops[i];
        if (target[i]) o << "op_" << i << ":;\n";
        const uint32_t* a = op.a;
        auto dst = [&](uint32_t t) { return "op_" + std::to_string(std::min<uint32_t>(t, (uint32_t)n)); };
        o << "    {  // " << i << ": code " << op.code << "\n        const uint32_t a[7] = ";
        put_args(o, a);
        o << ";\n";
        switch (op.code) {
        case OP_NOP: o << "        (void)a;\n"; break;
        case OP_IF: o << "        if (ctl_if<1>(C, L, li0, a)) goto " << dst(a[2]) << ";\n"; break;
        case OP_ELSE: o << "        if (ctl_else<1>(C, a)) goto " << dst(a[2]) << ";\n"; break;
        case OP_ENDIF: o << "        ctl_endif<1>(C, a);\n"; break;
        case OP_LOOP_BEGIN: o << "        ctl_loop_begin<1>(C, a);\n"; break;
        case OP_LOOP_TEST: o << "        if (ctl_loop_test<1>(C, L, li0, a)) goto " << dst(a[2]) << ";\n"; break;
        case OP_LOOP_STEP: o << "        ctl_loop_step<1>(C, a);\n"; break;
        case OP_JUMP:
            o << "        (void)a;\n";
            if (a[2] <= (uint32_t)i)  // a loop's back edge
                o << "        if (ctl_back_edge<1>(C, R, " << max_loop_iterations(*v.h) << "u)) goto op_" << n << ";\n";
            o << "        goto " << dst(a[2]) << ";\n";
            break;
        case OP_LOOP_END: o << "        ctl_loop_end<1>(C, a);\n"; break;
        case OP_BREAK: o << "        ctl_break<1>(C, a);\n"; break;
        case OP_CONTINUE: o << "        ctl_continue<1>(C, a);\n"; break;
        case OP_RETURN: o << "        (void)a;\n        ctl_return<1>(C);\n"; break;
        case OP_EXIT: o << "        (void)a;\n        ctl_exit<1>(C);\n"; break;
        case OP_LAYER_END: o << "        (void)a;\n        ctl_layer_end<1>(C);\n"; break;
        case OP_STORES_END: o << "        ctl_stores_end<1>(C, a);\n"; break;
        case OP_FUNC_BEGIN: o << "        if (ctl_func_begin<1>(C, a)) goto " << dst(a[2]) << ";\n"; break;
        case OP_FUNC_RETURN: o << "        ctl_func_return<1>(C, a);\n"; break;
        case OP_FUNC_END: o << "        ctl_func_end<1>(C, a);\n"; break;
        default:
            if (i + 1 < n) {
                // the next op, or every OP_NOP carrier that follows (operand
                // lists and term tables), as a literal array
                int k = 1;
                while (i + k < n && k < 9 && ops[i + k].code == OP_NOP) ++k;
                if (k > 1) --k;
                o << "        const Op nx[" << k << "] = {";
                for (int j = 1; j <= k; ++j) {
                    const Op& x = ops[i + j];
                    o << (j > 1 ? ", " : "") << "{" << x.code << ", " << (unsigned)x.nargs << ", " << (unsigned)x.flags
                      << ", ";
                    put_args(o, x.a);
                    o << "}";
                }
                o << "};\n        if (C.actm) exec_op_c<7, " << op.code << "u>(R, L, a, nx);\n";
            } else {
                o << "        if (C.actm) exec_op_c<7, " << op.code << "u>(R, L, a, nullptr);\n";
            }
            break;
        }
        o << "    }\n";
    }
    o << "op_" << n << ":;\n}\n\n";
}

// R/L set-up of one program and its body, for tile L.pt.
// Batch kernels keep each program's body a separate function (built in
// parallel by nvcc --split-compile, register allocation per program).
void emit_job(std::ostringstream& o, const ProgView& v, const std::string& sfx) {
    o << "__device__ __noinline__ void spec_job" << sfx << "(RunCtx& R, Lane& L, int64_t npoints) {\n";
    o << "    R.nops = " << v.n << ";\n";
    o << "    R.CP.base = " << v.h->closure_base << "u;\n    R.CP.max_nodes = " << v.h->max_comps << "u;\n";
    o << "    R.CP.nf = " << node_floats(*v.h) << "u;\n";
    o << "    R.uses_closures = " << (v.uses_cl ? "true" : "false") << ";\n";
    o << "    float hreg[" << std::max(1u, v.sym) << "];\n";
    o << "    L.heap = hreg;\n    L.pool = kPool" << sfx << ";\n    L.cbase = " << v.h->closure_base << "u;\n";
    o << "    spec_body" << sfx << "(R, L, npoints);\n}\n\n";
}

}  // namespace

std::string spec_source(const CompiledGroup& cg, int min_blocks) {
    const ProgView v = view(cg);
    const int n = v.n;
    const uint32_t sym = v.sym, cpool = v.cpool;
    const bool uses_cl = v.uses_cl;
    const ProgramHeader& h = cg.header;
    Bounds B;
    add_bounds(B, v);
    const uint32_t stage = staging_stride(v.ops, n);
    std::ostringstream o;
    o << "// generated: kernel specialized to one lowered program (" << n << " ops, " << sym
      << " symbol slots, " << cpool << " closure-pool slots)\n";
    o << "#define OSLG_SPEC 1\n";
    o << "#define OSLG_LOBE_KINDS 0x" << std::hex << lobe_kinds(v) << std::dec << "u\n";
    if (stage) o << "#define OSLG_STAGE_STRIDE " << stage << "\n";
    emit_bounds(o, B);
    o << "#include \"oslg_interp.cuh\"\n\nnamespace {\n";
    o << "using namespace oslg;\nusing namespace oslg::dev;\n\n";
    emit_body(o, v, "");
    if (stage) {
        // the tile's copy-out is a call of its own, so that the shading
        // body's register allocation does not depend on it
        o << "__device__ __noinline__ void spec_copy_out(const KArgs& k, const unsigned char* smem, int64_t tile, "
             "int fill_unwritten) {\n";
        o << "        const size_t rec = " << stage << "u;\n";
        o << "        const unsigned char* flags = smem + (size_t)blockDim.x * rec;\n";
        o << "    const int64_t npt = k.npoints - tile * blockDim.x < (int64_t)blockDim.x ? k.npoints - tile * "
             "blockDim.x : (int64_t)blockDim.x;\n";
        o << "    uint32_t* gout = reinterpret_cast<uint32_t*>(k.outputs + tile * blockDim.x * (int64_t)rec);\n";
        o << "    const uint32_t* sw = reinterpret_cast<const uint32_t*>(smem);\n";
        o << "    if (!k.shadeindex) {\n";
        o << "        for (int64_t w = threadIdx.x; w < npt * (int64_t)(rec / 4u); w += blockDim.x)\n";
        o << "            if (flags[w]) gout[w] = sw[w];\n";
        o << "            else if (fill_unwritten) gout[w] = 0u;\n";
        o << "    } else {  // each point's record goes to its shadeindex\n";
        // 32-bit word indices (a tile is at most 256 records): division by
        // the constant record size stays cheap and adds no register pressure
        o << "        const int32_t* si = k.shadeindex + tile * blockDim.x;\n";
        o << "        const uint32_t nw = (uint32_t)npt * (uint32_t)(rec / 4u);\n";
        o << "        for (uint32_t w = threadIdx.x; w < nw; w += blockDim.x) {\n";
        o << "            const uint32_t p = w / (uint32_t)(rec / 4u), q = w - p * (uint32_t)(rec / 4u);\n";
        o << "            uint32_t* dst = reinterpret_cast<uint32_t*>(k.outputs + (int64_t)__ldg(si + p) * (int64_t)rec) + q;\n";
        o << "            if (flags[w]) *dst = sw[w];\n";
        o << "            else if (fill_unwritten) *dst = 0u;\n";
        o << "        }\n";
        o << "    }\n";
        o << "}\n";
    }
    o << "}  // namespace\n\n";
    // registers per thread are capped at 65536 / (256 * min_blocks); by
    // default 48 for closure programs (latency-bound: more resident warps;
    // 0.279 ms against 0.297 ms at 64 on the layered-closure workload) and
    // 85 otherwise (the fBm workload)
    if (min_blocks <= 0) min_blocks = B.any ? 5 : 3;
    o << "extern \"C\" __global__ void __launch_bounds__(256, " << std::max(2, std::min(8, min_blocks)) << ") "
      << kKernelName
      << "(const __grid_constant__ oslg::dev::KArgs k, int pool_in_smem, int fill_unwritten) {\n";
    o << "    using namespace oslg;\n    using namespace oslg::dev;\n";
    if (stage) o << "    unsigned char* smem = oslg_smem;\n";
    else o << "    extern __shared__ __align__(16) unsigned char smem[];\n";
    o << "    RunCtx R;\n    R.sops = nullptr;\n    R.nops = " << n << ";\n";
    o << "    R.CP.base = " << h.closure_base << "u;\n    R.CP.max_nodes = " << h.max_comps << "u;\n";
    o << "    R.CP.nf = " << node_floats(h) << "u;\n";
    o << "    R.uses_closures = " << (uses_cl ? "true" : "false") << ";\n";
    o << "    R.G = &k.G;\n    R.userdata = k.userdata;\n    R.outputs = k.outputs;\n    R.status = k.status;\n";
    o << "    R.textures = k.textures;\n    R.ntextures = k.ntextures;\n";
    o << "    R.symheap = k.symheap;\n    R.symheap_stride = k.symheap_stride;\n";
    o << "    float hreg[" << std::max(1u, sym) << "];\n";
    o << "    Lane L;\n    L.heap = hreg;\n    L.pool = kPool;\n    L.hs = 1;\n    L.li = 0;\n    L.pt = 0;\n";
    o << "    L.si = k.shadeindex;\n";
    // dynamic shared memory: [staged records | written flags] then the closure pools
    o << "    const size_t stage_bytes = " << (stage ? "(size_t)blockDim.x * " + std::to_string(stage) + "u * 5u / 4u"
                                                    : std::string("0")) << ";\n";
    o << "    L.cheap = pool_in_smem ? reinterpret_cast<float*>(smem + stage_bytes) : k.gheap + (size_t)blockIdx.x * "
      << std::max(1u, cpool) << "u * blockDim.x;\n";
    o << "    L.chs = blockDim.x;\n    L.cli = threadIdx.x;\n    L.cbase = " << h.closure_base << "u;\n";
    o << "    const int64_t ntiles = (k.npoints + blockDim.x - 1) / blockDim.x;\n";
    o << "    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {\n";
    if (stage) {
        o << "        const size_t rec = " << stage << "u;\n";
        o << "        unsigned char* flags = smem + (size_t)blockDim.x * rec;\n";
        // one flag byte per staged word: blockDim * rec / 4 bytes, cleared as uint4
        o << "        for (size_t i = threadIdx.x; i < (size_t)blockDim.x * rec / 64u; i += blockDim.x)\n";
        o << "            reinterpret_cast<uint4*>(flags)[i] = make_uint4(0u, 0u, 0u, 0u);\n";
        o << "        __syncthreads();\n";
        o << "        R.outputs = reinterpret_cast<char*>(smem) - (ptrdiff_t)(tile * blockDim.x) * (ptrdiff_t)rec;\n";
    }
    o << "        L.pt = tile * blockDim.x + threadIdx.x;\n        spec_body(R, L, k.npoints);\n";
    if (stage) {
        o << "        __syncthreads();\n";
        o << "        spec_copy_out(k, smem, tile, fill_unwritten);\n";
        o << "        __syncthreads();\n";
    }
    o << "    }\n}\n";
    return o.str();
}

SpecBatchKernel::~SpecBatchKernel() {
    if (library) cudaLibraryUnload(static_cast<cudaLibrary_t>(library));
}

void canonical_cases(std::vector<const CompiledGroup*>& cases) {
    std::sort(cases.begin(), cases.end());
    cases.erase(std::unique(cases.begin(), cases.end()), cases.end());
    auto key = [](const CompiledGroup* cg) {
        return std::make_pair(fnv1a(std::string(cg->blob.begin(), cg->blob.end())), cg->blob.size());
    };
    std::stable_sort(cases.begin(), cases.end(),
                     [&](const CompiledGroup* a, const CompiledGroup* b) { return key(a) < key(b); });
}

std::string spec_batch_source(const std::vector<const CompiledGroup*>& cases) {
    Bounds B;
    std::vector<ProgView> vs;
    for (const CompiledGroup* cg : cases) {
        vs.push_back(view(*cg));
        add_bounds(B, vs.back());
    }
    std::ostringstream o;
    o << "// generated: persistent batch kernel specialized to " << cases.size() << " lowered programs\n";
    o << "#define OSLG_SPEC 1\n#define OSLG_SPEC_BATCH 1\n";
    uint32_t kinds = 0;
    for (const ProgView& pv : vs) kinds |= lobe_kinds(pv);
    o << "#define OSLG_LOBE_KINDS 0x" << std::hex << kinds << std::dec << "u\n";
    emit_bounds(o, B);
    o << "#include \"oslg_interp.cuh\"\n\nnamespace {\n";
    o << "using namespace oslg;\nusing namespace oslg::dev;\n\n";
    for (size_t j = 0; j < vs.size(); ++j) {
        emit_body(o, vs[j], "_" + std::to_string(j));
        emit_job(o, vs[j], "_" + std::to_string(j));
    }
    o << "}  // namespace\n\n";
    // up to 128 registers: the material bodies spill under tighter caps
    o << "extern \"C\" __global__ void __launch_bounds__(256, 2) oslg_specbatch_kernel("
         "const __grid_constant__ oslg::dev::BatchArgs b, int pool_in_smem) {\n";
    o << "    using namespace oslg;\n    using namespace oslg::dev;\n";
    o << "    extern __shared__ __align__(16) unsigned char smem[];\n";
    o << "    __shared__ uint32_t s_item;\n";
    o << "    const uint32_t nitems = b.nitems_dev ? *b.nitems_dev : b.nitems;\n";
    o << "    Lane L;\n    L.hs = 1;\n    L.li = 0;\n    L.chs = blockDim.x;\n    L.cli = threadIdx.x;\n";
    o << "    L.cheap = pool_in_smem ? reinterpret_cast<float*>(smem) : b.gheap + (size_t)blockIdx.x * b.heap_slots * "
         "blockDim.x;\n";
    o << "    RunCtx R;\n    R.sops = nullptr;\n    R.status = b.status;\n";
    o << "    R.textures = b.textures;\n    R.ntextures = b.ntextures;\n";
    o << "    for (;;) {\n";
    o << "        if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1u);\n";
    o << "        __syncthreads();\n        const uint32_t it = s_item;\n        __syncthreads();\n";
    o << "        if (it >= nitems) break;\n";
    o << "        const uint2 w = b.items[it];\n        const BatchJob* J = b.jobs + w.x;\n";
    o << "        R.G = &J->G;\n        R.userdata = J->userdata;\n        R.outputs = J->outputs;\n";
    o << "        R.status = J->status ? J->status : b.status;\n";
    o << "        L.pt = (int64_t)w.y * blockDim.x + threadIdx.x;\n";
    o << "        const int64_t np = J->npoints;\n";
    o << "        switch (J->spec_case) {\n";
    for (size_t j = 0; j < vs.size(); ++j)
        o << "        case " << j << ": spec_job_" << j << "(R, L, np); break;\n";
    o << "        default: if (threadIdx.x == 0) raise_status(b.status, ST_BAD_OPCODE); break;\n";
    o << "        }\n    }\n}\n";
    return o.str();
}

namespace {
// nvcc the source into the cache (once per content hash) and load `kname`.
int build_and_load(const std::string& src, const std::string& csrc, const std::string& cache, const char* kname,
                   const char* extra_flags, void** lib_out, void** kern_out, std::string* key_out, std::string* err);
}  // namespace

int spec_batch_build(const std::vector<const CompiledGroup*>& cases, const std::string& csrc,
                     const std::string& cache, SpecBatchKernel* out, std::string* err) {
    int rc = build_and_load(spec_batch_source(cases), csrc, cache, "oslg_specbatch_kernel", kBatchFlags,
                            &out->library, &out->kernel, &out->key, err);
    if (rc != OSLG_OK) return rc;
    out->cases = (int)cases.size();
    out->pool_slots = 0;
    for (const CompiledGroup* cg : cases) out->pool_slots = std::max(out->pool_slots, view(*cg).cpool);
    return OSLG_OK;
}

int spec_build(const CompiledGroup& cg, const std::string& csrc, const std::string& cache, SpecKernel* out,
               std::string* err, int min_blocks) {
    int rc = build_and_load(spec_source(cg, min_blocks), csrc, cache, kKernelName, "", &out->library, &out->kernel,
                            &out->key, err);
    if (rc != OSLG_OK) return rc;
    const bool uses_cl = (cg.header.flags & 1u) != 0;
    out->sym_slots = uses_cl ? cg.header.closure_base : cg.header.heap_slots;
    out->pool_slots = uses_cl ? cg.header.heap_slots - cg.header.closure_base : 0;
    out->stage_stride = staging_stride(reinterpret_cast<const Op*>(cg.blob.data() + sizeof(ProgramHeader)),
                                       (int)cg.header.nops);
    return OSLG_OK;
}

namespace {
int build_and_load(const std::string& src, const std::string& csrc, const std::string& cache, const char* kname,
                   const char* extra_flags, void** lib_out, void** kern_out, std::string* key_out, std::string* err) {
    const std::string flags = std::string(kFlags) + " " + extra_flags;
    const uint64_t key = fnv1a(flags + "\n" + src, headers_hash(csrc));
    char hex[17];
    snprintf(hex, sizeof(hex), "%016llx", (unsigned long long)key);
    const std::string base = cache + "/spec_" + hex;
    const std::string cubin = base + ".cubin";
    struct stat stt;
    if (stat(cubin.c_str(), &stt) != 0) {
        mkdir(cache.c_str(), 0755);
        const std::string cu = base + ".cu";
        {
            std::ofstream f(cu, std::ios::binary);
            f << src;
        }
        const char* ch = getenv("CUDA_HOME");
        const std::string nvcc = std::string(ch && *ch ? ch : "/usr/local/cuda") + "/bin/nvcc";
        const std::string tmp = base + "." + std::to_string((long long)getpid()) + ".tmp";
        const std::string cmd = nvcc + " " + flags + " -I" + csrc + " -o " + tmp + " " + cu + " > " + base +
                                ".log 2>&1";
        const int rc = std::system(cmd.c_str());
        if (rc != 0 || stat(tmp.c_str(), &stt) != 0) {
            if (err) *err = "specialized kernel build failed (" + cmd + "): " + read_file(base + ".log").substr(0, 2000);
            return OSLG_ERR_LOWER;
        }
        if (std::rename(tmp.c_str(), cubin.c_str()) != 0) {
            if (err) *err = "cannot place " + cubin;
            return OSLG_ERR_LOWER;
        }
    }
    cudaLibrary_t lib = nullptr;
    if (!ok(cudaLibraryLoadFromFile(&lib, cubin.c_str(), nullptr, nullptr, 0, nullptr, nullptr, 0), err,
            "load specialized kernel"))
        return OSLG_ERR_CUDA;
    cudaKernel_t kern = nullptr;
    if (!ok(cudaLibraryGetKernel(&kern, lib, kname), err, "specialized kernel lookup")) {
        cudaLibraryUnload(lib);
        return OSLG_ERR_CUDA;
    }
    *lib_out = lib;
    *kern_out = kern;
    *key_out = hex;
    return OSLG_OK;
}
}  // namespace

int spec_launch(DeviceState& ds, const SpecKernel& sk, const CompiledGroup& cg, int64_t npoints,
                const oslg_shaderglobals& G, void* userdata, void* outputs, void* stream, std::string* err,
                int block_req, int pool_req, bool fill_unwritten, const LaunchExtras* ex) {
    if (npoints <= 0) return OSLG_OK;
    int rc = device_init(ds, err);
    if (rc != OSLG_OK) return rc;
    const void* fn = reinterpret_cast<const void*>(sk.kernel);
    // measured on the layered-closure workload: with staged output records,
    // 128-thread CTAs and closure pools in HBM scratch (L2-resident) keep the
    // most warps resident; without staging, 256 threads with the pools in
    // shared memory
    if (block_req == 0 && sk.stage_stride) block_req = 128;
    if (pool_req < 0 && sk.stage_stride) pool_req = 0;
    const int block = block_req == 128 || block_req == 64 ? block_req : 256;
    const size_t pool_bytes = (size_t)sk.pool_slots * block * sizeof(float);
    const size_t stage_bytes = (size_t)block * sk.stage_stride * 5 / 4;
    // closure pools in shared memory when they fit beside the staged records
    // in 100 KiB (two CTAs per SM), else in HBM scratch
    int in_smem = pool_bytes > 0 && stage_bytes + pool_bytes <= 100 * 1024 ? 1 : 0;
    if (pool_req == 0) in_smem = 0;
    if (pool_req == 1 && pool_bytes > 0 && stage_bytes + pool_bytes + 1024 <= ds.smem_optin) in_smem = 1;
    const size_t shmem = stage_bytes + (in_smem ? pool_bytes : 0);
    if (shmem > 48 * 1024 &&
        !ok(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmem), err,
            "specialized kernel attribute"))
        return OSLG_ERR_CUDA;
    const int64_t ntiles = (npoints + block - 1) / block;
    int64_t grid = ntiles;
    dev::KArgs k;
    k.blob = static_cast<const uint8_t*>(cg.d_blob);
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
    if (sk.pool_slots > 0 && !in_smem) {
        int per_sm = 0;
        if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0), err, "occupancy"))
            return OSLG_ERR_CUDA;
        grid = std::min<int64_t>(ntiles, (int64_t)ds.sm_count * std::max(1, per_sm));
        const size_t need = (size_t)grid * pool_bytes;
        if (need > ds.gheap_bytes) {
            if (ds.gheap) cudaFree(ds.gheap);
            ds.gheap = nullptr;
            ds.gheap_bytes = 0;
            if (!ok(cudaMalloc(&ds.gheap, need), err, "cudaMalloc heap")) return OSLG_ERR_CUDA;
            ds.gheap_bytes = need;
        }
        k.gheap = ds.gheap;
    }
    grid = std::min<int64_t>(grid, 0x7FFFFFFF);
    int fill = fill_unwritten ? 1 : 0;
    void* args[] = { &k, &in_smem, &fill };
    if (!ok(cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(block), args, shmem, static_cast<cudaStream_t>(stream)),
            err, "specialized kernel launch"))
        return OSLG_ERR_CUDA;
    return OSLG_OK;
}

}  // namespace oslg
