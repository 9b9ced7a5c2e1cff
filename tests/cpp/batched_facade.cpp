// The C++ facade (include/oslg.hpp) used the way a renderer uses the
// reference's batched API: build a group, add symlocs, then
// batched<W>().execute over W-lane BatchedShaderGlobals (ragged batches
// leave the other lanes' records untouched), and the N-point overload over
// device SoA planes. Mode "lower" stops after optimize_group (no GPU).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "oslg.hpp"

static const char* kProbe =
    "OpenShadingLanguage 1.00\n"
    "shader facade_probe\n"
    "oparam\tfloat\to\t0\n"
    "oparam\tcolor\tc\t0\t0\t0\n"
    "global\tfloat\tu\n"
    "global\tfloat\tv\n"
    "temp\tfloat\t$tmp1\n"
    "const\tfloat\t$const1\t2\n"
    "temp\tfloat\t$tmp2\n"
    "code ___main___\n"
    "\tmul\t$tmp1\tu\t$const1\n"
    "\tadd\to\t$tmp1\tv\n"
    "\tmul\t$tmp2\tu\tv\n"
    "\tcolor\tc\tu\tv\t$tmp2\n"
    "\tend\n";

struct Record {
    float o;
    float c[3];
};

static int failures = 0;
#define CHECK(cond)                                                        \
    do {                                                                   \
        if (!(cond)) {                                                     \
            std::fprintf(stderr, "check failed line %d: %s\n", __LINE__, #cond); \
            ++failures;                                                    \
        }                                                                  \
    } while (0)

static bool expect(const Record& r, float u, float v) {
    const float o = u * 2.0f + v;
    return r.o == o && r.c[0] == u && r.c[1] == v && r.c[2] == u * v;
}

template <int W> static void run_width(oslg::ShadingSystem& ss, oslg::ShaderGroupRef g, int batch_size) {
    oslg::BatchedShaderGlobals<W> bsg;
    std::memset(&bsg.varying, 0, sizeof(bsg.varying));
    for (int lane = 0; lane < W; ++lane) {
        bsg.varying.u.set(lane, 0.125f * (float)lane + 0.01f);
        bsg.varying.v.set(lane, 1.0f - 0.0625f * (float)lane);
    }
    std::vector<Record> out(W, Record{ -7.0f, { -7.0f, -7.0f, -7.0f } });
    CHECK(ss.batched<W>().execute(g, batch_size, bsg, nullptr, out.data()));
    for (int lane = 0; lane < W; ++lane) {
        if (lane < batch_size) CHECK(expect(out[lane], bsg.varying.u.get(lane), bsg.varying.v.get(lane)));
        else CHECK(out[lane].o == -7.0f && out[lane].c[2] == -7.0f);  // lanes past batch_size untouched
    }
}

// the reference's signature: context + wide_shadeindex; lane i's record is
// shadeindex[i] (reversed, with one record never addressed)
template <int W> static void run_width_indexed(oslg::ShadingSystem& ss, oslg::ShaderGroupRef g, int batch_size) {
    oslg::BatchedShaderGlobals<W> bsg;
    std::memset(&bsg.varying, 0, sizeof(bsg.varying));
    oslg::Block<int, W> si;
    for (int lane = 0; lane < W; ++lane) {
        bsg.varying.u.set(lane, 0.25f * (float)lane + 0.03f);
        bsg.varying.v.set(lane, 0.5f - 0.125f * (float)lane);
        si.set(lane, batch_size - lane);  // records batch_size .. 1; record 0 untouched
    }
    std::vector<Record> out(W + 1, Record{ -7.0f, { -7.0f, -7.0f, -7.0f } });
    oslg::ShadingSystem::ShadingContext* ctx = ss.get_context();
    CHECK(ss.batched<W>().execute(*ctx, g, batch_size, si, bsg, nullptr, out.data()));
    ss.release_context(ctx);
    CHECK(out[0].o == -7.0f);
    for (int lane = 0; lane < batch_size; ++lane)
        CHECK(expect(out[(size_t)si.get(lane)], bsg.varying.u.get(lane), bsg.varying.v.get(lane)));
}

int main(int argc, char** argv) {
    const bool lower_only = argc > 1 && std::strcmp(argv[1], "lower") == 0;
    oslg::ShadingSystem ss;
    CHECK(ss.LoadMemoryCompiledShader("facade_probe", kProbe));
    oslg::ShaderGroupRef g = ss.ShaderGroupBegin("facade");
    CHECK(g != nullptr);
    CHECK(ss.Shader(g, "surface", "facade_probe", "L"));
    CHECK(ss.ShaderGroupEnd(g));
    const oslg_typedesc tf = { OSLG_BASE_FLOAT, OSLG_AGG_SCALAR, 0, 0 };
    const oslg_typedesc tc = { OSLG_BASE_FLOAT, OSLG_AGG_VEC3, OSLG_VEC_COLOR, 0 };
    CHECK(ss.add_symlocs(g, { { "L.o", tf, 0, OSLG_ARENA_OUTPUTS, 0, (int64_t)sizeof(Record) },
                              { "L.c", tc, 0, OSLG_ARENA_OUTPUTS, 4, (int64_t)sizeof(Record) } }));
    CHECK(ss.optimize_group(g));
    // a batch wider than W is refused with a message
    oslg::BatchedShaderGlobals<4> small;
    CHECK(!ss.batched<4>().execute(g, 5, small, nullptr, nullptr));
    CHECK(!ss.geterror().empty());
    if (lower_only) {
        std::printf("%s\n", failures ? "FAILED" : "lowered");
        return failures ? 1 : 0;
    }
    run_width<16>(ss, g, 16);
    run_width<16>(ss, g, 13);
    run_width<8>(ss, g, 5);
    run_width<4>(ss, g, 4);
    run_width_indexed<8>(ss, g, 8);
    run_width_indexed<16>(ss, g, 11);
    // N points on the device
    const int n = 100003;
    std::vector<float> hu(n), hv(n);
    for (int i = 0; i < n; ++i) {
        hu[i] = (float)i / (float)n;
        hv[i] = 0.5f + (float)(i % 97) * 0.001f;
    }
    float *du = nullptr, *dv = nullptr;
    Record* dout = nullptr;
    CHECK(cudaMalloc(&du, n * 4) == cudaSuccess && cudaMalloc(&dv, n * 4) == cudaSuccess &&
          cudaMalloc(&dout, n * sizeof(Record)) == cudaSuccess);
    cudaMemcpy(du, hu.data(), n * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(dv, hv.data(), n * 4, cudaMemcpyHostToDevice);
    oslg_shaderglobals sg = {};
    sg.u.data = du;
    sg.u.plane_stride = n;
    sg.v.data = dv;
    sg.v.plane_stride = n;
    CHECK(ss.batched<16>().execute(g, (int64_t)n, sg, nullptr, dout));
    std::vector<Record> out(n);
    cudaMemcpy(out.data(), dout, n * sizeof(Record), cudaMemcpyDeviceToHost);
    int bad = 0;
    for (int i = 0; i < n; ++i) bad += expect(out[i], hu[i], hv[i]) ? 0 : 1;
    CHECK(bad == 0);
    // the same points with a device shadeindex: point i's record is n-1-i
    std::vector<int32_t> hsi(n);
    for (int i = 0; i < n; ++i) hsi[i] = n - 1 - i;
    int32_t* dsi = nullptr;
    CHECK(cudaMalloc(&dsi, n * 4) == cudaSuccess);
    cudaMemcpy(dsi, hsi.data(), n * 4, cudaMemcpyHostToDevice);
    CHECK(ss.batched<16>().execute(g, (int64_t)n, sg, dsi, nullptr, dout, nullptr));
    cudaMemcpy(out.data(), dout, n * sizeof(Record), cudaMemcpyDeviceToHost);
    bad = 0;
    for (int i = 0; i < n; ++i) bad += expect(out[(size_t)hsi[i]], hu[i], hv[i]) ? 0 : 1;
    CHECK(bad == 0);
    cudaFree(dsi);
    cudaFree(du);
    cudaFree(dv);
    cudaFree(dout);
    std::printf("%s\n", failures ? "FAILED" : "ok");
    return failures ? 1 : 0;
}
