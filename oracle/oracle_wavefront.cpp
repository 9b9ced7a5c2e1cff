// ORACLE (test infrastructure only): CPU restatement of the wavefront path
// tracer. Used by the tests and by the CPU-baseline leg of the benchmark as
// the checker; nothing in the product links it.
//
// Each sampled path follows testrender's loop
// (src/testrender/simpleraytracer.cpp:960-1184): trace, build the shader
// globals from the hit (:890-932), shade, add emission, prepare the BSDF
// with the path weight and sample it, continue. Shading is batched the way
// the reference's batched executor runs it: per bounce, the hits of each
// material are one oracle_run() over SoA globals. Intersection scans every
// primitive in id order (no acceleration structure) with the nearest hit
// and, on equal distance, the lower id winning. All float arithmetic is
// single IEEE operations in a fixed order (built with -ffp-contract=off).
//
// Differences from testrender, shared with the GPU driver: analytic spheres
// and rectangles instead of tessellated ones, no light sampling (emission
// reaches the path through BSDF sampling with MIS weight 1), no background
// importance sampling or media, and Russian roulette with a fixed survival
// probability after every hit.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "../include/oslg.h"

extern "C" int oracle_run(const void* blob, size_t bytes, int64_t begin, int64_t end, const oslg_shaderglobals* G,
                          void* userdata, void* outputs, int nthreads, uint32_t* status_out);

namespace {

struct V {
    float x, y, z;
};
inline V mk(float x, float y, float z) { return V{ x, y, z }; }
inline V vadd(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V vsub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V vmul(V a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V vneg(V a) { return mk(-a.x, -a.y, -a.z); }
inline float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V vcross(V a, V b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V vnorm(V a) {
    const float inv = 1.0f / std::sqrt(vdot(a, a));
    return vmul(a, inv);
}

// Jarzynski and Olano, "Hash Functions for GPU Rendering" (JCGT 2020), PCG
// output permutation; the stream index is (path * 17 + slot) * 4 + dim.
inline uint32_t pcg_hash(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
inline float wf_rand(uint32_t seed, uint32_t path, uint32_t slot, uint32_t dim) {
    const uint32_t h = pcg_hash(((path * 17u + slot) * 4u + dim) ^ seed);
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

struct Prim {
    int kind, mat, id;
    V p, ex, ey, n, ux, uy;
    float r;
};

Prim setup(const oslg_primitive& q, int id) {
    Prim w{};
    w.kind = q.kind;
    w.mat = q.material;
    w.id = id;
    w.p = mk(q.p[0], q.p[1], q.p[2]);
    w.ex = mk(q.ex[0], q.ex[1], q.ex[2]);
    w.ey = mk(q.ey[0], q.ey[1], q.ey[2]);
    w.r = q.radius;
    if (q.kind != OSLG_PRIM_SPHERE) {
        w.n = vnorm(vcross(w.ex, w.ey));
        const float lx = vdot(w.ex, w.ex), ly = vdot(w.ey, w.ey);
        w.ux = mk(w.ex.x / lx, w.ex.y / lx, w.ex.z / lx);
        w.uy = mk(w.ey.x / ly, w.ey.y / ly, w.ey.z / ly);
    }
    return w;
}

// a t^2 + 2 b t + cc = 0 with a = d.d (a sampled direction is unit only
// to rounding)
bool hit_sphere(const Prim& q, V o, V d, bool self, float* t) {
    const V oc = vsub(o, q.p);
    const float a = vdot(d, d);
    const float b = vdot(oc, d);
    const float cc = vdot(oc, oc) - q.r * q.r;
    const float disc = b * b - a * cc;
    if (!(disc >= 0.0f)) return false;
    const float s = std::sqrt(disc);
    if (self) {
        if (!(b < 0.0f)) return false;
        *t = (s - b) / a;
        return *t > 0.0f;
    }
    const float t1 = (-b - s) / a;
    if (t1 > 0.0f) {
        *t = t1;
        return true;
    }
    const float t2 = (s - b) / a;
    if (t2 > 0.0f) {
        *t = t2;
        return true;
    }
    return false;
}

bool hit_quad(const Prim& q, V o, V d, float* t) {
    const float den = vdot(q.n, d);
    if (den == 0.0f) return false;
    const float tt = vdot(q.n, vsub(q.p, o)) / den;
    if (!(tt > 0.0f)) return false;
    const V h = vsub(vadd(o, vmul(d, tt)), q.p);
    const float u = vdot(h, q.ux), v = vdot(h, q.uy);
    if (!(u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f)) return false;
    *t = tt;
    return true;
}

int intersect(const std::vector<Prim>& prims, V o, V d, int skip, float* t_out) {
    float best = INFINITY;
    int best_id = -1;
    for (const Prim& q : prims) {
        float t;
        bool h;
        if (q.kind == OSLG_PRIM_SPHERE) {
            h = hit_sphere(q, o, d, q.id == skip, &t);
        } else {
            if (q.id == skip) continue;
            h = hit_quad(q, o, d, &t);
        }
        if (h && (t < best || (t == best && q.id < best_id))) {
            best = t;
            best_id = q.id;
        }
    }
    *t_out = best;
    return best_id;
}

struct Path {
    V o, d;
    float tp[3], L[3];
    float rough;  // roughness of the ray (the last sample's)
    int skip;
    uint32_t id;
};

}  // namespace

extern "C" {

// Render the paths path_begin + k * path_step (k < path_count) of the frame
// described by `o`. radiance: 3 planes of path_count floats. hits: shading
// points per bounce (16 entries). Returns 0, or the first nonzero status of
// a shading run.
int oracle_wavefront(const oslg_wavefront_options* o, const oslg_primitive* raw, int nprims,
                     const void* const* blobs, const size_t* blob_sizes, int nmat, int64_t path_begin,
                     int64_t path_count, int64_t path_step, int nthreads, float* radiance, int64_t* hits) {
    std::vector<Prim> prims(nprims);
    for (int i = 0; i < nprims; ++i) prims[i] = setup(raw[i], i);
    float cam[12];
    {
        double e[3] = { o->eye[0], o->eye[1], o->eye[2] };
        double d[3] = { (double)o->look[0] - e[0], (double)o->look[1] - e[1], (double)o->look[2] - e[2] };
        double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (double& x : d) x /= dl;
        const double u[3] = { o->up[0], o->up[1], o->up[2] };
        double r[3] = { d[1] * u[2] - d[2] * u[1], d[2] * u[0] - d[0] * u[2], d[0] * u[1] - d[1] * u[0] };
        double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (double& x : r) x /= rl;
        double v[3] = { r[1] * d[2] - r[2] * d[1], r[2] * d[0] - r[0] * d[2], r[0] * d[1] - r[1] * d[0] };
        const double th = std::tan((double)o->fov_deg * 3.14159265358979323846 / 360.0);
        const double aspect = (double)o->width / (double)o->height;
        for (int k = 0; k < 3; ++k) {
            cam[k] = (float)e[k];
            cam[3 + k] = (float)d[k];
            cam[6 + k] = (float)(r[k] * th * aspect);
            cam[9 + k] = (float)(v[k] * th);
        }
    }
    uint32_t seed = o->seed * 747796405u + 2891336453u;
    seed = ((seed >> ((seed >> 28u) + 4u)) ^ seed) * 277803737u;
    seed = (seed >> 22u) ^ seed;

    std::vector<Path> paths((size_t)path_count);
    for (int64_t k = 0; k < path_count; ++k) {
        const int64_t p = path_begin + k * path_step;
        const int64_t pix = p / o->spp;
        const int x = (int)(pix % o->width), y = (int)(pix / o->width);
        const float jx = wf_rand(seed, (uint32_t)p, 16u, 0u), jy = wf_rand(seed, (uint32_t)p, 16u, 1u);
        const float px = ((float)x + jx) / (float)o->width * 2.0f - 1.0f;
        const float py = 1.0f - ((float)y + jy) / (float)o->height * 2.0f;
        const V dir = mk(cam[3], cam[4], cam[5]), right = mk(cam[6], cam[7], cam[8]), up = mk(cam[9], cam[10], cam[11]);
        Path& P = paths[(size_t)k];
        P.o = mk(cam[0], cam[1], cam[2]);
        P.d = vnorm(vadd(vadd(dir, vmul(right, px)), vmul(up, py)));
        for (int c = 0; c < 3; ++c) {
            P.tp[c] = 1.0f;
            P.L[c] = 0.0f;
        }
        P.skip = -1;
        P.rough = 0.0f;
        P.id = (uint32_t)p;
    }
    for (int b = 0; b < 16; ++b) hits[b] = 0;

    std::vector<int64_t> active((size_t)path_count);
    for (int64_t k = 0; k < path_count; ++k) active[(size_t)k] = k;
    std::vector<int> hit_id;
    std::vector<float> hit_t;
    int status = 0;
    for (int b = 0; b < o->max_hits && !active.empty(); ++b) {
        const int64_t n = (int64_t)active.size();
        hit_id.assign((size_t)n, -1);
        hit_t.assign((size_t)n, 0.0f);
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : omp_get_max_threads())
        for (int64_t i = 0; i < n; ++i) {
            const Path& P = paths[(size_t)active[(size_t)i]];
            hit_id[(size_t)i] = intersect(prims, P.o, P.d, P.skip, &hit_t[(size_t)i]);
        }
        for (int64_t i = 0; i < n; ++i)
            if (hit_id[(size_t)i] < 0) {
                Path& P = paths[(size_t)active[(size_t)i]];
                for (int c = 0; c < 3; ++c) P.L[c] = P.L[c] + P.tp[c] * o->background[c];
            }
        std::vector<int64_t> next;
        for (int m = 0; m < nmat; ++m) {
            std::vector<int64_t> sel;
            for (int64_t i = 0; i < n; ++i)
                if (hit_id[(size_t)i] >= 0 && prims[hit_id[(size_t)i]].mat == m) sel.push_back(i);
            const int64_t nm = (int64_t)sel.size();
            if (nm == 0) continue;
            hits[b] += nm;
            std::vector<float> gl((size_t)nm * 20), ud((size_t)nm * 9), out((size_t)nm * 11, 0.0f);
            auto plane = [&](int k) { return gl.data() + (size_t)k * nm; };
            for (int64_t j = 0; j < nm; ++j) {
                const int64_t i = sel[(size_t)j];
                const Path& P = paths[(size_t)active[(size_t)i]];
                const Prim& q = prims[hit_id[(size_t)i]];
                const V Pt = vadd(P.o, vmul(P.d, hit_t[(size_t)i]));
                V N, dPdu, dPdv;
                float u, v;
                if (q.kind == OSLG_PRIM_SPHERE) {
                    N = vnorm(vsub(Pt, q.p));
                    // ortho() of src/testrender/raytracer.h:41-47
                    const V x = vnorm(std::fabs(N.x) > 0.01f ? mk(N.z, 0.0f, -N.x) : mk(0.0f, -N.z, N.y));
                    dPdu = vmul(x, q.r);
                    dPdv = vmul(vcross(N, x), q.r);
                    u = 0.5f * (N.x + 1.0f);
                    v = 0.5f * (N.y + 1.0f);
                } else {
                    N = q.n;
                    const V h = vsub(Pt, q.p);
                    u = vdot(h, q.ux);
                    v = vdot(h, q.uy);
                    dPdu = q.ex;
                    dPdv = q.ey;
                }
                V Ng = N;
                const bool backfacing = vdot(Ng, P.d) > 0.0f;
                if (backfacing) {
                    N = vneg(N);
                    Ng = vneg(Ng);
                }
                const float vals[20] = { Pt.x, Pt.y, Pt.z, P.d.x, P.d.y, P.d.z, N.x, N.y, N.z, Ng.x, Ng.y, Ng.z,
                                         u, v, dPdu.x, dPdu.y, dPdu.z, dPdv.x, dPdv.y, dPdv.z };
                for (int k = 0; k < 20; ++k) plane(k)[j] = vals[k];
                float* r = ud.data() + (size_t)j * 9;
                for (int c = 0; c < 3; ++c) r[c] = wf_rand(seed, P.id, (uint32_t)b, (uint32_t)c);
                for (int c = 0; c < 3; ++c) r[3 + c] = P.tp[c];
                r[6] = 0.0f;
                r[7] = P.rough;
                r[8] = backfacing ? 1.0f : 0.0f;
            }
            oslg_shaderglobals G;
            std::memset(&G, 0, sizeof(G));
            auto field = [&](oslg_field& f, int k) {
                f.data = plane(k);
                f.plane_stride = nm;
            };
            field(G.P, 0);
            field(G.I, 3);
            field(G.N, 6);
            field(G.Ng, 9);
            field(G.u, 12);
            field(G.v, 13);
            field(G.dPdu, 14);
            field(G.dPdv, 17);
            uint32_t st = 0;
            int rc = oracle_run(blobs[m], blob_sizes[m], 0, nm, &G, ud.data(), out.data(), nthreads, &st);
            if (rc != 0) return -1;
            if (st && !status) status = (int)st;
            for (int64_t j = 0; j < nm; ++j) {
                const int64_t i = sel[(size_t)j];
                Path& P = paths[(size_t)active[(size_t)i]];
                const float* r = out.data() + (size_t)j * 11;
                float tp[3];
                for (int c = 0; c < 3; ++c) {
                    tp[c] = P.tp[c];
                    P.L[c] = P.L[c] + tp[c] * r[7 + c];
                }
                if (b == o->max_hits - 1) continue;
                for (int c = 0; c < 3; ++c) tp[c] = tp[c] * r[3 + c];
                if (!(tp[0] > 0.0f) && !(tp[1] > 0.0f) && !(tp[2] > 0.0f)) continue;
                if (!(wf_rand(seed, P.id, (uint32_t)b, 3u) < o->rr_survival)) continue;
                for (int c = 0; c < 3; ++c) P.tp[c] = tp[c] / o->rr_survival;
                P.o = mk(plane(0)[j], plane(1)[j], plane(2)[j]);
                P.d = mk(r[0], r[1], r[2]);
                P.skip = hit_id[(size_t)i];
                P.rough = r[10];
                next.push_back(active[(size_t)i]);
            }
        }
        std::sort(next.begin(), next.end());
        active.swap(next);
    }
    for (int64_t k = 0; k < path_count; ++k)
        for (int c = 0; c < 3; ++c) radiance[(size_t)c * path_count + k] = paths[(size_t)k].L[c];
    return status;
}

}  // extern "C"
