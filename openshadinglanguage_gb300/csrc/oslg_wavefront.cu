// Wavefront path tracing over the persistent batch kernel: scene set-up
// and BVH, the per-bounce kernels (trace, plan, scatter, update) and the
// frame sequence captured as a CUDA graph. The per-path arithmetic follows
// testrender's loop (src/testrender/simpleraytracer.cpp:960-1184) and
// globals_from_hit (:890-932); every float operation is a single IEEE
// operation (this file builds with -fmad=false), so the CPU restatement in
// the oracle reproduces each path bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>

#include "oslg_wavefront.h"

namespace oslg {
namespace dev {
namespace {

// control words (uint32) in d_ctl_
enum { C_NACT = 0, C_COUNTER = 2, C_NITEMS = 3, C_COUNTS = 4, C_OFF = 68, C_CURSOR = 132, C_HITS = 196, C_SIZE = 256 };
// path-state planes (npaths floats each)
enum { S_O = 0, S_D = 3, S_TP = 6, S_L = 9, S_SKIP = 12, S_RO = 13, S_PLANES = 14 };
// hit-globals planes (cap floats each)
enum { G_P = 0, G_I = 3, G_N = 6, G_NG = 9, G_U = 12, G_V = 13, G_DPDU = 14, G_DPDV = 17, G_PLANES = 20 };

struct V {
    float x, y, z;
};
__device__ __forceinline__ V mk(float x, float y, float z) {
    V v;
    v.x = x;
    v.y = y;
    v.z = z;
    return v;
}
__device__ __forceinline__ V vadd(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V vsub(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V vmul(V a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V vneg(V a) { return mk(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float vdot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V vcross(V a, V b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ V vnorm(V a) {
    const float inv = 1.0f / sqrtf(vdot(a, a));
    return vmul(a, inv);
}
__device__ __forceinline__ V xyz(float4 f) { return mk(f.x, f.y, f.z); }

// PCG-style integer hash (Jarzynski and Olano, "Hash Functions for GPU
// Rendering", JCGT 2020): the random number of (path, slot, dimension).
// Slots 0..15 are bounces, slot 16 the camera.
__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    const uint32_t s = v * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
__device__ __forceinline__ float wf_rand(uint32_t seed, uint32_t path, uint32_t slot, uint32_t dim) {
    const uint32_t h = pcg_hash(((path * 17u + slot) * 4u + dim) ^ seed);
    return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// Warp-aggregated increment of ctr[key]: one atomic per distinct key per warp.
__device__ __forceinline__ uint32_t agg_inc(uint32_t* ctr, int key) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    const int lane = (int)(threadIdx.x & 31u);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&ctr[key], (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ int prim_kind(const WfPrim& q) { return __float_as_int(q.r[2].w); }
__device__ __forceinline__ int prim_mat(const WfPrim& q) { return __float_as_int(q.r[3].w); }
__device__ __forceinline__ int prim_id(const WfPrim& q) { return __float_as_int(q.r[4].w); }

// Sphere and rectangle intersection. `self`: the ray leaves this primitive
// (testrender skips the previous hit, simpleraytracer.cpp:979); a sphere
// can then only be hit again at its far root, when the ray enters it.
// The direction need not be unit length (a sampled direction is unit only
// to rounding): t solves a t^2 + 2 b t + cc = 0 with a = d.d.
__device__ __forceinline__ bool hit_sphere(const WfPrim& q, V o, V d, bool self, float* t) {
    const V oc = vsub(o, xyz(q.r[0]));
    const float r = q.r[0].w;
    const float a = vdot(d, d);
    const float b = vdot(oc, d);
    const float cc = vdot(oc, oc) - r * r;
    const float disc = b * b - a * cc;
    if (!(disc >= 0.0f)) return false;
    const float s = sqrtf(disc);
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
__device__ __forceinline__ bool hit_quad(const WfPrim& q, V o, V d, float* t) {
    const V n = xyz(q.r[3]);
    const float den = vdot(n, d);
    if (den == 0.0f) return false;
    const float tt = vdot(n, vsub(xyz(q.r[0]), o)) / den;
    if (!(tt > 0.0f)) return false;
    const V h = vsub(vadd(o, vmul(d, tt)), xyz(q.r[0]));
    const float u = vdot(h, xyz(q.r[4])), v = vdot(h, xyz(q.r[5]));
    if (!(u >= 0.0f && u <= 1.0f && v >= 0.0f && v <= 1.0f)) return false;
    *t = tt;
    return true;
}

// Slab test of one box: entry distance, or INFINITY when the box is missed
// or starts beyond `best` (a box starting exactly at `best` is kept: a hit
// at the same distance with a lower id may be inside).
__device__ __forceinline__ float box_entry(float lx, float ly, float lz, float hx, float hy, float hz, V o, V inv,
                                           float best) {
    const float tx0 = (lx - o.x) * inv.x, tx1 = (hx - o.x) * inv.x;
    const float ty0 = (ly - o.y) * inv.y, ty1 = (hy - o.y) * inv.y;
    const float tz0 = (lz - o.z) * inv.z, tz1 = (hz - o.z) * inv.z;
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
    return (tn <= tf && tn <= best) ? tn : INFINITY;
}

// Nearest hit over the BVH; ties go to the lower primitive id, so the
// result equals a scan of all primitives in id order. Children are visited
// near first; stacked subtrees whose entry lies beyond the current best are
// skipped when popped.
__device__ void traverse(const WfNode* __restrict__ nodes, const WfPrim* __restrict__ prims, V o, V d, int skip,
                         int* rec_out, float* t_out) {
    const V inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    float best = INFINITY;
    int best_rec = -1, best_id = INT_MAX;
    int stack_ref[kWfStack];
    float stack_t[kWfStack];
    int sp = 0;
    int ref = 0;
    for (;;) {
        if (ref >= 0) {
            const float4* nv = reinterpret_cast<const float4*>(nodes + ref);
            const float4 na = __ldg(nv), nb = __ldg(nv + 1), nc = __ldg(nv + 2);
            const int4 nd = __ldg(reinterpret_cast<const int4*>(nv + 3));
            const float tl = box_entry(na.x, na.y, na.z, na.w, nb.x, nb.y, o, inv, best);
            const float tr = box_entry(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, o, inv, best);
            const bool hl = tl != INFINITY, hr = tr != INFINITY;
            if (hl && hr) {
                const bool lfirst = tl <= tr;
                if (sp < kWfStack) {
                    stack_ref[sp] = lfirst ? nd.y : nd.x;
                    stack_t[sp] = lfirst ? tr : tl;
                    ++sp;
                }
                ref = lfirst ? nd.x : nd.y;
                continue;
            }
            if (hl) { ref = nd.x; continue; }
            if (hr) { ref = nd.y; continue; }
        } else {
            const int x = ~ref;
            const int first = x >> 4, count = x & 15;
            for (int k = first; k < first + count; ++k) {
                WfPrim q;
                const float4* src = reinterpret_cast<const float4*>(prims + k);
                q.r[0] = __ldg(src);
                q.r[2] = __ldg(src + 2);
                q.r[4] = __ldg(src + 4);
                const int id = prim_id(q);
                float t;
                bool h;
                if (prim_kind(q) == OSLG_PRIM_SPHERE) {
                    h = hit_sphere(q, o, d, id == skip, &t);
                } else {
                    if (id == skip) continue;
                    q.r[3] = __ldg(src + 3);
                    q.r[5] = __ldg(src + 5);
                    h = hit_quad(q, o, d, &t);
                }
                if (h && (t < best || (t == best && id < best_id))) {
                    best = t;
                    best_rec = k;
                    best_id = id;
                }
            }
        }
        // next stacked subtree that can still hold the nearest hit
        for (;;) {
            if (sp == 0) {
                *rec_out = best_rec;
                *t_out = best;
                return;
            }
            --sp;
            if (!(stack_t[sp] > best)) break;
        }
        ref = stack_ref[sp];
    }
}

struct WfArgs {
    const WfPrim* prims;
    const WfNode* nodes;
    float* st;           // path state planes
    int64_t np;          // paths
    int64_t cap;         // sorted-slot capacity
    uint32_t* ctl;
    uint32_t* act;       // 2 lists of np
    int32_t* hit_rec;
    float* hit_t;
    uint32_t* hit_slot;
    float* gl;           // hit-globals planes
    float* ud;           // cap x 7
    float* out;          // cap x 11
    const int32_t* order;
    const BatchJob* templ;
    BatchJob* jobs;
    uint2* items;
    int nmat, tile, spp, width, height;
    uint32_t seed;
    float rr;
    float bg[3];
    float cam[12];
};

__global__ void k_setup(const oslg_primitive* __restrict__ raw, const int32_t* __restrict__ order, int n,
                        WfPrim* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int id = order[k];
    const oslg_primitive q = raw[id];
    WfPrim w;
    for (int i = 0; i < 6; ++i) w.r[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    w.r[0] = make_float4(q.p[0], q.p[1], q.p[2], q.radius);
    w.r[1] = make_float4(q.ex[0], q.ex[1], q.ex[2], 0.0f);
    w.r[2] = make_float4(q.ey[0], q.ey[1], q.ey[2], __int_as_float(q.kind));
    w.r[3].w = __int_as_float(q.material);
    w.r[4].w = __int_as_float(id);
    if (q.kind != OSLG_PRIM_SPHERE) {
        const V ex = mk(q.ex[0], q.ex[1], q.ex[2]), ey = mk(q.ey[0], q.ey[1], q.ey[2]);
        const V n = vnorm(vcross(ex, ey));
        const float lx = vdot(ex, ex), ly = vdot(ey, ey);
        w.r[3] = make_float4(n.x, n.y, n.z, w.r[3].w);
        w.r[4] = make_float4(ex.x / lx, ex.y / lx, ex.z / lx, w.r[4].w);
        w.r[5] = make_float4(ey.x / ly, ey.y / ly, ey.z / ly, 0.0f);
    }
    out[k] = w;
}

// Camera rays (slot 16 of the random stream: pixel jitter), fresh state.
__global__ void k_camera(const __grid_constant__ WfArgs a) {
    const int64_t np = a.np;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < np; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t pix = p / a.spp;
        const int x = (int)(pix % a.width), y = (int)(pix / a.width);
        const float jx = wf_rand(a.seed, (uint32_t)p, 16u, 0u), jy = wf_rand(a.seed, (uint32_t)p, 16u, 1u);
        const float px = ((float)x + jx) / (float)a.width * 2.0f - 1.0f;
        const float py = 1.0f - ((float)y + jy) / (float)a.height * 2.0f;
        const V dir = mk(a.cam[3], a.cam[4], a.cam[5]);
        const V right = mk(a.cam[6], a.cam[7], a.cam[8]), up = mk(a.cam[9], a.cam[10], a.cam[11]);
        const V d = vnorm(vadd(vadd(dir, vmul(right, px)), vmul(up, py)));
        float* st = a.st;
        st[(S_O + 0) * np + p] = a.cam[0];
        st[(S_O + 1) * np + p] = a.cam[1];
        st[(S_O + 2) * np + p] = a.cam[2];
        st[(S_D + 0) * np + p] = d.x;
        st[(S_D + 1) * np + p] = d.y;
        st[(S_D + 2) * np + p] = d.z;
        for (int c = 0; c < 3; ++c) {
            st[(S_TP + c) * np + p] = 1.0f;
            st[(S_L + c) * np + p] = 0.0f;
        }
        st[S_SKIP * np + p] = __int_as_float(-1);
        st[S_RO * np + p] = 0.0f;  // camera rays have no roughness
        a.act[p] = (uint32_t)p;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctl[C_NACT] = (uint32_t)np;
}

__global__ void __launch_bounds__(256) k_trace(const __grid_constant__ WfArgs a, int cur) {
    __shared__ uint32_t s_cnt[kWfMaxMaterials];
    for (int m = threadIdx.x; m < a.nmat; m += blockDim.x) s_cnt[m] = 0;
    __syncthreads();
    const int64_t np = a.np;
    const uint32_t n = a.ctl[C_NACT + cur];
    const uint32_t* act = a.act + (int64_t)cur * np;
    float* st = a.st;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int64_t p = act[i];
        const V o = mk(st[(S_O + 0) * np + p], st[(S_O + 1) * np + p], st[(S_O + 2) * np + p]);
        const V d = mk(st[(S_D + 0) * np + p], st[(S_D + 1) * np + p], st[(S_D + 2) * np + p]);
        const int skip = __float_as_int(st[S_SKIP * np + p]);
        int rec;
        float t;
        traverse(a.nodes, a.prims, o, d, skip, &rec, &t);
        if (rec < 0) {
            for (int c = 0; c < 3; ++c)
                st[(S_L + c) * np + p] = st[(S_L + c) * np + p] + st[(S_TP + c) * np + p] * a.bg[c];
        } else {
            atomicAdd(&s_cnt[__float_as_int(__ldg(&a.prims[rec].r[3].w))], 1u);
        }
        a.hit_rec[i] = rec;
        a.hit_t[i] = t;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < a.nmat; m += blockDim.x)
        if (s_cnt[m]) atomicAdd(&a.ctl[C_COUNTS + m], s_cnt[m]);
}

// One CTA: slot ranges (tile aligned) per material, live job table, work
// list in cost order, counters for the next steps.
__global__ void __launch_bounds__(1024) k_plan(const __grid_constant__ WfArgs a, int cur, int bounce) {
    __shared__ uint32_t s_cnt[kWfMaxMaterials], s_off[kWfMaxMaterials], s_ioff[kWfMaxMaterials];
    const int nmat = a.nmat;
    const uint32_t tile = (uint32_t)a.tile;
    for (int m = threadIdx.x; m < nmat; m += blockDim.x) s_cnt[m] = a.ctl[C_COUNTS + m];
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t off = 0, it = 0, total = 0;
        for (int m = 0; m < nmat; ++m) {
            s_off[m] = off;
            off += (s_cnt[m] + tile - 1) / tile * tile;
            total += s_cnt[m];
        }
        for (int k = 0; k < nmat; ++k) {
            s_ioff[k] = it;
            it += (s_cnt[a.order[k]] + tile - 1) / tile;
        }
        a.ctl[C_NITEMS] = it;
        a.ctl[C_HITS + bounce] = total;
        a.ctl[C_COUNTER] = 0;
        a.ctl[C_NACT + (cur ^ 1)] = 0;
    }
    __syncthreads();
    for (int m = threadIdx.x; m < nmat; m += blockDim.x) {
        a.ctl[C_COUNTS + m] = 0;
        a.ctl[C_OFF + m] = s_off[m];
        a.ctl[C_CURSOR + m] = 0;
        const BatchJob* T = a.templ + m;
        BatchJob* J = a.jobs + m;
        const int64_t off = s_off[m];
        J->blob = T->blob;
        J->spec_case = T->spec_case;
        J->status = nullptr;
        J->npoints = s_cnt[m];
        J->userdata = reinterpret_cast<char*>(a.ud + off * kWfInFloats);
        J->outputs = reinterpret_cast<char*>(a.out + off * kWfOutFloats);
        const oslg_field* tf = reinterpret_cast<const oslg_field*>(&T->G);
        oslg_field* jf = reinterpret_cast<oslg_field*>(&J->G);
        for (size_t k = 0; k < sizeof(oslg_shaderglobals) / sizeof(oslg_field); ++k) {
            jf[k] = tf[k];
            if (tf[k].data) jf[k].data = tf[k].data + off;
        }
    }
    for (int k = 0; k < nmat; ++k) {
        const int m = a.order[k];
        const uint32_t nt = (s_cnt[m] + tile - 1) / tile;
        for (uint32_t t = threadIdx.x; t < nt; t += blockDim.x) a.items[s_ioff[k] + t] = make_uint2((unsigned)m, t);
    }
}

// globals_from_hit (simpleraytracer.cpp:890-932) for the analytic
// primitives, written material-sorted, plus the sampling record. Each CTA
// takes 256 active hits, orders them by material in shared memory and
// reserves one slot range per material, so that consecutive threads write
// consecutive slots.
__global__ void __launch_bounds__(256) k_scatter(const __grid_constant__ WfArgs a, int cur, int bounce) {
    __shared__ uint32_t s_cnt[kWfMaxMaterials], s_pre[kWfMaxMaterials], s_base[kWfMaxMaterials];
    __shared__ uint32_t s_order[256];
    const int64_t np = a.np, cap = a.cap;
    const uint32_t n = a.ctl[C_NACT + cur];
    const uint32_t* act = a.act + (int64_t)cur * np;
    const float* st = a.st;
    float* gl = a.gl;
    for (uint32_t chunk = blockIdx.x * 256u; chunk < n; chunk += gridDim.x * 256u) {
        for (int m = threadIdx.x; m < a.nmat; m += blockDim.x) s_cnt[m] = 0;
        __syncthreads();
        const uint32_t i0 = chunk + threadIdx.x;
        int mat = -1;
        uint32_t rank = 0;
        if (i0 < n) {
            const int rec0 = a.hit_rec[i0];
            if (rec0 >= 0) {
                mat = __float_as_int(__ldg(&a.prims[rec0].r[3].w));
                rank = atomicAdd(&s_cnt[mat], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t acc = 0;
            for (int m = 0; m < a.nmat; ++m) {
                s_pre[m] = acc;
                acc += s_cnt[m];
            }
        }
        for (int m = threadIdx.x; m < a.nmat; m += blockDim.x)
            s_base[m] = s_cnt[m] ? a.ctl[C_OFF + m] + atomicAdd(a.ctl + C_CURSOR + m, s_cnt[m]) : 0u;
        __syncthreads();
        if (mat >= 0) s_order[s_pre[mat] + rank] = i0;
        uint32_t hits = 0;
        for (int m = 0; m < a.nmat; ++m) hits += s_cnt[m];
        __syncthreads();
        if (threadIdx.x < hits) {
            const uint32_t i = s_order[threadIdx.x];
            const int rec = a.hit_rec[i];
            WfPrim q;
            const float4* src = reinterpret_cast<const float4*>(a.prims + rec);
            for (int k = 0; k < 6; ++k) q.r[k] = __ldg(src + k);
            const int m = prim_mat(q);
            const int64_t slot = (int64_t)s_base[m] + (threadIdx.x - s_pre[m]);
            const int64_t p = act[i];
            const V o = mk(st[(S_O + 0) * np + p], st[(S_O + 1) * np + p], st[(S_O + 2) * np + p]);
            const V d = mk(st[(S_D + 0) * np + p], st[(S_D + 1) * np + p], st[(S_D + 2) * np + p]);
            const float t = a.hit_t[i];
            const V P = vadd(o, vmul(d, t));
            V N, dPdu, dPdv;
            float u, v;
            if (prim_kind(q) == OSLG_PRIM_SPHERE) {
                const float r = q.r[0].w;
                N = vnorm(vsub(P, xyz(q.r[0])));
                // ortho() of src/testrender/raytracer.h:41-47
                const V x = vnorm(fabsf(N.x) > 0.01f ? mk(N.z, 0.0f, -N.x) : mk(0.0f, -N.z, N.y));
                dPdu = vmul(x, r);
                dPdv = vmul(vcross(N, x), r);
                u = 0.5f * (N.x + 1.0f);
                v = 0.5f * (N.y + 1.0f);
            } else {
                N = xyz(q.r[3]);
                const V h = vsub(P, xyz(q.r[0]));
                u = vdot(h, xyz(q.r[4]));
                v = vdot(h, xyz(q.r[5]));
                dPdu = xyz(q.r[1]);
                dPdv = xyz(q.r[2]);
            }
            V Ng = N;
            const bool backfacing = vdot(Ng, d) > 0.0f;
            if (backfacing) {
                N = vneg(N);
                Ng = vneg(Ng);
            }
            const float vals[G_PLANES] = { P.x, P.y, P.z, d.x, d.y, d.z, N.x, N.y, N.z, Ng.x, Ng.y, Ng.z,
                                           u, v, dPdu.x, dPdu.y, dPdu.z, dPdv.x, dPdv.y, dPdv.z };
#pragma unroll
            for (int k = 0; k < G_PLANES; ++k) gl[k * cap + slot] = vals[k];
            float* ud = a.ud + slot * kWfInFloats;
            ud[0] = wf_rand(a.seed, (uint32_t)p, (uint32_t)bounce, 0u);
            ud[1] = wf_rand(a.seed, (uint32_t)p, (uint32_t)bounce, 1u);
            ud[2] = wf_rand(a.seed, (uint32_t)p, (uint32_t)bounce, 2u);
            ud[3] = st[(S_TP + 0) * np + p];
            ud[4] = st[(S_TP + 1) * np + p];
            ud[5] = st[(S_TP + 2) * np + p];
            ud[6] = 0.0f;
            ud[7] = st[S_RO * np + p];
            ud[8] = backfacing ? 1.0f : 0.0f;
            a.hit_slot[i] = (uint32_t)slot;
        }
        __syncthreads();
    }
}

// Emission, path weight, Russian roulette, next ray and compaction
// (simpleraytracer.cpp:1060-1182 without light sampling: MIS weight 1).
__global__ void __launch_bounds__(256) k_update(const __grid_constant__ WfArgs a, int cur, int bounce, int last) {
    const int64_t np = a.np, cap = a.cap;
    const uint32_t n = a.ctl[C_NACT + cur];
    const uint32_t* act = a.act + (int64_t)cur * np;
    uint32_t* nxt = a.act + (int64_t)(cur ^ 1) * np;
    float* st = a.st;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int rec = a.hit_rec[i];
        if (rec < 0) continue;
        const int64_t p = act[i];
        const int64_t slot = a.hit_slot[i];
        const float* r = a.out + slot * kWfOutFloats;
        float tp[3];
        for (int c = 0; c < 3; ++c) {
            tp[c] = st[(S_TP + c) * np + p];
            st[(S_L + c) * np + p] = st[(S_L + c) * np + p] + tp[c] * r[7 + c];
        }
        if (last) continue;
        for (int c = 0; c < 3; ++c) tp[c] = tp[c] * r[3 + c];
        if (!(tp[0] > 0.0f) && !(tp[1] > 0.0f) && !(tp[2] > 0.0f)) continue;
        if (!(wf_rand(a.seed, (uint32_t)p, (uint32_t)bounce, 3u) < a.rr)) continue;
        for (int c = 0; c < 3; ++c) st[(S_TP + c) * np + p] = tp[c] / a.rr;
        for (int c = 0; c < 3; ++c) {
            st[(S_O + c) * np + p] = a.gl[(G_P + c) * cap + slot];
            st[(S_D + c) * np + p] = r[c];
        }
        st[S_SKIP * np + p] = __ldg(&a.prims[rec].r[4].w);  // primitive id bits
        st[S_RO * np + p] = r[10];                           // r.roughness = p.roughness
        nxt[agg_inc(a.ctl + C_NACT + (cur ^ 1), 0)] = (uint32_t)p;
    }
}

__global__ void k_resolve(const float* __restrict__ st, int64_t np, int spp, float* __restrict__ image) {
    const int64_t npix = np / spp;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < npix; q += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; ++c) {
            float s = 0.0f;
            for (int k = 0; k < spp; ++k) s = s + st[(S_L + c) * np + q * spp + k];
            image[q * 3 + c] = s / (float)spp;
        }
    }
}

}  // namespace
}  // namespace dev

namespace {
bool ok(cudaError_t e, std::string* err, const char* what) {
    if (e == cudaSuccess) return true;
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

struct BuildPrim {
    float lo[3], hi[3], c[3];
    int id;
};

// Binned-SAH BVH over padded primitive bounds (padding keeps rounding in
// the slab test from culling a primitive the exact scan would hit). Leaves
// hold up to 4 primitives; below a depth of 24 the split is the median so
// that the traversal stack never overflows.
struct TmpNode {
    float lo[3], hi[3];
    int left = -1, right = -1, first = 0, count = 0;
};

float half_area(const float* lo, const float* hi) {
    const float dx = std::max(0.0f, hi[0] - lo[0]), dy = std::max(0.0f, hi[1] - lo[1]),
                dz = std::max(0.0f, hi[2] - lo[2]);
    return dx * dy + dy * dz + dz * dx;
}

int build_sah(std::vector<BuildPrim>& bp, int begin, int end, int depth, std::vector<TmpNode>& out) {
    TmpNode N;
    float clo[3] = { INFINITY, INFINITY, INFINITY }, chi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int k = 0; k < 3; ++k) {
        N.lo[k] = INFINITY;
        N.hi[k] = -INFINITY;
    }
    for (int i = begin; i < end; ++i)
        for (int k = 0; k < 3; ++k) {
            N.lo[k] = std::min(N.lo[k], bp[i].lo[k]);
            N.hi[k] = std::max(N.hi[k], bp[i].hi[k]);
            clo[k] = std::min(clo[k], bp[i].c[k]);
            chi[k] = std::max(chi[k], bp[i].c[k]);
        }
    const int n = end - begin;
    const int me = (int)out.size();
    out.push_back(N);
    if (n <= 1) {
        out[me].first = begin;
        out[me].count = n;
        return me;
    }
    const int kBins = 16;
    int best_axis = -1, best_split = 0;
    float best_cost = INFINITY;
    if (depth < 24) {
        for (int ax = 0; ax < 3; ++ax) {
            const float ext = chi[ax] - clo[ax];
            if (!(ext > 0.0f)) continue;
            int cnt[kBins] = {};
            float blo[kBins][3], bhi[kBins][3];
            for (int b = 0; b < kBins; ++b)
                for (int k = 0; k < 3; ++k) {
                    blo[b][k] = INFINITY;
                    bhi[b][k] = -INFINITY;
                }
            for (int i = begin; i < end; ++i) {
                int b = (int)((bp[i].c[ax] - clo[ax]) / ext * kBins);
                b = std::min(kBins - 1, std::max(0, b));
                ++cnt[b];
                for (int k = 0; k < 3; ++k) {
                    blo[b][k] = std::min(blo[b][k], bp[i].lo[k]);
                    bhi[b][k] = std::max(bhi[b][k], bp[i].hi[k]);
                }
            }
            for (int s = 1; s < kBins; ++s) {
                float llo[3] = { INFINITY, INFINITY, INFINITY }, lhi[3] = { -INFINITY, -INFINITY, -INFINITY };
                float rlo[3] = { INFINITY, INFINITY, INFINITY }, rhi[3] = { -INFINITY, -INFINITY, -INFINITY };
                int nl = 0, nr = 0;
                for (int b = 0; b < kBins; ++b) {
                    float* lo = b < s ? llo : rlo;
                    float* hi = b < s ? lhi : rhi;
                    (b < s ? nl : nr) += cnt[b];
                    for (int k = 0; k < 3; ++k) {
                        lo[k] = std::min(lo[k], blo[b][k]);
                        hi[k] = std::max(hi[k], bhi[b][k]);
                    }
                }
                if (!nl || !nr) continue;
                const float cost = half_area(llo, lhi) * nl + half_area(rlo, rhi) * nr;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = ax;
                    best_split = s;
                }
            }
        }
        // a leaf when splitting costs more than intersecting everything here
        if (n <= 4 && !(best_cost + half_area(N.lo, N.hi) < half_area(N.lo, N.hi) * n)) best_axis = -2;
    }
    if (best_axis == -2) {
        out[me].first = begin;
        out[me].count = n;
        return me;
    }
    int mid;
    if (best_axis >= 0) {
        const float ext = chi[best_axis] - clo[best_axis];
        auto it = std::partition(bp.begin() + begin, bp.begin() + end, [&](const BuildPrim& p) {
            int b = (int)((p.c[best_axis] - clo[best_axis]) / ext * kBins);
            b = std::min(kBins - 1, std::max(0, b));
            return b < best_split;
        });
        mid = (int)(it - bp.begin());
    } else {
        mid = begin;
    }
    if (mid == begin || mid == end) {  // median of the longest centroid axis
        int axis = 0;
        for (int k = 1; k < 3; ++k)
            if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
        mid = begin + n / 2;
        std::nth_element(bp.begin() + begin, bp.begin() + mid, bp.begin() + end,
                         [axis](const BuildPrim& x, const BuildPrim& y) {
                             return x.c[axis] < y.c[axis] || (x.c[axis] == y.c[axis] && x.id < y.id);
                         });
    }
    const int l = build_sah(bp, begin, mid, depth + 1, out);
    const int r = build_sah(bp, mid, end, depth + 1, out);
    out[me].left = l;
    out[me].right = r;
    return me;
}

int tree_depth(const std::vector<TmpNode>& t, int i) {
    if (t[i].left < 0) return 1;
    return 1 + std::max(tree_depth(t, t[i].left), tree_depth(t, t[i].right));
}

// Flatten: one device node per inner node, children boxes in the parent.
void flatten(const std::vector<TmpNode>& t, std::vector<dev::WfNode>& out) {
    std::vector<int> index(t.size(), -1);
    // inner nodes in depth-first order; node 0 is the root (a lone leaf root
    // becomes a node with an empty right child)
    std::vector<int> order;
    std::vector<int> st = { 0 };
    while (!st.empty()) {
        const int i = st.back();
        st.pop_back();
        if (t[i].left < 0 && i != 0) continue;
        index[i] = (int)order.size();
        order.push_back(i);
        if (t[i].left >= 0) {
            st.push_back(t[i].right);
            st.push_back(t[i].left);
        }
    }
    auto ref_of = [&](int c) {
        if (t[c].left >= 0) return index[c];
        return ~((t[c].first << 4) | t[c].count);
    };
    out.resize(order.size());
    for (size_t k = 0; k < order.size(); ++k) {
        const TmpNode& N = t[order[k]];
        dev::WfNode& D = out[k];
        float llo[3], lhi[3], rlo[3], rhi[3];
        int lref, rref;
        if (N.left >= 0) {
            for (int j = 0; j < 3; ++j) {
                llo[j] = t[N.left].lo[j];
                lhi[j] = t[N.left].hi[j];
                rlo[j] = t[N.right].lo[j];
                rhi[j] = t[N.right].hi[j];
            }
            lref = ref_of(N.left);
            rref = ref_of(N.right);
        } else {  // root leaf
            for (int j = 0; j < 3; ++j) {
                llo[j] = N.lo[j];
                lhi[j] = N.hi[j];
                rlo[j] = INFINITY;
                rhi[j] = -INFINITY;
            }
            lref = ~((N.first << 4) | N.count);
            rref = ~0;
        }
        D.a = make_float4(llo[0], llo[1], llo[2], lhi[0]);
        D.b = make_float4(lhi[1], lhi[2], rlo[0], rlo[1]);
        D.c = make_float4(rlo[2], rhi[0], rhi[1], rhi[2]);
        D.d = make_int4(lref, rref, 0, 0);
    }
}
}  // namespace

Wavefront::~Wavefront() { release(); }

void Wavefront::release() {
    if (gexec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(gexec_));
    if (graph_) cudaGraphDestroy(static_cast<cudaGraph_t>(graph_));
    gexec_ = graph_ = nullptr;
    for (void*& e : ev_)
        if (e) {
            cudaEventDestroy(static_cast<cudaEvent_t>(e));
            e = nullptr;
        }
    void* bufs[] = { d_prims_, d_nodes_, d_state_, d_active_, d_hit_rec_, d_hit_t_, d_hit_slot_, d_globals_,
                     d_ud_, d_out_, d_ctl_, d_jobs_, d_templ_, d_items_, d_order_, d_heap_, d_spec_heap_ };
    for (void* b : bufs) cudaFree(b);
    d_prims_ = nullptr;
    d_nodes_ = nullptr;
    d_state_ = d_hit_t_ = d_globals_ = d_ud_ = d_out_ = d_heap_ = d_spec_heap_ = nullptr;
    d_active_ = d_hit_slot_ = d_ctl_ = nullptr;
    d_hit_rec_ = d_order_ = nullptr;
    d_jobs_ = d_templ_ = nullptr;
    d_items_ = nullptr;
}

int Wavefront::init(DeviceState& ds, const oslg_wavefront_options& o, const oslg_primitive* prims, int nprims,
                    const std::vector<const CompiledGroup*>& mats, const std::string* jit_dirs, std::string* err) {
    ds_ = &ds;
    opt_ = o;
    nprims_ = nprims;
    nmat_ = (int)mats.size();
    npaths_ = (int64_t)o.width * o.height * o.spp;
    block_ = o.block > 0 ? std::max(32, std::min(512, (o.block + 31) & ~31)) : 256;
    if (jit_dirs) block_ = o.block == 128 || o.block == 64 ? o.block : 256;  // specialized: one point per thread
    maxt_ = block_ > 256 ? 512 : 256;
    ppt_ = jit_dirs ? 1 : (o.points_per_thread >= 4 ? 4 : (o.points_per_thread >= 2 ? 2 : 1));
    tile_ = block_ * ppt_;
    cap_ = npaths_ + (int64_t)nmat_ * tile_;

    // camera basis in double: eye, dir, right * tan(fov/2) * aspect, up * tan(fov/2)
    {
        double e[3] = { o.eye[0], o.eye[1], o.eye[2] };
        double d[3] = { (double)o.look[0] - e[0], (double)o.look[1] - e[1], (double)o.look[2] - e[2] };
        double dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
        for (double& x : d) x /= dl;
        const double u[3] = { o.up[0], o.up[1], o.up[2] };
        double r[3] = { d[1] * u[2] - d[2] * u[1], d[2] * u[0] - d[0] * u[2], d[0] * u[1] - d[1] * u[0] };
        double rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (double& x : r) x /= rl;
        double v[3] = { r[1] * d[2] - r[2] * d[1], r[2] * d[0] - r[0] * d[2], r[0] * d[1] - r[1] * d[0] };
        const double th = std::tan((double)o.fov_deg * 3.14159265358979323846 / 360.0);
        const double aspect = (double)o.width / (double)o.height;
        for (int k = 0; k < 3; ++k) {
            cam_[k] = (float)e[k];
            cam_[3 + k] = (float)d[k];
            cam_[6 + k] = (float)(r[k] * th * aspect);
            cam_[9 + k] = (float)(v[k] * th);
        }
    }

    // BVH over padded bounds
    std::vector<BuildPrim> bp(nprims);
    for (int i = 0; i < nprims; ++i) {
        const oslg_primitive& q = prims[i];
        BuildPrim& b = bp[i];
        b.id = i;
        if (q.kind == OSLG_PRIM_SPHERE) {
            for (int k = 0; k < 3; ++k) {
                b.lo[k] = q.p[k] - q.radius;
                b.hi[k] = q.p[k] + q.radius;
            }
        } else {
            for (int k = 0; k < 3; ++k) {
                const float c[4] = { q.p[k], q.p[k] + q.ex[k], q.p[k] + q.ey[k], q.p[k] + q.ex[k] + q.ey[k] };
                b.lo[k] = std::min(std::min(c[0], c[1]), std::min(c[2], c[3]));
                b.hi[k] = std::max(std::max(c[0], c[1]), std::max(c[2], c[3]));
            }
        }
        float ext = 0.0f;
        for (int k = 0; k < 3; ++k) ext = std::max(ext, std::max(std::fabs(b.lo[k]), std::fabs(b.hi[k])));
        const float pad = 1e-4f * ext + 1e-4f;
        for (int k = 0; k < 3; ++k) {
            b.lo[k] -= pad;
            b.hi[k] += pad;
            b.c[k] = 0.5f * (b.lo[k] + b.hi[k]);
        }
    }
    std::vector<TmpNode> tree;
    tree.reserve(2 * std::max(1, nprims));
    if (nprims > 0) build_sah(bp, 0, nprims, 0, tree);
    if (!tree.empty() && tree_depth(tree, 0) > dev::kWfStack - 1) {
        // pathological scene: fall back to median splits (depth ~ log2 n)
        tree.clear();
        build_sah(bp, 0, nprims, 1 << 20, tree);
    }
    std::vector<dev::WfNode> nodes;
    if (tree.empty()) {
        dev::WfNode e;
        e.a = make_float4(INFINITY, INFINITY, INFINITY, -INFINITY);
        e.b = make_float4(-INFINITY, -INFINITY, INFINITY, INFINITY);
        e.c = make_float4(INFINITY, -INFINITY, -INFINITY, -INFINITY);
        e.d = make_int4(~0, ~0, 0, 0);
        nodes.push_back(e);
    } else {
        flatten(tree, nodes);
    }
    nnodes_ = (int)nodes.size();
    std::vector<int32_t> order(nprims);
    for (int i = 0; i < nprims; ++i) order[i] = bp[i].id;

    // material order, heaviest program first; launch shape as the batch executor
    std::vector<int32_t> morder(nmat_);
    std::iota(morder.begin(), morder.end(), 0);
    std::vector<double> cost(nmat_);
    uint32_t prog_bytes = 0, slots = 0;
    for (int m = 0; m < nmat_; ++m) {
        const ProgramHeader& h = mats[m]->header;
        cost[m] = program_cost(h, reinterpret_cast<const Op*>(mats[m]->blob.data() + sizeof(ProgramHeader)));
        prog_bytes = std::max(prog_bytes, h.nops * (uint32_t)sizeof(Op) + ((h.nconst + 3u) & ~3u) * 4u);
        slots = std::max(slots, h.heap_slots);
    }
    std::stable_sort(morder.begin(), morder.end(), [&](int x, int y) { return cost[x] > cost[y]; });
    prog_bytes = (prog_bytes + 15u) & ~15u;
    const size_t heap_b = (size_t)slots * tile_ * sizeof(float);
    // heap_smem: 1 shared memory, 2 HBM, otherwise shared memory when it fits in 100 KiB
    smem_heap_ = o.heap_smem == 1 || (o.heap_smem != 2 && prog_bytes + heap_b <= 100 * 1024);
    if (smem_heap_ && prog_bytes + heap_b + batch_static_smem() > ds.smem_optin) smem_heap_ = false;
    shmem_ = prog_bytes + (smem_heap_ ? heap_b : 0);
    if (shmem_ + batch_static_smem() > ds.smem_optin) {
        if (err) *err = "material programs do not fit in shared memory";
        return OSLG_ERR_LOWER;
    }
    if (!ok((cudaError_t)batch_variants_prepare(ds), err, "batch kernel attribute")) return OSLG_ERR_CUDA;
    int per_sm = 0;
    if (!ok((cudaError_t)batch_variant_occupancy(maxt_, ppt_, smem_heap_, block_, shmem_, &per_sm), err,
            "occupancy"))
        return OSLG_ERR_CUDA;
    if (per_sm < 1) {
        if (err) *err = "shading launch shape does not fit on an SM";
        return OSLG_ERR_LOWER;
    }
    grid_shade_ = ds.sm_count * per_sm;
    int per_sm_trace = 0;
    if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_trace, dev::k_trace, 256, 0), err, "occupancy"))
        return OSLG_ERR_CUDA;
    grid_trace_ = ds.sm_count * std::max(1, per_sm_trace);
    int per_sm_scatter = 0;
    if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_scatter, dev::k_scatter, 256, 0), err, "occupancy"))
        return OSLG_ERR_CUDA;
    grid_stream_ = ds.sm_count * std::max(1, per_sm_scatter);

    // device memory
    const int64_t np = npaths_, cap = cap_;
    const size_t items_cap = (size_t)(cap / tile_ + nmat_ + 1);
    oslg_primitive* d_raw = nullptr;
    int32_t* d_ord = nullptr;
    bool good = ok(cudaMalloc(&d_prims_, sizeof(dev::WfPrim) * std::max(1, nprims)), err, "cudaMalloc prims") &&
                ok(cudaMalloc(&d_nodes_, sizeof(dev::WfNode) * nnodes_), err, "cudaMalloc nodes") &&
                ok(cudaMalloc(&d_state_, sizeof(float) * dev::S_PLANES * np), err, "cudaMalloc path state") &&
                ok(cudaMalloc(&d_active_, sizeof(uint32_t) * 2 * np), err, "cudaMalloc path lists") &&
                ok(cudaMalloc(&d_hit_rec_, sizeof(int32_t) * np), err, "cudaMalloc hits") &&
                ok(cudaMalloc(&d_hit_t_, sizeof(float) * np), err, "cudaMalloc hits") &&
                ok(cudaMalloc(&d_hit_slot_, sizeof(uint32_t) * np), err, "cudaMalloc hits") &&
                ok(cudaMalloc(&d_globals_, sizeof(float) * dev::G_PLANES * cap), err, "cudaMalloc hit globals") &&
                ok(cudaMalloc(&d_ud_, sizeof(float) * kWfInFloats * cap), err, "cudaMalloc sample inputs") &&
                ok(cudaMalloc(&d_out_, sizeof(float) * kWfOutFloats * cap), err, "cudaMalloc sample outputs") &&
                ok(cudaMalloc(&d_ctl_, sizeof(uint32_t) * dev::C_SIZE), err, "cudaMalloc counters") &&
                ok(cudaMalloc(&d_jobs_, sizeof(dev::BatchJob) * nmat_), err, "cudaMalloc jobs") &&
                ok(cudaMalloc(&d_templ_, sizeof(dev::BatchJob) * nmat_), err, "cudaMalloc jobs") &&
                ok(cudaMalloc(&d_items_, sizeof(uint2) * items_cap), err, "cudaMalloc items") &&
                ok(cudaMalloc(&d_order_, sizeof(int32_t) * nmat_), err, "cudaMalloc order") &&
                ok(cudaMalloc(&d_raw, sizeof(oslg_primitive) * std::max(1, nprims)), err, "cudaMalloc prims") &&
                ok(cudaMalloc(&d_ord, sizeof(int32_t) * std::max(1, nprims)), err, "cudaMalloc prims");
    if (good && !smem_heap_)
        good = ok(cudaMalloc(&d_heap_, (size_t)grid_shade_ * heap_b + 16), err, "cudaMalloc shading heap");
    std::vector<dev::BatchJob> templ(nmat_);
    for (int m = 0; m < nmat_; ++m) {
        dev::BatchJob& j = templ[m];
        std::memset(&j, 0, sizeof(j));
        j.blob = static_cast<const uint8_t*>(mats[m]->d_blob);
        j.spec_case = m;
        j.npoints = 0;
        j.userdata = reinterpret_cast<char*>(d_ud_);
        j.outputs = reinterpret_cast<char*>(d_out_);
        auto field = [&](oslg_field& f, int plane) {
            f.data = d_globals_ + (int64_t)plane * cap;
            f.plane_stride = cap;
        };
        field(j.G.P, dev::G_P);
        field(j.G.I, dev::G_I);
        field(j.G.N, dev::G_N);
        field(j.G.Ng, dev::G_NG);
        field(j.G.u, dev::G_U);
        field(j.G.v, dev::G_V);
        field(j.G.dPdu, dev::G_DPDU);
        field(j.G.dPdv, dev::G_DPDV);
    }
    if (good)
        good = ok(cudaMemcpy(d_raw, prims, sizeof(oslg_primitive) * nprims, cudaMemcpyHostToDevice), err, "upload") &&
               ok(cudaMemcpy(d_ord, order.data(), sizeof(int32_t) * nprims, cudaMemcpyHostToDevice), err, "upload") &&
               ok(cudaMemcpy(d_nodes_, nodes.data(), sizeof(dev::WfNode) * nnodes_, cudaMemcpyHostToDevice), err,
                  "upload") &&
               ok(cudaMemcpy(d_templ_, templ.data(), sizeof(dev::BatchJob) * nmat_, cudaMemcpyHostToDevice), err,
                  "upload") &&
               ok(cudaMemcpy(d_order_, morder.data(), sizeof(int32_t) * nmat_, cudaMemcpyHostToDevice), err,
                  "upload") &&
               ok(cudaMemset(d_ctl_, 0, sizeof(uint32_t) * dev::C_SIZE), err, "memset");
    if (good && nprims > 0) {
        dev::k_setup<<<(nprims + 127) / 128, 128>>>(d_raw, d_ord, nprims, d_prims_);
        good = ok(cudaGetLastError(), err, "scene set-up") && ok(cudaDeviceSynchronize(), err, "scene set-up");
    }
    cudaFree(d_raw);
    cudaFree(d_ord);
    if (!good) return OSLG_ERR_CUDA;

    bargs_ = dev::BatchArgs{};
    bargs_.jobs = d_jobs_;
    bargs_.items = d_items_;
    bargs_.nitems = 0;
    bargs_.nitems_dev = d_ctl_ + dev::C_NITEMS;
    bargs_.counter = d_ctl_ + dev::C_COUNTER;
    bargs_.gheap = smem_heap_ ? nullptr : d_heap_;
    bargs_.status = ds.d_status;
    bargs_.textures = ds.d_textures;
    bargs_.ntextures = ds.ntextures;
    bargs_.prog_bytes = prog_bytes;
    bargs_.heap_slots = slots;
    if (jit_dirs) {
        // shading by a persistent kernel specialized to the materials
        int rc = spec_batch_build(mats, jit_dirs[0], jit_dirs[1], &spec_, err);
        if (rc != OSLG_OK) return rc;
        const void* fn = reinterpret_cast<const void*>(spec_.kernel);
        const size_t pool_b = (size_t)spec_.pool_slots * block_ * sizeof(float);
        spec_pool_smem_ = pool_b > 0 && pool_b <= 100 * 1024 ? 1 : 0;
        spec_shmem_ = spec_pool_smem_ ? pool_b : 0;
        if (spec_shmem_ > 48 * 1024 &&
            !ok(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)spec_shmem_), err,
                "specialized kernel attribute"))
            return OSLG_ERR_CUDA;
        int per = 0;
        if (!ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block_, spec_shmem_), err, "occupancy"))
            return OSLG_ERR_CUDA;
        grid_spec_ = ds.sm_count * std::max(1, per);
        if (!spec_pool_smem_ &&
            !ok(cudaMalloc(&d_spec_heap_, (size_t)grid_spec_ * std::max<size_t>(4, pool_b) + 16), err,
                "cudaMalloc shading heap"))
            return OSLG_ERR_CUDA;
        sbargs_ = bargs_;
        sbargs_.gheap = d_spec_heap_;
        sbargs_.heap_slots = spec_.pool_slots;
    }
    for (void*& e : ev_) {
        cudaEvent_t ev;
        if (!ok(cudaEventCreate(&ev), err, "event")) return OSLG_ERR_CUDA;
        e = ev;
    }
    last_.paths = npaths_;
    return OSLG_OK;
}

int Wavefront::enqueue_frame(void* stream, bool profile, std::string* err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    dev::WfArgs a;
    std::memset(&a, 0, sizeof(a));
    a.prims = d_prims_;
    a.nodes = d_nodes_;
    a.st = d_state_;
    a.np = npaths_;
    a.cap = cap_;
    a.ctl = d_ctl_;
    a.act = d_active_;
    a.hit_rec = d_hit_rec_;
    a.hit_t = d_hit_t_;
    a.hit_slot = d_hit_slot_;
    a.gl = d_globals_;
    a.ud = d_ud_;
    a.out = d_out_;
    a.order = d_order_;
    a.templ = d_templ_;
    a.jobs = d_jobs_;
    a.items = d_items_;
    a.nmat = nmat_;
    a.tile = tile_;
    a.spp = opt_.spp;
    a.width = opt_.width;
    a.height = opt_.height;
    // the random stream's seed is hashed once so that nearby seeds decorrelate
    uint32_t sv = opt_.seed * 747796405u + 2891336453u;
    sv = ((sv >> ((sv >> 28u) + 4u)) ^ sv) * 277803737u;
    a.seed = (sv >> 22u) ^ sv;
    a.rr = opt_.rr_survival;
    for (int k = 0; k < 3; ++k) a.bg[k] = opt_.background[k];
    std::memcpy(a.cam, cam_, sizeof(cam_));

    const unsigned g_cam = (unsigned)std::min<int64_t>((npaths_ + 255) / 256, (int64_t)grid_stream_ * 4);
    dev::k_camera<<<std::max(1u, g_cam), 256, 0, s>>>(a);
    if (!ok(cudaGetLastError(), err, "camera launch")) return OSLG_ERR_CUDA;
    std::vector<cudaEvent_t> pev;
    if (profile) {
        for (int k = 0; k < opt_.max_hits * 5 + 1; ++k) {
            cudaEvent_t e;
            if (!ok(cudaEventCreate(&e), err, "event")) return OSLG_ERR_CUDA;
            pev.push_back(e);
        }
        cudaEventRecord(pev[0], s);
    }
    for (int b = 0; b < opt_.max_hits; ++b) {
        const int cur = b & 1;
        dev::k_trace<<<grid_trace_, 256, 0, s>>>(a, cur);
        if (profile) cudaEventRecord(pev[b * 5 + 1], s);
        dev::k_plan<<<1, 1024, 0, s>>>(a, cur, b);
        if (profile) cudaEventRecord(pev[b * 5 + 2], s);
        dev::k_scatter<<<grid_stream_, 256, 0, s>>>(a, cur, b);
        if (profile) cudaEventRecord(pev[b * 5 + 3], s);
        if (!ok(cudaGetLastError(), err, "wavefront launch")) return OSLG_ERR_CUDA;
        if (spec_.kernel) {
            int pool_smem = spec_pool_smem_;
            void* args[] = { &sbargs_, &pool_smem };
            if (!ok(cudaLaunchKernel(reinterpret_cast<const void*>(spec_.kernel), dim3((unsigned)grid_spec_),
                                     dim3((unsigned)block_), args, spec_shmem_, s),
                    err, "specialized shading launch"))
                return OSLG_ERR_CUDA;
        } else if (!ok((cudaError_t)batch_variant_launch(maxt_, ppt_, smem_heap_, (unsigned)grid_shade_,
                                                         (unsigned)block_, shmem_, stream, bargs_),
                       err, "shading launch")) {
            return OSLG_ERR_CUDA;
        }
        if (profile) cudaEventRecord(pev[b * 5 + 4], s);
        dev::k_update<<<grid_stream_, 256, 0, s>>>(a, cur, b, b == opt_.max_hits - 1 ? 1 : 0);
        if (profile) cudaEventRecord(pev[b * 5 + 5], s);
        if (!ok(cudaGetLastError(), err, "wavefront launch")) return OSLG_ERR_CUDA;
    }
    if (d_image_out_) {
        const unsigned g = (unsigned)std::min<int64_t>((npaths_ / opt_.spp + 255) / 256, (int64_t)grid_stream_ * 4);
        dev::k_resolve<<<std::max(1u, g), 256, 0, s>>>(d_state_, npaths_, opt_.spp, d_image_out_);
        if (!ok(cudaGetLastError(), err, "resolve launch")) return OSLG_ERR_CUDA;
    }
    if (d_radiance_out_ &&
        !ok(cudaMemcpyAsync(d_radiance_out_, d_state_ + dev::S_L * npaths_, sizeof(float) * 3 * npaths_,
                            cudaMemcpyDeviceToDevice, s),
            err, "radiance copy"))
        return OSLG_ERR_CUDA;
    if (profile) {
        if (!ok(cudaEventSynchronize(pev.back()), err, "event sync")) return OSLG_ERR_CUDA;
        for (float& x : last_.ms_stage) x = 0.0f;
        for (int b = 0; b < opt_.max_hits; ++b)
            for (int k = 0; k < 5; ++k) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, pev[b * 5 + k], pev[b * 5 + k + 1]);
                last_.ms_stage[k] += ms;
            }
        for (cudaEvent_t e : pev) cudaEventDestroy(e);
    }
    return OSLG_OK;
}

int Wavefront::render(float* d_path_radiance, float* d_image, void* stream, bool profile, std::string* err) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool graph = opt_.use_graph >= 0 && !profile;
    if (d_path_radiance != d_radiance_out_ || d_image != d_image_out_) {
        if (gexec_) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(gexec_));
        if (graph_) cudaGraphDestroy(static_cast<cudaGraph_t>(graph_));
        gexec_ = graph_ = nullptr;
        d_radiance_out_ = d_path_radiance;
        d_image_out_ = d_image;
    }
    if (!ok(cudaEventRecord(static_cast<cudaEvent_t>(ev_[0]), s), err, "event record")) return OSLG_ERR_CUDA;
    if (!graph) {
        int rc = enqueue_frame(stream, profile, err);
        if (rc != OSLG_OK) return rc;
    } else {
        if (!gexec_) {
            cudaStream_t cs;
            if (!ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), err, "capture stream")) return OSLG_ERR_CUDA;
            if (!ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), err, "begin capture")) {
                cudaStreamDestroy(cs);
                return OSLG_ERR_CUDA;
            }
            std::string e2;
            int rc = enqueue_frame(cs, false, &e2);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(cs, &g);
            cudaStreamDestroy(cs);
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
        if (!ok(cudaGraphLaunch(static_cast<cudaGraphExec_t>(gexec_), s), err, "graph launch")) return OSLG_ERR_CUDA;
    }
    if (!ok(cudaEventRecord(static_cast<cudaEvent_t>(ev_[1]), s), err, "event record")) return OSLG_ERR_CUDA;
    return OSLG_OK;
}

int Wavefront::stats(WavefrontStats* out, std::string* err) {
    if (!ok(cudaEventSynchronize(static_cast<cudaEvent_t>(ev_[1])), err, "event sync")) return OSLG_ERR_CUDA;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, static_cast<cudaEvent_t>(ev_[0]), static_cast<cudaEvent_t>(ev_[1]));
    uint32_t h[kWfMaxHits] = {};
    if (!ok(cudaMemcpy(h, d_ctl_ + dev::C_HITS, sizeof(h), cudaMemcpyDeviceToHost), err, "stats copy"))
        return OSLG_ERR_CUDA;
    last_.ms_total = ms;
    last_.total_hits = 0;
    last_.bounces = 0;
    for (int b = 0; b < kWfMaxHits; ++b) {
        last_.hits[b] = b < opt_.max_hits ? h[b] : 0;
        last_.total_hits += last_.hits[b];
        if (last_.hits[b] > 0) last_.bounces = b + 1;
    }
    *out = last_;
    return OSLG_OK;
}

}  // namespace oslg
