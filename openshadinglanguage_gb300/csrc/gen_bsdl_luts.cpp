// Bakes the energy-compensation tables of the BSDL microfacet lobes this
// executor evaluates, the way BSDL's build does (src/libbsdl/src/genluts.cpp:
// the LP-sequence sampler :50-100, compute_E :103-145, bake_emiss_tables
// :147-171): for each table entry the missing energy 1 - E, E the average
// of the lobe's sampled weight over 128 x 128 scrambled (0,2)-sequence
// points, accumulated progressively. Tables, in bake order (a later one reads
// an earlier one):
//   spi::MiniMicrofacetGGX      16 roughness x 16 cosines (cos = (i/15)^2)
//   mtx::DielectricReflFront    32 IOR x 16 roughness x 16 cosines (i/15)
//   mtx::DielectricBothFront    same, reflection + refraction, front side
//   mtx::DielectricBothBack     same, back side (eta inverted)
// The lobes follow src/libbsdl/include/BSDL/microfacet_tools_impl.h (GGXDist,
// Walter's visible-normal sampling, Eto-Tokuyoshi bounded VNDF sampling,
// Turquin's multiple-scattering reflection) and MTX/bsdf_dielectric_impl.h
// (DielectricFresnel, DielectricBSDF eval/sample with bounded visible
// normals for refraction). BSDL's default configuration takes sin/cos from
// the math library here.
//
// usage: gen_bsdl_luts <output .inc>   (built and run by build.py)
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <thread>
#include <vector>

namespace {

struct V3 {
    float x, y, z;
};
V3 v3(float x, float y, float z) { return V3{ x, y, z }; }
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
float length(V3 a) { return std::sqrt(dot(a, a)); }
V3 normalized(V3 a) {
    const float l = length(a);
    return l > 0.0f ? v3(a.x / l, a.y / l, a.z / l) : a;
}
float sqr(float x) { return x * x; }
float clampf(float x, float a, float b) { return std::min(std::max(x, a), b); }
float lerp(float f, float a, float b) {
    f = clampf(f, 0.0f, 1.0f);
    return (1 - f) * a + f * b;
}
const float kPi = 3.14159265358979323846f;

// BSDL's quadrant polynomials (tools.h:201-238, minimax cos/sin of x*pi/4)
// for the concentric disc mapping
float cos_quadrant(float x) {
    const float x2 = x * x;
    float cp = 0.01578646f + -0.00029826362f * x2;
    cp = -0.30837047f + cp * x2;
    cp = 0.99998736f + cp * x2;
    return cp;
}
float sin_quadrant(float x) {
    const float x2 = x * x;
    float sp = 0.0024843954015523195266723632812500f + -0.0000341485538228880614042282104492f * x2;
    sp = -0.0807407423853874206542968750000000f + sp * x2;
    sp = 0.7853975892066955566406250000000000f + sp * x2;
    return sp * x;
}
void square_to_unit_disc(float u, float v, float* x, float* y) {
    const float a = 2 * u - 1, qa = std::fabs(a);
    const float b = 2 * v - 1, qb = std::fabs(b);
    const float rad = qa > qb ? qa : qb;
    const float phi = qa > qb ? qb / qa : ((qa == qb) ? 1.0f : 2 - qa / qb);
    *x = std::copysign(rad * cos_quadrant(phi), a);
    *y = std::copysign(rad * sin_quadrant(phi), b);
}

struct GGX {
    float ax, ay;
    GGX(float rough, float aniso) {
        ax = ay = sqr(rough);
        ax = std::max(ax * (1 + aniso), 1e-5f);
        ay = std::max(ay * (1 - aniso), 1e-5f);
    }
    float D(V3 h) const {
        const float cp = sqr(h.x / ax), sp = sqr(h.y / ay), c2 = sqr(h.z);
        return 1.0f / (kPi * ax * ay * sqr(c2 + (cp + sp)));
    }
    float G1(V3 w) const {
        w = v3(w.x * ax, w.y * ay, w.z);
        return 2.0f * w.z / (w.z + length(w));
    }
    float G2_G1(V3 wi, V3 wo) const {
        wi = v3(wi.x * ax, wi.y * ay, wi.z);
        wo = v3(wo.x * ax, wo.y * ay, wo.z);
        const float nl = length(wi), nv = length(wo);
        return wi.z * (wo.z + nv) / (wo.z * nl + wi.z * nv);
    }
    V3 sample(V3 wo, float u, float v) const {  // Walter's ellipsoidal visible normals
        const V3 V = normalized(v3(ax * wo.x, ay * wo.y, wo.z));
        const V3 T1 = V.z < 0.9999f ? normalized(v3(V.y, -V.x, 0)) : v3(1, 0, 0);
        const V3 T2 = cross(T1, V);
        float px, py;
        square_to_unit_disc(u, v, &px, &py);
        const float s = 0.5f * (1 + V.z);
        const float p2o = s * py + (1 - s) * std::sqrt(1 - px * px);
        const float p3 = std::sqrt(std::max(1.0f - sqr(px) - sqr(p2o), 0.0f));
        const V3 N = add(add(mul(T1, px), mul(T2, p2o)), mul(V, p3));
        return normalized(v3(ax * N.x, ay * N.y, std::max(N.z, 0.0f)));
    }
    V3 sample_for_refl(V3 wo, float u, float v) const {  // Eto-Tokuyoshi bounded VNDF
        const V3 i_std = normalized(v3(wo.x * ax, wo.y * ay, wo.z));
        const float phi = 2.0f * kPi * u;
        const float a = clampf(std::min(ax, ay), 0.0f, 1.0f);
        const float s = 1 + std::sqrt(sqr(wo.x) + sqr(wo.y));
        const float a2 = sqr(a), s2 = sqr(s);
        const float k = (1 - a2) * s2 / (s2 + a2 * sqr(wo.z));
        const float b = k * i_std.z;
        const float z = (1 - v) * (1 + b) - b;
        const float st = std::sqrt(clampf(1 - sqr(z), 0.0f, 1.0f));
        const V3 o_std = v3(st * std::cos(phi), st * std::sin(phi), z);
        const V3 m_std = add(i_std, o_std);
        return normalized(v3(m_std.x * ax, m_std.y * ay, m_std.z));
    }
    float D_refl_D(V3 wo) const {
        const float len2 = sqr(wo.x * ax) + sqr(wo.y * ay);
        const float t = std::sqrt(len2 + sqr(wo.z));
        const float a = clampf(std::min(ax, ay), 0.0f, 1.0f);
        const float s = 1 + std::sqrt(sqr(wo.x) + sqr(wo.y));
        const float a2 = sqr(a), s2 = sqr(s);
        const float k = (1 - a2) * s2 / (s2 + a2 * sqr(wo.z));
        return 2 * wo.z / (k * wo.z + t);
    }
    float roughness() const { return std::max(ax, ay); }
};

V3 reflect(V3 E, V3 N) { return add(mul(N, 2 * dot(N, E)), mul(E, -1.0f)); }
V3 refract(V3 E, V3 N, float eta) {
    if (eta == 0) return v3(0, 0, 0);
    float cosi = dot(E, N), neta;
    V3 Nn = N;
    if (cosi > 0) {
        neta = 1 / eta;
    } else {
        cosi = -cosi;
        neta = eta;
        Nn = mul(N, -1.0f);
    }
    const float arg = 1 - (neta * neta * (1 - (cosi * cosi)));
    if (arg >= 0) {
        const float dnp = std::sqrt(arg);
        const float nK = (neta * cosi) - dnp;
        return normalized(add(mul(E, -neta), mul(Nn, nK)));
    }
    return v3(0, 0, 0);
}

struct Fresnel {
    float eta;
    Fresnel(float e, bool backside) {
        if (backside) e = 1 / e;
        eta = e >= 1 ? clampf(e, 1.001f, 5.0f) : clampf(e, 1 / 5.0f, 1 / 1.001f);
    }
    float eval(float c) const {
        float g = (eta - 1.0f) * (eta + 1.0f) + c * c;
        if (g > 0) {
            g = std::sqrt(g);
            const float A = (g - c) / (g + c);
            const float B = (c * (g + c) - 1) / (c * (g - c) + 1);
            return 0.5f * A * A * (1 + B * B);
        }
        return 1.0f;
    }
    static Fresnel from_table_index(float tx, bool backside) {
        return Fresnel(lerp(sqr(tx), 1.001f, 5.0f), backside);
    }
};

// a baked table: [f][r][c], Nc cosines with cosine(i)
struct Table {
    int nf, nr, nc;
    bool squared;  // cosines (i/(nc-1))^2, else i/(nc-1)
    std::vector<float> e;
    float cosine(int i) const {
        const float t = float(i) * (1.0f / (nc - 1));
        return std::max(squared ? sqr(t) : t, 1e-6f);
    }
    float interpolate(float roughness, float fresnel_index, int i) const {
        float rf = roughness * (nr - 1);
        const int ra = (int)rf, rb = std::min(ra + 1, nr - 1);
        rf -= ra;
        if (nf == 1) return lerp(rf, e[ra * nc + i], e[rb * nc + i]);
        float ff = fresnel_index * (nf - 1);
        const int fa = (int)ff, fb = std::min(fa + 1, nf - 1);
        ff -= fa;
        return lerp(ff, lerp(rf, e[(fa * nr + ra) * nc + i], e[(fa * nr + rb) * nc + i]),
                    lerp(rf, e[(fb * nr + ra) * nc + i], e[(fb * nr + rb) * nc + i]));
    }
    float eval(float roughness, float fresnel_index, float c) const {
        float cos0 = cosine(0);
        if (c <= cos0) return interpolate(roughness, fresnel_index, 0);
        for (int i = 1; i < nc; ++i) {
            const float cos1 = cosine(i);
            if (c < cos1) {
                const float q = (c - cos0) / (cos1 - cos0);
                return lerp(q, interpolate(roughness, fresnel_index, i - 1), interpolate(roughness, fresnel_index, i));
            }
            cos0 = cos1;
        }
        return interpolate(roughness, fresnel_index, nc - 1);
    }
};

Table g_mini{ 1, 16, 16, true, std::vector<float>(256, 0.0f) };

// the sampled weight of one table lobe (0: MiniMicrofacetGGX, 1: reflection
// front, 2: both front, 3: both back)
float sample_weight(int kind, float cosNO, float rough_index, float fresnel_index, float u, float v, float w) {
    const V3 wo = v3(std::sqrt(1 - sqr(cosNO)), 0, cosNO);
    const GGX d(rough_index, 0.0f);
    if (kind == 0) {
        const V3 m = d.sample(wo, u, v);
        if (dot(m, wo) > 0) {
            const V3 wi = reflect(wo, m);
            if (wi.z > 0) return d.G2_G1(wi, wo);
        }
        return 0.0f;
    }
    const Fresnel f = Fresnel::from_table_index(fresnel_index, kind == 3);
    if (kind == 1) {  // Turquin multiple-scattering reflection
        const float E_ms = g_mini.eval(rough_index, 0.0f, cosNO);
        if (wo.z <= 0) return 0.0f;
        const V3 m = d.sample_for_refl(wo, u, v);
        const V3 wi = reflect(wo, m);
        if (wi.z <= 0) return 0.0f;
        const V3 h = normalized(add(wo, wi));
        const float cosMO = dot(h, wo);
        const float G1 = d.G1(wo);
        const float out = d.G2_G1(wi, wo) * G1 / d.D_refl_D(wo);
        const float F = f.eval(cosMO);
        const float msf = E_ms / std::max(0.01f, 1 - E_ms);
        return out * F * (1 + F * msf);
    }
    // reflection + refraction, bounded visible normals
    const V3 m = d.sample_for_refl(wo, u, v);
    const float cosMO = dot(wo, m);
    if (cosMO <= 0) return 0.0f;
    const float Fm = f.eval(cosMO);
    const bool refl = w < Fm;
    const V3 wi = refl ? reflect(wo, m) : refract(wo, m, f.eta);
    if ((refl && wi.z <= 0) || (!refl && wi.z >= 0)) return 0.0f;
    if (wi.z > 0) {
        const V3 h = normalized(add(wo, wi));
        const float cMO = dot(h, wo);
        if (cMO <= 0) return 0.0f;
        const float G1 = d.G1(wo);
        const float F = f.eval(cMO);
        if (F <= 0) return 0.0f;
        return F * (d.G2_G1(wi, wo) * G1 / (d.D_refl_D(wo) * F));
    }
    const V3 Ht = mul(normalized(add(mul(wi, f.eta), wo)), f.eta > 1 ? -1.0f : 1.0f);
    const float cosHO = dot(Ht, wo), cosHI = dot(Ht, wi);
    if (cosHO <= 0 || cosHI >= 0) return 0.0f;
    const float Ft = 1.0f - f.eval(cosHO);
    if (Ht.z <= 0 || Ft <= 0) return 0.0f;
    const float G1 = d.G1(wo);
    return Ft * (d.G2_G1(v3(wi.x, wi.y, -wi.z), wo) * G1 / (d.D_refl_D(wo) * Ft));
}

// genluts' sampler: the scrambled (0,2)-sequence of Larcher and Pillichshammer
uint32_t ri_lp(uint32_t i) {
    uint32_t r = 0;
    for (uint32_t v = 1u << 31; i; i >>= 1, v |= v >> 1)
        if (i & 1) r ^= v;
    return r;
}
uint32_t ri_lp_inv(uint32_t i) {
    uint32_t r = 0;
    for (uint32_t v = 3u << 30; i; i >>= 1, v >>= 1)
        if (i & 1) r ^= v;
    return r;
}
void lp_sample(int si, int AA, uint32_t sx, uint32_t sy, uint32_t sz, float* o) {
    const uint32_t ex = (uint32_t)(si % AA), ey = (uint32_t)(si / AA);
    const uint32_t upper = (ex ^ (sx >> 16)) << 16;
    const uint32_t lp_upper = ri_lp(upper) ^ sy;
    const uint32_t delta = (ey << 16) ^ (lp_upper & 0xFFFF0000u);
    const uint32_t lower = ri_lp_inv(delta);
    const uint32_t index = upper | lower;
    const uint32_t x = index ^ sx, y = lp_upper ^ delta;
    const float jx = (x & 65535) * (1 / 65536.0f), jy = (y & 65535) * (1 / 65536.0f);
    uint32_t rz = sz, ii = index;
    for (uint64_t v2 = uint64_t(3) << 62; ii; ii >>= 1, v2 ^= v2 >> 1)
        if (ii & 1) rz ^= uint32_t(v2 >> 31);
    o[0] = (ex + jx) / AA;
    o[1] = (ey + jy) / AA;
    o[2] = rz * 2.3283063e-10f;
}
uint64_t fh_mix(uint64_t h) {
    h ^= h >> 23;
    h *= 0x2127599bf4325c37ULL;
    h ^= h >> 47;
    return h;
}
uint32_t randhash3(uint32_t x, uint32_t y, uint32_t z) {  // fasthash64 of two words
    const uint64_t m = 0x880355f21e6d1965ULL;
    uint64_t h = (2 * sizeof(uint64_t)) * m;
    const uint64_t buf[2] = { (uint64_t(x) << 32) + y, uint64_t(z) };
    for (uint64_t v : buf) {
        h ^= fh_mix(v);
        h *= m;
    }
    return (uint32_t)fh_mix(h);
}

float compute_E(int kind, float cosNO, float r, float f, uint32_t fi, uint32_t ri) {
    const int AA = 128, N = AA * AA;
    const uint32_t sx = randhash3(fi, ri, 0), sy = randhash3(fi, ri, 1), sz = randhash3(fi, ri, 2);
    float E = 0.0f;
    float rnd[3];
    for (int i = 0; i < N; ++i) {
        lp_sample(i, AA, sx, sy, sz, rnd);
        const float out = sample_weight(kind, cosNO, r, f, rnd[0], rnd[1], rnd[2]);
        E = lerp(1.0f / (1.0f + i), E, out);
    }
    return std::min(E, 1.0f);
}

void bake(int kind, Table& t) {
    const int nthreads = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> pool;
    for (int th = 0; th < nthreads; ++th)
        pool.emplace_back([&, th]() {
            for (int f = th; f < t.nf; f += nthreads) {
                const float fi = float(f) * (1.0f / std::max(1, t.nf - 1));
                for (int r = 0; r < t.nr; ++r) {
                    const float ri = t.nr > 1 ? float(r) * (1.0f / (t.nr - 1)) : 0.0f;
                    for (int c = 0; c < t.nc; ++c)
                        t.e[(f * t.nr + r) * t.nc + c] =
                            1 - compute_E(kind, t.cosine(c), ri, fi, (uint32_t)f, (uint32_t)r);
                }
            }
        });
    for (std::thread& th : pool) th.join();
}

void emit(FILE* out, const char* name, const Table& t) {
    std::fprintf(out, "OSLG_LUT_QUAL float %s[%zu] = {\n", name, t.e.size());
    for (size_t i = 0; i < t.e.size(); ++i)
        std::fprintf(out, "%af,%s", t.e[i], (i % 8 == 7) ? "\n" : " ");  // hexadecimal: exact
    std::fprintf(out, "};\n");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s output.inc\n", argv[0]);
        return 1;
    }
    bake(0, g_mini);  // the dielectric reflection table reads this one
    Table refl{ 32, 16, 16, false, std::vector<float>(32 * 16 * 16) };
    Table front = refl, back = refl;
    bake(1, refl);
    bake(2, front);
    bake(3, back);
    FILE* out = std::fopen(argv[1], "w");
    if (!out) return 1;
    std::fprintf(out, "// generated by gen_bsdl_luts.cpp (BSDL energy-compensation tables)\n");
    emit(out, "kLutMiniGGX", g_mini);
    emit(out, "kLutDielReflFront", refl);
    emit(out, "kLutDielBothFront", front);
    emit(out, "kLutDielBothBack", back);
    std::fclose(out);
    return 0;
}
