"""The benchmark workloads: shader groups and seeded synthetic inputs.

C1  fbm_cell        single-layer fBm + hashed cell id, 1024x1024 grid
C2  layered_closure 3-layer pattern -> ramp -> closure group with BSDF eval,
                    2048x2048 grid
C3  random groups   64 seeded random op DAGs of 20-200 ops with noise,
                    transforms, if/else and data-dependent loops; point
                    counts log-uniform in [1K, 1M], P uniform in [-10,10]^3
C5  materials       16 seeded 2-4 layer material groups (noise patterns,
                    tint, a closure sum of diffuse / oren_nayar / GGX
                    microfacet / BSDL dielectric_bsdf (IOR 1.3-1.7) /
                    sheen / emission) with a BSDF sample output for the
                    wavefront path tracer
"""
import numpy as np

from . import shaders
from .shadingsys import (SymArenaOutputs, SymLocationDesc, TypeClosure, TypeColor, TypeInt, TypeDesc)
from ._capi import BASE_FLOAT, AGG_VEC3, VEC_COLOR

# ---- C2 ------------------------------------------------------------------------------
C2_CLOSURE_RECORDS = 2                       # components kept per point
C2_CLOSURE_BYTES = 4 + 64 * C2_CLOSURE_RECORDS  # [count][id, w.rgb, params x12] ...
C2_EVAL_OFFSET = C2_CLOSURE_BYTES
C2_STRIDE = C2_CLOSURE_BYTES + 16             # + {w.rgb, pdf}
C2_LIGHT = (0.5773502691896258, 0.5773502691896258, 0.5773502691896258)


def c2_group(ss):
    """Layer A c2_pattern -> layer B c2_ramp (x <- A.a) -> layer C c2_surface
    (a <- A.a, tint <- B.Cout); Ci stored as closure records and evaluated
    as a BSDF at the fixed light direction normalize(1,1,1)."""
    ss.LoadMemoryCompiledShader("c2_pattern", shaders.c2_pattern())
    ss.LoadMemoryCompiledShader("c2_ramp", shaders.c2_ramp())
    ss.LoadMemoryCompiledShader("c2_surface", shaders.c2_surface())
    g = ss.ShaderGroupBegin("layered_closure")
    ss.Shader(g, "surface", "c2_pattern", "A")
    ss.Parameter(g, "knots", TypeDesc(BASE_FLOAT, AGG_VEC3, VEC_COLOR, 8), shaders.c2_knots())
    ss.Shader(g, "surface", "c2_ramp", "B")
    ss.ConnectShaders(g, "A", "a", "B", "x")
    ss.Shader(g, "surface", "c2_surface", "C")
    ss.ConnectShaders(g, "A", "a", "C", "a")
    ss.ConnectShaders(g, "B", "Cout", "C", "tint")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [SymLocationDesc("C.Ci", TypeClosure.array(C2_CLOSURE_RECORDS), False, SymArenaOutputs, 0,
                                       C2_STRIDE)])
    ss.bsdf_eval_output(g, "C.Ci", C2_LIGHT, C2_EVAL_OFFSET, C2_STRIDE)
    return g


def c2_inputs(W, H, seed=0xC2):
    """u, v on testshade's default grid; I = -V with V uniform on the upper
    hemisphere (z = xi1, phi = 2*pi*xi2), so wo = -I faces the viewer."""
    x = np.arange(W, dtype=np.float32)
    y = np.arange(H, dtype=np.float32)
    u = (x / np.float32(max(1, W - 1))).astype(np.float32)
    v = (y / np.float32(max(1, H - 1))).astype(np.float32)
    uu = np.broadcast_to(u[None, :], (H, W)).ravel().copy()
    vv = np.broadcast_to(v[:, None], (H, W)).ravel().copy()
    rng = np.random.default_rng(seed)
    xi = rng.random((2, W * H))
    z = xi[0]
    phi = 2.0 * np.pi * xi[1]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    V = np.stack([r * np.cos(phi), r * np.sin(phi), z]).astype(np.float32)
    I = (-V).astype(np.float32)
    return uu, vv, np.ascontiguousarray(I)


def c2_globals(make_globals, u, v, I):
    return make_globals(u=u, v=v, I=I, N=(0.0, 0.0, 1.0), Ng=(0.0, 0.0, 1.0), dPdu=(1.0, 0.0, 0.0),
                        dPdv=(0.0, 1.0, 0.0))


# ---- C3 ------------------------------------------------------------------------------
C3_SEED = 0xC3
C3_GROUPS = 64
C3_REC = 4  # Cout.rgb, Fout


class _RandomShader:
    """Builds one random shader as a stream of OSL statements over a pool of
    float, vector and matrix variables. Statements only read variables
    assigned in an enclosing scope, so every value a point reads was written
    for that point (no dependence on heap contents)."""

    NOISE_KINDS = (("perlin", 0.28), ("uperlin", 0.1), ("simplex", 0.22), ("usimplex", 0.05), ("cell", 0.25),
                   ("gabor", 0.10))

    def __init__(self, name, rng, target_ops):
        from .oso import OsoBuilder
        self.b = b = OsoBuilder(name)
        self.rng = rng
        self.target = target_ops
        self.Cout = b.param("color", "Cout", [0, 0, 0], output=True)
        self.Fout = b.param("float", "Fout", 0.0, output=True)
        self.mats = []
        for k in range(3):
            m = rng.uniform(-1.0, 1.0, (4, 4))
            m[:3, :3] += 1.5 * np.eye(3)
            m[3, :3] *= 0.5
            m[:3, 3] = 0.0
            m[3, 3] = 1.0
            self.mats.append(b.param("matrix", "M%d" % k, [float(np.float32(x)) for x in m.ravel()]))
        P = b.glob("point", "P")
        self.F, self.V = [], []
        self.V.append(P)
        for c in range(3):
            f = self.newf()
            b.op("compref", f, P, b.const("int", c))
            self.F.append(f)

    def c(self, x):
        return self.b.const("float", float(np.float32(x)))

    def newf(self):
        return self.b.tmp("float")

    def newv(self):
        return self.b.tmp("vector")

    def nops(self):
        return len(self.b.ops)

    def pickf(self, pool):
        return pool[self.rng.integers(len(pool))]

    # -- statements ------------------------------------------------------------------------
    def st_farith(self, F, V):
        b, r = self.b, self.rng
        x, y, f = self.pickf(F), self.pickf(F), self.newf()
        k = r.integers(4)
        if k == 3:
            t, d = self.newf(), self.newf()
            b.op("abs", t, y)
            b.op("add", d, t, self.c(0.5))
            b.op("div", f, x, d)
        else:
            b.op(("add", "sub", "mul")[k], f, x, y)
        F.append(f)

    def st_varith(self, F, V):
        b, r = self.b, self.rng
        x, v = self.pickf(V), self.newv()
        k = r.integers(4)
        if k == 3:
            b.op("mul", v, x, self.pickf(F))
        else:
            b.op(("add", "sub", "mul")[k], v, x, self.pickf(V))
        V.append(v)

    def st_unary(self, F, V):
        b, r = self.b, self.rng
        x, f = self.pickf(F), self.newf()
        k = r.integers(6)
        if k < 4:
            b.op(("sin", "cos", "abs", "floor")[k], f, x)
        elif k == 4:
            t = self.newf()
            b.op("abs", t, x)
            b.op("sqrt", f, t)
        else:
            t, u = self.newf(), self.newf()
            b.op("abs", t, x)
            b.op("neg", u, t)
            b.op("exp", f, u)
        F.append(f)

    def st_vector(self, F, V):
        b, r = self.b, self.rng
        k = r.integers(6)
        a, c = self.pickf(V), self.pickf(V)
        if k == 0:
            f = self.newf(); b.op("dot", f, a, c); F.append(f)
        elif k == 1:
            f = self.newf(); b.op("length", f, a); F.append(f)
        elif k == 2:
            v = self.newv(); b.op("normalize", v, a); V.append(v)
        elif k == 3:
            v = self.newv(); b.op("cross", v, a, c); V.append(v)
        elif k == 4:
            t, v = self.newf(), self.newv()
            b.op("clamp", t, self.pickf(F), self.c(0.0), self.c(1.0))
            b.op("mix", v, a, c, t)
            V.append(v)
        else:
            v = self.newv(); b.op("max", v, a, c); V.append(v)

    def st_matrix(self, F, V):
        b, r = self.b, self.rng
        k = r.integers(4)
        M = self.mats[r.integers(len(self.mats))]
        if k == 3:
            M2 = self.mats[r.integers(len(self.mats))]
            Mm = b.tmp("matrix")
            b.op("mul", Mm, M, M2)
            M = Mm
            k = r.integers(3)
        src = self.pickf(V)
        if k == 0:
            pt, v = b.tmp("point"), b.tmp("point")
            b.op("point", pt, src)
            b.op("transform", v, M, pt)
        elif k == 1:
            v = self.newv()
            b.op("transformv", v, M, src)
        else:
            nn, v = b.tmp("normal"), b.tmp("normal")
            b.op("normal", nn, src)
            b.op("transformn", v, M, nn)
        V.append(v)

    def noise_kind(self, allow_gabor=True):
        names = [k for k, _ in self.NOISE_KINDS if allow_gabor or k != "gabor"]
        w = np.array([p for k, p in self.NOISE_KINDS if allow_gabor or k != "gabor"])
        return names[self.rng.choice(len(names), p=w / w.sum())]

    def st_noise(self, F, V, depth=0, loop=False):
        b, r = self.b, self.rng
        kind = self.noise_kind(allow_gabor=not loop)
        src, sc = self.pickf(V), b.tmp("point")
        b.op("mul", sc, src, self.c(r.uniform(0.2, 2.5)))
        if r.random() < 0.6:
            f = self.newf()
            b.op("noise", f, b.const("string", kind), sc)
            F.append(f)
        else:
            v = self.newv()
            b.op("noise", v, b.const("string", kind), sc)
            V.append(v)

    def block(self, F, V, n, depth, loop):
        for _ in range(n):
            if self.nops() >= self.target:
                return
            self.statement(F, V, depth, loop)

    def st_if(self, F, V, depth, loop):
        b, r = self.b, self.rng
        f, cond = self.newf(), b.tmp("int")
        src, sc = self.pickf(V), b.tmp("point")
        b.op("mul", sc, src, self.c(r.uniform(0.3, 1.5)))
        b.op("noise", f, b.const("string", "uperlin" if r.random() < 0.5 else "cell"), sc)
        b.op("gt", cond, f, self.c(r.uniform(0.3, 0.7)))
        acc_f, acc_v = self.pickf(F), self.pickf(V)
        with b.if_(cond) as br:
            F2, V2 = list(F), list(V)
            self.block(F2, V2, int(r.integers(1, 4)), depth + 1, loop)
            b.op("add", acc_f, acc_f, self.pickf(F2))
            b.op("add", acc_v, acc_v, self.pickf(V2))
            br.else_()
            F3, V3 = list(F), list(V)
            self.block(F3, V3, int(r.integers(1, 3)), depth + 1, loop)
            b.op("sub", acc_f, acc_f, self.pickf(F3))

    def st_loop(self, F, V, depth):
        """for (i = 0; i < n; ++i) with n = 1 + int(15.99 * cellnoise(p)):
        a data-dependent trip count in [1, 16]."""
        b, r = self.b, self.rng
        cn, t, nf = self.newf(), self.newf(), self.newf()
        n, i, cond = b.tmp("int"), b.tmp("int"), b.tmp("int")
        sc = b.tmp("point")
        b.op("mul", sc, self.pickf(V), self.c(r.uniform(0.5, 3.0)))
        b.op("cellnoise", cn, sc)
        b.op("mul", t, cn, self.c(15.99))
        b.op("add", nf, t, self.c(1.0))
        b.op("assign", n, nf)
        acc_f, acc_v = self.pickf(F), self.pickf(V)
        p = self.newv()
        b.op("assign", p, self.pickf(V))
        with b.loop("for", cond) as L:
            b.op("assign", i, b.const("int", 0))
            L.cond()
            b.op("lt", cond, i, n)
            L.body()
            F2, V2 = list(F) + [acc_f], list(V) + [p, acc_v]
            self.block(F2, V2, int(r.integers(2, 5)), depth + 1, True)
            b.op("add", acc_f, acc_f, self.pickf(F2))
            b.op("add", acc_v, acc_v, self.pickf(V2))
            b.op("mul", p, p, self.c(1.7))
            b.op("add", p, p, self.c(0.37))
            L.step()
            b.op("add", i, i, b.const("int", 1))

    def statement(self, F, V, depth=0, loop=False):
        r = self.rng
        kinds = ["farith", "varith", "unary", "vector", "matrix", "noise"]
        w = [0.18, 0.16, 0.12, 0.14, 0.12, 0.18]
        if depth < 2:
            kinds += ["if", "loop"] if not loop else ["if"]
            w += [0.06, 0.04] if not loop else [0.06]
        w = np.array(w) / np.sum(w)
        k = kinds[r.choice(len(kinds), p=w)]
        if k == "if":
            self.st_if(F, V, depth, loop)
        elif k == "loop":
            self.st_loop(F, V, depth)
        elif k == "noise":
            self.st_noise(F, V, depth, loop)
        else:
            getattr(self, "st_" + k)(F, V)

    def build(self):
        b = self.b
        while self.nops() < self.target:
            self.statement(self.F, self.V)
        # outputs: a colour from the last vectors and a float from the last floats
        v = self.newv()
        b.op("add", v, self.V[-1], self.V[-2] if len(self.V) > 1 else self.V[-1])
        b.op("assign", self.Cout, v)
        f = self.newf()
        b.op("add", f, self.F[-1], self.F[-2] if len(self.F) > 1 else self.F[-1])
        b.op("assign", self.Fout, f)
        return b.text()


def c3_specs(seed=C3_SEED, ngroups=C3_GROUPS, min_points=1000, max_points=1000000):
    """Per group: (name, oso text, point count, op count target). Target op
    counts are uniform in [20, 200]; point counts log-uniform in
    [min_points, max_points]."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(ngroups):
        target = int(rng.integers(20, 201))
        npts = int(np.exp(rng.uniform(np.log(min_points), np.log(max_points))))
        name = "c3_g%02d" % k
        oso = _RandomShader(name, np.random.default_rng([seed, k]), target).build()
        specs.append((name, oso, npts, target))
    return specs


def c3_group(ss, name, oso):
    ss.LoadMemoryCompiledShader(name, oso)
    g = ss.ShaderGroupBegin(name + "_group")
    ss.Shader(g, "surface", name, "L")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [SymLocationDesc("L.Cout", TypeColor, False, SymArenaOutputs, 0, 4 * C3_REC),
                       SymLocationDesc("L.Fout", TypeDesc(BASE_FLOAT), False, SymArenaOutputs, 12, 4 * C3_REC)])
    return g


def c3_points(k, npts, seed=C3_SEED):
    """P uniform in [-10, 10]^3 from the group's own stream, SoA (3, n)."""
    rng = np.random.default_rng([seed, 0x50, k])
    return rng.uniform(-10.0, 10.0, (3, npts)).astype(np.float32)


# ---- C5 ------------------------------------------------------------------------------
C5_SEED = 0xC5
C5_MATERIALS = 16
C5_IN_FLOATS = 9    # rx, ry, rz, path weight rgb, absorb, ray roughness, backfacing
C5_OUT_FLOATS = 11  # wi xyz, weight rgb, pdf, Le rgb, roughness


def _c5_pattern(name, kind, freq):
    from .oso import OsoBuilder
    b = OsoBuilder(name)
    a = b.param("float", "a", 0.0, output=True)
    P = b.glob("point", "P")
    p = b.tmp("point")
    b.op("mul", p, P, b.const("float", float(np.float32(freq))))
    if kind == "cell":
        b.op("cellnoise", a, p)
    else:
        b.op("noise", a, b.const("string", kind), p)
    return b.text()


def _c5_tint(name, c0, c1):
    from .oso import OsoBuilder
    b = OsoBuilder(name)
    x = b.param("float", "x", 0.5)
    tint = b.param("color", "tint", [1, 1, 1], output=True)
    b.op("mix", tint, b.const("color", [float(np.float32(v)) for v in c0]),
         b.const("color", [float(np.float32(v)) for v in c1]), x)
    return b.text()


def _c5_surface(name, lobes):
    """lobes: list of (kind, weight, extra) with kind in diffuse, oren_nayar,
    ggx, dielectric, sheen, emission; the closure sum is Ci."""
    from .oso import OsoBuilder
    b = OsoBuilder(name, "surface")
    a = b.param("float", "a", 0.5)
    r = b.param("float", "r", 0.5)
    tint = b.param("color", "tint", [1, 1, 1])
    Ci = b.glob("closure color", "Ci")
    N, dPdu = b.glob("normal", "N"), b.glob("vector", "dPdu")
    c = lambda x: b.const("float", float(np.float32(x)))
    acc = None
    for kind, weight, extra in lobes:
        cl, w, cw = b.tmp("closure color"), b.tmp("color"), b.tmp("closure color")
        if kind == "diffuse":
            b.op("closure", cl, b.const("string", "diffuse"), N)
        elif kind == "oren_nayar":
            b.op("closure", cl, b.const("string", "oren_nayar"), N, c(extra))
        elif kind == "sheen":  # sheen_bsdf(N, albedo, roughness): albedo from the tint
            b.op("closure", cl, b.const("string", "sheen_bsdf"), N, tint, c(extra))
        elif kind == "ggx":
            alpha, t = b.tmp("float"), b.tmp("float")
            b.op("mul", t, c(0.6), r)
            b.op("add", alpha, c(0.05), t)
            b.op("closure", cl, b.const("string", "microfacet"), b.const("string", "ggx"), N, dPdu, alpha, alpha,
                 c(1.5), b.const("int", 0))
        elif kind == "dielectric":  # dielectric_bsdf(N, U, reflection, transmission, rx, ry, ior, "ggx")
            alpha, t = b.tmp("float"), b.tmp("float")
            b.op("mul", t, c(0.6), r)
            b.op("add", alpha, c(0.05), t)
            one = b.const("color", [1.0, 1.0, 1.0])
            b.op("closure", cl, b.const("string", "dielectric_bsdf"), N, dPdu, one, one, alpha, alpha, c(extra),
                 b.const("string", "ggx"))
        else:  # emission, modulated by the pattern
            b.op("closure", cl, b.const("string", "emission"))
        tw = b.tmp("color")
        b.op("mul", tw, tint, c(weight))
        if kind == "emission":
            b.op("mul", w, tw, a)
            b.op("mul", w, w, c(extra))
        else:
            b.op("assign", w, tw)
        b.op("mul", cw, cl, w)
        if acc is None:
            acc = cw
        else:
            s2 = b.tmp("closure color")
            b.op("add", s2, acc, cw)
            acc = s2
    b.op("assign", Ci, acc)
    return b.text()


def c5_material_specs(seed=C5_SEED, n=C5_MATERIALS):
    """Per material: pattern layers (kind, frequency), tint colours or None,
    and the closure lobes. Two materials emit."""
    rng = np.random.default_rng([seed, 0x11])
    specs = []
    for k in range(n):
        nl = int(rng.integers(2, 5))  # 2..4 layers
        pats = [(str(rng.choice(["usimplex", "uperlin", "cell"])), float(rng.uniform(0.5, 4.0)))]
        if nl >= 3:
            pats.append((str(rng.choice(["usimplex", "uperlin"])), float(rng.uniform(1.0, 8.0))))
        tint = None
        if nl == 4:
            tint = (tuple(rng.uniform(0.1, 0.9, 3)), tuple(rng.uniform(0.1, 0.9, 3)))
        if k in (3, 11):
            lobes = [("emission", 1.0, float(rng.uniform(2.0, 8.0))), ("diffuse", 0.5, 0.0)]
        else:
            base = str(rng.choice(["diffuse", "oren_nayar"]))
            lobes = [(base, float(rng.uniform(0.4, 0.8)), float(rng.uniform(0.0, 0.5)))]
            extra = str(rng.choice(["ggx", "dielectric", "none"]))
            if extra != "none":
                lobes.append((extra, float(rng.uniform(0.2, 0.6)), float(rng.uniform(1.3, 1.7))))
            if k % 3 == 1:  # sheen on every third material
                lobes.append(("sheen", float(rng.uniform(0.3, 0.8)), float(rng.uniform(0.1, 0.9))))
            if rng.random() < 0.3:
                lobes.append(("oren_nayar" if base == "diffuse" else "diffuse", 0.2, float(rng.uniform(0.0, 0.5))))
        specs.append((pats, tint, lobes))
    return specs


def c5_material_group(ss, k, spec, out_offset=0, out_stride=4 * C5_OUT_FLOATS, in_offset=0,
                      in_stride=4 * C5_IN_FLOATS):
    """Build material k: pattern layer(s) -> optional tint -> surface; the
    surface's Ci is sampled per point (bsdf_sample_output)."""
    pats, tint, lobes = spec
    tag = "c5m%02d" % k
    g = ss.ShaderGroupBegin(tag)
    for i, (kind, freq) in enumerate(pats):
        nm = "%s_p%d" % (tag, i)
        ss.LoadMemoryCompiledShader(nm, _c5_pattern(nm, kind, freq))
        ss.Shader(g, "surface", nm, "P%d" % i)
    if tint is not None:
        nm = tag + "_tint"
        ss.LoadMemoryCompiledShader(nm, _c5_tint(nm, tint[0], tint[1]))
        ss.Shader(g, "surface", nm, "T")
        ss.ConnectShaders(g, "P0", "a", "T", "x")
    nm = tag + "_surf"
    ss.LoadMemoryCompiledShader(nm, _c5_surface(nm, lobes))
    ss.Shader(g, "surface", nm, "S")
    ss.ConnectShaders(g, "P0", "a", "S", "a")
    ss.ConnectShaders(g, "P%d" % (len(pats) - 1), "a", "S", "r")
    if tint is not None:
        ss.ConnectShaders(g, "T", "tint", "S", "tint")
    ss.ShaderGroupEnd(g)
    ss.bsdf_sample_output(g, "S.Ci", out_offset, out_stride, in_offset, in_stride)
    return g


def c5_hits(n, seed=0xC5A):
    """Seeded hit records for sampling tests: P in [-5, 5]^3, unit N facing
    the incoming direction, dPdu orthogonal to N, random inputs of the
    sample step (rx, ry, rz in [0, 1), path weight in [0.2, 1], absorb 0/1,
    ray roughness, backfacing 0/1)."""
    rng = np.random.default_rng(seed)
    P = rng.uniform(-5, 5, (3, n)).astype(np.float32)
    N = rng.normal(size=(3, n))
    N /= np.linalg.norm(N, axis=0)
    I = rng.normal(size=(3, n))
    I /= np.linalg.norm(I, axis=0)
    flip = np.sum(I * N, axis=0) > 0
    I[:, flip] *= -1.0
    T = np.cross(N.T, rng.normal(size=(n, 3))).T
    T /= np.linalg.norm(T, axis=0)
    rnd = np.zeros((n, C5_IN_FLOATS), np.float32)
    rnd[:, 0:3] = rng.random((n, 3), dtype=np.float32) * np.float32(0.99999994)
    rnd[:, 3:6] = rng.uniform(0.2, 1.0, (n, 3))
    rnd[:, 6] = (rng.random(n) < 0.3).astype(np.float32)
    rnd[:, 7] = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0.0, 0.8, n))  # ray roughness
    rnd[:, 8] = (rng.random(n) < 0.2).astype(np.float32)  # backfacing
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    return (P, f32(N), f32(I), f32(T), rnd)


PRIM_DTYPE = np.dtype([("kind", np.int32), ("material", np.int32), ("p", np.float32, 3), ("ex", np.float32, 3),
                       ("ey", np.float32, 3), ("radius", np.float32)])


def c5_scene(nprims=1000, seed=C5_SEED, nmat=C5_MATERIALS):
    """Seeded scene of spheres and rectangles ("planes"): a 200 x 200
    ground, a back wall, 24 tilted panels and spheres for the rest (70%
    resting on the ground, 30% floating), material uniform over nmat."""
    rng = np.random.default_rng([seed, 0x5C])
    prims = np.zeros(nprims, PRIM_DTYPE)

    def rect(i, p, ex, ey):
        prims[i]["kind"] = 1
        prims[i]["p"], prims[i]["ex"], prims[i]["ey"] = p, ex, ey

    rect(0, (-100.0, 0.0, -100.0), (0.0, 0.0, 200.0), (200.0, 0.0, 0.0))
    rect(1, (-60.0, 0.0, -45.0), (120.0, 0.0, 0.0), (0.0, 30.0, 0.0))
    npanels = min(24, max(0, nprims - 2))
    for k in range(npanels):
        i = 2 + k
        a, b = rng.uniform(0, 2 * np.pi), rng.uniform(0.3, 1.2)
        ex = np.array([np.cos(a), 0.0, np.sin(a)]) * rng.uniform(1.5, 4.0)
        up = np.array([-np.sin(a) * np.cos(b), np.sin(b), np.cos(a) * np.cos(b)])
        ey = up * rng.uniform(1.5, 4.0)
        p = (rng.uniform(-25, 25), rng.uniform(0.0, 4.0), rng.uniform(-40, 10))
        rect(i, p, ex.astype(np.float32), ey.astype(np.float32))
        # keep the edges orthogonal in float32
        e0 = prims[i]["ex"].astype(np.float64)
        e1 = prims[i]["ey"].astype(np.float64)
        e1 = e1 - e0 * (e0 @ e1) / (e0 @ e0)
        prims[i]["ey"] = e1.astype(np.float32)
    for i in range(2 + npanels, nprims):
        r = rng.uniform(0.3, 2.0)
        x, z = rng.uniform(-28, 28), rng.uniform(-42, 12)
        y = r if rng.random() < 0.7 else r + rng.uniform(0.5, 10.0)
        prims[i]["kind"] = 0
        prims[i]["p"] = (x, y, z)
        prims[i]["radius"] = r
    prims["material"] = rng.integers(0, nmat, nprims)
    return prims


def c5_materials(ss):
    """The 16 material groups, sampled with the wavefront record layout."""
    return [c5_material_group(ss, k, spec) for k, spec in enumerate(c5_material_specs())]
