"""Shader programs used by the benchmarks and tests, written as the .oso
that oslc plus the runtime optimizer would hand the executor (no oslc runs
here; see OsoBuilder).
"""
from .oso import OsoBuilder


def fbm_cell():
    """fBm of vector Perlin noise with derivatives plus a hashed cell id.

        shader fbm_cell(int octaves = 4, float lacunarity = 2, float gain = 0.5,
                        output color Cout = 0, output int cellhash = 0)
        {
            point p = point(8*u, 8*v, 0);
            color sum = 0; float amp = 1; point pp = p;
            for (int i = 0; i < octaves; ++i) {
                sum += amp * (color) noise("perlin", pp);
                pp *= lacunarity; amp *= gain;
            }
            Cout = sum;
            cellhash = hash(cellnoise(p * 4));
        }
    """
    b = OsoBuilder("fbm_cell")
    octaves = b.param("int", "octaves", 4)
    lac = b.param("float", "lacunarity", 2.0)
    gain = b.param("float", "gain", 0.5)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    cellhash = b.param("int", "cellhash", 0, output=True)
    u = b.glob("float", "u")
    v = b.glob("float", "v")
    p = b.local("point", "p")
    s = b.local("color", "sum")
    amp = b.local("float", "amp")
    pp = b.local("point", "pp")
    i = b.local("int", "i")
    t1, t2 = b.tmp("float"), b.tmp("float")
    c8, c0, c1, c4 = b.const("float", 8.0), b.const("float", 0.0), b.const("float", 1.0), b.const("float", 4.0)
    i0, i1 = b.const("int", 0), b.const("int", 1)
    perlin = b.const("string", "perlin")
    b.op("mul", t1, c8, u)
    b.op("mul", t2, c8, v)
    b.op("point", p, t1, t2, c0)
    b.op("assign", s, c0)
    b.op("assign", amp, c1)
    b.op("assign", pp, p)
    cond = b.tmp("int")
    with b.loop("for", cond) as L:
        b.op("assign", i, i0)
        L.cond()
        b.op("lt", cond, i, octaves)
        L.body()
        n = b.tmp("color")
        m = b.tmp("color")
        b.op("noise", n, perlin, pp)
        b.op("mul", m, amp, n)
        b.op("add", s, s, m)
        b.op("mul", pp, pp, lac)
        b.op("mul", amp, amp, gain)
        L.step()
        b.op("add", i, i, i1)
    b.op("assign", Cout, s)
    p4 = b.tmp("point")
    cn = b.tmp("float")
    b.op("mul", p4, p, c4)
    b.op("cellnoise", cn, p4)
    b.op("hash", cellhash, cn)
    return b.text()


def _testnoise_common(b, inscale_name="inscale", angle_default=10.0, inscale_default=20.0, hard_trig=False):
    """Coordinates shared by the testsuite noise shaders:
        float theta = radians(angle);
        float s = mod(u,0.25) - 0.125;  float t = mod(v,0.5) - 0.25;
        float ru = cos(theta)*s + sin(theta)*t;  float rv = sin(theta)*s - cos(theta)*t;
        ru *= inscale; rv *= inscale;
        float rz = (inscale*(s+t)) / M_SQRT2;  float ttime = s*inscale;
    mod() is stdosl.h's a - b*floor(a/b), inlined as oslc does."""
    angle = b.param("float", "angle", angle_default)
    inscale = b.param("float", inscale_name, inscale_default)
    u = b.glob("float", "u")
    v = b.glob("float", "v")
    theta, s, t = b.local("float", "theta"), b.local("float", "s"), b.local("float", "t")
    ru, rv, rz, ttime = (b.local("float", n) for n in ("ru", "rv", "rz", "ttime"))
    ct, st = b.local("float", "cos_theta"), b.local("float", "sin_theta")
    b.op("radians", theta, angle)
    if hard_trig:
        # testsuite/hashnoise/test.osl hard-codes the angle=10 values
        b.op("assign", ct, b.const("float", 0.984807729721069335))
        b.op("assign", st, b.const("float", 0.173648148775100708))
    else:
        b.op("cos", ct, theta)
        b.op("sin", st, theta)

    def mod(dst, a, m):
        q, f, pr = b.tmp("float"), b.tmp("float"), b.tmp("float")
        b.op("div", q, a, m)
        b.op("floor", f, q)
        b.op("mul", pr, m, f)
        b.op("sub", dst, a, pr)

    ms, mt = b.tmp("float"), b.tmp("float")
    mod(ms, u, b.const("float", 0.25))
    b.op("sub", s, ms, b.const("float", 0.125))
    mod(mt, v, b.const("float", 0.5))
    b.op("sub", t, mt, b.const("float", 0.25))
    a1, a2, a3, a4 = (b.tmp("float") for _ in range(4))
    b.op("mul", a1, ct, s)
    b.op("mul", a2, st, t)
    b.op("add", ru, a1, a2)
    b.op("mul", a3, st, s)
    b.op("mul", a4, ct, t)
    b.op("sub", rv, a3, a4)
    b.op("mul", ru, ru, inscale)
    b.op("mul", rv, rv, inscale)
    st_, prod = b.tmp("float"), b.tmp("float")
    b.op("add", st_, s, t)
    b.op("mul", prod, inscale, st_)
    b.op("div", rz, prod, b.const("float", 1.4142135623730951))
    b.op("mul", ttime, s, inscale)
    return u, v, ru, rv, rz, ttime


def _quadrants(b, u, v, emit):
    """The testsuite shaders' layout: float noise for v<0.49, color noise for
    v>0.51; 1D/2D/3D/4D in the four u bands."""
    c = lambda x: b.const("float", x)
    ci = b.tmp("int")

    def bands(vec):
        b1 = b.tmp("int")
        b.op("lt", b1, u, c(0.24))
        with b.if_(b1) as br1:
            emit(vec, 1)
            br1.else_()
            g, l, a = b.tmp("int"), b.tmp("int"), b.tmp("int")
            b.op("gt", g, u, c(0.26))
            b.op("lt", l, u, c(0.49))
            b.op("and", a, g, l)
            with b.if_(a) as br2:
                emit(vec, 2)
                br2.else_()
                g2, l2, a2 = b.tmp("int"), b.tmp("int"), b.tmp("int")
                b.op("gt", g2, u, c(0.51))
                b.op("lt", l2, u, c(0.74))
                b.op("and", a2, g2, l2)
                with b.if_(a2) as br3:
                    emit(vec, 3)
                    br3.else_()
                    g3 = b.tmp("int")
                    b.op("gt", g3, u, c(0.76))
                    with b.if_(g3):
                        emit(vec, 4)

    b.op("lt", ci, v, c(0.49))
    with b.if_(ci) as top:
        bands(False)
        top.else_()
        c2 = b.tmp("int")
        b.op("gt", c2, v, c(0.51))
        with b.if_(c2):
            bands(True)


def testnoise(shader_name="testnoise", noisename_default="noise", offset_default=0.5, scale_default=0.5,
              with_name=True, opname=None):
    """testsuite/common/shaders/testnoise.osl (with_name=True) and the
    per-noise test.osl shaders of testsuite/{noise,cellnoise,hashnoise}."""
    b = OsoBuilder(shader_name)
    noisename = b.param("string", "noisename", noisename_default) if with_name else None
    offset = b.param("float", "offset", offset_default)
    scale = b.param("float", "scale", scale_default)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    u, v, ru, rv, rz, ttime = _testnoise_common(b, hard_trig=(opname == "hashnoise"))
    b.op("assign", Cout, b.const("float", 0.0))

    def emit(vec, dim):
        r = b.tmp("color" if vec else "float")
        args = []
        if dim in (1, 2):
            args = [ru] if dim == 1 else [ru, rv]
        else:
            pt = b.tmp("point")
            b.op("point", pt, ru, rv, rz)
            args = [pt] if dim == 3 else [pt, ttime]
        if with_name:
            b.op("noise", r, noisename, *args)
        else:
            b.op(opname, r, *args)
        m, a = b.tmp("color" if vec else "float"), b.tmp("color" if vec else "float")
        b.op("mul", m, scale, r)
        b.op("add", a, offset, m)
        b.op("assign", Cout, a)

    _quadrants(b, u, v, emit)
    return b.text()


def testpnoise(shader_name="testpnoise", noisename_default="noise", offset_default=0.5, scale_default=0.5,
               period_default=3.0):
    """testsuite/common/shaders/testpnoise.osl: periodic noise with the
    testnoise layout, angle 0, inscale 30, period 3."""
    b = OsoBuilder(shader_name)
    noisename = b.param("string", "noisename", noisename_default)
    offset = b.param("float", "offset", offset_default)
    scale = b.param("float", "scale", scale_default)
    period = b.param("float", "period", period_default)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    u, v, ru, rv, rz, ttime = _testnoise_common(b, angle_default=0.0, inscale_default=30.0)
    b.op("assign", Cout, b.const("float", 0.0))

    def emit(vec, dim):
        r = b.tmp("color" if vec else "float")
        if dim == 1:
            b.op("pnoise", r, noisename, ru, period)
        elif dim == 2:
            b.op("pnoise", r, noisename, ru, rv, period, period)
        else:
            pt, pp = b.tmp("point"), b.tmp("point")
            b.op("point", pt, ru, rv, rz)
            b.op("assign", pp, period)
            if dim == 3:
                b.op("pnoise", r, noisename, pt, pp)
            else:
                b.op("pnoise", r, noisename, pt, ttime, pp, period)
        m, a = b.tmp("color" if vec else "float"), b.tmp("color" if vec else "float")
        b.op("mul", m, scale, r)
        b.op("add", a, offset, m)
        b.op("assign", Cout, a)

    _quadrants(b, u, v, emit)
    return b.text()


def gabor_options(shader_name="test_gabor_options", anisotropic=0, direction=(1.0, 0.0, 0.0), bandwidth=4.0,
                  impulses=16.0, do_filter=1):
    """testsuite/noise-gabor-reg/test_gabor_options.osl: the testnoise layout
    with every Gabor option passed by name from a shader parameter."""
    b = OsoBuilder(shader_name)
    offset = b.param("float", "offset", 0.5)
    scale = b.param("float", "scale", 0.5)
    aniso = b.param("int", "anisotropic", anisotropic)
    direc = b.param("vector", "direction", list(direction))
    bw = b.param("float", "bandwidth", bandwidth)
    imp = b.param("float", "impulses", impulses)
    filt = b.param("int", "do_filter", do_filter)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    u, v, ru, rv, rz, ttime = _testnoise_common(b)
    b.op("assign", Cout, b.const("float", 0.0))
    gname = b.const("string", "gabor")
    opts = [b.const("string", "anisotropic"), aniso, b.const("string", "direction"), direc,
            b.const("string", "bandwidth"), bw, b.const("string", "impulses"), imp,
            b.const("string", "do_filter"), filt]

    def emit(vec, dim):
        r = b.tmp("color" if vec else "float")
        if dim in (1, 2):
            args = [ru] if dim == 1 else [ru, rv]
        else:
            pt = b.tmp("point")
            b.op("point", pt, ru, rv, rz)
            args = [pt] if dim == 3 else [pt, ttime]
        b.op("noise", r, gname, *args, *opts)
        m, a = b.tmp("color" if vec else "float"), b.tmp("color" if vec else "float")
        b.op("mul", m, scale, r)
        b.op("add", a, offset, m)
        b.op("assign", Cout, a)

    _quadrants(b, u, v, emit)
    return b.text()


def gabor_filter_test(dims, shader_name=None, freq=5.0):
    """testsuite/noise-gabor{2d,3d}-filter/test.osl: p = P*freq*(1+10*v*v)*(1+10*u*u),
    Cout = noise("gabor", p[0], p[1]) (2-D) or noise("gabor", p) (3-D), *0.5+0.5."""
    b = OsoBuilder(shader_name or "gabor%dd_filter" % dims, "surface")
    noisename = b.param("string", "noisename", "gabor")
    fr = b.param("float", "freq", freq)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    P, u, v = b.glob("point", "P"), b.glob("float", "u"), b.glob("float", "v")
    c = lambda x: b.const("float", x)
    p, t1, t2, t3, t4, t5, t6 = b.tmp("point"), *(b.tmp("float") for _ in range(6))
    b.op("mul", p, P, fr)
    b.op("mul", t1, c(10.0), v)  # 10*v*v parses as (10*v)*v
    b.op("mul", t2, t1, v)
    b.op("add", t3, c(1.0), t2)
    b.op("mul", p, p, t3)
    b.op("mul", t4, c(10.0), u)
    b.op("mul", t5, t4, u)
    b.op("add", t6, c(1.0), t5)
    b.op("mul", p, p, t6)
    n = b.tmp("float")
    if dims == 2:
        px, py = b.tmp("float"), b.tmp("float")
        b.op("compref", px, p, b.const("int", 0))
        b.op("compref", py, p, b.const("int", 1))
        b.op("noise", n, noisename, px, py)
    else:
        b.op("noise", n, noisename, p)
    h, o = b.tmp("float"), b.tmp("float")
    b.op("mul", h, n, c(0.5))
    b.op("add", o, h, c(0.5))
    b.op("assign", Cout, o)
    return b.text()


def matrix_ops(M, M2):
    """Matrix and derivative ops on a per-point matrix: Mv = M * (1 + u)
    (varying), then transpose, determinant, M / M2, 1 / M, transform /
    transformv / transformn of P, area(P), filterwidth(u) and luminance of a
    colour built from P. Outputs: det, Pt, Vt, Nt, area, fw, lum, and the
    first rows of transpose(Mv), Mv / M2 and 1 / Mv."""
    b = OsoBuilder("matrix_ops")
    Mp = b.param("matrix", "M", list(M))
    M2p = b.param("matrix", "M2", list(M2))
    det = b.param("float", "det", 0.0, output=True)
    Pt = b.param("point", "Pt", [0, 0, 0], output=True)
    Vt = b.param("vector", "Vt", [0, 0, 0], output=True)
    Nt = b.param("normal", "Nt", [0, 0, 0], output=True)
    ar = b.param("float", "area", 0.0, output=True)
    fw = b.param("float", "fw", 0.0, output=True)
    lum = b.param("float", "lum", 0.0, output=True)
    rowT = b.param("color", "rowT", [0, 0, 0], output=True)
    rowD = b.param("color", "rowD", [0, 0, 0], output=True)
    rowI = b.param("color", "rowI", [0, 0, 0], output=True)
    P, u = b.glob("point", "P"), b.glob("float", "u")
    c = lambda x: b.const("float", x)
    s, Mv, T, D, I = b.tmp("float"), b.tmp("matrix"), b.tmp("matrix"), b.tmp("matrix"), b.tmp("matrix")
    b.op("add", s, c(1.0), u)
    b.op("mul", Mv, Mp, s)
    b.op("transpose", T, Mv)
    b.op("determinant", det, Mv)
    b.op("div", D, Mv, M2p)
    b.op("div", I, c(1.0), Mv)
    b.op("transform", Pt, Mv, P)
    V, Nn = b.tmp("vector"), b.tmp("normal")
    b.op("vector", V, P)
    b.op("normal", Nn, P)
    b.op("transformv", Vt, Mv, V)
    b.op("transformn", Nt, Mv, Nn)
    b.op("area", ar, P)
    b.op("filterwidth", fw, u)
    col = b.tmp("color")
    b.op("color", col, P)
    b.op("luminance", lum, col)
    for row, src in ((rowT, T), (rowD, D), (rowI, I)):
        for j in range(3):
            t = b.tmp("float")
            b.op("mxcompref", t, src, b.const("int", 0), b.const("int", j))
            b.op("compassign", row, b.const("int", j), t)
    return b.text()


def blackbody_test(temp_scale=10000.0):
    """testsuite/blackbody/test.osl: T = 10000*u; Cout = blackbody(T)/10000;
    for v > 0.5, Cout *= 0.7/luminance(Cout). temp_scale replaces the
    10000 K of T (past 12000 K the spectral path runs)."""
    b = OsoBuilder("test")
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    c = lambda x: b.const("float", x)
    T, bb, lum, sc, cond = b.tmp("float"), b.tmp("color"), b.tmp("float"), b.tmp("float"), b.tmp("int")
    b.op("mul", T, c(temp_scale), u)
    b.op("blackbody", bb, T)
    b.op("div", Cout, bb, c(10000.0))
    b.op("gt", cond, v, c(0.5))
    with b.if_(cond):
        b.op("luminance", lum, Cout)
        b.op("div", sc, c(0.7), lum)
        b.op("mul", Cout, Cout, sc)
    return b.text()


def getP():
    """testsuite/example-batched-deformer/getP.osl: output point out = P"""
    b = OsoBuilder("getP")
    out = b.param("point", "out", [0, 0, 0], output=True)
    P = b.glob("point", "P")
    b.op("assign", out, P)
    return b.text()


def vfBm3d():
    """testsuite/example-batched-deformer/vfBm3d.osl"""
    b = OsoBuilder("vfBm3d")
    position = b.param("point", "position", [0, 0, 0], lockgeom=False)
    frequency = b.param("float", "frequency", 1.0)
    amplitude = b.param("float", "amplitude", 1.0, lockgeom=False)
    octaves = b.param("int", "octaves", 1)
    lac = b.param("float", "lacunarity", 2.0)
    gain = b.param("float", "gain", 0.5)
    noisetype = b.param("string", "noisetype", "snoise")
    out = b.param("vector", "out", [0, 0, 0], output=True)
    r, p, amp, i = b.local("vector", "r"), b.local("point", "p"), b.local("float", "amp"), b.local("int", "i")
    b.op("assign", r, b.const("float", 0.0))
    b.op("mul", p, position, frequency)
    b.op("assign", amp, amplitude)
    cond = b.tmp("int")
    with b.loop("for", cond) as L:
        b.op("assign", i, b.const("int", 0))
        L.cond()
        b.op("lt", cond, i, octaves)
        L.body()
        n, m = b.tmp("vector"), b.tmp("vector")
        b.op("noise", n, noisetype, p)
        b.op("mul", m, amp, n)
        b.op("add", r, r, m)
        b.op("mul", p, p, lac)
        b.op("mul", amp, amp, gain)
        L.step()
        b.op("add", i, i, b.const("int", 1))
    b.op("assign", out, r)
    return b.text()


def vadd():
    """testsuite/example-batched-deformer/vadd.osl: out = a + b"""
    b = OsoBuilder("vadd")
    a = b.param("vector", "a", [0, 0, 0])
    bb = b.param("vector", "b", [0, 0, 0])
    out = b.param("vector", "out", [0, 0, 0], output=True)
    b.op("add", out, a, bb)
    return b.text()


def ctrlflow():
    """Varying control flow: data-dependent trip counts, continue, break,
    while, do-while, nested if/else and an early return.

        shader ctrlflow(output float r = 0, output int count = 0)
        {
            float acc = 0;
            int n = (int)(cellnoise(u*8, v*8) * 16);
            for (int i = 0; i < n; ++i) {
                if (i == 3) continue;
                float x = noise("perlin", u*4 + i);
                if (x > 0.3) { acc += x; if (acc > 2) break; }
                else acc -= 0.1*x;
                count += 1;
            }
            int j = 0;
            while (j < n) { j += 2; if (j > 9) break; }
            do { acc += 0.01; j -= 3; } while (j > 0);
            if (v > 0.9) { r = acc; return; }
            r = acc * 2 + j;
        }
    """
    b = OsoBuilder("ctrlflow")
    r = b.param("float", "r", 0.0, output=True)
    count = b.param("int", "count", 0, output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    cf = lambda x: b.const("float", x)
    ci = lambda x: b.const("int", x)
    acc, n, i, x, j = (b.local(t, nm) for t, nm in
                       (("float", "acc"), ("int", "n"), ("int", "i"), ("float", "x"), ("int", "j")))
    b.op("assign", acc, cf(0.0))
    u8, v8, cn, cn16 = b.tmp("float"), b.tmp("float"), b.tmp("float"), b.tmp("float")
    b.op("mul", u8, u, cf(8.0))
    b.op("mul", v8, v, cf(8.0))
    b.op("cellnoise", cn, u8, v8)
    b.op("mul", cn16, cn, cf(16.0))
    b.op("assign", n, cn16)
    cond = b.tmp("int")
    with b.loop("for", cond) as L:
        b.op("assign", i, ci(0))
        L.cond()
        b.op("lt", cond, i, n)
        L.body()
        e3 = b.tmp("int")
        b.op("eq", e3, i, ci(3))
        with b.if_(e3):
            b.op("continue")
        u4, fi, arg = b.tmp("float"), b.tmp("float"), b.tmp("float")
        b.op("mul", u4, u, cf(4.0))
        b.op("assign", fi, i)
        b.op("add", arg, u4, fi)
        b.op("noise", x, b.const("string", "perlin"), arg)
        g = b.tmp("int")
        b.op("gt", g, x, cf(0.3))
        with b.if_(g) as br:
            b.op("add", acc, acc, x)
            g2 = b.tmp("int")
            b.op("gt", g2, acc, cf(2.0))
            with b.if_(g2):
                b.op("break")
            br.else_()
            t = b.tmp("float")
            b.op("mul", t, cf(0.1), x)
            b.op("sub", acc, acc, t)
        b.op("add", count, count, ci(1))
        L.step()
        b.op("add", i, i, ci(1))
    b.op("assign", j, ci(0))
    wc = b.tmp("int")
    with b.loop("while", wc) as L:
        L.cond()
        b.op("lt", wc, j, n)
        L.body()
        b.op("add", j, j, ci(2))
        g3 = b.tmp("int")
        b.op("gt", g3, j, ci(9))
        with b.if_(g3):
            b.op("break")
        L.step()
    dc = b.tmp("int")
    with b.loop("dowhile", dc) as L:
        L.cond()
        b.op("gt", dc, j, ci(0))
        L.body()
        b.op("add", acc, acc, cf(0.01))
        b.op("sub", j, j, ci(3))
        L.step()
    g4 = b.tmp("int")
    b.op("gt", g4, v, cf(0.9))
    with b.if_(g4):
        b.op("assign", r, acc)
        b.op("return")
    t2, fj = b.tmp("float"), b.tmp("float")
    b.op("mul", t2, acc, cf(2.0))
    b.op("assign", fj, j)
    b.op("add", r, t2, fj)
    return b.text()


# ---- 3-layer closure group (pattern -> color ramp -> surface) -----------------------
def c2_pattern():
    """Layer A: simplex noise plus cell noise on P*16, P = (u, v, 0).

        shader c2_pattern(float scale = 16, output float a = 0)
        {
            point p = point(u, v, 0) * scale;
            a = 0.8 * noise("usimplex", p) + 0.2 * cellnoise(p);
        }
    """
    b = OsoBuilder("c2_pattern")
    scale = b.param("float", "scale", 16.0)
    a = b.param("float", "a", 0.0, output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    p0, p = b.tmp("point"), b.tmp("point")
    b.op("point", p0, u, v, b.const("float", 0.0))
    b.op("mul", p, p0, scale)
    s, c, t1, t2 = b.tmp("float"), b.tmp("float"), b.tmp("float"), b.tmp("float")
    b.op("noise", s, b.const("string", "usimplex"), p)
    b.op("cellnoise", c, p)
    b.op("mul", t1, b.const("float", 0.8), s)
    b.op("mul", t2, b.const("float", 0.2), c)
    b.op("add", a, t1, t2)
    return b.text()


def c2_ramp():
    """Layer B: 8-knot catmull-rom color ramp.

        shader c2_ramp(float x = 0, color knots[8] = {...}, output color Cout = 0)
        {
            Cout = spline("catmull-rom", x, knots);
        }
    """
    b = OsoBuilder("c2_ramp")
    x = b.param("float", "x", 0.0)
    knots = b.param("color[8]", "knots", [0.5] * 24)
    Cout = b.param("color", "Cout", [0, 0, 0], output=True)
    b.op("spline", Cout, b.const("string", "catmull-rom"), x, knots)
    return b.text()


def c2_surface():
    """Layer C: a closure sum with GGX roughness driven by the pattern.

        surface c2_surface(float a = 0, color tint = 1)
        {
            float alpha = 0.05 + 0.75 * a;
            Ci = 0.6 * tint * diffuse(N)
               + 0.4 * microfacet("ggx", N, dPdu, alpha, alpha, 1.5, 0);
        }
    """
    b = OsoBuilder("c2_surface", "surface")
    a = b.param("float", "a", 0.0)
    tint = b.param("color", "tint", [1, 1, 1])
    Ci = b.glob("closure color", "Ci")
    N = b.glob("normal", "N")
    dPdu = b.glob("vector", "dPdu")
    alpha, t = b.local("float", "alpha"), b.tmp("float")
    b.op("mul", t, b.const("float", 0.75), a)
    b.op("add", alpha, b.const("float", 0.05), t)
    w, d, dw = b.tmp("color"), b.tmp("closure color"), b.tmp("closure color")
    b.op("mul", w, b.const("float", 0.6), tint)
    b.op("closure", d, b.const("string", "diffuse"), N)
    b.op("mul", dw, d, w)
    m, mw = b.tmp("closure color"), b.tmp("closure color")
    b.op("closure", m, b.const("string", "microfacet"), b.const("string", "ggx"), N, dPdu, alpha, alpha,
         b.const("float", 1.5), b.const("int", 0))
    b.op("mul", mw, m, b.const("float", 0.4))
    b.op("add", Ci, dw, mw)
    return b.text()


def c2_knots(seed=0xC2B):
    """The ramp's 8 knot colors, seeded."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [float(x) for x in rng.uniform(0.05, 0.95, 24).astype(np.float32)]


def texture_lookup(name, scale, wrap=None, nc=3, width=None, first=None):
    """Cout = texture("img", u * k, v * k, options): k = scale, so the lookup
    footprint is scale / grid size in texture space (derivatives of u, v)."""
    from .oso import OsoBuilder
    b = OsoBuilder(name)
    out = b.param("color" if nc == 3 else "float", "Cout", [0, 0, 0] if nc == 3 else 0.0, output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    s, t = b.tmp("float"), b.tmp("float")
    k = b.param("float", "k", float(scale))
    b.op("mul", s, u, k)
    b.op("mul", t, v, k)
    args = [out, b.const("string", "img"), s, t]
    if wrap:
        args += [b.const("string", "wrap"), b.const("string", wrap)]
    if width is not None:
        args += [b.const("string", "width"), b.const("float", float(width))]
    if first is not None:
        args += [b.const("string", "firstchannel"), b.const("int", int(first))]
    b.op("texture", *args)
    return b.text()


def environment_lookup(name, width=None, first=None):
    """Cout = environment("env", R) with R the unit direction of the
    (u, v) grid: phi = 2 pi u around z, theta = pi v from +z.

        shader env(output color Cout = 0)
        {
            float phi = u * M_2PI, theta = v * M_PI, st = sin(theta);
            Cout = environment("env", vector(cos(phi) * st, sin(phi) * st, cos(theta)));
        }
    """
    from .oso import OsoBuilder
    b = OsoBuilder(name)
    cout = b.param("color", "Cout", [0, 0, 0], output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    phi, theta, st, cp, sp, ct = [b.tmp("float") for _ in range(6)]
    x, y = b.tmp("float"), b.tmp("float")
    R = b.tmp("vector")
    b.op("mul", phi, u, b.const("float", 6.2831855))
    b.op("mul", theta, v, b.const("float", 3.1415927))
    b.op("sin", st, theta)
    b.op("cos", cp, phi)
    b.op("sin", sp, phi)
    b.op("cos", ct, theta)
    b.op("mul", x, cp, st)
    b.op("mul", y, sp, st)
    b.op("vector", R, x, y, ct)
    args = [cout, b.const("string", "env"), R]
    if width is not None:
        args += [b.const("string", "width"), b.const("float", width)]
    if first is not None:
        args += [b.const("string", "firstchannel"), b.const("int", first)]
    b.op("environment", *args)
    return b.text()
