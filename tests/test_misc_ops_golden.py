"""Op-table entries pinned to the reference testsuite's printed output:
raytype (testsuite/raytype, run with --raytype glossy), isconnected
(testsuite/isconnected: an upstream and a downstream layer, a renderer
output, and the --userdata_isconnected run), isconstant
(testsuite/isconstant), the exponential suite (log, log with a base, log2,
log10, logb, exp, exp2, expm1, erf, erfc and the pow corner cases;
testsuite/exponential) and the .oso reader's refusal of an unknown
instruction (testsuite/unknown-instruction). The expected text is the
reference's ref/out.txt, copied to tests/golden/ by make_golden.py; each
printed value is an output of the group, formatted the way the shader
prints it. sincos, calculatenormal (with flipHandedness), backfacing,
surfacearea and arraycopy, which no testsuite text covers, are checked
against numpy. The GPU runs the same groups and must equal the oracle bit
for bit."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder

TYPES = {"int": (og.TypeInt, 1), "float": (og.TypeFloat, 1), "color": (og.TypeColor, 3),
         "vector": (og.TypeVector, 3)}


def ref_lines(name):
    return [ln for ln in open(os.path.join(GOLDEN, name)).read().splitlines()
            if ln and not ln.startswith("Compiled")]


class Outputs:
    """Output parameters of one layer, each placed in the output record."""

    def __init__(self, b, layer):
        self.b, self.layer, self.outs = b, layer, []

    def __call__(self, name, t="float", derivs=False):
        self.outs.append((name, t, derivs))
        n = TYPES[t][1]
        return self.b.param(t, name, [0] * n if n > 1 else 0, output=True)


def place(ss, g, layers):
    """Symlocs for every output of `layers` (list of Outputs); returns the
    record width in floats and {layer.name: (offset, floats, type)}."""
    cols, off = {}, 0
    for o in layers:
        for nm, t, d in o.outs:
            n = TYPES[t][1] * (3 if d else 1)
            cols[o.layer + "." + nm] = (off, n, t)
            off += n
    locs = [og.SymLocationDesc(k, TYPES[t][0], False, og.SymArenaOutputs, 4 * o, 4 * off)
            for k, (o, n, t) in cols.items()]
    ss.add_symlocs(g, locs)
    return off, cols


def column(out, cols, key, pt=0):
    o, n, t = cols[key]
    row = out[pt, o:o + n]
    if t == "int":
        return int(row.view(np.int32)[0])
    return row if n > 1 else float(row[0])


def run_oracle(g, rec, G, npts):
    out = np.zeros((npts, rec), np.float32)
    assert oracle_run(g.program_bytes(), npts, G, out) == 0
    return out


# ---- raytype -----------------------------------------------------------------
def raytype_group(ss):
    b = OsoBuilder("rt_suite")
    o = Outputs(b, "L")
    S = lambda s: b.const("string", s)
    for nm in ("camera", "glossy", "diffuse"):
        b.op("raytype", o("is_" + nm, "int"), S(nm))
    # a name known only at run time: "glossy" where u < 0.5, else "camera"
    nm = b.local("string", "nm")
    c = b.tmp("int")
    b.op("lt", c, b.glob("float", "u"), b.const("float", 0.5))
    with b.if_(c) as blk:
        b.op("assign", nm, S("glossy"))
        blk.else_()
        b.op("assign", nm, S("camera"))
    b.op("raytype", o("is_dyn", "int"), nm)
    ss.LoadMemoryCompiledShader("rt_suite", b.text())
    g = ss.ShaderGroupBegin("rt_g")
    ss.Shader(g, "surface", "rt_suite", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    return g, rec, cols


def glossy_globals(u, v, W, H, raytype_bit):
    G = grid_globals(u, v, W, H)
    G.raytype = raytype_bit
    return G


def test_raytype_matches_the_testsuite():
    ss = og.ShadingSystem()
    g, rec, cols = raytype_group(ss)
    u, v = pixel_grid(2, 1)
    out = run_oracle(g, rec, glossy_globals(u, v, 2, 1, 1 << 5), 2)  # testshade --raytype glossy
    got = ["%s? %d" % (nm, column(out, cols, "L.is_" + nm)) for nm in ("camera", "glossy", "diffuse")]
    assert got == ref_lines("raytype_out.txt")
    # run-time names: u = 0 asks for glossy, u = 1 for camera
    assert [column(out, cols, "L.is_dyn", p) for p in (0, 1)] == [1, 0]


def test_raytypes_attribute_renumbers_the_bits():
    ss = og.ShadingSystem()
    ss.attribute("raytypes", ["glossy", "camera"])
    g, rec, cols = raytype_group(ss)
    u, v = pixel_grid(2, 1)
    out = run_oracle(g, rec, glossy_globals(u, v, 2, 1, 1 << 0), 2)
    assert [column(out, cols, "L.is_" + nm) for nm in ("camera", "glossy", "diffuse")] == [0, 1, 0]
    assert [column(out, cols, "L.is_dyn", p) for p in (0, 1)] == [1, 0]


# ---- isconnected ---------------------------------------------------------------
UP_NAMES = ("out", "notout", "struct1.x", "struct1.y", "struct2.x", "struct2.y")
DOWN_NAMES = ("a", "b", "c", "mystruct1.x", "mystruct1.y", "mystruct2.x", "mystruct2.y", "Fout")


def isconnected_group(ss, fout_is_output):
    """testsuite/isconnected: struct members are the flattened fields oslc
    writes (struct1.x ...); a struct's own status is its first field's
    (runtimeoptimize.cpp:2481-2492)."""
    up = OsoBuilder("upstream")
    uo = Outputs(up, "upstream")
    syms = {nm: up.param("float", nm, 0.0, output=True) for nm in UP_NAMES}
    up.op("assign", syms["notout"], up.const("float", 10.0))
    for nm in UP_NAMES:
        up.op("isconnected", uo("ic_" + nm.replace(".", "_"), "int"), syms[nm])
    dn = OsoBuilder("test")
    do = Outputs(dn, "downstream")
    ds = {}
    for nm in DOWN_NAMES[:-1]:
        ds[nm] = dn.param("float", nm, 0.0, lockgeom=nm != "c")
    ds["Fout"] = dn.param("float", "Fout", 1.0, output=True)
    for nm in DOWN_NAMES[:-1]:
        dn.op("isconnected", do("ic_" + nm.replace(".", "_"), "int"), ds[nm])
    k, c = dn.tmp("int"), dn.tmp("int")
    dn.op("isconnected", k, ds["Fout"])
    dn.op("eq", c, k, dn.const("int", 2))
    with dn.if_(c) as blk:
        dn.op("assign", ds["Fout"], dn.const("float", 0.42))
        blk.else_()
        dn.op("assign", ds["Fout"], dn.const("float", 0.0))
    dn.op("isconnected", do("ic_Fout", "int"), ds["Fout"])
    dn.op("assign", do("Fout_value"), ds["Fout"])
    ss.LoadMemoryCompiledShader("upstream", up.text())
    ss.LoadMemoryCompiledShader("test", dn.text())
    g = ss.ShaderGroupBegin("ic_g")
    ss.Shader(g, "surface", "upstream", "upstream")
    ss.Shader(g, "surface", "test", "downstream")
    ss.ConnectShaders(g, "upstream", "out", "downstream", "a")
    ss.ConnectShaders(g, "upstream", "struct1.x", "downstream", "mystruct1.x")
    ss.ConnectShaders(g, "upstream", "struct1.y", "downstream", "mystruct1.y")
    ss.ShaderGroupEnd(g)
    if fout_is_output:  # testshade -o Fout
        ss.renderer_outputs(g, ["Fout"])
    rec, cols = place(ss, g, [uo, do])
    return g, rec, cols


def expected_isconnected():
    """{run: {name: status}} from the two testshade runs of ref/out.txt."""
    runs, cur = [], None
    for ln in ref_lines("isconnected_out.txt"):
        if ln.startswith("Connect upstream.out"):
            cur = {}
            runs.append(cur)
        elif " connected: " in ln:
            nm, rest = ln.split(" connected: ")
            cur[nm] = int(rest.split()[0])
    return runs


def isconnected_text(out, cols):
    d = {}
    for nm in UP_NAMES:
        d[nm] = column(out, cols, "upstream.ic_" + nm.replace(".", "_"))
    for nm in DOWN_NAMES[:-1]:
        d[nm] = column(out, cols, "downstream.ic_" + nm.replace(".", "_"))
    d["Fout"] = column(out, cols, "downstream.ic_Fout")
    for s in ("struct1", "struct2", "mystruct1", "mystruct2"):
        d[s] = d[s + ".x"]
    return d


@pytest.mark.parametrize("run", [0, 1])
def test_isconnected_matches_the_testsuite(run):
    ss = og.ShadingSystem()
    if run == 1:
        ss.attribute("userdata_isconnected", 1)
    g, rec, cols = isconnected_group(ss, fout_is_output=run == 0)
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1), 1)
    want = expected_isconnected()[run]
    got = isconnected_text(out, cols)
    assert {k: got[k] for k in want} == want
    assert column(out, cols, "downstream.Fout_value") == pytest.approx(0.42 if run == 0 else 0.0)


# ---- isconstant ------------------------------------------------------------------
def isconstant_group(ss):
    b = OsoBuilder("icst_suite")
    o = Outputs(b, "L")
    A = b.param("float", "A", 1.0)
    b.op("isconstant", o("ic_A", "int"), A)
    t = b.tmp("float")
    b.op("mul", t, b.const("float", 2.0), A)
    b.op("isconstant", o("ic_2A", "int"), t)
    n, c = b.tmp("float"), b.tmp("color")
    b.op("noise", n, b.glob("point", "P"))
    b.op("assign", c, n)
    b.op("isconstant", o("ic_noise", "int"), c)
    ss.LoadMemoryCompiledShader("icst_suite", b.text())
    g = ss.ShaderGroupBegin("icst_g")
    ss.Shader(g, "surface", "icst_suite", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    return g, rec, cols


def test_isconstant_matches_the_testsuite():
    ss = og.ShadingSystem()
    g, rec, cols = isconstant_group(ss)
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1, P=(0.3, 0.2, 0.1)), 1)
    got = ["Is param A const? %d" % column(out, cols, "L.ic_A"),
           "Is 2*A const? %d" % column(out, cols, "L.ic_2A"),
           "Is noise(P) const? %d" % column(out, cols, "L.ic_noise")]
    assert got == ref_lines("isconstant_out.txt")


# ---- exponential ---------------------------------------------------------------------
M_E = np.float32(2.7182818284590452354)
FUNCS = ("log", "logbase", "log2", "log10", "logb", "exp", "exp2", "expm1", "erf", "erfc")
POW_CASES = [(2.0, 1.5), (-2.0, 1.5), (-2.0, 0.0), (-2.0, 3.0), (0.0, 3.0), (0.0, -3.0), (0.0, 0.0),
             (2.2, 2.0), (-2.2, 2.0), (1e20, 2.0), (2.5, 1.0)]


def exponential_group(ss):
    """testsuite/exponential/test.osl: its float block, vector block and
    vector-vector pow block, each printed value an output."""
    b = OsoBuilder("exp_suite")
    o = Outputs(b, "L")
    f = lambda x: b.const("float", x)
    for vec in (False, True):
        t = "vector" if vec else "float"
        tag = "v" if vec else "f"
        funcs = FUNCS if not vec else tuple(x for x in FUNCS if x not in ("erf", "erfc"))
        a10 = b.tmp(t)
        ae = b.const(t, [float(M_E)] * 3 if vec else float(M_E))
        b.op("mul", a10, b.const(t, [10.0] * 3 if vec else 10.0), ae)  # a = 10.0*M_E
        for ai, a in enumerate((ae, a10)):
            for fn in funcs:
                r = o("%s_%s_%d" % (tag, fn, ai), t)
                if fn == "logbase":  # stdosl.h:91-94 log(a, b) = log(a) / log(b)
                    la, lb = b.tmp(t), b.tmp("float")
                    b.op("log", la, a)
                    b.op("log", lb, f(27.0))
                    b.op("div", r, la, lb)
                else:
                    b.op(fn, r, a)
        for bi, (x, y) in enumerate(((2.0, 2.0), (10.0, 10.0))):
            la, lb = b.tmp(t), b.tmp("float")
            b.op("log", la, b.const(t, [x] * 3 if vec else x))
            b.op("log", lb, f(y))
            b.op("div", o("%s_logself_%d" % (tag, bi), t), la, lb)
        cases = POW_CASES if not vec else POW_CASES[:7]
        for pi, (x, y) in enumerate(cases):
            b.op("pow", o("%s_pow_%d" % (tag, pi), t), b.const(t, [x] * 3 if vec else x), f(y))
    for pi, (x, y) in enumerate(POW_CASES[:7]):
        b.op("pow", o("vv_pow_%d" % pi, "vector"), b.const("vector", [x] * 3), b.const("vector", [y] * 3))
    ss.LoadMemoryCompiledShader("exp_suite", b.text())
    g = ss.ShaderGroupBegin("exp_g")
    ss.Shader(g, "surface", "exp_suite", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    return g, rec, cols


def fmt(x):
    return " ".join("%g" % float(v) for v in np.atleast_1d(np.asarray(x, np.float32)))


def exponential_text(out, cols):
    L = []
    for vec in (False, True):
        tag = "v" if vec else "f"
        funcs = FUNCS if not vec else tuple(x for x in FUNCS if x not in ("erf", "erfc"))
        a = [M_E, np.float32(10.0) * M_E]
        rep = (lambda x: [x] * 3) if vec else (lambda x: x)
        for ai in (0, 1):
            for fn in funcs:
                val = fmt(column(out, cols, "L.%s_%s_%d" % (tag, fn, ai)))
                arg = fmt(rep(a[ai]))
                if fn == "logbase":
                    L.append("  log (%s, 27) = %s" % (arg, val))
                else:
                    L.append("  %s (%s) = %s" % (fn, arg, val))
        for bi, x in enumerate((2.0, 10.0)):
            L.append("  log (%s, %g) = %s" % (fmt(rep(x)), x, fmt(column(out, cols, "L.%s_logself_%d" % (tag, bi)))))
        cases = POW_CASES if not vec else POW_CASES[:7]
        for pi, (x, y) in enumerate(cases):
            s = "  pow (%s, %g) = %s" % (fmt(rep(x)), y, fmt(column(out, cols, "L.%s_pow_%d" % (tag, pi))))
            if x == 1e20:
                s += "     [should be clamped, not inf!]"
            L.append(s)
    for pi, (x, y) in enumerate(POW_CASES[:7]):
        L.append("  pow (%s, %s) = %s" % (fmt([x] * 3), fmt([y] * 3), fmt(column(out, cols, "L.vv_pow_%d" % pi))))
    return L


def test_exponential_matches_the_testsuite():
    ss = og.ShadingSystem()
    g, rec, cols = exponential_group(ss)
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1), 1)
    got = exponential_text(out, cols)
    ref = ref_lines("exponential_out.txt")
    assert got == ref, [(a, b) for a, b in zip(got, ref) if a != b][:6]


def hyperb_group(ss):
    """testsuite/hyperb/test.osl: cosh, sinh, tanh of -e, 0, e as floats and vectors."""
    b = OsoBuilder("hyp_suite")
    o = Outputs(b, "L")
    for t in ("float", "vector"):
        for i, x in enumerate((-float(M_E), 0.0, float(M_E))):
            a = b.const(t, [x] * 3 if t == "vector" else x)
            for fn in ("cosh", "sinh", "tanh"):
                b.op(fn, o("%s_%s_%d" % (t, fn, i), t), a)
    ss.LoadMemoryCompiledShader("hyp_suite", b.text())
    g = ss.ShaderGroupBegin("hyp_g")
    ss.Shader(g, "surface", "hyp_suite", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    return g, rec, cols


def test_hyperbolic_functions_match_the_testsuite():
    ss = og.ShadingSystem()
    g, rec, cols = hyperb_group(ss)
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1), 1)
    got = []
    for t in ("float", "vector"):
        for i, x in enumerate((-M_E, np.float32(0.0), M_E)):
            arg = fmt([x] * 3 if t == "vector" else x)
            for fn in ("cosh", "sinh", "tanh"):
                got.append("  %s (%s) = %s" % (fn, arg, fmt(column(out, cols, "L.%s_%s_%d" % (t, fn, i)))))
    assert got == ref_lines("hyperb_out.txt")


def test_logb_edges():
    """OpenImageIO fast_logb: |x| clamped to the normal range first."""
    b = OsoBuilder("logb_edges")
    o = Outputs(b, "L")
    xs = [0.0, -0.0, 1.0, -8.5, 1e-40, 3.0e38, float("inf"), 0.75]
    for i, x in enumerate(xs):
        b.op("logb", o("r%d" % i), b.const("float", x))
    ss = og.ShadingSystem()
    ss.attribute("opt_constant_fold", 0)
    ss.LoadMemoryCompiledShader("logb_edges", b.text())
    g = ss.ShaderGroupBegin("lg")
    ss.Shader(g, "surface", "logb_edges", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1), 1)
    assert [column(out, cols, "L.r%d" % i) for i in range(len(xs))] == [-126, -126, 0, 3, -126, 127, 127, -1]


# ---- gettextureinfo -------------------------------------------------------------------------
GREEN = np.array([26, 128, 26, 255], np.float32) / np.float32(255.0)  # oiiotool constant 0.1,0.5,0.1,1 as uint8


def register_green(ss):
    ss.texture_create("green.tx", np.tile(GREEN, (128, 128, 1)))


def gettextureinfo_group(ss):
    """testsuite/gettextureinfo/test.osl run on green.tx (maketx of a
    128x128 constant uint8 image); strings are compared in the shader."""
    b = OsoBuilder("gti_suite")
    o = Outputs(b, "L")
    S = lambda x: b.const("string", x)
    fn = b.param("string", "filename", "green.tx")

    def q(name, t, data=None):
        d = data if data is not None else b.local(t, "d_" + name)
        b.op("gettextureinfo", o("r_" + name, "int"), fn, S(name), d)
        return d

    res = q("resolution", "int[2]")
    for i in range(2):
        b.op("aref", o("res%d" % i, "int"), res, b.const("int", i))
    b.op("assign", o("channels", "int"), q("channels", "int"))
    for nm in ("texturetype", "textureformat"):
        b.op("eq", o(nm + "_plain", "int"), q(nm, "string"), S("Plain Texture"))
    for nm in ("datawindow", "displaywindow"):
        w = q(nm, "int[4]")
        for i in range(4):
            b.op("aref", o("%s%d" % (nm, i), "int"), w, b.const("int", i))
    b.op("assign", o("averagecolor", "color"), q("averagecolor", "color"))
    b.op("assign", o("averagealpha"), q("averagealpha", "float"))
    b.op("assign", o("constantcolor", "color"), q("constantcolor", "color"))
    b.op("assign", o("constantalpha"), q("constantalpha", "float"))
    fb = b.local("string", "foobar")
    b.op("assign", fb, S("not found"))
    q("foobar", "string", fb)
    b.op("eq", o("foobar_kept", "int"), fb, S("not found"))
    bad = b.local("string", "bad")
    b.op("assign", bad, S("not found"))
    b.op("gettextureinfo", o("r_bad", "int"), S("badfile"), S("textureformat"), bad)
    b.op("eq", o("bad_kept", "int"), bad, S("not found"))
    b.op("assign", o("exists", "int"), q("exists", "int"))
    e3 = b.local("int", "e3")
    b.op("gettextureinfo", o("r_exists3", "int"), S("badfile3"), S("exists"), e3)
    b.op("assign", o("exists3", "int"), e3)
    ss.LoadMemoryCompiledShader("gti_suite", b.text())
    g = ss.ShaderGroupBegin("gti_g")
    ss.Shader(g, "surface", "gti_suite", "L")
    ss.ShaderGroupEnd(g)
    rec, cols = place(ss, g, [o])
    return g, rec, cols


def test_gettextureinfo_matches_the_testsuite():
    ss = og.ShadingSystem()
    register_green(ss)
    g, rec, cols = gettextureinfo_group(ss)
    u, v = pixel_grid(1, 1)
    out = run_oracle(g, rec, grid_globals(u, v, 1, 1), 1)
    C = lambda k: column(out, cols, "L." + k)
    F = "green.tx"
    got = ["%s resolution: %d %d (%d)" % (F, C("res0"), C("res1"), C("r_resolution")),
           "%s channels: %d (%d)" % (F, C("channels"), C("r_channels"))]
    for nm in ("texturetype", "textureformat"):
        assert C(nm + "_plain") == 1
        got.append("%s %s: Plain Texture (%d)" % (F, nm, C("r_" + nm)))
    for nm in ("datawindow", "displaywindow"):
        got.append("%s %s: %d %d %d %d (%d)" % ((F, nm) + tuple(C("%s%d" % (nm, i)) for i in range(4))
                                               + (C("r_" + nm),)))
    for nm in ("averagecolor", "averagealpha", "constantcolor", "constantalpha"):
        got.append("%s %s: %s" % (F, nm, fmt(C(nm))) if C("r_" + nm) else "%s unknown %s" % (F, nm))
    assert C("foobar_kept") == 1 and C("bad_kept") == 1
    got.append("%s foobar: not found (%d)" % (F, C("r_foobar")))
    got.append("badfile data: not found (%d)" % C("r_bad"))
    got.append("%s exists? %d (return %d)" % (F, C("exists"), C("r_exists")))
    got.append("badfile3 exists? %d (return %d)" % (C("exists3"), C("r_exists3")))
    text = ref_lines("gettextureinfo_out.txt")
    block = text[len(text) - text[::-1].index("Executing...") :]
    want = [ln for ln in block if not ln.startswith("ERROR")]
    assert got == want, [(a, b) for a, b in zip(got, want) if a != b]


# ---- unknown instruction ----------------------------------------------------------------
def test_unknown_instruction_is_refused_like_the_reference():
    ss = og.ShadingSystem()
    oso = open(os.path.join(GOLDEN, "unknown_instruction.oso")).read()
    with pytest.raises(og.OSLError) as e:
        ss.LoadMemoryCompiledShader("test", oso)
    first = ref_lines("unknown_instruction_out.txt")[0]
    assert first.startswith("ERROR: ")
    assert first[len("ERROR: "):] in str(e.value)


# ---- sincos, calculatenormal, backfacing, surfacearea, arraycopy ------------------------
def geometry_group(ss):
    b = OsoBuilder("geom_suite")
    o = Outputs(b, "L")
    u = b.glob("float", "u")
    s, c = b.tmp("float"), b.tmp("float")
    ang = b.tmp("float")
    b.op("mul", ang, u, b.const("float", 6.0))
    b.op("sincos", ang, s, c)
    b.op("assign", o("sin", derivs=True), s)
    b.op("assign", o("cos", derivs=True), c)
    P = b.glob("point", "P")
    b.op("calculatenormal", o("Ncalc", "vector"), P)
    b.op("backfacing", o("back", "int"))
    b.op("surfacearea", o("area"))
    src, dst = b.local("float[3]", "src"), b.local("float[2]", "dst")
    for i in range(3):
        b.op("aassign", src, b.const("int", i), u if i == 1 else b.const("float", 10.0 + i))
    b.op("arraycopy", dst, src)
    for i in range(2):
        b.op("aref", o("copy%d" % i), dst, b.const("int", i))
    ss.LoadMemoryCompiledShader("geom_suite", b.text())
    g = ss.ShaderGroupBegin("geom_g")
    ss.Shader(g, "surface", "geom_suite", "L")
    ss.ShaderGroupEnd(g)
    # derivative outputs: one symloc each carrying dx, dy
    cols, off = {}, 0
    locs = []
    specs = [("sin", og.TypeFloat, True, 3, "float"), ("cos", og.TypeFloat, True, 3, "float"),
             ("Ncalc", og.TypeVector, False, 3, "vector"), ("back", og.TypeInt, False, 1, "int"),
             ("area", og.TypeFloat, False, 1, "float"), ("copy0", og.TypeFloat, False, 1, "float"),
             ("copy1", og.TypeFloat, False, 1, "float")]
    rec = sum(s[3] for s in specs)
    for nm, td, d, n, t in specs:
        locs.append(og.SymLocationDesc("L." + nm, td, d, og.SymArenaOutputs, 4 * off, 4 * rec))
        cols["L." + nm] = (off, n, t if n == 1 or t == "vector" else "vec")
        off += n
    ss.add_symlocs(g, locs)
    return g, rec, cols


def geometry_inputs(W, H):
    u, v = pixel_grid(W, H)
    n = W * H
    rng = np.random.default_rng(7)
    dPdx = rng.standard_normal((3, n)).astype(np.float32)
    dPdy = rng.standard_normal((3, n)).astype(np.float32)
    P = rng.standard_normal((3, n)).astype(np.float32)
    flip = (np.arange(n) % 3 == 0).astype(np.int32)
    back = (np.arange(n) % 2 == 1).astype(np.int32)
    area = rng.random(n).astype(np.float32)
    return u, v, P, dPdx, dPdy, flip, back, area


def geometry_globals(W, H, arrays, conv=lambda x: x):
    u, v, P, dPdx, dPdy, flip, back, area = arrays
    du = 1.0 / max(1, W - 1)
    return og.make_globals(u=conv(u), v=conv(v), dudx=du, dudy=0.0, dvdx=0.0, dvdy=1.0, P=conv(P),
                           dPdx=conv(dPdx), dPdy=conv(dPdy), flipHandedness=conv(flip), backfacing=conv(back),
                           surfacearea=conv(area))


def test_sincos_calculatenormal_backfacing_surfacearea_arraycopy():
    ss = og.ShadingSystem()
    g, rec, cols = geometry_group(ss)
    W, H = 16, 4
    arrays = geometry_inputs(W, H)
    u, v, P, dPdx, dPdy, flip, back, area = arrays
    n = W * H
    out = run_oracle(g, rec, geometry_globals(W, H, arrays), n)
    ang = (u * np.float32(6.0)).astype(np.float32)
    s = np.sin(ang.astype(np.float64)).astype(np.float32)
    c = np.cos(ang.astype(np.float64)).astype(np.float32)
    du = np.float32(1.0 / (W - 1)) * np.float32(6.0)
    # OpenImageIO's fast sincos: within 2 ulp of 1 on [-2pi, 2pi]
    assert np.abs(out[:, 0] - s).max() <= 2.4e-7 and np.abs(out[:, 3] - c).max() <= 2.4e-7
    assert np.array_equal(out[:, 1], out[:, 3] * du) and np.array_equal(out[:, 4], -out[:, 0] * du)
    # the math-library forms are correctly rounded
    ss0 = og.ShadingSystem()
    ss0.attribute("fast_math", 0)
    g0, _, _ = geometry_group(ss0)
    out0 = run_oracle(g0, rec, geometry_globals(W, H, arrays), n)
    assert np.array_equal(out0[:, 0], s) and np.array_equal(out0[:, 3], c)
    x, y = dPdx.T, dPdy.T
    want = np.where(flip[:, None] != 0, np.cross(y, x), np.cross(x, y)).astype(np.float32)
    assert np.allclose(out[:, 6:9], want, rtol=1e-6, atol=1e-6)
    assert np.array_equal(out[:, 9].view(np.int32), back)
    assert np.array_equal(out[:, 10], area)
    assert np.array_equal(out[:, 11], np.full(n, 10.0, np.float32)) and np.array_equal(out[:, 12], u)


# ---- GPU == oracle ------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("which", ["raytype", "isconnected", "isconstant", "exponential", "hyperb", "gettextureinfo",
                                   "geometry"])
def test_gpu_misc_ops_equal_the_oracle(which, jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    W, H = 16, 4
    n = W * H
    if which == "geometry":
        g, rec, _ = geometry_group(ss)
        arrays = geometry_inputs(W, H)
        dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]
        Gd = geometry_globals(W, H, dev)
        Gh = geometry_globals(W, H, arrays)
    else:
        g, rec, _ = {"raytype": raytype_group, "isconstant": isconstant_group,
                     "exponential": exponential_group, "hyperb": hyperb_group,
                     "gettextureinfo": lambda s: (register_green(s), gettextureinfo_group(s))[1],
                     "isconnected": lambda s: isconnected_group(s, True)}[which](ss)
        u, v = pixel_grid(W, H)
        du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
        Gd, Gh = grid_globals(du, dv, W, H), grid_globals(u, v, W, H)
        Gd.raytype = Gh.raytype = 1 << 5
    out = torch.zeros(n * rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, Gd, 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    got = out.cpu().numpy().reshape(n, rec)
    ref = run_oracle(g, rec, Gh, n)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
