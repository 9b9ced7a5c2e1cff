"""The oracle against the reference testsuite's spline images
(testsuite/spline/test.osl, `testshade -g 256 256 -od uint8`): every basis
(catmull-rom, bezier, bspline, hermite, linear) over a constant color knot
array and a varying float knot array, their x derivatives (100 * Dx) and the
explicit knot count form, within runtest's thresholds.

The shader picks the basis per row band, basis = int(v * 5), from a string
array; this executor needs a constant basis name, so each band runs the
same shader with that band's basis."""
import numpy as np
import pytest

from helpers import golden_image, grid_globals, image_diff_ok, og, oracle_run, pixel_grid, to_uint8

BASES = ["catmull-rom", "bezier", "bspline", "hermite", "linear"]
COLORS = [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1)]
KNOT_SCALE = [0.0, 0.0, 1.0, 1.0, 1.0, 0.5, 0.5, 0.5, 1.0, 1.0, 1.0, 0.0, 0.0]


def spline_shader(k):
    """testsuite/spline/test.osl with basis k fixed."""
    b = og.OsoBuilder("spline_t%d" % k)
    outs = {nm: b.param(ty, nm, 0.0, output=True) for nm, ty in
            [("Cspline", "color"), ("DxCspline", "color"), ("Fspline", "float"), ("DxFspline", "float"),
             ("NumKnots", "float")]}
    u = b.glob("float", "u")
    col = COLORS[k]
    # colknots[i] = scale_i * knot_col: float products, as the shader computes them
    ck = [np.float32(s) * np.float32(c) for s in KNOT_SCALE for c in col]
    colknots = b.param("color[13]", "colknots", [float(x) for x in ck])
    fltknots = b.local("float[13]", "fltknots")
    for i, sc in enumerate(KNOT_SCALE):
        t = b.tmp("float")
        b.op("mul", t, b.const("float", sc), u)
        b.op("aassign", fltknots, b.const("int", i), t)
    basis = b.const("string", BASES[k])
    hundred = b.const("float", 100.0)
    b.op("spline", outs["Cspline"], basis, u, colknots)
    dc = b.tmp("color")
    b.op("Dx", dc, outs["Cspline"])
    b.op("mul", outs["DxCspline"], hundred, dc)
    b.op("spline", outs["Fspline"], basis, u, fltknots)
    df = b.tmp("float")
    b.op("Dx", df, outs["Fspline"])
    b.op("mul", outs["DxFspline"], hundred, df)
    b.op("spline", outs["NumKnots"], b.const("string", "linear"), u, b.const("int", 4), fltknots)
    return b.text()


def render():
    W = H = 256
    u, v = pixel_grid(W, H)
    band = np.minimum((v * np.float32(5.0)).astype(np.int32), 4)
    out = np.zeros((W * H, 9), np.float32)
    for k in range(5):
        ss = og.ShadingSystem()
        ss.LoadMemoryCompiledShader("spline_t%d" % k, spline_shader(k))
        g = ss.ShaderGroupBegin("gspline%d" % k)
        ss.Shader(g, "surface", "spline_t%d" % k, "l")
        ss.ShaderGroupEnd(g)
        off = 0
        locs = []
        for nm, ty, n in [("Cspline", og.TypeColor, 3), ("DxCspline", og.TypeColor, 3), ("Fspline", og.TypeFloat, 1),
                          ("DxFspline", og.TypeFloat, 1), ("NumKnots", og.TypeFloat, 1)]:
            locs.append(og.SymLocationDesc("l." + nm, ty, False, og.SymArenaOutputs, off, 36))
            off += 4 * n
        ss.add_symlocs(g, locs)
        idx = np.nonzero(band == k)[0]
        part = np.zeros((len(idx), 9), np.float32)
        G = grid_globals(np.ascontiguousarray(u[idx]), np.ascontiguousarray(v[idx]), W, H)
        assert oracle_run(g.program_bytes(), len(idx), G, part) == 0
        out[idx] = part
    return out.reshape(H, W, 9)


@pytest.fixture(scope="module")
def image():
    return render()


@pytest.mark.parametrize("name,cols,alts", [("spline_color", slice(0, 3), ()),
                                            ("spline_dcolor", slice(3, 6), ("spline_dcolor_alt",)),
                                            ("spline_float", slice(6, 7), ()),
                                            ("spline_dfloat", slice(7, 8), ()),
                                            ("spline_numknots", slice(8, 9), ())])
def test_oracle_matches_spline_images(image, name, cols, alts):
    results = []
    for fixture in (name,) + alts:
        ref, W, H, step = golden_image(fixture)
        got = to_uint8(image[:, :, cols])[::step, ::step]
        results.append(image_diff_ok(got, ref))
    assert any(r[0] for r in results), (name, [(r[1], r[2]) for r in results])
    # in practice every sampled pixel equals the primary reference image
    assert results[0][1] == 0.0 and results[0][2] == 0.0


# ---- splineinverse --------------------------------------------------------------------------

INV_KNOTS = [0.0, 0.0, 0.05, 0.1, 0.3, 1.0, 1.0]


def splineinverse_group(ss, basis, knots=INV_KNOTS, name=None):
    """x = splineinverse(basis, u, knots), with x and Dx(x) as outputs
    (testsuite/splineinverse/test.osl)."""
    name = name or "sinv_" + basis.replace("-", "_")
    b = og.OsoBuilder(name)
    x = b.param("float", "x", 0.0, output=True)
    dx = b.param("float", "dx", 0.0, output=True)
    u = b.glob("float", "u")
    kn = b.param("float[%d]" % len(knots), "knots", list(knots))
    b.op("splineinverse", x, b.const("string", basis), u, kn)
    b.op("Dx", dx, x)
    ss.LoadMemoryCompiledShader(name, b.text())
    g = ss.ShaderGroupBegin(name + "_g")
    ss.Shader(g, "surface", name, "l")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l.x", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
                       og.SymLocationDesc("l.dx", og.TypeFloat, False, og.SymArenaOutputs, 4, 8)])
    return g


def test_splineinverse_matches_reference_output():
    """testshade -g 3 1 --center: u = 1/6, 1/2, 5/6 with Dx(u) = 1/3; the
    printed values and x derivatives (%g) of every basis."""
    import os
    import re
    from helpers import GOLDEN
    txt = open(os.path.join(GOLDEN, "splineinverse_out.txt")).read()
    expected = re.findall(r'splineinverse\("([a-z-]+)", ([0-9.e-]+)\) = ([0-9.e-]+)  \(derivs ([0-9.e-]+) ', txt)
    assert len(expected) == 9
    u, v = pixel_grid(3, 1, centers=True)
    for basis in ("linear", "catmull-rom", "bspline"):
        ss = og.ShadingSystem()
        g = splineinverse_group(ss, basis)
        out = np.zeros((3, 2), np.float32)
        assert oracle_run(g.program_bytes(), 3, grid_globals(u, v, 3, 1, centers=True), out) == 0
        got = [(basis, "%g" % uu, "%g" % out[i, 0], "%g" % out[i, 1]) for i, uu in enumerate(u)]
        want = [e for e in expected if e[0] == basis]
        assert got == want, (got, want)


def test_spline_of_splineinverse_matches_nonuniform_knots_image():
    """testsuite/spline-nonuniformknots (testshade -g 256 64): Cout =
    spline("linear", splineinverse("linear", u, knots), colors)."""
    ss = og.ShadingSystem()
    b = og.OsoBuilder("nonuni")
    cout = b.param("color", "Cout", 0.0, output=True)
    u = b.glob("float", "u")
    kn = b.param("float[5]", "knots", [0.2, 0.2, 0.5, 0.8, 0.8])
    cols = b.param("color[5]", "colors", [1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 1])
    pos = b.tmp("float")
    lin = b.const("string", "linear")
    b.op("splineinverse", pos, lin, u, kn)
    b.op("spline", cout, lin, pos, cols)
    ss.LoadMemoryCompiledShader("nonuni", b.text())
    g = ss.ShaderGroupBegin("gnonuni")
    ss.Shader(g, "surface", "nonuni", "l")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l.Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    ref, W, H, step = golden_image("spline_nonuniform")
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    got = to_uint8(out.reshape(H, W, 3))[::step, ::step]
    ok, frac, mx = image_diff_ok(got, ref)
    assert ok and frac == 0.0, (frac, mx)


def ident_shader(k):
    """testsuite/splineinverse-ident/test.osl with the band's basis fixed:
    spline, splineinverse of u and of the spline value; red where
    splineinverse(spline(u)) strays from the spline value."""
    basis = ["linear", "catmull-rom", "bspline", "bezier"][k]
    cvs = [0.0, 1.0 / 3, 2.0 / 3, 1.0] if basis == "bezier" else [-1.0, 0.0, 1.0, 2.0]
    b = og.OsoBuilder("sident%d" % k)
    cout = b.param("color", "Cout", 0.0, output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    F = lambda x: b.const("float", x)
    kn = b.param("float[4]", "cvs", [float(np.float32(c)) for c in cvs])
    v4, vv = b.tmp("float"), b.tmp("float")
    b.op("mul", v4, v, F(4.0))
    b.op("fmod", vv, v4, F(1.0))
    c1, c2, edge = b.tmp("int"), b.tmp("int"), b.tmp("int")
    b.op("lt", c1, vv, F(0.1))
    b.op("gt", c2, vv, F(0.9))
    b.op("or", edge, c1, c2)
    name = b.const("string", basis)
    with b.if_(edge) as br:
        b.op("assign", cout, F(0.0))
        br.else_()
        s, inv_u, invs = b.tmp("float"), b.tmp("float"), b.tmp("float")
        b.op("spline", s, name, u, kn)
        b.op("splineinverse", inv_u, name, u, kn)
        b.op("splineinverse", invs, name, s, kn)
        lower = b.tmp("int")
        b.op("lt", lower, vv, F(0.5))
        with b.if_(lower) as br2:
            b.op("assign", cout, s)
            br2.else_()
            b.op("assign", cout, inv_u)
        d, ad, big = b.tmp("float"), b.tmp("float"), b.tmp("int")
        b.op("sub", d, s, invs)
        b.op("abs", ad, d)
        b.op("gt", big, ad, F(0.001))
        with b.if_(big):
            b.op("compassign", cout, b.const("int", 0), ad)
    return b.text()


def test_splineinverse_identity_image():
    """testsuite/splineinverse-ident (testshade -g 256 256), one band per
    basis: spline(u), splineinverse(u) and the red error marks."""
    ref, W, H, step = golden_image("splineinverse_ident")
    u, v = pixel_grid(W, H)
    band = np.clip((v * np.float32(4.0)), 0, 3).astype(np.int32)
    out = np.zeros((W * H, 3), np.float32)
    for k in range(4):
        ss = og.ShadingSystem()
        ss.LoadMemoryCompiledShader("sident%d" % k, ident_shader(k))
        g = ss.ShaderGroupBegin("gsident%d" % k)
        ss.Shader(g, "surface", "sident%d" % k, "l")
        ss.ShaderGroupEnd(g)
        ss.add_symlocs(g, [og.SymLocationDesc("l.Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
        idx = np.nonzero(band == k)[0]
        part = np.zeros((len(idx), 3), np.float32)
        G = grid_globals(np.ascontiguousarray(u[idx]), np.ascontiguousarray(v[idx]), W, H)
        assert oracle_run(g.program_bytes(), len(idx), G, part) == 0
        out[idx] = part
    got = to_uint8(out.reshape(H, W, 3))[::step, ::step]
    ok, frac, mx = image_diff_ok(got, ref)
    assert ok and frac == 0.0 and mx == 0.0, (frac, mx)  # every sampled pixel exact


def test_spline_with_too_few_knots_reports_bounds():
    """A knot count below four (here a varying count of 3) has no segment:
    the result is 0 and the index-out-of-range status bit is set, for spline
    and splineinverse alike."""
    ss = og.ShadingSystem()
    b = og.OsoBuilder("fewknots")
    r1 = b.param("float", "r1", 9.0, output=True)
    r2 = b.param("float", "r2", 9.0, output=True)
    u = b.glob("float", "u")
    kn = b.param("float[6]", "kn", [0.0, 0.1, 0.2, 0.3, 0.4, 0.5])
    cnt = b.tmp("int")
    b.op("assign", cnt, b.const("int", 3))
    lin = b.const("string", "linear")
    b.op("spline", r1, lin, u, cnt, kn)
    b.op("splineinverse", r2, lin, u, cnt, kn)
    ss.LoadMemoryCompiledShader("fewknots", b.text())
    g = ss.ShaderGroupBegin("gfew")
    ss.Shader(g, "surface", "fewknots", "l")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l.r1", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
                       og.SymLocationDesc("l.r2", og.TypeFloat, False, og.SymArenaOutputs, 4, 8)])
    u, v = pixel_grid(8, 1)
    out = np.zeros((8, 2), np.float32)
    st = oracle_run(g.program_bytes(), 8, grid_globals(u, v, 8, 1), out)
    assert st & 4 and np.all(out == 0.0)


def test_constant_and_linear_color_spline_image():
    """testsuite/spline constspline (constcolor.tif): 9 color knots,
    "constant" basis in the lower half (v < 0.5), "linear" in the upper."""
    cols = [0, 0, 0, 0, 0, 1, 0, 1, 0, 0, 1, 1, 1, 0, 0, 1, 0, 1, 1, 1, 0, 1, 1, 1, 0, 0, 0]
    ref, W, H, step = golden_image("spline_constcolor")
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 3), np.float32)
    for basis, sel in (("constant", v < 0.5), ("linear", v >= 0.5)):
        ss = og.ShadingSystem()
        b = og.OsoBuilder("cspl_" + basis)
        cs = b.param("color", "Cspline", 0.0, output=True)
        kn = b.param("color[9]", "colors", [float(c) for c in cols])
        b.op("spline", cs, b.const("string", basis), b.glob("float", "u"), kn)
        ss.LoadMemoryCompiledShader("cspl_" + basis, b.text())
        g = ss.ShaderGroupBegin("gcspl_" + basis)
        ss.Shader(g, "surface", "cspl_" + basis, "l")
        ss.ShaderGroupEnd(g)
        ss.add_symlocs(g, [og.SymLocationDesc("l.Cspline", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
        idx = np.nonzero(sel)[0]
        part = np.zeros((len(idx), 3), np.float32)
        G = grid_globals(np.ascontiguousarray(u[idx]), np.ascontiguousarray(v[idx]), W, H)
        assert oracle_run(g.program_bytes(), len(idx), G, part) == 0
        out[idx] = part
    got = to_uint8(out.reshape(H, W, 3))[::step, ::step]
    ok, frac, mx = image_diff_ok(got, ref)
    assert ok and frac == 0.0 and mx == 0.0, (frac, mx)


@pytest.mark.parametrize("name,cols,alts", [("spline_derivbug_color", slice(0, 3), ()),
                                            ("spline_derivbug_dx", slice(3, 6), ("spline_derivbug_dx_alt",)),
                                            ("spline_derivbug_dy", slice(6, 9), ())])
def test_spline_derivatives_image(name, cols, alts):
    """testsuite/spline-derivbug (testshade -g 64 64): a bspline over 8
    color knots with an explicit knot count; Cout, 0.5 + 10 Dx(Cout),
    0.5 + 10 Dy(Cout)."""
    vals = [0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 1, 1, 1, 1, 1, 1, 1, 1]
    b = og.OsoBuilder("derivbug")
    cout = b.param("color", "Cout", 0.0, output=True)
    cdx = b.param("color", "Cout_dx", 0.0, output=True)
    cdy = b.param("color", "Cout_dy", 0.0, output=True)
    kn = b.param("color[8]", "values", [float(x) for x in vals])
    b.op("spline", cout, b.const("string", "bspline"), b.glob("float", "u"), b.const("int", 8), kn)
    for out, op in ((cdx, "Dx"), (cdy, "Dy")):
        d, t = b.tmp("color"), b.tmp("color")
        b.op(op, d, cout)
        b.op("mul", t, b.const("float", 10.0), d)
        b.op("add", out, b.const("float", 0.5), t)
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("derivbug", b.text())
    g = ss.ShaderGroupBegin("gderivbug")
    ss.Shader(g, "surface", "derivbug", "l")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l." + nm, og.TypeColor, False, og.SymArenaOutputs, 12 * i, 36)
                       for i, nm in enumerate(("Cout", "Cout_dx", "Cout_dy"))])
    ref, W, H, step = golden_image(name)
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 9), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    results = []
    for fixture in (name,) + alts:
        r, W, H, step = golden_image(fixture)
        results.append(image_diff_ok(to_uint8(out.reshape(H, W, 9)[:, :, cols])[::step, ::step], r))
    assert any(r[0] for r in results), (name, [(r[1], r[2]) for r in results])
