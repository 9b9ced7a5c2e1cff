"""Colour spaces pinned to the reference testsuite: transformc (every space
of the colour system both ways, derivatives through YIQ and sRGB),
colorspace (RGB to XYZ, wavelength_color), color (constructors in a
colour space) and the wavelength_color image (testsuite/*/ref, copied to
tests/golden/ by make_golden.py). Each printed value is an output of the
group, formatted the way the shader prints it and compared as text; the
image within 1e-6 relative."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder

SPACES = ("hsv", "hsl", "YIQ", "XYZ", "xyY")


class Shader:
    """A single-layer shader whose outputs are named colours/floats."""

    def __init__(self, name):
        self.b = OsoBuilder(name)
        self.outs = []  # (name, floats, derivs)

    def out(self, name, derivs=False):
        self.outs.append((name, 3, derivs))
        return self.b.param("color", name, [0.0, 0.0, 0.0], output=True)

    def group(self, ss, name):
        ss.LoadMemoryCompiledShader(name, self.b.text())
        g = ss.ShaderGroupBegin(name + "_g")
        ss.Shader(g, "surface", name, "L")
        ss.ShaderGroupEnd(g)
        rec = sum(n * (3 if d else 1) for _, n, d in self.outs)
        locs, off = [], 0
        for nm, n, d in self.outs:
            locs.append(og.SymLocationDesc("L." + nm, og.TypeColor, d, og.SymArenaOutputs, off, 4 * rec))
            off += 4 * n * (3 if d else 1)
        ss.add_symlocs(g, locs)
        return g, rec

    def columns(self, row):
        d, k = {}, 0
        for nm, n, dv in self.outs:
            m = n * (3 if dv else 1)
            d[nm] = row[k:k + m].reshape(-1, 3)
            k += m
        return d


def pretty(x):
    x = np.asarray(x, np.float32).copy()
    x[np.abs(x) < 5e-6] = 0.0
    return x + np.float32(0.0)


def f3(x):
    return " ".join("%0.3f" % float(v) for v in pretty(x))


def transformc_shader():
    """testsuite/transformc/test.osl, each printed colour an output."""
    sh = Shader("tc_suite")
    b = sh.b
    u, v = b.glob("float", "u"), b.glob("float", "v")
    S = lambda x: b.const("string", x)
    c0 = b.const("color", [0.5, 1.0, 0.0])
    uv = b.local("color", "uv")
    b.op("color", uv, u, v, b.const("float", 0.5))
    for sp in SPACES:
        for tag, c in (("c", c0), ("uv", uv)):
            cs = sh.out("%s_%s" % (sp, tag))
            b.op("transformc", cs, S(sp), c)
            b.op("transformc", sh.out("%s_%s_back" % (sp, tag)), S(sp), S("rgb"), cs)
    b.op("transformc", sh.out("lin2srgb"), S("linear"), S("sRGB"), c0)
    b.op("transformc", sh.out("srgb2lin"), S("sRGB"), S("linear"), c0)
    b.op("assign", sh.out("uv_d", True), uv)
    b.op("transformc", sh.out("uv_yiq", True), S("rgb"), S("YIQ"), uv)
    b.op("transformc", sh.out("uv_srgb", True), S("rgb"), S("sRGB"), uv)
    return sh


def run(sh, name, W=1, H=1, colorspace=None):
    ss = og.ShadingSystem()
    if colorspace:
        ss.attribute("colorspace", colorspace)
    g, rec = sh.group(ss, name)
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    return g, out


def transformc_text(d):
    L = []
    c0 = np.array([0.5, 1.0, 0.0], np.float32)
    for sp in SPACES:
        for tag, c in (("c", c0), ("uv", d["uv_d"][0])):
            cs, back = d["%s_%s" % (sp, tag)][0], d["%s_%s_back" % (sp, tag)][0]
            L.append("rgb %s = %s %s" % (f3(c), sp, f3(cs)))
            L.append("%s %s = rgb %s" % (sp, f3(cs), f3(back)))
            L.append("    residual = %s" % f3(np.abs(back - c)))
    L.append('transformc ("linear","sRGB",(%s)) = %s' % (f3(c0), f3(d["lin2srgb"][0])))
    L.append('transformc ("sRGB","linear",(%s)) = %s' % (f3(c0), f3(d["srgb2lin"][0])))
    uvd, y, s = d["uv_d"], d["uv_yiq"], d["uv_srgb"]
    L.append('transformc ("rgb","YIQ",(%s / %s / %s)) = %s / %s / %s'
             % (f3(uvd[0]), f3(uvd[1]), f3(uvd[2]), f3(y[0]), f3(y[1]), f3(y[2])))
    L.append('transformc ("rgb","sRGB",(%s / %s / %s)) = %s / %s / %s'
             % (f3(uvd[0]), f3(uvd[1]), f3(uvd[2]), f3(s[0]), f3(s[1]), f3(s[2])))
    return L


def test_transformc_matches_the_testsuite():
    sh = transformc_shader()
    _, out = run(sh, "tc_suite")
    got = transformc_text(sh.columns(out.view(np.float32)[0]))
    ref = [ln for ln in open(os.path.join(GOLDEN, "transformc_out.txt")).read().splitlines()
           if ln and not ln.startswith("Compiled")]
    assert got == ref, [(a, b) for a, b in zip(got, ref) if a != b][:5]


def color_spaces_shader():
    """testsuite/color "testing with spaces" block and the colorspace test's
    RGB -> XYZ and wavelength_color(500)."""
    sh = Shader("col_suite")
    b = sh.b
    f = lambda x: b.const("float", x)
    S = lambda x: b.const("string", x)
    for i, (sp, a, bb, c) in enumerate([("rgb", .1, .2, .5), ("hsv", .1, .2, .5), ("hsv", 0, 0, .5),
                                        ("hsv", .5, 1, .5), ("hsl", 0, 0, .5), ("hsl", .5, 1, .1),
                                        ("YIQ", .5, .25, .25), ("XYZ", .25, .5, .25)]):
        b.op("color", sh.out("k%d" % i), S(sp), f(a), f(bb), f(c))
    b.op("transformc", sh.out("rgb2xyz"), S("RGB"), S("XYZ"), b.const("color", [0.1, 0.7, 0.2]))
    b.op("wavelength_color", sh.out("wl500"), f(500.0))
    b.op("blackbody", sh.out("bb1500"), f(1500.0))
    return sh


def g(x, fmt="%g"):
    return " ".join(fmt % float(v) for v in pretty(x))


def test_color_space_constructors_and_colorspace_match_the_testsuite():
    sh = color_spaces_shader()
    _, out = run(sh, "col_suite")
    d = sh.columns(out[0])
    got = ['  color ("rgb", 0.1, 0.2, 0.5) = ' + g(d["k0"][0]),
           '  color ("hsv", 0.1, 0.2, 0.5) = ' + g(d["k1"][0]),
           '  color ("hsv", 0, 0, 0.5) = ' + g(d["k2"][0]),
           '  color ("hsv", 0.5, 1, 0.5) = ' + g(d["k3"][0]),
           '  color ("hsl", 0, 0, 0.5) = ' + g(d["k4"][0]),
           '  color ("hsl", 0.5, 1, 0.1) = ' + g(d["k5"][0]),
           '  color ("YIQ", 0.5, 0.25, 0.25) = ' + g(d["k6"][0]),
           '  color ("XYZ", 0.25, 0.5, 0.25) = ' + g(d["k7"][0], "%0.4g")]
    text = open(os.path.join(GOLDEN, "color_out.txt")).read().splitlines()
    start = text.index("testing with spaces:") + 1
    assert got == text[start:start + len(got)], [(a, b) for a, b in zip(got, text[start:]) if a != b]

    # testsuite/colorspace runs with -colorspace ACEScg
    sh2 = color_spaces_shader()
    _, out2 = run(sh2, "col_suite_aces", colorspace="ACEScg")
    d2 = sh2.columns(out2[0])
    cs = open(os.path.join(GOLDEN, "colorspace_out.txt")).read().splitlines()
    assert "  RGB to XYZ (0.1 0.7 0.2) = (%s)" % g(d2["rgb2xyz"][0]) == cs[1]
    assert "  wavelength (500) = %s" % g(d2["wl500"][0]) == cs[3]
    # blackbody: the reference's table uses OIIO's fast expm1/cbrt, this one
    # double precision (agreement to about 1e-4 relative)
    want = np.array([float(x) for x in cs[2].split("=")[1].split()], np.float32)
    assert np.allclose(d2["bb1500"][0], want, rtol=2e-4), (d2["bb1500"][0], want)


def wavelength_shader():
    """testsuite/wavelength_color/test.osl: Cout = wavelength_color(1000 * u)."""
    sh = Shader("wl_suite")
    b = sh.b
    lam = b.tmp("float")
    b.op("mul", lam, b.const("float", 1000.0), b.glob("float", "u"))
    b.op("wavelength_color", sh.out("Cout"), lam)
    return sh


def test_wavelength_color_image():
    ref = np.load(os.path.join(GOLDEN, "wavelength_color.npz"))["imgs"][0]
    H, W = ref.shape[:2]
    _, out = run(wavelength_shader(), "wl_suite", W, H)
    img = out.reshape(H, W, 3)
    err = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert err.max() < 1e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("which", ["transformc", "spaces", "wavelength"])
def test_gpu_color_ops_equal_the_oracle(which, jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    sh, W, H = {"transformc": (transformc_shader(), 3, 2), "spaces": (color_spaces_shader(), 1, 1),
                "wavelength": (wavelength_shader(), 1000, 8)}[which]
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g, rec = sh.group(ss, "gpu_" + which)
    u, v = pixel_grid(W, H)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.zeros(W * H * rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, W * H, grid_globals(du, dv, W, H), 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    got = out.cpu().numpy().reshape(W * H, rec)
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
