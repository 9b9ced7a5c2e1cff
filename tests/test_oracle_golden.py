"""The CPU oracle against the reference's own known answers and golden
outputs (parity pinning). No GPU needed."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from helpers import (GOLDEN, golden_image, image_diff_ok, og, oracle, oracle_run, pixel_grid, shaders,
                     single_layer_group, grid_globals, to_uint8)

NK_PERLIN, NK_UPERLIN, NK_CELL, NK_HASH, NK_SIMPLEX, NK_USIMPLEX = 0, 1, 2, 3, 4, 5


def noise(kind, dims, vec, coords, derivs=False, periodic=False, periods=(1, 1, 1, 1)):
    """coords: list of (val, dx, dy) per input float; dims 3/4 pass a point
    (three entries) and, for 4D, a time."""
    inp = np.zeros(12, np.float32)
    for i, c in enumerate(coords):
        inp[3 * i: 3 * i + 3] = c
    out = np.zeros(9, np.float32)
    per = np.asarray(periods, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    oracle().oracle_noise(kind, dims, int(vec), int(derivs), int(periodic), inp.ctypes.data_as(fp),
                          per.ctypes.data_as(fp), out.ctypes.data_as(fp))
    return out.reshape(3, 3)  # [channel][val,dx,dy]


def _coords(dims, x, t=None):
    if dims == 1:
        return [(x, 0, 0)]
    if dims == 2:
        return [(x, 0, 0), (x, 0, 0)]
    if dims == 3:
        return [(x, 0, 0)] * 3
    return [(x, 0, 0)] * 3 + [(x if t is None else t, 0, 0)]


KNOWN = json.load(open(os.path.join(GOLDEN, "oslnoise_known.json")))


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
def test_perlin_known_answers(dims):
    # src/liboslnoise/oslnoise_test.cpp:85-181, eps 1e-3 (snoise, noise, vsnoise)
    ref = KNOWN["test_perlin.results_%dd" % dims]
    vref = KNOWN["test_perlin.vresults_%dd" % dims]
    for i in range(9):
        x = np.float32(i / 4.0)
        s = noise(NK_PERLIN, dims, False, _coords(dims, x))[0, 0]
        assert abs(s - ref[i]) < 1e-3, (dims, i, s, ref[i])
        n = noise(NK_UPERLIN, dims, False, _coords(dims, x))[0, 0]
        assert abs(n - (0.5 + 0.5 * s)) < 1e-3
        vs = noise(NK_PERLIN, dims, True, _coords(dims, x))[:, 0]
        assert np.all(np.abs(vs - np.asarray(vref[i])) < 1e-3), (dims, i, vs, vref[i])


@pytest.mark.parametrize("dims", [1, 2, 3, 4])
def test_cell_known_answers(dims):
    # oslnoise_test.cpp:211-252
    ref = KNOWN["test_cell.results_%dd" % dims]
    vref = KNOWN["test_cell.vresults_%dd" % dims]
    for i in range(2):
        x = np.float32(0.5 + i)
        s = noise(NK_CELL, dims, False, _coords(dims, x))[0, 0]
        assert abs(s - ref[i]) < 1e-3, (dims, i, s, ref[i])
        vs = noise(NK_CELL, dims, True, _coords(dims, x))[:, 0]
        assert np.all(np.abs(vs - np.asarray(vref[i])) < 1e-3)


def test_cell_integer_boundaries():
    # oslnoise_test.cpp:248-252
    c = lambda x: noise(NK_CELL, 1, False, [(np.float32(x), 0, 0)])[0, 0]
    assert c(1.0001) == c(1.0)
    assert c(0.9999) != c(1.0)
    assert c(0.9999) == c(0.0)
    assert c(0.0001) == c(0.0)
    assert c(-0.0001) != c(0.0)


def test_perlin_continuity_at_lattice():
    # oslnoise_test.cpp:176-181
    n = lambda x: noise(NK_UPERLIN, 1, False, [(np.float32(x), 0, 0)])[0, 0]
    for a, b in [(0.9999, 1.0), (1.0001, 1.0), (-0.0001, 0.0), (0.0001, 0.0), (-1.0001, -1.0), (-0.9999, -1.0)]:
        assert abs(n(a) - n(b)) < 1e-3


def test_perlin_derivatives_match_finite_differences():
    # the Dual2 partials of noise agree with a centred difference
    # (the property src/liboslexec/dual_test.cpp checks for Dual2 math)
    rng = np.random.default_rng(7)
    for dims in (1, 2, 3, 4):
        for _ in range(20):
            x = rng.uniform(-5, 5, 4).astype(np.float32)
            coords = [(x[k], 1.0 if k == 0 else 0.0, 1.0 if k == 1 else 0.0) for k in range(dims)]
            r = noise(NK_PERLIN, dims, True, coords, derivs=True)
            h = 1e-3
            xp = x.copy(); xp[0] += h
            xm = x.copy(); xm[0] -= h
            fp = noise(NK_PERLIN, dims, True, [(xp[k], 0, 0) for k in range(dims)])[:, 0]
            fm = noise(NK_PERLIN, dims, True, [(xm[k], 0, 0) for k in range(dims)])[:, 0]
            fd = (fp - fm) / (2 * h)
            assert np.all(np.abs(r[:, 1] - fd) < 5e-2 * (1 + np.abs(fd))), (dims, x, r[:, 1], fd)


def test_simplex_derivatives_match_finite_differences():
    rng = np.random.default_rng(8)
    for dims in (1, 2, 3, 4):
        for _ in range(20):
            x = rng.uniform(-5, 5, 4).astype(np.float32)
            coords = [(x[k], 1.0 if k == 0 else 0.0, 0.0) for k in range(dims)]
            r = noise(NK_SIMPLEX, dims, False, coords, derivs=True)
            h = 1e-3
            xp = x.copy(); xp[0] += h
            xm = x.copy(); xm[0] -= h
            fp = noise(NK_SIMPLEX, dims, False, [(xp[k], 0, 0) for k in range(dims)])[0, 0]
            fm = noise(NK_SIMPLEX, dims, False, [(xm[k], 0, 0) for k in range(dims)])[0, 0]
            fd = (fp - fm) / (2 * h)
            assert abs(r[0, 1] - fd) < 5e-2 * (1 + abs(fd)), (dims, x, r[0, 1], fd)


def test_hash_is_lookup3_final_mix():
    # inthash of one key (oslnoise.h:224-231): bjfinal(s+k, s, s), s = 0xdeadbeef + 4 + 13
    def rot(x, k):
        return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF

    def bjfinal(a, b, c):
        M = 0xFFFFFFFF
        c ^= b; c = (c - rot(b, 14)) & M
        a ^= c; a = (a - rot(c, 11)) & M
        b ^= a; b = (b - rot(a, 25)) & M
        c ^= b; c = (c - rot(b, 16)) & M
        a ^= c; a = (a - rot(c, 4)) & M
        b ^= a; b = (b - rot(a, 14)) & M
        c ^= b; c = (c - rot(b, 24)) & M
        return c

    s = (0xdeadbeef + 4 + 13) & 0xFFFFFFFF
    for k in [0, 1, 2, 12345, 0xFFFFFFFF]:
        arr = (ctypes.c_uint32 * 1)(k)
        assert oracle().oracle_inthash(arr, 1) == bjfinal((s + k) & 0xFFFFFFFF, s, s)


TESTSUITE = [
    # (fixture, shader kwargs) -- testsuite/<dir>/run.py command lines
    ("noise", dict(with_name=False, opname="noise", offset_default=0.0, scale_default=1.0)),
    ("cellnoise", dict(with_name=False, opname="cellnoise", offset_default=0.0, scale_default=1.0)),
    ("hashnoise", dict(with_name=False, opname="hashnoise", offset_default=0.0, scale_default=1.0)),
    ("noise_perlin", dict(noisename_default="perlin")),
    ("noise_cell", dict(noisename_default="cell", offset_default=0.0, scale_default=1.0)),
    ("noise_simplex", dict(noisename_default="simplex")),
    ("noise_gabor", dict(noisename_default="gabor", failpercent=0.05)),
    ("pnoise_perlin", dict(builder="testpnoise", noisename_default="perlin")),
    ("pnoise_cell", dict(builder="testpnoise", noisename_default="cell", offset_default=0.0, scale_default=1.0)),
    ("pnoise_gabor", dict(builder="testpnoise", noisename_default="gabor", failpercent=0.05)),
    ("noise_gabor2d_filter", dict(builder="gabor_filter", dims=2, failpercent=0.05)),
    ("noise_gabor3d_filter", dict(builder="gabor_filter", dims=3, failpercent=0.05)),
]


def suite_program(name, kw):
    kw = dict(kw)
    builder = kw.pop("builder", "testnoise")
    kw.pop("failpercent", None)
    ss = og.ShadingSystem()
    if builder == "gabor_filter":
        oso = shaders.gabor_filter_test(kw["dims"], shader_name="t_" + name)
    elif builder == "testpnoise":
        oso = shaders.testpnoise(shader_name="t_" + name, **kw)
    else:
        oso = shaders.testnoise(shader_name="t_" + name, **kw)
    g = single_layer_group(ss, "t_" + name, oso,
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    return ss, g


def suite_P(kw, u, v):
    """testshade's P = (u, v, 1) for the shaders that read P, else None."""
    if kw.get("builder") != "gabor_filter":
        return None
    return np.stack([u, v, np.ones_like(u)]).astype(np.float32)


@pytest.mark.parametrize("name,kw", TESTSUITE)
def test_oracle_matches_testsuite_images(name, kw):
    ss, g = suite_program(name, kw)
    blob = g.program_bytes()
    ref, W, H, step = golden_image(name)
    u, v = pixel_grid(W, H)
    G = grid_globals(u, v, W, H, P=suite_P(kw, u, v))
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(blob, W * H, G, out) == 0
    img = to_uint8(out.reshape(H, W, 3))[::step, ::step]
    ok, frac, mx = image_diff_ok(img, ref, failpercent=kw.get("failpercent", 0.02))
    assert ok, (name, frac, mx)
    # in practice the oracle reproduces every sampled pixel to within 1/255
    assert frac == 0.0


def deformer_group(ss):
    """testsuite/example-batched-deformer/oslbatcheddeformer.cpp:230-325"""
    ss.LoadMemoryCompiledShader("getP", shaders.getP())
    ss.LoadMemoryCompiledShader("vfBm3d", shaders.vfBm3d())
    ss.LoadMemoryCompiledShader("vadd", shaders.vadd())
    g = ss.ShaderGroupBegin("my_noise_deformer")
    ss.Shader(g, "displacement", "getP", "layer1")
    ss.Parameter(g, "amplitude", og.TypeFloat, 1.0, lockgeom=False)
    ss.Shader(g, "displacement", "vfBm3d", "layer2")
    ss.ConnectShaders(g, "layer1", "out", "layer2", "position")
    ss.Shader(g, "displacement", "vadd", "layer3")
    ss.ConnectShaders(g, "layer1", "out", "layer3", "a")
    ss.ConnectShaders(g, "layer2", "out", "layer3", "b")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("layer3.out", og.TypePoint, False, og.SymArenaOutputs, 0, 12),
                       og.SymLocationDesc("amplitude", og.TypeFloat, False, og.SymArenaUserData, 0, 4)])
    return g


def deformer_inputs():
    n = 20
    P = np.zeros((3, n), np.float32)
    P[0] = (np.float32(0.1) * np.arange(n, dtype=np.float32)).astype(np.float32)
    amp = np.array([0.0 + 1.0 * (i / float(n)) ** 3.0 for i in range(n)], np.float32)
    return n, P, amp


def deformer_expected():
    lines = [l for l in open(os.path.join(GOLDEN, "deformer_out.txt")) if "Deformed" in l]
    rows = []
    for l in lines:
        m = re.search(r"Deformed \(([^)]*)\)", l)
        rows.append(m.group(1))
    return rows


def fmt_g3(x):
    s = "%.3g" % x
    return s


def test_oracle_matches_batched_deformer_output():
    ss = og.ShadingSystem()
    g = deformer_group(ss)
    n, P, amp = deformer_inputs()
    G = og.make_globals(P=P)
    out = np.zeros((n, 3), np.float32)
    assert oracle_run(g.program_bytes(), n, G, out, userdata=amp) == 0
    exp = deformer_expected()
    got = [" ".join(fmt_g3(c) for c in row) for row in out]
    assert got == exp


def blackbody_program(ss, scale=10000.0):
    return single_layer_group(ss, "test", shaders.blackbody_test(scale),
                              outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])


def test_oracle_blackbody_matches_reference_image():
    """testsuite/blackbody: 1000x64 half-float image, runtest thresholds
    (failthresh 0.004, failpercent 0.05) against any of its reference images."""
    ss = og.ShadingSystem()
    g = blackbody_program(ss)
    refs = np.load(os.path.join(GOLDEN, "blackbody.npz"))["imgs"]
    W, H = 1000, 64
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    img = out.reshape(H, W, 3).astype(np.float16).astype(np.float32)
    fracs = [100.0 * np.mean(np.abs(img - r) > 0.004 + 1e-9) for r in refs]
    assert min(fracs) <= 0.05, fracs
