"""texture(): registration, lowering (options, errors) and the oracle's
mipmapped bilinear lookup against an independent numpy statement of the
same filter (texel centres at (i + 0.5) / size, rows from the top, 2x2 box
pyramid, level of detail log2 of the footprint in level-0 texels)."""
import ctypes

import numpy as np
import pytest

from helpers import grid_globals, og, oracle, oracle_run, pixel_grid, single_layer_group
from openshadinglanguage_gb300.shaders import texture_lookup as tex_shader

WRAPS = ("black", "clamp", "periodic", "mirror")


def make_image(h, w, nch, seed=5):
    return np.random.default_rng(seed).random((h, w, nch), dtype=np.float32)


def register(ss, img, name="img"):
    idx = ss.texture_create(name, img)
    L = oracle()
    L.oracle_texture_create.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p]
    a = np.ascontiguousarray(img, np.float32)
    h, w, nch = a.shape
    assert L.oracle_texture_create(idx, w, h, nch, a.ctypes.data) == 0
    return idx


def np_pyramid(img):
    levels = [img.astype(np.float32)]
    while levels[-1].shape[0] > 1 or levels[-1].shape[1] > 1:
        p = levels[-1]
        h, w = p.shape[:2]
        nh, nw = max(1, h // 2), max(1, w // 2)
        y0 = np.minimum(2 * np.arange(nh), h - 1)
        y1 = np.minimum(2 * np.arange(nh) + 1, h - 1)
        x0 = np.minimum(2 * np.arange(nw), w - 1)
        x1 = np.minimum(2 * np.arange(nw) + 1, w - 1)
        a, b2 = p[y0][:, x0], p[y0][:, x1]
        c, d = p[y1][:, x0], p[y1][:, x1]
        levels.append(((((a + b2) + c) + d) * np.float32(0.25)).astype(np.float32))
        if len(levels) == 16:
            break
    return levels


def np_wrap(i, n, mode):
    if mode == "periodic":
        return np.mod(i, n), np.ones_like(i, bool)
    if mode == "mirror":
        m = np.mod(i, 2 * n)
        return np.where(m < n, m, 2 * n - 1 - m), np.ones_like(i, bool)
    inside = (i >= 0) & (i < n)
    return np.clip(i, 0, n - 1), inside if mode == "black" else np.ones_like(i, bool)


def np_bilinear(lev, s, t, mode):
    H, W = lev.shape[:2]
    x = s.astype(np.float64) * W - 0.5
    y = t.astype(np.float64) * H - 0.5
    x0, y0 = np.floor(x), np.floor(y)
    fx, fy = (x - x0)[:, None], (y - y0)[:, None]
    ix, iy = x0.astype(int), y0.astype(int)
    cx0, in0 = np_wrap(ix, W, mode)
    cx1, in1 = np_wrap(ix + 1, W, mode)
    cy0, jn0 = np_wrap(iy, H, mode)
    cy1, jn1 = np_wrap(iy + 1, H, mode)
    g = lambda cy, cx, m: lev[cy, cx] * m[:, None]
    top = (1 - fx) * g(cy0, cx0, in0 & jn0) + fx * g(cy0, cx1, in1 & jn0)
    bot = (1 - fx) * g(cy1, cx0, in0 & jn1) + fx * g(cy1, cx1, in1 & jn1)
    return (1 - fy) * top + fy * bot


@pytest.mark.parametrize("wrap", WRAPS)
@pytest.mark.parametrize("scale", [1.0, 1.7, 6.0])
def test_oracle_matches_numpy_trilinear(wrap, scale):
    img = make_image(48, 64, 3)
    ss = og.ShadingSystem()
    register(ss, img)
    g = single_layer_group(ss, "tex_%s" % wrap, tex_shader("tex_%s" % wrap, scale, wrap),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    W, H = 40, 30
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out) == 0
    # footprint in level-0 texels: d(s)/dx = scale / W * 64, d(t)/dy = scale / H * 48
    pyr = np_pyramid(img)
    s, t = u * np.float32(scale), v * np.float32(scale)
    length = max(scale / W * 64, scale / H * 48)
    lod = min(np.log2(length) if length > 1 else 0.0, len(pyr) - 1)
    l0 = int(lod)
    f = lod - l0
    ref = np_bilinear(pyr[l0], s, t, wrap)
    if f > 0 and l0 + 1 < len(pyr):
        ref = (1 - f) * ref + f * np_bilinear(pyr[l0 + 1], s, t, wrap)
    assert np.allclose(out, ref, atol=2e-5), np.abs(out - ref).max()


def test_single_channel_and_first_channel():
    img = make_image(16, 16, 4)
    ss = og.ShadingSystem()
    register(ss, img)
    W = H = 16
    u, v = pixel_grid(W, H, centers=True)
    G = grid_globals(u, v, W, H, centers=True)
    g = single_layer_group(ss, "tf", tex_shader("tf", 1.0, "clamp", nc=1, first=2),
                           outputs=[og.SymLocationDesc("Cout", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    out = np.zeros((W * H, 1), np.float32)
    assert oracle_run(g.program_bytes(), W * H, G, out) == 0
    # pixel centres of a same-size image land on texel centres: exact texels
    assert np.array_equal(out[:, 0], img[:, :, 2].ravel())


def test_unregistered_texture_and_bad_options_fail_at_lowering():
    ss = og.ShadingSystem()
    with pytest.raises(og.OSLError, match="not registered"):
        g = single_layer_group(ss, "tn", tex_shader("tn", 1.0),
                               outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
        g.program_bytes()
    register(ss, make_image(4, 4, 3))
    with pytest.raises(og.OSLError, match="wrap mode"):
        g = single_layer_group(ss, "tw", tex_shader("tw", 1.0, wrap="periodic_pow2"),
                               outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
        g.program_bytes()


def test_texture_coordinates_carry_derivatives():
    """s and t feed the footprint: the lowering gives them derivatives."""
    ss = og.ShadingSystem()
    register(ss, make_image(8, 8, 3))
    g = single_layer_group(ss, "td", tex_shader("td", 2.0),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    hdr = np.frombuffer(g.program_bytes()[:64], np.uint32)
    assert hdr[5] & 2  # the program carries derivatives
