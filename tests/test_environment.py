"""environment(): a registered latitude-longitude image looked up by
direction (z up; s = atan2(y, x) / 2pi + 0.5 periodic, t = 0.5 -
atan2(z, hypot(x, y)) / pi clamped), filtered by the footprint of the
direction's derivatives; the oracle against an independent numpy statement
of the same mapping and mipmapped bilinear filter."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid, single_layer_group
from openshadinglanguage_gb300.shaders import environment_lookup
from test_texture import make_image, np_bilinear, np_pyramid, register


def env_group(ss, name, **kw):
    return single_layer_group(ss, name, environment_lookup(name, **kw),
                              outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])


def directions(u, v, W, H):
    """R and R + dR/dx, R + dR/dy in float64 for the shader's mapping."""
    phi, th = 2 * np.pi * u.astype(np.float64), np.pi * v.astype(np.float64)
    R = np.stack([np.cos(phi) * np.sin(th), np.sin(phi) * np.sin(th), np.cos(th)])
    dphi, dth = 2 * np.pi / W, np.pi / H
    Rx = R + np.stack([-np.sin(phi) * np.sin(th), np.cos(phi) * np.sin(th), np.zeros_like(phi)]) * dphi
    Ry = R + np.stack([np.cos(phi) * np.cos(th), np.sin(phi) * np.cos(th), -np.sin(th)]) * dth
    return R, Rx, Ry


def np_st(R):
    s = np.arctan2(R[1], R[0]) / (2 * np.pi) + 0.5
    t = 0.5 - np.arctan2(R[2], np.hypot(R[0], R[1])) / np.pi
    return s, t


def np_environment(img, u, v, W, H, width=1.0):
    pyr = np_pyramid(img)
    R, Rx, Ry = directions(u, v, W, H)
    s, t = np_st(R)
    sx, tx = np_st(Rx)
    sy, ty = np_st(Ry)
    wrap = lambda d: np.where(d > 0.5, d - 1, np.where(d < -0.5, d + 1, d))
    h0, w0 = img.shape[:2]
    dsx, dtx, dsy, dty = wrap(sx - s) * w0, (tx - t) * h0, wrap(sy - s) * w0, (ty - t) * h0
    length = np.maximum(np.hypot(dsx, dtx), np.hypot(dsy, dty)) * width
    lod = np.minimum(np.where(length > 1, np.log2(np.maximum(length, 1)), 0.0), len(pyr) - 1)
    out = np.zeros((len(u), img.shape[2]))
    for i in range(len(u)):
        l0 = int(lod[i])
        f = lod[i] - l0
        a = np_bilinear_mixed(pyr[l0], s[i:i + 1], t[i:i + 1])
        if f > 0 and l0 + 1 < len(pyr):
            a = (1 - f) * a + f * np_bilinear_mixed(pyr[l0 + 1], s[i:i + 1], t[i:i + 1])
        out[i] = a[0]
    return out, lod


def np_bilinear_mixed(lev, s, t):
    """bilinear with s periodic and t clamped"""
    H, W = lev.shape[:2]
    x, y = s * W - 0.5, t * H - 0.5
    x0, y0 = np.floor(x), np.floor(y)
    fx, fy = (x - x0)[:, None], (y - y0)[:, None]
    ix, iy = x0.astype(int), y0.astype(int)
    cx0, cx1 = np.mod(ix, W), np.mod(ix + 1, W)
    cy0, cy1 = np.clip(iy, 0, H - 1), np.clip(iy + 1, 0, H - 1)
    top = (1 - fx) * lev[cy0, cx0] + fx * lev[cy0, cx1]
    bot = (1 - fx) * lev[cy1, cx0] + fx * lev[cy1, cx1]
    return (1 - fy) * top + fy * bot


@pytest.mark.parametrize("grid,img_size,width", [((96, 48), (32, 64), 1.0), ((24, 12), (128, 256), 1.0),
                                                 ((40, 20), (64, 128), 3.0)])
def test_oracle_matches_numpy_latlong(grid, img_size, width):
    W, H = grid
    img = make_image(img_size[0], img_size[1], 3, seed=9)
    ss = og.ShadingSystem()
    register(ss, img, "env")
    g = env_group(ss, "env_%d_%d_%g" % (W, img_size[1], width), width=width)
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out) == 0
    ref, lod = np_environment(img, u, v, W, H, width)
    err = np.abs(out - ref).max(1)
    # float32 rounding of s, t and the footprint moves a sample by a tiny
    # fraction of a texel; a level-of-detail switch near an integer LOD can
    # move it more
    near_switch = np.abs(lod - np.round(lod)) < 1e-3
    assert np.all(err[~near_switch] < 2e-3), err.max()
    if width > 1:
        assert lod.max() > 1


def test_seam_keeps_a_small_footprint():
    """Points on both sides of s = 0/1 filter like their neighbours (the s
    differences wrap), so the seam column is no blurrier than the rest."""
    W, H = 64, 32
    img = make_image(64, 128, 3, seed=4)
    ss = og.ShadingSystem()
    register(ss, img, "env")
    g = env_group(ss, "env_seam")
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out) == 0
    ref, lod = np_environment(img, u, v, W, H)
    seam = np.abs(u - 0.5) < 1.0 / W  # phi near pi: s near 0 / 1
    assert seam.any() and lod[seam].max() <= lod.max()
    assert np.abs(out[seam] - ref[seam]).max() < 2e-3


def test_environment_errors():
    ss = og.ShadingSystem()
    with pytest.raises(og.OSLError, match="not registered"):
        env_group(ss, "env_missing").program_bytes()
