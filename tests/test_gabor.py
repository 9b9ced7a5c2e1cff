"""Gabor noise and the executor's own single-precision exp/sincos, on the
CPU oracle: accuracy of the exp/sincos pair against double precision, and
Gabor evaluated with that pair against Gabor evaluated with libm (the
reference's math) over the option space. The reference images of
testsuite/noise-gabor*, pnoise-gabor are checked in test_oracle_golden."""
import ctypes

import numpy as np
import pytest

from helpers import grid_globals, og, oracle, oracle_run, pixel_grid, shaders, single_layer_group

FP = ctypes.POINTER(ctypes.c_float)


def fp(a):
    return a.ctypes.data_as(FP)


def test_own_exp_within_two_ulp():
    x = np.concatenate([np.linspace(-87.0, 88.7, 400001, dtype=np.float32),
                        np.float32([0.0, -0.0, 1e-30, -1e-30, 88.72, -87.3, 1.0, -1.0])])
    y = np.zeros_like(x)
    oracle().oracle_own_exp(fp(x), len(x), fp(y))
    ref = np.exp(x.astype(np.float64))
    ulp = np.abs(y - ref) / np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert ulp.max() <= 2.0, ulp.max()


def test_own_exp_edges():
    x = np.float32([-200.0, -104.0, -103.0, -100.0, 89.0, np.inf, -np.inf, np.nan])
    y = np.zeros_like(x)
    oracle().oracle_own_exp(fp(x), len(x), fp(y))
    assert y[0] == 0.0 and y[1] == 0.0
    ref = np.exp(x[2:4].astype(np.float64))  # subnormal results: within one subnormal step
    assert np.all(np.abs(y[2:4] - ref) <= 2.0 ** -149)
    assert np.isinf(y[4]) and np.isinf(y[5]) and y[6] == 0.0 and np.isnan(y[7])


def test_own_sincos_within_2_pow_minus_23():
    x = np.concatenate([np.linspace(-6000.0, 6000.0, 400001, dtype=np.float32),
                        np.linspace(-7.0, 7.0, 20001, dtype=np.float32), np.float32([1e5, -3e7])])
    s, c = np.zeros_like(x), np.zeros_like(x)
    oracle().oracle_own_sincos(fp(x), len(x), fp(s), fp(c))
    xd = x.astype(np.float64)
    assert np.abs(s - np.sin(xd)).max() <= 2.0 ** -23
    assert np.abs(c - np.cos(xd)).max() <= 2.0 ** -23


def gabor(P, dPdx, dPdy, nc=1, libm=False, anisotropic=0, do_filter=1, direction=(1, 0, 0), bandwidth=1.0,
          impulses=16.0, period=None):
    inp = np.float32(list(P) + list(dPdx) + list(dPdy))
    d = np.float32(direction)
    per = np.float32(period if period is not None else (0, 0, 0))
    out = np.zeros(9, np.float32)
    oracle().oracle_gabor(anisotropic, do_filter, fp(d), ctypes.c_float(bandwidth), ctypes.c_float(impulses),
                          fp(inp), int(period is not None), fp(per), nc, int(libm), fp(out))
    return out[:3 * nc].reshape(nc, 3)


OPTION_SETS = [
    dict(),
    dict(anisotropic=1, direction=(2.0, 0.5, 0.0)),
    dict(anisotropic=2, direction=(1.5, 1.0, 0.25)),
    dict(do_filter=0),
    dict(bandwidth=4.0, impulses=8.0),
    dict(bandwidth=2.0, impulses=32.0, anisotropic=1, direction=(0.0, 3.0, 0.0)),
    dict(period=(3.0, 3.0, 3.0)),
    dict(impulses=1.0, bandwidth=0.5),
]


@pytest.mark.parametrize("opts", OPTION_SETS)
@pytest.mark.parametrize("nc", [1, 3])
def test_gabor_own_math_matches_libm(opts, nc):
    """Float tolerance for Gabor against the reference's libm exp/sincos:
    1e-4 absolute on values and derivatives scaled to the result's range."""
    rng = np.random.default_rng(7)
    worst = 0.0
    for _ in range(60):
        P = rng.uniform(-10, 10, 3)
        dx = rng.uniform(-0.05, 0.05, 3)
        dy = rng.uniform(-0.05, 0.05, 3)
        a = gabor(P, dx, dy, nc=nc, **opts)
        b = gabor(P, dx, dy, nc=nc, libm=True, **opts)
        assert np.all(np.isfinite(a))
        scale = np.maximum(1.0, np.abs(b))
        worst = max(worst, float(np.max(np.abs(a - b) / scale)))
    assert worst <= 1e-4, worst


def test_gabor_derivatives_match_finite_differences():
    rng = np.random.default_rng(11)
    for _ in range(10):
        P = rng.uniform(-5, 5, 3)
        dx = np.float32([1e-3, 0, 0])
        dy = np.float32([0, 1e-3, 0])
        base = gabor(P, dx, dy, do_filter=0)[0]
        h = 1e-3
        px = gabor(P + np.array([h, 0, 0]), dx, dy, do_filter=0)[0][0]
        mx = gabor(P - np.array([h, 0, 0]), dx, dy, do_filter=0)[0][0]
        fd = (px - mx) / (2 * h) * 1e-3
        assert abs(base[1] - fd) <= 2e-3 * max(1.0, abs(base[0])), (base, fd)


def test_gabor_options_shader_on_oracle():
    """test_gabor_options with per-option values runs to completion and stays
    in the noise's range."""
    ss = og.ShadingSystem()
    g = single_layer_group(ss, "tgo", shaders.gabor_options(anisotropic=2, direction=(2.0, 1.0, 0.0), bandwidth=2.0),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    W = H = 64
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out) == 0
    assert np.all(np.isfinite(out)) and out.min() > -1.0 and out.max() < 2.0
    assert np.count_nonzero(out) > W * H
