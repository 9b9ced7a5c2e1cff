"""Wavefront path tracer, host side: the oracle's path loop (background
only, determinism, path independence that the full-frame GPU check relies
on) and the C ABI's argument checks, none of which touch a GPU."""
import ctypes

import numpy as np
import pytest

from helpers import _capi, float_equal, og, oracle_wavefront
from openshadinglanguage_gb300 import workloads as W
from openshadinglanguage_gb300.shadingsys import OSLError, Wavefront, options_c, prims_c

SMALL = dict(width=40, height=24, spp=2)


@pytest.fixture(scope="module")
def scene():
    ss = og.ShadingSystem()
    return ss, W.c5_materials(ss), W.c5_scene()


def test_scene_is_seeded_and_valid():
    a, b = W.c5_scene(), W.c5_scene()
    assert a.tobytes() == b.tobytes()
    assert len(a) == 1000
    quads = a[a["kind"] == 1]
    ex, ey = quads["ex"].astype(np.float64), quads["ey"].astype(np.float64)
    cosang = np.abs((ex * ey).sum(1)) / np.sqrt((ex * ex).sum(1) * (ey * ey).sum(1))
    assert cosang.max() < 1e-6
    spheres = a[a["kind"] == 0]
    assert (spheres["radius"] > 0).all()
    assert set(np.unique(a["material"])) <= set(range(W.C5_MATERIALS))


def test_empty_scene_returns_background(scene):
    ss, mats, _ = scene
    bg = (0.25, 0.5, 0.75)
    rad, hits, st = oracle_wavefront(dict(SMALL, background=bg), [], mats)
    assert st == 0 and hits.sum() == 0
    for c in range(3):
        assert (rad[c] == np.float32(bg[c])).all()


def test_oracle_small_frame(scene):
    ss, mats, prims = scene
    rad, hits, st = oracle_wavefront(SMALL, prims, mats)
    n = SMALL["width"] * SMALL["height"] * SMALL["spp"]
    assert st == 0
    assert np.isfinite(rad).all() and (rad >= 0).all()
    assert 0 < hits[0] <= n
    # Russian roulette with survival 0.8 after every hit: each bounce holds
    # at most the survivors of the one before
    assert all(hits[b + 1] <= hits[b] for b in range(7)) and hits[8:].sum() == 0
    assert hits.sum() <= n * (1 - 0.8 ** 8) / 0.2
    # thread count does not change a bit
    rad1, hits1, _ = oracle_wavefront(SMALL, prims, mats, nthreads=1)
    assert float_equal(rad, rad1).all() and (hits == hits1).all()


def test_paths_are_independent(scene):
    """A strided sample of paths renders to the same bits as the same paths
    inside the whole frame (the full-size GPU check compares samples)."""
    ss, mats, prims = scene
    full, _, _ = oracle_wavefront(SMALL, prims, mats)
    sample, _, _ = oracle_wavefront(SMALL, prims, mats, begin=5, step=7)
    assert float_equal(sample, full[:, 5::7]).all()


def test_max_hits_one_is_emission_and_background(scene):
    ss, mats, prims = scene
    rad, hits, _ = oracle_wavefront(dict(SMALL, max_hits=1), prims, mats)
    assert hits[1:].sum() == 0 and hits[0] > 0


def _create(ss, mats, prims, **over):
    o = dict(Wavefront.OPTION_DEFAULTS)
    o.update(SMALL)
    o.update(over)
    oc = options_c(o)
    arr = prims_c(prims)
    ptrs = (ctypes.c_void_p * len(mats))(*[m.handle.value for m in mats])
    h = ctypes.c_void_p()
    rc = _capi.lib().oslg_wavefront_create(ss._h, ctypes.byref(oc), arr, len(prims), ptrs, len(mats),
                                           ctypes.byref(h))
    return rc, _capi.lib().oslg_last_error(ss._h).decode()


@pytest.mark.parametrize("over,msg", [(dict(width=0), "positive"), (dict(max_hits=17), "max_hits"),
                                      (dict(rr_survival=0.0), "rr_survival"), (dict(fov_deg=180.0), "fov"),
                                      (dict(block=1024), "block")])
def test_create_rejects_bad_options(scene, over, msg):
    ss, mats, prims = scene
    rc, err = _create(ss, mats, prims[:10], **over)
    assert rc == 1 and msg in err  # OSLG_ERR_ARG


def test_create_rejects_bad_primitives(scene):
    ss, mats, prims = scene
    bad = prims[:4].copy()
    bad[0]["ey"] = (1.0, 0.0, 1.0)  # not orthogonal to ex = (0, 0, 200)
    rc, err = _create(ss, mats, bad)
    assert rc == 1 and "orthogonal" in err
    bad = prims[:4].copy()
    bad[3]["material"] = 99
    rc, err = _create(ss, mats, bad)
    assert rc == 1 and "material" in err
    bad = prims[2:6].copy()
    bad[-1]["kind"], bad[-1]["radius"] = 0, -1.0
    rc, err = _create(ss, mats, bad)
    assert rc == 1 and "radius" in err


def test_create_requires_sampled_materials(scene):
    ss, mats, prims = scene
    oso = W._c5_surface("plain_surface", [("diffuse", 1.0, 0.0)])
    ss.LoadMemoryCompiledShader("plain_surface", oso)
    g = ss.ShaderGroupBegin("plain_surface_g")
    ss.Shader(g, "surface", "plain_surface", "S")
    ss.ShaderGroupEnd(g)
    one = prims[:2].copy()
    one["material"] = 0
    rc, err = _create(ss, [g], one)
    assert rc == 1 and "bsdf_sample" in err
    with pytest.raises(OSLError):
        Wavefront(ss, one, [g], **SMALL)
