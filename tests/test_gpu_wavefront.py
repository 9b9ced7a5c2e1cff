"""Wavefront path tracer on the GPU against the oracle's path loop: every
path of a small frame bit for bit, a strided sample of the full
1920x1080x4 frame bit for bit, graph replay and the stage-by-stage launch
equal, and the resolved image equal to the mean of each pixel's paths."""
import numpy as np
import pytest

from helpers import float_equal, og, oracle_wavefront

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from openshadinglanguage_gb300 import workloads as W  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


@pytest.fixture(scope="module")
def scene():
    ss = og.ShadingSystem()
    return ss, W.c5_materials(ss), W.c5_scene()


def render(wf, profile=False, image=False):
    rad = torch.zeros(3 * wf.paths, dtype=torch.float32, device="cuda")
    o = wf.options
    img = torch.zeros(o["width"] * o["height"] * 3, dtype=torch.float32, device="cuda") if image else None
    wf.render(rad.data_ptr(), img.data_ptr() if image else 0, torch.cuda.current_stream().cuda_stream,
              profile=profile)
    torch.cuda.synchronize()
    out = rad.cpu().numpy().reshape(3, wf.paths)
    return (out, img.cpu().numpy()) if image else out


def assert_paths_equal(gpu, ref, where=None):
    eq = float_equal(gpu, ref).all(0)
    bad = np.nonzero(~eq)[0]
    idx = where if where is not None else np.arange(gpu.shape[1])
    assert bad.size == 0, "%d paths differ; first (path, gpu, oracle): %s" % (
        bad.size, [(int(idx[b]), gpu[:, b].tolist(), ref[:, b].tolist()) for b in bad[:4]])


@pytest.mark.parametrize("opts", [dict(width=64, height=36, spp=2),
                                  dict(width=33, height=17, spp=3, max_hits=5, rr_survival=0.6,
                                       block=128, points_per_thread=2),
                                  dict(width=48, height=20, spp=1, heap_smem=2, block=512)])
def test_small_frame_matches_oracle(scene, opts):
    ss, mats, prims = scene
    wf = ss.wavefront(prims, mats, **opts)
    gpu = render(wf)
    ref, hits, st = oracle_wavefront(opts, prims, mats)
    assert st == 0
    assert_paths_equal(gpu, ref)
    s = wf.stats()
    assert s["hits"] == hits.tolist()
    assert s["paths"] == wf.paths
    assert ss.device_status() == 0


def test_full_frame_sampled_matches_oracle(scene):
    """1920x1080x4 paths on the GPU; every 2741st path re-rendered by the
    oracle (paths are independent, so a sample is exact)."""
    ss, mats, prims = scene
    wf = ss.wavefront(prims, mats)  # defaults: 1920x1080, 4 spp, 8 hits, survival 0.8
    gpu, img = render(wf, image=True)
    s = wf.stats()
    assert s["paths"] == 1920 * 1080 * 4
    assert 0 < s["hits"][0] <= s["paths"] and sum(s["hits"][8:]) == 0
    assert s["total_hits"] <= s["paths"] * (1 - 0.8 ** 8) / 0.2
    step = 2741
    ref, _, st = oracle_wavefront(wf.options, prims, mats, begin=17, step=step)
    assert st == 0
    idx = np.arange(17, wf.paths, step)
    assert_paths_equal(gpu[:, idx], ref, idx)
    # image = mean of each pixel's samples, summed in sample order
    per = gpu.reshape(3, -1, 4)
    mean = np.zeros(per.shape[:2], np.float32)
    for k in range(4):
        mean = (mean + per[:, :, k]).astype(np.float32)
    mean = (mean / np.float32(4)).astype(np.float32)
    assert float_equal(img.reshape(-1, 3).T, mean).all()
    assert ss.device_status() == 0


def test_graph_replay_and_profiled_frames_agree(scene):
    ss, mats, prims = scene
    opts = dict(width=160, height=90, spp=2)
    wf = ss.wavefront(prims, mats, **opts)
    a = render(wf)
    b = render(wf)  # graph replay
    c = render(wf, profile=True)
    assert float_equal(a, b).all() and float_equal(a, c).all()
    s = wf.stats()
    assert all(x >= 0 for x in s["ms_stage"]) and sum(s["ms_stage"]) > 0
    nog = ss.wavefront(prims, mats, use_graph=-1, **opts)
    assert float_equal(render(nog), a).all()


def test_specialized_shading_matches_oracle():
    """Attribute jit: the materials shade in one persistent batch kernel
    specialized to their programs; paths stay bit-exact."""
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    mats = W.c5_materials(ss)
    prims = W.c5_scene()
    opts = dict(width=64, height=36, spp=2)
    wf = ss.wavefront(prims, mats, **opts)
    gpu = render(wf)
    ref, hits, st = oracle_wavefront(opts, prims, mats)
    assert st == 0
    assert_paths_equal(gpu, ref)
    assert wf.stats()["hits"] == hits.tolist()
    assert ss.device_status() == 0
