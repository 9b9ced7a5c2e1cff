"""The allocation-free entry point (oslg_execute_batch_noalloc) against the
regular one, through the C ABI.

Some callers cannot allocate device memory: a renderer that hands out all
HBM from its own pool under a fixed budget, or code that must not take the
implicit device synchronisation of cudaMalloc/cudaFree. For them the
library runs the HBM-heap interpreter with all of its scratch inside one
static device array. This test runs the same lowered group both ways and
requires identical results, on two calls in a row (the second call finds
the previous call's contents in the shared array). This file sorts last so
a run that stops at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from helpers import float_equal, grid_globals, og, pixel_grid, shaders, single_layer_group
from openshadinglanguage_gb300 import _capi

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_noalloc_entry_matches_regular_entry_twice():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    ss.set_launch(block=256, heap_smem=0)
    rec = 10
    g = single_layer_group(ss, "fbm_cell", shaders.fbm_cell(), outputs=[
        og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 4 * rec),
        og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 4 * rec)])
    ss.optimize_group(g)
    W, H = 512, 300
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    G = grid_globals(du, dv, W, H, centers=True)
    stream = torch.cuda.current_stream().cuda_stream

    ref = torch.zeros(n * rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, G, 0, ref.data_ptr(), stream, sync=True)
    ref = ref.cpu().numpy().reshape(n, rec)

    L = _capi.lib()
    for call in range(2):
        out = torch.full((n * rec,), -7.0, dtype=torch.float32, device="cuda")
        bits = ctypes.c_uint32(123)
        rc = L.oslg_execute_batch_noalloc(ss._h, g.handle, n, ctypes.byref(G), None,
                                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream),
                                          ctypes.byref(bits))
        assert rc == 0, L.oslg_last_error(ss._h)
        assert bits.value == 0
        got = out.cpu().numpy().reshape(n, rec)
        # same tolerance as every other GPU test: value-identical floats,
        # bit-identical ints
        assert float_equal(got[:, :9], ref[:, :9]).all(), "call %d differs from the regular entry" % call
        assert np.array_equal(got[:, 9].view(np.int32), ref[:, 9].view(np.int32)), call


def _noalloc(ss, g, n, G, out, status=True):
    L = _capi.lib()
    bits = ctypes.c_uint32(0)
    rc = L.oslg_execute_batch_noalloc(ss._h, g.handle, n, ctypes.byref(G), None, ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                      ctypes.byref(bits) if status else None)
    return rc, bits.value, L.oslg_last_error(ss._h)


def test_noalloc_texture_lookups_use_the_uploaded_table():
    """texture() reads the system's texture table; the allocation-free entry
    cannot upload it, so it refuses the group until an allocating call has,
    then matches the regular entry."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_texture import make_image, register, tex_shader
    ss = og.ShadingSystem()
    ss.set_launch(block=256, heap_smem=0)
    register(ss, make_image(37, 53, 3))
    g = single_layer_group(ss, "na_tex", tex_shader("na_tex", 3.3, "periodic"),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    ss.optimize_group(g)
    W, H = 61, 45
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    G = grid_globals(du, dv, W, H, centers=True)
    out = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    rc, _, msg = _noalloc(ss, g, n, G, out)
    assert rc == 5, "expected OSLG_ERR_STATE before the texture table is uploaded"
    assert b"texture" in msg
    ref = torch.zeros(n * 3, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, G, 0, ref.data_ptr(), sync=True)
    for call in range(2):
        out.fill_(-7.0)
        rc, bits, msg = _noalloc(ss, g, n, G, out)
        assert rc == 0 and bits == 0, msg
        assert float_equal(out.cpu().numpy(), ref.cpu().numpy()).all(), call


def test_noalloc_status_without_status_out_reaches_device_status():
    """With status_out NULL the call only enqueues; a kernel status bit it
    raised is still reported (and cleared) by oslg_device_status."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_loop_limit import W as LW, H as LH, group
    ss, g = group(5)  # points take up to 200 loop back edges: past the limit of 5
    ss.optimize_group(g)
    u, v = pixel_grid(LW, LH)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    G = grid_globals(du, dv, LW, LH)
    out = torch.zeros(LW * LH, dtype=torch.int32, device="cuda")
    rc, _, msg = _noalloc(ss, g, LW * LH, G, out, status=False)
    assert rc == 0, msg
    torch.cuda.synchronize()
    assert ss.device_status() & 8  # the loop-limit bit
    assert ss.device_status() == 0  # read and cleared
