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
