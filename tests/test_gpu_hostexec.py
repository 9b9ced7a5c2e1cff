"""Execution over host buffers (oslg_execute_batch_host): chunked,
pipelined copies and launches give the same records as the device entry,
with and without specialized kernels, preserving untouched output bytes on
request, with userdata records, and rejecting mismatched record strides."""
import numpy as np
import pytest

from helpers import og

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import dev, gpu_run  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def c2_case(jit, W=700, H=500):
    from openshadinglanguage_gb300 import workloads
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = workloads.c2_group(ss)
    u, v, I = workloads.c2_inputs(W, H)
    return ss, g, workloads, u, v, I


@pytest.mark.parametrize("jit", [0, 1])
def test_layered_closure_host_equals_device(jit):
    ss, g, wl, u, v, I = c2_case(jit)
    n = u.size
    rec = wl.C2_STRIDE // 4
    ref = gpu_run(ss, g, n, wl.c2_globals(og.make_globals, dev(u), dev(v), dev(I)), rec)
    hu, hv, hI = (torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (u, v, I))
    G = wl.c2_globals(og.make_globals, hu, hv, hI)
    out = torch.full((n * rec,), 7.0, dtype=torch.float32).pin_memory()
    ss.execute_batch_host(g, n, G, out, wl.C2_STRIDE)
    got = out.numpy().reshape(n, rec)
    # device entry wrote into a zeroed buffer; the host entry zeroes untouched bytes
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_preserve_outputs_keeps_untouched_bytes():
    # fBm records padded to 48 bytes: bytes 40..47 of each record are never written
    from helpers import grid_globals, pixel_grid, shaders, single_layer_group
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    g = single_layer_group(ss, "fbm_cell", shaders.fbm_cell(), outputs=[
        og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 48),
        og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 48)])
    W, H = 500, 300
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    dout = torch.full((n * 12,), -3.5, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, grid_globals(dev(u), dev(v), W, H, centers=True), 0, dout.data_ptr(),
                     torch.cuda.current_stream().cuda_stream, sync=True)
    ref = dout.cpu().numpy().reshape(n, 12)
    out = np.full((n, 12), -3.5, np.float32)  # pageable host memory works too
    ss.execute_batch_host(g, n, grid_globals(u, v, W, H, centers=True), out, 48, preserve_outputs=True)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    assert (out[:, 10:] == -3.5).all()
    zeroed = np.full((n, 12), -3.5, np.float32)
    ss.execute_batch_host(g, n, grid_globals(u, v, W, H, centers=True), zeroed, 48)
    assert (zeroed[:, 10:] == 0.0).all() and np.array_equal(zeroed[:, :10].view(np.uint32), ref[:, :10].view(np.uint32))


def test_userdata_records_and_sampling():
    from openshadinglanguage_gb300 import workloads as W
    n = 200003
    P, N, I, T, rnd = W.c5_hits(n)
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    g = W.c5_material_group(ss, 12, W.c5_material_specs()[12])
    ref = gpu_run(ss, g, n, og.make_globals(P=dev(P), N=dev(N), Ng=dev(N), I=dev(I), dPdu=dev(T)),
                  W.C5_OUT_FLOATS, userdata=rnd)
    out = np.zeros((n, W.C5_OUT_FLOATS), np.float32)
    G = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    ss.execute_batch_host(g, n, G, out, 4 * W.C5_OUT_FLOATS, userdata=np.ascontiguousarray(rnd),
                          userdata_stride=4 * W.C5_IN_FLOATS)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_mismatched_strides_are_rejected():
    ss, g, wl, u, v, I = c2_case(0, W=64, H=64)
    n = u.size
    G = wl.c2_globals(og.make_globals, *(torch.from_numpy(np.ascontiguousarray(x)) for x in (u, v, I)))
    out = np.zeros(n * 64, np.float32)
    with pytest.raises(og.OSLError, match="output_stride"):
        ss.execute_batch_host(g, n, G, out, wl.C2_STRIDE + 4)


@pytest.mark.parametrize("direct", [1, 0])
def test_pinned_outputs_direct_and_copied(direct):
    """Pinned output records: the specialized kernel writes them straight
    into host memory (attribute host_direct_outputs, the default) or through
    device buffers and copies; both equal the device entry, zeroing or
    preserving the bytes no output op writes."""
    from helpers import grid_globals, pixel_grid, shaders, single_layer_group
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    ss.attribute("host_direct_outputs", direct)
    g = single_layer_group(ss, "fbm_cell", shaders.fbm_cell(), outputs=[
        og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 48),
        og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 48)])
    W, H = 640, 331
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    dout = torch.full((n * 12,), -3.5, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, grid_globals(dev(u), dev(v), W, H, centers=True), 0, dout.data_ptr(),
                     torch.cuda.current_stream().cuda_stream, sync=True)
    ref = dout.cpu().numpy().reshape(n, 12)
    hu, hv = torch.from_numpy(u).pin_memory(), torch.from_numpy(v).pin_memory()
    kept = torch.full((n * 12,), -3.5, dtype=torch.float32).pin_memory()
    ss.execute_batch_host(g, n, grid_globals(hu, hv, W, H, centers=True), kept, 48, preserve_outputs=True)
    assert np.array_equal(kept.numpy().reshape(n, 12).view(np.uint32), ref.view(np.uint32))
    zeroed = torch.full((n * 12,), -3.5, dtype=torch.float32).pin_memory()
    ss.execute_batch_host(g, n, grid_globals(hu, hv, W, H, centers=True), zeroed, 48)
    z = zeroed.numpy().reshape(n, 12)
    assert (z[:, 10:] == 0.0).all() and np.array_equal(z[:, :10].view(np.uint32), ref[:, :10].view(np.uint32))
