"""The benchmarked paths checked at the benchmarked sizes, every point.

The layered-closure group (simplex + cell noise -> catmull-rom ramp ->
0.6*diffuse + 0.4*GGX microfacet closure records and a BSDF evaluation) on
a 2048x2048 grid, shaded through the host-buffer entry with the kernel
specialized to the group writing the records straight into pinned host
memory; and the fBm + cell-hash group on a 1024x1024 grid through its
specialized kernel. Every one of the 4,194,304 (1,048,576) records equals
the oracle's: integer words bit-exact, float words value-identical."""
import numpy as np
import pytest

from helpers import float_equal, grid_globals, og, oracle_run, pixel_grid, shaders, single_layer_group

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def compare(got, ref, int_cols):
    cols = [c for c in range(got.shape[1]) if c not in int_cols]
    eq = float_equal(got[:, cols], ref[:, cols])
    bad = np.argwhere(~eq)
    assert bad.size == 0, "first float mismatches (point, col, gpu, oracle): %s" % [
        (int(p), cols[c], float(got[p, cols[c]]), float(ref[p, cols[c]])) for p, c in bad[:8]]
    gi = got[:, list(int_cols)].view(np.uint32)
    ri = ref[:, list(int_cols)].view(np.uint32)
    bad = np.argwhere(gi != ri)
    assert bad.size == 0, "first int mismatches: %s" % [(int(p), int(c)) for p, c in bad[:8]]


def test_layered_closure_2048_specialized_host_direct_matches_oracle():
    from openshadinglanguage_gb300 import workloads as wl
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    ss.attribute("host_direct_outputs", 1)
    g = wl.c2_group(ss)
    W = H = 2048
    n = W * H
    u, v, I = wl.c2_inputs(W, H)
    rec = wl.C2_STRIDE // 4
    hu, hv, hI = (torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in (u, v, I))
    out = torch.full((n * rec,), 7.0, dtype=torch.float32).pin_memory()
    ss.execute_batch_host(g, n, wl.c2_globals(og.make_globals, hu, hv, hI), out, wl.C2_STRIDE)
    assert g.is_specialized()
    assert ss.device_status() == 0
    got = out.numpy().reshape(n, rec)
    ref = np.zeros((n, rec), np.float32)
    assert oracle_run(g.program_bytes(), n, wl.c2_globals(og.make_globals, u, v, I), ref) == 0
    int_cols = [0] + [1 + 16 * k for k in range(wl.C2_CLOSURE_RECORDS)] + [5 + 16]
    compare(got, ref, int_cols)


def test_fbm_cell_1024_specialized_matches_oracle():
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    g = single_layer_group(ss, "fbm_cell", shaders.fbm_cell(), outputs=[
        og.SymLocationDesc("layer1.Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 40),
        og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 40)])
    W = H = 1024
    n = W * H
    u, v = pixel_grid(W, H, centers=True)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.zeros(n * 10, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, grid_globals(du, dv, W, H, centers=True), 0, out.data_ptr(), sync=True)
    assert g.is_specialized()
    got = out.cpu().numpy().reshape(n, 10)
    ref = np.zeros((n, 10), np.float32)
    assert oracle_run(g.program_bytes(), n, grid_globals(u, v, W, H, centers=True), ref) == 0
    compare(got, ref, (9,))
