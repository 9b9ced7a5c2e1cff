"""GPU parity: the sm_103a interpreter against the CPU oracle on the same
lowered programs and inputs, through the C ABI. Float outputs must be
value-identical (both follow the reference's non-FMA operation order),
integer outputs bit-exact; testsuite images also meet the reference's
runtest thresholds."""
import numpy as np
import pytest

from helpers import (float_equal, golden_image, grid_globals, image_diff_ok, og, oracle_run, pixel_grid,
                     shaders, single_layer_group, to_uint8)
from test_oracle_golden import (TESTSUITE, deformer_expected, deformer_group, deformer_inputs, fmt_g3, suite_P,
                                suite_program)

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def device_grid_globals(u, v, W, H, centers=False, P=None):
    du = dev(u)
    dv = dev(v)
    dP = dev(P) if P is not None else None
    G = grid_globals(du, dv, W, H, P=dP, centers=centers)
    G._keep += [du, dv] + ([dP] if dP is not None else [])
    return G


def gpu_run(ss, g, n, G, rec_floats, userdata=None, sync=True):
    out = torch.zeros(n * rec_floats, dtype=torch.float32, device="cuda")
    ud = dev(userdata) if userdata is not None else None
    ss.execute_batch(g, n, G, ud.data_ptr() if ud is not None else 0, out.data_ptr(),
                     torch.cuda.current_stream().cuda_stream, sync=sync)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(n, rec_floats)


def fbm_group(ss, derivs=True):
    rec = 10 if derivs else 4
    g = single_layer_group(ss, "fbm_cell", shaders.fbm_cell(), outputs=[
        og.SymLocationDesc("layer1.Cout", og.TypeColor, derivs, og.SymArenaOutputs, 0, 4 * rec),
        og.SymLocationDesc("layer1.cellhash", og.TypeInt, False, og.SymArenaOutputs, 4 * (rec - 1), 4 * rec)])
    return g, rec


def assert_same(gpu, ref, int_cols=()):
    cols = [c for c in range(gpu.shape[1]) if c not in int_cols]
    eq = float_equal(gpu[:, cols], ref[:, cols])
    bad = np.argwhere(~eq)
    assert bad.size == 0, "first mismatches (point, col, gpu, oracle): %s" % [
        (int(p), int(cols[c]), float(gpu[p, cols[c]]), float(ref[p, cols[c]])) for p, c in bad[:8]]
    for c in int_cols:
        gi, ri = gpu[:, c].view(np.int32), ref[:, c].view(np.int32)
        assert np.array_equal(gi, ri), (c, np.argwhere(gi != ri)[:8].ravel())


@pytest.mark.parametrize("heap", [1, 0])
@pytest.mark.parametrize("derivs", [True, False])
def test_fbm_cell_matches_oracle(heap, derivs):
    ss = og.ShadingSystem()
    ss.set_launch(block=256, heap_smem=heap)
    g, rec = fbm_group(ss, derivs)
    W = H = 128
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), rec)
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref, int_cols=(rec - 1,))


def test_fbm_cell_full_size_matches_oracle():
    # the benchmark workload itself: 1024x1024 points, Dual2 Cout + hashed cell id
    ss = og.ShadingSystem()
    g, rec = fbm_group(ss, True)
    W = H = 1024
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), rec)
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref, int_cols=(rec - 1,))


@pytest.mark.parametrize("name,kw", TESTSUITE)
def test_testsuite_shaders_match_oracle_and_golden(name, kw):
    ss, g = suite_program(name, kw)
    ref_img, W, H, step = golden_image(name)
    u, v = pixel_grid(W, H)
    P = suite_P(kw, u, v)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, P=P), 3)
    ref = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P), ref) == 0
    assert_same(got, ref)
    ok, frac, mx = image_diff_ok(to_uint8(got.reshape(H, W, 3))[::step, ::step], ref_img,
                                 failpercent=kw.get("failpercent", 0.02))
    assert ok, (frac, mx)


@pytest.mark.parametrize("heap", [1, 0])
def test_control_flow_matches_oracle(heap):
    ss = og.ShadingSystem()
    ss.set_launch(block=128, heap_smem=heap)
    g = single_layer_group(ss, "ctrlflow", shaders.ctrlflow(), outputs=[
        og.SymLocationDesc("r", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
        og.SymLocationDesc("count", og.TypeInt, False, og.SymArenaOutputs, 4, 8)])
    W, H = 256, 200  # not a multiple of the block: exercises the tail
    u, v = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H), 2)
    ref = np.zeros((W * H, 2), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert_same(got, ref, int_cols=(1,))


def test_batched_deformer_on_gpu():
    ss = og.ShadingSystem()
    g = deformer_group(ss)
    n, P, amp = deformer_inputs()
    G = og.make_globals(P=dev(P))
    dP = dev(P)
    G = og.make_globals(P=dP)
    got = gpu_run(ss, g, n, G, 3, userdata=amp)
    assert [" ".join(fmt_g3(c) for c in row) for row in got] == deformer_expected()


def test_empty_and_single_point_batches():
    ss = og.ShadingSystem()
    g, rec = fbm_group(ss, True)
    u, v = pixel_grid(1, 1, centers=True)
    G = device_grid_globals(u, v, 1, 1, centers=True)
    out = torch.zeros(rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, 0, G, 0, out.data_ptr(), sync=True)  # nothing to shade
    assert torch.count_nonzero(out).item() == 0
    got = gpu_run(ss, g, 1, G, rec)
    ref = np.zeros((1, rec), np.float32)
    oracle_run(g.program_bytes(), 1, grid_globals(u, v, 1, 1, centers=True), ref)
    assert_same(got, ref, int_cols=(rec - 1,))


@pytest.mark.parametrize("heap", [1, 0])
def test_layered_closure_group_matches_oracle(heap):
    from openshadinglanguage_gb300 import workloads
    ss = og.ShadingSystem()
    ss.set_launch(block=256, heap_smem=heap)
    g = workloads.c2_group(ss)
    W = H = 256
    u, v, I = workloads.c2_inputs(W, H)
    du, dv, dI = dev(u), dev(v), dev(I)
    Gd = workloads.c2_globals(og.make_globals, du, dv, dI)
    rec = workloads.C2_STRIDE // 4
    got = gpu_run(ss, g, W * H, Gd, rec)
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, workloads.c2_globals(og.make_globals, u, v, I), ref) == 0
    int_cols = [0] + [1 + 16 * k for k in range(workloads.C2_CLOSURE_RECORDS)] + [5 + 16]  # counts, ids, dist hash
    assert_same(got, ref, int_cols=tuple(int_cols))


@pytest.mark.parametrize("opts", [dict(anisotropic=0, bandwidth=1.0), dict(anisotropic=1, direction=(2.0, 0.5, 0.0)),
                                  dict(anisotropic=2, direction=(1.5, 1.0, 0.25), impulses=8.0),
                                  dict(do_filter=0, bandwidth=4.0)])
def test_gabor_options_match_oracle(opts):
    ss = og.ShadingSystem()
    g = single_layer_group(ss, "tgo", shaders.gabor_options(**opts),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    W = H = 128
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), 3)
    ref = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref)


def test_matrix_ops_match_oracle():
    from test_matrix_ops import REC, inputs, matrix_group
    ss = og.ShadingSystem()
    g, _, _ = matrix_group(ss)
    W = H = 64
    u, v, P = inputs(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True, P=P), REC)
    ref = np.zeros((W * H, REC), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P, centers=True), ref) == 0
    assert_same(got, ref)


@pytest.mark.parametrize("scale", [10000.0, 30000.0])
def test_blackbody_matches_oracle(scale):
    from test_oracle_golden import blackbody_program
    ss = og.ShadingSystem()
    g = blackbody_program(ss, scale)
    W, H = 1000, 64
    u, v = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H), 3)
    ref = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert_same(got, ref)


def test_single_op_programs_pick_the_right_tier():
    """A program whose only non-trivial op is one math-tier op runs (the
    tier chosen at lowering carries the op's handler)."""
    ss = og.ShadingSystem()
    b = og.OsoBuilder("tdet")
    M = b.param("matrix", "M", [float(i % 5 == 0) * 2.0 + 0.25 * (i % 3) for i in range(16)])
    out = b.param("float", "d", 0.0, output=True)
    b.op("determinant", out, M)
    g = single_layer_group(ss, "tdet", b.text(), outputs=[
        og.SymLocationDesc("d", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    W, H = 64, 4
    u_, v_ = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u_, v_, W, H), 1)
    ref = np.zeros((W * H, 1), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u_, v_, W, H), ref) == 0
    assert_same(got, ref)
    assert ss.device_status() == 0


def test_c5_material_sampling_matches_oracle():
    from openshadinglanguage_gb300 import workloads as W
    n = 8192
    P, N, I, T, rnd = W.c5_hits(n)
    ss = og.ShadingSystem()
    dP, dN, dI, dT, drnd = (dev(x) for x in (P, N, I, T, rnd))
    Gd = og.make_globals(P=dP, N=dN, Ng=dN, I=dI, dPdu=dT)
    Gh = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    for k, spec in enumerate(W.c5_material_specs()):
        g = W.c5_material_group(ss, k, spec)
        got = gpu_run(ss, g, n, Gd, W.C5_OUT_FLOATS, userdata=rnd)
        ref = np.zeros((n, W.C5_OUT_FLOATS), np.float32)
        assert oracle_run(g.program_bytes(), n, Gh, ref, userdata=rnd) == 0
        assert_same(got, ref)
    assert ss.device_status() == 0
