"""Specialized kernels (attribute "jit" = 1): each group compiled to its own
sm_103a kernel gives the same bits as the interpreter and the oracle, over
noise, derivatives, control flow, closures and BSDF evaluation/sampling,
userdata, matrices and ragged tails."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid, shaders, single_layer_group

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import assert_same, dev, device_grid_globals, fbm_group, gpu_run  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def jit_system():
    ss = og.ShadingSystem()
    ss.attribute("jit", 1)
    return ss


@pytest.mark.parametrize("derivs", [True, False])
def test_fbm_cell(derivs):
    ss = jit_system()
    g, rec = fbm_group(ss, derivs)
    W, H = 160, 97  # ragged tail
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), rec)
    assert g.is_specialized()
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref, int_cols=(rec - 1,))


def test_layered_closure_group():
    from openshadinglanguage_gb300 import workloads
    ss = jit_system()
    g = workloads.c2_group(ss)
    W = H = 256
    u, v, I = workloads.c2_inputs(W, H)
    Gd = workloads.c2_globals(og.make_globals, dev(u), dev(v), dev(I))
    rec = workloads.C2_STRIDE // 4
    got = gpu_run(ss, g, W * H, Gd, rec)
    assert g.is_specialized()
    ref = np.zeros((W * H, rec), np.float32)
    assert oracle_run(g.program_bytes(), W * H, workloads.c2_globals(og.make_globals, u, v, I), ref) == 0
    int_cols = [0] + [1 + 16 * k for k in range(workloads.C2_CLOSURE_RECORDS)] + [5 + 16]
    assert_same(got, ref, int_cols=tuple(int_cols))


def test_control_flow():
    ss = jit_system()
    g = single_layer_group(ss, "ctrlflow", shaders.ctrlflow(), outputs=[
        og.SymLocationDesc("r", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
        og.SymLocationDesc("count", og.TypeInt, False, og.SymArenaOutputs, 4, 8)])
    W, H = 256, 200
    u, v = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H), 2)
    assert g.is_specialized()
    ref = np.zeros((W * H, 2), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert_same(got, ref, int_cols=(1,))


@pytest.mark.parametrize("name", ["noise_perlin", "noise_simplex", "pnoise_cell", "hashnoise", "noise_gabor3d_filter"])
def test_testsuite_shaders(name):
    from test_oracle_golden import TESTSUITE, suite_P, suite_program
    kw = dict(TESTSUITE)[name]
    ss, g = suite_program(name, kw)
    ss.attribute("jit", 1)
    W, H = 128, 96
    u, v = pixel_grid(W, H)
    P = suite_P(kw, u, v)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, P=P), 3)
    assert g.is_specialized()
    ref = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P), ref) == 0
    assert_same(got, ref)


def test_deformer_userdata():
    from test_oracle_golden import deformer_expected, deformer_group, deformer_inputs, fmt_g3
    ss = jit_system()
    g = deformer_group(ss)
    n, P, amp = deformer_inputs()
    got = gpu_run(ss, g, n, og.make_globals(P=dev(P)), 3, userdata=amp)
    assert g.is_specialized()
    assert [" ".join(fmt_g3(c) for c in row) for row in got] == deformer_expected()


def test_matrix_ops():
    from test_matrix_ops import REC, inputs, matrix_group
    ss = jit_system()
    g, _, _ = matrix_group(ss)
    W = H = 64
    u, v, P = inputs(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True, P=P), REC)
    assert g.is_specialized()
    ref = np.zeros((W * H, REC), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P, centers=True), ref) == 0
    assert_same(got, ref)


def test_c5_material_sampling():
    from openshadinglanguage_gb300 import workloads as W
    n = 4096
    P, N, I, T, rnd = W.c5_hits(n)
    ss = jit_system()
    Gd = og.make_globals(P=dev(P), N=dev(N), Ng=dev(N), I=dev(I), dPdu=dev(T))
    Gh = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    specs = W.c5_material_specs()
    for k in (0, 3, 12, 14):
        g = W.c5_material_group(ss, k, specs[k])
        got = gpu_run(ss, g, n, Gd, W.C5_OUT_FLOATS, userdata=rnd)
        assert g.is_specialized()
        ref = np.zeros((n, W.C5_OUT_FLOATS), np.float32)
        assert oracle_run(g.program_bytes(), n, Gh, ref, userdata=rnd) == 0
        assert_same(got, ref)
    assert ss.device_status() == 0


def test_single_point_and_empty():
    ss = jit_system()
    g, rec = fbm_group(ss, True)
    u, v = pixel_grid(1, 1, centers=True)
    G = device_grid_globals(u, v, 1, 1, centers=True)
    out = torch.zeros(rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, 0, G, 0, out.data_ptr(), sync=True)
    assert torch.count_nonzero(out).item() == 0
    got = gpu_run(ss, g, 1, G, rec)
    ref = np.zeros((1, rec), np.float32)
    oracle_run(g.program_bytes(), 1, grid_globals(u, v, 1, 1, centers=True), ref)
    assert_same(got, ref, int_cols=(rec - 1,))
