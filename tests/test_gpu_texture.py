"""texture() on the GPU, interpreter and specialized kernel, bit-exact to
the oracle: every wrap mode, level-of-detail blends from the coordinate
derivatives, the width option, one- and three-channel results, coordinates
far outside [0, 1]."""
import numpy as np
import pytest

from helpers import float_equal, grid_globals, og, oracle_run, pixel_grid, single_layer_group

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import assert_same, device_grid_globals, gpu_run  # noqa: E402
from test_texture import make_image, register, tex_shader  # noqa: E402,F401


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


CASES = [dict(wrap=w, scale=s) for w in ("black", "clamp", "periodic", "mirror") for s in (1.0, 3.3, 40.0)]
CASES += [dict(wrap="periodic", scale=2.0, width=4.0), dict(wrap="clamp", scale=0.5, nc=1, first=1),
          dict(wrap="mirror", scale=-7.5)]


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join("%s%s" % kv for kv in c.items()))
def test_texture_matches_oracle(case, jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    register(ss, make_image(37, 53, 3))
    nc = case.get("nc", 3)
    name = "gt_%d" % abs(hash(tuple(sorted(case.items()))))
    oso = tex_shader(name, case["scale"], case["wrap"], nc=nc, width=case.get("width"), first=case.get("first"))
    ty = og.TypeColor if nc == 3 else og.TypeFloat
    g = single_layer_group(ss, name, oso, outputs=[og.SymLocationDesc("Cout", ty, False, og.SymArenaOutputs, 0, 4 * nc)])
    W, H = 61, 45
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), nc)
    if jit:
        assert g.is_specialized()
    ref = np.zeros((W * H, nc), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref)
    assert ss.device_status() == 0


ENV_CASES = [dict(width=None), dict(width=3.0), dict(first=1)]


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("case", ENV_CASES, ids=lambda c: "-".join("%s%s" % kv for kv in c.items()))
def test_environment_matches_oracle(case, jit):
    from openshadinglanguage_gb300.shaders import environment_lookup
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    register(ss, make_image(41, 83, 3, seed=2), "env")
    name = "genv_%d" % abs(hash(tuple(sorted(case.items()))))
    g = single_layer_group(ss, name, environment_lookup(name, **case),
                           outputs=[og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    W, H = 97, 51
    u, v = pixel_grid(W, H, centers=True)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H, centers=True), 3)
    ref = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), ref) == 0
    assert_same(got, ref)
    assert ss.device_status() == 0
