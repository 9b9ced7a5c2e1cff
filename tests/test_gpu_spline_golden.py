"""The testsuite's spline shader on the GPU (interpreter and specialized
kernel): bit-exact to the oracle, hence equal to the reference images."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from test_gpu_parity import assert_same, device_grid_globals, gpu_run  # noqa: E402
from test_spline_golden import spline_shader  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("k", range(5))
def test_spline_band_matches_oracle(k, jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    ss.LoadMemoryCompiledShader("spline_t%d" % k, spline_shader(k))
    g = ss.ShaderGroupBegin("gspline%d" % k)
    ss.Shader(g, "surface", "spline_t%d" % k, "l")
    ss.ShaderGroupEnd(g)
    locs, off = [], 0
    for nm, ty, n in [("Cspline", og.TypeColor, 3), ("DxCspline", og.TypeColor, 3), ("Fspline", og.TypeFloat, 1),
                      ("DxFspline", og.TypeFloat, 1), ("NumKnots", og.TypeFloat, 1)]:
        locs.append(og.SymLocationDesc("l." + nm, ty, False, og.SymArenaOutputs, off, 36))
        off += 4 * n
    ss.add_symlocs(g, locs)
    W = H = 256
    u, v = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H), 9)
    ref = np.zeros((W * H, 9), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert_same(got, ref)
    assert ss.device_status() == 0


@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("basis", ["linear", "catmull-rom", "bspline", "bezier", "hermite", "constant"])
def test_splineinverse_matches_oracle(basis, jit):
    from test_spline_golden import splineinverse_group
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    knots = [0.0, 0.0, 0.05, 0.1, 0.3, 1.0, 1.0] if basis != "bezier" else [0.0, 0.1, 0.2, 0.4, 0.5, 0.8, 1.0]
    g = splineinverse_group(ss, basis, knots, name="gsinv_%s_%d" % (basis.replace("-", "_"), jit))
    W, H = 301, 7
    u, v = pixel_grid(W, H)
    got = gpu_run(ss, g, W * H, device_grid_globals(u, v, W, H), 2)
    ref = np.zeros((W * H, 2), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), ref) == 0
    assert_same(got, ref)
    assert ss.device_status() == 0
