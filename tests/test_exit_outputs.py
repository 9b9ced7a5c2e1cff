"""exit() ends the group for a point, but what the point wrote before is
its result: the reference's outputs live in the output arena as the shader
writes them (symlocs, src/include/OSL/oslexec.h:69-105), so a point that
exits keeps its earlier writes, and the outputs of layers it never runs
keep what the buffer held. Here o = 1; if (u > 0.5) { o = 2; exit(); }
o = 3 gives 2 for u > 0.5 and 3 elsewhere, and the second layer's output
stays untouched on the exited points. The GPU (interpreter and
specialized kernel) equals the oracle."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder


def exit_group(ss):
    b = OsoBuilder("exit_probe")
    o = b.param("float", "o", 0.0, output=True)
    u = b.glob("float", "u")
    b.op("assign", o, b.const("float", 1.0))
    c = b.tmp("int")
    b.op("gt", c, u, b.const("float", 0.5))
    with b.if_(c):
        b.op("assign", o, b.const("float", 2.0))
        b.op("exit")
    b.op("assign", o, b.const("float", 3.0))
    b2 = OsoBuilder("after_exit")
    i = b2.param("float", "i", 0.0)
    r = b2.param("float", "r", -1.0, output=True)
    b2.op("add", r, i, b2.const("float", 10.0))
    ss.LoadMemoryCompiledShader("exit_probe", b.text())
    ss.LoadMemoryCompiledShader("after_exit", b2.text())
    g = ss.ShaderGroupBegin("exit_g")
    ss.Shader(g, "surface", "exit_probe", "A")
    ss.Shader(g, "surface", "after_exit", "B")
    ss.ConnectShaders(g, "A", "o", "B", "i")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("A.o", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
                       og.SymLocationDesc("B.r", og.TypeFloat, False, og.SymArenaOutputs, 4, 8)])
    return g


def test_outputs_written_before_exit_are_kept():
    ss = og.ShadingSystem()
    g = exit_group(ss)
    W, H = 8, 2
    u, v = pixel_grid(W, H)
    out = np.full((W * H, 2), 7.0, np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    exited = u > 0.5
    assert np.array_equal(out[:, 0], np.where(exited, 2.0, 3.0).astype(np.float32))
    # layer B never ran for exited points: their record keeps what it held
    assert np.array_equal(out[:, 1], np.where(exited, 7.0, 13.0).astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_outputs_written_before_exit_equal_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = exit_group(ss)
    W, H = 300, 7
    n = W * H
    u, v = pixel_grid(W, H)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.full((n * 2,), 7.0, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, grid_globals(du, dv, W, H), 0, out.data_ptr(), sync=True)
    got = out.cpu().numpy().reshape(n, 2)
    ref = np.full((n, 2), 7.0, np.float32)
    assert oracle_run(g.program_bytes(), n, grid_globals(u, v, W, H), ref) == 0
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
