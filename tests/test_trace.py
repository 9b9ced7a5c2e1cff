"""trace() under the default renderer services: RendererServices::trace
(src/liboslexec/rendservices.cpp:511-517) traces nothing and reports no
hit, so trace() is 0 and getmessage("trace", ...) finds nothing. The
shader follows testsuite/trace-reg's test_trace.osl (keyword options, a
masked second trace, the trace message queries); every point keeps Cout 0."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder


def trace_group(ss):
    b = OsoBuilder("test_trace")
    cout = b.param("vector", "Cout", [0.0, 0.0, 0.0], output=True)
    P, u = b.glob("point", "P"), b.glob("float", "u")
    d, res, got = b.tmp("vector"), b.tmp("int"), b.tmp("int")
    maxd, t = b.tmp("float"), b.tmp("float")
    hitdist = b.tmp("float")
    b.op("sub", d, b.const("vector", [1.0, 1.0, 1.0]), P)
    b.op("mul", t, b.const("float", 1000.0), u)
    b.op("add", maxd, b.const("float", 1000.0), t)
    b.op("trace", res, P, d, b.const("string", "mindist"), b.const("float", 1.0), b.const("string", "maxdist"),
         maxd, b.const("string", "shade"), b.const("int", 2), b.const("string", "traceset"),
         b.const("string", "teapot"))
    b.op("assign", hitdist, b.const("float", 1.0))
    b.op("getmessage", got, b.const("string", "trace"), b.const("string", "hitdist"), hitdist)
    b.op("assign", cout, b.const("vector", [0.0, 0.0, 0.0]))
    with b.if_(res):
        b.op("assign", cout, b.const("vector", [1.0, 1.0, 1.0]))
    with b.if_(got):
        b.op("vector", cout, hitdist, hitdist, hitdist)
    ss.LoadMemoryCompiledShader("test_trace", b.text())
    g = ss.ShaderGroupBegin("trace_g")
    ss.Shader(g, "surface", "test_trace", "L")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("L.Cout", og.TypeVector, False, og.SymArenaOutputs, 0, 12)])
    return g


def test_trace_reports_no_hit():
    ss = og.ShadingSystem()
    g = trace_group(ss)
    W = H = 64
    u, v = pixel_grid(W, H)
    out = np.full(W * H * 3, -1.0, np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    assert np.all(out == 0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_trace_equals_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = trace_group(ss)
    W = H = 64
    u, v = pixel_grid(W, H)
    out = torch.full((W * H * 3,), -1.0, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, W * H, grid_globals(torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda(), W, H), 0,
                     out.data_ptr(), sync=True)
    assert ss.device_status() == 0
    assert np.all(out.cpu().numpy() == 0.0)
