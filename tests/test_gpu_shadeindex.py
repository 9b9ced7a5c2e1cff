"""Execution with a shadeindex (BatchedExecutor::execute's wide_shadeindex,
src/include/OSL/oslexec.h:1000-1004): point i reads its userdata record and
writes its output record at shadeindex[i] (batched_llvm_instance.cpp:
1219-1229). Checked against the plain launch: with a permutation, record
shadeindex[i] of the indexed run equals record i of the plain run, bit for
bit, on the interpreter and on the specialized kernel (whose staged output
records are scattered when a tile is copied out)."""
import numpy as np
import pytest

from helpers import og
from openshadinglanguage_gb300.oso import OsoBuilder

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def userdata_group(ss):
    """o = 2 * x + u, c = (x, v, x * v) with x a lockgeom=0 parameter bound to
    the userdata arena."""
    b = OsoBuilder("si_probe")
    o = b.param("float", "o", 0.0, output=True)
    c = b.param("color", "c", [0.0, 0.0, 0.0], output=True)
    x = b.param("float", "x", 0.0, lockgeom=False)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    t, w = b.tmp("float"), b.tmp("float")
    b.op("mul", t, x, b.const("float", 2.0))
    b.op("add", o, t, u)
    b.op("mul", w, x, v)
    b.op("color", c, x, v, w)
    ss.LoadMemoryCompiledShader("si_probe", b.text())
    g = ss.ShaderGroupBegin("si_g")
    ss.Shader(g, "surface", "si_probe", "L")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("L.o", og.TypeFloat, False, og.SymArenaOutputs, 0, 16),
                       og.SymLocationDesc("L.c", og.TypeColor, False, og.SymArenaOutputs, 4, 16),
                       og.SymLocationDesc("L.x", og.TypeFloat, False, og.SymArenaUserData, 0, 4)])
    return g


@pytest.mark.parametrize("jit", [0, 1])
def test_shadeindex_scatters_userdata_and_outputs(torch, jit):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = userdata_group(ss)
    n = 70001
    rng = np.random.default_rng(11)
    u = rng.random(n, dtype=np.float32)
    v = rng.random(n, dtype=np.float32)
    x = rng.standard_normal(n).astype(np.float32)
    si = rng.permutation(n).astype(np.int32)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    G = og.make_globals(u=du, v=dv)
    out_plain = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, G, torch.from_numpy(x).cuda().data_ptr(), out_plain.data_ptr(), sync=True)
    x_scattered = np.empty_like(x)
    x_scattered[si] = x
    dx = torch.from_numpy(x_scattered).cuda()
    dsi = torch.from_numpy(si).cuda()
    out_idx = torch.full((n * 4,), -5.0, dtype=torch.float32, device="cuda")
    ss.execute_batch_indexed(g, n, G, dsi.data_ptr(), dx.data_ptr(), out_idx.data_ptr())
    torch.cuda.synchronize()
    assert ss.device_status() == 0
    assert g.is_specialized() == bool(jit)
    a = out_plain.cpu().numpy().reshape(n, 4)
    b = out_idx.cpu().numpy().reshape(n, 4)
    assert np.array_equal(b[si].view(np.uint32), a.view(np.uint32))


@pytest.mark.parametrize("jit", [0, 1])
def test_shadeindex_on_the_layered_closure_group(torch, jit):
    """The headline group: closure records and BSDF eval (staged records on
    the specialized kernel), records scattered in reverse order."""
    from openshadinglanguage_gb300 import workloads
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = workloads.c2_group(ss)
    W = H = 192
    n = W * H
    u, v, I = workloads.c2_inputs(W, H)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    G = workloads.c2_globals(og.make_globals, dev(u), dev(v), dev(I))
    rec = workloads.C2_STRIDE // 4
    out_plain = torch.zeros(n * rec, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, G, 0, out_plain.data_ptr(), sync=True)
    si = np.arange(n, dtype=np.int32)[::-1].copy()
    out_idx = torch.zeros(n * rec, dtype=torch.float32, device="cuda")
    ss.execute_batch_indexed(g, n, G, dev(si).data_ptr(), 0, out_idx.data_ptr())
    torch.cuda.synchronize()
    assert ss.device_status() == 0
    a = out_plain.cpu().numpy().reshape(n, rec)
    b = out_idx.cpu().numpy().reshape(n, rec)
    assert np.array_equal(b[si].view(np.uint32), a.view(np.uint32))
