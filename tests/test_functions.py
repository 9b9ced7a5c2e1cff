"""User functions: oslc inlines each call inside a functioncall op whose
jump is the end of the body (src/liboslcomp/codegen.cpp:1890-1905); a
return inside the body leaves the function, not the layer. Checked: an
early return in an if with an else, a return inside a loop, nested calls
(an outer function calling an inner one after its own early return), a
layer return and exit() around them, and bodies without a return (no
masking needed). The oracle matches the values computed here in Python;
the GPU (interpreter and specialized kernel) equals the oracle bit for
bit."""
import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder


def helper_body(b, x, res, tag):
    """float helper(float x) {
           if (x < 0.25) return 1; else res = -1;
           float acc = 0;
           for (int i = 0; i < 4; i++) { acc += x; if (acc > 1.0) return acc * 10; }
           return acc; }"""
    f = lambda v: b.const("float", v)
    c = b.tmp("int")
    with b.function("helper"):
        b.op("lt", c, x, f(0.25))
        with b.if_(c) as blk:
            b.op("assign", res, f(1.0))
            b.op("return")
            blk.else_()
            b.op("assign", res, f(-1.0))
        acc, i = b.local("float", "acc" + tag), b.local("int", "i" + tag)
        b.op("assign", acc, f(0.0))
        lc = b.tmp("int")
        with b.loop("for", lc) as lp:
            b.op("assign", i, b.const("int", 0))
            lp.cond()
            b.op("lt", lc, i, b.const("int", 4))
            lp.body()
            b.op("add", acc, acc, x)
            big = b.tmp("int")
            b.op("gt", big, acc, f(1.0))
            with b.if_(big):
                b.op("mul", res, acc, f(10.0))
                b.op("return")
            lp.step()
            b.op("add", i, i, b.const("int", 1))
        b.op("assign", res, acc)
        b.op("return")


def helper_py(x):
    x = np.float32(x)
    if x < np.float32(0.25):
        return np.float32(1.0)
    acc = np.float32(0.0)
    for _ in range(4):
        acc = np.float32(acc + x)
        if acc > np.float32(1.0):
            return np.float32(acc * np.float32(10.0))
    return acc


def function_group(ss):
    b = OsoBuilder("fn_probe")
    o1 = b.param("float", "o1", 0.0, output=True)
    o2 = b.param("float", "o2", 0.0, output=True)
    o3 = b.param("float", "o3", 0.0, output=True)
    o4 = b.param("float", "o4", 0.0, output=True)
    u, v = b.glob("float", "u"), b.glob("float", "v")
    f = lambda x: b.const("float", x)
    # o1 = helper(u)
    helper_body(b, u, o1, "a")
    # o2 = outer(v): { if (v > 0.9) return 5; t = helper(v); return t + 1; }
    c, t = b.tmp("int"), b.local("float", "t")
    with b.function("outer"):
        b.op("gt", c, v, f(0.9))
        with b.if_(c):
            b.op("assign", o2, f(5.0))
            b.op("return")
        helper_body(b, v, t, "b")
        b.op("add", o2, t, f(1.0))
        b.op("return")
    # o3 = plain(u) with no return inside: u * 3
    with b.function("plain"):
        b.op("mul", o3, u, f(3.0))
    # a layer return after the calls for u > 0.75, exit for v < 0.1
    o4v = b.tmp("float")
    b.op("add", o4v, o1, o2)
    b.op("assign", o4, o4v)
    r, e = b.tmp("int"), b.tmp("int")
    b.op("gt", r, u, f(0.75))
    with b.if_(r):
        b.op("return")
    b.op("lt", e, v, f(0.1))
    with b.if_(e):
        b.op("exit")
    b.op("assign", o4, f(-2.0))
    ss.LoadMemoryCompiledShader("fn_probe", b.text())
    g = ss.ShaderGroupBegin("fn_g")
    ss.Shader(g, "surface", "fn_probe", "L")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("L.o%d" % (k + 1), og.TypeFloat, False, og.SymArenaOutputs, 4 * k, 16)
                       for k in range(4)])
    return g


def expected(u, v):
    out = np.zeros((u.size, 4), np.float32)
    for k, (x, y) in enumerate(zip(u, v)):
        a = helper_py(x)
        b = np.float32(5.0) if y > np.float32(0.9) else np.float32(helper_py(y) + np.float32(1.0))
        o4 = np.float32(a + b)
        if not (x > np.float32(0.75)) and not (y < np.float32(0.1)):
            o4 = np.float32(-2.0)
        out[k] = (a, b, np.float32(x * np.float32(3.0)), o4)
    return out


@pytest.mark.parametrize("fold", [1, 0])
def test_functions_on_the_oracle(fold):
    ss = og.ShadingSystem()
    ss.attribute("opt_constant_fold", fold)
    g = function_group(ss)
    W, H = 17, 13
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, 4), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    assert np.array_equal(out, expected(u, v))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_functions_equal_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = function_group(ss)
    W, H = 333, 41
    n = W * H
    u, v = pixel_grid(W, H)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.zeros(n * 4, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, grid_globals(du, dv, W, H), 0, out.data_ptr(), sync=True)
    assert ss.device_status() == 0
    got = out.cpu().numpy().reshape(n, 4)
    ref = np.zeros((n, 4), np.float32)
    assert oracle_run(g.program_bytes(), n, grid_globals(u, v, W, H), ref) == 0
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(ref, expected(u, v))
