"""Closure trees pinned to the reference testsuite's printed closures.

The testsuite shaders `closure`, `closure-conditional` and `closure-zero`
(testsuite/*/test.osl, a.osl, b.osl) print their closures with printf("%s");
their expected outputs (ref/out.txt, copied into tests/golden/ by
make_golden.py) pin the closure tree: component weights through MUL and ADD
nodes, parameter values, keyword parameters (the last repeated keyword
wins), null closures in sums and connections between layers. Here each
printed state is stored as a closure output instead of printed, rendered by
the test-side printer in the reference's format, and compared as text with
the reference's output. The oracle is checked on the CPU; the GPU kernels
(interpreter and specialized) must then store the same records.

Not covered: the `closure` shader's last step adds a keyword parameter made
by format("%f", u), a string operation this executor does not run; the
`closure-parameters` shader passes arrays of five vectors and colors, more
than a component's 12 parameter words.
"""
import os

import numpy as np
import pytest

from closure_print import Printer, printed_states
from helpers import GOLDEN, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder

REC = 1 + 16 * 8  # [count] + 8 components of 16 words
STRINGS = ("label", "first", "second", "one", "MyAOV", "test")


def closure_loc(name, offset, stride):
    return og.SymLocationDesc(name, og.TypeClosure.array(8), False, og.SymArenaOutputs, offset, stride)


def closure_shader():
    """testsuite/closure/test.osl with each printed state stored in an
    output closure s1..s6 instead of printed:

        shader test(float Kd = 0.5, float Ks = 0.5, float exponent = 20,
                    color opacity = 0.5, output closure color s1..s6 = 0)
        {
            Ci = Kd * diffuse(N, "label", "first", "label", "second");  s1 = Ci;
            closure color spec = Ks * phong(N, exponent, "label", "one");
            Ci += spec;                                                  s2 = Ci;
            Ci = opacity * Ci + (1 - opacity) * transparent();          s3 = Ci;
            Ci += emission();                                            s4 = Ci;
            Ci += 0.25 * debug("MyAOV");                                 s5 = Ci;
            Ci += 0.5 * holdout();                                       s6 = Ci;
        }
    """
    b = OsoBuilder("closure_test")
    Kd, Ks = b.param("float", "Kd", 0.5), b.param("float", "Ks", 0.5)
    exponent = b.param("float", "exponent", 20.0)
    opacity = b.param("color", "opacity", [0.5, 0.5, 0.5])
    outs = [b.param("closure color", "s%d" % k, 0.0, output=True) for k in range(1, 7)]
    Ci, N = b.glob("closure color", "Ci"), b.glob("normal", "N")
    s = lambda x: b.const("string", x)
    cl = lambda: b.tmp("closure color")
    t1, t2 = cl(), cl()
    b.op("closure", t1, s("diffuse"), N, s("label"), s("first"), s("label"), s("second"))
    b.op("mul", t2, Kd, t1)
    b.op("assign", Ci, t2)
    b.op("assign", outs[0], Ci)
    spec, t3 = b.local("closure color", "spec"), cl()
    b.op("closure", t3, s("phong"), N, exponent, s("label"), s("one"))
    b.op("mul", spec, Ks, t3)
    b.op("add", Ci, Ci, spec)
    b.op("assign", outs[1], Ci)
    t4, t5, t6, t7 = cl(), b.tmp("color"), cl(), cl()
    b.op("mul", t4, opacity, Ci)
    b.op("sub", t5, b.const("float", 1.0), opacity)
    b.op("closure", t6, s("transparent"))
    b.op("mul", t7, t5, t6)
    b.op("add", Ci, t4, t7)
    b.op("assign", outs[2], Ci)
    t8 = cl()
    b.op("closure", t8, s("emission"))
    b.op("add", Ci, Ci, t8)
    b.op("assign", outs[3], Ci)
    t9, t10 = cl(), cl()
    b.op("closure", t9, s("debug"), s("MyAOV"))
    b.op("mul", t10, b.const("float", 0.25), t9)
    b.op("add", Ci, Ci, t10)
    b.op("assign", outs[4], Ci)
    t11, t12 = cl(), cl()
    b.op("closure", t11, s("holdout"))
    b.op("mul", t12, b.const("float", 0.5), t11)
    b.op("add", Ci, Ci, t12)
    b.op("assign", outs[5], Ci)
    return b.text()


def conditional_shader():
    """testsuite/closure-conditional/test.osl:

        shader test()
        {
            if (u > 0.5) Ci = u * emission();
            else         Ci = color(1, 0, 0) * emission();
        }
    """
    b = OsoBuilder("closure_cond")
    Ci, u = b.glob("closure color", "Ci"), b.glob("float", "u")
    c, e1, e2 = b.tmp("int"), b.tmp("closure color"), b.tmp("closure color")
    b.op("gt", c, u, b.const("float", 0.5))
    with b.if_(c) as br:
        b.op("closure", e1, b.const("string", "emission"))
        b.op("mul", Ci, u, e1)
        br.else_()
        b.op("closure", e2, b.const("string", "emission"))
        b.op("mul", Ci, b.const("color", [1, 0, 0]), e2)
    return b.text()


def zero_shaders():
    """testsuite/closure-zero a.osl and b.osl (b's sum stored in an output
    instead of printed):

        shader a(output closure color output_closure = 0)
        { output_closure = debug("test"); }
        shader b(closure color in0 = 0, closure color in1 = 0,
                 output closure color out = 0)
        { out = in0 + in1; }
    """
    a = OsoBuilder("closure_zero_a")
    oc = a.param("closure color", "output_closure", 0.0, output=True)
    a.op("closure", oc, a.const("string", "debug"), a.const("string", "test"))
    b = OsoBuilder("closure_zero_b")
    in0, in1 = b.param("closure color", "in0", 0.0), b.param("closure color", "in1", 0.0)
    out = b.param("closure color", "out", 0.0, output=True)
    b.op("add", out, in0, in1)
    return a.text(), b.text()


def system(jit=0):
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    return ss


def closure_group(ss):
    ss.LoadMemoryCompiledShader("closure_test", closure_shader())
    g = ss.ShaderGroupBegin("closure_test_group")
    ss.Shader(g, "surface", "closure_test", "test")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [closure_loc("test.s%d" % k, 4 * REC * (k - 1), 4 * REC * 6) for k in range(1, 7)])
    return g, 6


def conditional_group(ss):
    ss.LoadMemoryCompiledShader("closure_cond", conditional_shader())
    g = ss.ShaderGroupBegin("closure_cond_group")
    ss.Shader(g, "surface", "closure_cond", "test")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [closure_loc("test.Ci", 0, 4 * REC)])
    return g, 1


def zero_group(ss):
    a, b = zero_shaders()
    ss.LoadMemoryCompiledShader("closure_zero_a", a)
    ss.LoadMemoryCompiledShader("closure_zero_b", b)
    g = ss.ShaderGroupBegin("closure_zero_group")
    ss.Shader(g, "surface", "closure_zero_a", "a")
    ss.Shader(g, "surface", "closure_zero_b", "b")
    ss.ConnectShaders(g, "a", "output_closure", "b", "in0")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [closure_loc("b.out", 0, 4 * REC)])
    return g, 1


# (group builder, testshade grid -g W H, fixture, printed marker, states per point used, states per point printed)
CASES = {
    "closure": (closure_group, (2, 2), "closure_out.txt", "Ci = ", 6, 7),
    "closure-conditional": (conditional_group, (5, 1), "closure_conditional_out.txt", "Ci = ", 1, 1),
    "closure-zero": (zero_group, (2, 1), "closure_zero_out.txt", "out =  ", 1, 1),
}


def names_by_id(ss):
    from openshadinglanguage_gb300 import _capi  # noqa: F401
    # the executor registers testrender's closure ids in this order
    order = ["emission", "background", "diffuse", "oren_nayar", "translucent", "phong", "ward", "microfacet",
             "reflection", "fresnel_reflection", "refraction", "transparent", "debug", "holdout"]
    return {i + 1: n for i, n in enumerate(order)}


def run_oracle(g, W, H, nout):
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, REC * nout), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    return out.view(np.uint32)


def expected(case):
    _, (W, H), fixture, marker, used, printed = CASES[case]
    states = printed_states(open(os.path.join(GOLDEN, fixture)).read(), marker)
    assert len(states) == W * H * printed
    return [[states[p * printed + k] for k in range(used)] for p in range(W * H)]


@pytest.mark.parametrize("case", sorted(CASES))
def test_oracle_prints_the_reference_closures(case):
    build, (W, H), _, _, used, _ = CASES[case]
    ss = system()
    g, nout = build(ss)
    rec = run_oracle(g, W, H, nout)
    pr = Printer(names_by_id(ss), STRINGS)
    exp = expected(case)
    for p in range(W * H):
        got = [pr.closure(rec[p, REC * k: REC * (k + 1)]) for k in range(used)]
        assert got == exp[p], "point %d:\n%s\n--- reference ---\n%s" % (p, "\n".join(got), "\n".join(exp[p]))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_stores_the_oracle_closures(case, jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build, (W, H), _, _, used, _ = CASES[case]
    ss = system(jit)
    g, nout = build(ss)
    u, v = pixel_grid(W, H)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.zeros(W * H * REC * nout, dtype=torch.int32, device="cuda")
    ss.execute_batch(g, W * H, grid_globals(du, dv, W, H), 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    got = out.cpu().numpy().view(np.uint32).reshape(W * H, REC * nout)
    assert np.array_equal(got, run_oracle(g, W, H, nout))
