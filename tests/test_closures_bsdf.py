"""Closures, spline and BSDF evaluation on the oracle (CPU): the closure
tree semantics of src/liboslexec/opclosure.cpp and testrender's
CompositeBSDF evaluation on simple, analytically known cases."""
import numpy as np

from helpers import og, oracle_run
from openshadinglanguage_gb300 import OsoBuilder, workloads


def run_single(oso, name, n, G, stride, extra=None):
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader(name, oso)
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", name, "L")
    ss.ShaderGroupEnd(g)
    if extra:
        extra(ss, g)
    out = np.zeros((n, stride // 4), np.float32)
    st = oracle_run(g.program_bytes(), n, G, out)
    return out, st


def diffuse_shader(weight):
    b = OsoBuilder("dif", "surface")
    Ci = b.glob("closure color", "Ci")
    N = b.glob("normal", "N")
    d = b.tmp("closure color")
    b.op("closure", d, b.const("string", "diffuse"), N)
    b.op("mul", Ci, d, b.const("float", weight))
    return b.text()


def test_single_diffuse_lobe_eval_is_cosine_over_pi():
    n = 16
    rng = np.random.default_rng(3)
    I = -np.abs(rng.normal(size=(3, n))).astype(np.float32)
    I /= np.linalg.norm(I, axis=0)
    G = og.make_globals(I=np.ascontiguousarray(I), N=(0, 0, 1))
    wi = (0.0, 0.6, 0.8)

    def extra(ss, g):
        ss.add_symlocs(g, [og.SymLocationDesc("Ci", og.TypeClosure.array(1), False, og.SymArenaOutputs, 0, 84)])
        ss.bsdf_eval_output(g, "Ci", wi, 68, 84)

    out, st = run_single(diffuse_shader(0.5), "dif", n, G, 84, extra)
    assert st == 0
    assert np.all(out[:, 0].view(np.int32) == 1)
    assert np.all(out[:, 1].view(np.int32) == 3)              # DIFFUSE_ID
    assert np.allclose(out[:, 2:5], 0.5)                      # MUL weight folded by the walk
    np.testing.assert_allclose(out[:, 17:20], 0.5, rtol=1e-6)  # eval weight = closure weight
    np.testing.assert_allclose(out[:, 20], 0.8 / np.pi, rtol=1e-6)


def test_zero_weight_closure_is_null_and_one_weight_is_identity():
    G = og.make_globals(N=(0, 0, 1))

    def extra(ss, g):
        ss.add_symlocs(g, [og.SymLocationDesc("Ci", og.TypeClosure.array(2), False, og.SymArenaOutputs, 0, 132)])

    out, st = run_single(diffuse_shader(0.0), "dif", 4, G, 132, extra)
    assert st == 0 and np.all(out[:, 0].view(np.int32) == 0)
    out, st = run_single(diffuse_shader(1.0), "dif", 4, G, 132, extra)
    assert st == 0 and np.all(out[:, 0].view(np.int32) == 1) and np.all(out[:, 2:5] == 1.0)


def test_closure_pool_overflow_sets_status():
    """Closures made inside a loop draw on a pool of max_closure_components
    nodes per point (a loop-free program gets one node per closure op and
    cannot overflow); running past it raises the overflow status bit.

        for (int i = 0; i < 20; ++i) Ci += diffuse(N);
    """
    b = OsoBuilder("many", "surface")
    Ci = b.glob("closure color", "Ci")
    N = b.glob("normal", "N")
    i = b.local("int", "i")
    c = b.tmp("int")
    with b.loop("for", c) as L:
        b.op("assign", i, b.const("int", 0))
        L.cond()
        b.op("lt", c, i, b.const("int", 20))
        L.body()
        d = b.tmp("closure color")
        b.op("closure", d, b.const("string", "diffuse"), N)
        b.op("add", Ci, Ci, d)
        L.step()
        b.op("add", i, i, b.const("int", 1))

    def extra(ss, g):
        ss.attribute("max_closure_components", 8)
        ss.add_symlocs(g, [og.SymLocationDesc("Ci", og.TypeClosure.array(4), False, og.SymArenaOutputs, 0, 260)])

    out, st = run_single(b.text(), "many", 2, og.make_globals(N=(0, 0, 1)), 260, extra)
    assert st & 1, "closure arena overflow must be reported"


def test_spline_catmull_rom_interpolates_knots():
    # catmull-rom passes through the interior knots at segment boundaries
    b = OsoBuilder("spl")
    r = b.param("float", "r", 0.0, output=True)
    x = b.param("float", "x", 0.0, lockgeom=False)
    knots = b.const("float[6]", [0.0, 1.0, 4.0, 9.0, 16.0, 25.0])
    b.op("spline", r, b.const("string", "catmull-rom"), x, knots)
    xs = np.array([0.0, 1 / 3, 2 / 3, 1.0], np.float32)

    def extra(ss, g):
        ss.add_symlocs(g, [og.SymLocationDesc("r", og.TypeFloat, False, og.SymArenaOutputs, 0, 4),
                           og.SymLocationDesc("x", og.TypeFloat, False, og.SymArenaUserData, 0, 4)])

    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("spl", b.text())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "spl", "L")
    ss.ShaderGroupEnd(g)
    extra(ss, g)
    out = np.zeros((4, 1), np.float32)
    assert oracle_run(g.program_bytes(), 4, og.make_globals(), out, userdata=xs) == 0
    np.testing.assert_allclose(out[:, 0], [1.0, 4.0, 9.0, 16.0], rtol=1e-5)


def test_layered_closure_group_on_oracle():
    ss = og.ShadingSystem()
    g = workloads.c2_group(ss)
    W = H = 32
    u, v, I = workloads.c2_inputs(W, H)
    G = workloads.c2_globals(og.make_globals, u, v, I)
    out = np.zeros((W * H, workloads.C2_STRIDE // 4), np.float32)
    assert oracle_run(g.program_bytes(), W * H, G, out) == 0
    assert np.all(out[:, 0].view(np.int32) == 2)
    assert np.all(out[:, 1].view(np.int32) == 3) and np.all(out[:, 17].view(np.int32) == 8)
    alpha = out[:, 28]
    assert np.all((alpha >= 0.05) & (alpha <= 0.8))
    ev = out[:, workloads.C2_EVAL_OFFSET // 4: workloads.C2_EVAL_OFFSET // 4 + 4]
    assert np.all(np.isfinite(ev)) and np.all(ev[:, 3] > 0)
