"""Static closures: when no closure value depends on control flow, the
lowering replaces the run-time closure tree (node pool, MUL/ADD nodes,
tree walks) with one node per closure op and a term table per consumer
(attribute opt_static_closures, on by default). The tree walk itself is
pinned to the reference's printed closures (test_closure_print); here the
same groups lowered both ways must give the same outputs on the oracle,
bit for bit (floats value-identical), including null closures from zero
MUL weights, zero component weights, nested products of float and color
weights, a subtree added twice, and BSDF evaluation and sampling. Groups
whose closures depend on control flow keep the tree."""
import numpy as np
import pytest

from helpers import float_equal, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300 import _capi, workloads
from openshadinglanguage_gb300.oso import OsoBuilder

OP_CLOSURE = 116
OP_CLOSURE_NODE = 127


def opcodes(blob):
    h = np.frombuffer(blob[:64], np.uint32)
    ops = np.frombuffer(blob[64:64 + 32 * int(h[2])], np.uint16).reshape(-1, 16)
    return set(int(c) for c in ops[:, 0])


def stress_shader():
    """Products, sums and nulls that exercise every rule of the walk:

        closure color d = diffuse(N), m = microfacet("ggx", N, dPdu, 0.2, 0.2, 1.5, 0);
        closure color w1 = u * d;                    // null where u == 0
        closure color w2 = color(u, v, 0.5) * (w1 + m);
        closure color w3 = 0.5 * (w2 + d + w1);
        closure color z = (closure weighted by v - 0.5) oren_nayar(N, 0.3);  // null at v == 0.5
        Ci = w3 + (v * emission()) + z + 0 * d;  // the last term is null
        big = w3 + w3 + (v * emission()) + z;    // 10 terms, 8 records kept
    """
    b = OsoBuilder("stat", "surface")
    big = b.param("closure color", "big", 0.0, output=True)
    Ci, N, dPdu = b.glob("closure color", "Ci"), b.glob("normal", "N"), b.glob("vector", "dPdu")
    u, v = b.glob("float", "u"), b.glob("float", "v")
    cl = lambda: b.tmp("closure color")
    S = lambda x: b.const("string", x)
    f = lambda x: b.const("float", x)
    d, m, e = cl(), cl(), cl()
    b.op("closure", d, S("diffuse"), N)
    b.op("closure", m, S("microfacet"), S("ggx"), N, dPdu, f(0.2), f(0.2), f(1.5), b.const("int", 0))
    w1, s1, w2, s2, s3, w3 = cl(), cl(), cl(), cl(), cl(), cl()
    b.op("mul", w1, u, d)
    b.op("add", s1, w1, m)
    c = b.tmp("color")
    b.op("color", c, u, v, f(0.5))
    b.op("mul", w2, c, s1)
    b.op("add", s2, w2, d)
    b.op("add", s3, s2, w1)
    b.op("mul", w3, f(0.5), s3)
    ve, z, vw = cl(), cl(), b.tmp("color")
    b.op("closure", e, S("emission"))
    b.op("mul", ve, v, e)
    vm = b.tmp("float")
    b.op("sub", vm, v, f(0.5))
    b.op("color", vw, vm, vm, vm)
    b.op("closure", z, vw, S("oren_nayar"), N, f(0.3))
    t2, t3, zd, t4 = cl(), cl(), cl(), cl()
    b.op("add", t2, w3, ve)
    b.op("add", t3, t2, z)
    b.op("mul", zd, f(0.0), d)
    b.op("add", t4, t3, zd)
    b.op("assign", Ci, t4)
    b1, b2, b3 = cl(), cl(), cl()
    b.op("add", b1, w3, w3)
    b.op("add", b2, b1, ve)
    b.op("add", b3, b2, z)
    b.op("assign", big, b3)
    return b.text()


REC = 1 + 16 * 8
STRIDE = 4 * (2 * REC + 4)


def stress_group(ss):
    ss.LoadMemoryCompiledShader("stat", stress_shader())
    g = ss.ShaderGroupBegin("stat_group")
    ss.Shader(g, "surface", "stat", "L")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("Ci", og.TypeClosure.array(8), False, og.SymArenaOutputs, 0, STRIDE),
                       og.SymLocationDesc("L.big", og.TypeClosure.array(8), False, og.SymArenaOutputs, 4 * REC, STRIDE)])
    ss.bsdf_eval_output(g, "Ci", (0.3, 0.4, 0.866), 8 * REC, STRIDE)
    return g


def stress_inputs(W=9, H=7):
    u, v = pixel_grid(W, H)  # u and v hit 0, 0.5 and 1 exactly
    rng = np.random.default_rng(5)
    I = -np.abs(rng.normal(size=(3, W * H))).astype(np.float32)
    I /= np.linalg.norm(I, axis=0)
    return u, v, np.ascontiguousarray(I)


def both(build):
    """The group lowered with static closures and with the tree."""
    out = []
    for st in (1, 0):
        ss = og.ShadingSystem()
        ss.attribute("opt_static_closures", st)
        out.append(build(ss))
    return out


def test_stress_group_static_equals_tree():
    gs, gt = both(stress_group)
    assert OP_CLOSURE_NODE in opcodes(gs.program_bytes()) and OP_CLOSURE not in opcodes(gs.program_bytes())
    assert OP_CLOSURE in opcodes(gt.program_bytes())
    u, v, I = stress_inputs()
    n = u.size
    res = []
    for g in (gs, gt):
        G = grid_globals(u, v, 9, 7)
        G.I.data = _capi.ctypes.c_void_p(I.ctypes.data)
        G.I.plane_stride = n
        out = np.zeros((n, STRIDE // 4), np.float32)
        assert oracle_run(g.program_bytes(), n, G, out) == 0
        res.append(out)
    s, t = res
    assert np.array_equal(s[:, 0].view(np.int32), t[:, 0].view(np.int32))  # component counts
    counts = s[:, 0].view(np.int32)
    assert counts.min() < counts.max()  # nulls removed components at some points
    assert float_equal(s, t).all()
    assert np.array_equal(s.view(np.int32)[:, REC], t.view(np.int32)[:, REC])
    assert s.view(np.int32)[:, REC].max() == 8  # the big sum keeps its first 8 components
    for base in (0, REC):
        ids = s[:, base + 1:base + REC].reshape(n, 8, 16)[:, :, 0].view(np.int32)
        assert np.array_equal(ids, t[:, base + 1:base + REC].reshape(n, 8, 16)[:, :, 0].view(np.int32))


def test_layered_closure_group_static_equals_tree():
    gs, gt = both(workloads.c2_group)
    assert OP_CLOSURE_NODE in opcodes(gs.program_bytes())
    u, v, I = workloads.c2_inputs(64, 48)
    n = u.size
    res = []
    for g in (gs, gt):
        out = np.zeros((n, workloads.C2_STRIDE // 4), np.float32)
        assert oracle_run(g.program_bytes(), n, workloads.c2_globals(og.make_globals, u, v, I), out) == 0
        res.append(out)
    assert float_equal(res[0], res[1]).all()
    assert np.array_equal(res[0][:, 0].view(np.int32), res[1][:, 0].view(np.int32))


def test_material_groups_static_equal_tree():
    n = 4000
    P, N, I, T, rnd = workloads.c5_hits(n)
    G = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    for k, spec in enumerate(workloads.c5_material_specs()):
        gs, gt = both(lambda ss: workloads.c5_material_group(ss, k, spec))
        assert OP_CLOSURE_NODE in opcodes(gs.program_bytes()), k
        res = []
        for g in (gs, gt):
            out = np.zeros((n, workloads.C5_OUT_FLOATS), np.float32)
            assert oracle_run(g.program_bytes(), n, G, out, userdata=np.ascontiguousarray(rnd)) == 0
            res.append(out)
        assert float_equal(res[0], res[1]).all(), "material %d" % k


def test_control_flow_dependent_closures_keep_the_tree():
    from test_closure_print import conditional_group, zero_group
    ss = og.ShadingSystem()
    g, _ = conditional_group(ss)
    assert OP_CLOSURE in opcodes(g.program_bytes())
    g2, _ = zero_group(og.ShadingSystem())  # closures through a connection: static
    assert OP_CLOSURE_NODE in opcodes(g2.program_bytes())


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_static_closures_equal_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = stress_group(ss)
    u, v, I = stress_inputs(61, 37)
    n = u.size
    du, dv, dI = (torch.from_numpy(x).cuda() for x in (u, v, I))
    Gd = grid_globals(du, dv, 61, 37)
    Gd.I.data = _capi.ctypes.c_void_p(dI.data_ptr())
    Gd.I.plane_stride = n
    Gd._keep += [dI]
    out = torch.zeros(n * STRIDE // 4, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, Gd, 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    got = out.cpu().numpy().reshape(n, STRIDE // 4)
    G = grid_globals(u, v, 61, 37)
    G.I.data = _capi.ctypes.c_void_p(I.ctypes.data)
    G.I.plane_stride = n
    ref = np.zeros((n, STRIDE // 4), np.float32)
    assert oracle_run(g.program_bytes(), n, G, ref) == 0
    assert float_equal(got, ref).all()
    assert np.array_equal(got[:, 0].view(np.int32), ref[:, 0].view(np.int32))
