"""Matrix operations pinned to the reference testsuite's `matrix` shader
output (testsuite/matrix/test.osl, expected text ref/out.txt copied to
tests/golden/matrix_out.txt by make_golden.py).

The testsuite shader prints its matrices with printf("%.5g") (after the
testsuite's pretty(), which turns |x| < 5e-6 into 0); here each printed
value is an output of the group, formatted the same way by the test and
compared as text with the reference's lines for every point of its
`-g 2 2` grid. testshade's "shader" space is a 45-degree rotation about z
followed by a translation (1, 0, 0), its "object" space a 90-degree
rotation followed by (0, 1, 0) (src/testshade/testshade.cpp:925-944); they
are registered as renderer matrices. Covered: constructors (diagonal, 16
values, varying), constructors in a named space, matrix(from, to) and
getmatrix against each other, an unknown space, component read and write,
negation, products and quotients with scalars, the identity and each other
(the quotients through the matrix inverse), transpose, determinant and
(in)equality. The parameter-initialisation block is not covered."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder

W = H = 2


def _rot_z(angle, t):
    c, s = np.float32(np.cos(np.float32(angle))), np.float32(np.sin(np.float32(angle)))
    M = np.eye(4, dtype=np.float32)
    M[0, :2] = (c, s)
    M[1, :2] = (-s, c)
    M[3, :3] = t
    return M


M_SHADER = _rot_z(np.pi / 4, (1, 0, 0))
M_OBJECT = _rot_z(np.pi / 2, (0, 1, 0))

# output name -> (type, number of floats)
OUTS = []


def build_shader():
    b = OsoBuilder("matrix_suite")
    outs = {}

    def out(name, t="matrix"):
        outs[name] = b.param(t, name, 0, output=True)
        OUTS.append((name, t))
        return outs[name]

    u, v = b.glob("float", "u"), b.glob("float", "v")
    f = lambda x: b.const("float", x)
    S = lambda s: b.const("string", s)
    vals = [f(round(0.1 * k, 1)) for k in range(1, 17)]
    # constructors
    b.op("matrix", out("m_a"), vals[0])
    b.op("matrix", out("m_16"), *vals)
    b.op("matrix", out("m_av"), u)
    b.op("matrix", out("m_16v"), u, v, *vals[2:])
    # in a named space
    one, zero = f(1.0), f(0.0)
    ident16 = [one, zero, zero, zero, zero, one, zero, zero, zero, zero, one, zero, zero, zero, zero, one]
    b.op("matrix", out("s_a"), S("shader"), one)
    b.op("matrix", out("s_16"), S("shader"), *ident16)
    b.op("matrix", out("s_av"), S("shader"), u)
    b.op("matrix", out("s_16v"), S("shader"), u, *ident16[1:])
    b.op("matrix", out("m_world"), S("world"), one)
    b.op("matrix", out("m_common"), S("common"), one)
    # from-to and getmatrix
    for fr, to in (("common", "shader"), ("common", "object"), ("shader", "object")):
        for x, y in ((fr, to), (to, fr)):
            tag = x[0] + y[0]
            M = out("ft_" + tag)
            b.op("matrix", M, S(x), S(y))
            Mg, ok, same, both = b.tmp("matrix"), b.tmp("int"), b.tmp("int"), out("ok_" + tag, "int")
            b.op("getmatrix", ok, S(x), S(y), Mg)
            b.op("eq", same, M, Mg)
            b.op("and", both, ok, same)
    Mf = b.tmp("matrix")
    b.op("getmatrix", out("found_foobar", "int"), S("foobar"), S("common"), Mf)
    # component access
    M = out("c_M")
    b.op("matrix", M, S("shader"), one)
    for j in range(4):
        b.op("mxcompref", out("c_m1%d" % j, "float"), M, b.const("int", 1), b.const("int", j))
    M2 = out("c_set5")
    b.op("assign", M2, M)
    b.op("mxcompassign", M2, b.const("int", 1), b.const("int", 3), f(5.0))
    M3 = out("c_set6u")
    b.op("assign", M3, M2)
    six = out("c_6u", "float")
    b.op("add", six, f(6.0), u)
    b.op("mxcompassign", M3, b.const("int", 1), b.const("int", 2), six)
    # arithmetic
    Id = b.local("matrix", "Ident")
    b.op("assign", Id, one)
    b.op("neg", out("a_neg"), M)
    b.op("mul", out("a_2M"), f(2.0), M)
    b.op("mul", out("a_M2"), M, f(2.0))
    b.op("div", out("a_Md2"), M, f(2.0))
    b.op("mul", out("a_MI"), M, Id)
    b.op("mul", out("a_IM"), Id, M)
    b.op("mul", out("a_MM"), M, M)
    b.op("div", out("a_MdM"), M, M)
    b.op("div", out("a_MdI"), M, Id)
    b.op("div", out("a_IdM"), Id, M)
    b.op("div", out("a_1dM"), one, M)
    b.op("transpose", out("a_T"), M)
    b.op("determinant", out("a_det", "float"), M)
    b.op("eq", out("a_eqMM", "int"), M, M)
    b.op("neq", out("a_neMM", "int"), M, M)
    b.op("eq", out("a_eqMI", "int"), M, Id)
    b.op("neq", out("a_neMI", "int"), M, Id)
    return b.text()


SHADER = build_shader()
NF = {"matrix": 16, "float": 1, "int": 1}
REC = sum(NF[t] for _, t in OUTS)


def group(ss):
    ss.renderer_matrix("shader", M_SHADER)
    ss.renderer_matrix("object", M_OBJECT)
    ss.LoadMemoryCompiledShader("matrix_suite", SHADER)
    g = ss.ShaderGroupBegin("matrix_suite_group")
    ss.Shader(g, "surface", "matrix_suite", "l1")
    ss.ShaderGroupEnd(g)
    locs, off = [], 0
    ty = {"matrix": og.TypeMatrix, "float": og.TypeFloat, "int": og.TypeInt}
    for name, t in OUTS:
        locs.append(og.SymLocationDesc("l1." + name, ty[t], False, og.SymArenaOutputs, off, 4 * REC))
        off += 4 * NF[t]
    ss.add_symlocs(g, locs)
    return g


def columns(rec):
    """{output name: float32 values, or int for int outputs} of one point."""
    d, k = {}, 0
    for name, t in OUTS:
        w = rec[k:k + NF[t]]
        d[name] = int(w.view(np.int32)[0]) if t == "int" else w.view(np.float32)
        k += NF[t]
    return d


def pretty(x):
    x = np.asarray(x, np.float32).copy()
    x[np.abs(x) < 5e-6] = 0.0
    return x + np.float32(0.0)  # -0 -> +0


def g5(x):
    return " ".join("%.5g" % float(e) for e in np.atleast_1d(x))


def printed(d, u, v):
    """The lines the reference shader prints for one point, rebuilt from
    the group's outputs with the shader's own format strings."""
    P = lambda n: g5(pretty(d[n]))
    vals = " ".join([])  # noqa: F841
    c16 = "0.1, 0.2, 0.3, 0.4,  0.5, 0.6, 0.7, 0.8,  0.9, 1, 1.1, 1.2,  1.3, 1.4, 1.5, 1.6"
    c16v = "%.5g, %.5g, 0.3, 0.4,  0.5, 0.6, 0.7, 0.8,  0.9, 1, 1.1, 1.2,  1.3, 1.4, 1.5, 1.6" % (u, v)
    L = ["  matrix (0.1) = " + g5(d["m_a"]),
         "  matrix (%s) \n\t= %s" % (c16, g5(d["m_16"])),
         " varying:",
         "  matrix (%.5g) = %s" % (u, g5(d["m_av"])),
         "  matrix (%s) \n\t= %s" % (c16v, g5(d["m_16v"])),
         "",
         "testing with spaces:",
         '  matrix ("shader", 1) = ' + P("s_a"),
         '  matrix ("shader", 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1) \n\t= ' + P("s_16"),
         " varying:",
         '  matrix ("shader", %.5g) = %s' % (u, P("s_av")),
         '  matrix ("shader", %.5g, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1) \n\t= %s' % (u, P("s_16v")),
         '  matrix ("world", 1) = ' + "%s" % " ".join("%g" % x for x in d["m_world"]),
         '  matrix ("common", 1) = ' + "%s" % " ".join("%g" % x for x in d["m_common"]),
         "",
         "Testing matrix from-to construction:"]
    for fr, to in (("common", "shader"), ("common", "object"), ("shader", "object")):
        for x, y in ((fr, to), (to, fr)):
            tag = x[0] + y[0]
            L.append('  matrix ("%s", "%s") = (%s)' % (x, y, P("ft_" + tag)))
            if d["ok_" + tag] != 1:
                L.append("  Hey, matrix ctr didn't match getmatrix!")
    L += ["", "Testing getmatrix for unknown space name:",
          "  found???" if d["found_foobar"] else "  'foobar' matrix not found, as expected",
          "", "", "Testing matrix component access:",
          "  M = " + g5(d["c_M"]),
          "  M[1][0..3] = " + " ".join("%.5g" % d["c_m1%d" % j][0] for j in range(4)),
          "  after M[1][3] = 5, M = " + P("c_set5"),
          " varying:",
          "  after M[1][2] = %.5g, M = %s" % (d["c_6u"][0], P("c_set6u")),
          "", "", "Testing matrix math:",
          "  M = [%s]" % P("c_M"), "  -M = [%s]" % P("a_neg"), "  2*M = [%s]" % P("a_2M"),
          "  M*2 = [%s]" % P("a_M2"), "  M/2 = [%s]" % P("a_Md2"), "  M*Ident = [%s]" % P("a_MI"),
          "  Ident*M = [%s]" % P("a_IM"), "  M*M = [%s]" % P("a_MM"), "  M/M = [%s]" % P("a_MdM"),
          "  M/Ident = [%s]" % P("a_MdI"), "  Ident/M = [%s]" % P("a_IdM"), "  1/M = [%s]" % P("a_1dM"),
          "  transpose(M) = " + P("a_T"), "  determinant(M) = " + P("a_det"),
          "  (M==M) ? %d" % d["a_eqMM"], "  (M!=M) ? %d" % d["a_neMM"],
          "  (M==Ident) ? %d" % d["a_eqMI"], "  (M!=Ident) ? %d" % d["a_neMI"]]
    return "\n".join(L)


def reference_blocks():
    """Each point's printed text from the matrix constructors on (the
    parameter block and the renderer's error line are left out)."""
    text = open(os.path.join(GOLDEN, "matrix_out.txt")).read()
    blocks = text.split("Parameter initialization:\n")[1:]
    out = []
    for blk in blocks:
        lines = [ln for ln in blk.split("\n") if not ln.startswith("ERROR:")]
        start = next(i for i, ln in enumerate(lines) if ln.startswith("  matrix (0.1) ="))
        out.append("\n".join(lines[start:]).rstrip("\n"))
    return out


def run_oracle(g):
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, REC), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    return out.view(np.uint32), u, v


def test_oracle_prints_the_reference_matrices():
    g = group(og.ShadingSystem())
    rec, u, v = run_oracle(g)
    ref = reference_blocks()
    assert len(ref) == W * H
    for p in range(W * H):
        got = printed(columns(rec[p]), float(u[p]), float(v[p]))
        if got != ref[p]:
            gl, rl = got.split("\n"), ref[p].split("\n")
            diff = [(a, b) for a, b in zip(gl, rl) if a != b][:5]
            pytest.fail("point %d differs from the reference (got, reference): %s" % (p, diff))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_matrices_equal_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = group(ss)
    u, v = pixel_grid(W, H)
    du, dv = torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda()
    out = torch.zeros(W * H * REC, dtype=torch.int32, device="cuda")
    ss.execute_batch(g, W * H, grid_globals(du, dv, W, H), 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    got = out.cpu().numpy().view(np.uint32).reshape(W * H, REC)
    ref, _, _ = run_oracle(g)
    assert np.array_equal(got.view(np.float32) == got.view(np.float32), ref.view(np.float32) == ref.view(np.float32))
    assert np.array_equal(got, ref)
