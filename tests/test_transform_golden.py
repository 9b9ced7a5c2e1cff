"""Point, vector and normal transforms pinned to the reference testsuite's
`transform` shader output (testsuite/transform/test.osl, expected text
ref/out.txt copied to tests/golden/transform_out.txt by make_golden.py).

The shader transforms a constant point, the origin, and the point plus
(u, v, 0) (with derivatives) into "shader" space, between "common" and
"shader" both ways and from "shader" to "object", as point, vector and
normal, and prints each result (%.5g, through the testsuite's pretty() for
the from/to forms) and the derivatives (%g). Here every printed value is an
output of the group; the test rebuilds the whole printed text of the
`-g 2 2` run from the outputs with the shader's format strings and compares
it with the reference's text. The spaces are testshade's (see
test_matrix_golden)."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, grid_globals, og, oracle_run, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder
from test_matrix_golden import M_OBJECT, M_SHADER, g5, pretty

W = H = 2
# (label point, from, to): "to" alone is transform(to, p) (from "common")
CALLS = [("p", None, "shader"), ("z", None, "shader"), ("p", "common", "shader"), ("z", "common", "shader"),
         ("p", "shader", "common"), ("z", "shader", "common"), ("p", "shader", "object"), ("z", "shader", "object")]
KINDS = ("point", "vector", "normal")
OUTS = []  # (name, floats)


def build_shader():
    b = OsoBuilder("transform_suite")
    u, v = b.glob("float", "u"), b.glob("float", "v")
    S = lambda s: b.const("string", s)

    def out(name, t, derivs=False):
        OUTS.append((name, t, derivs))
        return b.param(t, name, 0, output=True)

    z = b.local("point", "z")
    b.op("assign", z, b.const("point", [0, 0, 0]))
    for ps in (0, 1):
        p = b.local("point", "p%d" % ps)
        b.op("assign", p, b.const("point", [1, 1.41421, 0]))
        if ps:
            uv = b.tmp("vector")
            b.op("vector", uv, u, v, b.const("float", 0.0))
            b.op("add", p, p, uv)
        b.op("assign", out("p_%d" % ps, "point", True), p)
        for ci, (which, fr, to) in enumerate(CALLS):
            src = p if which == "p" else z
            for kind in KINDS:
                cast = b.tmp(kind)
                b.op("assign", cast, src)
                r = out("t_%d_%d_%s" % (ps, ci, kind), kind, ci == 0 and kind != "normal")
                opname = {"point": "transform", "vector": "transformv", "normal": "transformn"}[kind]
                if fr is None:
                    b.op(opname, r, S(to), cast)
                else:
                    b.op(opname, r, S(fr), S(to), cast)
    return b.text()


SHADER = build_shader()
TY = {"point": og.TypePoint, "vector": og.TypeVector, "normal": og.TypeNormal}


def nfloats(t, derivs):
    return 3 * (3 if derivs else 1)


REC = sum(nfloats(t, d) for _, t, d in OUTS)


def group(ss):
    ss.renderer_matrix("shader", M_SHADER)
    ss.renderer_matrix("object", M_OBJECT)
    ss.LoadMemoryCompiledShader("transform_suite", SHADER)
    g = ss.ShaderGroupBegin("transform_suite_group")
    ss.Shader(g, "surface", "transform_suite", "l1")
    ss.ShaderGroupEnd(g)
    locs, off = [], 0
    for name, t, d in OUTS:
        locs.append(og.SymLocationDesc("l1." + name, TY[t], d, og.SymArenaOutputs, off, 4 * REC))
        off += 4 * nfloats(t, d)
    ss.add_symlocs(g, locs)
    return g


def columns(rec):
    d, k = {}, 0
    for name, t, dv in OUTS:
        n = nfloats(t, dv)
        d[name] = rec[k:k + n].view(np.float32).reshape(-1, 3)
        k += n
    return d


def gg(x):
    return " ".join("%g" % float(e) for e in x)


def printed(d):
    L = []
    for ps in (0, 1):
        pv = d["p_%d" % ps]
        for ci, (which, fr, to) in enumerate(CALLS):
            pts = gg(pv[0]) if which == "p" else "0 0 0"
            r = {k: d["t_%d_%d_%s" % (ps, ci, k)] for k in KINDS}
            if fr is None:
                L += ["", "transform to '%s':" % to]
                if ci == 0:
                    L.append("  p = %s, Dx(p) = %s, Dy(p) = %s" % (gg(pv[0]), gg(pv[1]), g5(pv[2])))
                for k in KINDS:
                    L.append(' transform("%s", %s(%s)) = %s' % (to, k, pts, g5(r[k][0])))
                    if ci == 0 and k != "normal":
                        L.append('  derivs of transform("%s", %s(%s)): Dx = %s, Dy = %s'
                                 % (to, k, pts, gg(r[k][1]), gg(r[k][2])))
            else:
                L += ["", "transform '%s' to '%s':" % (fr, to)]
                for k in KINDS:
                    L.append(' transform("%s", "%s", %s(%s)) = %s' % (fr, to, k, pts, g5(pretty(r[k][0]))))
        if ps == 0:
            L += ["", "", " varying:", ""]
    return "\n".join(L) + "\n"


def run_oracle(g):
    u, v = pixel_grid(W, H)
    out = np.zeros((W * H, REC), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H), out) == 0
    return out.view(np.uint32)


def test_oracle_prints_the_reference_transforms():
    g = group(og.ShadingSystem())
    rec = run_oracle(g)
    got = "".join(printed(columns(rec[p])) for p in range(W * H))
    ref = open(os.path.join(GOLDEN, "transform_out.txt")).read().split("\n", 1)[1]
    got, ref = got.rstrip("\n"), ref.rstrip("\n")  # the file ends with an extra newline
    if got != ref:
        gl, rl = got.split("\n"), ref.split("\n")
        diff = [(i, a, b) for i, (a, b) in enumerate(zip(gl, rl)) if a != b][:6]
        pytest.fail("differs from the reference (line, got, reference): %s; %d vs %d lines"
                    % (diff, len(gl), len(rl)))


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_transforms_equal_the_oracle(jit):
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
    assert np.array_equal(got, run_oracle(g))
