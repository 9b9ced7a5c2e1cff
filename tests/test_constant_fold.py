"""Constant folding in the lowering (attribute opt_constant_fold, the
reference's RuntimeOptimizer folding): programs shrink, and the oracle gives
bit-identical outputs with and without it on the workload shaders and on a
probe with branches and loops (knowledge is dropped where a branch or a
loop writes)."""
import struct

import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid, shaders
from openshadinglanguage_gb300 import workloads


def nops(g):
    return struct.unpack("<I", g.program_bytes()[8:12])[0]


def probe_shader(name="fold_probe"):
    b = og.OsoBuilder(name)
    u = b.glob("float", "u")
    F = lambda v: b.const("float", v)
    I = lambda v: b.const("int", v)
    a, bb, d, e = b.local("float", "a"), b.local("float", "b"), b.local("float", "d"), b.local("float", "e")
    i, j, k, n = b.local("int", "i"), b.local("int", "j"), b.local("int", "k"), b.local("int", "n")
    cout = b.param("color", "Cout", 0.0, output=True)
    outs = [b.param("float", "d_out", 0.0, output=True), b.param("float", "e_out", 0.0, output=True),
            b.param("int", "j_out", 0, output=True), b.param("int", "k_out", 0, output=True),
            b.param("int", "eq_out", 0, output=True), b.param("float", "m_out", 0.0, output=True),
            b.param("float", "br_out", 0.0, output=True), b.param("float", "kept_out", 0.0, output=True)]
    b.op("assign", a, F(2.0))
    b.op("mul", bb, a, F(3.0))             # 6
    b.op("color", cout, bb, a, F(1.0))     # (6, 2, 1)
    b.op("assign", i, I(7))
    b.op("mul", j, i, I(3))                # 21
    b.op("div", k, j, I(4))                # 5
    b.op("eq", outs[4], j, I(21))          # 1
    cond = b.tmp("int")
    b.op("gt", cond, u, F(0.5))
    with b.if_(cond):
        b.op("assign", a, u)               # a unknown after the if
    b.op("add", d, a, bb)
    cnd = b.tmp("int")
    with b.loop("for", cnd) as lp:
        b.op("assign", n, I(0))
        lp.cond()
        b.op("lt", cnd, n, I(3))
        lp.body()
        b.op("add", bb, bb, F(1.0))        # b unknown inside and after the loop
        lp.step()
        b.op("add", n, n, I(1))
    b.op("mul", e, bb, F(2.0))             # 18
    m = b.tmp("float")
    b.op("div", m, F(1.0), F(0.0))         # OSL division by zero: 0
    b.op("assign", outs[5], m)
    for o, v in ((outs[0], d), (outs[1], e), (outs[2], j), (outs[3], k)):
        b.op("assign", o, v)
    # constant conditions: only the taken branch remains
    c1 = b.tmp("int")
    b.op("gt", c1, j, I(20))               # 1
    with b.if_(c1) as br:
        b.op("add", outs[6], d, F(10.0))
        br.else_()
        b.op("assign", outs[6], F(-1.0))
    c0 = b.tmp("int")
    b.op("lt", c0, e, F(0.0))              # e is only known after the loop: kept
    with b.if_(c0) as br:
        b.op("assign", outs[7], F(1.0))
        br.else_()
        b.op("assign", outs[7], F(2.0))
    return b.text()


def probe_group(ss):
    ss.LoadMemoryCompiledShader("fold_probe", probe_shader())
    g = ss.ShaderGroupBegin("gfold")
    ss.Shader(g, "surface", "fold_probe", "l1")
    ss.ShaderGroupEnd(g)
    names = [("Cout", og.TypeColor, 12), ("d_out", og.TypeFloat, 4), ("e_out", og.TypeFloat, 4),
             ("j_out", og.TypeInt, 4), ("k_out", og.TypeInt, 4), ("eq_out", og.TypeInt, 4),
             ("m_out", og.TypeFloat, 4), ("br_out", og.TypeFloat, 4), ("kept_out", og.TypeFloat, 4)]
    locs, off = [], 0
    for nm, ty, sz in names:
        locs.append(og.SymLocationDesc("l1." + nm, ty, False, og.SymArenaOutputs, off, 44))
        off += sz
    ss.add_symlocs(g, locs)
    return g


def run_grid(g, nfloats, W=24, H=10):
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, nfloats), np.float32)
    st = oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out)
    return u, out, st


def test_probe_folds_and_keeps_results():
    res = {}
    for fold in (0, 1):
        ss = og.ShadingSystem()
        ss.attribute("opt_constant_fold", fold)
        g = probe_group(ss)
        res[fold] = (nops(g),) + run_grid(g, 11)
        res[fold] += (g.program_bytes(),)
    assert res[1][0] < res[0][0]
    u, out, st = res[1][1:4]
    assert st == 0
    assert np.array_equal(out.view(np.uint32), res[0][2].view(np.uint32))
    ints = out.view(np.int32)
    assert np.all(out[:, 0:3] == np.float32([6, 2, 1]))
    a = np.where(u > 0.5, u, np.float32(2.0)).astype(np.float32)
    assert np.array_equal(out[:, 3], (a + np.float32(6)).astype(np.float32))
    assert np.all(out[:, 4] == 18.0)
    assert np.all(ints[:, 5] == 21) and np.all(ints[:, 6] == 5) and np.all(ints[:, 7] == 1)
    assert np.all(out[:, 8] == 0.0)
    assert np.array_equal(out[:, 9], (out[:, 3] + np.float32(10)).astype(np.float32))
    assert np.all(out[:, 10] == 2.0)
    # the constant-condition if is gone, the one on a loop result stays
    import re
    src = open(__file__.replace("test_constant_fold.py", "../openshadinglanguage_gb300/csrc/oslg_program.h")).read()
    body = src.split("enum OpCode : uint16_t {")[1].split("};")[0]
    names = []
    for nm in re.findall(r"\b(OP_[A-Z0-9_]+)\b", body):
        if nm not in names:
            names.append(nm)
    count_if = lambda blob: sum(1 for i in range(struct.unpack("<I", blob[8:12])[0])
                                if struct.unpack("<H", blob[64 + 32 * i:66 + 32 * i])[0] == names.index("OP_IF"))
    assert count_if(res[0][4]) == 3 and count_if(res[1][4]) == 2


def both(build, nfloats, n_runs=(0, 1), G=None, n=None, userdata=None):
    outs = []
    for fold in n_runs:
        ss = og.ShadingSystem()
        ss.attribute("opt_constant_fold", fold)
        g = build(ss)
        out = np.zeros((n, nfloats), np.float32)
        st = oracle_run(g.program_bytes(), n, G, out, userdata=userdata)
        outs.append((nops(g), out, st))
    return outs


def test_fbm_and_layered_closure_unchanged_by_folding():
    W = H = 32
    u, v = pixel_grid(W, H, centers=True)
    P = np.stack([u * np.float32(8), v * np.float32(8), np.zeros_like(u)]).astype(np.float32)

    def fbm(ss):
        ss.LoadMemoryCompiledShader("fbm_cell", shaders.fbm_cell())
        g = ss.ShaderGroupBegin("g")
        ss.Shader(g, "surface", "fbm_cell", "l1")
        ss.ShaderGroupEnd(g)
        ss.add_symlocs(g, [og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 0, 16),
                           og.SymLocationDesc("cellhash", og.TypeInt, False, og.SymArenaOutputs, 12, 16)])
        return g
    a, b = both(fbm, 4, G=grid_globals(u, v, W, H, P=P, centers=True), n=W * H)
    assert a[2] == b[2] == 0 and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))

    uu, vv, I = workloads.c2_inputs(W, H)
    G = workloads.c2_globals(og.make_globals, uu, vv, I)
    a, b = both(workloads.c2_group, 37, G=G, n=W * H)
    assert a[2] == b[2] == 0 and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


@pytest.mark.parametrize("part", range(4))
def test_random_groups_unchanged_by_folding(part):
    specs = workloads.c3_specs()
    for k, (name, oso, _npts, _t) in enumerate(specs):
        if k % 4 != part:
            continue
        P = workloads.c3_points(k, 256)
        G = og.make_globals(P=P)
        a, b = both(lambda ss: workloads.c3_group(ss, name, oso), workloads.C3_REC, G=G, n=256)
        assert a[2] == b[2]
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), name


def test_wavefront_materials_unchanged_by_folding():
    P, N, I, T, rnd = workloads.c5_hits(1024)
    G = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    shrunk = 0
    for k, spec in enumerate(workloads.c5_material_specs()):
        a, b = both(lambda ss: workloads.c5_material_group(ss, k, spec), workloads.C5_OUT_FLOATS, G=G,
                    n=P.shape[1], userdata=rnd)
        assert a[2] == b[2] == 0
        assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), k
        shrunk += a[0] - b[0]
    assert shrunk > 0
