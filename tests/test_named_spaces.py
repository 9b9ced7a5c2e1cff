"""Named coordinate systems (transform/transformv/transformn with space
names, matrix(from, to), matrix(space, f), getmatrix) against registered
renderer matrices, through the lowering and the oracle, checked against
numpy statements of osl_transform_triple / osl_get_from_to_matrix
(src/liboslexec/opmatrix.cpp:141-300): points as row vectors with the
homogeneous divide, vectors by the upper 3x3, normals by the inverse
transpose; "common"/"world" the identity; unknown spaces copy the input and
make getmatrix return 0."""
import numpy as np

from helpers import og, oracle_run

M_OBJECT = np.array([[0.8, 0.3, -0.2, 0.0], [-0.25, 0.9, 0.1, 0.0], [0.15, -0.05, 1.2, 0.0],
                     [1.5, -2.0, 0.5, 1.0]], np.float32)
M_CAMERA = np.array([[1.1, 0.0, 0.2, 0.01], [0.1, 0.95, 0.0, 0.0], [0.0, -0.3, 1.05, 0.02],
                     [-0.5, 0.25, 3.0, 1.0]], np.float32)

OUT = [("p_obj", og.TypePoint), ("p_w", og.TypePoint), ("v_cam", og.TypeVector), ("n_obj", og.TypeNormal),
       ("p_same", og.TypePoint), ("p_unk", og.TypePoint), ("Mo", og.TypeMatrix), ("Ms", og.TypeMatrix),
       ("Mg", og.TypeMatrix), ("r_ok", og.TypeInt), ("r_bad", og.TypeInt)]
SIZES = {"point": 3, "vector": 3, "normal": 3, "matrix": 16, "int": 1}
NFLOATS = 6 * 3 + 3 * 16 + 2


def spaces_shader(name="spaces"):
    b = og.OsoBuilder(name)
    P, N, T = b.glob("point", "P"), b.glob("normal", "N"), b.glob("vector", "dPdu")
    o = {nm: b.param({og.TypePoint: "point", og.TypeVector: "vector", og.TypeNormal: "normal",
                      og.TypeMatrix: "matrix", og.TypeInt: "int"}[ty], nm, 0, output=True) for nm, ty in OUT}
    S = lambda s: b.const("string", s)
    b.op("transform", o["p_obj"], S("object"), P)
    b.op("transform", o["p_w"], S("object"), S("world"), P)
    b.op("transformv", o["v_cam"], S("camera"), T)
    b.op("transformn", o["n_obj"], S("object"), S("camera"), N)
    b.op("transform", o["p_same"], S("camera"), S("camera"), P)
    b.op("transform", o["p_unk"], S("nowhere"), P)
    b.op("matrix", o["Mo"], S("object"), S("camera"))
    b.op("matrix", o["Ms"], S("object"), b.const("float", 2.0))
    b.op("getmatrix", o["r_ok"], S("object"), S("world"), o["Mg"])
    m = b.tmp("matrix")
    b.op("getmatrix", o["r_bad"], S("nowhere"), S("world"), m)
    return b.text()


def spaces_group(ss, tag=""):
    ss.renderer_matrix("object", M_OBJECT)
    ss.renderer_matrix("camera", M_CAMERA)
    ss.LoadMemoryCompiledShader("spaces" + tag, spaces_shader("spaces" + tag))
    g = ss.ShaderGroupBegin("gsp" + tag)
    ss.Shader(g, "surface", "spaces" + tag, "l1")
    ss.ShaderGroupEnd(g)
    locs, off = [], 0
    for nm, ty in OUT:
        locs.append(og.SymLocationDesc("l1." + nm, ty, False, og.SymArenaOutputs, off, 4 * NFLOATS))
        off += 4 * (16 if ty == og.TypeMatrix else 1 if ty == og.TypeInt else 3)
    ss.add_symlocs(g, locs)
    return g


def inputs(n, seed=11):
    rng = np.random.default_rng(seed)
    P = rng.uniform(-3, 3, (3, n)).astype(np.float32)
    N = rng.normal(size=(3, n)).astype(np.float32)
    T = rng.normal(size=(3, n)).astype(np.float32)
    return P, N, T


def xform_point(M, p):
    h = np.concatenate([p.T.astype(np.float64), np.ones((p.shape[1], 1))], 1) @ M.astype(np.float64)
    return h[:, :3] / h[:, 3:4]


def check(out, P, N, T):
    Mo, Mc = M_OBJECT.astype(np.float64), M_CAMERA.astype(np.float64)
    close = lambda a, b: np.allclose(a, b, rtol=2e-5, atol=2e-5)
    assert close(out[:, 0:3], xform_point(np.linalg.inv(Mo), P))
    assert close(out[:, 3:6], xform_point(Mo, P))
    assert close(out[:, 6:9], T.T @ np.linalg.inv(Mc)[:3, :3])
    from_to = Mo @ np.linalg.inv(Mc)
    assert close(out[:, 9:12], N.T @ np.linalg.inv(from_to).T[:3, :3])
    assert np.array_equal(out[:, 12:15], P.T) and np.array_equal(out[:, 15:18], P.T)
    assert close(out[:, 18:34], np.broadcast_to(from_to.reshape(16), (len(out), 16)))
    assert close(out[:, 34:50], np.broadcast_to((Mo @ np.diag([2.0, 2, 2, 2])).reshape(16), (len(out), 16)))
    assert np.array_equal(out[:, 50:66], np.broadcast_to(M_OBJECT.reshape(16), (len(out), 16)))
    ints = out.view(np.int32)
    assert np.all(ints[:, 66] == 1) and np.all(ints[:, 67] == 0)


def test_named_spaces_match_numpy():
    ss = og.ShadingSystem()
    g = spaces_group(ss)
    n = 300
    P, N, T = inputs(n)
    out = np.zeros((n, NFLOATS), np.float32)
    assert oracle_run(g.program_bytes(), n, og.make_globals(P=P, N=N, dPdu=T), out) == 0
    check(out, P, N, T)


def test_space_names_must_be_constant():
    ss = og.ShadingSystem()
    b = og.OsoBuilder("spvar")
    u = b.glob("float", "u")
    P = b.glob("point", "P")
    sp = b.tmp("string")
    b.op("assign", sp, b.const("string", "object"))
    c = b.tmp("int")
    b.op("gt", c, u, b.const("float", 0.5))
    with b.if_(c):
        b.op("assign", sp, b.const("string", "camera"))
    o = b.param("point", "o", 0, output=True)
    b.op("transform", o, sp, P)
    ss.LoadMemoryCompiledShader("spvar", b.text())
    g = ss.ShaderGroupBegin("gspv")
    ss.Shader(g, "surface", "spvar", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l1.o", og.TypePoint, False, og.SymArenaOutputs, 0, 12)])
    import pytest
    with pytest.raises(og.OSLError, match="constant strings"):
        g.program_bytes()
