"""Matrix, derivative-measure and colour ops on the CPU oracle against
numpy: transpose, determinant, matrix division and inverse, point/vector/
normal transforms, area, filterwidth and luminance. Inverse-dependent
results follow the executor's own Gauss-Jordan inverse (Imath's code is
not in the reference tree), so they are compared with a tolerance."""
import numpy as np

from helpers import grid_globals, og, oracle_run, pixel_grid, shaders, single_layer_group

REC = 22  # det, Pt(3), Vt(3), Nt(3), area, fw, lum, rowT(3), rowD(3), rowI(3)


def mats(seed=5):
    rng = np.random.default_rng(seed)
    M = rng.uniform(-1, 1, (4, 4)).astype(np.float32) + 2.0 * np.eye(4, dtype=np.float32)
    M2 = rng.uniform(-1, 1, (4, 4)).astype(np.float32) + 2.0 * np.eye(4, dtype=np.float32)
    return M, M2


def matrix_group(ss):
    M, M2 = mats()
    names = [("det", og.TypeFloat, 1), ("Pt", og.TypePoint, 3), ("Vt", og.TypeVector, 3), ("Nt", og.TypeNormal, 3),
             ("area", og.TypeFloat, 1), ("fw", og.TypeFloat, 1), ("lum", og.TypeFloat, 1),
             ("rowT", og.TypeColor, 3), ("rowD", og.TypeColor, 3), ("rowI", og.TypeColor, 3)]
    locs, off = [], 0
    for n, t, k in names:
        locs.append(og.SymLocationDesc(n, t, False, og.SymArenaOutputs, 4 * off, 4 * REC))
        off += k
    g = single_layer_group(ss, "matrix_ops", shaders.matrix_ops(M.ravel(), M2.ravel()), outputs=locs)
    return g, M, M2


def inputs(W=32, H=32):
    u, v = pixel_grid(W, H, centers=True)
    P = np.stack([u * 3 - 1, v * 2 + 0.5, u * v + 1]).astype(np.float32)
    return u, v, P


def test_matrix_ops_on_oracle_match_numpy():
    ss = og.ShadingSystem()
    g, M, M2 = matrix_group(ss)
    W = H = 32
    u, v, P = inputs(W, H)
    out = np.zeros((W * H, REC), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P, centers=True), out) == 0
    for i in range(0, W * H, 37):
        Mv = (M * np.float32(1.0 + u[i])).astype(np.float64)
        p = P[:, i].astype(np.float64)
        assert np.isclose(out[i, 0], np.linalg.det(Mv), rtol=1e-4, atol=1e-5)
        h = np.append(p, 1.0) @ Mv
        np.testing.assert_allclose(out[i, 1:4], h[:3] / h[3], rtol=1e-4, atol=1e-5)
        np.testing.assert_allclose(out[i, 4:7], p @ Mv[:3, :3], rtol=1e-5, atol=1e-5)
        Ninv = np.linalg.inv(Mv).T
        np.testing.assert_allclose(out[i, 7:10], p @ Ninv[:3, :3], rtol=1e-4, atol=1e-5)
        # P has derivatives dPdx = (du, 0, 0), dPdy = (0, dv, 0) only through the globals
        np.testing.assert_allclose(out[i, 13:16], Mv.T[0, :3], rtol=1e-6)
        np.testing.assert_allclose(out[i, 16:19], (Mv @ np.linalg.inv(M2.astype(np.float64)))[0, :3], rtol=1e-4,
                                   atol=1e-5)
        np.testing.assert_allclose(out[i, 19:22], np.linalg.inv(Mv)[0, :3], rtol=1e-4, atol=1e-5)
        lum = p @ np.array([0.2126, 0.7152, 0.0722])
        assert abs(out[i, 12] - lum) < 1e-3 * max(1.0, abs(lum))
    # area(P) = |dPdx x dPdy| = du*dv and filterwidth(u) = du for the grid
    assert np.allclose(out[:, 10], (1.0 / W) * (1.0 / H), rtol=1e-6)
    assert np.allclose(out[:, 11], 1.0 / W, rtol=1e-6)


def test_singular_matrix_inverse_is_identity():
    ss = og.ShadingSystem()
    g = single_layer_group(ss, "matrix_ops", shaders.matrix_ops([0.0] * 16, [1.0 if i % 5 == 0 else 0.0 for i in range(16)]),
                           outputs=[og.SymLocationDesc("rowI", og.TypeColor, False, og.SymArenaOutputs, 0, 12)])
    W = H = 4
    u, v, P = inputs(W, H)
    out = np.zeros((W * H, 3), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, P=P, centers=True), out) == 0
    assert np.array_equal(out, np.tile(np.float32([1, 0, 0]), (W * H, 1)))
