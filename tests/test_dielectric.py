"""BSDL dielectric_bsdf (libbsdl MTX/bsdf_dielectric_impl.h, as testrender
wraps it with BSDL_WRAP, src/testrender/shading.cpp:73-115).

The lobe renormalizes its sampled weight by the energy it misses, read from
tables baked at build time (BSDL genluts' method, src/libbsdl/src/
genluts.cpp). Two furnace properties pin lobe and tables together on the
oracle:
  * a white dielectric (reflection and transmission tints 1) keeps all the
    energy: the mean sampled weight is 1, seen from outside (front table)
    and from inside (back table);
  * layer(reflection-only white dielectric, white diffuse) is white: the
    base receives what the coating's tabulated energy says the coating does
    not reflect (evaluate_layer_opacity, shading.cpp:1242-1248), so the
    material's total albedo is 1.
The "absorption" keyword scales the coating's opacity and so darkens the
layer. On the GPU, the interpreter and the specialized kernel give the
oracle's samples bit for bit (pool nodes for the layer, static nodes for a
plain sum)."""
import numpy as np
import pytest

from helpers import og, oracle_run
from openshadinglanguage_gb300 import workloads as W
from openshadinglanguage_gb300.oso import OsoBuilder

NPTS = 1 << 15


def dielectric_group(ss, name, refl, refr, alpha, ior, base=None, absorption=None, aniso=0.0):
    """Ci = dielectric_bsdf(N, dPdu, refl, refr, alpha * (1 - aniso), alpha, ior, "ggx"),
    layered over diffuse(N) * base when base is given."""
    b = OsoBuilder(name, "surface")
    Ci = b.glob("closure color", "Ci")
    N, dPdu = b.glob("normal", "N"), b.glob("vector", "dPdu")
    c = lambda x: b.const("float", float(np.float32(x)))
    args = [N, dPdu, b.const("color", list(refl)), b.const("color", list(refr)), c(alpha * (1.0 - aniso)), c(alpha),
            c(ior), b.const("string", "ggx")]
    if absorption is not None:
        args += [b.const("string", "absorption"), b.const("color", list(absorption))]
    top = b.tmp("closure color")
    b.op("closure", top, b.const("string", "dielectric_bsdf"), *args)
    if base is None:
        b.op("assign", Ci, top)
    else:
        d, dw = b.tmp("closure color"), b.tmp("closure color")
        b.op("closure", d, b.const("string", "diffuse"), N)
        b.op("mul", dw, d, b.const("color", list(base)))
        b.op("closure", Ci, b.const("string", "layer"), top, dw)
    ss.LoadMemoryCompiledShader(name, b.text())
    g = ss.ShaderGroupBegin(name + "_g")
    ss.Shader(g, "surface", name, "S")
    ss.ShaderGroupEnd(g)
    ss.bsdf_sample_output(g, "S.Ci", 0, 4 * W.C5_OUT_FLOATS, 0, 4 * W.C5_IN_FLOATS)
    return g


def fixed_view(n, cos_theta, backfacing, seed=7):
    """n samples of one view: N = +z (the facing normal, as a renderer
    passes it), wo at angle acos(cos_theta) from N; uniform random numbers."""
    rng = np.random.default_rng(seed)
    st = np.sqrt(1.0 - cos_theta * cos_theta)
    wo = np.array([st, 0.0, cos_theta], np.float32)
    P = np.zeros((3, n), np.float32)
    N = np.tile(np.array([[0.0], [0.0], [1.0]], np.float32), (1, n))
    T = np.tile(np.array([[1.0], [0.0], [0.0]], np.float32), (1, n))
    I = np.tile(-wo[:, None], (1, n)).astype(np.float32)
    rnd = np.zeros((n, W.C5_IN_FLOATS), np.float32)
    rnd[:, 0:3] = rng.random((n, 3), dtype=np.float32)
    rnd[:, 3:6] = 1.0    # path weight
    rnd[:, 6] = 0.0      # no absorption (the lobe is always chosen)
    rnd[:, 7] = 0.0      # ray roughness
    rnd[:, 8] = 1.0 if backfacing else 0.0
    return P, N, I, T, rnd


def sample_oracle(g, view):
    P, N, I, T, rnd = view
    out = np.zeros((P.shape[1], W.C5_OUT_FLOATS), np.float32)
    st = oracle_run(g.program_bytes(), P.shape[1], og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T), out, userdata=rnd)
    assert st == 0
    assert np.all(np.isfinite(out))
    return out


CASES = [(0.05, 1.5, 0.9), (0.2, 1.33, 0.5), (0.45, 1.7, 0.7), (0.3, 2.4, 0.3), (0.12, 1.45, 0.15)]


@pytest.mark.parametrize("alpha,ior,cos_theta", CASES)
@pytest.mark.parametrize("backfacing", [0, 1])
def test_white_dielectric_keeps_the_energy(alpha, ior, cos_theta, backfacing):
    ss = og.ShadingSystem()
    g = dielectric_group(ss, "diel_white", (1, 1, 1), (1, 1, 1), alpha, ior)
    out = sample_oracle(g, fixed_view(NPTS, cos_theta, backfacing))
    w = out[:, 3:6]
    assert np.array_equal(w[:, 0], w[:, 1]) and np.array_equal(w[:, 0], w[:, 2])
    up = out[:, 2] > 0
    assert 0.0 < up.mean() < 1.0  # both reflection and refraction are sampled
    assert abs(w[:, 0].mean() - 1.0) < 0.03, w[:, 0].mean()
    rough = out[out[:, 6] > 0, 10]
    assert np.all(rough > 0) and np.all(rough < 1)


@pytest.mark.parametrize("alpha,ior,cos_theta", CASES)
def test_coated_white_diffuse_is_white(alpha, ior, cos_theta):
    ss = og.ShadingSystem()
    g = dielectric_group(ss, "diel_coat", (1, 1, 1), (0, 0, 0), alpha, ior, base=(1, 1, 1))
    out = sample_oracle(g, fixed_view(NPTS, cos_theta, 0))
    assert np.all(out[out[:, 6] > 0, 2] > 0)  # reflection only
    assert abs(out[:, 3].mean() - 1.0) < 0.03, out[:, 3].mean()


def test_absorption_darkens_the_coated_base():
    ss = og.ShadingSystem()
    view = fixed_view(NPTS, 0.4, 0)
    plain = sample_oracle(dielectric_group(ss, "diel_a0", (1, 1, 1), (0, 0, 0), 0.3, 1.5, base=(1, 1, 1)), view)
    absorb = sample_oracle(dielectric_group(ss, "diel_a1", (1, 1, 1), (0, 0, 0), 0.3, 1.5, base=(1, 1, 1),
                                            absorption=(2.0, 0.5, 0.0)), view)
    m0, m1 = plain[:, 3:6].mean(0), absorb[:, 3:6].mean(0)
    assert m1[0] < m1[1] < m0[0] - 0.01
    assert abs(m1[2] - m0[2]) < 0.01  # no absorption in blue (lobe choice shifts a little)


def test_black_tints_give_nothing():
    ss = og.ShadingSystem()
    out = sample_oracle(dielectric_group(ss, "diel_black", (0, 0, 0), (0, 0, 0), 0.3, 1.5), fixed_view(256, 0.5, 0))
    assert np.all(out[:, 3:7] == 0)


def test_anisotropic_roughness_and_tangent():
    """rx != ry: the lobe is anisotropic along U (dPdu); swapping the two
    roughnesses mirrors the sampled directions between x and y."""
    ss = og.ShadingSystem()
    view = fixed_view(4096, 1.0, 0)
    a = sample_oracle(dielectric_group(ss, "diel_an", (1, 1, 1), (0, 0, 0), 0.5, 1.5, aniso=0.6), view)
    ok = a[:, 6] > 0
    sx, sy = np.abs(a[ok, 0]).mean(), np.abs(a[ok, 1]).mean()
    assert sx < 0.8 * sy


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_dielectric_samples_equal_the_oracle(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    rng = np.random.default_rng(3)
    n = 20011
    P, N, I, T, rnd = W.c5_hits(n)
    rnd[:, 8] = (rng.random(n) < 0.3).astype(np.float32)  # some back faces
    for name, kw in (("gd_white", dict(refl=(1, 1, 1), refr=(1, 1, 1), alpha=0.2, ior=1.5)),
                     ("gd_tint", dict(refl=(0.9, 0.5, 0.2), refr=(0.2, 0.7, 0.9), alpha=0.4, ior=1.33, aniso=0.5)),
                     ("gd_coat", dict(refl=(1, 1, 1), refr=(0, 0, 0), alpha=0.3, ior=1.6, base=(0.8, 0.4, 0.2),
                                      absorption=(0.5, 1.0, 0.0)))):
        g = dielectric_group(ss, name, **kw)
        want = sample_oracle(g, (P, N, I, T, rnd))
        dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        G = og.make_globals(P=dev(P), N=dev(N), Ng=dev(N), I=dev(I), dPdu=dev(T))
        out = torch.zeros(n * W.C5_OUT_FLOATS, dtype=torch.float32, device="cuda")
        ud = dev(rnd)
        ss.execute_batch(g, n, G, ud.data_ptr(), out.data_ptr(), sync=True)
        assert ss.device_status() == 0
        assert g.is_specialized() == bool(jit)
        got = out.cpu().numpy().reshape(n, W.C5_OUT_FLOATS)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name
