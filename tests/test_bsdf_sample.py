"""The BSDF sample step (testrender's per-hit closure processing, prepare
and CompositeBSDF::sample) on the CPU oracle for the wavefront workload's
16 materials: finite results, unit directions, and the closed forms the
single-lobe cases must follow."""
import numpy as np
import pytest

from helpers import og, oracle_run
from openshadinglanguage_gb300 import shaders, workloads as W


def run_material(ss, k, spec, hits):
    P, N, I, T, rnd = hits
    g = W.c5_material_group(ss, k, spec)
    out = np.zeros((P.shape[1], W.C5_OUT_FLOATS), np.float32)
    st = oracle_run(g.program_bytes(), P.shape[1], og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T), out, userdata=rnd)
    return st, out


@pytest.fixture(scope="module")
def hits():
    return W.c5_hits(2048)


def test_all_materials_sample(hits):
    ss = og.ShadingSystem()
    for k, spec in enumerate(W.c5_material_specs()):
        st, out = run_material(ss, k, spec, hits)
        assert st == 0, k
        assert np.all(np.isfinite(out)), k
        ok = out[:, 6] > 0
        assert ok.mean() > 0.5, k
        wl = np.linalg.norm(out[ok, 0:3], axis=1)
        assert np.allclose(wl, 1.0, atol=1e-4), k
        emits = any(l[0] == "emission" for l in spec[2])
        assert (out[:, 7:10].max() > 0) == emits, k


def single_lobe_group(ss, name, lobe):
    oso = W._c5_surface(name, [lobe])
    ss.LoadMemoryCompiledShader(name, oso)
    g = ss.ShaderGroupBegin(name + "_g")
    ss.Shader(g, "surface", name, "S")
    ss.ShaderGroupEnd(g)
    ss.bsdf_sample_output(g, "S.Ci", 0, 4 * W.C5_OUT_FLOATS, 0, 4 * W.C5_IN_FLOATS)
    return g


@pytest.mark.parametrize("lobe", [("diffuse", 0.7, 0.0), ("oren_nayar", 0.7, 0.0)])
def test_lambertian_lobes_follow_cosine_sampling(hits, lobe):
    """diffuse, and oren_nayar with sigma 0 (A = 1, B = 0): weight = the
    closure weight, pdf = cos(N, wi) / pi, wi in the hemisphere of N."""
    P, N, I, T, rnd = hits
    rnd = rnd.copy()
    rnd[:, 6] = 0.0  # no absorption: the lobe is always chosen
    ss = og.ShadingSystem()
    g = single_lobe_group(ss, "lam_" + lobe[0], lobe)
    out = np.zeros((P.shape[1], W.C5_OUT_FLOATS), np.float32)
    assert oracle_run(g.program_bytes(), P.shape[1], og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T), out,
                      userdata=rnd) == 0
    wi = out[:, 0:3]
    cos = np.sum(wi * N.T, axis=1)
    assert np.all(cos >= -1e-6)
    assert np.allclose(out[:, 6], np.maximum(cos, 0) / np.pi, atol=2e-6)
    assert np.allclose(out[:, 3:6], 0.7, atol=1e-6)


def test_dielectric_reflects_and_refracts(hits):
    P, N, I, T, rnd = hits
    ss = og.ShadingSystem()
    g = single_lobe_group(ss, "diel", ("dielectric", 1.0, 1.5))
    out = np.zeros((P.shape[1], W.C5_OUT_FLOATS), np.float32)
    assert oracle_run(g.program_bytes(), P.shape[1], og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T), out,
                      userdata=rnd) == 0
    ok = out[:, 6] > 0
    side = np.sum(out[ok, 0:3] * N.T[ok], axis=1)
    assert (side > 0).mean() > 0.02 and (side < 0).mean() > 0.5


def test_sheen_lobe_samples_the_uniform_hemisphere(hits):
    """sheen_bsdf (Conty-Kulla mode): uniform hemisphere sampling, pdf
    1/(2 pi) for a lone lobe, directions above the surface, weight
    D*G2*pi/(2 cos_o) * tint * closure weight >= 0; nothing when the hit is
    backfacing (BSDL's rule) and roughness regularized by the ray's."""
    P, N, I, T, rnd = hits
    rnd = rnd.copy()
    rnd[:, 6] = 0.0
    ss = og.ShadingSystem()
    g = single_lobe_group(ss, "sheen_only", ("sheen", 0.7, 0.4))
    G = og.make_globals(P=P, N=N, Ng=N, I=I, dPdu=T)
    out = np.zeros((P.shape[1], W.C5_OUT_FLOATS), np.float32)
    assert oracle_run(g.program_bytes(), P.shape[1], G, out, userdata=rnd) == 0
    front = rnd[:, 8] == 0
    ok = front & (out[:, 6] > 0)
    assert ok.mean() > 0.5
    assert np.allclose(out[ok, 6], np.float32(0.5) * (np.float32(1) / np.float32(np.pi)))
    assert (np.einsum("ij,ji->i", out[ok, 0:3], N[:, ok]) > -1e-6).all()
    assert (out[ok, 3:6] >= 0).all()
    # reported roughness: 1 - (1 - 0.4) * (1 - ray roughness)
    expect = (np.float32(1) - (np.float32(1) - np.float32(0.4)) * (np.float32(1) - rnd[ok, 7])).astype(np.float32)
    assert np.array_equal(out[ok, 10], expect)
    assert (out[~front, 6] == 0).all() and (out[~front, 3:6] == 0).all()
