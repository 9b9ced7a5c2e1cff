"""execute_layer: the program that runs a group's layers up to a named
layer (BatchedExecutor::execute_init + execute_layer, oslexec.h:1006-1027)
stores exactly the outputs those layers write, with the same values as the
whole group; later layers' outputs are left untouched."""
import numpy as np
import pytest

from helpers import og, oracle_run
from openshadinglanguage_gb300 import workloads


def test_layer_programs_match_the_whole_group():
    W = H = 24
    u, v, I = workloads.c2_inputs(W, H)
    G = workloads.c2_globals(og.make_globals, u, v, I)
    n = W * H
    full = np.zeros((n, 41), np.float32)
    g = c2_full(og.ShadingSystem())
    assert oracle_run(g.program_bytes(), n, G, full) == 0
    for layer, cols in (("A", [37]), ("B", [37, 38, 39, 40])):
        part = np.full((n, 41), -9.0, np.float32)
        assert oracle_run(g.layer_program_bytes(layer), n, G, part) == 0
        assert np.array_equal(part[:, cols].view(np.uint32), full[:, cols].view(np.uint32))
        untouched = [c for c in range(41) if c not in cols]
        assert np.all(part[:, untouched] == -9.0), layer
    assert g.layer_program_bytes("C") == g.program_bytes()


def c2_full(ss):
    """The C2 group with 164-byte records: closure records and the BSDF
    eval as in C2 (bytes 0..147), then A.a and B.Cout."""
    from openshadinglanguage_gb300 import shaders
    from openshadinglanguage_gb300._capi import AGG_VEC3, BASE_FLOAT, VEC_COLOR
    from openshadinglanguage_gb300.shadingsys import TypeDesc
    ss.LoadMemoryCompiledShader("c2_pattern", shaders.c2_pattern())
    ss.LoadMemoryCompiledShader("c2_ramp", shaders.c2_ramp())
    ss.LoadMemoryCompiledShader("c2_surface", shaders.c2_surface())
    g = ss.ShaderGroupBegin("layered_closure_l")
    ss.Shader(g, "surface", "c2_pattern", "A")
    ss.Parameter(g, "knots", TypeDesc(BASE_FLOAT, AGG_VEC3, VEC_COLOR, 8), shaders.c2_knots())
    ss.Shader(g, "surface", "c2_ramp", "B")
    ss.ConnectShaders(g, "A", "a", "B", "x")
    ss.Shader(g, "surface", "c2_surface", "C")
    ss.ConnectShaders(g, "A", "a", "C", "a")
    ss.ConnectShaders(g, "B", "Cout", "C", "tint")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("C.Ci", og.TypeClosure.array(2), False, og.SymArenaOutputs, 0, 164),
                       og.SymLocationDesc("A.a", og.TypeFloat, False, og.SymArenaOutputs, 148, 164),
                       og.SymLocationDesc("B.Cout", og.TypeColor, False, og.SymArenaOutputs, 152, 164)])
    ss.bsdf_eval_output(g, "C.Ci", workloads.C2_LIGHT, 132, 164)
    return g


@pytest.mark.gpu
def test_gpu_execute_layer_matches_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from test_gpu_parity import dev
    W = H = 200
    u, v, I = workloads.c2_inputs(W, H)
    n = W * H
    ss = og.ShadingSystem()
    g = c2_full(ss)
    du, dv, dI = dev(u), dev(v), dev(I)
    Gd = workloads.c2_globals(og.make_globals, du, dv, dI)
    for layer in ("A", "B", "C"):
        out = torch.full((n * 41,), -9.0, dtype=torch.float32, device="cuda")
        ss.execute_layer(g, layer, n, Gd, 0, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        ref = np.full((n, 41), -9.0, np.float32)
        prog = g.layer_program_bytes(layer) if layer != "C" else g.program_bytes()
        assert oracle_run(prog, n, workloads.c2_globals(og.make_globals, u, v, I), ref) == 0
        got = out.cpu().numpy().reshape(n, 41)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), layer
    assert ss.device_status() == 0

