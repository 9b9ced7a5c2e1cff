"""find_symbol / symbol_typedesc / symbol_address (src/include/OSL/
oslexec.h:950-971): a found symbol's final values of the last device
execution, as SoA planes. Checked on the CPU: lookup by layer, by
"layer.symbol", last layer first, refusals (unknown names, closures,
globals, no execution yet) and the type; on the GPU: the planes of a float,
a color, an int array element and a local equal what the same run wrote to
its output records, on the interpreter and the specialized kernel."""
import numpy as np
import pytest

from helpers import grid_globals, og, pixel_grid
from openshadinglanguage_gb300.oso import OsoBuilder


def symbol_group(ss):
    up = OsoBuilder("sym_up")
    a = up.param("float", "a", 0.0, output=True)
    k = up.param("int[2]", "k", [0, 0], output=True)
    up.op("mul", a, up.glob("float", "u"), up.const("float", 3.0))
    up.op("aassign", k, up.const("int", 1), up.const("int", 7))
    dn = OsoBuilder("sym_dn")
    x = dn.param("float", "x", 0.0)
    c = dn.param("color", "c", [0.0, 0.0, 0.0], output=True)
    t = dn.local("float", "t")
    dn.op("add", t, x, dn.glob("float", "v"))
    dn.op("color", c, t, x, dn.const("float", 0.5))
    dn.op("closure", dn.glob("closure color", "Ci"), dn.const("string", "diffuse"), dn.glob("normal", "N"))
    ss.LoadMemoryCompiledShader("sym_up", up.text())
    ss.LoadMemoryCompiledShader("sym_dn", dn.text())
    g = ss.ShaderGroupBegin("sym_g")
    ss.Shader(g, "surface", "sym_up", "U")
    ss.Shader(g, "surface", "sym_dn", "D")
    ss.ConnectShaders(g, "U", "a", "D", "x")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("U.a", og.TypeFloat, False, og.SymArenaOutputs, 0, 24),
                       og.SymLocationDesc("D.c", og.TypeColor, False, og.SymArenaOutputs, 4, 24),
                       og.SymLocationDesc("U.k", og.TypeInt.array(2), False, og.SymArenaOutputs, 16, 24)])
    return g


def test_find_symbol_lookup_and_refusals():
    ss = og.ShadingSystem()
    g = symbol_group(ss)
    ss.optimize_group(g)
    s1 = ss.find_symbol(g, "a", "U")
    assert ss.find_symbol(g, "U.a") == s1 and ss.find_symbol(g, "a") == s1
    assert ss.symbol_typedesc(s1) == og.TypeFloat
    assert ss.symbol_typedesc(ss.find_symbol(g, "c")) == og.TypeColor
    assert ss.symbol_typedesc(ss.find_symbol(g, "k", "U")) == og.TypeInt.array(2)
    for bad in (("nope", None), ("a", "D"), ("u", None)):
        with pytest.raises(og.OSLError):
            ss.find_symbol(g, *bad)
    with pytest.raises(og.OSLError, match="execute the group"):
        ss.symbol_address(g, s1)
    # the group lowers again with the retained symbols' stores
    assert len(g.program_bytes()) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("jit", [0, 1])
def test_gpu_symbol_address_holds_the_final_values(jit):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ss = og.ShadingSystem()
    if jit:
        ss.attribute("jit", 1)
    g = symbol_group(ss)
    syms = {n: ss.find_symbol(g, n) for n in ("a", "c", "k", "t")}
    W, H = 97, 31
    n = W * H
    u, v = pixel_grid(W, H)
    G = grid_globals(torch.from_numpy(u).cuda(), torch.from_numpy(v).cuda(), W, H)
    out = torch.zeros(n * 6, dtype=torch.float32, device="cuda")
    ss.execute_batch(g, n, G, 0, out.data_ptr(), sync=True)
    assert g.is_specialized() == bool(jit)
    rec = out.cpu().numpy().reshape(n, 6)
    view = {k: torch.as_tensor(ss.symbol_array(g, s, n), device="cuda").cpu().numpy() for k, s in syms.items()}
    assert np.array_equal(view["a"][0], rec[:, 0])
    assert np.array_equal(view["c"].T, rec[:, 1:4])
    assert np.array_equal(view["k"].T, rec[:, 4:6].view(np.int32)) and np.all(view["k"][1] == 7)
    assert np.array_equal(view["t"][0], (rec[:, 0] + v).astype(np.float32))
