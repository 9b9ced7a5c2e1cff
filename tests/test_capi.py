"""C ABI boundary: the library loads, exports every entry point the header
declares, and reports failures as status codes with messages (host-side
failure injection; no GPU needed)."""
import ctypes
import os
import re

import pytest

from helpers import ROOT, og, shaders
from openshadinglanguage_gb300 import _capi


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "oslg.h")).read()
    return sorted(set(re.findall(r"\b(oslg_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(native):
    L = ctypes.CDLL(native)
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(L, s), s
    # and the Python binding covers the same set
    assert set(_capi.exported_symbols()) == set(syms)


def test_unknown_op_is_rejected_at_lowering(native):
    ss = og.ShadingSystem()
    b = og.OsoBuilder("bad")
    x = b.param("float", "x", 1.0, output=True)
    b.op("pointcloud_search", x, x)
    ss.LoadMemoryCompiledShader("bad", b.text())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "bad", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l1.x", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    with pytest.raises(og.OSLError, match="pointcloud_search"):
        ss.optimize_group(g)


def test_dead_ops_are_removed(native):
    """An op whose result nothing reads is dropped before lowering (the
    RuntimeOptimizer's dead-code removal): even an unsupported one."""
    import struct
    ss = og.ShadingSystem()
    ss.attribute("opt_constant_fold", 0)  # keep the add: x is a constant parameter
    b = og.OsoBuilder("deadops")
    x = b.param("float", "x", 1.0, output=True)
    y = b.param("float", "y", 0.0, output=True)
    t = b.tmp("float")
    b.op("pointcloud_search", t, x)  # result unused
    b.op("add", y, x, b.const("float", 2.0))
    b.op("mul", t, y, y)  # result unused
    ss.LoadMemoryCompiledShader("deadops", b.text())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "deadops", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l1.y", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    blob = g.program_bytes()  # lowering succeeds: the unsupported op was dead
    nops = struct.unpack("<I", blob[8:12])[0]
    codes = [struct.unpack("<H", blob[64 + 32 * i:66 + 32 * i])[0] for i in range(nops)]
    assert _opcode("OP_MUL") not in codes
    assert codes.count(_opcode("OP_ADD")) == 1
    # y's initial value, the add, the output store and the layer marker
    assert len(codes) <= 4


def test_malformed_oso_is_rejected(native):
    ss = og.ShadingSystem()
    with pytest.raises(og.OSLError, match="unknown symbol"):
        ss.LoadMemoryCompiledShader("m", "OpenShadingLanguage 1.00\nshader m\ncode ___main___\n\tadd a b c\n\tend\n")


def test_group_use_before_end_is_rejected(native):
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("fbm_cell", shaders.fbm_cell())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "fbm_cell", "l1")
    with pytest.raises(og.OSLError, match="ShaderGroupEnd"):
        ss.optimize_group(g)


def test_misaligned_symloc_is_rejected(native):
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("fbm_cell", shaders.fbm_cell())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "fbm_cell", "l1")
    ss.ShaderGroupEnd(g)
    with pytest.raises(og.OSLError, match="multiples of 4"):
        ss.add_symlocs(g, [og.SymLocationDesc("Cout", og.TypeColor, False, og.SymArenaOutputs, 2, 12)])


def test_unknown_parameter_and_connection_are_rejected(native):
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("getP", shaders.getP())
    ss.LoadMemoryCompiledShader("vadd", shaders.vadd())
    g = ss.ShaderGroupBegin("g")
    ss.Parameter(g, "nosuch", og.TypeFloat, 1.0)
    with pytest.raises(og.OSLError, match="no parameter"):
        ss.Shader(g, "surface", "getP", "l1")
    ss.Shader(g, "surface", "getP", "l1")
    ss.Shader(g, "surface", "vadd", "l2")
    with pytest.raises(og.OSLError, match="no input param"):
        ss.ConnectShaders(g, "l1", "out", "l2", "out")
    with pytest.raises(og.OSLError, match="precede"):
        ss.ConnectShaders(g, "l2", "out", "l1", "out")


def test_lowering_marks_derivatives_and_pools_constants(native):
    import numpy as np
    ss = og.ShadingSystem()
    ss.LoadMemoryCompiledShader("fbm_cell", shaders.fbm_cell())
    g = ss.ShaderGroupBegin("g")
    ss.Shader(g, "surface", "fbm_cell", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("Cout", og.TypeColor, True, og.SymArenaOutputs, 0, 40),
                       og.SymLocationDesc("cellhash", og.TypeInt, False, og.SymArenaOutputs, 36, 40)])
    blob = g.program_bytes()
    hdr = np.frombuffer(blob[:64], np.uint32)
    assert hdr[0] == 0x4F534C47
    assert hdr[5] & 2, "Cout requested with derivatives must make the program carry them"
    nops = int(hdr[2])
    ops = np.frombuffer(blob[64:64 + 32 * nops], np.uint32).reshape(nops, 8)
    codes = ops[:, 0] & 0xFFFF
    # the Perlin noise op computes Dual2 results (kind word bit 9); the cell
    # noise lookup never carries derivatives
    noise_rows = [r for r in ops if (r[0] & 0xFFFF) == _opcode("OP_NOISE")]
    perlin = [r for r in noise_rows if (r[4] & 15) == 0]
    cell = [r for r in noise_rows if (r[4] & 15) == 2]
    assert perlin and all(r[4] & 512 for r in perlin)
    assert cell and not any(r[4] & 512 for r in cell)
    assert len(codes) == nops


def _opcode(name):
    src = open(os.path.join(ROOT, "openshadinglanguage_gb300", "csrc", "oslg_program.h")).read()
    body = src.split("enum OpCode : uint16_t {")[1].split("};")[0]
    names = re.findall(r"\b(OP_[A-Z0-9_]+)\b", body)
    seen = []
    for n in names:
        if n not in seen:
            seen.append(n)
    return seen.index(name)
