"""The benchmark workloads: shader groups and seeded synthetic inputs.

C1  fbm_cell        single-layer fBm + hashed cell id, 1024x1024 grid
C2  layered_closure 3-layer pattern -> ramp -> closure group with BSDF eval,
                    2048x2048 grid
"""
import numpy as np

from . import shaders
from .shadingsys import (SymArenaOutputs, SymLocationDesc, TypeClosure, TypeColor, TypeInt, TypeDesc)
from ._capi import BASE_FLOAT, AGG_VEC3, VEC_COLOR

# ---- C2 ------------------------------------------------------------------------------
C2_CLOSURE_RECORDS = 2                       # components kept per point
C2_CLOSURE_BYTES = 4 + 64 * C2_CLOSURE_RECORDS  # [count][id, w.rgb, params x12] ...
C2_EVAL_OFFSET = C2_CLOSURE_BYTES
C2_STRIDE = C2_CLOSURE_BYTES + 16             # + {w.rgb, pdf}
C2_LIGHT = (0.5773502691896258, 0.5773502691896258, 0.5773502691896258)


def c2_group(ss):
    """Layer A c2_pattern -> layer B c2_ramp (x <- A.a) -> layer C c2_surface
    (a <- A.a, tint <- B.Cout); Ci stored as closure records and evaluated
    as a BSDF at the fixed light direction normalize(1,1,1)."""
    ss.LoadMemoryCompiledShader("c2_pattern", shaders.c2_pattern())
    ss.LoadMemoryCompiledShader("c2_ramp", shaders.c2_ramp())
    ss.LoadMemoryCompiledShader("c2_surface", shaders.c2_surface())
    g = ss.ShaderGroupBegin("layered_closure")
    ss.Shader(g, "surface", "c2_pattern", "A")
    ss.Parameter(g, "knots", TypeDesc(BASE_FLOAT, AGG_VEC3, VEC_COLOR, 8), shaders.c2_knots())
    ss.Shader(g, "surface", "c2_ramp", "B")
    ss.ConnectShaders(g, "A", "a", "B", "x")
    ss.Shader(g, "surface", "c2_surface", "C")
    ss.ConnectShaders(g, "A", "a", "C", "a")
    ss.ConnectShaders(g, "B", "Cout", "C", "tint")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [SymLocationDesc("C.Ci", TypeClosure.array(C2_CLOSURE_RECORDS), False, SymArenaOutputs, 0,
                                       C2_STRIDE)])
    ss.bsdf_eval_output(g, "C.Ci", C2_LIGHT, C2_EVAL_OFFSET, C2_STRIDE)
    return g


def c2_inputs(W, H, seed=0xC2):
    """u, v on testshade's default grid; I = -V with V uniform on the upper
    hemisphere (z = xi1, phi = 2*pi*xi2), so wo = -I faces the viewer."""
    x = np.arange(W, dtype=np.float32)
    y = np.arange(H, dtype=np.float32)
    u = (x / np.float32(max(1, W - 1))).astype(np.float32)
    v = (y / np.float32(max(1, H - 1))).astype(np.float32)
    uu = np.broadcast_to(u[None, :], (H, W)).ravel().copy()
    vv = np.broadcast_to(v[:, None], (H, W)).ravel().copy()
    rng = np.random.default_rng(seed)
    xi = rng.random((2, W * H))
    z = xi[0]
    phi = 2.0 * np.pi * xi[1]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    V = np.stack([r * np.cos(phi), r * np.sin(phi), z]).astype(np.float32)
    I = (-V).astype(np.float32)
    return uu, vv, np.ascontiguousarray(I)


def c2_globals(make_globals, u, v, I):
    return make_globals(u=u, v=v, I=I, N=(0.0, 0.0, 1.0), Ng=(0.0, 0.0, 1.0), dPdu=(1.0, 0.0, 0.0),
                        dPdv=(0.0, 1.0, 0.0))
