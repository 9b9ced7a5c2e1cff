"""Shader-globals descriptors (the device form of BatchedShaderGlobals,
src/include/OSL/batched_shaderglobals.h:77-197).

Each field is either a per-point SoA array (component c of point i at
data[c*plane_stride + i]) or one value shared by every point. Arrays are
device tensors for the GPU executor and numpy arrays for the CPU oracle;
the descriptor only stores their addresses, so the caller keeps them alive.
"""
import ctypes

from . import _capi as C


def _addr(arr):
    if hasattr(arr, "data_ptr"):
        return arr.data_ptr()
    return arr.ctypes.data


def make_globals(**fields):
    """make_globals(u=tensor, v=tensor, dudx=1/W, P=(x,y,z), N=tensor[3,N] ...)

    A field given as an array (1-D for floats, [3, N] planes for triples)
    is per point; a float or 3-tuple is uniform. flipHandedness and
    backfacing take int32 arrays (or a uniform number); raytype is the
    uniform int of raytype bits.
    """
    g = C.ShaderGlobalsC()
    keep = []
    for name, val in fields.items():
        if name == "raytype":
            g.raytype = int(val)
            continue
        if name in C.INT_GLOBAL_FIELDS and hasattr(val, "dtype") and str(val.dtype) not in ("int32", "torch.int32"):
            raise ValueError("global '%s' takes int32 values" % name)
        if name not in C.GLOBAL_FIELDS:
            raise KeyError("unknown shader global '%s'" % name)
        f = getattr(g, name)
        if isinstance(val, (int, float)):
            f.data = None
            f.value[0] = f.value[1] = f.value[2] = float(val)
        elif isinstance(val, (tuple, list)):
            f.data = None
            for i in range(3):
                f.value[i] = float(val[i])
        else:
            if hasattr(val, "is_contiguous") and not val.is_contiguous():
                raise ValueError("global '%s' must be contiguous" % name)
            if hasattr(val, "flags") and not val.flags["C_CONTIGUOUS"]:
                raise ValueError("global '%s' must be C-contiguous (x, y, z planes)" % name)
            f.data = ctypes.c_void_p(_addr(val))
            f.plane_stride = int(val.shape[-1]) if len(val.shape) == 2 else 0
            keep.append(val)
    g._keep = keep
    return g
