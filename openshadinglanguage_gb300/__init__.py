"""osl-gb300: a GB300-native executor for OSL's batched shading hot path.

The package exposes the reference-shaped ShadingSystem API (shadingsys),
shader-global descriptors (globals), an .oso writer (oso) and the shader
programs of the benchmark workloads (shaders). The compute path is the
native library liboslg_gb300.so (C ABI in include/oslg.h): host C++
lowering plus hand-written sm_103a CUDA kernels.
"""
from .shadingsys import (  # noqa: F401
    OSLError, ShadingSystem, ShaderGroup, SymLocationDesc, TypeDesc, TypeColor, TypeFloat, TypeInt,
    TypeMatrix, TypeNormal, TypePoint, TypeString, TypeVector, TypeClosure, SymArenaHeap, SymArenaOutputs,
    SymArenaUserData)
from .globals import make_globals  # noqa: F401
from .oso import OsoBuilder  # noqa: F401

__version__ = "0.1.0"


def build():
    """Compile the native library in-tree (sm_103a)."""
    from .build import build as _b
    return _b()
