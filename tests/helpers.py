"""Shared test utilities: build/load the native library and the oracle,
make testshade-style grids, run a group on the oracle or on the GPU."""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import openshadinglanguage_gb300 as og  # noqa: E402
from openshadinglanguage_gb300 import _capi, shaders  # noqa: E402
from openshadinglanguage_gb300.build import build as build_native  # noqa: E402
from oracle.build import build as build_oracle  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")

_oracle = None


def oracle():
    global _oracle
    if _oracle is None:
        L = ctypes.CDLL(build_oracle())
        L.oracle_run.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.POINTER(_capi.ShaderGlobalsC), ctypes.c_void_p, ctypes.c_void_p,
                                 ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
        L.oracle_run.restype = ctypes.c_int
        L.oracle_noise.argtypes = [ctypes.c_int] * 5 + [ctypes.POINTER(ctypes.c_float)] * 3
        L.oracle_hash_f.argtypes = [ctypes.c_float]
        L.oracle_hash_f.restype = ctypes.c_int
        L.oracle_inthash.argtypes = [ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]
        L.oracle_inthash.restype = ctypes.c_uint32
        L.oracle_wavefront.argtypes = [ctypes.POINTER(_capi.WavefrontOptionsC), ctypes.POINTER(_capi.PrimitiveC),
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                       ctypes.POINTER(ctypes.c_size_t), ctypes.c_int, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int64)]
        L.oracle_wavefront.restype = ctypes.c_int
        _oracle = L
    return _oracle


def oracle_run(blob, npoints, G, outputs, userdata=None, nthreads=0, begin=0):
    st = ctypes.c_uint32(0)
    ud = userdata.ctypes.data if userdata is not None else None
    rc = oracle().oracle_run(blob, len(blob), begin, npoints, ctypes.byref(G), ud, outputs.ctypes.data,
                             nthreads, ctypes.byref(st))
    assert rc == 0, "oracle rejected the program"
    return st.value


def oracle_wavefront(options, prims, groups, begin=0, count=None, step=1, nthreads=0):
    """The oracle's path tracer over paths begin + k*step: returns
    (radiance float32 (3, count), hits per bounce int64 (16,), status)."""
    from openshadinglanguage_gb300.shadingsys import Wavefront, options_c, prims_c
    o = dict(Wavefront.OPTION_DEFAULTS)
    o.update(options)
    npaths = o["width"] * o["height"] * o["spp"]
    if count is None:
        count = (npaths - begin + step - 1) // step
    blobs = [g.program_bytes() for g in groups]
    bufs = [ctypes.create_string_buffer(b, len(b)) for b in blobs]
    ptrs = (ctypes.c_void_p * len(bufs))(*[ctypes.addressof(b) for b in bufs])
    sizes = (ctypes.c_size_t * len(bufs))(*[len(b) for b in blobs])
    oc = options_c(o)
    arr = prims_c(prims)
    rad = np.zeros((3, count), np.float32)
    hits = np.zeros(16, np.int64)
    st = oracle().oracle_wavefront(ctypes.byref(oc), arr, len(prims), ptrs, sizes, len(groups), begin, count, step,
                                   nthreads, rad.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                   hits.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    assert st >= 0, "oracle rejected a material program"
    return rad, hits, st


def pixel_grid(W, H, centers=False):
    """testshade's u,v: the default Reyes-style grid u = x/(W-1), or pixel
    centres u = (x+0.5)/W with --center (src/testshade/testshade.cpp:1790-1803)."""
    x = np.arange(W, dtype=np.float32)
    y = np.arange(H, dtype=np.float32)
    if centers:
        u = ((x + np.float32(0.5)) / np.float32(W)).astype(np.float32)
        v = ((y + np.float32(0.5)) / np.float32(H)).astype(np.float32)
    else:
        u = (x / np.float32(max(1, W - 1))).astype(np.float32) if W > 1 else np.full(W, 0.5, np.float32)
        v = (y / np.float32(max(1, H - 1))).astype(np.float32) if H > 1 else np.full(H, 0.5, np.float32)
    uu = np.broadcast_to(u[None, :], (H, W)).ravel().copy()
    vv = np.broadcast_to(v[:, None], (H, W)).ravel().copy()
    return uu, vv


def grid_globals(u, v, W, H, P=None, centers=False):
    """Uniform fields as testshade's setup_uniform_shaderglobals
    (testshade.cpp:1681-1775)."""
    du = 1.0 / W if centers else 1.0 / max(1, W - 1)
    dv = 1.0 / H if centers else 1.0 / max(1, H - 1)
    f = dict(u=u, v=v, dudx=du, dudy=0.0, dvdx=0.0, dvdy=dv, N=(0, 0, 1), Ng=(0, 0, 1),
             dPdu=(1, 0, 0), dPdv=(0, 1, 0), dPdx=(du, 0, 0), dPdy=(0, dv, 0), surfacearea=1.0)
    if P is not None:
        f["P"] = P
    return og.make_globals(**f)


def single_layer_group(ss, shadername, oso, params=(), layer="layer1", outputs=()):
    ss.LoadMemoryCompiledShader(shadername, oso)
    g = ss.ShaderGroupBegin(shadername + "_group")
    for name, t, val in params:
        ss.Parameter(g, name, t, val)
    ss.Shader(g, "surface", shadername, layer)
    ss.ShaderGroupEnd(g)
    if outputs:
        ss.add_symlocs(g, list(outputs))
    return g


def float_equal(a, b):
    """Value equality for float arrays: +0 == -0 and NaN == NaN."""
    a = np.asarray(a)
    b = np.asarray(b)
    return (a == b) | (np.isnan(a) & np.isnan(b))


def to_uint8(img):
    """OIIO float -> uint8 conversion used by testshade -od uint8."""
    return np.clip(np.floor(np.clip(img, 0.0, 1.0) * 255.0 + 0.5), 0, 255).astype(np.uint8)


def golden_image(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return z["img"], int(z["full_w"]), int(z["full_h"]), int(z["step"])


def image_diff_ok(got_u8, ref_u8, failthresh=0.004, failpercent=0.02, hardfail=0.01):
    """runtest.py:82-89 thresholds on 0..1 pixel values."""
    d = np.abs(got_u8.astype(np.float64) - ref_u8.astype(np.float64)) / 255.0
    nfail = np.count_nonzero(d > failthresh + 1e-9)
    frac = 100.0 * nfail / d.size
    return (frac <= failpercent and d.max() <= max(hardfail, 1.0 / 255.0 + 1e-9)), frac, d.max()
