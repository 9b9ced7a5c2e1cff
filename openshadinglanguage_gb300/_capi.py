"""ctypes binding of include/oslg.h (the library's C ABI).

The native library is required: importing this module raises if
liboslg_gb300.so has not been built (there is no CPU fallback).
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboslg_gb300.so")

OSLG_OK = 0
OSLG_ERR_DEVICE = 6

BASE_INT32 = 7
BASE_FLOAT = 11
BASE_STRING = 13
AGG_SCALAR = 1
AGG_VEC3 = 3
AGG_MATRIX44 = 16
VEC_NOXFORM, VEC_COLOR, VEC_POINT, VEC_VECTOR, VEC_NORMAL = 0, 1, 2, 3, 4

ARENA_HEAP = 1
ARENA_OUTPUTS = 2
ARENA_USERDATA = 3


class TypeDescC(ctypes.Structure):
    _fields_ = [("basetype", ctypes.c_int32), ("aggregate", ctypes.c_int32),
                ("vecsemantics", ctypes.c_int32), ("arraylen", ctypes.c_int32)]


class SymLocC(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("type", TypeDescC), ("derivs", ctypes.c_int32),
                ("arena", ctypes.c_int32), ("offset", ctypes.c_int64), ("stride", ctypes.c_int64)]


class FieldC(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("plane_stride", ctypes.c_int64),
                ("value", ctypes.c_float * 3), ("pad", ctypes.c_float)]


GLOBAL_FIELDS = ["P", "dPdx", "dPdy", "dPdz", "I", "dIdx", "dIdy", "N", "Ng", "u", "dudx", "dudy",
                 "v", "dvdx", "dvdy", "dPdu", "dPdv", "time", "dtime", "dPdtime", "Ps", "dPsdx",
                 "dPsdy", "surfacearea", "flipHandedness", "backfacing"]
# fields whose per-point data is int32
INT_GLOBAL_FIELDS = ("flipHandedness", "backfacing")


class BatchTuningC(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int), ("points_per_thread", ctypes.c_int), ("heap_smem", ctypes.c_int),
                ("grid", ctypes.c_int),
                ("ctas_per_sm", ctypes.c_int), ("ms", ctypes.c_float)]


class ServerOptionsC(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_size_t), ("streams", ctypes.c_int), ("block", ctypes.c_int),
                ("points_per_thread", ctypes.c_int), ("max_wave_points", ctypes.c_int64),
                ("max_wave_requests", ctypes.c_int), ("arena_bytes", ctypes.c_size_t)]


class RequestStatsC(ctypes.Structure):
    _fields_ = [("submit_ns", ctypes.c_int64), ("admit_ns", ctypes.c_int64), ("done_ns", ctypes.c_int64),
                ("wave", ctypes.c_int), ("status", ctypes.c_int)]


class ServerStatsC(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("waves", ctypes.c_uint64), ("points_done", ctypes.c_int64), ("arena_capacity", ctypes.c_size_t),
                ("arena_high_water", ctypes.c_size_t), ("program_bytes", ctypes.c_size_t),
                ("scratch_bytes", ctypes.c_size_t), ("in_flight_waves", ctypes.c_int), ("pending", ctypes.c_int)]


class PrimitiveC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("material", ctypes.c_int32), ("p", ctypes.c_float * 3),
                ("ex", ctypes.c_float * 3), ("ey", ctypes.c_float * 3), ("radius", ctypes.c_float)]


class WavefrontOptionsC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("max_hits", ctypes.c_int32), ("rr_survival", ctypes.c_float), ("eye", ctypes.c_float * 3),
                ("look", ctypes.c_float * 3), ("up", ctypes.c_float * 3), ("fov_deg", ctypes.c_float),
                ("background", ctypes.c_float * 3), ("seed", ctypes.c_uint32), ("block", ctypes.c_int32),
                ("points_per_thread", ctypes.c_int32), ("heap_smem", ctypes.c_int32), ("use_graph", ctypes.c_int32)]


class WavefrontStatsC(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_int64), ("hits", ctypes.c_int64 * 16), ("total_hits", ctypes.c_int64),
                ("bounces", ctypes.c_int32), ("ms_total", ctypes.c_float), ("ms_stage", ctypes.c_float * 5)]


class ShaderGlobalsC(ctypes.Structure):
    _fields_ = [(n, FieldC) for n in GLOBAL_FIELDS] + [("raytype", ctypes.c_int32),
                                                       ("reserved", ctypes.c_int32 * 3)]


_EXPORTS = {
    "oslg_create_system": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_destroy_system": (ctypes.c_int, [ctypes.c_void_p]),
    "oslg_attribute_int": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "oslg_attribute_string": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]),
    "oslg_attribute_strings": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p),
                                              ctypes.c_int]),
    "oslg_register_closure": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]),
    "oslg_load_memory_compiled_shader": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p]),
    "oslg_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "oslg_shader_group_begin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_parameter": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, TypeDescC,
                                      ctypes.c_void_p, ctypes.c_int]),
    "oslg_shader": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                   ctypes.c_char_p]),
    "oslg_connect_shaders": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                            ctypes.c_char_p, ctypes.c_char_p]),
    "oslg_shader_group_end": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_group_renderer_outputs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                                   ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]),
    "oslg_add_symlocs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SymLocC), ctypes.c_int]),
    "oslg_group_bsdf_eval": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                            ctypes.POINTER(ctypes.c_float), ctypes.c_int64, ctypes.c_int64]),
    "oslg_group_bsdf_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64,
                                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]),
    "oslg_optimize_group": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_release_group": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_group_program": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t)]),
    "oslg_execute_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "oslg_execute_batch_indexed": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_jit_groups": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_int]),
    "oslg_find_symbol": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_symbol_typedesc": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(TypeDescC)]),
    "oslg_symbol_address": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]),
    "oslg_execute_batch_sync": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "oslg_device_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]),
    "oslg_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "oslg_execute_batch_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.POINTER(ctypes.c_uint32)]),
    "oslg_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "oslg_batch_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "oslg_batch_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ShaderGlobalsC),
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_batch_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "oslg_batch_execute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(BatchTuningC),
                                           ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(BatchTuningC)]),
    "oslg_batch_last_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchTuningC)]),
    "oslg_server_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerOptionsC),
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "oslg_server_register": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_uint64)]),
    "oslg_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int,
                                        ctypes.POINTER(RequestStatsC)]),
    "oslg_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int),
                                        ctypes.POINTER(RequestStatsC)]),
    "oslg_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ServerStatsC)]),
    "oslg_texture_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "oslg_renderer_attribute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, TypeDescC,
                                               ctypes.c_void_p]),
    "oslg_execute_layer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int64,
                                          ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "oslg_group_layer_program": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p,
                                                ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "oslg_group_record_strides": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                                 ctypes.POINTER(ctypes.c_int64)]),
    "oslg_renderer_matrix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]),
    "oslg_execute_batch_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.POINTER(ShaderGlobalsC), ctypes.c_void_p, ctypes.c_int64,
                                               ctypes.c_void_p, ctypes.c_int64, ctypes.c_int]),
    "oslg_group_specialized_source": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                                     ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
    "oslg_groups_specialized_batch_source": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                            ctypes.c_int, ctypes.c_char_p, ctypes.c_size_t,
                                                            ctypes.POINTER(ctypes.c_size_t)]),
    "oslg_group_is_specialized": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "oslg_wavefront_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WavefrontOptionsC),
                                             ctypes.POINTER(PrimitiveC), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p), ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "oslg_wavefront_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "oslg_wavefront_render": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "oslg_wavefront_render_profiled": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_void_p]),
    "oslg_wavefront_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(WavefrontStatsC)]),
}

_lib = None


def lib():
    """Load the native library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("liboslg_gb300.so is not built; run openshadinglanguage_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_EXPORTS.keys())
