"""Python mirror of the reference's ShadingSystem API over the C ABI.

Names and argument meaning follow src/include/OSL/oslexec.h
(ShaderGroupBegin / Parameter / Shader / ConnectShaders / ShaderGroupEnd,
attribute, add_symlocs, optimize_group, batched<W>().execute): a test
written against the reference reads the same here. Errors raise OSLError
carrying the library's message (the reference reports through bool
returns plus an ErrorHandler).
"""
import ctypes
from dataclasses import dataclass

from . import _capi as C


class OSLError(RuntimeError):
    pass


@dataclass(frozen=True)
class TypeDesc:
    basetype: int
    aggregate: int = C.AGG_SCALAR
    vecsemantics: int = C.VEC_NOXFORM
    arraylen: int = 0

    def c(self):
        return C.TypeDescC(self.basetype, self.aggregate, self.vecsemantics, self.arraylen)

    def array(self, n):
        return TypeDesc(self.basetype, self.aggregate, self.vecsemantics, n)

    @property
    def nfloats(self):
        return self.aggregate * max(1, self.arraylen)


TypeInt = TypeDesc(C.BASE_INT32)
TypeFloat = TypeDesc(C.BASE_FLOAT)
TypeString = TypeDesc(C.BASE_STRING)
TypeColor = TypeDesc(C.BASE_FLOAT, C.AGG_VEC3, C.VEC_COLOR)
TypePoint = TypeDesc(C.BASE_FLOAT, C.AGG_VEC3, C.VEC_POINT)
TypeVector = TypeDesc(C.BASE_FLOAT, C.AGG_VEC3, C.VEC_VECTOR)
TypeNormal = TypeDesc(C.BASE_FLOAT, C.AGG_VEC3, C.VEC_NORMAL)
TypeMatrix = TypeDesc(C.BASE_FLOAT, C.AGG_MATRIX44)
TypeClosure = TypeDesc(0)

SymArenaHeap = C.ARENA_HEAP
SymArenaOutputs = C.ARENA_OUTPUTS
SymArenaUserData = C.ARENA_USERDATA


@dataclass
class SymLocationDesc:
    """SymLocationDesc (oslexec.h:69-105): point i of `name` lives at
    base + offset + i*stride; with derivs the value is followed by its
    x and y partials."""
    name: str
    type: TypeDesc
    derivs: bool = False
    arena: int = SymArenaOutputs
    offset: int = 0
    stride: int = 0


class ShaderGroup:
    def __init__(self, ss, handle, name):
        self._ss, self._h, self.name = ss, handle, name

    @property
    def handle(self):
        return self._h

    def specialized_source(self):
        """CUDA source of the kernel specialized to this group."""
        L = C.lib()
        size = ctypes.c_size_t(0)
        self._ss._check(L.oslg_group_specialized_source(self._ss._h, self._h, None, 0, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._ss._check(L.oslg_group_specialized_source(self._ss._h, self._h, buf, size.value, ctypes.byref(size)))
        return buf.value.decode()

    def is_specialized(self):
        out = ctypes.c_int(0)
        self._ss._check(C.lib().oslg_group_is_specialized(self._ss._h, self._h, ctypes.byref(out)))
        return bool(out.value)

    def program_bytes(self):
        """The lowered op program (what replaces the JIT'd module)."""
        L = C.lib()
        size = ctypes.c_size_t(0)
        self._ss._check(L.oslg_group_program(self._ss._h, self._h, None, 0, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._ss._check(L.oslg_group_program(self._ss._h, self._h, buf, size.value, ctypes.byref(size)))
        return buf.raw[: size.value]

    def layer_program_bytes(self, layername):
        """The program that runs layers up to and including `layername`."""
        L = C.lib()
        size = ctypes.c_size_t(0)
        self._ss._check(L.oslg_group_layer_program(self._ss._h, self._h, layername.encode(), None, 0,
                                                   ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._ss._check(L.oslg_group_layer_program(self._ss._h, self._h, layername.encode(), buf, size.value,
                                                   ctypes.byref(size)))
        return buf.raw[: size.value]

    def release(self):
        if self._h:
            C.lib().oslg_release_group(self._ss._h, self._h)
            self._h = None


class ShadingSystem:
    def __init__(self):
        L = C.lib()
        h = ctypes.c_void_p()
        if L.oslg_create_system(ctypes.byref(h)) != C.OSLG_OK:
            raise OSLError("could not create the shading system")
        self._h = h
        self._keep = []

    def close(self):
        if self._h:
            C.lib().oslg_destroy_system(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != C.OSLG_OK:
            msg = C.lib().oslg_last_error(self._h)
            raise OSLError("osl-gb300 error %d: %s" % (rc, msg.decode() if msg else ""))

    # ---- configuration -------------------------------------------------------
    def attribute(self, name, value):
        if isinstance(value, str):
            self._check(C.lib().oslg_attribute_string(self._h, name.encode(), value.encode()))
        elif isinstance(value, (list, tuple)):
            arr = (ctypes.c_char_p * max(1, len(value)))(*[str(v).encode() for v in value])
            self._check(C.lib().oslg_attribute_strings(self._h, name.encode(), arr, len(value)))
        else:
            self._check(C.lib().oslg_attribute_int(self._h, name.encode(), int(value)))

    def register_closure(self, name, closure_id):
        self._check(C.lib().oslg_register_closure(self._h, name.encode(), int(closure_id)))

    def LoadMemoryCompiledShader(self, shadername, oso_text):
        self._check(C.lib().oslg_load_memory_compiled_shader(self._h, shadername.encode(), oso_text.encode()))
        return True

    # ---- groups --------------------------------------------------------------
    def ShaderGroupBegin(self, groupname=""):
        g = ctypes.c_void_p()
        self._check(C.lib().oslg_shader_group_begin(self._h, groupname.encode(), ctypes.byref(g)))
        return ShaderGroup(self, g, groupname)

    def renderer_attribute(self, name, type_, value, object=""):
        """RendererServices::get_attribute for a uniform attribute
        (oslg_renderer_attribute): getattribute([object,] name, ...) in a
        shader answers with `value` (a scalar, or a flat list for arrays and
        triples). Register before the groups that read it are optimized."""
        ptr, arr = self._values(type_, value)
        self._keep.append(arr)
        self._check(C.lib().oslg_renderer_attribute(self._h, object.encode(), name.encode(), type_.c(), ptr))

    def renderer_matrix(self, name, matrix):
        """RendererServices::get_matrix for a named space
        (oslg_renderer_matrix): the 4x4 space-to-common matrix, row major,
        points as row vectors. Register before the groups that use the
        space are optimized."""
        import numpy as np
        m = np.ascontiguousarray(np.asarray(matrix, np.float32).reshape(16))
        self._check(C.lib().oslg_renderer_matrix(self._h, name.encode(), ctypes.c_void_p(m.ctypes.data)))

    @staticmethod
    def _values(type_, value):
        if type_.basetype == C.BASE_STRING:
            vals = value if isinstance(value, (list, tuple)) else [value]
            arr = (ctypes.c_char_p * len(vals))(*[v.encode() for v in vals])
        elif type_.basetype == C.BASE_INT32:
            vals = value if isinstance(value, (list, tuple)) else [value]
            arr = (ctypes.c_int * len(vals))(*[int(v) for v in vals])
        else:
            vals = value if isinstance(value, (list, tuple)) else [value] * type_.nfloats
            arr = (ctypes.c_float * len(vals))(*[float(v) for v in vals])
        return ctypes.cast(arr, ctypes.c_void_p), arr

    def Parameter(self, group, name, type_, value, lockgeom=True):
        ptr, arr = self._values(type_, value)
        self._keep.append(arr)
        self._check(C.lib().oslg_parameter(self._h, group.handle, name.encode(), type_.c(), ptr,
                                           1 if lockgeom else 0))

    def Shader(self, group, shaderusage, shadername, layername=""):
        self._check(C.lib().oslg_shader(self._h, group.handle, shaderusage.encode(), shadername.encode(),
                                        layername.encode()))

    def ConnectShaders(self, group, srclayer, srcparam, dstlayer, dstparam):
        self._check(C.lib().oslg_connect_shaders(self._h, group.handle, srclayer.encode(), srcparam.encode(),
                                                 dstlayer.encode(), dstparam.encode()))

    def ShaderGroupEnd(self, group):
        self._check(C.lib().oslg_shader_group_end(self._h, group.handle))

    def renderer_outputs(self, group, names):
        arr = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        self._check(C.lib().oslg_group_renderer_outputs(self._h, group.handle, arr, len(names)))

    def add_symlocs(self, group, symlocs):
        locs = symlocs if isinstance(symlocs, (list, tuple)) else [symlocs]
        arr = (C.SymLocC * len(locs))()
        names = []
        for i, s in enumerate(locs):
            nm = s.name.encode()
            names.append(nm)
            arr[i] = C.SymLocC(nm, s.type.c(), 1 if s.derivs else 0, s.arena, s.offset, s.stride)
        self._check(C.lib().oslg_add_symlocs(self._h, group.handle, arr, len(locs)))

    def bsdf_sample_output(self, group, closure, offset, stride, in_offset, in_stride):
        """Per point: read {rx, ry, rz, path_weight.rgb, absorb} from the
        userdata arena, write {wi.xyz, weight.rgb, pdf, Le.rgb, roughness}
        to the output arena (include/oslg.h, oslg_group_bsdf_sample)."""
        self._check(C.lib().oslg_group_bsdf_sample(self._h, group.handle, closure.encode(), int(offset), int(stride),
                                                   int(in_offset), int(in_stride)))

    def bsdf_eval_output(self, group, closure, wi, offset, stride):
        """Evaluate closure output `closure` as testrender's CompositeBSDF at
        wo = -I and light direction wi; writes weight rgb + pdf per point."""
        w = (ctypes.c_float * 3)(*[float(x) for x in wi])
        self._check(C.lib().oslg_group_bsdf_eval(self._h, group.handle, closure.encode(), w, offset, stride))

    def optimize_group(self, group):
        self._check(C.lib().oslg_optimize_group(self._h, group.handle))

    def set_launch(self, block=256, points_per_thread=1, heap_smem=-1):
        self._check(C.lib().oslg_set_launch(self._h, block, points_per_thread, heap_smem))

    # ---- execution --------------------------------------------------------------
    def execute_batch(self, group, npoints, globals_c, userdata_ptr=0, output_ptr=0, stream=0, sync=False):
        """BatchedExecutor::execute over npoints device-resident points.
        globals_c is a ShaderGlobalsC (see globals.make_globals)."""
        fn = C.lib().oslg_execute_batch_sync if sync else C.lib().oslg_execute_batch
        self._check(fn(self._h, group.handle, int(npoints), ctypes.byref(globals_c),
                       ctypes.c_void_p(userdata_ptr or None), ctypes.c_void_p(output_ptr or None),
                       ctypes.c_void_p(stream or None)))

    def execute_batch_indexed(self, group, npoints, globals_c, shadeindex_ptr, userdata_ptr=0, output_ptr=0,
                              stream=0):
        """BatchedExecutor::execute with wide_shadeindex: point i's userdata
        and output records are record shadeindex[i] (a device int32 array)."""
        self._check(C.lib().oslg_execute_batch_indexed(self._h, group.handle, int(npoints), ctypes.byref(globals_c),
                                                       ctypes.c_void_p(shadeindex_ptr or None),
                                                       ctypes.c_void_p(userdata_ptr or None),
                                                       ctypes.c_void_p(output_ptr or None),
                                                       ctypes.c_void_p(stream or None)))

    def jit_groups(self, groups, nthreads=0):
        """BatchedExecutor::jit_all_groups: lower and upload the groups and,
        with attribute jit, build their specialized kernels in parallel."""
        arr = (ctypes.c_void_p * max(1, len(groups)))(*[g.handle for g in groups])
        self._check(C.lib().oslg_jit_groups(self._h, arr, len(groups), int(nthreads)))

    def find_symbol(self, group, symbolname, layername=None):
        """ShadingSystem::find_symbol: a handle to the symbol; from now on
        every device execution of the group keeps its final values."""
        h = ctypes.c_void_p()
        self._check(C.lib().oslg_find_symbol(self._h, group.handle, layername.encode() if layername else None,
                                             symbolname.encode(), ctypes.byref(h)))
        return h.value

    def symbol_typedesc(self, sym):
        t = C.TypeDescC()
        self._check(C.lib().oslg_symbol_typedesc(ctypes.c_void_p(sym), ctypes.byref(t)))
        return TypeDesc(t.basetype, t.aggregate, t.vecsemantics, t.arraylen)

    def symbol_address(self, group, sym):
        """ShadingSystem::symbol_address for the last device execution:
        (device address, plane stride); word c of point i at
        address[c * stride + i]."""
        p, stride = ctypes.c_void_p(), ctypes.c_int64()
        self._check(C.lib().oslg_symbol_address(self._h, group.handle, ctypes.c_void_p(sym), ctypes.byref(p),
                                                ctypes.byref(stride)))
        return p.value, stride.value

    def symbol_array(self, group, sym, npoints):
        """The symbol's values as a (words, npoints) device array view
        (__cuda_array_interface__, e.g. for torch.as_tensor)."""
        t = self.symbol_typedesc(sym)
        ptr, stride = self.symbol_address(group, sym)
        words = t.nfloats

        class _View:
            __cuda_array_interface__ = {"shape": (words, int(npoints)), "typestr": "<i4" if t.basetype == C.BASE_INT32
                                        else "<f4", "data": (ptr, False), "version": 3,
                                        "strides": (4 * stride, 4)}
        return _View()

    def execute_layer(self, group, layername, npoints, globals_c, userdata_ptr=0, output_ptr=0, stream=0):
        """BatchedExecutor::execute_init + execute_layer(layername): the
        layers up to and including `layername`, over device points."""
        self._check(C.lib().oslg_execute_layer(self._h, group.handle, layername.encode(), int(npoints),
                                               ctypes.byref(globals_c), ctypes.c_void_p(userdata_ptr or None),
                                               ctypes.c_void_p(output_ptr or None), ctypes.c_void_p(stream or None)))

    def batch(self):
        """A persistent multi-group batch on this system (see Batch)."""
        return Batch(self)

    def server(self, **options):
        """A continuous-batching shading server on this system (see Server)."""
        return Server(self, **options)

    def specialized_batch_source(self, groups):
        """CUDA source of a persistent batch kernel specialized to `groups`."""
        L = C.lib()
        arr = (ctypes.c_void_p * len(groups))(*[g.handle.value for g in groups])
        size = ctypes.c_size_t(0)
        self._check(L.oslg_groups_specialized_batch_source(self._h, arr, len(groups), None, 0, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._check(L.oslg_groups_specialized_batch_source(self._h, arr, len(groups), buf, size.value,
                                                           ctypes.byref(size)))
        return buf.value.decode()

    def wavefront(self, prims, materials, **options):
        """A wavefront path tracer over `prims` shaded by `materials` (see Wavefront)."""
        return Wavefront(self, prims, materials, **options)

    def texture_create(self, name, texels):
        """Register an image for texture(name, ...): texels is a float32
        array (height, width, nchannels) or (height, width); returns its index."""
        import numpy as np
        a = np.ascontiguousarray(texels, dtype=np.float32)
        if a.ndim == 2:
            a = a[:, :, None]
        h, w, nch = a.shape
        idx = ctypes.c_int(-1)
        self._check(C.lib().oslg_texture_create(self._h, name.encode(), int(w), int(h), int(nch),
                                                ctypes.c_void_p(a.ctypes.data), ctypes.byref(idx)))
        return idx.value

    def execute_batch_host(self, group, npoints, globals_c, outputs, output_stride, userdata=None,
                           userdata_stride=0, preserve_outputs=False):
        """BatchedExecutor::execute over host buffers (oslg_execute_batch_host):
        globals_c has host SoA planes; outputs/userdata are host arrays or
        CPU tensors (pinned for overlapped copies) of per-point records."""
        def addr(x):
            if x is None:
                return None
            if hasattr(x, "data_ptr"):
                return x.data_ptr()
            if hasattr(x, "ctypes"):
                return x.ctypes.data
            return int(x)
        self._check(C.lib().oslg_execute_batch_host(self._h, group.handle, int(npoints), ctypes.byref(globals_c),
                                                    ctypes.c_void_p(addr(userdata)), int(userdata_stride),
                                                    ctypes.c_void_p(addr(outputs)), int(output_stride),
                                                    1 if preserve_outputs else 0))

    def device_status(self):
        bits = ctypes.c_uint32(0)
        self._check(C.lib().oslg_device_status(self._h, ctypes.byref(bits)))
        return bits.value


class Batch:
    """Many groups' requests run in one persistent kernel launch, replayed
    as a CUDA graph while unchanged (include/oslg.h, oslg_batch_*). Results
    equal one execute_batch call per request. Keep every globals structure
    and device buffer alive until clear() or close()."""

    def __init__(self, ss):
        self._ss = ss
        h = ctypes.c_void_p()
        ss._check(C.lib().oslg_batch_create(ss._h, ctypes.byref(h)))
        self._h = h
        self._keep = []

    def close(self):
        if self._h:
            C.lib().oslg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        self._ss._check(C.lib().oslg_batch_clear(self._h))
        self._keep = []

    def add(self, group, npoints, globals_c, userdata_ptr=0, output_ptr=0):
        self._keep.append(globals_c)
        self._ss._check(C.lib().oslg_batch_add(self._h, group.handle, int(npoints), ctypes.byref(globals_c),
                                               ctypes.c_void_p(userdata_ptr or None),
                                               ctypes.c_void_p(output_ptr or None)))

    def set_launch(self, block=0, heap_smem=-1, use_graph=True, points_per_thread=0):
        self._ss._check(C.lib().oslg_batch_set_launch(self._h, int(block), int(points_per_thread), int(heap_smem),
                                                      1 if use_graph else 0))

    def execute(self, stream=0):
        self._ss._check(C.lib().oslg_batch_execute(self._h, ctypes.c_void_p(stream or None)))

    @staticmethod
    def _tuning(t):
        return dict(block=t.block, points_per_thread=t.points_per_thread, heap_smem=t.heap_smem, grid=t.grid,
                    ctas_per_sm=t.ctas_per_sm, ms=t.ms)

    def autotune(self, stream=0, reps=3):
        """Sweep points per thread {1,2,4} x block {128,256,512} x heap
        {shared, HBM}; returns (best, all measured)."""
        res = (C.BatchTuningC * 32)()
        n = ctypes.c_int(0)
        best = C.BatchTuningC()
        self._ss._check(C.lib().oslg_batch_autotune(self._h, ctypes.c_void_p(stream or None), int(reps), res, 32,
                                                    ctypes.byref(n), ctypes.byref(best)))
        return self._tuning(best), [self._tuning(res[i]) for i in range(n.value)]

    def last_launch(self):
        t = C.BatchTuningC()
        self._ss._check(C.lib().oslg_batch_last_launch(self._h, ctypes.byref(t)))
        return self._tuning(t)


class Server:
    """Continuous-batching request server (include/oslg.h, oslg_server_*).
    Requests carry host inputs (globals whose per-point fields are host
    arrays) and a host output buffer; submit() returns a ticket, wait()
    blocks until that request's outputs are in the host buffer and returns
    its timing (host steady-clock nanoseconds)."""

    def __init__(self, ss, budget_bytes=40 << 30, streams=3, block=512, points_per_thread=1,
                 max_wave_points=8 << 20, max_wave_requests=512, arena_bytes=0):
        self._ss = ss
        o = C.ServerOptionsC(int(budget_bytes), int(streams), int(block), int(points_per_thread),
                             int(max_wave_points), int(max_wave_requests), int(arena_bytes))
        h = ctypes.c_void_p()
        ss._check(C.lib().oslg_server_create(ss._h, ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def close(self):
        if self._h:
            C.lib().oslg_server_destroy(self._h)
            self._h = None
            self._keep = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def register(self, group):
        self._ss._check(C.lib().oslg_server_register(self._h, group.handle))

    def submit(self, group, npoints, globals_c, output, output_bytes=None):
        """output: a host array (numpy or CPU tensor) or an address with
        output_bytes. Inputs and output must stay alive until wait()."""
        if hasattr(output, "data_ptr"):
            ptr, nb = output.data_ptr(), output.numel() * output.element_size()
        elif hasattr(output, "ctypes"):
            ptr, nb = output.ctypes.data, output.nbytes
        else:
            ptr, nb = int(output), int(output_bytes)
        t = ctypes.c_uint64(0)
        self._ss._check(C.lib().oslg_server_submit(self._h, group.handle, int(npoints), ctypes.byref(globals_c),
                                                   ctypes.c_void_p(ptr), ctypes.c_size_t(nb), ctypes.byref(t)))
        self._keep[t.value] = (globals_c, output)
        return t.value

    @staticmethod
    def _stats(st):
        return dict(submit_ns=st.submit_ns, admit_ns=st.admit_ns, done_ns=st.done_ns, wave=st.wave, status=st.status)

    def wait(self, ticket, timeout_ms=-1):
        st = C.RequestStatsC()
        rc = C.lib().oslg_server_wait(self._h, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(st))
        self._keep.pop(ticket, None)
        self._ss._check(rc)
        return self._stats(st)

    def poll(self, ticket):
        st = C.RequestStatsC()
        done = ctypes.c_int(0)
        rc = C.lib().oslg_server_poll(self._h, ctypes.c_uint64(ticket), ctypes.byref(done), ctypes.byref(st))
        if done.value:
            self._keep.pop(ticket, None)
        self._ss._check(rc)
        return self._stats(st) if done.value else None

    def stats(self):
        s = C.ServerStatsC()
        self._ss._check(C.lib().oslg_server_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in C.ServerStatsC._fields_}


class Wavefront:
    """Wavefront path tracing of a frame (include/oslg.h, oslg_wavefront_*):
    every camera path advances one bounce per wavefront; the hits of a
    bounce are sorted by material and shaded by the persistent batch
    kernel. `prims` is a sequence of (kind, material, p, ex, ey, radius)
    tuples or a numpy structured array with those fields; `materials` are
    groups whose closure output is sampled with bsdf_sample_output(offset 0,
    stride 44, in_offset 0, in_stride 36)."""

    OPTION_DEFAULTS = dict(width=1920, height=1080, spp=4, max_hits=8, rr_survival=0.8, eye=(0.0, 6.0, 30.0),
                           look=(0.0, 2.0, -10.0), up=(0.0, 1.0, 0.0), fov_deg=50.0,
                           background=(0.25, 0.3, 0.4), seed=0xC5, block=0, points_per_thread=0, heap_smem=0,
                           use_graph=0)

    def __init__(self, ss, prims, materials, **options):
        self._ss = ss
        o = dict(self.OPTION_DEFAULTS)
        for k in options:
            if k not in o:
                raise KeyError("unknown wavefront option '%s'" % k)
        o.update(options)
        self.options = o
        self._opts = options_c(o)
        arr = prims_c(prims)
        mats = (ctypes.c_void_p * len(materials))(*[m.handle.value if hasattr(m.handle, "value") else m.handle
                                                   for m in materials])
        h = ctypes.c_void_p()
        ss._check(C.lib().oslg_wavefront_create(ss._h, ctypes.byref(self._opts), arr, len(arr), mats,
                                                len(materials), ctypes.byref(h)))
        self._h = h
        self._materials = list(materials)
        self.paths = o["width"] * o["height"] * o["spp"]

    def close(self):
        if self._h:
            C.lib().oslg_wavefront_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, path_radiance=0, image=0, stream=0, profile=False):
        """Enqueue one frame on `stream`. path_radiance: device address of 3
        planes of `paths` floats; image: device address of width*height*3
        floats (0 to skip either)."""
        fn = C.lib().oslg_wavefront_render_profiled if profile else C.lib().oslg_wavefront_render
        self._ss._check(fn(self._h, ctypes.c_void_p(int(path_radiance) or None),
                           ctypes.c_void_p(int(image) or None), ctypes.c_void_p(int(stream) or None)))

    def stats(self):
        s = C.WavefrontStatsC()
        self._ss._check(C.lib().oslg_wavefront_get_stats(self._h, ctypes.byref(s)))
        return dict(paths=s.paths, hits=list(s.hits), total_hits=s.total_hits, bounces=s.bounces,
                    ms_total=s.ms_total, ms_stage=list(s.ms_stage))


def options_c(o):
    """oslg_wavefront_options from a dict of Wavefront.OPTION_DEFAULTS keys."""
    f3 = lambda v: (ctypes.c_float * 3)(*[float(x) for x in v])
    return C.WavefrontOptionsC(int(o["width"]), int(o["height"]), int(o["spp"]), int(o["max_hits"]),
                               float(o["rr_survival"]), f3(o["eye"]), f3(o["look"]), f3(o["up"]),
                               float(o["fov_deg"]), f3(o["background"]), int(o["seed"]) & 0xFFFFFFFF,
                               int(o["block"]), int(o["points_per_thread"]), int(o["heap_smem"]),
                               int(o["use_graph"]))


def prims_c(prims):
    """oslg_primitive array from tuples or a structured array."""
    n = len(prims)
    arr = (C.PrimitiveC * max(1, n))()
    for i in range(n):
        q = prims[i]
        kind, mat, p, ex, ey, r = (q["kind"], q["material"], q["p"], q["ex"], q["ey"], q["radius"]) \
            if hasattr(q, "dtype") else q
        arr[i].kind = int(kind)
        arr[i].material = int(mat)
        for k in range(3):
            arr[i].p[k] = float(p[k])
            arr[i].ex[k] = float(ex[k])
            arr[i].ey[k] = float(ey[k])
        arr[i].radius = float(r)
    return arr if n else (C.PrimitiveC * 0)()
