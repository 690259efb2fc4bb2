"""ctypes binding of libeuc_gb300.so (the C ABI in include/euc_gb300.h).

There is no fallback: if the library is missing or a call fails, this module
raises.  The library is built by `python -m euc_gb300.build`.
"""
import ctypes as C
import os

from . import abi
from . import build as _build

_lib = None

# every function that include/euc_gb300.h declares, with (restype, argtypes)
SIGNATURES = {
    "euc_abi_version": (C.c_int, []),
    "euc_status_string": (C.c_char_p, [C.c_int]),
    "euc_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "euc_ctx_destroy": (C.c_int, [C.c_void_p]),
    "euc_ctx_reserve": (C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64]),
    "euc_ctx_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "euc_ctx_stats": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(abi.Stats)]),
    "euc_render": (C.c_int, [C.c_void_p, C.POINTER(abi.PipelineDesc), C.c_void_p, C.c_size_t,
                             C.POINTER(abi.VertexLayout), C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                             C.POINTER(abi.Target), C.POINTER(abi.Target), C.c_void_p]),
    "euc_render_host": (C.c_int, [C.c_void_p, C.POINTER(abi.PipelineDesc), C.c_void_p, C.c_size_t,
                                  C.POINTER(abi.VertexLayout), C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t,
                                  C.POINTER(abi.Target), C.POINTER(abi.Target)]),
    "euc_render_batch": (C.c_int, [C.c_void_p, C.POINTER(abi.Scene), C.c_size_t, C.c_void_p]),
    "euc_render_host_batch": (C.c_int, [C.c_void_p, C.POINTER(abi.Scene), C.c_size_t, C.c_int]),
    "euc_graph_create": (C.c_int, [C.c_void_p, C.POINTER(abi.Scene), C.c_size_t, C.POINTER(C.c_void_p)]),
    "euc_graph_launch": (C.c_int, [C.c_void_p, C.c_void_p]),
    "euc_graph_destroy": (C.c_int, [C.c_void_p]),
    "euc_ctx_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(abi.Tuning)]),
    "euc_ctx_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(abi.Tuning)]),
    "euc_ctx_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "euc_ctx_profile": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "euc_server_create": (C.c_int, [C.POINTER(abi.ServerConfig), C.POINTER(C.c_void_p)]),
    "euc_server_destroy": (C.c_int, [C.c_void_p]),
    "euc_server_add_mesh": (C.c_int, [C.c_void_p, C.POINTER(abi.VertexLayout), C.c_void_p, C.c_size_t, C.c_void_p,
                                      C.c_size_t, C.POINTER(C.c_uint32)]),
    "euc_server_add_texture": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                         C.POINTER(C.c_uint32)]),
    "euc_server_now_ns": (C.c_uint64, [C.c_void_p]),
    "euc_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_size_t)]),
    "euc_server_poll": (C.c_int, [C.c_void_p, C.POINTER(abi.ServerCompletion), C.c_size_t, C.POINTER(C.c_size_t),
                                  C.c_int]),
    "euc_server_drain": (C.c_int, [C.c_void_p, C.c_int]),
    "euc_server_stats_get": (C.c_int, [C.c_void_p, C.POINTER(abi.ServerStats)]),
    "euc_texture_ingest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32,
                                     C.c_void_p, C.c_uint64, C.c_void_p]),
    "euc_sample_nearest": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                                     C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "euc_render_noalloc": (C.c_int, [C.POINTER(abi.PipelineDesc), C.c_void_p, C.c_size_t, C.POINTER(abi.VertexLayout),
                                     C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(abi.Target),
                                     C.POINTER(abi.Target), C.c_void_p, C.c_void_p]),
}


class EucError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        super().__init__("%s%s (%s)" % (what + ": " if what else "", abi.status_name(code), status_string(code)))


def lib_path():
    return _build.LIB


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError("libeuc_gb300.so is not built (%s); run `python -m euc_gb300.build`" % path)
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.euc_abi_version() != abi.ABI_VERSION:
            raise RuntimeError("ABI version mismatch: library %d, bindings %d" % (L.euc_abi_version(), abi.ABI_VERSION))
        _lib = L
    return _lib


def status_string(code):
    try:
        return lib().euc_status_string(code).decode()
    except Exception:  # the library may be what failed to load
        return abi.status_name(code)


def check(code, what=""):
    if code != abi.OK:
        raise EucError(code, what)
    return code


class Context:
    """Owns an euc_ctx (scratch buffers, staging ring) on one CUDA device."""

    def __init__(self, device=0):
        self.device = device
        h = C.c_void_p()
        check(lib().euc_ctx_create(device, C.byref(h)), "euc_ctx_create")
        self.handle = h

    def close(self):
        if self.handle:
            lib().euc_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reserve(self, max_verts, max_tris, max_pixels, max_scenes=1):
        check(lib().euc_ctx_reserve(self.handle, max_verts, max_tris, max_pixels, max_scenes), "euc_ctx_reserve")

    def sync(self, stream=None):
        return lib().euc_ctx_sync(self.handle, stream)

    def stats(self, stream=None):
        s = abi.Stats()
        check(lib().euc_ctx_stats(self.handle, stream, C.byref(s)), "euc_ctx_stats")
        return s

    def set_tuning(self, tuning=None, **kw):
        """Sets the launch shape (abi.Tuning or its fields as keywords; None or
        no fields restores the defaults)."""
        t = tuning if tuning is not None else abi.Tuning(**kw)
        check(lib().euc_ctx_set_tuning(self.handle, C.byref(t)), "euc_ctx_set_tuning")

    def get_tuning(self):
        t = abi.Tuning()
        check(lib().euc_ctx_get_tuning(self.handle, C.byref(t)), "euc_ctx_get_tuning")
        return t

    def host_copy_direct(self):
        """True when host-buffer renders use their buffers in place (the
        device reads pageable host memory and host_copy is not STAGED)."""
        t = self.get_tuning()
        if t.host_copy == abi.HOST_COPY_STAGED:
            return False
        probe = abi.Tuning(**t.as_dict())
        probe.host_copy = abi.HOST_COPY_DIRECT
        ok = lib().euc_ctx_set_tuning(self.handle, C.byref(probe)) == abi.OK
        self.set_tuning(t)
        return ok

    def set_profiling(self, on):
        check(lib().euc_ctx_set_profiling(self.handle, 1 if on else 0), "euc_ctx_set_profiling")

    def profile(self):
        """(ms per stage dict, kernel launches) since the last call."""
        ms = (C.c_double * abi.STAGE_COUNT)()
        n = C.c_uint64()
        check(lib().euc_ctx_profile(self.handle, ms, C.byref(n)), "euc_ctx_profile")
        return dict(zip(abi.STAGE_NAMES, list(ms))), n.value

    def render(self, desc, uniforms, layout, vertices_ptr, nverts, indices_ptr, nindices, pixel, depth, stream=None):
        """Raw euc_render: device pointers; returns the status code."""
        return lib().euc_render(self.handle, C.byref(desc), C.addressof(uniforms), C.sizeof(uniforms),
                                C.byref(layout), vertices_ptr, nverts, indices_ptr, nindices,
                                C.byref(pixel) if pixel is not None else None,
                                C.byref(depth) if depth is not None else None, stream)

    def render_host(self, desc, uniforms, layout, vertices_ptr, nverts, indices_ptr, nindices, pixel, depth):
        return lib().euc_render_host(self.handle, C.byref(desc), C.addressof(uniforms), C.sizeof(uniforms),
                                     C.byref(layout), vertices_ptr, nverts, indices_ptr, nindices,
                                     C.byref(pixel) if pixel is not None else None,
                                     C.byref(depth) if depth is not None else None)

    def render_host_batch(self, arr, threads=0):
        """euc_render_host_batch on a ctypes array of abi.Scene with host pointers."""
        return lib().euc_render_host_batch(self.handle, arr, len(arr), threads)

    def render_batch(self, scenes, stream=None):
        arr = (abi.Scene * len(scenes))(*scenes)
        return lib().euc_render_batch(self.handle, arr, len(scenes), stream)

    def render_scene_array(self, arr, stream=None):
        """euc_render_batch on a prebuilt ctypes array of abi.Scene."""
        return lib().euc_render_batch(self.handle, arr, len(arr), stream)

    def graph(self, arr):
        """Records a batch (ctypes array of abi.Scene) as a replayable Graph."""
        return Graph(self, arr)


class Graph:
    """euc_graph: a batch recorded once, replayed with one launch."""

    def __init__(self, ctx, arr):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().euc_graph_create(ctx.handle, arr, len(arr), C.byref(h)), "euc_graph_create")
        self.handle = h

    def launch(self, stream=None):
        check(lib().euc_graph_launch(self.handle, stream), "euc_graph_launch")

    def close(self):
        if self.handle:
            lib().euc_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
