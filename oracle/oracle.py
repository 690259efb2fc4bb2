"""ctypes front end of the C++ oracle (test infrastructure only).

PARITY UNPINNED: the oracle restates euc 0.6.0 (src/pipeline.rs:248-614,
src/rasterizer/triangles.rs:15-367, src/sampler/*.rs, src/math.rs) but has no
euc output to be checked against; it is cross-checked against the pure-Python
restatement in euc_pyref.py and hand-derived known answers.
"""
import ctypes as C
import os

import numpy as np

from euc_gb300 import abi
from . import build as _build


class OracleStats(C.Structure):
    _fields_ = [("triangles", C.c_uint64), ("culled", C.c_uint64), ("candidates", C.c_uint64),
                ("passed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        L.oracle_render.restype = C.c_int
        L.oracle_render.argtypes = [C.POINTER(abi.PipelineDesc), C.c_void_p, C.c_size_t,
                                    C.POINTER(abi.VertexLayout), C.c_void_p, C.c_size_t, C.c_void_p,
                                    C.c_size_t, C.POINTER(abi.Target), C.POINTER(abi.Target), C.c_int,
                                    C.POINTER(OracleStats)]
        L.oracle_as_usize.restype = C.c_uint64
        L.oracle_as_usize.argtypes = [C.c_float]
        L.oracle_as_u8.restype = C.c_uint8
        L.oracle_as_u8.argtypes = [C.c_float]
        L.oracle_rem_euclid.restype = C.c_float
        L.oracle_rem_euclid.argtypes = [C.c_float, C.c_float]
        L.oracle_fract.restype = C.c_float
        L.oracle_fract.argtypes = [C.c_float]
        L.oracle_sample.restype = None
        L.oracle_sample.argtypes = [C.POINTER(abi.Sampler), C.c_float, C.c_float, C.POINTER(C.c_float)]
        L.oracle_hw_threads.restype = C.c_int
        L.oracle_sample_nearest.restype = C.c_int
        L.oracle_sample_nearest.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                                            C.c_void_p, C.c_uint64, C.c_void_p]
        L.oracle_texture_ingest.restype = C.c_int
        L.oracle_texture_ingest.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_void_p,
                                            C.c_uint64]
        _lib = L
    return _lib


def hw_threads():
    return lib().oracle_hw_threads()


def _target(arr, fmt):
    if arr is None:
        return abi.Target(None, 0, 0, 0, abi.FMT_NONE)
    assert arr.flags["C_CONTIGUOUS"]
    h, w = arr.shape[0], arr.shape[1]
    return abi.Target(arr.ctypes.data, w, h, arr.strides[0], fmt)


def render(desc, uniforms, layout, vertices, nverts, indices, pixel, pixel_fmt, depth, threads=1):
    """Renders in place into numpy targets; returns (status, OracleStats).

    pixel: uint8 array (H, W, bpp) or None; depth: float32 array (H, W) or None.
    Texture pointers inside `uniforms` must point at host memory.
    """
    st = OracleStats()
    vptr = vertices.ctypes.data if vertices is not None and vertices.size else None
    iptr = indices.ctypes.data if indices is not None else None
    nidx = int(indices.size) if indices is not None else 0
    pt = _target(pixel, pixel_fmt)
    dt = _target(depth, abi.FMT_R32F)
    rc = lib().oracle_render(C.byref(desc), C.addressof(uniforms), C.sizeof(uniforms), C.byref(layout), vptr,
                             int(nverts), iptr, nidx, C.byref(pt), C.byref(dt), int(threads), C.byref(st))
    return rc, st


def as_usize(v):
    return lib().oracle_as_usize(v)


def as_u8(v):
    return lib().oracle_as_u8(v)


def rem_euclid(x, m):
    return lib().oracle_rem_euclid(x, m)


def fract(x):
    return lib().oracle_fract(x)


def sample(sampler, u, v):
    out = (C.c_float * 4)()
    lib().oracle_sample(C.byref(sampler), u, v, out)
    return np.array(list(out), dtype=np.float32)


def sample_nearest(texels, queries, wrap):
    """N-D nearest sampling: texels (s_{N-1}, ..., s_0, texel bytes...) numpy
    array, axis 0 fastest; queries (count, N) f32.  Returns (count, texel
    bytes) uint8, or raises on a refused shape."""
    ndim = queries.shape[1]
    tex = np.ascontiguousarray(texels)
    size = (C.c_uint32 * ndim)(*[tex.shape[ndim - 1 - a] for a in range(ndim)])
    tb = tex.itemsize * int(np.prod(tex.shape[ndim:], dtype=np.int64))
    q = np.ascontiguousarray(queries, dtype=np.float32)
    out = np.zeros((len(q), tb), dtype=np.uint8)
    rc = lib().oracle_sample_nearest(tex.ctypes.data, ndim, size, tb, wrap, q.ctypes.data, len(q), out.ctypes.data)
    if rc:
        raise ValueError("oracle_sample_nearest: %d" % rc)
    return out


def texture_ingest(src, fmt):
    """Image rows (h, w, channels) uint8 or (h, w) float32 -> (h, w, 4) uint8
    RGBA8 texels (or the f32 bits as 4 bytes)."""
    a = np.ascontiguousarray(src)
    h, w = a.shape[:2]
    out = np.zeros((h, w, 4), dtype=np.uint8)
    rc = lib().oracle_texture_ingest(a.ctypes.data, w, h, a.strides[0], fmt, out.ctypes.data, out.strides[0])
    if rc:
        raise ValueError("oracle_texture_ingest: %d" % rc)
    return out


def run_frame(frame, threads=1):
    """Runs every pass of a scenes.FrameSpec on the oracle.

    Returns (targets dict name -> numpy array, list of OracleStats per pass,
    list of status codes).
    """
    targets = frame.alloc_host_targets()
    stats, codes = [], []
    for p in frame.passes:
        uni, keep = p.bind_uniforms(lambda src: frame.host_texture_ptr(src, targets))
        pix = targets[p.pixel] if p.pixel else None
        dep = targets[p.depth] if p.depth else None
        pfmt = frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
        rc, st = render(p.desc, uni, p.layout, p.vertices, p.nverts, p.indices, pix, pfmt, dep, threads)
        del keep
        codes.append(rc)
        stats.append(st)
    return targets, stats, codes
