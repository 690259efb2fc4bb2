"""Host-side mirror of euc's `Pipeline` API (src/pipeline.rs, src/rasterizer/
mod.rs, src/texture.rs, src/buffer.rs, src/index.rs, src/sampler/mod.rs).

Same names, argument meaning and error behaviour as euc 0.6.0; shader stages
are the CUDA functors selected by `Pipeline.SHADER` (euc's Rust closures cannot
run on the GPU, so each Pipeline impl names its device functor and provides
its uniforms).  `render` raises `EucError` where euc panics.

    class Cube(Pipeline):                       # examples/spinning_cube.rs
        SHADER = abi.SHADER_GOURAUD
        def depth_mode(self): return DepthMode.LESS_WRITE
        def uniforms(self): ...                  # an abi.GouraudUniforms
        def vertex_layout(self): return abi.VertexLayout(24, 0, 12, -1, -1)

    color = Buffer2d.fill([640, 480], 0, fmt=abi.FMT_RGB8)
    depth = Buffer2d.fill([640, 480], 1.0)
    Cube().render(IndexedVertices(indices, vertices), color, depth)
"""
from dataclasses import dataclass
import ctypes as C

import numpy as np

from . import abi, capi

# ---------------------------------------------------------------------------
# Modes (pipeline.rs:12-163, rasterizer/mod.rs:9-18)
# ---------------------------------------------------------------------------
LESS, EQUAL, GREATER = "Less", "Equal", "Greater"  # core::cmp::Ordering
_ORDERING = {None: abi.TEST_NONE, LESS: abi.TEST_LESS, EQUAL: abi.TEST_EQUAL, GREATER: abi.TEST_GREATER}


@dataclass(frozen=True)
class DepthMode:
    test: object = None  # None or LESS / EQUAL / GREATER
    write: bool = False

    def uses_depth(self):
        return self.test is not None or self.write


DepthMode.NONE = DepthMode(None, False)
DepthMode.LESS_WRITE = DepthMode(LESS, True)
DepthMode.GREATER_WRITE = DepthMode(GREATER, True)
DepthMode.LESS_PASS = DepthMode(LESS, False)
DepthMode.GREATER_PASS = DepthMode(GREATER, False)


@dataclass(frozen=True)
class PixelMode:
    write: bool = True


PixelMode.WRITE = PixelMode(True)
PixelMode.PASS = PixelMode(False)


class Handedness:
    Left, Right = abi.LEFT, abi.RIGHT


class YAxisDirection:
    Down, Up = abi.Y_DOWN, abi.Y_UP


@dataclass(frozen=True)
class CoordinateMode:
    handedness: int = Handedness.Left
    y_axis_direction: int = YAxisDirection.Down
    z_clip_range: object = (0.0, 1.0)  # (start, end), inclusive, or None

    def without_z_clip(self):
        return CoordinateMode(self.handedness, self.y_axis_direction, None)


CoordinateMode.OPENGL = CoordinateMode(Handedness.Right, YAxisDirection.Up, (-1.0, 1.0))
CoordinateMode.VULKAN = CoordinateMode(Handedness.Left, YAxisDirection.Down, (0.0, 1.0))
CoordinateMode.METAL = CoordinateMode(Handedness.Right, YAxisDirection.Down, (0.0, 1.0))
CoordinateMode.DIRECTX = CoordinateMode(Handedness.Left, YAxisDirection.Up, (0.0, 1.0))


@dataclass(frozen=True)
class AaMode:
    level: int = 0  # 0 = AaMode::None; n = AaMode::Msaa { level: n }

    @staticmethod
    def Msaa(level):
        return AaMode(int(level))


AaMode.None_ = AaMode(0)


class CullMode:
    None_, Back, Front = abi.CULL_NONE, abi.CULL_BACK, abi.CULL_FRONT


class BandMode:
    """How rows are split into euc's render_par bands (not in euc's API:
    euc fixes it by the `par` cargo feature)."""
    PAR = abi.BANDS_PAR     # euc default; small targets fall back to one band
    SEQ = abi.BANDS_SEQ     # euc built without `par` (render_seq)


# ---------------------------------------------------------------------------
# Targets, textures, samplers (buffer.rs, texture.rs, sampler/*.rs)
# ---------------------------------------------------------------------------
class Buffer2d:
    """Row-major 2-D buffer usable as a render target or a texture.

    Backed by a numpy array (host; rendered through euc_render_host) or a
    CUDA torch tensor (device; rendered through euc_render)."""

    def __init__(self, data, fmt):
        self.data = data
        self.fmt = fmt

    @staticmethod
    def fill(size, value, fmt=None, device=None):
        w, h = size
        if fmt is None:
            fmt = abi.FMT_R32F if isinstance(value, float) else abi.FMT_RGBA8
        if fmt == abi.FMT_R32F:
            arr = np.full((h, w), np.float32(value), dtype=np.float32)
        elif fmt == abi.FMT_RGBA32F:  # Buffer2d<[f32; 4]>: value is a float or four floats
            arr = np.empty((h, w, 4), dtype=np.float32)
            arr[...] = np.asarray(value, dtype=np.float32)
        else:
            bpp = abi.FMT_BPP[fmt]
            px = np.frombuffer(int(value).to_bytes(8, "little")[:bpp], dtype=np.uint8)
            arr = np.ascontiguousarray(np.broadcast_to(px, (h, w, bpp)))
        if device is not None:
            import torch
            arr = torch.from_numpy(arr).to(device)
        return Buffer2d(arr, fmt)

    def size(self):
        return [int(self.data.shape[1]), int(self.data.shape[0])]

    @property
    def on_device(self):
        return not isinstance(self.data, np.ndarray)

    def clear(self, value):
        if self.fmt == abi.FMT_R32F:
            self.data[...] = float(np.float32(value))
        elif self.fmt == abi.FMT_RGBA32F:
            px = np.asarray(value, dtype=np.float32) * np.ones(4, dtype=np.float32)
            if self.on_device:
                import torch
                self.data.copy_(torch.from_numpy(px).to(self.data.device).expand_as(self.data))
            else:
                self.data[...] = px
        else:
            bpp = abi.FMT_BPP[self.fmt]
            px = np.frombuffer(int(value).to_bytes(8, "little")[:bpp], dtype=np.uint8)
            if self.on_device:
                import torch
                self.data.copy_(torch.from_numpy(px.copy()).to(self.data.device).expand_as(self.data))
            else:
                self.data[...] = px

    def raw(self):
        return self.data

    def ptr(self):
        return self.data.data_ptr() if self.on_device else self.data.ctypes.data

    def pitch(self):
        if self.on_device:
            return self.data.stride(0) * self.data.element_size()
        return self.data.strides[0]

    def target(self):
        w, h = self.size()
        return abi.Target(self.ptr(), w, h, self.pitch(), self.fmt)

    # Texture::linear / nearest (texture.rs:59-81) -> a sampler chain
    def linear(self, texel_div=1.0):
        return Sampler(self, abi.FILTER_LINEAR, abi.WRAP_NONE, texel_div)

    def nearest(self, texel_div=1.0):
        return Sampler(self, abi.FILTER_NEAREST, abi.WRAP_NONE, texel_div)


class Empty:
    """euc's `Empty` target (texture.rs:285-319): size 0, writes dropped."""

    on_device = False

    def size(self):
        return [0, 0]

    def target(self):
        return abi.Target(None, 0, 0, 0, abi.FMT_NONE)


@dataclass
class Sampler:
    texture: Buffer2d
    filter: int
    wrap: int
    texel_div: float = 1.0

    def clamped(self):
        return Sampler(self.texture, self.filter, abi.WRAP_CLAMP, self.texel_div)

    def tiled(self):
        return Sampler(self.texture, self.filter, abi.WRAP_TILE, self.texel_div)

    def mirrored(self):
        return Sampler(self.texture, self.filter, abi.WRAP_MIRROR, self.texel_div)

    def descriptor(self):
        if self.texture.size()[0] < 1 or self.texture.size()[1] < 1:
            raise ValueError("Linearly-interpolated texture cannot have no size")  # texture.rs:63-66
        w, h = self.texture.size()
        return abi.Sampler(self.texture.ptr(), w, h, self.texture.pitch(), self.texture.fmt, self.filter, self.wrap,
                           self.texel_div, 0)


# ---------------------------------------------------------------------------
# Vertex streams (index.rs, primitives.rs)
# ---------------------------------------------------------------------------
class IndexedVertices:
    """`IndexedVertices::new(indices, vertices)` (index.rs:4-55)."""

    def __init__(self, indices, vertices):
        self.indices = indices
        self.vertices = vertices


class TriangleList:
    """`0 1 2 3 4 5` -> triangles `0 1 2`, `3 4 5` (primitives.rs:18-44)."""
    KIND = abi.PRIM_TRIANGLE_LIST


class LineTriangleList:
    """Triangles drawn as lines: `0 1 2` -> `0 1`, `1 2`, `2 0` (primitives.rs:46-77)."""
    KIND = abi.PRIM_LINE_TRIANGLE_LIST


class LineList:
    """`0 1 2 3` -> lines `0 1`, `2 3` (primitives.rs:79-104)."""
    KIND = abi.PRIM_LINE_LIST


# ---------------------------------------------------------------------------
# Pipeline (pipeline.rs:171-301)
# ---------------------------------------------------------------------------
_CONTEXTS = {}


def default_context(device=0):
    if device not in _CONTEXTS:
        _CONTEXTS[device] = capi.Context(device)
    return _CONTEXTS[device]


class Pipeline:
    """Subclass, set SHADER, implement uniforms() and vertex_layout(), and
    override the mode methods as euc's trait allows."""

    SHADER = None
    Primitives = TriangleList
    BLEND = abi.BLEND_REPLACE

    def pixel_mode(self):
        return PixelMode.WRITE

    def depth_mode(self):
        return DepthMode.NONE

    def coordinate_mode(self):
        return CoordinateMode.VULKAN

    def aa_mode(self):
        return AaMode.None_

    def rasterizer_config(self):
        return CullMode.Back

    def band_mode(self):
        return BandMode.PAR

    def uniforms(self):
        raise NotImplementedError

    def vertex_layout(self):
        raise NotImplementedError

    def desc(self):
        d = abi.PipelineDesc()
        d.shader = self.SHADER
        d.pixel_write = 1 if self.pixel_mode().write else 0
        dm = self.depth_mode()
        d.depth_test = _ORDERING[dm.test]
        d.depth_write = 1 if dm.write else 0
        cm = self.coordinate_mode()
        d.handedness = cm.handedness
        d.y_axis = cm.y_axis_direction
        if cm.z_clip_range is None:
            d.z_clip, d.z_clip_min, d.z_clip_max = 0, 0.0, 0.0
        else:
            d.z_clip, d.z_clip_min, d.z_clip_max = 1, cm.z_clip_range[0], cm.z_clip_range[1]
        d.aa_level = max(0, int(self.aa_mode().level))
        d.cull = self.rasterizer_config()
        d.blend = self.BLEND
        d.band_rows = self.band_mode()
        d.flags = 0
        d.primitives = self.Primitives.KIND
        return d

    def render(self, vertices, pixel, depth, ctx=None, stream=None, sync=True):
        """`Pipeline::render(vertices, pixel, depth)`.

        vertices: a byte/float array (numpy or CUDA tensor) of packed vertices,
        or IndexedVertices(indices, vertices).  pixel / depth: Buffer2d or
        Empty.  Host buffers render through the blocking euc_render_host;
        device buffers through euc_render on `stream` (synchronised when
        `sync`, so that errors surface here like euc's panics)."""
        ctx = ctx or default_context()
        lay = self.vertex_layout()
        idx = None
        if isinstance(vertices, IndexedVertices):
            idx, vertices = vertices.indices, vertices.vertices
        uni = self.uniforms()
        desc = self.desc()
        nbytes = vertices.nbytes if isinstance(vertices, np.ndarray) else vertices.numel() * vertices.element_size()
        nverts = nbytes // lay.stride
        on_dev = any(getattr(t, "on_device", False) for t in (pixel, depth))
        if on_dev:
            import torch
            from .frames import _stream_ptr
            vptr = vertices.data_ptr()
            iptr = idx.data_ptr() if idx is not None else None
            nidx = idx.numel() if idx is not None else 0
            sp = _stream_ptr(stream)
            rc = ctx.render(desc, uni, lay, vptr, nverts, iptr, nidx, pixel.target(), depth.target(), sp)
            capi.check(rc, "render")
            if sync:
                capi.check(ctx.sync(sp), "render")
            del torch
        else:
            v = np.ascontiguousarray(vertices)
            i = np.ascontiguousarray(idx, dtype=np.uint32) if idx is not None else None
            rc = ctx.render_host(desc, uni, lay, v.ctypes.data, nverts, i.ctypes.data if i is not None else None,
                                 i.size if i is not None else 0, pixel.target(), depth.target())
            capi.check(rc, "render")


def sampler_uniform(sampler):
    """euc_sampler for a `Sampler` (None -> an absent texture)."""
    return sampler.descriptor() if sampler is not None else abi.Sampler(None, 0, 0, 0, 0, 0, 0, 1.0, 0)


def as_floats(values, n):
    return (C.c_float * n)(*[float(v) for v in values])
