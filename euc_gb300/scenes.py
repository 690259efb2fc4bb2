"""Seeded synthetic scenes for the euc triangle pipeline.

A scene is a `FrameSpec`: named targets (cleared at the start of a frame) and
an ordered list of passes, each one `Pipeline::render` call.  The same spec
is executed by the GPU path (euc_gb300.frames) and by the CPU oracle, so both
see byte-identical inputs.

Generators (all deterministic in `seed`, numpy PCG64):
  * sphere_frame  — UV sphere, Gouraud, 640x480 RGB8 (the small plain scene);
  * soup_frame    — clip-space triangle soup with log-uniform areas, per-vertex
                    RGBA8 colour (the fill-rate scene);
  * knot_frame    — (2,3) torus knot, shadow-map pass + textured Phong pass
                    with coarse-grid MSAA (the two-pass scene);
  * batch_frames  — many independent scenes of uneven size for the batched form;
  * serve_assets / serve_frame — resident meshes and textures, and two-pass
                    requests over them for the serving loop.
"""
from dataclasses import dataclass, field
import ctypes as C
import math

import numpy as np

from . import abi


# ---------------------------------------------------------------------------
# Frame description
# ---------------------------------------------------------------------------
@dataclass
class TargetSpec:
    name: str
    width: int
    height: int
    fmt: int
    clear: object  # int (packed little-endian pixel), float (depth), float or 4 floats (RGBA32F)

    @property
    def bpp(self):
        return abi.FMT_BPP[self.fmt]

    def host_alloc(self):
        if self.fmt == abi.FMT_R32F:
            return np.full((self.height, self.width), np.float32(self.clear), dtype=np.float32)
        if self.fmt == abi.FMT_RGBA32F:  # four floats a pixel
            arr = np.empty((self.height, self.width, 4), dtype=np.float32)
            arr[...] = np.asarray(self.clear, dtype=np.float32)
            return arr
        px = np.frombuffer(int(self.clear).to_bytes(8, "little")[: self.bpp], dtype=np.uint8)
        return np.ascontiguousarray(np.broadcast_to(px, (self.height, self.width, self.bpp)))


@dataclass
class SamplerSpec:
    field: str            # uniform field: "tex" or "shadow"
    source: object        # numpy texture (H,W,4 uint8 | H,W float32) or a target name
    filter: int = abi.FILTER_LINEAR
    wrap: int = abi.WRAP_TILE
    texel_div: float = 255.0


@dataclass
class PassSpec:
    desc: abi.PipelineDesc
    layout: abi.VertexLayout
    vertices: np.ndarray          # flat uint8 buffer
    nverts: int
    indices: object               # uint32 array or None
    uniforms: object              # ctypes uniform struct (sampler pointers unbound)
    samplers: list = field(default_factory=list)
    pixel: object = None          # target name or None (Empty)
    depth: object = None          # target name or None (Empty)

    def bind_uniforms(self, resolve):
        """Copy of the uniforms with sampler pointers set by `resolve(source)`.

        `resolve` returns (ptr, width, height, pitch, fmt, keepalive)."""
        uni = type(self.uniforms).from_buffer_copy(self.uniforms)
        keep = []
        for s in self.samplers:
            ptr, w, h, pitch, fmt, k = resolve(s.source)
            keep.append(k)
            setattr(uni, s.field, abi.Sampler(ptr, w, h, pitch, fmt, s.filter, s.wrap, s.texel_div, 0))
        return uni, keep

    @property
    def ntris(self):
        n = self.indices.size if self.indices is not None else self.nverts
        return n // 3


@dataclass
class FrameSpec:
    name: str
    targets: list
    passes: list
    meta: dict = field(default_factory=dict)

    def target(self, name):
        for t in self.targets:
            if t.name == name:
                return t
        raise KeyError(name)

    def alloc_host_targets(self):
        return {t.name: t.host_alloc() for t in self.targets}

    def host_texture_ptr(self, src, targets):
        arr = targets[src] if isinstance(src, str) else src
        arr = np.ascontiguousarray(arr)
        fmt = abi.FMT_R32F if arr.dtype == np.float32 else abi.FMT_RGBA8
        return arr.ctypes.data, arr.shape[1], arr.shape[0], arr.strides[0], fmt, arr

    @property
    def ntris(self):
        return sum(p.ntris for p in self.passes)

    def algorithmic_bytes(self):
        """Bytes the pipeline must move per frame: indices + vertices + each
        used target read once and written once + sampled textures once."""
        total = 0
        for p in self.passes:
            total += (p.indices.size * 4 if p.indices is not None else 0) + p.nverts * p.layout.stride
            uses_depth = p.desc.depth_test != abi.TEST_NONE or p.desc.depth_write
            if p.desc.pixel_write and p.pixel:
                t = self.target(p.pixel)
                total += 2 * t.width * t.height * t.bpp
            if uses_depth and p.depth:
                t = self.target(p.depth)
                total += 2 * t.width * t.height * 4
            for s in p.samplers:
                if isinstance(s.source, str):
                    t = self.target(s.source)
                    total += t.width * t.height * t.bpp
                else:
                    total += s.source.nbytes
        return total


def make_desc(shader, pixel_write=1, depth_test=abi.TEST_LESS, depth_write=1, y_axis=abi.Y_DOWN,
              z_clip=(0.0, 1.0), aa_level=0, cull=abi.CULL_BACK, blend=abi.BLEND_REPLACE,
              band_rows=abi.BANDS_PAR, flags=0, handedness=abi.LEFT, primitives=abi.PRIM_TRIANGLE_LIST,
              geometry=abi.GEOM_NONE, geometry_param=0.0):
    """PipelineDesc with euc's defaults (CoordinateMode::VULKAN, CullMode::Back)."""
    d = abi.PipelineDesc()
    d.shader = shader
    d.pixel_write = pixel_write
    d.depth_test = depth_test
    d.depth_write = depth_write
    d.handedness = handedness
    d.y_axis = y_axis
    if z_clip is None:
        d.z_clip, d.z_clip_min, d.z_clip_max = 0, 0.0, 0.0
    else:
        d.z_clip, d.z_clip_min, d.z_clip_max = 1, z_clip[0], z_clip[1]
    d.aa_level = aa_level
    d.cull = cull
    d.blend = blend
    d.band_rows = band_rows
    d.flags = flags
    d.primitives = primitives
    d.geometry = geometry
    d.geometry_param = geometry_param
    return d


def layout(stride, position=0, normal=-1, uv=-1, color=-1):
    return abi.VertexLayout(stride, position, normal, uv, color)


# ---------------------------------------------------------------------------
# Matrices (float64 maths, handed to the pipeline as float32 row-major)
# ---------------------------------------------------------------------------
def perspective_lh_zo(fov_y, aspect, near, far):
    f = 1.0 / math.tan(fov_y / 2.0)
    return np.array([[f / aspect, 0, 0, 0],
                     [0, f, 0, 0],
                     [0, 0, far / (far - near), -near * far / (far - near)],
                     [0, 0, 1, 0]], dtype=np.float64)


def translation(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def rotation_x(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1]], dtype=np.float64)


def rotation_y(a):
    c, s = math.cos(a), math.sin(a)
    return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1]], dtype=np.float64)


def quat_rotation(rng):
    """Uniform random rotation (Shoemake's method)."""
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    m = np.eye(4)
    m[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return m


def look_at_lh(eye, target, up):
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    z = target - eye
    z /= np.linalg.norm(z)
    x = np.cross(up, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = x, y, z
    m[:3, 3] = [-x @ eye, -y @ eye, -z @ eye]
    return m


def f32mat(m):
    return abi.mat4(np.asarray(m, dtype=np.float32).reshape(-1).tolist())


# ---------------------------------------------------------------------------
# Meshes
# ---------------------------------------------------------------------------
def uv_sphere(lon=64, lat=32, radius=1.0):
    """(lat+1)*(lon+1) vertices (seam duplicated), 2*lon*(lat-1) triangles
    (pole fans without their degenerate halves).  Returns pos, nrm, uv, idx."""
    i = np.arange(lat + 1)[:, None]
    j = np.arange(lon + 1)[None, :]
    th = i / lat * math.pi
    ph = j / lon * 2 * math.pi
    nrm = np.stack(np.broadcast_arrays(np.sin(th) * np.cos(ph), np.cos(th) + 0 * ph, np.sin(th) * np.sin(ph)),
                   axis=-1).reshape(-1, 3)
    pos = nrm * radius
    uv = np.stack(np.broadcast_arrays(j / lon + 0 * th, i / lat + 0 * ph), axis=-1).reshape(-1, 2)
    tris = []
    for r in range(lat):
        a = r * (lon + 1) + np.arange(lon)
        b = a + lon + 1
        if r != 0:
            tris.append(np.stack([a, b, a + 1], axis=-1))
        if r != lat - 1:
            tris.append(np.stack([a + 1, b, b + 1], axis=-1))
    idx = np.concatenate(tris).astype(np.uint32).reshape(-1)
    return pos, nrm, uv, idx


def torus_knot(tubular=1250, radial=200, p=2, q=3, radius=1.0, tube=0.4):
    """(tubular+1)*(radial+1) vertices, 2*tubular*radial triangles."""
    def curve(u):
        cs = np.cos(q / p * u)
        return np.stack([radius * (2 + cs) * 0.5 * np.cos(u), radius * (2 + cs) * np.sin(u) * 0.5,
                         radius * np.sin(q / p * u) * 0.5], axis=-1)

    u = np.arange(tubular + 1) / tubular * p * 2 * math.pi
    p1 = curve(u)
    p2 = curve(u + 0.01)
    t = p2 - p1
    n = p2 + p1
    b = np.cross(t, n)
    n = np.cross(b, t)
    b /= np.linalg.norm(b, axis=-1, keepdims=True)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    v = np.arange(radial + 1) / radial * 2 * math.pi
    cx = (-tube * np.cos(v))[None, :, None]
    cy = (tube * np.sin(v))[None, :, None]
    pos = p1[:, None, :] + cx * n[:, None, :] + cy * b[:, None, :]
    nrm = pos - p1[:, None, :]
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    uvs = np.stack(np.broadcast_arrays((np.arange(tubular + 1) / tubular)[:, None],
                                       (np.arange(radial + 1) / radial)[None, :]), axis=-1)
    i = np.arange(1, tubular + 1)[:, None]
    j = np.arange(1, radial + 1)[None, :]
    a = (radial + 1) * (i - 1) + (j - 1)
    bb = (radial + 1) * i + (j - 1)
    c = (radial + 1) * i + j
    d = (radial + 1) * (i - 1) + j
    idx = np.stack([a, d, bb, bb, d, c], axis=-1).astype(np.uint32).reshape(-1)
    return pos.reshape(-1, 3), nrm.reshape(-1, 3), uvs.reshape(-1, 2), idx


def pack_vertices(*attrs):
    """Interleave float32 attribute arrays into a flat uint8 buffer; returns
    (buffer, stride, byte offsets)."""
    cols = [np.asarray(a, dtype=np.float32).reshape(len(attrs[0]), -1) for a in attrs]
    offs, o = [], 0
    for c in cols:
        offs.append(o)
        o += c.shape[1] * 4
    buf = np.ascontiguousarray(np.concatenate(cols, axis=1)).view(np.uint8).reshape(-1)
    return buf, o, offs


def value_noise_texture(rng, size=1024, cells=16):
    """size x size RGBA8 seeded value noise (smoothstep-interpolated lattice)."""
    lattice = rng.random((cells + 1, cells + 1, 3))
    lattice[cells, :] = lattice[0, :]
    lattice[:, cells] = lattice[:, 0]
    t = (np.arange(size) + 0.5) / size * cells
    i0 = np.floor(t).astype(int)
    f = t - i0
    f = f * f * (3 - 2 * f)
    fy, fx = f[:, None, None], f[None, :, None]
    iy, ix = i0[:, None], i0[None, :]
    v = (lattice[iy, ix] * (1 - fx) * (1 - fy) + lattice[iy, ix + 1] * fx * (1 - fy)
         + lattice[iy + 1, ix] * (1 - fx) * fy + lattice[iy + 1, ix + 1] * fx * fy)
    rgba = np.empty((size, size, 4), dtype=np.uint8)
    rgba[..., :3] = np.clip(v * 255.0, 0, 255).astype(np.uint8)
    rgba[..., 3] = 255
    return rgba


# ---------------------------------------------------------------------------
# Frames
# ---------------------------------------------------------------------------
def sphere_frame(seed=0, width=640, height=480, lon=64, lat=32, band_rows=abi.BANDS_PAR):
    """UV sphere (pos+normal f32, u32 indices), Gouraud Lambert with one
    directional light, MVP = perspective(60 deg, W/H, 0.1, 100) * translate(0,0,3)
    * seeded rotation.  RGB8 colour + f32 depth, LESS_WRITE, back-face culling,
    Vulkan coordinates, no MSAA."""
    rng = np.random.default_rng(seed)
    pos, nrm, _, idx = uv_sphere(lon, lat)
    buf, stride, offs = pack_vertices(pos, nrm)
    model = translation(0, 0, 3) @ quat_rotation(rng)
    proj = perspective_lh_zo(math.radians(60), width / height, 0.1, 100.0)
    u = abi.GouraudUniforms()
    u.mvp = f32mat(proj @ model)
    u.model = f32mat(model)
    light = np.array([-0.4, 0.7, -0.6])
    light /= np.linalg.norm(light)
    u.to_light = (C.c_float * 3)(*light.astype(np.float32).tolist())
    u.ambient = 0.15
    u.color = (C.c_float * 3)(0.9, 0.6, 0.3)
    u.diffuse = 0.85
    p = PassSpec(make_desc(abi.SHADER_GOURAUD, cull=abi.CULL_BACK, band_rows=band_rows),
                 layout(stride, position=offs[0], normal=offs[1]), buf, len(pos), idx, u,
                 pixel="color", depth="depth")
    return FrameSpec("sphere%dx%d" % (width, height),
                     [TargetSpec("color", width, height, abi.FMT_RGB8, 0),
                      TargetSpec("depth", width, height, abi.FMT_R32F, 1.0)], [p],
                     {"seed": seed, "kind": "sphere"})


def soup_triangles(rng, ntris, width, height, area_lo=1.0, area_hi=1e4, extent=1.2, zlo=0.05, zhi=0.95):
    """Triangles with centroids ~U[-extent, extent]^2 in clip space, screen
    areas log-uniform in [area_lo, area_hi] px, random orientation and an
    anisotropy in [1/2, 2]; returns clip positions (ntris*3, 4) with w=1."""
    area = np.exp(rng.uniform(math.log(area_lo), math.log(area_hi), ntris))
    theta = rng.uniform(0, 2 * math.pi, ntris)
    k = np.exp(rng.uniform(math.log(0.5), math.log(2.0), ntris))
    base = np.array([[0.0, 1.0], [-math.sqrt(3) / 2, -0.5], [math.sqrt(3) / 2, -0.5]])
    base_area = 3 * math.sqrt(3) / 4
    s = np.sqrt(area / base_area)
    pts = base[None, :, :] * np.stack([k, 1 / k], axis=-1)[:, None, :] * s[:, None, None]
    c, sn = np.cos(theta)[:, None], np.sin(theta)[:, None]
    px = pts[..., 0] * c - pts[..., 1] * sn
    py = pts[..., 0] * sn + pts[..., 1] * c
    cen = rng.uniform(-extent, extent, (ntris, 2))
    x = cen[:, 0:1] + px * (2.0 / width)
    y = cen[:, 1:2] + py * (2.0 / height)
    z = rng.uniform(zlo, zhi, (ntris, 3))
    clip = np.stack([x, y, z, np.ones_like(z)], axis=-1).reshape(-1, 4)
    return clip


def soup_frame(seed=0, width=1920, height=1080, ntris=200_000, area_lo=1.0, area_hi=1e4,
               band_rows=abi.BANDS_PAR, alpha=False):
    """Clip-space triangle soup: x,y centroids in [-1.2, 1.2] (some cross the
    target edges), z in [0.05, 0.95], w = 1, screen areas log-uniform, per-vertex
    RGBA8 colours, a seeded-permutation u32 index buffer.  RGBA8 + f32 depth,
    LESS_WRITE, replace blend, no culling (soup orientation is random).  With
    `alpha` the colours carry alpha in [32, 255] and the blend is src-over."""
    rng = np.random.default_rng(seed)
    clip = soup_triangles(rng, ntris, width, height, area_lo, area_hi)
    nv = ntris * 3
    col = rng.integers(0, 256, (nv, 4), dtype=np.uint8)
    col[:, 3] = rng.integers(32, 256, nv, dtype=np.uint8) if alpha else 255
    perm = rng.permutation(nv).astype(np.uint32)
    vb = np.empty((nv, 20), dtype=np.uint8)
    seq = np.concatenate([clip.astype(np.float32).view(np.uint8).reshape(nv, 16), col], axis=1)
    vb[perm] = seq
    u = abi.VColorUniforms()
    u.mvp = f32mat(np.eye(4))
    p = PassSpec(make_desc(abi.SHADER_VCOLOR, cull=abi.CULL_NONE, band_rows=band_rows,
                           blend=abi.BLEND_ALPHA if alpha else abi.BLEND_REPLACE),
                 layout(20, position=0, color=16), vb.reshape(-1), nv, perm, u, pixel="color", depth="depth")
    return FrameSpec("soup%dx%d_%d" % (width, height, ntris),
                     [TargetSpec("color", width, height, abi.FMT_RGBA8, 0),
                      TargetSpec("depth", width, height, abi.FMT_R32F, 1.0)], [p],
                     {"seed": seed, "kind": "soup"})


def lines_frame(seed=0, width=640, height=360, nlines=5000, prims=abi.PRIM_LINE_LIST, len_lo=1.0, len_hi=400.0,
                extent=1.2, perspective=False, alpha=False, **desc):
    """Clip-space line soup (LineList), or the same vertices drawn as
    LineTriangleList: end points around centres ~U[-extent, extent]^2,
    screen lengths log-uniform in [len_lo, len_hi] px, z in [0.05, 0.95],
    per-vertex RGBA8 colours, a seeded-permutation u32 index buffer, RGBA8 +
    f32 depth, LESS_WRITE.  `perspective` gives each vertex a w in [0.5, 2]
    (and z beyond the clip range for some); `alpha` blends src-over."""
    rng = np.random.default_rng(seed)
    per = 2 if prims == abi.PRIM_LINE_LIST else 3
    nv = nlines * per
    cen = np.repeat(rng.uniform(-extent, extent, (nlines, 2)), per, axis=0)
    ln = np.exp(rng.uniform(math.log(len_lo), math.log(len_hi), nv))
    th = rng.uniform(0, 2 * math.pi, nv)
    x = cen[:, 0] + 0.5 * ln * np.cos(th) * (2.0 / width)
    y = cen[:, 1] + 0.5 * ln * np.sin(th) * (2.0 / height)
    z = rng.uniform(0.05, 0.95, nv)
    w = np.ones(nv)
    if perspective:
        w = rng.uniform(0.5, 2.0, nv)
        z = rng.uniform(-0.3, 1.3, nv)
    clip = np.stack([x * w, y * w, z * w, w], axis=-1).astype(np.float32)
    col = rng.integers(0, 256, (nv, 4), dtype=np.uint8)
    col[:, 3] = rng.integers(32, 256, nv, dtype=np.uint8) if alpha else 255
    perm = rng.permutation(nv).astype(np.uint32)
    vb = np.empty((nv, 20), dtype=np.uint8)
    vb[perm] = np.concatenate([clip.view(np.uint8).reshape(nv, 16), col], axis=1)
    u = abi.VColorUniforms()
    u.mvp = f32mat(np.eye(4))
    kw = dict(cull=abi.CULL_NONE, primitives=prims, blend=abi.BLEND_ALPHA if alpha else abi.BLEND_REPLACE)
    kw.update(desc)
    p = PassSpec(make_desc(abi.SHADER_VCOLOR, **kw), layout(20, position=0, color=16), vb.reshape(-1), nv, perm, u,
                 pixel="color", depth="depth")
    return FrameSpec("lines%dx%d_%d_p%d" % (width, height, nlines, prims),
                     [TargetSpec("color", width, height, abi.FMT_RGBA8, 0),
                      TargetSpec("depth", width, height, abi.FMT_R32F, 1.0)], [p],
                     {"seed": seed, "kind": "lines"})


def wireframe_frame(seed=0, width=640, height=480, lon=48, lat=24, fmt=abi.FMT_BGRA8, aa_level=0):
    """The wireframes example's pipeline (examples/wireframes.rs): a mesh drawn
    as LineTriangleList, flat red, BGRA8 colour target, no depth target (Empty,
    so no depth test and no depth write); here a UV sphere with a seeded
    rotation."""
    rng = np.random.default_rng(seed)
    pos, nrm, _, idx = uv_sphere(lon, lat)
    buf, stride, offs = pack_vertices(pos, nrm)
    mvp = perspective_lh_zo(1.3, width / height, 0.01, 100.0) @ translation(0, 0, 3.0) @ quat_rotation(rng)
    u = abi.FlatUniforms()
    u.mvp = f32mat(mvp)
    u.color = (C.c_float * 4)(1.0, 0.0, 0.0, 1.0)
    p = PassSpec(make_desc(abi.SHADER_FLAT, depth_test=abi.TEST_NONE, depth_write=0, cull=abi.CULL_NONE,
                           aa_level=aa_level, primitives=abi.PRIM_LINE_TRIANGLE_LIST),
                 layout(stride, position=offs[0], normal=offs[1]), buf, len(pos), idx, u, pixel="color", depth=None)
    return FrameSpec("wireframe%dx%d_%d" % (width, height, len(idx) // 3),
                     [TargetSpec("color", width, height, fmt, 0)], [p], {"seed": seed, "kind": "wireframe"})


def clip_triangles_frame(clip, colors, width, height, indices=None, pixel_fmt=abi.FMT_RGBA8, depth_clear=1.0,
                         color_clear=0, **desc):
    """A one-pass VCOLOR frame from explicit clip-space vertices (n, 4) and
    RGBA8 colours (n, 4); `desc` overrides make_desc's defaults."""
    clip = np.asarray(clip, dtype=np.float32).reshape(-1, 4)
    col = np.asarray(colors, dtype=np.uint8).reshape(-1, 4)
    vb = np.concatenate([clip.view(np.uint8).reshape(-1, 16), col], axis=1)
    u = abi.VColorUniforms()
    u.mvp = f32mat(np.eye(4))
    kw = dict(cull=abi.CULL_NONE)
    kw.update(desc)
    idx = None if indices is None else np.asarray(indices, dtype=np.uint32)
    p = PassSpec(make_desc(abi.SHADER_VCOLOR, **kw), layout(20, position=0, color=16),
                 np.ascontiguousarray(vb).reshape(-1), len(clip), idx, u, pixel="color", depth="depth")
    return FrameSpec("clip_tris", [TargetSpec("color", width, height, pixel_fmt, color_clear),
                                   TargetSpec("depth", width, height, abi.FMT_R32F, depth_clear)], [p])


def _phong_uniforms(model, view, proj, light_vp, light_pos, cam_pos, normal_sign=1.0):
    u = abi.PhongUniforms()
    u.model = f32mat(model)
    u.view = f32mat(view)
    u.proj = f32mat(proj)
    u.light_vp = f32mat(light_vp)
    u.light_pos = (C.c_float * 3)(*np.asarray(light_pos, dtype=np.float32).tolist())
    u.normal_sign = normal_sign
    u.cam_pos = (C.c_float * 3)(*np.asarray(cam_pos, dtype=np.float32).tolist())
    u.ambient = 0.1
    u.surf_color = (C.c_float * 4)(1.0, 0.8, 0.7, 1.0)
    return u


def knot_frame(seed=0, width=1920, height=1080, shadow_size=2048, tubular=1250, radial=200, tex_size=1024,
               aa_level=1, band_rows=abi.BANDS_PAR):
    """Two passes over a (2,3) torus knot (pos+normal+uv f32, u32 indices):
    a shadow_size^2 f32 depth-only pass from a spotlight (PixelMode::PASS,
    LESS_WRITE, no culling), then a textured Phong pass into RGBA8 + f32 depth
    with Msaa{level: aa_level}; the texture is seeded value noise sampled
    linear + tiled, the shadow map linear + clamped (examples/teapot.rs)."""
    rng = np.random.default_rng(seed)
    pos, nrm, uv, idx = torus_knot(tubular, radial)
    buf, stride, offs = pack_vertices(pos, nrm, uv)
    tex = value_noise_texture(rng, tex_size)
    yaw, pitch = rng.uniform(-math.pi, math.pi), rng.uniform(-0.5, 0.5)
    model = rotation_y(yaw) @ rotation_x(pitch)
    light_pos = np.array([-8.0, 5.0, -5.0])
    light_p = perspective_lh_zo(0.75, 1.0, 0.1, 100.0)
    light_v = look_at_lh(light_pos, [0, 0, 0], [0, 1, 0])
    light_vp = light_p @ light_v
    dist = 4.5
    view = translation(0, 0, dist)
    proj = perspective_lh_zo(1.3, width / height, 0.01, 100.0)
    cam_pos = np.linalg.inv(view)[:3, 3]
    lay = layout(stride, position=offs[0], normal=offs[1], uv=offs[2])
    su = abi.ShadowUniforms()
    su.mvp = f32mat(light_vp @ model)
    shadow_pass = PassSpec(make_desc(abi.SHADER_SHADOW, pixel_write=0, cull=abi.CULL_NONE, band_rows=band_rows),
                           lay, buf, len(pos), idx, su, pixel=None, depth="shadow")
    pu = _phong_uniforms(model, view, proj, light_vp, light_pos, cam_pos)
    color_pass = PassSpec(make_desc(abi.SHADER_PHONG, aa_level=aa_level, cull=abi.CULL_BACK, band_rows=band_rows),
                          lay, buf, len(pos), idx, pu,
                          [SamplerSpec("tex", tex, abi.FILTER_LINEAR, abi.WRAP_TILE, 255.0),
                           SamplerSpec("shadow", "shadow", abi.FILTER_LINEAR, abi.WRAP_CLAMP, 1.0)],
                          pixel="color", depth="depth")
    return FrameSpec("knot%dx%d_%d" % (width, height, 2 * tubular * radial),
                     [TargetSpec("shadow", shadow_size, shadow_size, abi.FMT_R32F, 1.0),
                      TargetSpec("color", width, height, abi.FMT_RGBA8, 0),
                      TargetSpec("depth", width, height, abi.FMT_R32F, 1.0)],
                     [shadow_pass, color_pass], {"seed": seed, "kind": "knot"})


def _mesh_for(kind, ntris, rng):
    """Mesh of about `ntris` triangles: pos, nrm, uv, idx (model space)."""
    if kind == "sphere":
        lon = max(4, int(round(math.sqrt(ntris))))
        lat = max(3, int(round(ntris / (2 * lon))) + 1)
        return uv_sphere(lon, lat)
    if kind == "knot":
        radial = max(3, int(round(math.sqrt(ntris / 12.5))))
        tubular = max(3, int(round(ntris / (2 * radial))))
        pos, nrm, uv, idx = torus_knot(tubular, radial)
        return pos * 0.6, nrm, uv, idx
    # soup in a box in front of the camera, face normals, random uvs
    area_px = rng.uniform(2.0, 200.0)
    clip = soup_triangles(rng, ntris, 256, 256, area_lo=area_px / 4, area_hi=area_px * 4, extent=1.0)
    pos = np.stack([clip[:, 0] * 1.5, clip[:, 1] * 1.5, (clip[:, 2] - 0.5) * 2.0], axis=-1)
    tri = pos.reshape(-1, 3, 3)
    fn = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    fn /= np.maximum(np.linalg.norm(fn, axis=-1, keepdims=True), 1e-12)
    nrm = np.repeat(fn, 3, axis=0)
    uv = rng.random((len(pos), 2)) * 4.0
    return pos, nrm, uv, np.arange(len(pos), dtype=np.uint32)


def batch_frames(seed=0, n=256, tri_lo=100, tri_hi=100_000, resolutions=(64, 128, 256, 512), tex_size=256,
                 band_rows=abi.BANDS_PAR):
    """n independent one-pass scenes: triangle counts log-uniform in
    [tri_lo, tri_hi] from the sphere / torus-knot / soup generators, square
    resolutions drawn uniformly from `resolutions`, half with Msaa{level: 1},
    each with its own tex_size^2 RGBA8 value-noise texture (textured Phong,
    no shadow map), seeded camera."""
    rng = np.random.default_rng(seed)
    frames = []
    for s in range(n):
        kind = ("sphere", "knot", "soup")[int(rng.integers(0, 3))]
        nt = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        res = int(resolutions[int(rng.integers(0, len(resolutions)))])
        aa = int(rng.integers(0, 2))
        pos, nrm, uv, idx = _mesh_for(kind, nt, rng)
        buf, stride, offs = pack_vertices(pos, nrm, uv)
        tex = value_noise_texture(rng, tex_size, cells=8)
        model = quat_rotation(rng)
        view = translation(0, 0, 3.2)
        proj = perspective_lh_zo(1.0, 1.0, 0.05, 50.0)
        light_pos = rng.uniform(-6, 6, 3) + np.array([0, 6, -6])
        pu = _phong_uniforms(model, view, proj, np.eye(4), light_pos, np.linalg.inv(view)[:3, 3])
        cull = abi.CULL_NONE if kind == "soup" else abi.CULL_BACK
        p = PassSpec(make_desc(abi.SHADER_PHONG, aa_level=aa, cull=cull, band_rows=band_rows),
                     layout(stride, position=offs[0], normal=offs[1], uv=offs[2]), buf, len(pos), idx, pu,
                     [SamplerSpec("tex", tex, abi.FILTER_LINEAR, abi.WRAP_TILE, 255.0)],
                     pixel="color", depth="depth")
        frames.append(FrameSpec("batch%d_%s_%d_%d_aa%d" % (s, kind, len(idx) // 3, res, aa),
                                [TargetSpec("color", res, res, abi.FMT_RGBA8, 0),
                                 TargetSpec("depth", res, res, abi.FMT_R32F, 1.0)], [p],
                                {"seed": seed, "kind": kind, "index": s}))
    return frames


@dataclass
class ServeAssets:
    """Resident inputs of the serving workload: meshes (packed vertex buffer,
    layout, vertex count, u32 indices) and RGBA8 textures."""
    meshes: list
    textures: list


def serve_assets(seed=0, nmeshes=64, ntextures=32, tex_size=512, tri_lo=100, tri_hi=100_000):
    """`nmeshes` meshes from the batch generators (sphere / torus knot / soup,
    triangle counts log-uniform in [tri_lo, tri_hi], pos+normal+uv f32) and
    `ntextures` tex_size^2 RGBA8 value-noise textures."""
    rng = np.random.default_rng(seed)
    meshes = []
    for m in range(nmeshes):
        kind = ("sphere", "knot", "soup")[int(rng.integers(0, 3))]
        nt = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        pos, nrm, uv, idx = _mesh_for(kind, nt, rng)
        buf, stride, offs = pack_vertices(pos, nrm, uv)
        meshes.append({"kind": kind, "vertices": buf, "nverts": len(pos), "indices": idx,
                       "layout": layout(stride, position=offs[0], normal=offs[1], uv=offs[2])})
    textures = [value_noise_texture(rng, tex_size, cells=8) for _ in range(ntextures)]
    return ServeAssets(meshes, textures)


def serve_frame(assets, rng, resolutions=(64, 128, 256, 512), band_rows=abi.BANDS_PAR):
    """One serving request as a FrameSpec: a resident mesh and texture drawn
    uniformly, a square resolution from `resolutions`, Msaa{level: 1} for
    half, a seeded camera and spotlight.  Two passes as in the two-pass
    shadow-mapped configuration: a res^2 f32 shadow map from the light
    (PixelMode::PASS, LESS_WRITE, no culling), then textured Phong with the
    shadow map into RGBA8 + f32 depth."""
    mi = int(rng.integers(0, len(assets.meshes)))
    ti = int(rng.integers(0, len(assets.textures)))
    res = int(resolutions[int(rng.integers(0, len(resolutions)))])
    aa = int(rng.integers(0, 2))
    m = assets.meshes[mi]
    model = quat_rotation(rng)
    view = translation(0, 0, 3.2)
    proj = perspective_lh_zo(1.0, 1.0, 0.05, 50.0)
    light_pos = rng.uniform(-3, 3, 3) + np.array([-6.0, 5.0, -5.0])
    light_vp = perspective_lh_zo(0.9, 1.0, 0.1, 100.0) @ look_at_lh(light_pos, [0, 0, 0], [0, 1, 0])
    su = abi.ShadowUniforms()
    su.mvp = f32mat(light_vp @ model)
    shadow_pass = PassSpec(make_desc(abi.SHADER_SHADOW, pixel_write=0, cull=abi.CULL_NONE, band_rows=band_rows),
                           m["layout"], m["vertices"], m["nverts"], m["indices"], su, pixel=None, depth="shadow")
    cull = abi.CULL_NONE if m["kind"] == "soup" else abi.CULL_BACK
    pu = _phong_uniforms(model, view, proj, light_vp, light_pos, np.linalg.inv(view)[:3, 3])
    color_pass = PassSpec(make_desc(abi.SHADER_PHONG, aa_level=aa, cull=cull, band_rows=band_rows),
                          m["layout"], m["vertices"], m["nverts"], m["indices"], pu,
                          [SamplerSpec("tex", assets.textures[ti], abi.FILTER_LINEAR, abi.WRAP_TILE, 255.0),
                           SamplerSpec("shadow", "shadow", abi.FILTER_LINEAR, abi.WRAP_CLAMP, 1.0)],
                          pixel="color", depth="depth")
    return FrameSpec("serve_m%d_t%d_%d_aa%d" % (mi, ti, res, aa),
                     [TargetSpec("shadow", res, res, abi.FMT_R32F, 1.0),
                      TargetSpec("color", res, res, abi.FMT_RGBA8, 0),
                      TargetSpec("depth", res, res, abi.FMT_R32F, 1.0)],
                     [shadow_pass, color_pass], {"mesh": mi, "texture": ti, "kind": "serve"})
