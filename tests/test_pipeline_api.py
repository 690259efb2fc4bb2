"""The Python mirror of euc's Pipeline API (euc_gb300.pipeline)."""
import numpy as np
import pytest

from euc_gb300 import abi, scenes
from euc_gb300.pipeline import (AaMode, Buffer2d, CoordinateMode, CullMode, DepthMode, Empty, IndexedVertices,
                                LineList, LineTriangleList, Pipeline, PixelMode, TriangleList)


class Sphere(Pipeline):
    """examples/spinning_cube.rs shape: Gouraud, LESS_WRITE, default culling."""
    SHADER = abi.SHADER_GOURAUD

    def __init__(self, spec):
        self.spec = spec

    def depth_mode(self):
        return DepthMode.LESS_WRITE

    def uniforms(self):
        return self.spec.uniforms

    def vertex_layout(self):
        return self.spec.layout


class ShadowOnly(Sphere):
    SHADER = abi.SHADER_SHADOW

    def pixel_mode(self):
        return PixelMode.PASS

    def rasterizer_config(self):
        return CullMode.None_

    def uniforms(self):
        u = abi.ShadowUniforms()
        u.mvp = self.spec.uniforms.mvp
        return u


def test_depth_mode_consts_match_euc():
    # pipeline.rs:22-46
    assert (DepthMode.NONE.test, DepthMode.NONE.write) == (None, False)
    assert (DepthMode.LESS_WRITE.test, DepthMode.LESS_WRITE.write) == ("Less", True)
    assert (DepthMode.GREATER_PASS.test, DepthMode.GREATER_PASS.write) == ("Greater", False)
    assert not DepthMode.NONE.uses_depth() and DepthMode.LESS_PASS.uses_depth()


def test_coordinate_modes_match_euc():
    # pipeline.rs:115-142
    assert CoordinateMode.VULKAN.z_clip_range == (0.0, 1.0) and CoordinateMode.VULKAN.y_axis_direction == abi.Y_DOWN
    assert CoordinateMode.OPENGL.z_clip_range == (-1.0, 1.0) and CoordinateMode.OPENGL.y_axis_direction == abi.Y_UP
    assert CoordinateMode.DIRECTX.without_z_clip().z_clip_range is None


def test_desc_from_mode_methods():
    spec = scenes.sphere_frame(seed=1).passes[0]
    d = Sphere(spec).desc()
    assert (d.shader, d.pixel_write, d.depth_test, d.depth_write) == (abi.SHADER_GOURAUD, 1, abi.TEST_LESS, 1)
    assert (d.cull, d.y_axis, d.z_clip, d.z_clip_min, d.z_clip_max) == (abi.CULL_BACK, abi.Y_DOWN, 1, 0.0, 1.0)
    assert d.aa_level == 0 and d.band_rows == abi.BANDS_PAR
    s = ShadowOnly(spec).desc()
    assert (s.pixel_write, s.cull, s.shader) == (0, abi.CULL_NONE, abi.SHADER_SHADOW)
    assert AaMode.Msaa(2).level == 2


class Wireframe(Pipeline):
    """examples/wireframes.rs: LineTriangleList, flat red, BGRA8, no depth."""
    SHADER = abi.SHADER_FLAT
    Primitives = LineTriangleList

    def __init__(self, spec):
        self.spec = spec

    def rasterizer_config(self):
        return CullMode.None_

    def uniforms(self):
        return self.spec.uniforms

    def vertex_layout(self):
        return self.spec.layout


def test_primitive_kinds_set_the_desc():
    spec = scenes.wireframe_frame(seed=1).passes[0]
    assert Wireframe(spec).desc().primitives == abi.PRIM_LINE_TRIANGLE_LIST
    assert Sphere(scenes.sphere_frame(seed=1).passes[0]).desc().primitives == abi.PRIM_TRIANGLE_LIST
    assert (TriangleList.KIND, LineTriangleList.KIND, LineList.KIND) == (0, 1, 2)


def test_buffer2d_fill_and_clear():
    b = Buffer2d.fill([5, 3], 0x11223344, fmt=abi.FMT_RGBA8)
    assert b.size() == [5, 3] and (b.data[..., 0] == 0x44).all()
    b.clear(0)
    assert (b.data == 0).all()
    d = Buffer2d.fill([5, 3], 1.0)
    assert d.fmt == abi.FMT_R32F and (d.data == 1.0).all()
    assert Empty().size() == [0, 0]


def test_buffer2d_f32_colour():
    # Buffer2d<[f32; 4]>: four floats a pixel, 16 bytes, the pitch a row of them
    b = Buffer2d.fill([5, 3], (0.25, 0.5, 0.75, 1.0), fmt=abi.FMT_RGBA32F)
    assert b.size() == [5, 3] and b.data.dtype == np.float32 and b.data.shape == (3, 5, 4)
    assert np.array_equal(b.data[2, 4], np.float32([0.25, 0.5, 0.75, 1.0]))
    t = b.target()
    assert (t.width, t.height, t.pitch, t.format) == (5, 3, 5 * 16, abi.FMT_RGBA32F)
    b.clear(0.5)
    assert (b.data == 0.5).all()
    b.clear((1.0, 2.0, 3.0, 4.0))
    assert np.array_equal(b.data[0, 0], np.float32([1.0, 2.0, 3.0, 4.0]))
    assert abi.FMT_BPP[abi.FMT_RGBA32F] == 16


@pytest.mark.gpu
@pytest.mark.parametrize("where", ["host", "device"])
def test_render_matches_oracle(where):
    from oracle import oracle
    frame = scenes.sphere_frame(seed=7)
    ref, st, _ = oracle.run_frame(frame)
    spec = frame.passes[0]
    dev = "cuda:0" if where == "device" else None
    color = Buffer2d.fill([640, 480], 0, fmt=abi.FMT_RGB8, device=dev)
    depth = Buffer2d.fill([640, 480], 1.0, device=dev)
    verts, idx = spec.vertices, spec.indices
    if dev:
        import torch
        verts = torch.from_numpy(verts).to(dev)
        idx = torch.from_numpy(idx.view(np.int32)).to(dev)
    Sphere(spec).render(IndexedVertices(idx, verts), color, depth)
    got_c = color.data.cpu().numpy() if dev else color.data
    got_d = depth.data.cpu().numpy() if dev else depth.data
    assert np.array_equal(got_c, ref["color"])
    assert np.array_equal(got_d.view(np.uint32), ref["depth"].view(np.uint32))


@pytest.mark.gpu
def test_render_errors_like_euc_panics():
    from euc_gb300.capi import EucError
    spec = scenes.sphere_frame(seed=7, width=32, height=32, lon=8, lat=4).passes[0]
    idx = spec.indices.copy()
    idx[5] = 10_000
    with pytest.raises(EucError) as e:
        Sphere(spec).render(IndexedVertices(idx, spec.vertices), Buffer2d.fill([32, 32], 0, fmt=abi.FMT_RGB8),
                            Buffer2d.fill([32, 32], 1.0))
    assert e.value.code == abi.ERR_INDEX_OOB
    with pytest.raises(EucError) as e:
        Sphere(spec).render(IndexedVertices(spec.indices, spec.vertices), Buffer2d.fill([32, 32], 0, fmt=abi.FMT_RGB8),
                            Buffer2d.fill([32, 31], 1.0))
    assert e.value.code == abi.ERR_SIZE_MISMATCH


@pytest.mark.gpu
def test_wireframe_render_matches_oracle():
    from oracle import oracle
    frame = scenes.wireframe_frame(seed=9, width=320, height=240)
    ref, _, _ = oracle.run_frame(frame)
    spec = frame.passes[0]
    color = Buffer2d.fill([320, 240], 0, fmt=abi.FMT_BGRA8)
    Wireframe(spec).render(IndexedVertices(spec.indices, spec.vertices), color, Empty())
    assert np.array_equal(color.data, ref["color"])
    assert (color.data[..., 2] == 255).sum() > 1000  # red lines in BGRA
