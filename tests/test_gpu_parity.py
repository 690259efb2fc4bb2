"""GPU pipeline vs the CPU oracle on the same seeded inputs.

Bar: depth bit-exact, per-pass candidate-fragment counts exact, colour exact
for shaders without transcendental functions and within +-1 LSB per 8-bit
channel for the Phong shader (its lighting uses the hardware reciprocal square
root and power; texel and shadow-map coordinates stay exact); on an f32 colour
target Phong within a relative 1e-5, the others bit-exact.
"""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, scenes
from frameutil import assert_same_inputs, assert_targets_match, run_gpu, run_oracle

pytestmark = pytest.mark.gpu


def _sphere(seed=3, **kw):
    return lambda: scenes.sphere_frame(seed=seed, **kw)


def _mod(make, **desc):
    def wrapped():
        f = make()
        for p in f.passes:
            for k, v in desc.items():
                setattr(p.desc, k, v)
        return f
    return wrapped


def _soup(seed=1, w=320, h=180, n=4000, hi=3000.0, alpha=False, **desc):
    return _mod(lambda: scenes.soup_frame(seed=seed, width=w, height=h, ntris=n, area_hi=hi, alpha=alpha), **desc)


def _fmt(make, fmt):
    def wrapped():
        f = make()
        t = f.target("color")
        f.targets[f.targets.index(t)] = scenes.TargetSpec("color", t.width, t.height, fmt, 0x80402010)
        return f
    return wrapped


def _f32(make, clear=(0.25, 0.5, 0.75, 1.0)):
    """The colour target as four floats a pixel (Buffer2d<[f32; 4]>)."""
    def wrapped():
        f = make()
        t = f.target("color")
        f.targets[f.targets.index(t)] = scenes.TargetSpec("color", t.width, t.height, abi.FMT_RGBA32F, clear)
        return f
    return wrapped


def _clear(make, name, value):
    def wrapped():
        f = make()
        f.target(name).clear = value
        return f
    return wrapped


def _perspective_soup(seed=7, zclip=True):
    """Soup with w != 1 and z outside the clip range (per-fragment z clip)."""
    def make():
        f = scenes.soup_frame(seed=seed, width=257, height=131, ntris=3000, area_hi=4000.0)
        p = f.passes[0]
        rng = np.random.default_rng(seed + 100)
        vb = p.vertices.reshape(p.nverts, 20).copy()
        pos = vb[:, :16].copy().view(np.float32).reshape(-1, 4)
        w = rng.uniform(0.5, 2.0, len(pos)).astype(np.float32)
        pos[:, 0] *= w
        pos[:, 1] *= w
        pos[:, 2] = rng.uniform(-0.3, 1.3, len(pos)).astype(np.float32) * w
        pos[:, 3] = w
        vb[:, :16] = pos.view(np.uint8).reshape(-1, 16)
        p.vertices = vb.reshape(-1)
        if not zclip:
            p.desc.z_clip = 0
        return f
    return make


def _knot(aa, seed=2, w=320, h=180, shadow=256):
    return lambda: scenes.knot_frame(seed=seed, width=w, height=h, shadow_size=shadow, tubular=180, radial=20,
                                     tex_size=64, aa_level=aa)


def _textured(filt, wrap, seed=4, w=200, h=150):
    def make():
        rng = np.random.default_rng(seed)
        pos, nrm, uv, idx = scenes.uv_sphere(20, 10)
        uv = uv * 3.0 - 1.0  # exercise the wrap modes outside [0, 1]
        buf, stride, offs = scenes.pack_vertices(pos, uv)
        model = scenes.translation(0, 0, 2.6) @ scenes.quat_rotation(rng)
        proj = scenes.perspective_lh_zo(1.0, w / h, 0.1, 50.0)
        u = abi.TexturedUniforms()
        u.mvp = scenes.f32mat(proj @ model)
        tex = rng.integers(0, 256, (13, 17, 4), dtype=np.uint8)
        p = scenes.PassSpec(scenes.make_desc(abi.SHADER_TEXTURED), scenes.layout(stride, position=offs[0], uv=offs[1]),
                            buf, len(pos), idx, u, [scenes.SamplerSpec("tex", tex, filt, wrap, 1.0)],
                            pixel="color", depth="depth")
        return scenes.FrameSpec("tex", [scenes.TargetSpec("color", w, h, abi.FMT_BGRA8, 0x20406080),
                                        scenes.TargetSpec("depth", w, h, abi.FMT_R32F, 1.0)], [p])
    return make


def _flat(seed=6):
    def make():
        f = scenes.sphere_frame(seed=seed, width=160, height=120, lon=16, lat=8)
        p = f.passes[0]
        u = abi.FlatUniforms()
        u.mvp = p.uniforms.mvp
        u.color = (C.c_float * 4)(0.25, 0.5, 0.75, 1.0)
        p.uniforms = u
        p.desc.shader = abi.SHADER_FLAT
        return f
    return make


def _unindexed():
    def make():
        f = scenes.soup_frame(seed=9, width=150, height=100, ntris=500, area_hi=800.0)
        p = f.passes[0]
        nv = p.nverts
        vb = p.vertices.reshape(nv, 20)[p.indices].reshape(-1)  # un-permute
        p.vertices = np.ascontiguousarray(vb)
        p.indices = None
        return f
    return make


def _ragged(nverts, prims=abi.PRIM_TRIANGLE_LIST, indexed=False):
    """A stream of `nverts` vertices: empty, or shorter than one primitive."""
    def make():
        rng = np.random.default_rng(nverts)
        clip = np.concatenate([rng.uniform(-0.9, 0.9, (nverts, 2)), rng.uniform(0.1, 0.9, (nverts, 1)),
                               np.ones((nverts, 1))], axis=1)
        col = np.full((nverts, 4), 200, dtype=np.uint8)
        idx = np.arange(nverts, dtype=np.uint32)[::-1].copy() if indexed else None
        return scenes.clip_triangles_frame(clip, col, 32, 24, indices=idx, primitives=prims)
    return make


def _lines(seed=31, prims=abi.PRIM_LINE_LIST, **kw):
    return lambda: scenes.lines_frame(seed=seed, prims=prims, **kw)


CASES = {
    "sphere640x480": (_sphere(seed=3), 0),
    "sphere_small_odd": (_sphere(seed=5, width=97, height=61, lon=24, lat=12), 0),
    "sphere_cull_none": (_mod(_sphere(seed=8), cull=abi.CULL_NONE), 0),
    "sphere_cull_front_yup": (_mod(_sphere(seed=8), cull=abi.CULL_FRONT, y_axis=abi.Y_UP), 0),
    "sphere_bands_seq": (_mod(_sphere(seed=11), band_rows=abi.BANDS_SEQ), 0),
    "sphere_bands_7": (_mod(_sphere(seed=11), band_rows=7), 0),
    "sphere_par_small_fallback": (_sphere(seed=12, width=64, height=64, lon=16, lat=8), 0),
    "sphere_par_empty": (_mod(_sphere(seed=12, width=64, height=64, lon=16, lat=8), flags=abi.FLAG_PAR_EMPTY), 0),
    "soup_less": (_soup(), 0),
    "soup_greater": (_clear(_soup(seed=2, depth_test=abi.TEST_GREATER), "depth", 0.0), 0),
    "soup_equal_write": (_clear(_soup(seed=3, depth_test=abi.TEST_EQUAL), "depth", 0.5), 0),
    "soup_none_write": (_soup(seed=4, depth_test=abi.TEST_NONE), 0),
    "soup_less_pass": (_soup(seed=5, depth_write=0), 0),
    "soup_depth_only": (_soup(seed=6, pixel_write=0), 0),
    "soup_color_only": (_soup(seed=13, depth_test=abi.TEST_NONE, depth_write=0), 0),
    "soup_perspective_zclip": (_perspective_soup(7, True), 0),
    "soup_perspective_noclip": (_perspective_soup(8, False), 0),
    "soup_large_tris": (_soup(seed=14, w=640, h=360, n=300, hi=150000.0), 0),
    "knot_aa0": (_knot(0), 1),
    "knot_aa1": (_knot(1), 1),
    "knot_aa2": (_knot(2, seed=3), 1),
    "knot_aa3": (_knot(3, seed=4, w=333, h=211), 1),
    "tex_linear_tile": (_textured(abi.FILTER_LINEAR, abi.WRAP_TILE), 0),
    "tex_linear_clamp": (_textured(abi.FILTER_LINEAR, abi.WRAP_CLAMP), 0),
    "tex_linear_mirror": (_textured(abi.FILTER_LINEAR, abi.WRAP_MIRROR), 0),
    "tex_linear_none": (_textured(abi.FILTER_LINEAR, abi.WRAP_NONE), 0),
    "tex_nearest_tile": (_textured(abi.FILTER_NEAREST, abi.WRAP_TILE), 0),
    "tex_nearest_clamp": (_textured(abi.FILTER_NEAREST, abi.WRAP_CLAMP), 0),
    "tex_nearest_mirror": (_textured(abi.FILTER_NEAREST, abi.WRAP_MIRROR), 0),
    "tex_nearest_none": (_textured(abi.FILTER_NEAREST, abi.WRAP_NONE), 0),
    "flat": (_flat(), 0),
    "f32_sphere": (_f32(_sphere(seed=3)), 0),
    "f32_flat": (_f32(_flat()), 0),
    "f32_tex_linear_tile": (_f32(_textured(abi.FILTER_LINEAR, abi.WRAP_TILE)), 0),
    "f32_soup_less": (_f32(_soup(seed=2)), 0),
    "f32_alpha_soup": (_f32(_soup(seed=21, alpha=True)), 0),
    "f32_alpha_soup_msaa1": (_f32(_soup(seed=24, alpha=True, aa_level=1)), 0),
    "f32_knot_aa1": (_f32(_knot(1)), 1),
    "unindexed": (_unindexed(), 0),
    # order-dependent blend: per-pixel fragment lists replayed in order
    "alpha_soup_less": (_soup(seed=21, alpha=True), 0),
    "alpha_soup_less_pass": (_soup(seed=22, alpha=True, depth_write=0), 0),
    "alpha_soup_no_depth": (_soup(seed=23, alpha=True, depth_test=abi.TEST_NONE, depth_write=0), 0),
    "alpha_soup_msaa1": (_soup(seed=24, alpha=True, aa_level=1), 0),
    "alpha_soup_msaa2_bands": (_soup(seed=25, w=333, h=177, alpha=True, aa_level=2, band_rows=11), 0),
    "alpha_soup_rgb8": (_fmt(_soup(seed=26, alpha=True), abi.FMT_RGB8), 0),
    "alpha_soup_bgra8": (_fmt(_soup(seed=27, alpha=True), abi.FMT_BGRA8), 0),
    # replace blends forced through the ordered path must give the same bytes
    # empty and ragged streams: nothing is drawn (primitives.rs collect_primitive)
    "empty_stream": (_ragged(0), 0),
    "empty_indexed": (_ragged(0, indexed=True), 0),
    "two_vertices": (_ragged(2), 0),
    "five_vertices_indexed": (_ragged(5, indexed=True), 0),
    "one_vertex_lines": (_ragged(1, prims=abi.PRIM_LINE_LIST), 0),
    "five_vertices_line_tris": (_ragged(5, prims=abi.PRIM_LINE_TRIANGLE_LIST), 0),
    # lines (lines.rs) and the wireframe example's LineTriangleList pipeline
    "lines_less": (_lines(), 0),
    "lines_tri_list": (_lines(seed=32, prims=abi.PRIM_LINE_TRIANGLE_LIST, nlines=2000), 0),
    "lines_perspective_zclip": (_lines(seed=33, perspective=True), 0),
    "lines_perspective_noclip": (_lines(seed=34, perspective=True, z_clip=None, depth_test=abi.TEST_NONE), 0),
    "lines_equal_pass": (_clear(_lines(seed=35, depth_test=abi.TEST_EQUAL, depth_write=0), "depth", 0.5), 0),
    "lines_msaa1_bands": (_lines(seed=36, width=333, height=177, aa_level=1, band_rows=9), 0),
    "lines_msaa2": (_lines(seed=37, aa_level=2), 0),
    "lines_long_offscreen": (_lines(seed=38, nlines=300, len_lo=500.0, len_hi=5000.0, extent=2.0), 0),
    "lines_alpha": (_lines(seed=39, alpha=True), 0),
    "lines_ordered": (_lines(seed=40, flags=abi.FLAG_ORDERED), 0),
    "wireframe_bgra8": (lambda: scenes.wireframe_frame(seed=41), 0),
    "wireframe_msaa1_rgba8": (lambda: scenes.wireframe_frame(seed=42, fmt=abi.FMT_RGBA8, aa_level=1), 0),
    # built-in geometry stages (Pipeline::geometry)
    "geom_sphere_subdivide": (_mod(_sphere(seed=43), geometry=abi.GEOM_SUBDIVIDE), 0),
    "geom_soup_shrink": (_soup(seed=44, geometry=abi.GEOM_SHRINK, geometry_param=0.6), 0),
    "geom_soup_duplicate": (_soup(seed=45, geometry=abi.GEOM_DUPLICATE, geometry_param=0.05), 0),
    "geom_soup_discard": (_soup(seed=46, geometry=abi.GEOM_DISCARD, geometry_param=0.5), 0),
    "geom_knot_subdivide_aa1": (_mod(_knot(1, seed=47), geometry=abi.GEOM_SUBDIVIDE), 1),
    "geom_tex_shrink": (_mod(_textured(abi.FILTER_LINEAR, abi.WRAP_TILE, seed=48), geometry=abi.GEOM_SHRINK,
                             geometry_param=0.8), 0),
    "geom_alpha_duplicate": (_soup(seed=49, alpha=True, geometry=abi.GEOM_DUPLICATE, geometry_param=-0.03), 0),
    "ordered_sphere": (_mod(_sphere(seed=3), flags=abi.FLAG_ORDERED), 0),
    "ordered_soup_less": (_soup(seed=1, flags=abi.FLAG_ORDERED), 0),
    "ordered_soup_equal": (_clear(_soup(seed=3, depth_test=abi.TEST_EQUAL, flags=abi.FLAG_ORDERED), "depth", 0.5), 0),
    "ordered_soup_greater": (_clear(_soup(seed=2, depth_test=abi.TEST_GREATER, flags=abi.FLAG_ORDERED), "depth", 0.0), 0),
    "ordered_knot_aa1": (_mod(_knot(1), flags=abi.FLAG_ORDERED), 1),
    "ordered_tex_linear_mirror": (_mod(_textured(abi.FILTER_LINEAR, abi.WRAP_MIRROR), flags=abi.FLAG_ORDERED), 0),
}


_ORACLE = {}


def _oracle(name):
    """The oracle's targets and statistics of case `name`, computed once."""
    if name not in _ORACLE:
        _ORACLE[name] = run_oracle(CASES[name][0]())
    return _ORACLE[name]


@pytest.fixture(scope="module")
def strip_ctx():
    """A context that sends every scene the shared-memory strips can take to
    them, whatever its overdraw (the default routes only overdrawn scenes)."""
    from euc_gb300 import capi
    ctx = capi.Context(0)
    ctx.set_tuning(strip_path=2)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_oracle(name, gpu_ctx):
    make, tol = CASES[name]
    assert_same_inputs(make(), make())
    ref, ref_stats = _oracle(name)
    got, got_stats = run_gpu(gpu_ctx, make())
    assert [s[0] for s in got_stats] == [s[0] for s in ref_stats]
    assert [s[1] for s in got_stats] == [s[1] for s in ref_stats], "candidate fragment counts"
    assert [s[2] for s in got_stats] == [s[2] for s in ref_stats], "culled primitive counts"
    assert_targets_match(make(), ref, got, color_tol=tol)


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_oracle_on_the_strips(name, strip_ctx):
    make, tol = CASES[name]
    ref, ref_stats = _oracle(name)
    got, got_stats = run_gpu(strip_ctx, make())
    assert [s[0] for s in got_stats] == [s[0] for s in ref_stats]
    assert [s[1] for s in got_stats] == [s[1] for s in ref_stats], "candidate fragment counts"
    assert [s[2] for s in got_stats] == [s[2] for s in ref_stats], "culled primitive counts"
    assert_targets_match(make(), ref, got, color_tol=tol)


@pytest.mark.parametrize("strips", [False, True])
def test_index_out_of_bounds_draws_nothing(gpu_ctx, strip_ctx, strips):
    ctx = strip_ctx if strips else gpu_ctx
    def make():
        f = scenes.sphere_frame(seed=1, width=120, height=90, lon=12, lat=6)
        f.passes[0].indices = f.passes[0].indices.copy()
        f.passes[0].indices[-1] = f.passes[0].nverts  # one past the end: index.rs:53 panics
        return f
    ref, ref_stats = run_oracle(make())
    got, got_stats = run_gpu(ctx, make())
    assert ref_stats[0][0] == abi.ERR_INDEX_OOB
    assert got_stats[0][0] == abi.ERR_INDEX_OOB
    clean = make().alloc_host_targets()
    for k in clean:
        assert np.array_equal(got[k], clean[k])
