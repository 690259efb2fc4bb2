"""Known answers derived by hand from euc's Rust semantics, checked against the
CPU oracle.  The GPU path is held to the oracle on the same modes in
test_gpu_parity.py and test_gpu_errors.py.

Each expected value is worked out in the comment beside it from the cited
euc source lines, not from running any restatement.
"""
import math

import numpy as np
import pytest

from euc_gb300 import abi, scenes
from oracle import oracle

U64_MAX = (1 << 64) - 1


# --- Rust scalar semantics --------------------------------------------------
@pytest.mark.parametrize("v,expected", [
    (float("nan"), 0), (-1.5, 0), (-0.5, 0), (-0.0, 0), (0.0, 0), (0.999, 0), (1.0, 1), (2.7, 2),
    (16777216.0, 16777216), (1e30, U64_MAX), (float("inf"), U64_MAX), (float("-inf"), 0)])
def test_as_usize_saturates(v, expected):
    # `f32 as usize` saturates at both ends and maps NaN to 0 (Rust reference, "as" casts)
    assert oracle.as_usize(v) == expected


@pytest.mark.parametrize("v,expected", [
    (float("nan"), 0), (-3.0, 0), (0.5, 0), (254.9, 254), (255.0, 255), (300.0, 255), (float("inf"), 255)])
def test_as_u8_saturates(v, expected):
    assert oracle.as_u8(v) == expected


def test_fract_is_x_minus_trunc():
    assert oracle.fract(-1.25) == -0.25  # f32::fract = self - self.trunc()
    assert oracle.fract(2.5) == 0.5
    assert oracle.fract(1.0) == 0.0


def test_rem_euclid_edge_cases():
    assert oracle.rem_euclid(-0.25, 1.0) == 0.75           # r = -0.25 < 0 -> r + 1
    assert oracle.rem_euclid(1.0, 1.0) == 0.0
    r = oracle.rem_euclid(-0.0, 1.0)                        # -0.0 % 1 = -0.0, and -0.0 < 0 is false
    assert r == 0.0 and math.copysign(1.0, r) == -1.0
    assert oracle.rem_euclid(-1e-9, 1.0) == 1.0             # 1 - 1e-9 rounds to 1.0 in f32
    assert oracle.rem_euclid(2.5, 2.0) == 0.5


# --- samplers (sampler/mod.rs:100-179, linear.rs:30-66, math.rs:51-53) -----
def _sampler(tex, filt, wrap):
    return abi.Sampler(tex.ctypes.data, tex.shape[1], tex.shape[0], tex.strides[0], abi.FMT_RGBA8, filt, wrap, 1.0, 0)


@pytest.fixture
def ramp():
    tex = np.zeros((4, 8, 4), dtype=np.uint8)
    tex[..., 0] = (np.arange(8) * 10)[None, :]   # red = 10 * column
    tex[..., 1] = (np.arange(4) * 50)[:, None]   # green = 50 * row
    tex[..., 3] = 255
    return tex


def test_clamped_linear_at_one_samples_column_zero(ramp):
    s = _sampler(ramp, abi.FILTER_LINEAR, abi.WRAP_CLAMP)
    # clamp -> 1.0; 1.0.fract() == 0 (linear.rs:33) -> column 0, fract 0
    assert oracle.sample(s, 1.0, 0.0)[0] == 0.0
    assert np.array_equal(oracle.sample(s, 1.0, 0.0), oracle.sample(s, 0.0, 0.0))


def test_linear_interpolates_between_columns(ramp):
    s = _sampler(ramp, abi.FILTER_LINEAR, abi.WRAP_NONE)
    # u = 0.3125 -> 0.3125 * 8 = 2.5 -> columns 2 and 3, fract 0.5: 20*0.5 + 30*0.5 = 25
    assert oracle.sample(s, 0.3125, 0.0)[0] == 25.0
    # last column: u = 0.9375 -> 7.5 -> p0x = 7, p1x = min(8, 7) = 7: 70
    assert oracle.sample(s, 0.9375, 0.0)[0] == 70.0


def test_nearest_denormalize_clamps(ramp):
    s = _sampler(ramp, abi.FILTER_NEAREST, abi.WRAP_NONE)
    assert oracle.sample(s, 1.0, 1.0)[0] == 70.0    # (1.0 * 8) as usize = 8 -> min(7)
    assert oracle.sample(s, 1.0, 1.0)[1] == 150.0   # row 3
    assert oracle.sample(s, -0.5, 0.0)[0] == 0.0    # max(0.0) -> 0
    assert oracle.sample(s, 0.49, 0.0)[0] == 30.0   # 3.92 -> 3


def test_mirror_and_tile(ramp):
    m = _sampler(ramp, abi.FILTER_NEAREST, abi.WRAP_MIRROR)
    # 1.25: rem_euclid(2) = 1.25 >= 1 -> 1 - 0.25 = 0.75 -> column 6
    assert oracle.sample(m, 1.25, 0.0)[0] == 60.0
    t = _sampler(ramp, abi.FILTER_NEAREST, abi.WRAP_TILE)
    # -0.125 -> 0.875 -> column 7; -1e-9 -> 1.0 -> 8 -> min(7)
    assert oracle.sample(t, -0.125, 0.0)[0] == 70.0
    assert oracle.sample(t, -1e-9, 0.0)[0] == 70.0


# --- rasteriser and pipeline behaviour --------------------------------------
RED = [255, 0, 0, 255]


def _render(frame):
    tg, st, codes = oracle.run_frame(frame)
    return tg, st[0], codes[0]


def _tri(a, b, c, z=0.5, w=1.0):
    return [[a[0] * w, a[1] * w, z * w, w], [b[0] * w, b[1] * w, z * w, w], [c[0] * w, c[1] * w, z * w, w]]


def test_winding_and_cull_modes():
    ccw = _tri((-0.5, -0.5), (0.5, -0.5), (0.0, 0.5))   # cross(e1-e0, e2-e0).z = 1*1 - 0*0.5 = 1 > 0
    cw = _tri((-0.5, -0.5), (0.0, 0.5), (0.5, -0.5))    # = -1 < 0
    flat = _tri((-0.5, -0.5), (0.0, 0.0), (0.5, 0.5))   # collinear: winding 0
    for verts, cull, culled in [(ccw, abi.CULL_BACK, 0), (cw, abi.CULL_BACK, 1), (ccw, abi.CULL_FRONT, 1),
                                (cw, abi.CULL_FRONT, 0), (flat, abi.CULL_BACK, 0), (flat, abi.CULL_FRONT, 0),
                                (cw, abi.CULL_NONE, 0)]:
        # CullMode::Back culls `winding * 1.0 < 0`, Front `winding * -1.0 < 0` (triangles.rs:73-77)
        _, st, rc = _render(scenes.clip_triangles_frame(verts, [RED] * 3, 16, 16, cull=cull))
        assert rc == abi.OK and st.culled == culled, (cull, culled)


def test_full_screen_triangle_covers_every_pixel():
    # one triangle far larger than the target: every integer pixel corner is inside
    frame = scenes.clip_triangles_frame(_tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0)), [RED] * 3, 13, 9)
    tg, st, rc = _render(frame)
    assert rc == abi.OK and st.candidates == 13 * 9
    # the perspective-correct weights sum to 1 only up to rounding, and `(e * 255.0) as u8`
    # truncates: 0.99999994 * 255 = 254.99998 -> 254 (triangle.rs:24 blend)
    assert set(np.unique(tg["color"][..., 0])) <= {254, 255} and (tg["color"][..., 1:3] == 0).all()
    assert (tg["depth"] < 1.0).all() and (np.abs(tg["depth"] - 0.5) < 1e-6).all()


def test_offscreen_triangle_has_no_candidates():
    # bbox lies left of the target; the clamp to [0, W] leaves an empty range (triangles.rs:114-139)
    frame = scenes.clip_triangles_frame(_tri((-3.0, -0.5), (-2.0, -0.5), (-2.5, 0.5)), [RED] * 3, 16, 16)
    _, st, rc = _render(frame)
    assert rc == abi.OK and st.candidates == 0


def test_z_clip_rejects_fragments_outside_the_range():
    verts = _tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0), z=1.5)
    # every vertex fails 0 <= z <= 1 -> per-fragment test, z ~ 1.5 fails everywhere (pipeline.rs:151-156)
    _, st, _ = _render(scenes.clip_triangles_frame(verts, [RED] * 3, 8, 8))
    assert st.candidates == 0
    # without a clip range everything is a candidate; depth test Less vs 1.0 then fails for z = 1.5
    tg, st, _ = _render(scenes.clip_triangles_frame(verts, [RED] * 3, 8, 8, z_clip=None))
    assert st.candidates == 64 and st.passed == 0 and (tg["depth"] == 1.0).all()


def test_nan_depth_never_passes():
    frame = scenes.clip_triangles_frame(_tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0)), [RED] * 3, 8, 8,
                                        depth_clear=float("nan"))
    tg, st, _ = _render(frame)
    # z.partial_cmp(&NaN) is None, never Some(Less) (pipeline.rs:522)
    assert st.candidates == 64 and st.passed == 0 and (tg["color"] == 0).all()


def test_first_of_equal_depths_wins_with_less():
    big = _tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0))
    colors = [[255, 0, 0, 255]] * 3 + [[0, 0, 255, 255]] * 3
    tg, st, _ = _render(scenes.clip_triangles_frame(big + big, colors, 8, 8))
    # identical z: the second triangle fails `z < old` everywhere
    assert st.candidates == 128 and st.passed == 64 and (tg["color"][..., 0] == 255).all()
    tg, st, _ = _render(scenes.clip_triangles_frame(big + big, colors, 8, 8, depth_test=abi.TEST_NONE))
    # no test: both pass, the last write wins
    assert st.passed == 128 and (tg["color"][..., 2] == 255).all()


def test_par_bands_empty_small_target():
    frame = scenes.clip_triangles_frame(_tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0)), [RED] * 3, 64, 64,
                                        flags=abi.FLAG_PAR_EMPTY)
    # group_rows = 20000 / 64 = 312; needed_threads = 64 / 312 = 0 -> nothing drawn (pipeline.rs:328-330)
    tg, st, rc = _render(frame)
    assert rc == abi.OK and st.candidates == 0 and (tg["color"] == 0).all()
    # default policy: one band (render_seq semantics)
    tg, st, rc = _render(scenes.clip_triangles_frame(_tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0)), [RED] * 3, 64, 64))
    assert st.candidates == 64 * 64


def test_band_height_zero_is_an_error():
    # width 20001, level 0: group_rows = 20000 / 20001 = 0 -> division by zero panic (pipeline.rs:330)
    frame = scenes.clip_triangles_frame(_tri((-0.5, -0.5), (0.5, -0.5), (0.0, 0.5)), [RED] * 3, 20001, 1)
    _, _, rc = _render(frame)
    assert rc == abi.ERR_BAND


def test_size_mismatch_is_an_error():
    frame = scenes.clip_triangles_frame(_tri((-0.5, -0.5), (0.5, -0.5), (0.0, 0.5)), [RED] * 3, 16, 16)
    frame.targets[1] = scenes.TargetSpec("depth", 16, 15, abi.FMT_R32F, 1.0)
    _, _, rc = _render(frame)
    assert rc == abi.ERR_SIZE_MISMATCH  # assert_eq!(pixel.size(), depth.size()) (pipeline.rs:262-266)


def test_trailing_partial_primitive_is_dropped_but_its_index_is_checked():
    verts = _tri((-3.0, -3.0), (3.0, -3.0), (0.0, 5.0)) + [[0, 0, 0.5, 1]]
    f = scenes.clip_triangles_frame(verts, [RED] * 4, 8, 8, indices=[0, 1, 2, 3])
    _, st, rc = _render(f)
    assert rc == abi.OK and st.triangles == 1   # TriangleList drops the lone 4th vertex
    f = scenes.clip_triangles_frame(verts, [RED] * 4, 8, 8, indices=[0, 1, 2, 9])
    tg, _, rc = _render(f)
    assert rc == abi.ERR_INDEX_OOB and (tg["color"] == 0).all()  # the 4th index is fetched and panics


# --- geometry stages (enum euc_geometry, Pipeline::geometry) -----------------
def _geom_soup(geometry, param, **kw):
    f = scenes.soup_frame(seed=5, width=96, height=64, ntris=300, area_hi=600.0)
    f.passes[0].desc.geometry = geometry
    f.passes[0].desc.geometry_param = param
    for k, v in kw.items():
        setattr(f.passes[0].desc, k, v)
    return f


def test_geometry_duplicate_in_place_changes_nothing_under_less():
    # the copy (x += 0 * w) repeats every fragment; z == stored depth fails
    # `Less`, so only the first copy draws (pipeline.rs:519-526)
    ref = oracle.run_frame(_geom_soup(abi.GEOM_NONE, 0.0))[0]
    dup = oracle.run_frame(_geom_soup(abi.GEOM_DUPLICATE, 0.0))[0]
    assert np.array_equal(ref["color"], dup["color"]) and np.array_equal(ref["depth"], dup["depth"])


def test_geometry_discard_all_or_nothing():
    # soup z in [0.05, 0.95], w = 1: z / w > 2 never holds, z / w > -1 always does
    ref = oracle.run_frame(_geom_soup(abi.GEOM_NONE, 0.0))[0]
    keep = oracle.run_frame(_geom_soup(abi.GEOM_DISCARD, 2.0))[0]
    gone = oracle.run_frame(_geom_soup(abi.GEOM_DISCARD, -1.0))[0]
    assert np.array_equal(ref["color"], keep["color"])
    assert (gone["color"] == 0).all() and (gone["depth"] == 1.0).all()


def test_geometry_is_refused_for_lines():
    f = scenes.lines_frame(seed=1, width=32, height=32, nlines=10)
    f.passes[0].desc.geometry = abi.GEOM_SUBDIVIDE
    assert oracle.run_frame(f)[2] == [abi.ERR_INVALID]
