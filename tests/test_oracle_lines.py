"""The oracle's line rasteriser (euc's `Lines`, src/rasterizer/lines.rs) and its
restatement of clipline's Bresenham walk.

clipline 0.2 is a dependency of euc that is not in the reference tree, so
its exact pixel sequence is not pinned; the oracle defines it as the classic
Bresenham line (both ends included) clipped to the window.  These tests pin
that definition two ways: the closed form the kernels use equals the classic
error-term loop, and lines rendered by the oracle cover exactly those pixels.
"""
import itertools

import numpy as np
import pytest

from euc_gb300 import abi, scenes
from oracle import oracle


def bresenham_loop(x1, y1, x2, y2):
    """Classic error-term Bresenham from (x1, y1) to (x2, y2), both ends."""
    dx, dy = x2 - x1, y2 - y1
    xmaj = abs(dx) >= abs(dy)
    a1, a2, b = (x1, x2, y1) if xmaj else (y1, y2, x1)
    dmaj, dmin = (dx, dy) if xmaj else (dy, dx)
    smaj, smin = (1 if dmaj >= 0 else -1), (1 if dmin >= 0 else -1)
    amaj, amin = abs(dmaj), abs(dmin)
    err = 2 * amin - amaj
    out = []
    a = a1
    for _ in range(amaj + 1):
        out.append((a, b) if xmaj else (b, a))
        if err > 0:
            b += smin
            err -= 2 * amaj
        err += 2 * amin
        a += smaj
    return out


def bresenham_closed(x1, y1, x2, y2):
    """The closed form of the same walk: minor offset after i major steps."""
    dx, dy = x2 - x1, y2 - y1
    xmaj = abs(dx) >= abs(dy)
    a1, b1 = (x1, y1) if xmaj else (y1, x1)
    dmaj, dmin = (dx, dy) if xmaj else (dy, dx)
    smaj, smin = (1 if dmaj >= 0 else -1), (1 if dmin >= 0 else -1)
    amaj, amin = abs(dmaj), abs(dmin)
    out = []
    for i in range(amaj + 1):
        m = (2 * amin * i + amaj - 1) // (2 * amaj) if amaj else 0
        a, b = a1 + smaj * i, b1 + smin * m
        out.append((a, b) if xmaj else (b, a))
    return out


def test_closed_form_equals_error_term_loop():
    rng = np.random.default_rng(1)
    pts = [tuple(int(v) for v in rng.integers(-40, 41, 4)) for _ in range(3000)]
    pts += list(itertools.product([-3, 0, 2], [-3, 0, 2], [-3, 0, 2], [-3, 0, 2]))
    for x1, y1, x2, y2 in pts:
        assert bresenham_loop(x1, y1, x2, y2) == bresenham_closed(x1, y1, x2, y2), (x1, y1, x2, y2)


def _line_frame(ends, width=16, height=16, prims=abi.PRIM_LINE_LIST, z=(0.5, 0.5), **desc):
    """Lines between screen points: clip x = 2 sx / W - 1, y = 1 - 2 sy / H, w = 1."""
    clip, col = [], []
    for k, (sx, sy) in enumerate(ends):
        clip.append([2.0 * sx / width - 1.0, 1.0 - 2.0 * sy / height, z[k % len(z)], 1.0])
        col.append([255, 255, 255, 255])
    kw = dict(depth_test=abi.TEST_NONE, depth_write=0, primitives=prims)
    kw.update(desc)
    return scenes.clip_triangles_frame(clip, col, width, height, **kw)


def _drawn(frame):
    out = oracle.run_frame(frame, threads=1)
    img = out[0] if isinstance(out, tuple) else out
    ys, xs = np.nonzero(img["color"][..., 3])
    return set(zip(xs.tolist(), ys.tolist())), out


def _screen(frame, k):
    """The f32 screen point of vertex k as lines.rs:53-58 computes it."""
    v = np.frombuffer(frame.passes[0].vertices.tobytes(), dtype=np.float32).reshape(-1, 5)[k]
    W, H = frame.targets[0].width, frame.targets[0].height
    w = np.float32(max(v[3], np.float32(0.0001)))
    ex, ey = np.float32(v[0] / w), np.float32(v[1] / w)
    return (np.float32(W) * (ex * np.float32(0.5) + np.float32(0.5)),
            np.float32(H) * (ey * np.float32(-0.5) + np.float32(0.5)))


@pytest.mark.parametrize("ends", [
    [(2.3, 3.6), (13.7, 9.2)],     # x-major, down-right
    [(12.5, 1.5), (4.5, 14.5)],    # y-major, down-left
    [(1.5, 12.5), (14.5, 12.5)],   # horizontal
    [(3.2, 1.1), (3.9, 15.8)],     # vertical
    [(-5.0, -3.0), (20.0, 19.0)],  # crosses the target edges
])
def test_line_pixels_are_the_clipped_bresenham_walk(ends):
    f = _line_frame(ends)
    got, _ = _drawn(f)
    (sx0, sy0), (sx1, sy1) = _screen(f, 0), _screen(f, 1)
    W = H = 16
    wx1 = int(np.clip(min(sx0, sx1), 0, W)); wx2 = int(np.clip(max(sx0, sx1) + 1, 0, W)) - 1
    wy1 = int(np.clip(min(sy0, sy1), 0, H)); wy2 = int(np.clip(max(sy0, sy1) + 1, 0, H)) - 1
    want = {(x, y) for x, y in bresenham_loop(int(sx0), int(sy0), int(sx1), int(sy1))
            if wx1 <= x <= wx2 and wy1 <= y <= wy2}
    assert got == want


def test_a_point_line_has_nan_depth():
    # norm = 1 / 0 = inf, frac = (7 - 7.5) * inf = -inf, z = 0.5 + (-inf) * 0 =
    # NaN (lines.rs:76-93): the z clip (VULKAN 0..=1) rejects it; without a
    # clip range and without a depth test the pixel is emitted, its depth is
    # the NaN and its colour, weighted by the NaN frac, packs to 0
    assert _drawn(_line_frame([(7.5, 7.5), (7.5, 7.5)]))[0] == set()
    f = _line_frame([(7.5, 7.5), (7.5, 7.5)], z_clip=None, depth_write=1)
    img = oracle.run_frame(f, threads=1)[0]
    nan = np.isnan(img["depth"])
    assert nan[7, 7] and nan.sum() == 1 and (img["color"] == 0).all()


def test_line_triangle_list_draws_three_edges():
    tri = [(2.5, 2.5), (13.5, 4.5), (6.5, 13.5)]
    f = _line_frame(tri, prims=abi.PRIM_LINE_TRIANGLE_LIST)
    got, _ = _drawn(f)
    pts = [tuple(int(c) for c in _screen(f, k)) for k in range(3)]
    want = set()
    for a, b in [(0, 1), (1, 2), (2, 0)]:
        want |= set(bresenham_loop(*pts[a], *pts[b]))
    assert got == want


def test_trailing_partial_line_is_dropped():
    f = _line_frame([(1.5, 1.5), (10.5, 1.5), (3.5, 9.5)])  # 3 vertices: one line
    got, _ = _drawn(f)
    assert got == {(x, 1) for x in range(1, 11)}


def test_line_depth_is_euc_lerp_and_first_of_equal_wins():
    # line 0 z 0.25 -> 0.75 along x; line 1 covers the same row at z 0.5 flat
    ends = [(1.5, 5.5), (14.5, 5.5), (1.5, 5.5), (14.5, 5.5)]
    zs = [0.25, 0.75, 0.5, 0.5]
    clip = [[2.0 * sx / 16 - 1.0, 1.0 - 2.0 * sy / 16, z, 1.0] for (sx, sy), z in zip(ends, zs)]
    cols = [[255, 0, 0, 255], [255, 0, 0, 255], [0, 255, 0, 255], [0, 255, 0, 255]]
    f = scenes.clip_triangles_frame(clip, cols, 16, 16, primitives=abi.PRIM_LINE_LIST,
                                    depth_test=abi.TEST_LESS, depth_write=1)
    out = oracle.run_frame(f, threads=1)
    img = out[0] if isinstance(out, tuple) else out
    sx0, _ = _screen(f, 0)
    sx1, _ = _screen(f, 1)
    norm = np.float32(1.0) / np.float32(sx1 - sx0)
    for x in range(1, 15):
        frac = (np.float32(x) - sx0) * norm
        z = np.float32(np.float32(0.25) + frac * (np.float32(0.75) - np.float32(0.25)))
        green = z > np.float32(0.5)  # line 1 wins only where it is strictly nearer
        assert img["depth"][5, x] == min(z, np.float32(0.5)), x
        assert img["color"][5, x, 1] == (255 if green else 0), x


@pytest.mark.parametrize("aa", [0, 1])
def test_lines_do_not_depend_on_the_bands(aa):
    ends = [(0.5, 0.5), (15.5, 15.0), (15.2, 0.3), (0.1, 14.9), (3.3, 0.2), (4.1, 15.9)]
    a = _drawn(_line_frame(ends, aa_level=aa, band_rows=abi.BANDS_SEQ))[0]
    b = _drawn(_line_frame(ends, aa_level=aa, band_rows=1))[0]
    c = _drawn(_line_frame(ends, aa_level=aa, band_rows=5))[0]
    assert a == b == c
