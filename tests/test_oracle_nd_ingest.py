"""Known answers for the oracle's N-D nearest sampler (sampler/nearest.rs,
math.rs Denormalize, buffer.rs linear_index) and texture ingest (image's
to_rgba8 expansion read through Buffer::from_texture).  Each expected value
is worked out by hand beside it."""
import numpy as np
import pytest

from euc_gb300 import abi
from oracle import oracle


def _tex1d(n):
    return np.arange(n, dtype=np.uint8).reshape(n, 1)


@pytest.mark.parametrize("u,wrap,expected", [
    (0.5, abi.WRAP_NONE, 2),     # (0.5 * 4 = 2.0).max(0) as usize = 2
    (0.99, abi.WRAP_NONE, 3),    # 3.96 -> 3
    (1.0, abi.WRAP_NONE, 3),     # 4.0 -> 4, .min(4 - 1) = 3
    (-0.1, abi.WRAP_NONE, 0),    # -0.4.max(0.0) = 0
    (float("nan"), abi.WRAP_NONE, 0),  # NaN * 4 = NaN; f32::max ignores NaN -> 0.0
    (7.0, abi.WRAP_NONE, 3),     # 28 -> .min(3)
    (1.25, abi.WRAP_TILE, 1),    # rem_euclid(1) = 0.25 -> 1.0 -> 1
    (-0.25, abi.WRAP_TILE, 3),   # rem_euclid(1) = 0.75 -> 3.0 -> 3
    (1.25, abi.WRAP_MIRROR, 3),  # rem_euclid(2) = 1.25 >= 1 -> 1 - 0.25 = 0.75 -> 3
    (0.25, abi.WRAP_MIRROR, 1),  # 0.25 < 1 -> 0.25 -> 1
    (-3.0, abi.WRAP_CLAMP, 0),   # max(0).min(1) = 0
    (3.0, abi.WRAP_CLAMP, 3),    # 1.0 -> 4 -> 3
])
def test_nearest_1d_denormalize(u, wrap, expected):
    out = oracle.sample_nearest(_tex1d(4), np.array([[u]], dtype=np.float32), wrap)
    assert out[0, 0] == expected


def test_nearest_nd_linear_index_axis0_fastest():
    # 3-D texture 5 x 3 x 2 (x fastest): texel value = x + 5 * (y + 3 * z)
    tex = np.arange(30, dtype=np.uint16).reshape(2, 3, 5)
    q = np.array([[0.1, 0.5, 0.9], [0.99, 0.0, 0.0], [0.5, 0.99, 0.5]], dtype=np.float32)
    out = oracle.sample_nearest(tex, q, abi.WRAP_NONE).view(np.uint16)[:, 0]
    # (0.5, 1.5, 1.8) -> (0, 1, 1) -> 0 + 5 * (1 + 3) = 20
    # (4.95, 0, 0) -> 4;  (2.5, 2.97, 1.0) -> (2, 2, 1) -> 2 + 5 * (2 + 3) = 27
    assert out.tolist() == [20, 4, 27]


def test_nearest_4d_multibyte_texels():
    tex = np.arange(2 * 3 * 4 * 5 * 16, dtype=np.uint8).reshape(2, 3, 4, 5, 16)
    q = np.array([[0.3, 0.6, 0.4, 0.7]], dtype=np.float32)
    # (1.5, 2.4, 1.2, 1.4) -> (1, 2, 1, 1): x + 5 (y + 4 (z + 3 w)) = 1 + 5 * (2 + 4 * (1 + 3)) = 91
    out = oracle.sample_nearest(tex, q, abi.WRAP_NONE)
    assert out[0].tolist() == tex.reshape(-1, 16)[91].tolist()


def test_nearest_refuses_empty_axes():
    with pytest.raises(ValueError):
        oracle.sample_nearest(np.zeros((0, 4), dtype=np.uint8), np.zeros((1, 1), dtype=np.float32), 0)


@pytest.mark.parametrize("fmt,pix,expected", [
    (abi.SRC_RGBA8, [10, 20, 30, 40], [10, 20, 30, 40]),
    (abi.SRC_BGRA8, [10, 20, 30, 40], [30, 20, 10, 40]),
    (abi.SRC_RGB8, [10, 20, 30], [10, 20, 30, 255]),
    (abi.SRC_LUMA8, [77], [77, 77, 77, 255]),
    (abi.SRC_LUMA_ALPHA8, [77, 9], [77, 77, 77, 9]),
])
def test_ingest_expands_like_to_rgba8(fmt, pix, expected):
    img = np.tile(np.array(pix, dtype=np.uint8), (3, 5, 1))
    out = oracle.texture_ingest(img, fmt)
    assert (out == np.array(expected, dtype=np.uint8)).all()


def test_ingest_copies_f32_bits():
    img = np.array([[1.5, -0.0, float("nan")]], dtype=np.float32)
    out = oracle.texture_ingest(img, abi.SRC_R32F)
    assert out.reshape(-1).view(np.uint32).tolist() == img.view(np.uint32).reshape(-1).tolist()
