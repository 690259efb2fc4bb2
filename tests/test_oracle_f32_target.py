"""An f32 colour target (EUC_FMT_RGBA32F, euc's Buffer2d<[f32; 4]>) keeps each
winning fragment as it is; an 8-bit target stores `(pack(c)) as u8`.  With
the REPLACE blend the two must agree: the oracle renders the same inputs into
both, and packing the f32 target with the shader's own pack and the
saturating `as u8` gives the 8-bit target byte for byte (MSAA's coarse
combine happens before either store).  CPU only."""
import numpy as np
import pytest

from euc_gb300 import abi, scenes


def _pack(shader, c):
    c = c.astype(np.float32)
    if shader == abi.SHADER_TEXTURED:
        return c  # `e as u8`
    if shader == abi.SHADER_PHONG:
        return np.minimum(np.maximum(c, np.float32(0.0)), np.float32(1.0)) * np.float32(255.0)
    return c * np.float32(255.0)  # flat, vertex colour, Gouraud: (e * 255.0) as u8


def _as_u8(v):
    out = np.trunc(np.where(np.isnan(v) | (v < 1.0), 0.0, np.minimum(v, 255.0)))
    return out.astype(np.uint8)


def _with_color(frame, fmt, clear):
    t = frame.target("color")
    frame.targets[frame.targets.index(t)] = scenes.TargetSpec("color", t.width, t.height, fmt, clear)
    return frame


FRAMES = {
    "sphere_gouraud": lambda: scenes.sphere_frame(seed=3, width=96, height=64, lon=16, lat=8),
    "soup_vcolor": lambda: scenes.soup_frame(seed=2, width=80, height=48, ntris=300, area_hi=400.0),
    "knot_phong_msaa": lambda: scenes.knot_frame(seed=1, width=64, height=40, shadow_size=64, tubular=40, radial=8,
                                                 tex_size=16, aa_level=1),
}


@pytest.mark.parametrize("name", sorted(FRAMES))
def test_f32_target_packs_to_the_8bit_target(name):
    from oracle import oracle
    f8 = FRAMES[name]()
    fmt8 = f8.target("color").fmt
    f8 = _with_color(f8, fmt8, 0)
    f32 = _with_color(FRAMES[name](), abi.FMT_RGBA32F, 0.0)
    shader = [p.desc.shader for p in f8.passes if p.pixel == "color"][-1]
    t8, _, c8 = oracle.run_frame(f8)
    t32, _, c32 = oracle.run_frame(f32)
    assert c8 == c32 == [abi.OK] * len(f8.passes)
    for name_t in ("depth", "shadow"):  # the other targets are untouched by the colour format
        if name_t in t8:
            assert np.array_equal(t8[name_t].view(np.uint32), t32[name_t].view(np.uint32))
    packed = _as_u8(_pack(shader, t32["color"]))
    got8 = t8["color"]
    order = {abi.FMT_RGBA8: [0, 1, 2, 3], abi.FMT_BGRA8: [2, 1, 0, 3], abi.FMT_RGB8: [0, 1, 2]}[fmt8]
    want = packed[..., order]
    assert want.shape == got8.shape
    bad = np.argwhere(want != got8)
    assert bad.size == 0, "%d channels differ, first at %s: f32 %r packs to %r, 8-bit %r" % (
        len(bad), bad[0].tolist(), t32["color"][tuple(bad[0][:2])], want[tuple(bad[0][:2])], got8[tuple(bad[0][:2])])
