"""Generates the golden fixtures in this directory.

    python tests/golden/make_golden.py

Each fixture holds a small scene's full inputs and the CPU oracle's outputs
(targets and per-pass candidate-fragment counts).  euc itself cannot run in
this environment (no Rust toolchain), so these fixtures pin regressions of
the oracle and of the GPU path; they are checked by tests/test_golden.py.
The pure-Python restatement (oracle/euc_pyref.py) reproduces every fixture.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

from euc_gb300 import abi, scenes  # noqa: E402
from oracle import oracle  # noqa: E402
import golden_io  # noqa: E402


def textured_frame():
    rng = np.random.default_rng(21)
    pos, _, uv, idx = scenes.uv_sphere(10, 5)
    uv = uv * 2.5 - 0.75
    buf, stride, offs = scenes.pack_vertices(pos, uv)
    mvp = scenes.perspective_lh_zo(1.0, 1.0, 0.1, 10.0) @ scenes.translation(0, 0, 2.5) @ scenes.quat_rotation(rng)
    u = abi.TexturedUniforms()
    u.mvp = scenes.f32mat(mvp)
    tex = rng.integers(0, 256, (5, 7, 4), dtype=np.uint8)
    p = scenes.PassSpec(scenes.make_desc(abi.SHADER_TEXTURED), scenes.layout(stride, position=offs[0], uv=offs[1]),
                        buf, len(pos), idx, u, [scenes.SamplerSpec("tex", tex, abi.FILTER_NEAREST, abi.WRAP_MIRROR, 1.0)],
                        pixel="color", depth="depth")
    return scenes.FrameSpec("textured32", [scenes.TargetSpec("color", 32, 32, abi.FMT_RGBA8, 0),
                                           scenes.TargetSpec("depth", 32, 32, abi.FMT_R32F, 1.0)], [p])


FIXTURES = {
    "sphere64x48": lambda: scenes.sphere_frame(seed=31, width=64, height=48, lon=16, lat=8),
    "sphere_bands5": lambda: scenes.sphere_frame(seed=32, width=50, height=40, lon=12, lat=6, band_rows=5),
    "soup64x48": lambda: scenes.soup_frame(seed=33, width=64, height=48, ntris=120, area_lo=2.0, area_hi=600.0),
    "knot48x32_msaa1": lambda: scenes.knot_frame(seed=34, width=48, height=32, shadow_size=32, tubular=30, radial=8,
                                                 tex_size=16, aa_level=1, band_rows=7),
    "knot40x40_msaa2": lambda: scenes.knot_frame(seed=35, width=40, height=40, shadow_size=24, tubular=24, radial=6,
                                                 tex_size=8, aa_level=2),
    "textured32": textured_frame,
}


def main():
    for name, make in FIXTURES.items():
        frame = make()
        targets, stats, codes = oracle.run_frame(frame)
        assert all(c == abi.OK for c in codes), (name, codes)
        golden_io.save(os.path.join(HERE, name + ".npz"), frame, targets,
                       [[int(s.candidates), int(s.culled), int(s.passed)] for s in stats])
        print(name, [int(s.candidates) for s in stats])


if __name__ == "__main__":
    main()
