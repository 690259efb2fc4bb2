"""euc's panics as status codes: the GPU path returns the oracle's code for
the same inputs and draws nothing (pipeline.rs:262-266 size assert,
pipeline.rs:330 zero band height, index.rs:53 index bounds; the C ABI's own
argument checks).  Every buffer here is as large as the target it describes,
so nothing depends on a check firing to stay in bounds."""
import numpy as np
import pytest

from euc_gb300 import abi, scenes
from frameutil import run_gpu, run_oracle

pytestmark = pytest.mark.gpu

RED = [255, 0, 0, 255]


def _tri():
    return [[-0.5, -0.5, 0.5, 1.0], [0.5, -0.5, 0.5, 1.0], [0.0, 0.5, 0.5, 1.0]]


def _band_zero():
    return scenes.clip_triangles_frame(_tri(), [RED] * 3, 20001, 2)


def _size_mismatch():
    f = scenes.clip_triangles_frame(_tri(), [RED] * 3, 16, 16)
    f.targets[1] = scenes.TargetSpec("depth", 16, 15, abi.FMT_R32F, 1.0)
    return f


def _index_oob():
    verts = _tri() + [[0.0, 0.0, 0.5, 1.0]]
    return scenes.clip_triangles_frame(verts, [RED] * 4, 8, 8, indices=[0, 1, 2, 9])


def _geometry_on_lines():
    f = scenes.lines_frame(seed=1, width=32, height=32, nlines=10)
    f.passes[0].desc.geometry = abi.GEOM_SUBDIVIDE
    return f


def _bad_enum(field, value):
    def make():
        f = scenes.clip_triangles_frame(_tri(), [RED] * 3, 16, 16)
        setattr(f.passes[0].desc, field, value)
        return f
    return make


CASES = {
    "band_height_zero": (_band_zero, abi.ERR_BAND),
    "size_mismatch": (_size_mismatch, abi.ERR_SIZE_MISMATCH),
    "index_out_of_bounds": (_index_oob, abi.ERR_INDEX_OOB),
    "geometry_on_lines": (_geometry_on_lines, abi.ERR_INVALID),
    "depth_test_enum": (_bad_enum("depth_test", 7), abi.ERR_INVALID),
    "cull_enum": (_bad_enum("cull", 5), abi.ERR_INVALID),
    "primitives_enum": (_bad_enum("primitives", 9), abi.ERR_INVALID),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_status_matches_oracle_and_nothing_is_drawn(name, gpu_ctx):
    make, code = CASES[name]
    frame = make()
    ref, ref_stats = run_oracle(frame)
    got, got_stats = run_gpu(gpu_ctx, frame)
    assert ref_stats[0][0] == code
    assert got_stats[0][0] == code
    for t in frame.targets:
        clear = np.asarray(t.host_alloc())
        assert np.array_equal(got[t.name].view(np.uint8), clear.view(np.uint8)), t.name
        assert np.array_equal(ref[t.name].view(np.uint8), clear.view(np.uint8)), t.name
