"""Parity at the benchmark configurations' full sizes.

The oracle renders these in about a second on the host's cores, so the GPU
output is compared with it directly, not only through size-independent
properties: the 1080p 200k-triangle soup, the two-pass 500k-triangle knot
(2048^2 shadow map, 1080p MSAA colour) and the 256-scene batch, plus the
property that the batch equals its scenes rendered one at a time, and a
16384^2 target for the index arithmetic of large targets.  Depth is
bit-exact and candidate counts exact; colour is exact except under Phong
(+-1 LSB, powf).  This file sorts late: its cases are the slowest.
"""
import numpy as np
import pytest

from euc_gb300 import abi, scenes
from euc_gb300 import frames as fr
from frameutil import assert_targets_match, run_gpu, run_oracle

pytestmark = pytest.mark.gpu


def _tol(frame):
    return 1 if any(p.desc.shader == abi.SHADER_PHONG for p in frame.passes) else 0


@pytest.mark.parametrize("name", ["soup1080p_200k", "knot_two_pass_500k"])
def test_full_size_frame_matches_oracle(name, gpu_ctx):
    from oracle import oracle
    frame = scenes.soup_frame(seed=0) if name.startswith("soup") else scenes.knot_frame(seed=0)
    ref, ref_stats = run_oracle(frame, threads=oracle.hw_threads())
    got, got_stats = run_gpu(gpu_ctx, frame)
    assert [s[0] for s in got_stats] == [abi.OK] * len(frame.passes)
    assert [s[1] for s in got_stats] == [s[1] for s in ref_stats], "candidate counts differ"
    assert_targets_match(frame, ref, got, color_tol=_tol(frame))


def test_full_batch_matches_oracle_and_per_scene(gpu_ctx):
    import torch
    from oracle import oracle
    specs = scenes.batch_frames(seed=0)  # the bench's 256 scenes
    batch = fr.DeviceBatch(specs, "cuda:0")
    fr.render_batch(gpu_ctx, batch, clear=True)
    torch.cuda.synchronize()
    batched = [df.to_host() for df in batch.frames]
    # the batch equals its scenes rendered one at a time (euc_render)
    for df, b in zip(batch.frames, batched):
        for t in df.frame.targets:  # a batch's targets clear to colour 0 and one depth value
            if t.fmt == abi.FMT_R32F:
                df.targets[t.name].fill_(batch.depth_clear)
            else:
                df.targets[t.name].zero_()
        fr.render_frame(gpu_ctx, df, clear=False)
        torch.cuda.synchronize()
        one = df.to_host()
        for k in b:
            assert np.array_equal(b[k].view(np.uint8), one[k].view(np.uint8)), (df.frame.name, k)
    # and the oracle
    threads = oracle.hw_threads()
    for f, b in zip(specs, batched):
        ref, _ = run_oracle(f, threads=threads)
        assert_targets_match(f, ref, b, color_tol=_tol(f))


def test_large_target_index_arithmetic(gpu_ctx):
    """A 16384 x 16384 target (2^28 pixels, 4 GB of targets and keys on the
    device): triangles in its corners reach row offsets beyond 2^31 bytes and
    key indices beyond 2^27; depth bit-exact, colour exact."""
    from oracle import oracle
    big = 16384
    tris = []
    for cx, cy in ((-0.9995, -0.9995), (0.9995, 0.9995), (0.9995, -0.9995), (-0.9995, 0.9995)):
        s = 0.0004
        tris += [[cx - s, cy - s, 0.25, 1.0], [cx + s, cy - s, 0.5, 1.0], [cx, cy + s, 0.75, 1.0]]
    cols = [[255, 0, 0, 255], [0, 255, 0, 255], [0, 0, 255, 255]] * 4
    frame = scenes.clip_triangles_frame(tris, cols, big, big, pixel_fmt=abi.FMT_RGBA8)
    ref, ref_stats = run_oracle(frame, threads=oracle.hw_threads())
    got, got_stats = run_gpu(gpu_ctx, frame)
    assert got_stats[0][0] == abi.OK
    assert got_stats[0][1] == ref_stats[0][1] and ref_stats[0][1] > 4 * 10
    # the drawn corners lie in both halves of the 2^31-byte row range
    ys = np.nonzero(ref["depth"] < 1.0)[0]
    assert ys.min() < 64 and ys.max() > big - 64
    assert_targets_match(frame, ref, got)
