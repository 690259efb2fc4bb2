"""euc_render's recorded shapes.

From the second call of a scene shape on (the same mesh and target sizes,
modes and launch shape), euc_render replays a CUDA graph recorded for that
shape, with the new call's scene table and uniforms copied in first.  Every
call must still give the oracle's image and candidate count, whatever the
uniforms, buffers, launch shape and streams of the calls around it, and a
render that moves the context's scratch buffers must retire the recorded
graphs instead of letting them touch freed memory.
"""
import pytest

from euc_gb300 import abi, capi, scenes
from frameutil import assert_targets_match, run_gpu, run_oracle

pytestmark = pytest.mark.gpu


def _check(ctx, frame, tol=0):
    got, gst = run_gpu(ctx, frame)
    ref, rst = run_oracle(frame)
    assert [c for c, _, _ in gst] == [abi.OK] * len(gst)
    assert [n for _, n, _ in gst] == [n for _, n, _ in rst], frame.name
    assert_targets_match(frame, ref, got, color_tol=tol)


def test_repeated_shape_renders_match_the_oracle():
    ctx = capi.Context(0)
    try:
        # one shape, eight rotations: the first call is plain, the second
        # records the graph, the others replay it with new uniforms
        for seed in range(8):
            _check(ctx, scenes.sphere_frame(seed=seed, width=320, height=240))
    finally:
        ctx.close()


def test_repeated_two_pass_textured_shape():
    ctx = capi.Context(0)
    try:
        # the Phong pass's uniforms hold texture and shadow-map pointers that
        # differ per frame: they travel with the replayed scene table
        for seed in range(4):
            _check(ctx, scenes.knot_frame(seed=seed, width=160, height=90, shadow_size=128, tubular=60, radial=10,
                                          tex_size=32, aa_level=1), tol=1)
    finally:
        ctx.close()


def test_shapes_across_scratch_moves_streams_and_tuning():
    import torch
    from euc_gb300 import frames
    ctx = capi.Context(0)
    try:
        small = [scenes.sphere_frame(seed=s, width=160, height=120) for s in range(4)]
        big = scenes.soup_frame(seed=2, width=640, height=360, ntris=20000, area_hi=2000.0)
        bigger = scenes.soup_frame(seed=3, width=960, height=540, ntris=60000, area_hi=2000.0)
        for f in (small[0], small[1], small[2], big, small[3], small[0], bigger, small[1], big):
            _check(ctx, f)
        ctx.set_tuning(raster_warp_rows=64, strip_path=2)  # a new launch shape is a new key
        for f in (small[2], small[3], big, big):
            _check(ctx, f)
        ctx.set_tuning(None)
        # alternate two streams: a replay waits for the shape's previous one
        side = torch.cuda.Stream()
        outs = []
        for k in range(6):
            f = small[k % 4]
            df = frames.DeviceFrame(f, "cuda:0")
            df.clear()
            torch.cuda.synchronize()
            st = side if k % 2 else torch.cuda.current_stream()
            frames.render_frame(ctx, df, st, clear=False)
            capi.check(ctx.sync(frames._stream_ptr(st)))
            outs.append((f, df.to_host()))
        for f, got in outs:
            ref, _ = run_oracle(f)
            assert_targets_match(f, ref, got)
    finally:
        ctx.close()


def test_ordered_scenes_repeat_on_the_plain_path():
    ctx = capi.Context(0)
    try:
        for _ in range(3):
            _check(ctx, scenes.soup_frame(seed=5, width=128, height=80, ntris=600, area_hi=900.0, alpha=True))
    finally:
        ctx.close()
