"""Recorded batches (euc_graph_*) and launch shapes (euc_ctx_set_tuning).

Both change how a batch is launched, never what it renders: every check here
compares bytes with a plain euc_render_batch of the same batch.
"""
import pytest

from euc_gb300 import abi, capi, scenes
from euc_gb300 import frames as fr

pytestmark = pytest.mark.gpu


def _batch(seed=5, n=24, tri_hi=20_000):
    return scenes.batch_frames(seed=seed, n=n, tri_lo=50, tri_hi=tri_hi, resolutions=(64, 96, 128, 200),
                               tex_size=64)


def _knot():
    return [scenes.knot_frame(seed=s, width=160, height=96, shadow_size=128, tubular=120, radial=16, tex_size=32,
                              aa_level=s % 2) for s in range(3)]


def _render(ctx, batch):
    import torch
    fr.render_batch(ctx, batch, clear=True)
    torch.cuda.synchronize()
    return batch.color.clone(), batch.depth.clone()


def _same(a, b):
    import torch
    return torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


@pytest.mark.parametrize("which", ["mixed", "knot_two_pass"])
def test_graph_replays_are_byte_identical(which):
    import torch
    specs = _batch() if which == "mixed" else _knot()
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(specs, "cuda:0")
        ref = _render(ctx, batch)
        g = fr.BatchGraph(ctx, batch)
        for _ in range(3):  # replays start from cleared targets each time
            batch.color.fill_(7)
            g.launch()
            torch.cuda.synchronize()
            assert _same((batch.color, batch.depth), ref)
        # plain renders and replays interleave on one context
        assert _same(_render(ctx, batch), ref)
        g.launch()
        torch.cuda.synchronize()
        assert _same((batch.color, batch.depth), ref)
        g.close()
    finally:
        ctx.close()


def test_two_pass_graph_on_a_fresh_context():
    """Recording pass 1 grows the scratch that pass 0 was recorded against;
    BatchGraph records again so that every pass replays."""
    import torch
    specs = _knot()
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(specs, "cuda:0")
        g = fr.BatchGraph(ctx, batch)  # before any render on this context
        g.launch()
        torch.cuda.synchronize()
        got = (batch.color.clone(), batch.depth.clone())
        g.close()
        assert _same(got, _render(ctx, batch))
    finally:
        ctx.close()


def test_graph_sees_new_buffer_contents():
    """The graph holds pointers, not contents: new vertex data in the same
    buffers renders as a plain batch of the new data does."""
    import torch
    specs = _batch(seed=8, n=6, tri_hi=3000)
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(specs, "cuda:0")
        g = fr.BatchGraph(ctx, batch)
        for df in batch.frames:
            v = df.passes[0][0].view(torch.float32)  # interleaved f32 attributes as bytes
            v.mul_(1.0625)
        ref = _render(ctx, batch)
        g.launch()
        torch.cuda.synchronize()
        assert _same((batch.color, batch.depth), ref)
        g.close()
    finally:
        ctx.close()


def test_graph_refuses_after_scratch_moved():
    import torch
    ctx = capi.Context(0)
    try:
        small = fr.DeviceBatch(_batch(seed=1, n=2, tri_hi=500), "cuda:0")
        g = fr.BatchGraph(ctx, small)
        g.launch()
        big = fr.DeviceBatch(_batch(seed=2, n=8, tri_hi=60_000), "cuda:0")
        fr.render_batch(ctx, big)  # grows the context's scratch
        torch.cuda.synchronize()
        with pytest.raises(capi.EucError) as e:
            g.launch()
        assert e.value.code == abi.ERR_STALE
        g.close()
        g2 = fr.BatchGraph(ctx, small)  # recreated against the new scratch
        ref = _render(ctx, small)
        g2.launch()
        torch.cuda.synchronize()
        assert _same((small.color, small.depth), ref)
        g2.close()
    finally:
        ctx.close()


def test_graph_rejects_ordered_scenes():
    ctx = capi.Context(0)
    try:
        f = scenes.soup_frame(seed=1, width=96, height=64, ntris=200, area_hi=400.0, alpha=True)
        batch = fr.DeviceBatch([f], "cuda:0")
        with pytest.raises(capi.EucError) as e:
            fr.BatchGraph(ctx, batch)
        assert e.value.code == abi.ERR_INVALID
    finally:
        ctx.close()


SHAPES = [
    dict(raster_warp_rows=32),
    dict(raster_warp_rows=96, raster_blocks_per_sm=1),
    dict(raster_blocks_per_sm=9),
    dict(chunk_group=1, chunk_blocks_per_sm=1),
    dict(chunk_group=7, chunk_blocks_per_sm=3),
    dict(chunk_group=1024, chunk_blocks_per_sm=64, raster_warp_rows=224, raster_blocks_per_sm=2),
    dict(raster_probe=2),
    dict(raster_probe=1, raster_warp_rows=64),
    dict(strip_path=1),
    dict(strip_path=2),
    dict(strip_path=2, raster_warp_rows=64, chunk_group=1),
]


@pytest.mark.parametrize("which", ["mixed", "knot_two_pass", "alpha"])
def test_launch_shapes_do_not_change_results(which):
    if which == "mixed":
        specs = _batch(seed=11, n=16)
    elif which == "knot_two_pass":
        specs = _knot()
    else:
        specs = [scenes.soup_frame(seed=s, width=128, height=80, ntris=600, area_hi=900.0, alpha=True)
                 for s in range(3)]
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(specs, "cuda:0")
        ref = _render(ctx, batch)
        for shape in SHAPES:
            ctx.set_tuning(**shape)
            t = ctx.get_tuning().as_dict()
            assert all(t[k] == v for k, v in shape.items())
            assert _same(_render(ctx, batch), ref), shape
        ctx.set_tuning(None)
        assert ctx.get_tuning().as_dict() == {k: 0 for k in t}
    finally:
        ctx.close()


@pytest.mark.parametrize("bad", [dict(raster_warp_rows=48), dict(raster_warp_rows=288),
                                 dict(raster_blocks_per_sm=65), dict(chunk_group=1025),
                                 dict(chunk_blocks_per_sm=100), dict(raster_probe=3),
                                 dict(strip_path=3)])
def test_invalid_launch_shapes_are_refused(bad):
    ctx = capi.Context(0)
    try:
        with pytest.raises(capi.EucError) as e:
            ctx.set_tuning(**bad)
        assert e.value.code == abi.ERR_INVALID
        assert ctx.get_tuning().as_dict() == {k: 0 for k, _ in abi.Tuning._fields_}
    finally:
        ctx.close()


def test_autotune_picks_a_shape_with_identical_output(tmp_path):
    from euc_gb300 import autotune
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(_batch(seed=13, n=12, tri_hi=8000), "cuda:0")
        ref = _render(ctx, batch)
        cache = str(tmp_path / "tune.json")
        t, info = autotune.tune(ctx, batch, reps=2, cache=cache)
        assert not info["cached"] and info["tried"] >= 2
        assert ctx.get_tuning().as_dict() == t.as_dict()
        assert _same(_render(ctx, batch), ref)
        t2, info2 = autotune.tune(ctx, batch, reps=2, cache=cache)
        assert info2["cached"] and t2.as_dict() == t.as_dict()
    finally:
        ctx.close()
