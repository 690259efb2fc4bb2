"""euc_render_noalloc: the render entry point for callers that may not
allocate device memory (an engine or plugin host that owns a fixed
device-memory budget, or a render thread that cannot pay for the device-wide
synchronisation of cudaMalloc/cudaFree).

It is checked through the C ABI against euc_render on the same inputs, twice
in a row, because every call reuses the library's one scratch array and must
not see the previous call's leftovers, and against the CPU oracle directly.  This file sorts last so that a run
stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, capi, frames, scenes
from frameutil import assert_targets_match
from oracle import oracle

pytestmark = pytest.mark.gpu


def _render_noalloc(df, status):
    """Every pass of a DeviceFrame through euc_render_noalloc."""
    lib = capi.lib()
    sp = frames._stream_ptr(None)
    for k in range(len(df.frame.passes)):
        p, uni, keep = df.bound_pass(k)
        v, i, _ = df.passes[k]
        fmt = df.frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
        pt = frames.tensor_target(df.targets[p.pixel] if p.pixel else None, fmt)
        dt = frames.tensor_target(df.targets[p.depth] if p.depth else None, abi.FMT_R32F)
        rc = lib.euc_render_noalloc(C.byref(p.desc), C.addressof(uni), C.sizeof(uni), C.byref(p.layout),
                                    v.data_ptr(), p.nverts, i.data_ptr() if i is not None else None,
                                    i.numel() if i is not None else 0, C.byref(pt), C.byref(dt), sp,
                                    status.data_ptr())
        assert rc == abi.OK, capi.status_string(rc)
        del keep


CASES = {
    "sphere640x480": lambda: scenes.sphere_frame(seed=3),
    "soup320x180": lambda: scenes.soup_frame(seed=1, width=320, height=180, ntris=4000, area_hi=3000.0),
    "knot_shadow_msaa": lambda: scenes.knot_frame(seed=2, width=320, height=180, shadow_size=256, tubular=180,
                                                  radial=20, tex_size=64, aa_level=1),
    # line primitives: one slot per line, three per triangle of a LineTriangleList
    "lines320x180": lambda: scenes.lines_frame(seed=4, width=320, height=180, nlines=3000),
    "wireframe320x240": lambda: scenes.wireframe_frame(seed=5, width=320, height=240, lon=24, lat=12),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_noalloc_matches_render_on_two_calls(name):
    import torch
    make = CASES[name]
    frame = make()
    tol = 1 if any(p.desc.shader == abi.SHADER_PHONG for p in frame.passes) else 0
    ctx = capi.Context(0)
    try:
        ref_df = frames.DeviceFrame(frame, "cuda:0")
        frames.render_frame(ctx, ref_df)
        capi.check(ctx.sync(frames._stream_ptr(None)))
        ref = ref_df.to_host()
    finally:
        ctx.close()
    oref, _, codes = oracle.run_frame(frame)
    assert all(c == abi.OK for c in codes)
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda:0")
    for call in range(2):
        df = frames.DeviceFrame(frame, "cuda:0")
        df.clear()
        status.fill_(-1)
        _render_noalloc(df, status)
        torch.cuda.synchronize()
        assert int(status.item()) == abi.OK, "call %d" % call
        got = df.to_host()
        assert_targets_match(frame, ref, got, color_tol=tol)
        assert_targets_match(frame, oref, got, color_tol=tol)


def test_noalloc_rejects_scenes_beyond_its_limits():
    import torch
    frame = scenes.sphere_frame(seed=1, width=1100, height=1000)  # 1.1 M pixels > 1,048,576
    df = frames.DeviceFrame(frame, "cuda:0")
    df.clear()
    p, uni, keep = df.bound_pass(0)
    v, i, _ = df.passes[0]
    pt = frames.tensor_target(df.targets["color"], abi.FMT_RGB8)
    dt = frames.tensor_target(df.targets["depth"], abi.FMT_R32F)
    rc = capi.lib().euc_render_noalloc(C.byref(p.desc), C.addressof(uni), C.sizeof(uni), C.byref(p.layout),
                                       v.data_ptr(), p.nverts, i.data_ptr(), i.numel(), C.byref(pt), C.byref(dt),
                                       None, None)
    assert rc == abi.ERR_CAPACITY
    torch.cuda.synchronize()
    assert (df.targets["depth"] == 1.0).all()


def test_noalloc_reports_out_of_bounds_index_on_device():
    import torch
    frame = scenes.sphere_frame(seed=1, width=120, height=90, lon=12, lat=6)
    frame.passes[0].indices = frame.passes[0].indices.copy()
    frame.passes[0].indices[4] = frame.passes[0].nverts + 5
    df = frames.DeviceFrame(frame, "cuda:0")
    df.clear()
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda:0")
    lib = capi.lib()
    p, uni, keep = df.bound_pass(0)
    v, i, _ = df.passes[0]
    pt = frames.tensor_target(df.targets["color"], abi.FMT_RGB8)
    dt = frames.tensor_target(df.targets["depth"], abi.FMT_R32F)
    rc = lib.euc_render_noalloc(C.byref(p.desc), C.addressof(uni), C.sizeof(uni), C.byref(p.layout), v.data_ptr(),
                                p.nverts, i.data_ptr(), i.numel(), C.byref(pt), C.byref(dt), None,
                                status.data_ptr())
    assert rc == abi.OK
    torch.cuda.synchronize()
    assert int(status.item()) == abi.ERR_INDEX_OOB
    assert (df.targets["depth"] == 1.0).all() and (df.targets["color"] == 0).all()
    # the next call on the same scratch starts clean: the error flag is cleared
    # and the render matches euc_render
    frame2 = scenes.sphere_frame(seed=1, width=120, height=90, lon=12, lat=6)
    df2 = frames.DeviceFrame(frame2, "cuda:0")
    df2.clear()
    status.fill_(-1)
    _render_noalloc(df2, status)
    torch.cuda.synchronize()
    assert int(status.item()) == abi.OK
    ctx = capi.Context(0)
    try:
        ref_df = frames.DeviceFrame(frame2, "cuda:0")
        frames.render_frame(ctx, ref_df)
        capi.check(ctx.sync(frames._stream_ptr(None)))
        assert_targets_match(frame2, ref_df.to_host(), df2.to_host(), color_tol=0)
    finally:
        ctx.close()
    assert np.any(df2.to_host()["depth"] < 1.0)
