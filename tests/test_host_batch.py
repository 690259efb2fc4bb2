"""euc_render_host_batch (host buffers, one call per pass) against the
oracle and against euc_render_host per scene: byte-identical targets, under either way of
moving host buffers (page-locked staging, or kernels that read and write
host memory directly)."""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, capi, scenes
from frameutil import assert_targets_match, run_oracle

pytestmark = pytest.mark.gpu


def _host_scene(f, p, h, keep):
    uni, kp = p.bind_uniforms(lambda src: f.host_texture_ptr(src, h))
    keep.append((uni, kp))
    s = abi.Scene()
    s.desc = p.desc
    s.layout = p.layout
    s.vertices = p.vertices.ctypes.data
    s.nverts = p.nverts
    s.indices = p.indices.ctypes.data if p.indices is not None else None
    s.nindices = p.indices.size if p.indices is not None else 0
    pix = h[p.pixel] if p.pixel else None
    dep = h[p.depth] if p.depth else None
    fmt = f.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
    s.pixel = abi.Target(pix.ctypes.data, pix.shape[1], pix.shape[0], pix.strides[0], fmt) if pix is not None \
        else abi.Target(None, 0, 0, 0, 0)
    s.depth = abi.Target(dep.ctypes.data, dep.shape[1], dep.shape[0], dep.strides[0], abi.FMT_R32F) \
        if dep is not None else abi.Target(None, 0, 0, 0, 0)
    s.uniforms = C.addressof(uni)
    s.uniforms_size = C.sizeof(uni)
    return s


def _context(host_copy):
    """A context whose host-buffer renders use `host_copy`; skips where the
    device cannot read pageable host memory and DIRECT is asked for."""
    ctx = capi.Context(0)
    t = abi.Tuning()
    t.host_copy = host_copy
    rc = capi.lib().euc_ctx_set_tuning(ctx.handle, C.byref(t))
    if rc == abi.ERR_INVALID and host_copy == abi.HOST_COPY_DIRECT:
        ctx.close()
        pytest.skip("the device does not access pageable host memory")
    assert rc == abi.OK
    return ctx


def _render_host_batch(ctx, frames, threads, hosts=None):
    hosts = hosts or [f.alloc_host_targets() for f in frames]
    keep = []
    for k in range(max(len(f.passes) for f in frames)):
        sc = [_host_scene(f, f.passes[k], h, keep) for f, h in zip(frames, hosts) if k < len(f.passes)]
        rc = ctx.render_host_batch((abi.Scene * len(sc))(*sc), threads)
        assert rc == abi.OK, capi.status_string(rc)
    return hosts


@pytest.mark.parametrize("threads,host_copy", [(1, abi.HOST_COPY_STAGED), (0, abi.HOST_COPY_STAGED),
                                               (0, abi.HOST_COPY_AUTO), (0, abi.HOST_COPY_DIRECT)])
def test_host_batch_matches_oracle(threads, host_copy):
    frames = scenes.batch_frames(seed=17, n=10, tri_lo=50, tri_hi=20000, resolutions=(64, 128, 200), tex_size=32)
    frames += [scenes.knot_frame(seed=3, width=160, height=96, shadow_size=128, tubular=120, radial=16, tex_size=32),
               scenes.sphere_frame(seed=9, width=97, height=61, lon=24, lat=12),
               scenes.lines_frame(seed=2, width=128, height=80, nlines=500)]
    ctx = _context(host_copy)
    try:
        got = _render_host_batch(ctx, frames, threads)
    finally:
        ctx.close()
    for f, g in zip(frames, got):
        ref = run_oracle(f, threads=4)
        ref = ref[0] if isinstance(ref, tuple) else ref
        tol = 1 if any(p.desc.shader == abi.SHADER_PHONG for p in f.passes) else 0
        assert_targets_match(f, ref, g, color_tol=tol)


@pytest.mark.parametrize("host_copy", [abi.HOST_COPY_STAGED, abi.HOST_COPY_DIRECT])
def test_host_batch_unaligned_targets(host_copy):
    """RGB8 targets at odd host addresses with odd row lengths: the copies
    fall back to narrower words and still land byte for byte."""
    frames = [scenes.sphere_frame(seed=s, width=w, height=h, lon=16, lat=8)
              for s, (w, h) in enumerate([(97, 61), (33, 17), (64, 48)])]
    ctx = _context(host_copy)
    try:
        ref = _render_host_batch(ctx, frames, 0)
        odd = []
        for f in frames:
            h = f.alloc_host_targets()
            c = h["color"]
            raw = np.zeros(c.size + 1, dtype=np.uint8)
            view = raw[1:].reshape(c.shape)
            view[...] = c
            h["color"] = view
            odd.append(h)
        got = _render_host_batch(ctx, frames, 0, hosts=odd)
    finally:
        ctx.close()
    for r, g in zip(ref, got):
        assert g["color"].ctypes.data % 2 == 1
        for k in r:
            assert np.array_equal(r[k].view(np.uint8), g[k].view(np.uint8)), k


@pytest.mark.parametrize("host_copy", [abi.HOST_COPY_STAGED, abi.HOST_COPY_DIRECT])
def test_host_batch_failing_scene_draws_nothing(host_copy):
    """A scene with an index out of bounds leaves its targets as they were;
    the other scene of the batch is drawn as it is alone (euc_render_batch's
    rule)."""
    good = scenes.sphere_frame(seed=1, width=64, height=48, lon=12, lat=6)
    bad = scenes.sphere_frame(seed=2, width=64, height=48, lon=12, lat=6)
    bad.passes[0].indices = bad.passes[0].indices.copy()
    bad.passes[0].indices[4] = 100000
    ctx = _context(host_copy)
    try:
        alone = _render_host_batch(ctx, [good], 0)[0]
        hosts = [f.alloc_host_targets() for f in (good, bad)]
        keep = []
        sc = [_host_scene(f, f.passes[0], h, keep) for f, h in zip((good, bad), hosts)]
        rc = ctx.render_host_batch((abi.Scene * 2)(*sc), 0)
        assert rc == abi.ERR_INDEX_OOB
        assert (hosts[1]["color"] == 0).all() and (hosts[1]["depth"] == 1.0).all()
        for k in alone:
            assert np.array_equal(alone[k].view(np.uint8), hosts[0][k].view(np.uint8)), k
        assert (hosts[0]["color"] != 0).any()
    finally:
        ctx.close()


@pytest.mark.parametrize("host_copy", [abi.HOST_COPY_STAGED, abi.HOST_COPY_DIRECT])
def test_host_batch_sees_host_writes_between_calls(host_copy):
    """The host clears the same target buffers between calls and edits the
    vertices in place: every call renders what the host memory holds then."""
    frames = [scenes.sphere_frame(seed=s, width=80, height=60, lon=16, lat=8) for s in range(3)]
    ctx = _context(host_copy)
    try:
        hosts = [f.alloc_host_targets() for f in frames]
        clean = [{k: v.copy() for k, v in h.items()} for h in hosts]
        first = [{k: v.copy() for k, v in h.items()} for h in _render_host_batch(ctx, frames, 0, hosts=hosts)]
        for _ in range(3):
            for h, c in zip(hosts, clean):
                for k in h:
                    np.copyto(h[k], c[k])
            _render_host_batch(ctx, frames, 0, hosts=hosts)
            for a, b in zip(first, hosts):
                for k in a:
                    assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
        # move every vertex of frame 0 off screen, in the host array the scene points at
        v = frames[0].passes[0].vertices
        saved = v.copy()
        v.view(np.float32).reshape(frames[0].passes[0].nverts, -1)[:, 0] += 1e4
        for h, c in zip(hosts, clean):
            for k in h:
                np.copyto(h[k], c[k])
        _render_host_batch(ctx, frames, 0, hosts=hosts)
        v[...] = saved
        assert (hosts[0]["color"] == 0).all()
        for a, b in zip(first[1:], hosts[1:]):
            for k in a:
                assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
    finally:
        ctx.close()


def test_host_batch_large_matches_device_batch():
    """A 24-scene batch of 20k-100k triangles each (71 MB of vertices and
    indices): byte-identical to the same batch rendered from device memory."""
    import torch
    from euc_gb300 import frames as fr
    specs = scenes.batch_frames(seed=23, n=24, tri_lo=20000, tri_hi=100000, resolutions=(128, 256), tex_size=64)
    ctx = capi.Context(0)
    try:
        batch = fr.DeviceBatch(specs, "cuda:0")
        fr.render_batch(ctx, batch, clear=True)
        torch.cuda.synchronize()
        want = [df.to_host() for df in batch.frames]
        got = _render_host_batch(ctx, specs, 0)
        direct = ctx.host_copy_direct()
    finally:
        ctx.close()
    nbytes = sum(p.vertices.nbytes + (p.indices.nbytes if p.indices is not None else 0)
                 for f in specs for p in f.passes)
    assert nbytes > 64 << 20
    for f, a, b in zip(specs, want, got):
        for k in a:
            assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), (f.name, k, direct)
