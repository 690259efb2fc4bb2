"""euc_render_host_batch (host buffers, one call per pass) against the
oracle and against euc_render_host per scene: byte-identical targets."""
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


def _render_host_batch(ctx, frames, threads):
    hosts = [f.alloc_host_targets() for f in frames]
    keep = []
    for k in range(max(len(f.passes) for f in frames)):
        sc = [_host_scene(f, f.passes[k], h, keep) for f, h in zip(frames, hosts) if k < len(f.passes)]
        rc = ctx.render_host_batch((abi.Scene * len(sc))(*sc), threads)
        assert rc == abi.OK, capi.status_string(rc)
    return hosts


@pytest.mark.parametrize("threads", [1, 0])
def test_host_batch_matches_oracle(threads):
    frames = scenes.batch_frames(seed=17, n=10, tri_lo=50, tri_hi=20000, resolutions=(64, 128, 200), tex_size=32)
    frames += [scenes.knot_frame(seed=3, width=160, height=96, shadow_size=128, tubular=120, radial=16, tex_size=32),
               scenes.sphere_frame(seed=9, width=97, height=61, lon=24, lat=12),
               scenes.lines_frame(seed=2, width=128, height=80, nlines=500)]
    ctx = capi.Context(0)
    try:
        got = _render_host_batch(ctx, frames, threads)
    finally:
        ctx.close()
    for f, g in zip(frames, got):
        ref = run_oracle(f, threads=4)
        ref = ref[0] if isinstance(ref, tuple) else ref
        tol = 1 if any(p.desc.shader == abi.SHADER_PHONG for p in f.passes) else 0
        assert_targets_match(f, ref, g, color_tol=tol)


def test_host_batch_writes_nothing_back_on_failure():
    good = scenes.sphere_frame(seed=1, width=64, height=48, lon=12, lat=6)
    bad = scenes.sphere_frame(seed=2, width=64, height=48, lon=12, lat=6)
    bad.passes[0].indices = bad.passes[0].indices.copy()
    bad.passes[0].indices[4] = 100000
    ctx = capi.Context(0)
    try:
        hosts = [f.alloc_host_targets() for f in (good, bad)]
        keep = []
        sc = [_host_scene(f, f.passes[0], h, keep) for f, h in zip((good, bad), hosts)]
        rc = ctx.render_host_batch((abi.Scene * 2)(*sc), 0)
        assert rc == abi.ERR_INDEX_OOB
        assert (hosts[0]["color"] == 0).all() and (hosts[0]["depth"] == 1.0).all()
    finally:
        ctx.close()
