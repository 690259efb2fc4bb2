"""Helpers shared by the parity tests: run a FrameSpec on the oracle and on
the GPU (pass by pass, with statistics) and compare the targets."""
import numpy as np

from euc_gb300 import abi


def run_oracle(frame, threads=1):
    from oracle import oracle
    targets, stats, codes = oracle.run_frame(frame, threads=threads)
    return targets, [(c, s.candidates, s.culled) for c, s in zip(codes, stats)]


def run_gpu(ctx, frame, device="cuda:0"):
    """Returns (host targets, [(status, candidates, culled) per pass])."""
    import torch
    from euc_gb300 import frames
    df = frames.DeviceFrame(frame, device)
    df.clear()
    out = []
    for k in range(len(frame.passes)):
        p, uni, keep = df.bound_pass(k)
        v, i, _ = df.passes[k]
        fmt = frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
        pt = frames.tensor_target(df.targets[p.pixel] if p.pixel else None, fmt)
        dt = frames.tensor_target(df.targets[p.depth] if p.depth else None, abi.FMT_R32F)
        sp = frames._stream_ptr(None)
        rc = ctx.render(p.desc, uni, p.layout, v.data_ptr(), p.nverts, i.data_ptr() if i is not None else None,
                        i.numel() if i is not None else 0, pt, dt, sp)
        if rc == abi.OK:
            rc = ctx.sync(sp)
        st = ctx.stats(sp)
        out.append((rc, st.candidates, st.culled))
        del keep
    torch.cuda.synchronize()
    return df.to_host(), out


def assert_targets_match(frame, ref, got, color_tol=0):
    """Depth bit-exact; colour exact or within color_tol per 8-bit channel
    (an f32 colour target: bit-exact, or within a relative 1e-5 where
    color_tol allows a step); the set of written colour pixels identical."""
    for t in frame.targets:
        a, b = ref[t.name], got[t.name]
        assert a.shape == b.shape, t.name
        if t.fmt == abi.FMT_RGBA32F:
            if color_tol == 0:
                ai, bi = a.view(np.uint32), b.view(np.uint32)
                bad = np.argwhere(ai != bi)
            else:
                bad = np.argwhere(~np.isclose(a, b, rtol=1e-5, atol=1e-6))
            assert bad.size == 0, "%s: %d f32 channels differ, first at %s: %r vs %r" % (
                t.name, len(bad), bad[0].tolist(), a[tuple(bad[0][:2])], b[tuple(bad[0][:2])])
        elif t.fmt == abi.FMT_R32F:
            ai, bi = a.view(np.uint32), b.view(np.uint32)
            bad = np.argwhere(ai != bi)
            assert bad.size == 0, "%s: %d depth words differ, first at %s: %r vs %r" % (
                t.name, len(bad), bad[0].tolist(), a[tuple(bad[0])], b[tuple(bad[0])])
        else:
            d = np.abs(a.astype(np.int16) - b.astype(np.int16))
            bad = np.argwhere(d > color_tol)
            assert bad.size == 0, "%s: %d channels differ by > %d, first at %s: %r vs %r" % (
                t.name, len(bad), color_tol, bad[0].tolist(), a[tuple(bad[0][:2])], b[tuple(bad[0][:2])])


def assert_same_inputs(fa, fb):
    """Two FrameSpecs built by the same generator call hold identical inputs."""
    import ctypes as C
    assert len(fa.passes) == len(fb.passes)
    for pa, pb in zip(fa.passes, fb.passes):
        assert np.array_equal(pa.vertices, pb.vertices)
        assert (pa.indices is None) == (pb.indices is None)
        if pa.indices is not None:
            assert np.array_equal(pa.indices, pb.indices)
        assert C.string_at(C.addressof(pa.uniforms), C.sizeof(pa.uniforms)) == \
            C.string_at(C.addressof(pb.uniforms), C.sizeof(pb.uniforms))
        assert bytes(pa.desc) == bytes(pb.desc)
