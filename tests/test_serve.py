"""The serving loop (euc_server_*): every served image equals the plain
euc_render of the same passes, whether the request ran alone or batched
among others; admission keeps the framebuffer budget; submissions are
checked before anything is queued."""
import ctypes as C

import numpy as np
import pytest

from euc_gb300 import abi, capi, scenes, serve
from euc_gb300 import frames as fr

pytestmark = pytest.mark.gpu

READ = ("shadow", "color", "depth")


def _assets():
    return scenes.serve_assets(seed=4, nmeshes=6, ntextures=3, tex_size=64, tri_lo=50, tri_hi=8000)


def _frames(assets, n, seed, resolutions=(64, 96, 128)):
    rng = np.random.default_rng(seed)
    return [scenes.serve_frame(assets, rng, resolutions) for _ in range(n)]


def _plain(frames):
    import torch
    ctx = capi.Context(0)
    try:
        out = []
        for f in frames:
            df = fr.DeviceFrame(f, "cuda:0")
            fr.render_frame(ctx, df)
            torch.cuda.synchronize()
            out.append(df.to_host())
        return out
    finally:
        ctx.close()


def _requests(frames, resident, tag0=0):
    reqs, keep, outs = [], [], []
    for k, f in enumerate(frames):
        buf = np.zeros(serve.out_bytes(f, READ), dtype=np.uint8)
        r, kp = serve.request_for(f, resident, READ, tag=tag0 + k, out=buf.ctypes.data, out_size=buf.nbytes)
        reqs.append(r)
        keep.append(kp)
        outs.append(buf)
    return reqs, keep, outs


def _check(frame, ref, buf):
    got = serve.split_readback(frame, buf, READ)
    for name in READ:
        a, b = ref[name], got[name]
        assert a.shape == b.shape, name
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), "%s: %s differs" % (frame.name, name)


def _collect(server, n, timeout_ms=60000):
    assert server.drain(timeout_ms) == abi.OK
    comps = []
    while sum(len(c) for c in comps) < n:
        c = server.poll(4096, wait_ms=1000)
        assert len(c), "missing completions"
        comps.append(c)
    return np.concatenate(comps)


def test_served_images_equal_plain_alone_and_in_mix():
    assets = _assets()
    probes = _frames(assets, 8, seed=1)
    others = _frames(assets, 160, seed=2, resolutions=(64, 128, 200))
    ref = _plain(probes)
    srv = serve.Server(0, framebuffer_budget=256 << 20, max_batch=48, slots=3)
    try:
        res = serve.Resident(srv)
        # alone: one request at a time
        reqs, keep, outs = _requests(probes, res)
        for k, r in enumerate(reqs):
            srv.submit((abi.ServerRequest * 1)(r))
            c = _collect(srv, 1)
            assert c["status"][0] == abi.OK and c["batch_size"][0] == 1
            _check(probes[k], ref[k], outs[k])
        # in the mix: the probes interleaved with other requests, submitted
        # in several waves so that batches form while others run
        reqs2, keep2, outs2 = _requests(probes, res, tag0=1000)
        oreqs, okeep, oouts = _requests(others, res, tag0=2000)
        order = list(range(len(oreqs)))
        rng = np.random.default_rng(7)
        mixed = [oreqs[i] for i in order]
        for k, r in enumerate(reqs2):
            mixed.insert(int(rng.integers(0, len(mixed))), r)
        for w in range(0, len(mixed), 21):
            wave = mixed[w:w + 21]
            srv.submit((abi.ServerRequest * len(wave))(*wave))
        comp = _collect(srv, len(mixed))
        assert (comp["status"] == abi.OK).all()
        assert comp["batch_size"].max() > 1, "nothing was batched"
        by_tag = {int(t): int(b) for t, b in zip(comp["tag"], comp["batch_size"])}
        assert any(by_tag[1000 + k] > 1 for k in range(len(probes)))
        for k in range(len(probes)):
            _check(probes[k], ref[k], outs2[k])
        st = srv.stats()
        assert st["completed"] == len(probes) + len(mixed) and st["failed"] == 0
        assert st["pending"] == 0 and st["in_flight"] == 0 and st["budget_used"] == 0
    finally:
        srv.close()


def test_admission_keeps_the_budget():
    assets = _assets()
    frames = _frames(assets, 24, seed=3, resolutions=(128,))
    per_req = 3 * 128 * 128 * 4  # shadow + colour + depth, 256-byte multiples already
    srv = serve.Server(0, framebuffer_budget=2 * per_req, max_batch=64, slots=3)
    try:
        res = serve.Resident(srv)
        reqs, keep, outs = _requests(frames, res)
        srv.submit((abi.ServerRequest * len(reqs))(*reqs))
        comp = _collect(srv, len(reqs))
        assert (comp["status"] == abi.OK).all()
        st = srv.stats()
        assert st["budget_peak"] <= 2 * per_req
        assert comp["batch_size"].max() <= 2
        ref = _plain(frames[:4])
        for k in range(4):
            _check(frames[k], ref[k], outs[k])
    finally:
        srv.close()


def test_submissions_are_checked_before_queueing():
    assets = _assets()
    f = _frames(assets, 1, seed=5, resolutions=(64,))[0]
    srv = serve.Server(0, framebuffer_budget=1 << 20, max_batch=8, slots=2, max_pending=4)
    try:
        res = serve.Resident(srv)
        (r,), keep, outs = _requests([f], res)
        # unknown mesh id
        bad = abi.ServerRequest.from_buffer_copy(r)
        passes = (abi.ServerPass * 2)(r.passes[0], r.passes[1])
        passes[1].mesh = 99
        bad.passes = C.cast(passes, C.POINTER(abi.ServerPass))
        with pytest.raises(capi.EucError) as e:
            srv.submit((abi.ServerRequest * 2)(r, bad))
        assert e.value.code == abi.ERR_INVALID
        # readback buffer too small
        small = abi.ServerRequest.from_buffer_copy(r)
        small.out_size = 16
        with pytest.raises(capi.EucError) as e:
            srv.submit((abi.ServerRequest * 1)(small))
        assert e.value.code == abi.ERR_INVALID
        # sampling the target the pass writes
        passes2 = (abi.ServerPass * 2)(r.passes[0], r.passes[1])
        b = (abi.ServerBinding * 2)(r.passes[1].bindings[0], r.passes[1].bindings[1])
        b[1].target = passes2[1].depth_target
        passes2[1].bindings = C.cast(b, C.POINTER(abi.ServerBinding))
        hazard = abi.ServerRequest.from_buffer_copy(r)
        hazard.passes = C.cast(passes2, C.POINTER(abi.ServerPass))
        with pytest.raises(capi.EucError) as e:
            srv.submit((abi.ServerRequest * 1)(hazard))
        assert e.value.code == abi.ERR_INVALID
        assert srv.stats()["submitted"] == 0
        # larger than the whole budget
        big = scenes.serve_frame(assets, np.random.default_rng(1), resolutions=(1024,))
        (rb,), kb, ob = _requests([big], res)
        with pytest.raises(capi.EucError) as e:
            srv.submit((abi.ServerRequest * 1)(rb))
        assert e.value.code == abi.ERR_BUDGET
        # out-of-range index at upload
        m = assets.meshes[0]
        with pytest.raises(capi.EucError) as e:
            srv.add_mesh(m["layout"], m["vertices"], m["nverts"], np.array([0, 1, m["nverts"]], dtype=np.uint32))
        assert e.value.code == abi.ERR_INDEX_OOB
        # a full admission queue refuses the rest (arrivals far in the future)
        later = abi.ServerRequest.from_buffer_copy(r)
        later.arrival_ns = srv.now_ns() + 3_600_000_000_000
        first, acc = srv.submit((abi.ServerRequest * 10)(*([later] * 10)))
        assert acc == 4
        st = srv.stats()
        assert st["pending"] == 4 and st["refused"] == 6 and st["in_flight"] == 0
    finally:
        srv.close()  # drops the pending requests


def test_poisson_run_reports_latency():
    import torch
    assets = _assets()
    pool_frames = _frames(assets, 32, seed=6, resolutions=(64, 128))
    srv = serve.Server(0, framebuffer_budget=256 << 20, max_batch=64, slots=3)
    try:
        res = serve.Resident(srv)
        pins, keep, pool = [], [], []
        outs = []
        for k, f in enumerate(pool_frames):
            n = serve.out_bytes(f, ("color",))
            bufs = [torch.empty(n, dtype=torch.uint8).pin_memory() for _ in range(4)]
            pins += bufs
            outs.append([(b.data_ptr(), n) for b in bufs])
            r, kp = serve.request_for(f, res, ("color",), tag=k, out=bufs[0].data_ptr(), out_size=n)
            pool.append(r)
            keep.append(kp)
        arr = (abi.ServerRequest * len(pool))(*pool)
        comp, summary = serve.run_poisson(srv, arr, outs, rate=2000, seconds=0.5, seed=1)
        assert summary["completed"] == summary["offered"] - summary["refused"] and summary["failed"] == 0
        assert summary["refused"] == 0 and summary["offered"] > 500
        assert 0 < summary["p50_ms"] <= summary["p99_ms"]
        assert (comp["admit_ns"] >= comp["arrival_ns"]).all() and (comp["done_ns"] >= comp["admit_ns"]).all()
    finally:
        srv.close()
