"""The serving loop (euc_server_* in libeuc_gb300.so) from Python.

`Server` wraps the C ABI: resident meshes and textures, request submission,
completions.  `Resident` uploads the arrays a set of `scenes.FrameSpec`s
reference (by identity) once, and `request_for` turns a FrameSpec over
resident arrays into an `abi.ServerRequest`, so that the same spec can be
rendered by the plain path (frames.render_frame) and served, and the two
images compared byte for byte.

`run_poisson` drives a server with open-loop Poisson arrivals: the arrival
time of every request is fixed in advance and handed to the server, which
admits no request before it, so latencies (done - arrival) include every
queueing delay and no client-side lag hides one.
"""
import ctypes as C

import numpy as np

from . import abi, capi


class Server:
    def __init__(self, device=0, framebuffer_budget=40 << 30, max_batch=256, slots=3, max_pending=1 << 20):
        cfg = abi.ServerConfig(device, max_batch, framebuffer_budget, slots, max_pending)
        h = C.c_void_p()
        capi.check(capi.lib().euc_server_create(C.byref(cfg), C.byref(h)), "euc_server_create")
        self.handle = h
        self.config = cfg

    def close(self):
        if self.handle:
            capi.lib().euc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_mesh(self, layout, vertices, nverts, indices=None):
        v = np.ascontiguousarray(vertices)
        i = None if indices is None else np.ascontiguousarray(indices, dtype=np.uint32)
        mid = C.c_uint32()
        capi.check(capi.lib().euc_server_add_mesh(self.handle, C.byref(layout), v.ctypes.data, nverts,
                                                  i.ctypes.data if i is not None else None,
                                                  i.size if i is not None else 0, C.byref(mid)),
                   "euc_server_add_mesh")
        return mid.value

    def add_texture(self, texels):
        t = np.ascontiguousarray(texels)
        fmt = abi.FMT_R32F if t.dtype == np.float32 else abi.FMT_RGBA8
        tid = C.c_uint32()
        capi.check(capi.lib().euc_server_add_texture(self.handle, t.ctypes.data, t.shape[1], t.shape[0],
                                                     t.strides[0], fmt, C.byref(tid)), "euc_server_add_texture")
        return tid.value

    def now_ns(self):
        return capi.lib().euc_server_now_ns(self.handle)

    def submit(self, reqs, n=None, ptr=None):
        """Submits a ctypes array of abi.ServerRequest (or `n` requests at a
        raw pointer); returns (first id, accepted count).  Raises on a
        refused request (invalid, over budget); a full queue is not an error
        here: the caller sees accepted < n."""
        if ptr is None:
            ptr, n = C.addressof(reqs), len(reqs)
        first, acc = C.c_uint64(), C.c_size_t()
        rc = capi.lib().euc_server_submit(self.handle, ptr, n, C.byref(first), C.byref(acc))
        if rc not in (abi.OK, abi.ERR_BUSY):
            raise capi.EucError(rc, "euc_server_submit")
        return first.value, acc.value

    def poll(self, max_n=4096, wait_ms=0):
        buf = (abi.ServerCompletion * max_n)()
        n = C.c_size_t()
        capi.check(capi.lib().euc_server_poll(self.handle, buf, max_n, C.byref(n), wait_ms), "euc_server_poll")
        if n.value == 0:
            return np.zeros(0, dtype=COMPLETION_DTYPE)
        return np.frombuffer(buf, dtype=COMPLETION_DTYPE, count=n.value).copy()

    def drain(self, timeout_ms=-1):
        return capi.lib().euc_server_drain(self.handle, timeout_ms)

    def stats(self):
        s = abi.ServerStats()
        capi.check(capi.lib().euc_server_stats_get(self.handle, C.byref(s)), "euc_server_stats_get")
        return s.as_dict()


COMPLETION_DTYPE = np.dtype([("id", "<u8"), ("tag", "<u8"), ("status", "<i4"), ("batch_size", "<u4"),
                             ("arrival_ns", "<u8"), ("admit_ns", "<u8"), ("done_ns", "<u8")])
assert COMPLETION_DTYPE.itemsize == C.sizeof(abi.ServerCompletion)


class Resident:
    """Uploads each distinct vertex buffer (with its index buffer) and each
    texture array that a FrameSpec references, once, keyed by identity."""

    def __init__(self, server):
        self.server = server
        self.meshes = {}
        self.textures = {}
        self._keep = []

    def mesh(self, p):
        key = (id(p.vertices), id(p.indices), p.layout.stride, p.layout.position, p.layout.normal, p.layout.uv,
               p.layout.color, p.nverts)
        if key not in self.meshes:
            self.meshes[key] = self.server.add_mesh(p.layout, p.vertices, p.nverts, p.indices)
            self._keep.append((p.vertices, p.indices))
        return self.meshes[key]

    def texture(self, arr):
        if id(arr) not in self.textures:
            self.textures[id(arr)] = self.server.add_texture(arr)
            self._keep.append(arr)
        return self.textures[id(arr)]


def clear_bits(t):
    if t.fmt == abi.FMT_R32F:
        return int(np.array([t.clear], dtype=np.float32).view(np.uint32)[0])
    return int(t.clear) & ((1 << (8 * t.bpp)) - 1)


def out_bytes(frame, readback):
    return sum(t.width * t.height * t.bpp for t in frame.targets if t.name in readback)


def request_for(frame, resident, readback=("color",), tag=0, out=None, out_size=0):
    """(abi.ServerRequest, keepalive) for `frame` over resident arrays;
    targets named in `readback` are copied to `out` in target order."""
    names = [t.name for t in frame.targets]
    targets = (abi.ServerTarget * len(frame.targets))()
    for k, t in enumerate(frame.targets):
        targets[k] = abi.ServerTarget(t.width, t.height, t.fmt, clear_bits(t), 1 if t.name in readback else 0, 0)
    passes = (abi.ServerPass * len(frame.passes))()
    keep = [targets, passes]
    for k, p in enumerate(frame.passes):
        uni = type(p.uniforms).from_buffer_copy(p.uniforms)
        binds = (abi.ServerBinding * max(1, len(p.samplers)))()
        for j, s in enumerate(p.samplers):
            off = getattr(type(uni), s.field).offset
            setattr(uni, s.field, abi.Sampler(None, 0, 0, 0, 0, s.filter, s.wrap, s.texel_div, 0))
            if isinstance(s.source, str):
                binds[j] = abi.ServerBinding(off, -1, names.index(s.source), 0)
            else:
                binds[j] = abi.ServerBinding(off, resident.texture(s.source), -1, 0)
        ps = passes[k]
        ps.desc = p.desc
        ps.mesh = resident.mesh(p)
        ps.pixel_target = names.index(p.pixel) if p.pixel else -1
        ps.depth_target = names.index(p.depth) if p.depth else -1
        ps.nbindings = len(p.samplers)
        ps.bindings = C.cast(binds, C.POINTER(abi.ServerBinding))
        ps.uniforms = C.addressof(uni)
        ps.uniforms_size = C.sizeof(uni)
        keep += [uni, binds]
    r = abi.ServerRequest()
    r.tag = tag
    r.arrival_ns = 0
    r.out = out
    r.out_size = out_size
    r.ntargets = len(frame.targets)
    r.npasses = len(frame.passes)
    r.targets = C.cast(targets, C.POINTER(abi.ServerTarget))
    r.passes = C.cast(passes, C.POINTER(abi.ServerPass))
    return r, keep


def split_readback(frame, buf, readback=("color",)):
    """name -> array views of a readback buffer filled by the server."""
    out, o = {}, 0
    for t in frame.targets:
        if t.name not in readback:
            continue
        n = t.width * t.height * t.bpp
        a = np.frombuffer(buf, dtype=np.uint8, count=n, offset=o)
        out[t.name] = a.view(np.float32).reshape(t.height, t.width) if t.fmt == abi.FMT_R32F else \
            a.reshape(t.height, t.width, t.bpp)
        o += n
    return out


def latency_summary(comp):
    """p50 / p99 / mean / max latency (ms) of completions, done - arrival."""
    if len(comp) == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None, "max_ms": None}
    lat = (comp["done_ns"].astype(np.int64) - comp["arrival_ns"].astype(np.int64)) / 1e6
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max())}


def run_poisson(server, pool, pool_outs, rate, seconds, seed=0, lead_s=0.05, chunk_s=0.01, log=None):
    """Open-loop Poisson arrivals at `rate` requests/s for `seconds`.

    `pool`: ctypes array of abi.ServerRequest to draw from (uniformly,
    seeded); `pool_outs`: per pool entry, a list of pinned host buffers
    (pointer, size), the same count for every entry, used in turn as
    readback destinations.  Requests are
    submitted `lead_s` ahead of their arrival in chunks of `chunk_s`.
    Returns (completions array, summary dict)."""
    import time
    rng = np.random.default_rng(seed)
    n_total = int(rng.poisson(rate * seconds))
    gaps = rng.exponential(1.0 / rate, n_total)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < seconds]
    n_total = len(arrivals)
    picks = rng.integers(0, len(pool), n_total)
    rsize = C.sizeof(abi.ServerRequest)
    pool_bytes = np.frombuffer((C.c_char * (rsize * len(pool))).from_address(C.addressof(pool)),
                               dtype=np.uint8).reshape(len(pool), rsize)
    off_arrival = abi.ServerRequest.arrival_ns.offset // 8
    off_out = abi.ServerRequest.out.offset // 8
    off_size = abi.ServerRequest.out_size.offset // 8
    off_tag = abi.ServerRequest.tag.offset // 8
    nout = len(pool_outs[0])
    if any(len(o) != nout for o in pool_outs):
        raise ValueError("every pool entry needs the same number of readback buffers")
    outs_ptr = np.array([[p for p, _ in o] for o in pool_outs], dtype=np.uint64)
    outs_size = np.array([[s for _, s in o] for o in pool_outs], dtype=np.uint64)
    t0 = server.now_ns() + int(lead_s * 1e9)
    arr_ns = (t0 + arrivals * 1e9).astype(np.uint64)
    comps = []
    refused = 0
    sent = 0
    done = 0
    start = time.perf_counter()
    while sent < n_total or done < sent - refused:
        now = server.now_ns()
        horizon = now + int(lead_s * 1e9)
        hi = int(np.searchsorted(arr_ns, horizon, side="right"))
        if hi > sent:
            idx = picks[sent:hi]
            chunk = pool_bytes[idx].copy()
            w = chunk.view(np.uint64)
            w[:, off_arrival] = arr_ns[sent:hi]
            seq = np.arange(sent, hi, dtype=np.int64)
            w[:, off_tag] = seq.astype(np.uint64)
            w[:, off_out] = outs_ptr[idx, seq % nout]
            w[:, off_size] = outs_size[idx, seq % nout]
            _, acc = server.submit(None, n=hi - sent, ptr=chunk.ctypes.data)
            refused += (hi - sent) - acc
            sent = hi
        c = server.poll(8192, wait_ms=int(chunk_s * 1e3) if sent >= n_total else 0)
        if len(c):
            comps.append(c)
            done += len(c)
        elif sent < n_total:
            nxt = arr_ns[sent] if sent < n_total else 0
            sleep = (int(nxt) - int(server.now_ns()) - int(lead_s * 1e9)) / 1e9
            if sleep > 0:
                time.sleep(min(sleep, chunk_s))
        if time.perf_counter() - start > seconds + 120:
            raise RuntimeError("serving run did not finish")
    comp = np.concatenate(comps) if comps else np.zeros(0, dtype=COMPLETION_DTYPE)
    ok = comp[comp["status"] == abi.OK]
    span_ns = (int(comp["done_ns"].max()) - int(arr_ns[0])) if len(comp) else 1
    summary = dict(latency_summary(ok), rate=rate, seconds=seconds, offered=n_total, refused=refused,
                   completed=int(len(ok)), failed=int(len(comp) - len(ok)),
                   throughput=len(ok) / (span_ns / 1e9),
                   mean_batch=float(comp["batch_size"].mean()) if len(comp) else None,
                   stats=server.stats())
    if log:
        log(summary)
    return comp, summary
