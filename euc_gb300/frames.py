"""Runs `scenes.FrameSpec`s on the GPU through the C ABI.

Device memory comes from PyTorch (plumbing only); every render goes through
`euc_render` / `euc_render_batch` in libeuc_gb300.so.
"""
import ctypes as C

import numpy as np
import torch

from . import abi, capi


def _stream_ptr(stream):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


def tensor_target(t, fmt):
    if t is None:
        return abi.Target(None, 0, 0, 0, abi.FMT_NONE)
    return abi.Target(t.data_ptr(), t.shape[1], t.shape[0], t.stride(0) * t.element_size(), fmt)


def _tex_info(t):
    fmt = abi.FMT_R32F if t.dtype == torch.float32 else abi.FMT_RGBA8
    return t.data_ptr(), t.shape[1], t.shape[0], t.stride(0) * t.element_size(), fmt, t


class DeviceFrame:
    """A FrameSpec whose inputs (vertices, indices, textures) and targets are
    resident in device memory."""

    def __init__(self, frame, device="cuda:0"):
        self.frame = frame
        self.device = torch.device(device)
        cache = {}

        def up(arr, view=None):
            if arr is None:
                return None
            key = id(arr)
            if key not in cache:
                a = np.ascontiguousarray(arr if view is None else arr.view(view))
                cache[key] = torch.from_numpy(a).to(self.device)
            return cache[key]

        self.passes = []
        for p in frame.passes:
            texs = {s.field: up(s.source) for s in p.samplers if not isinstance(s.source, str)}
            self.passes.append((up(p.vertices), up(p.indices, np.int32), texs))
        self.targets = {}
        for t in frame.targets:
            if t.fmt == abi.FMT_R32F:
                self.targets[t.name] = torch.empty((t.height, t.width), dtype=torch.float32, device=self.device)
            elif t.fmt == abi.FMT_RGBA32F:
                self.targets[t.name] = torch.empty((t.height, t.width, 4), dtype=torch.float32, device=self.device)
            else:
                self.targets[t.name] = torch.empty((t.height, t.width, t.bpp), dtype=torch.uint8, device=self.device)
        self._clear_px = {t.name: torch.from_numpy(t.host_alloc()[:1, :1].copy()).to(self.device)
                          for t in frame.targets if t.fmt != abi.FMT_R32F}

    def clear(self):
        for t in self.frame.targets:
            if t.fmt == abi.FMT_R32F:
                self.targets[t.name].fill_(float(np.float32(t.clear)))
            else:
                self.targets[t.name].copy_(self._clear_px[t.name].expand_as(self.targets[t.name]))

    def load_targets(self, host):
        """Copies host numpy targets (name -> array) into the device targets."""
        for k, v in host.items():
            self.targets[k].copy_(torch.from_numpy(np.ascontiguousarray(v)))

    def to_host(self):
        return {k: v.cpu().numpy() for k, v in self.targets.items()}

    def bound_pass(self, k):
        """(pass spec, uniforms with device texture pointers, keepalive)."""
        p = self.frame.passes[k]
        _, _, texs = self.passes[k]
        by_field = {s.field: s for s in p.samplers}

        def resolve(src):
            if isinstance(src, str):
                return _tex_info(self.targets[src])
            for f, s in by_field.items():
                if s.source is src:
                    return _tex_info(texs[f])
            raise KeyError("texture not uploaded")

        uni, keep = p.bind_uniforms(resolve)
        return p, uni, keep

    def scene(self, k):
        """euc_scene for pass k (device pointers) plus keepalive objects."""
        p, uni, keep = self.bound_pass(k)
        v, i, _ = self.passes[k]
        fmt = self.frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
        s = abi.Scene()
        s.desc = p.desc
        s.layout = p.layout
        s.vertices = v.data_ptr()
        s.nverts = p.nverts
        s.indices = i.data_ptr() if i is not None else None
        s.nindices = i.numel() if i is not None else 0
        s.pixel = tensor_target(self.targets[p.pixel] if p.pixel else None, fmt)
        s.depth = tensor_target(self.targets[p.depth] if p.depth else None, abi.FMT_R32F)
        s.uniforms = C.addressof(uni)
        s.uniforms_size = C.sizeof(uni)
        return s, (uni, keep)


class DeviceBatch:
    """Many DeviceFrames whose colour and depth targets are carved out of two
    device buffers, so that clearing every target of the batch is two fills
    (all colour targets of a batch must share one clear value, and so must all
    depth targets)."""

    def __init__(self, frame_specs, device="cuda:0"):
        self.frames = []
        ncol = ndep = 0
        for f in frame_specs:
            for t in f.targets:
                if t.fmt == abi.FMT_R32F:
                    ndep += t.width * t.height
                else:
                    ncol += t.width * t.height * t.bpp + 15
        dev = torch.device(device)
        self.color = torch.empty(max(ncol, 1), dtype=torch.uint8, device=dev)
        self.depth = torch.empty(max(ndep, 1), dtype=torch.float32, device=dev)
        cclear = {t.clear for f in frame_specs for t in f.targets if t.fmt != abi.FMT_R32F}
        dclear = {float(np.float32(t.clear)) for f in frame_specs for t in f.targets if t.fmt == abi.FMT_R32F}
        if len(cclear) > 1 or len(dclear) > 1 or (cclear and next(iter(cclear)) != 0):
            raise ValueError("DeviceBatch needs one clear value per target kind (colour 0)")
        self.depth_clear = next(iter(dclear)) if dclear else 1.0
        co = do = 0
        for f in frame_specs:
            df = DeviceFrame.__new__(DeviceFrame)
            df.frame = f
            df.device = dev
            df.targets = {}
            for t in f.targets:
                if t.fmt == abi.FMT_R32F:
                    n = t.width * t.height
                    df.targets[t.name] = self.depth[do:do + n].view(t.height, t.width)
                    do += n
                else:
                    co = (co + 15) & ~15
                    n = t.width * t.height * t.bpp
                    view = self.color[co:co + n].view(t.height, t.width, t.bpp)
                    if t.fmt == abi.FMT_RGBA32F:  # four floats a pixel (the offset is 16-byte aligned)
                        view = view.view(torch.float32)
                    df.targets[t.name] = view
                    co += n
            df._clear_px = {}
            self.frames.append(df)
        self._upload(dev)

    def _upload(self, dev):
        cache = {}

        def up(arr, view=None):
            if arr is None:
                return None
            key = id(arr)
            if key not in cache:
                a = np.ascontiguousarray(arr if view is None else arr.view(view))
                cache[key] = torch.from_numpy(a).to(dev)
            return cache[key]

        for df in self.frames:
            df.passes = []
            for p in df.frame.passes:
                texs = {s.field: up(s.source) for s in p.samplers if not isinstance(s.source, str)}
                df.passes.append((up(p.vertices), up(p.indices, np.int32), texs))

    def clear(self):
        self.color.zero_()
        self.depth.fill_(self.depth_clear)

    def scene_arrays(self):
        """Per pass k, a ctypes array of the euc_scene of every frame that has
        a pass k.  Built once: the device pointers do not change between
        renders, so repeated renders pay no per-scene host work."""
        if getattr(self, "_arrays", None) is None:
            npass = max(len(f.frame.passes) for f in self.frames)
            arrays, keep = [], []
            for k in range(npass):
                scenes = []
                for f in self.frames:
                    if k < len(f.frame.passes):
                        s, kp = f.scene(k)
                        scenes.append(s)
                        keep.append(kp)
                arrays.append((abi.Scene * len(scenes))(*scenes))
            self._arrays, self._keep = arrays, keep
        return self._arrays


def render_frame(ctx, dframe, stream=None, clear=True):
    """Clears the targets (if asked) and runs every pass with euc_render."""
    if clear:
        dframe.clear()
    sp = _stream_ptr(stream)
    for k, p in enumerate(dframe.frame.passes):
        p, uni, keep = dframe.bound_pass(k)
        v, i, _ = dframe.passes[k]
        fmt = dframe.frame.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
        pt = tensor_target(dframe.targets[p.pixel] if p.pixel else None, fmt)
        dt = tensor_target(dframe.targets[p.depth] if p.depth else None, abi.FMT_R32F)
        rc = ctx.render(p.desc, uni, p.layout, v.data_ptr(), p.nverts, i.data_ptr() if i is not None else None,
                        i.numel() if i is not None else 0, pt, dt, sp)
        capi.check(rc, "euc_render(%s pass %d)" % (dframe.frame.name, k))
        del keep
    return dframe.targets


def render_batch(ctx, dframes, stream=None, clear=True):
    """Renders many frames with euc_render_batch: pass k of every frame goes
    into the k-th batch call (passes of one frame stay in order)."""
    if isinstance(dframes, DeviceBatch):
        if clear:
            dframes.clear()
        sp = _stream_ptr(stream)
        for k, arr in enumerate(dframes.scene_arrays()):
            capi.check(ctx.render_scene_array(arr, sp), "euc_render_batch(pass %d)" % k)
        return
    elif clear:
        for f in dframes:
            f.clear()
    sp = _stream_ptr(stream)
    npass = max(len(f.frame.passes) for f in dframes)
    for k in range(npass):
        scenes, keep = [], []
        for f in dframes:
            if k < len(f.frame.passes):
                s, kp = f.scene(k)
                scenes.append(s)
                keep.append(kp)
        capi.check(ctx.render_batch(scenes, sp), "euc_render_batch(pass %d)" % k)
        del keep


class BatchGraph:
    """A DeviceBatch recorded as one euc_graph per pass; `launch` clears the
    targets (two fills) and replays the passes in order."""

    def __init__(self, ctx, batch):
        self.batch = batch
        arrays = batch.scene_arrays()
        self.graphs = [ctx.graph(arr) for arr in arrays]
        if len(arrays) > 1:
            # recording a later pass may have grown the context scratch that
            # an earlier pass was recorded against: record again, now that the
            # scratch holds every pass
            for g in self.graphs:
                g.close()
            self.graphs = [ctx.graph(arr) for arr in arrays]

    def launch(self, stream=None, clear=True):
        if clear:
            self.batch.clear()
        sp = _stream_ptr(stream)
        for g in self.graphs:
            g.launch(sp)

    def close(self):
        for g in self.graphs:
            g.close()
        self.graphs = []


def frame_stats(ctx, stream=None):
    return ctx.stats(_stream_ptr(stream))
