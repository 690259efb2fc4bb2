"""Launch-shape autotuner for batched renders.

`euc_ctx_set_tuning` changes how a batch is spread over the GPU: which
scenes go to the shared-memory strips, persistent raster blocks per SM, the
(primitive, row) items a raster warp claims at a time, whether the raster
reads a key before its atomicMin, and the chunk grouping and grid cap of the
init/resolve kernels.  None of these changes a result.  The tuner times a
`frames.DeviceBatch` under a set of candidate shapes (coordinate descent: the
strip path, then the raster knobs, then the chunk knobs), checks that every
candidate's targets are byte-identical to the default shape's, keeps the
fastest and caches the choice per device, library build and workload
signature in a JSON file next to the built library.
"""
import json
import os

import torch

from . import abi
from . import build as _build
from . import frames as fr

CACHE = os.path.join(os.path.dirname(_build.LIB), "autotune.json")

RASTER_BLOCKS = (0, 2, 3)          # 0: the occupancy limit
RASTER_WARP_ROWS = (256, 128, 64)
CHUNK_GROUP = (0, 1, 4, 16)        # 0: adaptive
CHUNK_BLOCKS = (0, 8, 32)          # 0: 16 per SM
RASTER_PROBE = (0, 1)              # 0: atomics only; 1: read keys before their atomics
STRIP_PATH = (0, 1, 2)             # shared-memory strips: 0 for overdrawn scenes, 1 off, 2 always


def workload_key(batch):
    """Device name, SM count and the batch's shape: scenes, primitives,
    target pixels and shader kinds per pass."""
    props = torch.cuda.get_device_properties(batch.color.device)
    try:
        build = "%d" % int(os.path.getmtime(_build.LIB))
    except OSError:
        build = "?"
    parts = [props.name.replace(" ", "_"), str(props.multi_processor_count), "lib" + build]
    for arr in batch.scene_arrays():
        tris = sum(s.nindices // 3 for s in arr)
        pix = sum(max(s.pixel.width * s.pixel.height, s.depth.width * s.depth.height) for s in arr)
        shaders = sorted({s.desc.shader for s in arr})
        parts.append("n%d-t%d-p%d-s%s" % (len(arr), tris, pix, ".".join(map(str, shaders))))
    return "/".join(parts)


def _time(ctx, batch, stream, reps):
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
    fr.render_batch(ctx, batch, stream, clear=True)  # warm
    for r in range(reps):
        ev[2 * r].record(stream)
        fr.render_batch(ctx, batch, stream, clear=True)
        ev[2 * r + 1].record(stream)
    stream.synchronize()
    ts = sorted(ev[2 * r].elapsed_time(ev[2 * r + 1]) for r in range(reps))
    return ts[len(ts) // 2]


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(ctx, batch, stream=None, reps=5, cache=CACHE, verify=True, log=None):
    """Finds the fastest launch shape for `batch`, sets it on `ctx` and
    returns (abi.Tuning, {"ms": best, "default_ms": ..., "tried": n,
    "cached": bool}).  Raises if a candidate changes any output byte."""
    stream = stream or torch.cuda.current_stream()
    key = workload_key(batch)
    if cache:
        hit = _load_cache(cache).get(key)
        if hit:
            t = abi.Tuning(**hit["tuning"])
            ctx.set_tuning(t)
            return t, dict(hit.get("info", {}), cached=True)

    ctx.set_tuning(None)
    fr.render_batch(ctx, batch, stream, clear=True)
    stream.synchronize()
    ref_c, ref_d = batch.color.clone(), batch.depth.clone()

    tried = {}

    def run(cand):
        k = tuple(sorted(cand.items()))
        if k in tried:
            return tried[k]
        ctx.set_tuning(abi.Tuning(**cand))
        ms = _time(ctx, batch, stream, reps)
        if verify and not (torch.equal(batch.color, ref_c) and torch.equal(batch.depth, ref_d)):
            ctx.set_tuning(None)
            raise RuntimeError("launch shape %r changed the rendered bytes" % (cand,))
        tried[k] = ms
        if log:
            log("autotune %s: %.3f ms" % (cand, ms))
        return ms

    best = {k: 0 for k, _ in abi.Tuning._fields_}
    default_ms = best_ms = run(best)
    for sp in STRIP_PATH:
        cand = dict(best, strip_path=sp)
        ms = run(cand)
        if ms < best_ms:
            best, best_ms = cand, ms
    for pr in RASTER_PROBE:
        for rb in RASTER_BLOCKS:
            for wr in RASTER_WARP_ROWS:
                cand = dict(best, raster_probe=pr, raster_blocks_per_sm=rb, raster_warp_rows=wr)
                ms = run(cand)
                if ms < best_ms:
                    best, best_ms = cand, ms
    for cg in CHUNK_GROUP:
        for cb in CHUNK_BLOCKS:
            cand = dict(best, chunk_group=cg, chunk_blocks_per_sm=cb)
            ms = run(cand)
            if ms < best_ms:
                best, best_ms = cand, ms
    # re-time the winner against the default: keep the default unless the
    # winner is still ahead (the first pass saw single medians)
    if best != {k: 0 for k in best}:
        ctx.set_tuning(None)
        d = _time(ctx, batch, stream, reps)
        ctx.set_tuning(abi.Tuning(**best))
        b = _time(ctx, batch, stream, reps)
        if b >= d:
            best, best_ms = {k: 0 for k in best}, d
        default_ms = d
    t = abi.Tuning(**best)
    ctx.set_tuning(t)
    info = {"ms": best_ms, "default_ms": default_ms, "tried": len(tried)}
    if cache:
        data = _load_cache(cache)
        data[key] = {"tuning": best, "info": info}
        try:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            tmp = cache + ".tmp%d" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        except OSError:
            pass
    return t, dict(info, cached=False)
