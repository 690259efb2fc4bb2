"""Benchmark of the GB300 euc triangle pipeline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

Workload (one "step" = clear + render of one batch): 256 independent scenes,
triangle counts log-uniform in [100, 100k] from the sphere / torus-knot / soup
generators, square resolutions from {64, 128, 256, 512}, half of them with
Msaa{level: 1}, each with its own 256^2 RGBA8 texture (textured Phong).
Inputs are synthetic and seeded (no dataset is involved); they stay resident
in HBM for `value`.

Printed as one JSON line (rank 0):
  value        batched scenes/s through euc_render_batch (whole job)
  per_scene    scenes/s for the same scenes through euc_render one scene pass
               at a time, with the call arguments built once
  e2e          scenes/s through the blocking host-buffer batch call
               euc_render_host_batch (host->device copies of inputs and targets,
               device->host copy of the targets, all inside the timed region);
               per_scene_value: the same through euc_render_host per scene
  mfrag_per_s  candidate fragments (inside + z-clip, exact counts) per second
  roofline     algorithmic bytes per batch / the dominant stage's CUDA-event
               time per batch, against the measured HBM copy bandwidth; the
               stage's kernels' DRAM bytes (ncu, profiles/traffic.json) over
               the same time; and `issue`: candidate fragments per second of
               the raster stage against every issue slot running full warps of
               the fewest instructions a candidate needs
  pipeline_roofline  the whole step's algorithmic bytes against the same peak
  cpu_baseline the CPU oracle (a port of euc's render_par: row bands over all
               host threads) on a bounded sample of the same scenes
  other_configs  measured after the headline in the same process (unless
               --no-extras): the 640x480 sphere stream (1024 frames per step),
               the 1080p 200k-triangle soup, the two-pass torus knot (4 frames
               per step), each batched and per scene with rates, stage times
               and rooflines, and a serving sweep at 2k, 10k and 50k
               requests/s (--serve-short-seconds each), with their own clocks

With --impl reference the CPU oracle is timed alone on the same workload (the
reference's CPU path; euc itself is Rust and cannot be built here).
The launch shape is autotuned per workload (strip path, raster and chunk
knobs); --no-tune keeps the default shape and --tuning '{"strip_path": 2}'
(fields of euc_tuning as JSON) fixes one, for profiles of a known shape.
With torchrun (N > 1) every rank renders its own 256 scenes (replicas, no
collective on the data path) and the slowest rank's time is used.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_SCENES = 256
# name -> (description, frames per step by default, unit)
WORKLOADS = {
    "batch": ("256 scenes, tris logU[100,1e5] (sphere/knot/soup), res U{64,128,256,512}^2, "
              "50% Msaa{level:1}, 256^2 RGBA8 textures, textured Phong", N_SCENES, "scenes/s"),
    "sphere": ("640x480 RGB8 + f32 depth, UV sphere 64x32 (3,968 tris), Gouraud, seeded rotation per frame, "
               "LESS_WRITE, back-face culling", 1024, "frames/s"),
    "soup": ("1920x1080 RGBA8 + f32 depth, 200k-triangle clip-space soup, areas logU[1,1e4] px, "
             "per-vertex RGBA8, LESS_WRITE, permuted u32 indices", 1, "frames/s"),
    "knot": ("two passes: 2048^2 f32 shadow map, then 1920x1080 RGBA8 textured Phong (1024^2 value noise, "
             "tiled bilinear) with Msaa{level:1}; (2,3) torus knot, 500k tris", 4, "frames/s"),
    "serve": ("serving loop: Poisson arrivals, 64 resident meshes (tris logU[100,1e5], sphere/knot/soup) and 32 "
              "resident 512^2 RGBA8 textures, two passes (res^2 f32 shadow map, textured Phong + shadow into "
              "RGBA8 + f32 depth), res U{64,128,256,512}^2, 50% Msaa{level:1}, colour read back to pinned host "
              "memory, 40 GB framebuffer budget", 512, "requests/s"),
}
WORKLOAD = WORKLOADS["batch"][0]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--scenes", type=int, default=N_SCENES)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-baseline", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    ap.add_argument("--only-batched", action="store_true",
                    help="run only the batched leg (no per-scene, e2e or CPU legs), e.g. under ncu")
    ap.add_argument("--workload", default="batch", choices=sorted(WORKLOADS),
                    help="batch: the 256 uneven scenes (default); sphere / soup / knot: the small plain, "
                         "fill-rate and two-pass configurations, --frames of them per step")
    ap.add_argument("--frames", type=int, default=0, help="frames per step for sphere/soup/knot (0 = default)")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape (no autotuning)")
    ap.add_argument("--tuning", default=None,
                    help='fixed launch shape instead of autotuning, as JSON fields of euc_tuning, e.g. \'{"strip_path": 2}\'')
    ap.add_argument("--no-graph", action="store_true", help="time plain euc_render_batch calls only")
    ap.add_argument("--rates", default="2000,10000,50000", help="serve: Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="serve: length of each rate's run")
    ap.add_argument("--max-batch", type=int, default=256, help="serve: requests per batch at most")
    ap.add_argument("--slots", type=int, default=3, help="serve: batches in flight at once")
    ap.add_argument("--no-extras", action="store_true",
                    help="batch: skip the other configurations (sphere, soup, knot, serving) after the headline")
    ap.add_argument("--serve-short-seconds", type=float, default=2.0,
                    help="the serving sweep's length per rate when it runs after the headline")
    args = ap.parse_args()
    if args.workload != "batch":
        args.scenes = args.frames or WORKLOADS[args.workload][1]
    return args


def dist_env():
    from euc_gb300 import replicas
    return replicas.dist_env()


def run_config(args, specs, world):
    """The `config` of a bench line; both arms print the same one."""
    alg_bytes = sum(f.algorithmic_bytes() for f in specs)
    keys = 8 * sum(t.width * t.height for f in specs for t in f.targets if t.fmt != 4)
    return {"workload": WORKLOADS[args.workload][0], "name": args.workload, "scenes": args.scenes, "seed": args.seed,
            "l2": "no flush: %.0f MB of inputs and targets per step > 129 MB L2" % ((alg_bytes + keys) / 1e6),
            "parallelism": "replicas" if world > 1 else "1 GPU"}


def make_frames(args, rank):
    from euc_gb300 import replicas, scenes
    seed = replicas.replica_seed(args.seed, rank)
    if args.workload == "sphere":
        return [scenes.sphere_frame(seed=seed + i) for i in range(args.scenes)]
    if args.workload == "soup":
        return [scenes.soup_frame(seed=seed + i) for i in range(args.scenes)]
    if args.workload == "knot":
        return [scenes.knot_frame(seed=seed + i) for i in range(args.scenes)]
    if args.workload == "serve":
        assets = scenes.serve_assets(seed=seed)
        rng = np.random.default_rng(seed + 1)
        return [scenes.serve_frame(assets, rng) for _ in range(args.scenes)]
    return scenes.batch_frames(seed=seed, n=args.scenes)


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, bus_id=None):
        self.bus_id = bus_id
        self.proc = None
        self.lines = []

    def start(self):
        cmd = ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits", "-lms", "200"]
        if self.bus_id:
            cmd += ["-i", self.bus_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU legs (oracle = CPU restatement of euc's render_par)
# ---------------------------------------------------------------------------
def cpu_sample(frames, budget_s, start=0, cap=None):
    """Renders scenes start, start+1, ... (rotating through `frames`) with the
    oracle on every host thread until `budget_s` has passed, or `cap` scenes;
    returns (scenes, seconds, threads)."""
    from oracle import oracle
    threads = oracle.hw_threads()
    n, t0 = 0, time.perf_counter()
    while (cap is None or n < cap) and (time.perf_counter() - t0) < budget_s:
        oracle.run_frame(frames[(start + n) % len(frames)], threads=threads)
        n += 1
    return n, time.perf_counter() - t0, threads


def run_reference(args):
    """--impl reference: the CPU oracle alone, on rank 0 only."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    frames = make_frames(args, 0)
    per_step = max(2.0, 150.0 / max(1, args.steps + args.warmup))
    pos = 0
    for _ in range(args.warmup):
        n, _, _ = cpu_sample(frames, per_step / 4, pos)
        pos += n
    total_n, total_t, threads = 0, 0.0, 1
    for _ in range(args.steps):
        n, t, threads = cpu_sample(frames, per_step, pos)
        pos += n
        total_n += n
        total_t += t
    v = total_n / total_t
    desc, _, unit = WORKLOADS[args.workload]
    out = {"metric": "%s (batched render, exact coverage)" % unit, "impl": "reference", "value": v,
           "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * total_t / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators)",
           "config": run_config(args, frames, world),
           "cpu_baseline": {"value": v, "unit": unit, "cores": threads, "kind": "port",
                            "sample": "%d scenes (rotating through the %d) in %.1f s" % (total_n, len(frames), total_t)},
           "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# ---------------------------------------------------------------------------
# GPU legs
# ---------------------------------------------------------------------------
def host_bytes(frames):
    h2d = d2h = 0
    for f in frames:
        for p in f.passes:
            h2d += p.vertices.nbytes + (p.indices.nbytes if p.indices is not None else 0)
            h2d += sum(s.source.nbytes for s in p.samplers if not isinstance(s.source, str))
        for t in f.targets:
            b = t.width * t.height * t.bpp
            h2d += b
            d2h += b
    return h2d, d2h


def run_e2e(ctx, frames, reps):
    """Blocking host-buffer renders (euc_render_host), one per scene pass,
    called with their arguments ready (as a caller holding its uniforms and
    buffers would).  The host targets are reset to their clear values before
    each repetition, outside the timed region."""
    import ctypes as C
    from euc_gb300 import abi, capi
    hosts = [f.alloc_host_targets() for f in frames]
    clean = [{k: v.copy() for k, v in h.items()} for h in hosts]
    calls, keep = [], []
    for f, h in zip(frames, hosts):
        for p in f.passes:
            uni, kp = p.bind_uniforms(lambda src, f=f, h=h: f.host_texture_ptr(src, h))
            pix = h[p.pixel] if p.pixel else None
            dep = h[p.depth] if p.depth else None
            fmt = f.target(p.pixel).fmt if p.pixel else abi.FMT_NONE
            pt = abi.Target(pix.ctypes.data, pix.shape[1], pix.shape[0], pix.strides[0], fmt) if pix is not None \
                else abi.Target(None, 0, 0, 0, 0)
            dt = abi.Target(dep.ctypes.data, dep.shape[1], dep.shape[0], dep.strides[0], abi.FMT_R32F) \
                if dep is not None else abi.Target(None, 0, 0, 0, 0)
            keep.append((uni, kp, pt, dt))
            calls.append((ctx.handle, C.byref(p.desc), C.addressof(uni), C.sizeof(uni), C.byref(p.layout),
                          p.vertices.ctypes.data, p.nverts,
                          p.indices.ctypes.data if p.indices is not None else None,
                          p.indices.size if p.indices is not None else 0, C.byref(pt), C.byref(dt)))
    render_host = capi.lib().euc_render_host

    def reset():
        for h, c in zip(hosts, clean):
            for k in h:
                np.copyto(h[k], c[k])

    def one_pass():
        for a in calls:
            rc = render_host(*a)
            if rc != abi.OK:
                raise RuntimeError("euc_render_host failed: %d" % rc)

    reset()
    one_pass()  # warm-up (allocations)
    total = 0.0
    for _ in range(reps):
        reset()
        t0 = time.perf_counter()
        one_pass()
        total += time.perf_counter() - t0
    return reps * len(frames) / total


def run_e2e_batch(ctx, frames, reps):
    """The batched form on host buffers (euc_render_host_batch): pass k of
    every frame in the k-th call; inputs and targets go up, targets come
    back, inside each timed call.  The host targets are reset to their clear
    values before each step, outside the timed region."""
    import ctypes as C
    from euc_gb300 import abi
    hosts = [f.alloc_host_targets() for f in frames]
    clean = [{k: v.copy() for k, v in h.items()} for h in hosts]
    npass = max(len(f.passes) for f in frames)
    keep = []

    def scene_arrays():
        arrays = []
        for k in range(npass):
            sc = []
            for f, h in zip(frames, hosts):
                if k >= len(f.passes):
                    continue
                p = f.passes[k]
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
                s.pixel = abi.Target(pix.ctypes.data, pix.shape[1], pix.shape[0], pix.strides[0], fmt) \
                    if pix is not None else abi.Target(None, 0, 0, 0, 0)
                s.depth = abi.Target(dep.ctypes.data, dep.shape[1], dep.shape[0], dep.strides[0], abi.FMT_R32F) \
                    if dep is not None else abi.Target(None, 0, 0, 0, 0)
                s.uniforms = C.addressof(uni)
                s.uniforms_size = C.sizeof(uni)
                sc.append(s)
            arrays.append((abi.Scene * len(sc))(*sc))
        return arrays

    arrays = scene_arrays()

    def reset():
        for h, c in zip(hosts, clean):
            for k in h:
                np.copyto(h[k], c[k])

    def step():
        for arr in arrays:
            rc = ctx.render_host_batch(arr)
            if rc != abi.OK:
                raise RuntimeError("euc_render_host_batch failed: %d" % rc)

    reset()
    step()  # warm-up (allocations, page-locked staging)
    total = 0.0
    for _ in range(reps):
        reset()
        t0 = time.perf_counter()
        step()
        total += time.perf_counter() - t0
    return reps * len(frames) / total


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_profile_json(name):
    """A summary committed under profiles/ (ncu figures), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", name)) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


# The kernels each profiled stage holds (CUDA-event stage times).
STAGE_KERNELS = {"vertex": ["k_vertex"], "setup": ["k_setup", "k_bin_count"], "scan": ["k_scan_plan"],
                 "init": ["k_init"], "raster": ["k_bin", "k_strip", "k_raster"], "resolve": ["k_resolve"]}

# The fewest thread instructions a candidate fragment needs in euc's walk
# (triangles.rs:257-301): three additions that advance the weights, two for
# the third weight, three compares, the z dot product (three multiplies, two
# additions), the key (five integer operations) and its reduction.
MIN_INST_PER_CANDIDATE = 19


def prebuilt_render_calls(ctx, batch, sp):
    """The euc_render argument tuples of every scene pass of `batch`, built
    once, as a caller that holds its pipeline, uniforms and buffers calls
    it: pass k of every frame after pass k - 1 of every frame."""
    import ctypes as C
    calls = []
    for arr in batch.scene_arrays():
        for sc in arr:
            calls.append((ctx.handle, C.byref(sc.desc), sc.uniforms, sc.uniforms_size, C.byref(sc.layout),
                          sc.vertices, sc.nverts, sc.indices, sc.nindices, C.byref(sc.pixel), C.byref(sc.depth), sp))
    return calls


def measure(ctx, specs, dev, stream, steps, warmup, tune, graph_ok=True, world=1, tune_reps=9, per_scene_reps=2,
            fixed_tuning=None):
    """One workload on the GPU: the batched form (plain calls with per-stage
    CUDA events, and the recorded graph), the candidate count of one step,
    and the plain per-scene path (euc_render per scene pass, arguments built
    once).  Times are device times of `steps` steps, max over ranks."""
    import torch
    import torch.distributed as dist
    from euc_gb300 import abi, capi, replicas, frames as fr

    batch = fr.DeviceBatch(specs, dev)

    def step():
        fr.render_batch(ctx, batch, stream, clear=True)

    tuning, tune_info = None, None
    if fixed_tuning:
        tuning = abi.Tuning(**fixed_tuning)
        ctx.set_tuning(tuning)
        tune_info = {"fixed": fixed_tuning}
    elif tune:
        from euc_gb300 import autotune
        tuning, tune_info = autotune.tune(ctx, batch, stream, reps=tune_reps)
    graph = None
    if graph_ok and not any(s.desc.blend == 1 or s.desc.flags & 2 for arr in batch.scene_arrays() for s in arr):
        graph = fr.BatchGraph(ctx, batch)
    for _ in range(max(warmup, 3)):
        step()
        if graph:
            graph.launch(stream)
    capi.check(ctx.sync(fr._stream_ptr(stream)), "warm-up")
    # candidate fragments of one step, pass by pass (statistics cover one batch call)
    cand = 0
    batch.clear()
    sp = fr._stream_ptr(stream)
    for arr in batch.scene_arrays():
        capi.check(ctx.render_scene_array(arr, sp), "render_batch")
        cand += ctx.stats(sp).candidates
    ctx.profile()  # reset the counters

    def timed(fn, n):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(n):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        t = replicas.max_over_ranks(e0.elapsed_time(e1), device=dev)
        if world > 1:
            dist.barrier()
        return t

    ctx.set_profiling(True)
    ms_plain = timed(step, steps)
    ctx.set_profiling(False)
    stage_ms, launches = ctx.profile()
    ms_graph, graph_launches = None, None
    if graph:
        ms_graph = timed(lambda: graph.launch(stream), steps)
        _, graph_launches = ctx.profile()
    form = "graph" if ms_graph and ms_graph <= ms_plain else "plain"
    ms = ms_graph if form == "graph" else ms_plain
    # the plain per-scene path with the default launch shape
    per_scene = None
    if per_scene_reps:
        tuned = ctx.get_tuning()
        ctx.set_tuning(None)
        calls = prebuilt_render_calls(ctx, batch, sp)
        render = capi.lib().euc_render

        def per_scene_pass():
            batch.clear()
            for a in calls:
                rc = render(*a)
                if rc != abi.OK:
                    raise RuntimeError("euc_render failed: %d" % rc)
        for _ in range(2):  # euc_render records a scene shape's launches the second time it sees it
            per_scene_pass()
        capi.check(ctx.sync(sp), "per-scene warm-up")
        t = timed(per_scene_pass, per_scene_reps)
        per_scene = len(specs) / (t / per_scene_reps / 1e3)
        ctx.set_tuning(tuned)
    if graph:
        graph.close()
    alg = sum(f.algorithmic_bytes() for f in specs)
    clear = sum(t.width * t.height * t.bpp for f in specs for t in f.targets)
    return {"ms_step": ms / steps, "ms_plain_step": ms_plain / steps,
            "ms_graph_step": ms_graph / steps if ms_graph else None, "form": form,
            "stage_ms": {k: v / steps for k, v in stage_ms.items()},
            "launches": int(graph_launches if form == "graph" else launches) // steps,
            "cand": cand, "alg_bytes": alg, "clear_bytes": clear, "per_scene": per_scene,
            "tuning": tuning.as_dict() if tuning is not None else None, "autotune": tune_info, "batch": batch}


def rooflines(m, name, peak, peak_kind, clk_mhz):
    """The HBM roofline of the dominant stage (algorithmic bytes over its
    CUDA-event time; its kernels' measured DRAM bytes over the same time,
    where a profile of this workload holds them), the whole step's HBM
    fraction, and the issue-side roofline of the raster stage."""
    stage = m["stage_ms"]
    dom = max(stage, key=lambda k: stage[k])
    dom_s = stage[dom] / 1e3
    achieved = m["alg_bytes"] / dom_s / 1e9
    traffic = load_profile_json("traffic.json") or {}
    tw = traffic.get(name, {})
    kb = [tw.get(k) for k in STAGE_KERNELS[dom]]
    dram = sum(b for b in kb if b) if any(kb) else None
    step_s = m["ms_step"] / 1e3
    roof = {"bound": "hbm", "stage": dom, "kernels": STAGE_KERNELS[dom], "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
            "algorithmic_bytes_per_launch": m["alg_bytes"],
            "traffic": dram,
            "dram_frac": (dram / dom_s / 1e9 / peak) if dram else None}
    # issue side: candidate fragments per second against every issue slot of
    # the GPU running full warps of the fewest instructions a candidate needs
    rs = stage["raster"] / 1e3
    sm_mhz = clk_mhz or 2070.0
    peak_cand = 152 * 4 * sm_mhz * 1e6 * 32 / MIN_INST_PER_CANDIDATE
    issue = {"stage": "raster", "candidates_per_step": m["cand"], "achieved": m["cand"] / rs, "peak": peak_cand,
             "unit": "candidates/s", "frac": m["cand"] / rs / peak_cand,
             "min_thread_inst_per_candidate": MIN_INST_PER_CANDIDATE, "sm_mhz": sm_mhz}
    prof = (load_profile_json("issue.json") or {}).get(name)
    if prof:
        issue["ncu"] = prof
    roof["issue"] = issue
    pipe = {"achieved": m["alg_bytes"] / step_s / 1e9, "peak": peak, "unit": "GB/s",
            "frac": m["alg_bytes"] / step_s / 1e9 / peak, "peak_kind": peak_kind,
            "clear_bytes_per_step": m["clear_bytes"],
            "frac_with_clear": (m["alg_bytes"] + m["clear_bytes"]) / step_s / 1e9 / peak}
    return roof, pipe


def serve_sweep(local, frames, rates, seconds, max_batch, slots, warmup, seed, rank=0):
    """The serving loop under open-loop Poisson arrivals, one run per rate.
    Requests draw uniformly from a pool of seeded two-pass requests over the
    resident meshes and textures; each run reports latency percentiles
    (arrival to colour on the host) and throughput."""
    import torch
    from euc_gb300 import abi, serve

    srv = serve.Server(local, framebuffer_budget=40 << 30, max_batch=max_batch, slots=slots)
    res = serve.Resident(srv)
    pins, keep, pool, outs = [], [], [], []
    for k, f in enumerate(frames):
        n = serve.out_bytes(f, ("color",))
        bufs = [torch.empty(n, dtype=torch.uint8).pin_memory() for _ in range(4)]
        pins += bufs
        outs.append([(b.data_ptr(), n) for b in bufs])
        r, kp = serve.request_for(f, res, ("color",), tag=k, out=bufs[0].data_ptr(), out_size=n)
        pool.append(r)
        keep.append(kp)
    arr = (abi.ServerRequest * len(pool))(*pool)
    for _ in range(max(warmup, 3)):
        # enough at once that every slot takes full batches: each slot's
        # scratch is sized before the timed runs
        for _ in range(max(slots, 1)):
            srv.submit(arr)
        srv.drain()
        while len(srv.poll(8192)):
            pass
    base = srv.stats()
    runs = []
    for i, rate in enumerate(rates):
        _, summ = serve.run_poisson(srv, arr, outs, rate, seconds, seed=seed + 17 * i + rank)
        summ.pop("stats")
        runs.append(summ)
    st = srv.stats()
    srv.close()
    out_mean = float(np.mean([serve.out_bytes(f, ("color",)) for f in frames]))
    return runs, int(st["launches"] - base["launches"]), out_mean


def other_configs(args, ctx, dev, stream, peak, peak_kind):
    """The other configurations, measured after the headline one in the
    same process: the 640x480 sphere stream, the 1080p soup, the two-pass
    knot (each batched and per scene), and a shortened serving sweep."""
    from euc_gb300 import scenes
    out = {}
    plan = [("sphere", [scenes.sphere_frame(seed=i) for i in range(1024)], 5, "frames/s"),
            ("soup", [scenes.soup_frame(seed=0)], 20, "frames/s"),
            ("knot", [scenes.knot_frame(seed=i) for i in range(4)], 10, "frames/s")]
    clocks = ClockSampler(_bus_id(dev))
    clocks.start()
    time.sleep(1.0)
    for name, specs, steps, unit in plan:
        m = measure(ctx, specs, dev, stream, steps, 3, tune=True, tune_reps=5, per_scene_reps=2)
        rate = len(specs) / (m["ms_step"] / 1e3)
        roof, pipe = rooflines(m, name, peak, peak_kind, None)
        out[name] = {"workload": WORKLOADS[name][0], "frames_per_step": len(specs), "value": rate, "unit": unit,
                     "form": m["form"], "plain_value": len(specs) / (m["ms_plain_step"] / 1e3),
                     "per_scene": m["per_scene"], "batched_speedup": rate / m["per_scene"] if m["per_scene"] else None,
                     "ms_per_step": m["ms_step"], "stage_ms_per_step": m["stage_ms"], "gpu_launches": m["launches"],
                     "mfrag_per_s": m["cand"] / (m["ms_step"] / 1e3) / 1e6,
                     "mtri_per_s": sum(f.ntris for f in specs) / (m["ms_step"] / 1e3) / 1e6,
                     "tuning": m["tuning"], "roofline": roof, "pipeline_roofline": pipe}
        del m
    runs, launches, out_mean = serve_sweep(dev.index if hasattr(dev, "index") else 0,
                                           make_frames(argparse.Namespace(workload="serve", seed=args.seed,
                                                                          scenes=WORKLOADS["serve"][1]), 0),
                                           [2000.0, 10000.0, 50000.0], args.serve_short_seconds, 256, 3, 3,
                                           args.seed)
    out["serve"] = {"workload": WORKLOADS["serve"][0], "unit": "requests/s", "seconds_per_rate": args.serve_short_seconds,
                    "runs": runs, "gpu_launches": launches, "readback_bytes_per_request": out_mean}
    out["clocks"] = clocks.stop()
    return out


def _bus_id(dev):
    import torch
    try:
        return torch.cuda.get_device_properties(dev).pci_bus_id
    except AttributeError:
        return None


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from euc_gb300 import capi

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    specs = make_frames(args, rank)
    ctx = capi.Context(local)
    stream = torch.cuda.current_stream()
    peak, peak_kind = load_peaks()

    clocks = ClockSampler(_bus_id(dev))
    clocks.start()
    time.sleep(0.3)
    m = measure(ctx, specs, dev, stream, args.steps, args.warmup, tune=not args.no_tune, graph_ok=not args.no_graph,
                fixed_tuning=json.loads(args.tuning) if args.tuning else None,
                world=world, per_scene_reps=0 if args.only_batched else max(2, args.steps // 4))
    clk = clocks.stop()
    value = world * args.scenes / (m["ms_step"] / 1e3)
    e2e = e2e_per_scene = None
    if not args.only_batched:
        e2e_per_scene = run_e2e(ctx, specs, reps=1)
        e2e = run_e2e_batch(ctx, specs, reps=max(2, min(args.steps, 5)))
    h2d, d2h = host_bytes(specs)
    host_copy = ("in place: kernels read vertices and indices and update targets in host memory over "
                 "NVLink-C2C; one kernel gathers the textures") if ctx.host_copy_direct() else \
        "staged through page-locked memory by host threads, one copy each way"
    roof, pipe = rooflines(m, args.workload if not args.frames and args.scenes == WORKLOADS[args.workload][1]
                           else "", peak, peak_kind, clk.get("sm_mhz"))
    cpu = None
    if rank == 0 and not args.no_baseline and not args.only_batched:
        n, t, threads = cpu_sample(specs, args.cpu_seconds)
        cpu = {"value": n / t, "unit": WORKLOADS[args.workload][2], "cores": threads, "kind": "port",
               "sample": "%d scenes (rotating through the %d of one step) in %.1f s (oracle render_par, %d threads)"
                         % (n, len(specs), t, threads)}
    others = None
    if args.workload == "batch" and not args.only_batched and not args.no_extras and world == 1:
        del m["batch"]
        others = other_configs(args, ctx, dev, stream, peak, peak_kind)
    if rank == 0:
        unit = WORKLOADS[args.workload][2]
        out = {
            "metric": "%s (batched render, exact coverage)" % unit, "value": value, "unit": unit,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators), resident in HBM",
            "config": run_config(args, specs, world),
            "form": {"timed": "euc_graph replay" if m["form"] == "graph" else "euc_render_batch calls",
                     "plain_value": world * args.scenes / (m["ms_plain_step"] / 1e3),
                     "graph_value": world * args.scenes / (m["ms_graph_step"] / 1e3) if m["ms_graph_step"] else None,
                     "tuning": m["tuning"], "autotune": m["autotune"]},
            "per_scene": {"value": m["per_scene"], "unit": unit,
                          "path": "euc_render per scene pass, arguments built once"},
            "batched_speedup": value / world / m["per_scene"] if m["per_scene"] else None,
            "mfrag_per_s": m["cand"] * world / (m["ms_step"] / 1e3) / 1e6,
            "mtri_per_s": sum(f.ntris for f in specs) * world / (m["ms_step"] / 1e3) / 1e6,
            "stage_ms_per_step": m["stage_ms"],
            "gpu_launches": m["launches"] * args.steps,
            "roofline": roof,
            "pipeline_roofline": pipe,
            "e2e": {"value": e2e, "unit": unit, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "path": "euc_render_host_batch (host buffers, blocking; one call per pass)",
                    "host_copy": host_copy,
                    "bytes": "host-buffer bytes each step's calls read (inputs, textures, targets) and write "
                             "(targets); in place, only the covered pixels of a target cross the link",
                    "per_scene_value": e2e_per_scene,
                    "per_scene_path": "euc_render_host per scene (host buffers, blocking)"},
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        if others is not None:
            out["other_configs"] = others
        print(json.dumps(out), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def run_serve(args):
    """--workload serve: the serving loop alone, at --rates for --serve-seconds each."""
    import torch
    import torch.distributed as dist

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    frames = make_frames(args, rank)
    clocks = ClockSampler(_bus_id(torch.device("cuda", local)))
    clocks.start()
    time.sleep(1.0)  # the sampler's start (NVML set-up) stays out of the first run
    runs, launches, out_mean = serve_sweep(local, frames, [float(r) for r in args.rates.split(",")],
                                           args.serve_seconds, args.max_batch, args.slots, args.warmup,
                                           args.seed, rank)
    clk = clocks.stop()
    top = runs[-1]
    tot = [torch.tensor([r["throughput"]], device="cuda:%d" % local) for r in runs]
    if world > 1:
        for t in tot:
            dist.all_reduce(t)
        dist.destroy_process_group()
    if rank == 0:
        desc, _, unit = WORKLOADS["serve"]
        out = {
            "metric": "served requests/s with p50/p99 latency (arrival to colour on host)", "value": float(tot[-1].item()),
            "unit": unit, "n_gpus": world, "steps": len(runs), "warmup": max(args.warmup, 3),
            "ms_per_step": 1e3 * args.serve_seconds, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators), meshes/textures resident",
            "config": {"workload": desc, "name": "serve", "pool": len(frames), "seed": args.seed,
                       "rates": args.rates, "seconds_per_rate": args.serve_seconds, "max_batch": args.max_batch,
                       "slots": args.slots, "parallelism": "replicas" if world > 1 else "1 GPU"},
            "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
            "serving": runs,
            "gpu_launches": launches,
            "e2e": {"value": float(tot[-1].item()), "unit": unit, "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": out_mean * top["completed"],
                    "path": "euc_server_submit -> completion with colour in pinned host memory"},
            "roofline": None, "cpu_baseline": None, "clocks": clk,
        }
        print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
