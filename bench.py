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
  per_scene    scenes/s for the same scenes through euc_render one at a time
  e2e          scenes/s through the blocking host-buffer batch call
               euc_render_host_batch (host->device copies of inputs and targets,
               device->host copy of the targets, all inside the timed region);
               per_scene_value: the same through euc_render_host per scene
  mfrag_per_s  candidate fragments (inside + z-clip, exact counts) per second
  roofline     algorithmic bytes per batch / the dominant stage's CUDA-event
               time per batch, against the measured HBM copy bandwidth
  cpu_baseline the CPU oracle (a port of euc's render_par: row bands over all
               host threads) on a bounded sample of the same scenes

With --impl reference the CPU oracle is timed alone on the same workload (the
reference's CPU path; euc itself is Rust and cannot be built here).
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
    ap.add_argument("--no-graph", action="store_true", help="time plain euc_render_batch calls only")
    ap.add_argument("--rates", default="2000,10000,50000", help="serve: Poisson arrival rates (requests/s)")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="serve: length of each rate's run")
    ap.add_argument("--max-batch", type=int, default=256, help="serve: requests per batch at most")
    ap.add_argument("--slots", type=int, default=3, help="serve: batches in flight at once")
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


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from euc_gb300 import capi, replicas, frames as fr

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = "cuda:%d" % local
    specs = make_frames(args, rank)
    ctx = capi.Context(local)
    batch = fr.DeviceBatch(specs, dev)
    stream = torch.cuda.current_stream()

    def step():
        fr.render_batch(ctx, batch, stream, clear=True)

    tuning, tune_info = None, None
    if not args.no_tune:
        from euc_gb300 import autotune
        tuning, tune_info = autotune.tune(ctx, batch, stream, reps=9)
    # the recorded form of the same batch (scenes on the ordered path cannot be recorded)
    graph = None
    if not args.no_graph and not any(s.desc.blend == 1 or s.desc.flags & 2 for arr in batch.scene_arrays()
                                     for s in arr):
        graph = fr.BatchGraph(ctx, batch)

    for _ in range(max(args.warmup, 3)):
        step()
        if graph:
            graph.launch(stream)
    capi.check(ctx.sync(fr._stream_ptr(stream)), "warm-up")
    # candidate fragments of one step, pass by pass (stats cover one batch call)
    cand_per_step = 0
    batch.clear()
    npass = max(len(f.frame.passes) for f in batch.frames)
    for k in range(npass):
        scenes_k, keep = [], []
        for df in batch.frames:
            if k < len(df.frame.passes):
                s, kp = df.scene(k)
                scenes_k.append(s)
                keep.append(kp)
        capi.check(ctx.render_batch(scenes_k, fr._stream_ptr(stream)), "render_batch")
        cand_per_step += ctx.stats(fr._stream_ptr(stream)).candidates
    ctx.profile()  # reset counters

    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id
    except AttributeError:
        pass
    clocks = ClockSampler(bus)
    ctx.set_profiling(True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)

    def timed(fn):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        t = replicas.max_over_ranks(e0.elapsed_time(e1), device=dev)
        if world > 1:
            dist.barrier()
        return t

    # plain calls with per-stage CUDA events (the stage times of the roofline)
    ms_plain = timed(step)
    ctx.set_profiling(False)
    stage_ms, launches = ctx.profile()
    ms_graph = None
    if graph:
        ms_graph = timed(lambda: graph.launch(stream))
        _, graph_launches = ctx.profile()
    clk = clocks.stop()
    ms = min(ms_plain, ms_graph) if ms_graph else ms_plain
    form = "graph" if ms_graph and ms_graph <= ms_plain else "plain"
    if form == "graph":
        launches = graph_launches
    ms_step = ms / args.steps
    value = world * args.scenes / (ms_step / 1e3)

    # per-scene plain path on the same scenes (euc_render, one call per scene)
    def per_scene_pass():
        batch.clear()
        for df in batch.frames:
            fr.render_frame(ctx, df, stream, clear=False)
    per_scene = e2e = e2e_per_scene = None
    if not args.only_batched:
        # the per-scene paths run with the default launch shape (the tuned one
        # is chosen for the batch)
        tuned = ctx.get_tuning()
        ctx.set_tuning(None)
        per_scene_pass()
        torch.cuda.synchronize()
        reps = max(2, args.steps // 4)
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for _ in range(reps):
            per_scene_pass()
        p1.record(stream)
        torch.cuda.synchronize()
        per_scene = args.scenes / (p0.elapsed_time(p1) / reps / 1e3)
        e2e_per_scene = run_e2e(ctx, specs, reps=1)
        ctx.set_tuning(tuned)
        e2e = run_e2e_batch(ctx, specs, reps=max(2, min(args.steps, 5)))
    h2d, d2h = host_bytes(specs)
    host_copy = ("in place: kernels read vertices and indices and update targets in host memory over "
                 "NVLink-C2C; one kernel gathers the textures") if ctx.host_copy_direct() else \
        "staged through page-locked memory by host threads, one copy each way"

    alg_bytes = sum(f.algorithmic_bytes() for f in specs)
    # each step also clears every target first, as euc's own bench loop does
    # (benches/teapot.rs:182-184): one more write of each target
    clear_bytes = sum(t.width * t.height * t.bpp for f in specs for t in f.targets)
    dom = max(stage_ms, key=lambda k: stage_ms[k])
    dom_ms = stage_ms[dom] / args.steps
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (dom_ms / 1e3) / 1e9
    traffic = load_traffic()
    cpu = None
    if rank == 0 and not args.no_baseline and not args.only_batched:
        n, t, threads = cpu_sample(specs, args.cpu_seconds)
        cpu = {"value": n / t, "unit": WORKLOADS[args.workload][2], "cores": threads, "kind": "port",
               "sample": "%d scenes (rotating through the %d of one step) in %.1f s (oracle render_par, %d threads)"
                         % (n, len(specs), t, threads)}
    if rank == 0:
        desc, _, unit = WORKLOADS[args.workload]
        out = {
            "metric": "%s (batched render, exact coverage)" % unit, "value": value, "unit": unit,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generators), resident in HBM",
            "config": run_config(args, specs, world),
            "form": {"timed": "euc_graph replay" if form == "graph" else "euc_render_batch calls",
                     "plain_value": world * args.scenes / (ms_plain / args.steps / 1e3),
                     "graph_value": world * args.scenes / (ms_graph / args.steps / 1e3) if ms_graph else None,
                     "tuning": tuning.as_dict() if tuning is not None else None, "autotune": tune_info},
            "per_scene": {"value": per_scene, "unit": unit, "path": "euc_render per scene"},
            "batched_speedup": value / world / per_scene if per_scene else None,
            "mfrag_per_s": cand_per_step * world / (ms_step / 1e3) / 1e6,
            "mtri_per_s": sum(f.ntris for f in specs) * world / (ms_step / 1e3) / 1e6,
            "stage_ms_per_step": {k: v / args.steps for k, v in stage_ms.items()},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "kernel": "k_" + dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         # captured at the default workload sizes only
                         "traffic": traffic.get(args.workload, {}).get("k_" + dom)
                         if traffic and not args.frames and args.scenes == N_SCENES else None},
            # the whole step (every stage, launch gaps included) against the same peak
            "pipeline_roofline": {"achieved": alg_bytes / (ms_step / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                                  "frac": alg_bytes / (ms_step / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
                                  "clear_bytes_per_step": clear_bytes,
                                  "frac_with_clear": (alg_bytes + clear_bytes) / (ms_step / 1e3) / 1e9 / peak},
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
        print(json.dumps(out), flush=True)
    if graph:
        graph.close()
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def run_serve(args):
    """The serving loop under open-loop Poisson arrivals, one run per rate.
    Requests draw uniformly from a pool of `--scenes` seeded two-pass
    requests over the resident meshes and textures; each run reports
    latency percentiles (arrival to colour on the host) and throughput."""
    import ctypes as C

    import torch
    import torch.distributed as dist
    from euc_gb300 import abi, serve

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    frames = make_frames(args, rank)
    srv = serve.Server(local, framebuffer_budget=40 << 30, max_batch=args.max_batch, slots=args.slots)
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
    for _ in range(max(args.warmup, 3)):
        # enough at once that every slot takes full batches: each slot's
        # scratch is sized before the timed runs
        for _ in range(max(args.slots, 1)):
            srv.submit(arr)
        srv.drain()
        while len(srv.poll(8192)):
            pass
    base = srv.stats()
    bus = None
    try:
        bus = torch.cuda.get_device_properties(local).pci_bus_id
    except AttributeError:
        pass
    runs = []
    clocks = ClockSampler(bus)
    clocks.start()
    time.sleep(1.0)  # the sampler's start (NVML set-up) stays out of the first run
    for i, rate in enumerate(float(r) for r in args.rates.split(",")):
        _, summ = serve.run_poisson(srv, arr, outs, rate, args.serve_seconds, seed=args.seed + 17 * i + rank)
        summ.pop("stats")
        runs.append(summ)
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    top = runs[-1]
    tot = [torch.tensor([r["throughput"]], device="cuda:%d" % local) for r in runs]
    if world > 1:
        for t in tot:
            dist.all_reduce(t)
        dist.destroy_process_group()
    if rank == 0:
        desc, _, unit = WORKLOADS["serve"]
        per_req_out = float(np.mean([serve.out_bytes(f, ("color",)) for f in frames]))
        out = {
            "metric": "served requests/s with p50/p99 latency (arrival to colour on host)", "value": float(tot[-1].item()),
            "unit": unit, "n_gpus": world, "steps": len(runs), "warmup": max(args.warmup, 3),
            "ms_per_step": 1e3 * args.serve_seconds, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators), meshes/textures resident",
            "config": {"workload": desc, "name": "serve", "pool": len(frames), "seed": args.seed,
                       "rates": args.rates, "seconds_per_rate": args.serve_seconds, "max_batch": args.max_batch, "slots": args.slots,
                       "parallelism": "replicas" if world > 1 else "1 GPU"},
            "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"],
            "serving": runs,
            "gpu_launches": int(st["launches"] - base["launches"]),
            "e2e": {"value": float(tot[-1].item()), "unit": unit, "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": per_req_out * top["completed"],
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
