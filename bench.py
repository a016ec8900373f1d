"""Benchmark of the draw hot path (one JSON line on rank 0).

Default workload: 4096 indexed icosphere draws in one render pass (755 M
triangles with instancing, 2560x1440 RGBA8 + D32, opaque and src-over
pipelines), rendered through the Vulkan ICD per draw and batched (the
metric is batched vs per-draw). Other workloads: cube, heightfield (1024x1024
grid, trilinear texture), blend (200k quads), serve (64 clients). A step is
one frame: one vkQueueSubmit of the recorded command buffer (render-pass
clear + the draws) and its fence.

  value  Mtri/s with scene data resident in HBM, device time of K frames
         (queue events around each frame; a 256 MiB vkCmdFillBuffer before
         every frame evicts the 129 MB L2 and is not timed).
  plain  the same frames through the per-draw path (many-draw workloads).
  e2e    the same metric through the public API with host buffers: the
         vertex, index, uniform and texture bytes sit in a host-visible
         (pinned) staging buffer; every step maps and unmaps it (the ICD
         copies it to HBM), copies
         them to device-local buffers, renders, copies the colour image to a
         host-visible buffer and reads it back, wall-clock timed.

--impl reference times the reference's CPU draw path (its C++ restatement in
oracle/) on all host cores on the same scene. --gpus N under torchrun runs N
independent replicas (the path does not shard a frame).
"""
import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (harness config, params, description)
    "cube": (1, [30], "spinning cube 500x500 BGRA8+D16, 12 triangles, 1 draw"),
    "heightfield": (2, [], "textured heightfield 1024x1024 grid (2,093,058 tris, u32 indices), 1920x1080 RGBA8+D32, trilinear, Lambert"),
    "blend": (3, [], "200k screen-space quads (400k tris), sides log-uniform 4-256 px, src-over blend, 1920x1080 RGBA8"),
    "batch": (4, [], "4096 indexed icosphere draws (12-200k tris, 25% instanced 1-64x), 70/30 opaque/blended, 2560x1440 RGBA8+D32"),
    "serve": (6, [], "64 offscreen clients, Poisson arrivals (mean 2 ms each), 256-2048 px RGBA8+D32 images of 1k-500k textured "
                     "triangles, resident pipelines and attachments, 16 queues"),
}
FLUSH_BYTES = 256 << 20
FALLBACK_HBM_GBS = 6800.0


def workload(args):
    """(harness config, scene parameters, description) of the run; --params
    replaces the scene parameters (smaller cases for profiling)."""
    cfg, params, desc = CONFIGS[args.config]
    if args.params:
        params = [int(v) for v in args.params.split(",")]
        desc += " [params %s]" % args.params
    return cfg, params, desc


def algorithmic_bytes(name, scene, frag_written):
    """Bytes the frame must move at least once: every vertex, index, uniform
    and texture byte read once, plus the attachments — colour stored and
    depth read and written per pixel, or for the blend workloads an RGBA8
    read and write per blended fragment (the immediate-mode blend traffic)."""
    px = scene.width * scene.height
    if name.startswith("blend"):
        return 8 * frag_written + scene.input_bytes
    depth = 2 if name == "cube" else 4  # D16 / D32
    return scene.input_bytes + px * 4 + px * depth * 2


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def committed_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu summary, else None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            return json.load(fh).get(workload, {}).get(kernel)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, interval_ms=100):
        self.proc = None
        self.path = None
        self.interval_ms = interval_ms

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits", "-lms",
                                          str(self.interval_ms)],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}
        return out


def cpu_baseline(scene, seconds, threads=1):
    """Times the oracle (the reference's CPU draw path restated) on this host.

    Work units are whole frames for a one-draw scene and single draws of a
    many-draw scene (a 4096-draw frame takes minutes on one core). Each
    thread renders its units into its own attachments, pulling units in API
    order until `seconds` have passed (at least one unit per thread).
    Returns (triangles rendered, elapsed seconds, description).
    """
    import threading
    from tests import oracle_binding
    oracle = oracle_binding.load()
    per_draw = scene.draws > 1
    units = scene.draws if per_draw else None
    lock = threading.Lock()
    state = {"next": 0, "tris": 0, "units": 0}
    t0 = time.time()

    def worker(_):
        color = depth = None
        first = True
        while True:
            with lock:
                if state["units"] >= threads and time.time() - t0 >= seconds:
                    return
                i = state["next"]
                state["next"] += 1
            if per_draw:
                i %= units
                color, depth, st = oracle.render(scene, i, i + 1, color=color, depth=depth, clear=first)
                first = False
            else:
                color, depth, st = oracle.render(scene)
            with lock:
                state["tris"] += st["triangles"]
                state["units"] += 1

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(worker, range(threads)))
    dt = time.time() - t0
    what = "draws" if per_draw else "whole frames"
    desc = "%d %s (%d triangles) in %.1f s on %d thread(s)" % (state["units"], what, state["tris"], dt, threads)
    return state["tris"], dt, desc


def reference_frame(scene):
    """The CPU-baseline leg's whole frame: the oracle (the reference's CPU
    draw path restated) renders the full image on every host core, which
    also gives the frame's fragment counts and the image the GPU's is
    compared with. Returns (colour, depth, stats, seconds, threads)."""
    from tests import oracle_binding
    oracle = oracle_binding.load()
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    t0 = time.time()
    color, depth, st = oracle.render_threaded(scene, threads)
    return color, depth, st, time.time() - t0, threads


def image_diff(gpu_color, gpu_depth, ref_color, ref_depth):
    """Differing pixels of two renders (colour: any channel; depth: any
    byte of the texel), and the largest colour difference in LSB."""
    import numpy as np
    d = np.abs(gpu_color.astype(np.int16) - ref_color.astype(np.int16))
    out = {"color_pixels_differing": int(np.count_nonzero(d.max(axis=2))), "color_max_lsb": int(d.max()) if d.size else 0}
    if ref_depth is not None and gpu_depth is not None:
        out["depth_pixels_differing"] = int(np.count_nonzero(np.any(gpu_depth != ref_depth, axis=-1)))
    return out


def limiter(workload):
    """Compute-side utilisation of the workload's raster from the committed ncu capture, else None."""
    try:
        with open(os.path.join(ROOT, "profiles", "limiters.json")) as fh:
            return json.load(fh).get(workload)
    except Exception:
        return None


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and args.impl == "ours":
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(0)
        dist.init_process_group(backend)
    return world, rank, dist


def max_over_ranks(dist, value):
    if dist is None:
        return value
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_reference(args, world, rank, dist):
    """The reference arm: the reference's CPU draw path (the oracle, its
    line-cited restatement: the reference itself cannot be built here) on
    every host core, rendering the workload's own frame — its draws in API
    order into the frame's attachments — a chunk of draws per step of about
    --ref-seconds, continuing where the previous step stopped (a one-draw
    frame is rendered whole every step)."""
    import cpvulkan_gb300 as c
    c.build()
    if rank != 0:
        return
    from tests import oracle_binding
    oracle = oracle_binding.load()
    cfg, params, cfg_desc = workload(args)
    scene = c.Scene(cfg, 1, params)
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    color = depth = None
    cursor, chunk = 0, 8
    per_step = []
    for i in range(args.warmup + args.steps):
        t0 = time.time()
        tris = draws = 0
        while True:
            if scene.draws <= 1 or cursor >= scene.draws:
                cursor = 0
            end = scene.draws if scene.draws <= 1 else min(scene.draws, cursor + chunk)
            c0 = time.time()
            color, depth, st = oracle.render_threaded(scene, threads, cursor, end, color=color, depth=depth, clear=cursor == 0)
            dt_chunk = time.time() - c0
            tris += st["triangles"]
            draws += end - cursor
            cursor = end
            if scene.draws > 1 and dt_chunk < 0.5:
                chunk = min(chunk * 2, 512)
            if time.time() - t0 >= args.ref_seconds or scene.draws <= 1:
                break
        if i >= args.warmup:
            per_step.append((tris, time.time() - t0, draws))
    tris = sum(f for f, _, _ in per_step)
    dt = sum(t for _, t, _ in per_step)
    draws = sum(d for _, _, d in per_step)
    value = tris / dt / 1e6
    sample = ("whole frame (%d triangles) per step" % scene.triangles if scene.draws <= 1 else
              "the frame's draws in API order into its attachments, continuing across steps: %d draws (%d triangles) in %d timed steps "
              "of about %.0f s" % (draws, tris, len(per_step), args.ref_seconds))
    line = {
        "impl": "reference", "metric": "Mtri/s", "value": round(value, 3), "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * dt / len(per_step), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene)",
        "config": {"workload": args.config, "description": cfg_desc, "triangles": scene.triangles},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mtri/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


PLAIN_KERNELS = ("cpv_raster", "cpv_setup_rects", "cpv_bins_zero", "cpv_span_count", "cpv_scan", "cpv_span_write", "cpv_blend_tables")
BATCH_KERNELS = ("cpv_batch", "cpv_batch_vs", "cpv_batch_setup", "cpv_batch_bin", "cpv_batch_raster")

# Workloads measured beside the headline frame in the default run:
# (name, harness config, scene parameters, environment, description).
SIDE_WORKLOADS = [
    ("cube", 1, [30], {}, CONFIGS["cube"][2]),
    ("heightfield", 2, [], {}, CONFIGS["heightfield"][2]),
    ("blend", 3, [], {}, CONFIGS["blend"][2] + "; flat colour: per-primitive blend tables"),
    ("blend_general", 3, [], {"CPV_BLEND_TABLES": "0"}, CONFIGS["blend"][2] + "; blend computed per fragment (no tables)"),
    ("blend_interpolated", 3, [200000, 1920, 1080, 1], {}, CONFIGS["blend"][2] + "; a colour per corner, interpolated per fragment"),
    ("heightfield_spec_lod", 2, [], {"CPV_SPEC_LOD": "1"},
     CONFIGS["heightfield"][2] + "; labelled spec-LOD mode: implicit-LOD lambda from quad derivatives over the mip chain "
     "(not the reference's lambda 0); compared with the oracle in the same mode"),
]


def timed_frames(h, r, frames):
    """Device milliseconds of `frames` frames (queue events around each
    submission; a 256 MiB fill before each evicts the L2, untimed)."""
    import ctypes
    arr = (ctypes.c_double * frames)()
    res = h.cpvh_render_timed(r.ptr, frames, FLUSH_BYTES, arr)
    if res != 0:
        raise RuntimeError("render failed: %d" % res)
    return list(arr)


def kernel_profile(h, icd, r, names, frames):
    """Per-kernel device time of `frames` eager frames (CUDA events around each kernel)."""
    import ctypes
    icd.cpv_profile_reset()
    icd.cpv_profile_enable(1)
    timed_frames(h, r, frames)
    icd.cpv_profile_enable(0)
    out = {}
    for k in names:
        n, ms = ctypes.c_uint64(0), ctypes.c_double(0.0)
        icd.cpv_profile_get(k.encode(), ctypes.byref(n), ctypes.byref(ms))
        if n.value:
            out[k] = {"launches": n.value, "ms_per_launch": round(ms.value / n.value, 4), "ms_per_frame": round(ms.value / frames, 4)}
    return out


def batch_stats(icd):
    """Primitives, vertex-stage slots and (primitive, tile) pairs of the
    last completed batched frame (cpv_batch_stats)."""
    import ctypes
    out = (ctypes.c_uint64 * 3)()
    icd.cpv_batch_stats(out)
    return {"primitives": out[0], "vertex_slots": out[1], "pairs": out[2]}


def roofline_of(name, scene, kernels, frag_written):
    """HBM roofline of the frame's dominant raster kernel: algorithmic bytes
    per launch over its CUDA-event time, against the measured copy
    bandwidth; with the compute-side utilisation of the committed capture."""
    dom = "cpv_batch_raster" if "cpv_batch_raster" in kernels else "cpv_raster"
    peak, peak_kind = measured_peak()
    alg = algorithmic_bytes(name, scene, frag_written)
    achieved = alg / (kernels[dom]["ms_per_launch"] / 1000.0) / 1e9 if dom in kernels else None
    # committed captures cover the workloads' default modes only
    base = name if name.endswith("spec_lod") else name.split("_")[0]
    return {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2) if achieved else None, "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None, "traffic": committed_traffic(dom, base),
            "algorithmic_bytes_per_launch": alg, "compute_side": limiter(base) if base != "cube" else
            {"limiter": "launch and submission latency (one 12-triangle draw)"}}


def measure_workload(ctx, h, icd, name, cfg, params, env, desc, min_seconds=1.5):
    """One side workload at its full size: device-timed frames (at least
    `min_seconds` of them, clocks sampled meanwhile), per-kernel times, the
    roofline, and the image against the oracle's whole frame."""
    import math
    import cpvulkan_gb300 as c
    saved = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        scene = c.Scene(cfg, 1, params)
        scene.spec_lod = env.get("CPV_SPEC_LOD") == "1"
        r = c.Renderer(ctx, scene)
        try:
            timed_frames(h, r, 3)
            t0 = time.time()
            timed_frames(h, r, 5)
            probe = (time.time() - t0) * 1000.0 / 5  # wall ms per frame, L2 flush and submission included
            frames = int(min(50000, max(10, math.ceil(min_seconds * 1000.0 / probe))))
            clocks = ClockSampler(100)
            clocks.start()
            l0 = icd.cpv_kernel_launches()
            ms = timed_frames(h, r, frames)
            launches = icd.cpv_kernel_launches() - l0
            clock_info = clocks.stop()
            kernels = kernel_profile(h, icd, r, BATCH_KERNELS + PLAIN_KERNELS, 3)
            stats = batch_stats(icd) if "cpv_batch_raster" in kernels else None
            color, depth = r.readback()
        finally:
            r.close()
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    ref_color, ref_depth, st, ref_s, threads = reference_frame(scene)
    mpf = sum(ms) / frames
    tris = scene.triangles
    return {
        "description": desc, "triangles": tris, "draws": scene.draws, "frames": frames,
        "ms_per_frame": round(mpf, 5), "mtri_s": round(tris / (mpf / 1000.0) / 1e6, 3),
        "gfrag_s": round(st["fragments"] / (mpf / 1000.0) / 1e9, 4), "frames_s": round(1000.0 / mpf, 2),
        "fragments": st["fragments"], "fragments_written": st["fragments_written"],
        "mode": "batched" if "cpv_batch_raster" in kernels else "plain", "gpu_launches_per_frame": round(launches / frames, 2),
        "batch_stats": stats,
        "kernels": kernels, "roofline": roofline_of(name, scene, kernels, st["fragments_written"]), "clocks": clock_info,
        "parity": dict(image_diff(color, depth, ref_color, ref_depth), against="oracle whole frame"),
        "cpu_baseline": {"full_frame": {"seconds": round(ref_s, 3), "threads": threads, "kind": "port",
                                        "mtri_s": round(tris / ref_s / 1e6, 4)}},
        "env": env or None,
    }


def serve_sweep(ctx, seconds, seed=5, fractions=(0.25, 0.5, 0.8)):
    """The serving workload at its configured load (64 clients, mean 2 ms
    between one client's requests: above what one GPU serves, so it
    measures capacity) and then at fractions of the measured capacity."""
    import cpvulkan_gb300 as c
    server = c.Server(ctx, clients=64, slots=16, mean_interarrival_ms=2.0, duration_s=seconds, seed=seed)

    def point(label, ia, st):
        return {"offered": label, "mean_interarrival_ms_per_client": round(ia, 3),
                "offered_requests_s": round(64 * 1000.0 / ia, 1), "requests": st["requests"], "completed": st["completed"],
                "served_requests_s": round(st["completed"] / st["wall_s"], 1) if st["wall_s"] else None,
                "mtri_s": round(st["mtri_s"], 2), "max_in_flight": st["max_in_flight"],
                "latency_ms": {"p50": round(st["latency_p50_ms"], 3), "p99": round(st["latency_p99_ms"], 3), "from": "arrival"},
                "submit_to_fence_ms": {"p50": round(st["submit_p50_ms"], 3), "p99": round(st["submit_p99_ms"], 3)},
                "queue_wait_ms": {"p50": round(st["queue_p50_ms"], 3), "p99": round(st["queue_p99_ms"], 3)},
                "residencies": st["residencies"], "evictions": st["evictions"]}

    try:
        first = server.run()
        capacity = first["completed"] / first["wall_s"]
        out = {"resident_clients": first["resident_clients"], "resident_bytes": first["resident_bytes"],
               "capacity_requests_s": round(capacity, 1), "points": [point("configured", 2.0, first)]}
        for f in fractions:
            ia = 64 / (f * capacity) * 1000.0
            server.set_load(ia, seconds)
            out["points"].append(point("%.2f of capacity" % f, ia, server.run()))
        return out, first
    finally:
        server.close()


def run_ours(args, world, rank, dist):
    import numpy as np
    import cpvulkan_gb300 as c
    c.build()
    if not c.device_available():
        raise SystemExit("bench.py: no CUDA device — the GB300 path needs a GPU (no CPU fallback exists)")
    import ctypes
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_kernel_launches.restype = ctypes.c_uint64
    icd.cpv_profile_get.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double)]
    cfg, params, desc = workload(args)
    scene = c.Scene(cfg, 1, params)
    tris = scene.triangles
    # Many-draw scenes: the per-draw path (CPV_BATCH=0), then the ICD's
    # default, which batches the pass. One-draw scenes: the ICD's default
    # only (it batches a pass of 2^20+ primitives without blend tables).
    modes = ["plain", "default"] if scene.draws >= 16 and args.mode == "auto" else ["default"]
    if args.mode == "plain":
        modes = ["plain"]
    if args.mode == "batched":
        os.environ["CPV_BATCH_MIN_DRAWS"] = "1"  # a one-draw pass runs as a batch of one
        modes = ["default"]
    icd.cpv_kernel_launches.restype = ctypes.c_uint64
    ctx = c.Context()
    h = c.harness()
    h.cpvh_render_timed.restype = ctypes.c_int
    h.cpvh_render_timed.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)]

    def timed(frames):
        return timed_frames(h, r, frames)

    def profile(names, frames):
        return kernel_profile(h, icd, r, names, frames)

    results = {}
    r = None
    create_s = 0.0
    for mode in modes:
        # A fresh renderer per mode: the ICD decides batching when a command
        # buffer first runs and then replays that decision (its CUDA graph).
        if r is not None:
            r.close()
        os.environ["CPV_BATCH"] = "0" if mode == "plain" else "1"
        t0 = time.time()
        r = c.Renderer(ctx, scene)
        create_s = time.time() - t0
        timed(args.warmup)
        barrier(dist)
        clocks = ClockSampler()
        clocks.start()
        launches0 = icd.cpv_kernel_launches()
        frame_ms = timed(args.steps)
        launches = icd.cpv_kernel_launches() - launches0
        clock_info = clocks.stop()
        barrier(dist)
        total_ms = max_over_ranks(dist, sum(frame_ms))
        kernels = profile(PLAIN_KERNELS if mode == "plain" else BATCH_KERNELS + PLAIN_KERNELS, min(args.steps, 5))
        if mode == "default":
            mode = "batched" if "cpv_batch_raster" in kernels else "plain"  # what the ICD ran
        results[mode] = {"total_ms": total_ms, "launches": int(launches), "clocks": clock_info, "kernels": kernels,
                         "stats": batch_stats(icd)}
        head = mode
    total_ms = results[head]["total_ms"]
    ms_per_step = total_ms / args.steps
    value = tris * args.steps * world / (total_ms / 1000.0) / 1e6
    # Submit-to-fence latency of fenced frames, one at a time.
    _, lat = r.render(args.steps, latencies=True)
    # End to end through the API with host buffers.
    r.render_e2e(2)
    e2e_ms, h2d, d2h = r.render_e2e(args.steps)
    e2e_ms = max_over_ranks(dist, e2e_ms)
    e2e = tris * args.steps * world / (e2e_ms / 1000.0) / 1e6
    color, depth = r.readback()
    r.close()
    line = None
    if rank == 0:
        # the CPU-baseline leg: the oracle's whole frame on every host core
        # (its fragment counts and the image this frame is compared with),
        # then a single-thread sample for the baseline rate
        ref_color, ref_depth, st, ref_s, ref_threads = reference_frame(scene)
        tris_cpu, dt_cpu, cpu_desc = cpu_baseline(scene, args.cpu_seconds, 1)
        cpu_value = tris_cpu / dt_cpu / 1e6
        kernels = results[head]["kernels"]
        frags = st.get("fragments")
        line = {
            "metric": "Mtri/s", "value": round(value, 3), "unit": "Mtri/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator, same bytes as the CPU oracle)",
            "config": {"workload": args.config, "description": desc, "triangles": tris, "draws": scene.draws, "mode": head,
                       "l2": "256 MiB fill between frames (untimed)", "pipeline_create_s": round(create_s, 3)},
            "gfrag_s": round(frags * args.steps * world / (total_ms / 1000.0) / 1e9, 4) if frags else None,
            "frames_s": round(1000.0 * world / ms_per_step, 3),
            "submit_to_fence_ms": {"p50": round(float(np.percentile(lat, 50)), 4), "p99": round(float(np.percentile(lat, 99)), 4)},
            "e2e": {"value": round(e2e, 3), "unit": "Mtri/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": round(e2e_ms / args.steps, 3)},
            "gpu_launches": results[head]["launches"],
            "kernels": kernels,
            "roofline": roofline_of(args.config, scene, kernels, st.get("fragments_written")),
            "cpu_baseline": {"value": round(cpu_value, 4), "unit": "Mtri/s", "cores": 1, "kind": "port", "sample": cpu_desc,
                             "full_frame": {"seconds": round(ref_s, 3), "threads": ref_threads, "kind": "port",
                                            "mtri_s": round(tris / ref_s / 1e6, 4)}},
            "parity": dict(image_diff(color, depth, ref_color, ref_depth), against="oracle whole frame"),
            "clocks": results[head]["clocks"],
        }
        if head == "batched":
            line["config"]["tuning"] = c.batch_tuning() or "default configuration (pass below the tuning threshold)"
            line["batch_stats"] = results[head].get("stats")
        if "plain" in results and head != "plain":
            pm = results["plain"]["total_ms"] / args.steps
            line["plain"] = {"value": round(tris * world / (pm / 1000.0) / 1e6, 3), "unit": "Mtri/s", "ms_per_step": round(pm, 4),
                             "frames_s": round(1000.0 * world / pm, 3), "gpu_launches": results["plain"]["launches"],
                             "kernels": results["plain"]["kernels"], "clocks": results["plain"]["clocks"]}
            line["batched_over_plain_frames"] = round(pm / ms_per_step, 3)
        if args.configs:
            # the other workloads at full size, and the serving sweep
            configs = {}
            for name, cfg_i, params_i, env_i, desc_i in SIDE_WORKLOADS:
                configs[name] = measure_workload(ctx, h, icd, name, cfg_i, params_i, env_i, desc_i)
            sweep, _ = serve_sweep(ctx, args.side_serve_seconds)
            configs["serve"] = dict(sweep, description=CONFIGS["serve"][2], arrival_window_s=args.side_serve_seconds)
            line["configs"] = configs
        print(json.dumps(line), flush=True)
    ctx.close()
    return line


def run_serve(args, world, rank, dist):
    """Serving: the arrivals of args.serve_seconds per client, admitted into
    16 queues as slots free up, through vkQueueSubmit and fences; first at
    the configured load (above capacity), then at fractions of the measured
    capacity."""
    import cpvulkan_gb300 as c
    c.build()
    if not c.device_available():
        raise SystemExit("bench.py: no CUDA device — the GB300 path needs a GPU (no CPU fallback exists)")
    import ctypes
    icd = ctypes.CDLL(c.ICD_PATH)
    icd.cpv_kernel_launches.restype = ctypes.c_uint64
    ctx = c.Context()
    barrier(dist)
    clocks = ClockSampler()
    clocks.start()
    launches0 = icd.cpv_kernel_launches()
    t0 = time.time()
    sweep, st = serve_sweep(ctx, args.serve_seconds, seed=5 + rank)
    sweep_s = time.time() - t0
    launches = icd.cpv_kernel_launches() - launches0
    clock_info = clocks.stop()
    barrier(dist)
    wall_ms = max_over_ranks(dist, st["wall_s"] * 1000.0)
    tris = st["triangles"] * world  # replicas: every rank serves its own clients
    value = tris / (wall_ms / 1000.0) / 1e6
    line = None
    if rank == 0:
        scene = c.Scene(6, 5, [512, 20000, 0])
        tris_cpu, dt_cpu, cpu_desc = cpu_baseline(scene, args.cpu_seconds, 1)
        line = {
            "metric": "Mtri/s", "value": round(value, 3), "unit": "Mtri/s", "n_gpus": world, "steps": int(st["completed"]),
            "warmup": 16, "ms_per_step": round(wall_ms / max(1, st["completed"]), 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded client scenes and arrivals)",
            "config": {"workload": "serve", "description": CONFIGS["serve"][2], "clients": 64, "queues": 16,
                       "arrival_window_s": args.serve_seconds, "resident_clients": st["resident_clients"],
                       "resident_bytes": st["resident_bytes"], "value_at": "the configured load (above capacity)"},
            "requests": st["requests"], "completed": st["completed"], "max_in_flight": st["max_in_flight"],
            "latency_ms": {"p50": round(st["latency_p50_ms"], 3), "p99": round(st["latency_p99_ms"], 3), "from": "arrival"},
            "submit_to_fence_ms": {"p50": round(st["submit_p50_ms"], 3), "p99": round(st["submit_p99_ms"], 3)},
            "queue_wait_ms": {"p50": round(st["queue_p50_ms"], 3), "p99": round(st["queue_p99_ms"], 3)},
            "sweep": sweep,
            "e2e": {"value": round(value, 3), "unit": "Mtri/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0,
                    "note": "clients' data are resident by design; requests go through vkQueueSubmit and fences, wall-clock timed"},
            "gpu_launches": int(launches), "sweep_wall_s": round(sweep_s, 2),
            "roofline": {"bound": "hbm", "kernel": "cpv_raster", "achieved": None, "peak": measured_peak()[0], "unit": "GB/s",
                         "frac": None, "traffic": None, "note": "many small launches; see the per-draw workloads"},
            "cpu_baseline": {"value": round(tris_cpu / dt_cpu / 1e6, 4), "unit": "Mtri/s", "cores": 1, "kind": "port", "sample": cpu_desc},
            "clocks": clock_info,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="batch")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window of the serving workload")
    ap.add_argument("--params", default="", help="comma-separated scene parameters replacing the workload's (profiling cases)")
    ap.add_argument("--mode", choices=["auto", "plain", "batched"], default="auto",
                    help="auto: per-draw and batched where batching applies (render passes of 16+ draws)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="oracle time for the cpu_baseline figure")
    ap.add_argument("--ref-seconds", type=float, default=3.0, help="oracle time per step of --impl reference")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the other workloads the default run measures beside the headline frame")
    ap.add_argument("--side-serve-seconds", type=float, default=2.0, help="arrival window of each serving point in the default run")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.config != "batch" or args.params or args.mode != "auto":
        args.configs = False  # side workloads only beside the default headline frame
    world, rank, dist = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
    elif args.config == "serve":
        run_serve(args, world, rank, dist)
    else:
        run_ours(args, world, rank, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
