"""Benchmark of the voxel ray tracer on GB300: Mrays/s of the 1080p / 16-light frame.

One step = one frame of the full scene: world 512x256x512 (seeded terrain, resident in
HBM), 1920x1080, 16 local lights + the global light, 1024 DDA steps per ray; rays =
primary rays + shadow rays actually cast (counted on the device, equal to the oracle's
count).  L2 is flushed (a 256 MiB write) before every timed frame; each frame is timed
with CUDA events on the launching stream.

  value      Mrays/s of vrt_render (device buffers), whole job over N GPUs (replicas)
  e2e        the same through vrt_render_to_host: uniforms in, RGBA8 image out to
             pinned host memory every step (the kernel stores the pixels into it over the
             host link), wall clock
  roofline   instruction issue, the render kernel's bound: warp instructions per frame
             (ncu, profiles/counters.json, captured on the same kernel sources) / frame
             time, against 4 issue slots per SM per cycle at the sampled SM clock; beside
             it the effective bandwidth (B = 4*steps + 4*primary hits + 4*pixels: one
             4-byte voxel word per DDA step of the reference shader) and the physical
             DRAM / L2 traffic ncu measured, against the measured HBM copy bandwidth
  batched    64 cameras of uneven size in one CUDA-graph-captured persistent launch vs
             one launch per camera
  served     Poisson stream over 4 resident worlds: p50/p99 latency and Mrays/s per rate
  cpu_baseline  the CPU oracle (scalar C++ restatement of the shader, OpenMP over rows)
             on a bounded row sample of the same frame

--impl reference times the CPU restatement of the reference shader (the reference
itself is a GLSL fragment shader; it cannot run here) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "voxel-rt_gb300"))

METRIC = "Mrays/s @1080p 16 lights; served p50/p99 ms vs plain per-frame launch"
UNIT = "Mrays/s"


def rank_info():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        import statistics
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def cpu_baseline(scene, target_s: float, threads: int):
    """Oracle (-O3, no contraction, OpenMP over rows) on the same frame: whole frames
    repeated until about target_s of CPU time, or an even row sample when one frame
    alone would take longer."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import vrt_oracle
    vrt_oracle.build()
    u = scene.uniforms
    t0 = time.perf_counter()
    probe = vrt_oracle.render(scene.words, scene.W, scene.H, u, scene.width, scene.height,
                              rows=(0, scene.height, 30), threads=threads, fast=True, outputs=False)
    est_frame = max(time.perf_counter() - t0, 1e-4) * 30.0
    stride = 1 if est_frame <= target_s else max(1, int(round(est_frame / target_s)))
    reps = max(1, min(50, int(target_s / est_frame))) if stride == 1 else 1
    rays, dt = 0, 0.0
    for _ in range(reps):
        t0 = time.perf_counter()
        res = vrt_oracle.render(scene.words, scene.W, scene.H, u, scene.width, scene.height,
                                rows=(0, scene.height, stride), threads=threads, fast=True, outputs=False)
        dt += time.perf_counter() - t0
        rays += res["totals"]["rays"]
    nrows = len(range(0, scene.height, stride))
    what = (f"{reps} whole {scene.width}x{scene.height} frames" if stride == 1 else
            f"every {stride}th row of the {scene.width}x{scene.height} frame ({nrows} rows)")
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port", "cpu": cpu_model(),
            "sample": f"{what}: {rays} rays in {dt:.2f} s", "seconds": dt / reps}


def workload_config(sc, world_size: int) -> dict:
    """The config object of both arms: what the workload is, nothing about who ran it."""
    return {"workload": sc.workload, "world": f"{sc.W}x{sc.H}x{sc.W}", "image": f"{sc.width}x{sc.height}",
            "max_steps": int(sc.uniforms.maxSteps),
            "local_lights": sum(1 for i in range(16) if sc.uniforms.localLights[i][0] >= 0),
            "seed": getattr(sc, "seed", None), "l2": "GPU arm: flushed before every timed frame (256 MiB write)",
            "parallelism": f"replicas x{world_size}"}


def run_reference(args):
    rank, world_size, _ = rank_info()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import vrt_oracle
    import vrt
    # the scene's host-only helpers from the oracle library's build: libvrt.so (the CUDA
    # library) is never loaded by this arm
    vrt.use_host_library(vrt_oracle.library_path(fast=True))
    import scenes
    threads = os.cpu_count() or 1
    sc = scenes.full(2, threads=threads)
    steps = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(sc, args.cpu_seconds / 2.0, threads)
        if i >= args.warmup:
            steps.append(r)
    val = sum(s["value"] for s in steps) / len(steps)
    ms = sum(s["seconds"] for s in steps) / len(steps) * 1000.0
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded terrain)",
        "config": workload_config(sc, world_size),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port", "cpu": steps[-1]["cpu"],
                         "sample": steps[-1]["sample"]},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference path is a GLSL fragment shader (no graphics stack here); its CPU restatement "
                "(the oracle, bit-exact with the shader source compiled via GLM) is timed on all host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


# the ray tile each render kernel takes when the options name none
DEFAULT_TILES = {"render_tiles_kernel": "8x16", "render_word_kernel": "16x8", "render_mask_kernel": "8x4"}

COUNTER_SOURCES = [os.path.join("voxel-rt_gb300", "csrc", n) for n in ("render.cu", "shade_common.cuh")]


def kernel_source_hash() -> str:
    """sha256 (16 hex digits) of the render kernels' code, to match ncu counters to a build.
    Comments, whitespace at line ends and blank lines are left out (the sources have no
    comment markers inside string literals), so a change of a comment keeps the counters;
    any change of code drops them."""
    import hashlib
    import re
    h = hashlib.sha256()
    for rel in COUNTER_SOURCES:
        with open(os.path.join(ROOT, rel), encoding="utf-8") as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        lines = (re.sub(r"//.*", "", line).rstrip() for line in text.splitlines())
        h.update("\n".join(line for line in lines if line).encode())
    return h.hexdigest()[:16]


def load_counters(kernel: str, workload: str):
    """ncu counters of one launch of kernel on workload (profiles/counters.json): warp
    instructions, DRAM and L2 bytes.  Returns (entry or None, fresh), fresh when they were
    captured on the current kernel sources."""
    p = os.path.join(ROOT, "profiles", "counters.json")
    if not os.path.exists(p):
        return None, False
    with open(p) as f:
        d = json.load(f)
    e = d.get(f"{kernel}:{workload}")
    return e, bool(e) and e.get("source_sha16") == kernel_source_hash()


def roofline_of(kname, workload, ms, clk, hbm_peak, peak_src, algo_bytes, sms):
    """The render kernels are bound by instruction issue (integer/logic pipe), not by memory:
    achieved = warp instructions per launch (ncu, profiles/counters.json) / the launch's
    CUDA-event time; peak = 4 warp schedulers x one issue per cycle x SMs x the median SM
    clock sampled during the timed frames.  Beside it: the effective bandwidth (the bytes
    the reference shader would read: 4 B per DDA iteration + hit colour + pixel) and the
    physical DRAM and L2 traffic ncu measured, against the measured HBM copy peak."""
    t = ms * 1e-3
    cnt, fresh = load_counters(kname, workload)
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0
    r = {"bound": "issue", "kernel": kname, "unit": "G warp-instructions/s", "achieved": None,
         "peak": sms * 4 * mhz * 1e6 / 1e9, "frac": None, "traffic": None,
         "sms": sms, "sm_mhz": mhz, "peak_source": "4 issue slots per SM per cycle at the sampled SM clock",
         "effective_bytes_per_launch": algo_bytes, "effective_gbs": algo_bytes / t / 1e9}
    if cnt:
        r["counters"] = {"source": cnt.get("source"), "fresh": fresh, "captured_on": cnt.get("source_sha16")}
    if cnt and fresh:
        inst = cnt["warp_inst_per_launch"]
        dram = cnt["dram_bytes_per_launch"]
        r.update(achieved=inst / t / 1e9, traffic=dram, warp_inst_per_launch=inst)
        r["frac"] = r["achieved"] / r["peak"]
        r["physical"] = {"dram_bytes_per_launch": dram, "l2_bytes_per_launch": cnt.get("l2_bytes_per_launch"),
                         "dram_gbs": dram / t / 1e9, "hbm_peak_gbs": hbm_peak, "hbm_peak_source": peak_src,
                         "dram_frac_of_hbm": dram / t / 1e9 / hbm_peak}
        if cnt.get("l2_bytes_per_launch"):
            r["physical"]["l2_gbs"] = cnt["l2_bytes_per_launch"] / t / 1e9
    else:
        r["note"] = "no ncu counters captured on these kernel sources: frac not computed"
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-extras", action="store_true", help="skip the batched / served / CPU legs")
    ap.add_argument("--kernel", default="pixel", choices=["pixel", "mask", "word", "auto"])
    ap.add_argument("--workload", default="full", choices=["full", "reference"],
                    help="full: the 1080p/16-light frame; reference: the reference's own world (initVoxels + "
                         "fixDepthField on the device) at 800x600, 384 steps, rendered by the kernel AUTO picks")
    ap.add_argument("--tile", default="default",
                    help="ray tile WxH, or default: the kernel's own (8x16 tile kernel, 16x8 word kernel)")
    ap.add_argument("--refill", type=int, default=8)
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import build as vbuild
    import replicas
    import scenes
    import vrt

    rank, world_size, local_rank = rank_info()
    torch.cuda.set_device(local_rank)
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if rank == 0 or world_size == 1:
        vbuild.build()
    if dist:
        dist.barrier()
    vrt.lib()
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    threads = max(1, (os.cpu_count() or 1) // max(1, world_size))
    if args.workload == "reference":
        sc = reference_scene(vrt, scenes, np)
        world = sc.world
        args.no_extras = True  # the batched / served / stress legs use the full workload's world
        if args.kernel == "pixel":
            args.kernel = "auto"
    else:
        sc = scenes.full(2, threads=threads)
        sc.data = "synthetic (seeded terrain, seed 2)"
        world = vrt.World(sc.W, sc.H)
        world.upload(sc.words)
    r = vrt.Renderer()
    opts = vrt.RenderOpts()
    opts.kernel = {"pixel": vrt.KERNEL_MASK_PIXEL, "mask": vrt.KERNEL_BITMASK, "word": vrt.KERNEL_WORD,
                   "auto": vrt.KERNEL_AUTO}[args.kernel]
    if args.tile != "default":
        opts.tile_w, opts.tile_h = (int(v) for v in args.tile.split("x"))
    opts.refill_min = args.refill
    opts.blocks_per_sm = args.blocks_per_sm
    W, H = sc.width, sc.height
    img = torch.empty(W * H * 4, dtype=torch.uint8, device=dev)
    stats = torch.zeros(vrt.STAT_COUNT, dtype=torch.int64, device=dev)
    # counting frames: exact shader step accounting (the reference's DDA iterations, S), and
    # the iterations the timed path performs (rays that cannot hit end early)
    exact_opts = vrt.RenderOpts.from_buffer_copy(opts)
    exact_opts.exact_steps = 1
    r.render(world, sc.uniforms, W, H, img.data_ptr(), None, stats.data_ptr(), exact_opts, sh)
    torch.cuda.synchronize()
    st = stats.cpu().numpy()
    rays, steps, hits, pixels = (int(st[i]) for i in range(4))
    stats.zero_()
    r.render(world, sc.uniforms, W, H, img.data_ptr(), None, stats.data_ptr(), opts, sh)
    torch.cuda.synchronize()
    st_fast = stats.cpu().numpy()
    assert int(st_fast[0]) == rays and int(st_fast[2]) == hits, "ray counts differ between counting frames"
    steps_performed = int(st_fast[1])
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    for _ in range(args.warmup):
        r.render(world, sc.uniforms, W, H, img.data_ptr(), None, 0, opts, sh)
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in evs:
        flush.zero_()  # evict L2 (256 MiB > 129 MB) outside the timed span
        a.record(stream)
        r.render(world, sc.uniforms, W, H, img.data_ptr(), None, 0, opts, sh)
        b.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    times = [a.elapsed_time(b) for a, b in evs]
    ms = replicas.max_over_ranks(sum(times) / len(times), dist, dev)  # replicas: each rank renders a frame
    value = replicas.whole_job_rate(rays, ms * 1e-3, world_size) / 1e6

    # end to end through the public API: uniforms in, image out to pinned host memory
    host = torch.empty(W * H * 4, dtype=torch.uint8, pin_memory=True)
    for _ in range(2):
        r.render_to_host(world, sc.uniforms, W, H, host.data_ptr(), opts, sh)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.render_to_host(world, sc.uniforms, W, H, host.data_ptr(), opts, sh)
    e2e_s = replicas.max_over_ranks((time.perf_counter() - t0) / args.steps, dist, dev)
    e2e = {"value": replicas.whole_job_rate(rays, e2e_s, world_size) / 1e6, "unit": UNIT, "ms_per_step": e2e_s * 1e3,
           "h2d_bytes_per_step": int(C_sizeof_uniforms()), "d2h_bytes_per_step": W * H * 4,
           "path": "vrt_render_to_host into page-locked host memory: the kernel's pixel stores cross the host "
                   "link as it renders (no staging copy); uniforms go in as kernel parameters"}

    hbm_peak, peak_src = measured_peaks()
    algo_bytes = 4 * steps + 4 * hits + 4 * pixels
    kauto = "word" if world.info().has_depth_field else "pixel"
    kname = {"pixel": "render_tiles_kernel", "mask": "render_mask_kernel", "word": "render_word_kernel"}[
        kauto if args.kernel == "auto" else args.kernel]
    roofline = roofline_of(kname, args.workload, ms, clk, hbm_peak, peak_src, algo_bytes,
                           torch.cuda.get_device_properties(dev).multi_processor_count)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": sc.data,
        "config": workload_config(sc, world_size),
        "frame": {"rays": rays, "dda_steps": steps, "dda_steps_performed": steps_performed,
                  "box_lookups": int(st_fast[4]), "primary_hits": hits, "pixels": pixels, "kernel": kname,
                  "tile": args.tile if args.tile != "default" else DEFAULT_TILES[kname], "refill_min": args.refill},
        "clocks": clk, "gpu_launches": args.steps, "roofline": roofline, "e2e": e2e,
        "frame_ms_min": min(times), "frame_ms_max": max(times),
    }
    if rank == 0 and world_size == 1 and not args.no_extras:
        line["batched"] = bench_batched(vrt, torch, scenes, sc, world, r, dev, stream)
        line["served"] = bench_served(vrt, torch, scenes, sc, world)
        line["served"]["plain_frame_ms"] = ms
        line["stress"] = bench_stress(vrt, torch, scenes, dev, stream)
    if rank == 0 and world_size == 1 and (not args.no_extras or args.workload == "reference"):
        line["cpu_baseline"] = cpu_baseline(sc, args.cpu_seconds, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def reference_scene(vrt, scenes, np):
    """The reference app's first frame: its own world (initVoxels + fixDepthField, built
    on the device), camera (195, 55, 155), the rotated sun, 800x600, RENDER_DIST 384."""
    class Scene:
        pass
    sc = Scene()
    sc.W, sc.H, sc.width, sc.height = 512, 96, 800, 600
    sc.world = vrt.World(sc.W, sc.H)
    sc.world.init_reference()
    sc.world.fix_depth_field()
    sc.words = sc.world.download(np.empty(sc.W * sc.H * sc.W, np.int32))
    sc.uniforms = scenes.reference_scene_uniforms()
    sc.uniforms.aspectRatio = sc.width / sc.height
    sc.workload = "reference: initVoxels + fixDepthField 512x96x512, 800x600, 384 steps, no local lights"
    sc.data = "the reference's own world (initVoxels + fixDepthField, built on the device)"
    return sc


def C_sizeof_uniforms():
    import ctypes
    import vrt
    return ctypes.sizeof(vrt.Uniforms)


def bench_batched(vrt, torch, scenes, sc, world, r, dev, stream):
    """64 cameras: one CUDA-graph-captured launch with autotuned ray tiles per resolution
    class, against one vrt_render launch per camera."""
    import ctypes as C
    import autotune
    views = scenes.batch_views(sc, 64, seed=3)
    imgs = [torch.empty(w * h * 4, dtype=torch.uint8, device=dev) for (_, w, h) in views]
    ptrs = [im.data_ptr() for im in imgs]
    stats = torch.zeros((len(views), vrt.STAT_COUNT), dtype=torch.int64, device=dev)
    sh = stream.cuda_stream
    plan = autotune.tune(torch, r, world, views, ptrs, reps=3)
    vv = plan.views(world, views, ptrs, [stats[i].data_ptr() for i in range(len(views))])
    r.render_batch(vv, plan.opts(), sh)
    torch.cuda.synchronize()
    rays = int(stats[:, vrt.STAT_RAYS].sum().item())
    arr = (vrt.View * len(views))(*plan.views(world, views, ptrs))
    g = C.c_void_p()
    opts = plan.opts()
    vrt.check(vrt.lib().vrt_batch_graph_create(r.handle, arr, len(views), C.byref(opts), sh, C.byref(g)))
    for _ in range(2):
        vrt.check(vrt.lib().vrt_batch_graph_launch(g, sh))
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5
    a.record(stream)
    for _ in range(reps):
        vrt.check(vrt.lib().vrt_batch_graph_launch(g, sh))
    b.record(stream)
    torch.cuda.synchronize()
    batched_ms = a.elapsed_time(b) / reps
    vrt.lib().vrt_batch_graph_destroy(g)
    # plain: one vrt_render launch per camera, default options
    for (u, w, h), p in zip(views, ptrs):
        r.render(world, u, w, h, p, None, 0, None, sh)
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        for (u, w, h), p in zip(views, ptrs):
            r.render(world, u, w, h, p, None, 0, None, sh)
    b.record(stream)
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b) / reps
    # plain and synchronous: each camera rendered and copied to host before the next
    host = torch.empty(max(w * h for _, w, h in views) * 4, dtype=torch.uint8, pin_memory=True)
    for (u, w, h) in views[:4]:
        r.render_to_host(world, u, w, h, host.data_ptr(), None, sh)
    t0 = time.perf_counter()
    for (u, w, h) in views:
        r.render_to_host(world, u, w, h, host.data_ptr(), None, sh)
    sync_ms = (time.perf_counter() - t0) * 1e3
    top = sorted(plan.table, key=lambda e: e["ms"])[:4]
    return {"cameras": len(views), "pixels": sum(w * h for _, w, h in views), "rays": rays,
            "batched_ms": batched_ms, "batched_mrays_per_s": rays / (batched_ms * 1e-3) / 1e6,
            "plain_ms": plain_ms, "plain_mrays_per_s": rays / (plain_ms * 1e-3) / 1e6,
            "speedup": plain_ms / batched_ms,
            "plain_sync_ms": sync_ms, "plain_sync_mrays_per_s": rays / (sync_ms * 1e-3) / 1e6,
            "speedup_vs_sync": sync_ms / batched_ms,
            "note": "plain = one vrt_render launch per camera, back to back on one stream; plain_sync = "
                    "vrt_render_to_host per camera (render into page-locked host memory, wait) -- the "
                    "batched result stays in device memory",
            "autotuned": plan.describe(), "autotune_best": top}


def bench_stress(vrt, torch, scenes, dev, stream):
    """2048x256x2048 world (4 GiB of words), 3840x2160, 16 local lights + global light,
    4096 steps, camera 1 voxel above the terrain at pitch -2 deg (grazing rays)."""
    st = scenes.stress(5, threads=os.cpu_count() or 1)
    world = vrt.World(st.W, st.H)
    world.upload(st.words)
    st.words = None
    r = vrt.Renderer()
    W, H = st.width, st.height
    img = torch.empty(W * H * 4, dtype=torch.uint8, device=dev)
    stats = torch.zeros(vrt.STAT_COUNT, dtype=torch.int64, device=dev)
    sh = stream.cuda_stream
    exact = vrt.RenderOpts()
    exact.exact_steps = 1
    r.render(world, st.uniforms, W, H, img.data_ptr(), None, stats.data_ptr(), exact, sh)
    torch.cuda.synchronize()
    s_exact = stats.cpu().tolist()
    stats.zero_()
    r.render(world, st.uniforms, W, H, img.data_ptr(), None, stats.data_ptr(), None, sh)
    torch.cuda.synchronize()
    s_fast = stats.cpu().tolist()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    times = []
    for i in range(5):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r.render(world, st.uniforms, W, H, img.data_ptr(), None, 0, None, sh)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ms = sorted(times)[2]
    rays = int(s_exact[0])
    res = {"workload": st.workload, "ms": ms, "mrays_per_s": rays / (ms * 1e-3) / 1e6, "rays": rays,
           "dda_steps": int(s_exact[1]), "dda_steps_performed": int(s_fast[1]), "box_lookups": int(s_fast[4]),
           "effective_gbs": (4 * s_exact[1] + 4 * s_exact[2] + 4 * s_exact[3]) / (ms * 1e-3) / 1e9}
    world.close()
    return res


SERVED_BATCH_PIXELS = 1920 * 1080


def bench_served(vrt, torch, scenes, sc, full_world):
    """4 resident worlds (256^3, 512x256x512, 1024x256x1024 x2), Poisson arrivals."""
    import serving
    threads = os.cpu_count() or 1
    specs = []
    worlds = [scenes.full(21, W=256, H=256, threads=threads), sc,
              scenes.full(22, W=1024, H=256, threads=threads), scenes.full(23, W=1024, H=256, threads=threads)]
    for i, s in enumerate(worlds):
        w = full_world if s is sc else vrt.World(s.W, s.H)
        if s is not sc:
            w.upload(s.words)
            s.words = None
        specs.append(serving.WorldSpec(s, w))
    # a launch takes up to 8 requests and at most one 1080p frame of pixels, so that a request
    # arriving under load waits behind at most about one frame of work per slot
    srv = serving.Server(40 << 30, slots=4, max_batch=8, max_batch_pixels=SERVED_BATCH_PIXELS)
    wids = [srv.add_world(s.world) for s in specs]
    results = []
    for rate in (250.0, 1000.0, 4000.0, 8000.0, 16000.0):
        reqs = serving.make_requests(specs, rate, 1.0, seed=int(rate))
        done, wall = serving.run_open_loop(srv, wids, reqs)
        res = serving.summarize(done, wall)
        res["rate_hz"] = rate
        results.append(res)
    srv.close()
    # plain one-request-at-a-time serving of a request stream like the 4000 req/s one: each
    # render launched, copied to host and waited for; each edit applied and waited for
    reqs = serving.make_requests(specs, 4000.0, 0.25, seed=7)
    r = vrt.Renderer()
    host = torch.empty(1920 * 1080 * 4, dtype=torch.uint8, pin_memory=True)
    stream = torch.cuda.current_stream().cuda_stream
    counts = torch.zeros(vrt.STAT_COUNT, dtype=torch.int64, device="cuda")
    t0 = time.perf_counter()
    n_render = 0
    for (_, kind, wi, payload) in reqs:
        if kind == vrt.REQ_RENDER:
            u, w, h = payload
            r.render_to_host(specs[wi].world, u, w, h, host.data_ptr(), None, stream)
            n_render += 1
        else:
            specs[wi].world.remove_sphere(*payload, specs[wi].world.info().has_depth_field, stream)
            torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    # the same renders once more with counters, to count their rays
    for (_, kind, wi, payload) in reqs:
        if kind == vrt.REQ_RENDER:
            u, w, h = payload
            img = torch.empty(w * h * 4, dtype=torch.uint8, device="cuda")
            r.render(specs[wi].world, u, w, h, img.data_ptr(), None, counts.data_ptr(), None, stream)
    torch.cuda.synchronize()
    plain_rays = int(counts[vrt.STAT_RAYS].item())
    r.close()
    full_world.upload(sc.words)  # the served edits changed the shared world: restore it
    sat = max(x["mrays_per_s"] for x in results if "mrays_per_s" in x)
    return {"worlds": ["256x256x256", "512x256x512", "1024x256x1024", "1024x256x1024"], "budget_gib": 40,
            "slots": 4, "max_batch": 8, "max_batch_pixels": SERVED_BATCH_PIXELS,
            "images": "page-locked host memory, stored by the render kernel",
            "sweep": results,
            "plain_sync": {"renders": n_render, "seconds": plain_s, "mrays_per_s": plain_rays / plain_s / 1e6,
                           "ms_per_render": plain_s * 1e3 / max(n_render, 1)},
            "served_vs_plain_sync": sat / (plain_rays / plain_s / 1e6)}


if __name__ == "__main__":
    sys.exit(main())
