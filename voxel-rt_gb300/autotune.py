"""Autotuner for batched rendering: picks the ray-tile shape per resolution class.

A batch (vrt_render_batch) renders cameras of uneven size in one launch of the tile
kernel; every view may use its own tile shape as long as all shapes have the launch's
thread count.  The tuner times, on the caller's own views, each candidate shape for
each resolution class (small < 0.25 MP, medium < 1 MP, large >= 1 MP) with the other
classes fixed, and keeps the fastest; it also compares the persistent kernel with its
lane-refill interval, and reports the whole table so a caller can see what was chosen.

Timings are CUDA events on the launching stream around one batched launch, median of
`reps` after one warm-up.
"""
from __future__ import annotations

import statistics

import vrt

CLASSES = ("small", "medium", "large")
# shapes by thread count of the tile kernel (tile_w * tile_h threads per CTA)
SHAPES = {64: [(8, 8), (16, 4), (32, 2), (4, 16)], 128: [(8, 16), (16, 8), (32, 4), (64, 2)]}
PERSISTENT = [((8, 4), 4), ((8, 4), 8), ((16, 8), 8), ((32, 1), 8), ((8, 8), 16)]


def resolution_class(width: int, height: int) -> str:
    mp = width * height / 1e6
    return "small" if mp < 0.25 else ("medium" if mp < 1.0 else "large")


class Plan:
    """The tuner's choice: a kernel, the launch's tile, and a tile shape per class."""

    def __init__(self, kernel: int, launch_tile, class_tiles: dict, refill: int = 0, table=None):
        self.kernel = kernel
        self.launch_tile = launch_tile
        self.class_tiles = class_tiles
        self.refill = refill
        self.table = table or []

    def opts(self) -> vrt.RenderOpts:
        o = vrt.RenderOpts()
        o.kernel = self.kernel
        o.tile_w, o.tile_h = self.launch_tile
        o.refill_min = self.refill
        return o

    def views(self, world, cams, images, stats=None):
        out = []
        for i, ((u, w, h), img) in enumerate(zip(cams, images)):
            tile = self.class_tiles.get(resolution_class(w, h)) if self.kernel == vrt.KERNEL_MASK_PIXEL else None
            out.append(vrt.make_view(world, u, w, h, img, stats[i] if stats else 0, tile))
        return out

    def describe(self) -> dict:
        name = "tile" if self.kernel == vrt.KERNEL_MASK_PIXEL else "persistent"
        d = {"kernel": name, "launch_tile": "x".join(map(str, self.launch_tile))}
        if self.kernel == vrt.KERNEL_MASK_PIXEL:
            d["tiles_per_class"] = {k: "x".join(map(str, v)) for k, v in self.class_tiles.items()}
        else:
            d["refill_min"] = self.refill
        return d


def _time(torch, renderer, world, cams, images, plan: Plan, stream, reps: int) -> float:
    views = plan.views(world, cams, images)
    opts = plan.opts()
    renderer.render_batch(views, opts, stream.cuda_stream)
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        renderer.render_batch(views, opts, stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def tune(torch, renderer, world, cams, images, reps: int = 3) -> Plan:
    """cams: [(uniforms, width, height)], images: device pointers, one per camera."""
    stream = torch.cuda.current_stream()
    table = []
    best = None
    for threads, shapes in SHAPES.items():
        choice = {c: shapes[0] for c in CLASSES}
        present = {resolution_class(w, h) for (_, w, h) in cams}
        for cls in CLASSES:  # coordinate descent, one class at a time
            if cls not in present:
                continue
            results = []
            for shape in shapes:
                trial = dict(choice)
                trial[cls] = shape
                plan = Plan(vrt.KERNEL_MASK_PIXEL, shapes[0], trial)
                ms = _time(torch, renderer, world, cams, images, plan, stream, reps)
                results.append((ms, shape))
                table.append({"kernel": "tile", "threads": threads, "class": cls, "tile": "x".join(map(str, shape)),
                              "ms": ms})
            choice[cls] = min(results)[1]
        plan = Plan(vrt.KERNEL_MASK_PIXEL, shapes[0], choice)
        ms = _time(torch, renderer, world, cams, images, plan, stream, reps)
        if best is None or ms < best[0]:
            best = (ms, plan)
    for tile, refill in PERSISTENT:
        plan = Plan(vrt.KERNEL_BITMASK, tile, {}, refill)
        ms = _time(torch, renderer, world, cams, images, plan, stream, reps)
        table.append({"kernel": "persistent", "tile": "x".join(map(str, tile)), "refill_min": refill, "ms": ms})
        if ms < best[0]:
            best = (ms, plan)
    best[1].table = table
    return best[1]
