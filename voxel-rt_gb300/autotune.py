"""Autotuner for batched rendering: picks the ray-tile shape and the live-ray compaction
interval per resolution class.

A batch (vrt_render_batch) renders cameras of uneven size in one launch.  With the tile
kernel every view may use its own tile shape as long as all shapes have the launch's
thread count; the tile kernel has no compaction step (a lane keeps its pixel until every
ray of the pixel is done).  With the persistent kernel every view may use its own tile
and its own refill interval: the number of a warp's lanes whose rays have ended before the
warp compacts -- refills those lanes with the next rays of their pixels or with new pixels
from the tile queue.  The tuner times, on the caller's own views, each candidate for each
resolution class (small < 0.25 MP, medium < 1 MP, large >= 1 MP) with the other classes
fixed (coordinate descent), keeps the fastest plan of either kernel, and reports the whole
table so a caller can see what was chosen.

Timings are CUDA events on the launching stream around one batched launch, median of
`reps` after one warm-up.
"""
from __future__ import annotations

import statistics

import vrt

CLASSES = ("small", "medium", "large")
# shapes by thread count of the tile kernel (tile_w * tile_h threads per CTA)
SHAPES = {64: [(8, 8), (16, 4), (32, 2), (4, 16)], 128: [(8, 16), (16, 8), (32, 4), (64, 2)]}
# persistent kernel: (tile, refill interval) candidates per class
PERSISTENT = [(tile, refill) for tile in [(8, 4), (16, 8), (32, 1), (8, 8)] for refill in (4, 8, 16)]


def resolution_class(width: int, height: int) -> str:
    mp = width * height / 1e6
    return "small" if mp < 0.25 else ("medium" if mp < 1.0 else "large")


class Plan:
    """The tuner's choice: a kernel, the launch's tile, and a tile shape per class."""

    def __init__(self, kernel: int, launch_tile, class_tiles: dict, refill: int = 0, table=None,
                 class_refill: dict | None = None):
        self.kernel = kernel
        self.launch_tile = launch_tile
        self.class_tiles = class_tiles
        self.refill = refill
        self.class_refill = class_refill or {}
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
            cls = resolution_class(w, h)
            out.append(vrt.make_view(world, u, w, h, img, stats[i] if stats else 0, self.class_tiles.get(cls),
                                     self.class_refill.get(cls, 0)))
        return out

    def describe(self) -> dict:
        name = "tile" if self.kernel == vrt.KERNEL_MASK_PIXEL else "persistent"
        d = {"kernel": name, "launch_tile": "x".join(map(str, self.launch_tile)),
             "tiles_per_class": {k: "x".join(map(str, v)) for k, v in self.class_tiles.items()}}
        if self.kernel != vrt.KERNEL_MASK_PIXEL:
            d["refill_min"] = self.refill
            d["refill_per_class"] = dict(self.class_refill)
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


def tune(torch, renderer, world, cams, images, reps: int = 3, persistent: bool = True) -> Plan:
    """cams: [(uniforms, width, height)], images: device pointers, one per camera.
    persistent=False leaves the persistent kernel out of the search."""
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
    if persistent:
        present = [c for c in CLASSES if c in {resolution_class(w, h) for (_, w, h) in cams}]
        tiles = {c: (8, 4) for c in present}
        refills = {c: 8 for c in present}
        for cls in present:  # coordinate descent over (tile, refill) per class
            results = []
            for tile, refill in PERSISTENT:
                t2, r2 = dict(tiles), dict(refills)
                t2[cls], r2[cls] = tile, refill
                plan = Plan(vrt.KERNEL_BITMASK, (8, 4), t2, 8, class_refill=r2)
                ms = _time(torch, renderer, world, cams, images, plan, stream, reps)
                results.append((ms, tile, refill))
                table.append({"kernel": "persistent", "class": cls, "tile": "x".join(map(str, tile)),
                              "refill_min": refill, "ms": ms})
            _, tiles[cls], refills[cls] = min(results)
        plan = Plan(vrt.KERNEL_BITMASK, (8, 4), tiles, 8, class_refill=refills)
        ms = _time(torch, renderer, world, cams, images, plan, stream, reps)
        if ms < best[0]:
            best = (ms, plan)
    best[1].table = table
    return best[1]
