"""Small, self-contained workloads of the library's kernels, one per ncu capture.

Each case builds its world, runs the kernel under study a few times and exits; the ncu
commands in profiles/*.md name the case and the kernel (-k) they capture.

  frame1080      the 1080p frame of bench.py: world 512x256x512 (seed 2), 1920x1080, 16
                 local lights + global, 1024 steps; tile kernel, 8x16 tiles, inexact
                 (render_tiles_kernel<false,false,false>), 2 launches
  stress_scaled  the stress camera (1 voxel above the terrain, pitch -2 degrees, 16 lights,
                 3840x2160, 4096 steps) on a 1024x256x1024 world instead of 2048x256x2048
                 (1 GiB of words instead of 4), 2 launches
  batch          the 64 cameras of the bench's batch over the 1080p world, tile kernel with
                 a tile shape per resolution class, replayed twice from a CUDA graph
  edits          removeSphere of radius 8 at 8 surface points of the 1080p world
                 (remove_sphere_kernel, then the mask and distance refresh of each edit)
  depth_edits    the reference world (initVoxels + fixDepthField) edited by removeSphere
                 of radius 7 with the depth-field refresh, 4 times: the first
                 fix_depth_field_kernel launch is the whole world, the next are edit-sized
  stop_masks     the reference world after an edit, rendered by the tile kernel
                 (stop_mask_kernel rebuilds the stop masks, then the render), 2 rounds
  probe          1 Mi voxel probes of the 1080p world (probe_kernel), 3 launches
  world_build    upload of the 1080p world (brick_mask, parent_mask, dir_pass, cheb_pass)
  reference_build  the reference world on the device: initVoxels (init_reference_layers,
                 init_reference_trees), then fixDepthField over the whole world
  reference_frame  the reference app's first frame (its world with the depth field, camera
                 (195,55,155), 800x600, 384 steps), rendered as bench.py --workload reference
                 does: the kernel AUTO picks (the word kernel) with its own 16x8 pixel tiles,
                 2 launches
  all            every case above, one after the other

Usage: python voxel-rt_gb300/profile_cases.py CASE
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import build as vbuild  # noqa: E402
import scenes  # noqa: E402
import vrt  # noqa: E402

THREADS = os.cpu_count() or 1


def _torch():
    import torch
    torch.cuda.init()
    return torch


def _frame_world():
    sc = scenes.full(2, threads=THREADS)
    w = vrt.World(sc.W, sc.H)
    w.upload(sc.words)
    return sc, w


def _render(torch, w, u, width, height, n, opts=None):
    img = torch.empty(width * height * 4, dtype=torch.uint8, device="cuda")
    r = vrt.Renderer()
    for _ in range(n):
        r.render(w, u, width, height, img.data_ptr(), None, 0, opts, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    r.close()


def case_frame1080(torch):
    sc, w = _frame_world()
    o = vrt.RenderOpts()
    o.kernel = vrt.KERNEL_MASK_PIXEL
    o.tile_w, o.tile_h = 8, 16
    _render(torch, w, sc.uniforms, sc.width, sc.height, 2, o)
    return f"{sc.workload}: 2 frames"


def case_stress_scaled(torch):
    st = scenes.stress(5, threads=THREADS, W=1024)
    w = vrt.World(st.W, st.H)
    w.upload(st.words)
    _render(torch, w, st.uniforms, st.width, st.height, 2)
    return f"{st.workload}: 2 frames"


def case_batch(torch):
    import ctypes as C
    import autotune
    sc, w = _frame_world()
    cams = scenes.batch_views(sc, 64, seed=3)
    imgs = [torch.empty(cw * ch * 4, dtype=torch.uint8, device="cuda") for (_, cw, ch) in cams]
    plan = autotune.Plan(vrt.KERNEL_MASK_PIXEL, (8, 16), {"small": (16, 8), "medium": (32, 4), "large": (8, 16)})
    views = plan.views(w, cams, [i.data_ptr() for i in imgs])
    arr = (vrt.View * len(views))(*views)
    r = vrt.Renderer()
    g = C.c_void_p()
    stream = torch.cuda.current_stream().cuda_stream
    opts = plan.opts()
    vrt.check(vrt.lib().vrt_batch_graph_create(r.handle, arr, len(views), C.byref(opts), stream, C.byref(g)))
    for _ in range(2):
        vrt.check(vrt.lib().vrt_batch_graph_launch(g, stream))
    torch.cuda.synchronize()
    vrt.lib().vrt_batch_graph_destroy(g)
    return f"64 cameras, {sum(cw * ch for _, cw, ch in cams)} pixels, 2 graph replays"


def case_edits(torch):
    sc, w = _frame_world()
    rng = scenes.SplitMix64(17)
    for _ in range(8):
        x, z = rng.randint(16, sc.W - 17), rng.randint(16, sc.W - 17)
        y = vrt.terrain_height(sc.W, sc.seed, x, z) - 1
        w.remove_sphere(x, y, z, 8, 0)
    torch.cuda.synchronize()
    return "8 removeSphere edits of radius 8"


def _reference_world():
    w = vrt.World(512, 96)
    w.init_reference()
    w.fix_depth_field()
    return w


def case_depth_edits(torch):
    w = _reference_world()
    for (x, y, z) in [(195, 40, 170), (100, 38, 300), (400, 39, 60), (260, 41, 450)]:
        w.remove_sphere(x, y, z, 7, 1)
    torch.cuda.synchronize()
    return "reference world: initVoxels, fixDepthField, 4 removeSphere(7) edits with the depth-field refresh"


def case_stop_masks(torch):
    w = _reference_world()
    u = scenes.reference_scene_uniforms()
    o = vrt.RenderOpts()
    o.kernel = vrt.KERNEL_MASK_PIXEL
    for (x, y, z) in [(195, 40, 170), (100, 38, 300)]:
        w.remove_sphere(x, y, z, 7, 1)
        _render(torch, w, u, 800, 600, 1, o)
    return "reference world, 2 rounds of edit + tile-kernel render (stop-mask rebuild)"


def case_probe(torch):
    sc, w = _frame_world()
    n = 1 << 20
    rng = np.random.default_rng(5)
    xyz = np.stack([rng.integers(-8, sc.W + 8, n), rng.integers(-8, sc.H + 8, n), rng.integers(-8, sc.W + 8, n)],
                   -1).astype(np.int32)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_out = torch.empty(n, dtype=torch.int32, device="cuda")
    for _ in range(3):
        w.probe(d_xyz.data_ptr(), n, d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return f"3 x {n} probes"


def case_world_build(torch):
    _frame_world()
    torch.cuda.synchronize()
    return "upload of the 512x256x512 world"


def case_reference_build(torch):
    _reference_world()
    torch.cuda.synchronize()
    return "reference world: initVoxels + fixDepthField (512x96x512)"


def case_reference_frame(torch):
    w = _reference_world()
    u = scenes.reference_scene_uniforms()
    o = vrt.RenderOpts()  # bench.py --workload reference: AUTO (the word kernel), its own 16x8 pixel tiles
    _render(torch, w, u, 800, 600, 2, o)
    return "reference world, 800x600, AUTO kernel, default (16x8) tiles: 2 frames"


CASES = {name[5:]: fn for name, fn in globals().items() if name.startswith("case_")}


def main(argv):
    if len(argv) != 2 or (argv[1] not in CASES and argv[1] != "all"):
        print(__doc__)
        return 2
    vbuild.build()
    torch = _torch()
    for name in (CASES if argv[1] == "all" else [argv[1]]):
        t0 = time.perf_counter()
        what = CASES[name](torch)
        print(f"{name}: {what} ({time.perf_counter() - t0:.2f} s)", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
