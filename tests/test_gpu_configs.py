"""Parity with the CPU oracle at the benchmark workloads' real sizes, through the C ABI.

  1080p frame   world 512x256x512, 1920x1080, 16 local lights + global, 1024 steps: the
                launch the bench times (tile kernel, 8x16 ray tiles, no step counts asked
                for, so rays that cannot hit end early), whole frame, with its hit index,
                cast and occlusion bits and light multipliers made visible; the same launch
                without side outputs; the exact-steps counting frame; the word and
                persistent kernels on the same frame
  stress        world 2048x256x2048 (4 GiB of words), 3840x2160, 4096 steps, camera one
                voxel above the terrain at pitch -2 degrees: every 54th row
  batch         the bench's 64 cameras (320x240 ... 1920x1080, 0-16 lights) over the 1080p
                frame's world in one launch, every view whole: tile kernel with one tile
                shape per resolution class replayed from a CUDA graph, and the persistent
                kernel
  serving       a request stream with edits over four resident worlds (256^3, 512x256x512,
                1024x256x1024 twice): every render against the oracle on the words its
                world held when it ran, renders looking at each edit before and after it

Hit indices, cast and occlusion bits and light multipliers are bit-exact, RGBA8 equal
(the bar is RGB within RGB_TOL = 1), and ray, hit and pixel counts equal the oracle's.
Reference: fshader.glsl:33-190 (the path), level.cpp:30-56 (edits).
"""
import os

import numpy as np
import pytest

import autotune
import scenes
import serving
import vrt
from helpers import INEXACT_OUTPUTS, assert_same_frame, gpu_render, make_world

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _counts_match(o, g, steps=False):
    t = o["totals"]
    s = g["stats"]
    assert [int(s[vrt.STAT_RAYS]), int(s[vrt.STAT_HITS]), int(s[vrt.STAT_PIXELS])] == [t["rays"], t["hits"], t["pixels"]]
    if steps:
        assert int(s[vrt.STAT_STEPS]) == t["steps"]


@pytest.fixture(scope="module")
def frame1080(oracle):
    sc = scenes.full(2, threads=THREADS)
    o = oracle.render(sc.words, sc.W, sc.H, sc.uniforms, sc.width, sc.height, threads=THREADS)
    return sc, o


def test_bench_frame_1080p_whole(cuda, frame1080):
    """The timed launch: vrt_render, tile kernel, 8x16 tiles, inexact."""
    sc, o = frame1080
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=vrt.KERNEL_MASK_PIXEL, tile=(8, 16), refill_min=8,
                   outputs=INEXACT_OUTPUTS)
    assert_same_frame(o, g, outputs=INEXACT_OUTPUTS)
    _counts_match(o, g)
    assert int(g["stats"][vrt.STAT_STEPS]) < o["totals"]["steps"]  # rays that cannot hit ended early
    assert (o["cast"] > 1).sum() > 1000 and (o["occ"] & 1).sum() > 1000  # local lights cast, sun shadows
    # exactly the bench's launch: no side outputs (the pixel store is the only store)
    g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=vrt.KERNEL_MASK_PIXEL, tile=(8, 16), refill_min=8,
                   debug=False)
    assert np.array_equal(g["rgba"], o["rgba"])
    _counts_match(o, g)
    # the bench's counting frame: every DDA iteration of the shader counted
    g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=vrt.KERNEL_MASK_PIXEL, tile=(8, 16), debug=False,
                   exact_steps=1)
    assert np.array_equal(g["rgba"], o["rgba"])
    _counts_match(o, g, steps=True)
    w.close()


@pytest.mark.parametrize("kernel", [vrt.KERNEL_WORD, vrt.KERNEL_BITMASK])
def test_other_kernels_1080p_whole(cuda, frame1080, kernel):
    sc, o = frame1080
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=kernel, outputs=INEXACT_OUTPUTS)
    assert_same_frame(o, g, outputs=INEXACT_OUTPUTS)
    _counts_match(o, g)
    w.close()


def test_stress_frame_rows(cuda, oracle):
    """2048x256x2048, 3840x2160, 4096 steps, grazing camera: every 54th row (40 rows),
    through the tile kernel's inexact launch and the bench's launch without side outputs."""
    st = scenes.stress(5, threads=THREADS)
    rows = (27, st.height, 54)
    o = oracle.render(st.words, st.W, st.H, st.uniforms, st.width, st.height, rows=rows, threads=THREADS)
    w = make_world(st.words, st.W, st.H)
    st.words = None
    sel = slice(*rows)
    g = gpu_render(w, st.uniforms, st.width, st.height, outputs=INEXACT_OUTPUTS)
    assert_same_frame(o, g, rows=sel, outputs=INEXACT_OUTPUTS)
    assert (o["hit"][sel] >= 0).mean() > 0.3  # the grazing rays meet terrain
    g = gpu_render(w, st.uniforms, st.width, st.height, debug=False)
    assert np.array_equal(g["rgba"][sel], o["rgba"][sel])
    w.close()


def _batch_images(cuda, world, cams, plan, graph):
    import ctypes as C
    imgs = [cuda.zeros(w * h * 4, dtype=cuda.uint8, device="cuda") for (_, w, h) in cams]
    stats = cuda.zeros((len(cams), vrt.STAT_COUNT), dtype=cuda.int64, device="cuda")
    views = plan.views(world, cams, [i.data_ptr() for i in imgs], [stats[i].data_ptr() for i in range(len(cams))])
    stream = cuda.cuda.current_stream().cuda_stream
    opts = plan.opts()
    renderer = vrt.Renderer()
    if graph:
        arr = (vrt.View * len(views))(*views)
        g = C.c_void_p()
        vrt.check(vrt.lib().vrt_batch_graph_create(renderer.handle, arr, len(views), C.byref(opts), stream,
                                                   C.byref(g)))
        for _ in range(2):  # a replay renders the same images
            stats.zero_()
            vrt.check(vrt.lib().vrt_batch_graph_launch(g, stream))
        cuda.cuda.synchronize()
        vrt.lib().vrt_batch_graph_destroy(g)
    else:
        renderer.render_batch(views, opts, stream)
        cuda.cuda.synchronize()
    return [i.cpu().numpy() for i in imgs], stats.cpu().numpy()


def test_batch_64_views_whole(cuda, oracle, frame1080):
    sc, _ = frame1080
    cams = scenes.batch_views(sc, 64, seed=3)
    assert len({autotune.resolution_class(w, h) for (_, w, h) in cams}) == 3
    refs = [oracle.render(sc.words, sc.W, sc.H, u, w, h, threads=THREADS, outputs=("rgba",)) for (u, w, h) in cams]
    world = make_world(sc.words, sc.W, sc.H)
    plans = [(autotune.Plan(vrt.KERNEL_MASK_PIXEL, (8, 16), {"small": (16, 8), "medium": (32, 4), "large": (8, 16)}),
              True),
             (autotune.Plan(vrt.KERNEL_BITMASK, (8, 4), {}, 8), False)]
    for plan, graph in plans:
        imgs, stats = _batch_images(cuda, world, cams, plan, graph)
        for i, ((u, w, h), o) in enumerate(zip(cams, refs)):
            assert np.array_equal(imgs[i].reshape(h, w, 4), o["rgba"]), f"{plan.describe()}: view {i} ({w}x{h})"
            t = o["totals"]
            got = [int(stats[i, vrt.STAT_RAYS]), int(stats[i, vrt.STAT_HITS]), int(stats[i, vrt.STAT_PIXELS])]
            assert got == [t["rays"], t["hits"], t["pixels"]], f"{plan.describe()}: view {i} counts"
    world.close()


def _edit_camera(sc, edit, width, height):
    """A camera 12 voxels above an edit's centre, looking down at it."""
    x, y, z, _ = edit
    u = scenes.base_uniforms(width, height, sc.uniforms.maxSteps, 70.0, sc.uniforms.localLightDist)
    scenes.set_lights(u, sc.lights[:4])
    scenes.aim(u, (x + 0.5, y + 12.5, z - 6.5), 0.0, -60.0)
    u.lightPos[:] = list(sc.uniforms.lightPos)
    return u


def test_served_stream_with_edits(cuda, oracle):
    import torch
    worlds = [scenes.full(21, W=256, H=256, threads=THREADS), scenes.full(2, threads=THREADS),
              scenes.full(22, W=1024, H=256, threads=THREADS), scenes.full(23, W=1024, H=256, threads=THREADS)]
    devs = [make_world(s.words, s.W, s.H) for s in worlds]
    specs = [serving.WorldSpec(s, d) for s, d in zip(worlds, devs)]
    stream = serving.make_requests(specs, 400.0, 0.12, seed=24)
    # around every edit, a render looking at it from above, before and after
    reqs = []
    for (_, kind, wi, payload) in stream:
        if kind == vrt.REQ_EDIT:
            look = (_edit_camera(worlds[wi], payload, 320, 240), 320, 240)
            reqs += [(vrt.REQ_RENDER, wi, look), (kind, wi, payload), (vrt.REQ_RENDER, wi, look)]
        else:
            reqs.append((kind, wi, payload))
    assert sum(1 for r in reqs if r[0] == vrt.REQ_EDIT and r[1] >= 2) >= 3  # edits on the 1024-wide worlds
    srv = serving.Server(40 << 30, slots=4, max_batch=8)
    wids = [srv.add_world(d) for d in devs]
    images, done = {}, {}
    for tag, (kind, wi, payload) in enumerate(reqs):
        q = vrt.Request()
        q.kind, q.world_id, q.user_tag = kind, wids[wi], tag
        if kind == vrt.REQ_RENDER:
            u, w, h = payload
            q.uniforms, q.width, q.height = u, w, h
            # alternately page-locked (the kernel stores into it) and pageable (copied) results
            img = torch.zeros(w * h * 4, dtype=torch.uint8, pin_memory=True) if tag % 2 else np.zeros(w * h * 4, np.uint8)
            images[tag] = img
            q.host_rgba = img.data_ptr() if tag % 2 else img.ctypes.data
        else:
            q.cx, q.cy, q.cz, q.radius = payload
        srv.submit(q)
        for c in srv.poll():  # admit as requests arrive: later ones join while earlier ones run
            done[c.user_tag] = c
    for c in srv.drain():
        done[c.user_tag] = c
    srv.close()
    assert len(done) == len(reqs) and all(c.status == 0 for c in done.values())
    # replay on the host in submission order: each world's words at each render
    looks = {}
    for tag, (kind, wi, payload) in enumerate(reqs):
        sc = worlds[wi]
        if kind == vrt.REQ_EDIT:
            x, y, z, r = payload
            oracle.remove_sphere(sc.words, sc.W, sc.H, x, y, z, r, 0)
            continue
        u, w, h = payload
        o = oracle.render(sc.words, sc.W, sc.H, u, w, h, threads=THREADS, outputs=("rgba",))
        img = images[tag]
        got = (img.numpy() if hasattr(img, "numpy") else img).reshape(h, w, 4)
        assert np.array_equal(got, o["rgba"]), f"request {tag} (world {wi}, {w}x{h})"
        assert int(done[tag].rays) == o["totals"]["rays"], f"request {tag}: rays"
        if w == 320:
            looks.setdefault(id(u), []).append(got)
    assert sum(1 for v in looks.values() if len(v) == 2 and not np.array_equal(v[0], v[1])) >= 3  # edits seen
    for d in devs:
        d.close()
