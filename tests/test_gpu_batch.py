"""Batched rendering: many cameras of uneven size in one persistent launch, and the
same launch captured in a CUDA graph, are bit-identical to one render per camera."""
import numpy as np
import pytest

import scenes
import vrt
from helpers import gpu_render, make_world

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch_setup():
    sc = scenes.full(2, W=256, H=128, width=64, height=64, max_steps=512)
    views = scenes.batch_views(sc, 24, seed=7)
    # scale the sizes down so the per-camera references stay quick
    views = [(u, max(8, w // 4), max(6, h // 4)) for (u, w, h) in views]
    for (u, w, h) in views:
        u.aspectRatio = w / h
    return sc, views


def _batch(torch, renderer, world, views, opts=None, graph=False):
    imgs = [torch.zeros(w * h * 4, dtype=torch.uint8, device="cuda") for (_, w, h) in views]
    stats = torch.zeros((len(views), vrt.STAT_COUNT), dtype=torch.int64, device="cuda")
    vv = [vrt.make_view(world, u, w, h, img.data_ptr(), stats[i].data_ptr())
          for i, ((u, w, h), img) in enumerate(zip(views, imgs))]
    stream = torch.cuda.current_stream().cuda_stream
    if graph:
        import ctypes as C
        arr = (vrt.View * len(vv))(*vv)
        g = C.c_void_p()
        vrt.check(vrt.lib().vrt_batch_graph_create(renderer.handle, arr, len(vv), C.byref(opts) if opts else None,
                                                   stream, C.byref(g)))
        for _ in range(3):
            stats.zero_()
            vrt.check(vrt.lib().vrt_batch_graph_launch(g, stream))
        torch.cuda.synchronize()
        vrt.lib().vrt_batch_graph_destroy(g)
    else:
        renderer.render_batch(vv, opts, stream)
        torch.cuda.synchronize()
    return [i.cpu().numpy() for i in imgs], stats.cpu().numpy()


def test_batch_equals_single_renders(cuda, batch_setup):
    sc, views = batch_setup
    w = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    imgs, stats = _batch(cuda, r, w, views)
    for i, (u, width, height) in enumerate(views):
        g = gpu_render(w, u, width, height, kernel=vrt.KERNEL_WORD)
        assert np.array_equal(imgs[i].reshape(height, width, 4), g["rgba"]), f"view {i}"
        assert int(stats[i, vrt.STAT_RAYS]) == int(g["stats"][vrt.STAT_RAYS])
        assert int(stats[i, vrt.STAT_HITS]) == int(g["stats"][vrt.STAT_HITS])


@pytest.mark.parametrize("tile,refill", [((16, 8), 4), ((32, 1), 16), ((8, 8), 32)])
def test_batch_tilings_and_graph(cuda, batch_setup, tile, refill):
    sc, views = batch_setup
    w = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    base, bstats = _batch(cuda, r, w, views)
    opts = vrt.RenderOpts()
    opts.kernel = vrt.KERNEL_BITMASK
    opts.tile_w, opts.tile_h = tile
    opts.refill_min = refill
    got, gstats = _batch(cuda, r, w, views, opts, graph=True)
    for a, b in zip(base, got):
        assert np.array_equal(a, b)
    # rays, hits and pixels are fixed by the frame; iterations performed (rays that cannot
    # hit end early) and the traversal diagnostics depend on the kernel
    assert np.array_equal(bstats[:, [0, 2, 3]], gstats[:, [0, 2, 3]])


def test_batch_rejects_mixed_worlds(cuda, batch_setup):
    sc, views = batch_setup
    w1 = make_world(sc.words, sc.W, sc.H)
    w2 = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    img = cuda.zeros(64 * 64 * 4, dtype=cuda.uint8, device="cuda")
    vv = [vrt.make_view(w1, views[0][0], 8, 8, img.data_ptr()), vrt.make_view(w2, views[1][0], 8, 8, img.data_ptr())]
    with pytest.raises(vrt.VrtError):
        r.render_batch(vv)


def test_per_view_tiles_and_autotuner(cuda, batch_setup):
    import autotune
    sc, views = batch_setup
    w = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    base, _ = _batch(cuda, r, w, views)
    imgs = [cuda.zeros(vw * vh * 4, dtype=cuda.uint8, device="cuda") for (_, vw, vh) in views]
    ptrs = [im.data_ptr() for im in imgs]
    plan = autotune.tune(cuda, r, w, views, ptrs, reps=1)
    assert plan.table and plan.describe()["kernel"] in ("tile", "persistent")
    for im in imgs:
        im.zero_()
    r.render_batch(plan.views(w, views, ptrs), plan.opts(), cuda.cuda.current_stream().cuda_stream)
    cuda.cuda.synchronize()
    for a, b in zip(base, imgs):
        assert np.array_equal(a, b.cpu().numpy())
    # mixed shapes of one thread count in one launch
    mixed = [vrt.make_view(w, u, vw, vh, p, 0, [(8, 16), (16, 8), (32, 4)][i % 3])
             for i, ((u, vw, vh), p) in enumerate(zip(views, ptrs))]
    for im in imgs:
        im.zero_()
    r.render_batch(mixed, None, cuda.cuda.current_stream().cuda_stream)
    cuda.cuda.synchronize()
    for a, b in zip(base, imgs):
        assert np.array_equal(a, b.cpu().numpy())
    bad = [vrt.make_view(w, views[0][0], views[0][1], views[0][2], ptrs[0], 0, (8, 8))]
    with pytest.raises(vrt.VrtError):
        r.render_batch(bad, None)  # 64 threads in a 128-thread launch


def test_persistent_kernel_per_view_tiles_and_refill(cuda, batch_setup):
    """The persistent kernel takes a tile and a live-ray refill interval per view (any tile
    of up to 1024 pixels): images and ray counts stay those of the tile kernel's batch."""
    import autotune
    sc, views = batch_setup
    w = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    base, bstats = _batch(cuda, r, w, views)
    plan = autotune.Plan(vrt.KERNEL_BITMASK, (8, 4), {}, 8)
    imgs = [cuda.zeros(vw * vh * 4, dtype=cuda.uint8, device="cuda") for (_, vw, vh) in views]
    stats = cuda.zeros((len(views), vrt.STAT_COUNT), dtype=cuda.int64, device="cuda")
    shapes = [((16, 8), 4), ((32, 1), 16), ((8, 8), 32), ((5, 3), 1), ((64, 16), 8)]
    vv = [vrt.make_view(w, u, vw, vh, imgs[i].data_ptr(), stats[i].data_ptr(), *shapes[i % len(shapes)])
          for i, (u, vw, vh) in enumerate(views)]
    r.render_batch(vv, plan.opts(), cuda.cuda.current_stream().cuda_stream)
    cuda.cuda.synchronize()
    for a, b in zip(base, imgs):
        assert np.array_equal(a, b.cpu().numpy())
    assert np.array_equal(bstats[:, [0, 2, 3]], stats.cpu().numpy()[:, [0, 2, 3]])
    bad = plan.views(w, views[:1], [imgs[0].data_ptr()])
    bad[0].refill_min = 33
    with pytest.raises(vrt.VrtError):
        r.render_batch(bad, plan.opts())
    bad[0].refill_min = 0
    bad[0].tile_w, bad[0].tile_h = 64, 32  # 2048 pixels
    with pytest.raises(vrt.VrtError):
        r.render_batch(bad, plan.opts())
