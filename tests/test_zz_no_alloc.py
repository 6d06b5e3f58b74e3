"""vrt_render_batch_noalloc: the batch render for callers that may not allocate device
memory (a plugin inside a host application that owns every device allocation, or a frame
loop that cannot afford cudaMalloc's implicit synchronisation).  Its scratch lives in a
static device array of the library, so its images must equal vrt_render_batch's, call
after call, although every call reuses that one array.

This file is collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test.  It passes alone and after the others.
"""
import ctypes as C

import numpy as np
import pytest

import scenes
import vrt
from helpers import RGB_TOL, make_world

pytestmark = pytest.mark.gpu


def _views(cuda, world, cams):
    imgs = [cuda.zeros(w * h * 4, dtype=cuda.uint8, device="cuda") for (_, w, h) in cams]
    stats = cuda.zeros((len(cams), vrt.STAT_COUNT), dtype=cuda.int64, device="cuda")
    vv = [vrt.make_view(world, u, w, h, img.data_ptr(), stats[i].data_ptr())
          for i, ((u, w, h), img) in enumerate(zip(cams, imgs))]
    return imgs, stats, (vrt.View * len(vv))(*vv)


@pytest.mark.parametrize("count", [1, 12, 40])
@pytest.mark.parametrize("kernel", [vrt.KERNEL_AUTO, vrt.KERNEL_BITMASK])
def test_noalloc_batch_equals_batch_on_two_calls_in_a_row(cuda, kernel, count):
    """Both kernels a batch can run: the tile kernel (AUTO), whose views travel in the static
    array or, for one view, in the launch itself; and the persistent kernel (BITMASK), whose
    tile counter lives in the static array too and must be cleared by every call.  40 views
    take two copies of the view table."""
    sc = scenes.full(2, W=128, H=64, width=64, height=64, max_steps=256)
    world = make_world(sc.words, sc.W, sc.H)
    cams = [(u, max(8, w // 8), max(6, h // 8)) for (u, w, h) in scenes.batch_views(sc, count, seed=5)]
    for (u, w, h) in cams:
        u.aspectRatio = w / h
    stream = cuda.cuda.current_stream().cuda_stream
    opts = vrt.RenderOpts()
    opts.kernel = kernel
    if kernel == vrt.KERNEL_BITMASK:
        opts.tile_w, opts.tile_h = 8, 4

    ref_imgs, ref_stats, ref_arr = _views(cuda, world, cams)
    r = vrt.Renderer()
    vrt.check(vrt.lib().vrt_render_batch(r.handle, ref_arr, len(cams), C.byref(opts), stream))
    cuda.cuda.synchronize()
    ref = [i.cpu().numpy() for i in ref_imgs]

    for call in range(2):
        imgs, stats, arr = _views(cuda, world, cams)
        vrt.check(vrt.lib().vrt_render_batch_noalloc(arr, len(cams), C.byref(opts), stream))
        cuda.cuda.synchronize()
        for i, (a, b) in enumerate(zip(ref, imgs)):
            d = np.abs(a.astype(np.int32) - b.cpu().numpy().astype(np.int32))
            assert d.max(initial=0) <= RGB_TOL, f"call {call}, view {i}: differs by {d.max()}"
        cols = [vrt.STAT_RAYS, vrt.STAT_HITS, vrt.STAT_PIXELS]
        assert np.array_equal(ref_stats.cpu().numpy()[:, cols], stats.cpu().numpy()[:, cols]), f"call {call}: ray counts"


def test_noalloc_batch_rejects_more_views_than_its_scratch_holds(cuda):
    sc = scenes.small(1)
    world = make_world(sc.words, sc.W, sc.H)
    n = vrt.NOALLOC_MAX_VIEWS + 1
    img = cuda.zeros(8 * 8 * 4, dtype=cuda.uint8, device="cuda")
    vv = [vrt.make_view(world, sc.uniforms, 8, 8, img.data_ptr()) for _ in range(n)]
    arr = (vrt.View * n)(*vv)
    st = vrt.lib().vrt_render_batch_noalloc(arr, n, None, cuda.cuda.current_stream().cuda_stream)
    assert st == vrt.ERANGE
    assert b"scratch" in vrt.lib().vrt_last_error()
