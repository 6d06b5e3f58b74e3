"""The tile kernel on worlds with depth-field words -- the reference's own worlds, where
fixDepthField leaves a jump distance in almost every air voxel near a solid.  The
kernel follows the shader's jumps (fshader.glsl:114-121) and its float distance cap
(:83); its frames must equal the oracle's and the reference shader's golden outputs."""
import json

import numpy as np
import pytest

import vrt
from helpers import assert_same_frame, fcolor_from_outputs, gpu_render, load_golden, make_world, uniforms_from_dict
from test_gpu_fuzz import random_case

pytestmark = pytest.mark.gpu


def test_reference_scene(cuda, oracle):
    case = load_golden("shader_reference_scene.npz")
    w = vrt.World(512, 96)
    w.init_reference()
    w.fix_depth_field()
    assert w.info().has_depth_field == 1
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    u = uniforms_from_dict(json.loads(str(case["uniforms"])))
    g = gpu_render(w, u, 800, 600, kernel=vrt.KERNEL_MASK_PIXEL)
    px, py = case["px"], case["py"]
    assert np.array_equal(g["hit"][py, px], case["hit"])
    assert np.array_equal(g["steps"][py, px], case["steps"])
    col = fcolor_from_outputs(words, g["hit"][py, px], g["shade"][py, px])
    assert (col.view(np.uint32) == case["color_bits"][:, :3]).all()
    o = oracle.render(words, 512, 96, u, 800, 600)
    assert_same_frame(o, g)
    for k in (vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD):  # inexact launches
        f = gpu_render(w, u, 800, 600, kernel=k, debug=False)
        assert np.array_equal(f["rgba"], o["rgba"]), k
        assert int(f["stats"][vrt.STAT_RAYS]) == o["totals"]["rays"]


@pytest.mark.parametrize("kernel", [vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD])
def test_edits_refresh_the_stop_masks(cuda, oracle, vrt_lib, kernel):
    """The tile kernel's stop masks and the word kernel's z-major copy of the words are
    caches of the words: after each edit the next render sees the edited world."""
    W, H = 96, 48
    w = make_world(vrt_lib.terrain_generate(W, H, 17, 2), W, H)
    w.fix_depth_field()
    u = vrt.default_uniforms()
    u.camPos[:] = [20.5, 40.25, 18.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.6, 0.9)
    u.lightPos[:] = [48.0, 400.0, 20.0]
    u.maxSteps = 200
    u.localLightDist = 24.0
    u.localLights[0][:] = [40.5, 30.5, 44.5, 0.7]
    u.aspectRatio = 80 / 60
    for edit in range(3):
        words = w.download(np.empty(W * H * W, np.int32))
        o = oracle.render(words, W, H, u, 80, 60)
        assert (o["hit"] >= 0).sum() > 100
        assert_same_frame(o, gpu_render(w, u, 80, 60, kernel=kernel))
        w.remove_sphere(40 + 9 * edit, 20, 40 - 7 * edit, 6, 1)  # with the depth-field refresh


@pytest.mark.parametrize("seed", range(10))
def test_random_depth_field_scenes(cuda, oracle, seed):
    words, W, H, u, width, height = random_case(seed)
    w = make_world(words, W, H)
    w.fix_depth_field()
    words = w.download(np.empty_like(words))
    o = oracle.render(words, W, H, u, width, height)
    for k in (vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD):
        try:
            assert_same_frame(o, gpu_render(w, u, width, height, kernel=k))
        except AssertionError as e:
            raise AssertionError(f"seed {seed}, kernel {k}: {e}") from None
    for k in (vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD):
        g = gpu_render(w, u, width, height, kernel=k, debug=False)
        assert np.array_equal(o["rgba"], g["rgba"]), f"seed {seed}, kernel {k}: inexact launch"


def test_batch_on_a_depth_field_world(cuda, oracle):
    """vrt_render_batch renders a reference-format world with the tile kernel; the graph
    and allocation-free forms refuse it (a replay would keep stale stop masks after an
    edit, and the stop masks are allocated on first use)."""
    import ctypes as C
    import torch
    W, H = 64, 32
    w = make_world(vrt.terrain_generate(W, H, 5, 2), W, H)
    w.fix_depth_field()
    words = w.download(np.empty(W * H * W, np.int32))
    cams = []
    for i, (wd, ht) in enumerate([(40, 30), (23, 17), (64, 48)]):
        u = vrt.default_uniforms()
        u.camPos[:] = [10.5 + 7 * i, 28.25, 12.5 + 5 * i]
        u.rotateMatrix[:] = vrt.rotate_matrix(0.5 + 0.1 * i, 0.7 * i)
        u.lightPos[:] = [32.0, 300.0, 10.0]
        u.maxSteps = 150
        u.aspectRatio = wd / ht
        cams.append((u, wd, ht))
    imgs = [torch.zeros(wd * ht * 4, dtype=torch.uint8, device="cuda") for (_, wd, ht) in cams]
    views = [vrt.make_view(w, u, wd, ht, img.data_ptr()) for (u, wd, ht), img in zip(cams, imgs)]
    r = vrt.Renderer()
    r.render_batch(views)
    torch.cuda.synchronize()
    for (u, wd, ht), img in zip(cams, imgs):
        o = oracle.render(words, W, H, u, wd, ht)
        assert np.array_equal(img.cpu().numpy().reshape(ht, wd, 4), o["rgba"])
    arr = (vrt.View * len(views))(*views)
    g = C.c_void_p()
    stream = torch.cuda.current_stream().cuda_stream
    assert vrt.lib().vrt_batch_graph_create(r.handle, arr, len(views), None, stream, C.byref(g)) == vrt.ESTATE
    assert vrt.lib().vrt_render_batch_noalloc(arr, len(views), None, stream) == vrt.ESTATE


@pytest.mark.parametrize("kernel", [vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD])
def test_two_streams_after_an_edit(cuda, oracle, vrt_lib, kernel):
    """The first render after an edit rebuilds the stop masks (tile kernel) or updates the
    z-major copy of the words (word kernel) on its stream; a render of the same world on
    another stream right after it must wait for that."""
    import torch
    W, H = 96, 48
    w = make_world(vrt_lib.terrain_generate(W, H, 23, 2), W, H)
    w.fix_depth_field()
    u = vrt.default_uniforms()
    u.camPos[:] = [30.5, 38.25, 20.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.55, 0.4)
    u.lightPos[:] = [48.0, 400.0, 20.0]
    u.maxSteps = 200
    u.aspectRatio = 96 / 64
    o_opts = vrt.RenderOpts()
    o_opts.kernel = kernel
    r1, r2 = vrt.Renderer(), vrt.Renderer()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for edit in range(3):
        w.remove_sphere(44 + 6 * edit, 22, 46, 7, 1)
        torch.cuda.synchronize()
        img1 = torch.zeros(96 * 64 * 4, dtype=torch.uint8, device="cuda")
        img2 = torch.zeros_like(img1)
        r1.render(w, u, 96, 64, img1.data_ptr(), None, 0, o_opts, s1.cuda_stream)
        r2.render(w, u, 96, 64, img2.data_ptr(), None, 0, o_opts, s2.cuda_stream)
        torch.cuda.synchronize()
        words = w.download(np.empty(W * H * W, np.int32))
        o = oracle.render(words, W, H, u, 96, 64)
        assert np.array_equal(img1.cpu().numpy().reshape(64, 96, 4), o["rgba"])
        assert np.array_equal(img2.cpu().numpy().reshape(64, 96, 4), o["rgba"])


def test_banded_host_render_after_an_edit(cuda, oracle, vrt_lib):
    """vrt_render_to_host with the tile kernel on a depth-field world: the bands run on
    their own streams, the first rebuilds the stop masks and the others wait for it."""
    import torch
    W, H = 96, 48
    w = make_world(vrt_lib.terrain_generate(W, H, 29, 2), W, H)
    w.fix_depth_field()
    u = vrt.default_uniforms()
    u.camPos[:] = [26.5, 37.25, 22.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.5, 0.6)
    u.lightPos[:] = [48.0, 400.0, 20.0]
    u.maxSteps = 200
    width, height = 120, 300
    u.aspectRatio = width / height
    o_opts = vrt.RenderOpts()
    o_opts.kernel = vrt.KERNEL_MASK_PIXEL
    o_opts.host_bands = 5
    r = vrt.Renderer()
    host = torch.zeros(width * height * 4, dtype=torch.uint8, pin_memory=True)
    for edit in range(2):
        w.remove_sphere(40 + 8 * edit, 24, 50, 6, 1)
        torch.cuda.synchronize()
        r.render_to_host(w, u, width, height, host.data_ptr(), o_opts)
        words = w.download(np.empty(W * H * W, np.int32))
        o = oracle.render(words, W, H, u, width, height)
        assert np.array_equal(host.numpy().reshape(height, width, 4), o["rgba"])


def test_word_kernel_copy_follows_every_kind_of_edit(cuda, oracle, vrt_lib):
    """The word kernel reads z steps from a z-major copy of the words, brought up to date
    over the changed box at its next render: after placeVoxel, a partial upload, removeSphere
    with the depth-field refresh and a fixDepthField box, each frame equals the oracle's on
    the words of that moment, and the world's device bytes include the copy once."""
    W, H = 80, 40
    w = make_world(vrt_lib.terrain_generate(W, H, 29, 2), W, H)
    w.fix_depth_field()
    u = vrt.default_uniforms()
    u.camPos[:] = [12.5, 34.25, 10.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.45, 0.7)  # looking along +z and +x, downwards
    u.lightPos[:] = [40.0, 300.0, 60.0]
    u.maxSteps = 160
    u.aspectRatio = 72 / 48
    before = w.info().device_bytes

    def check():
        words = w.download(np.empty(W * H * W, np.int32))
        assert_same_frame(oracle.render(words, W, H, u, 72, 48), gpu_render(w, u, 72, 48, kernel=vrt.KERNEL_WORD))

    check()  # makes the copy
    assert w.info().device_bytes == before + 4 * W * H * W
    w.place_voxel(30, 30, 34, 0x01FF0000)
    check()
    slab = np.full(W * 3, 0x0100FF00, np.int32)  # three rows of solid words at y = 26
    w.upload(slab, first=26 * W + 40 * W * H)
    check()
    w.remove_sphere(36, 22, 40, 6, 1)
    check()
    w.fix_depth_field((20, 10, 20, 60, 40, 60))
    check()
    assert w.info().device_bytes == before + 4 * W * H * W


def test_word_kernel_launches_heaviest_tiles_first(cuda, oracle):
    """Each word-kernel render records its tiles' costs, and the next render of the same
    grid on the same renderer launches the tiles heaviest first.  The order moves tiles,
    not results: the first (row order) and the later (ordered) frames of the reference
    scene equal the oracle's, also after the camera moved (an order from the old view),
    when the tile grid changes (the order starts over) and with every debug output."""
    case = load_golden("shader_reference_scene.npz")
    w = vrt.World(512, 96)
    w.init_reference()
    w.fix_depth_field()
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    u = uniforms_from_dict(json.loads(str(case["uniforms"])))
    r = vrt.Renderer()
    o = oracle.render(words, 512, 96, u, 800, 600)
    for _ in range(3):
        f = gpu_render(w, u, 800, 600, kernel=vrt.KERNEL_WORD, debug=False, renderer=r)
        assert np.array_equal(f["rgba"], o["rgba"])
        assert int(f["stats"][vrt.STAT_RAYS]) == o["totals"]["rays"]
        assert int(f["stats"][vrt.STAT_PIXELS]) == 800 * 600
    u2 = uniforms_from_dict(json.loads(str(case["uniforms"])))
    u2.camPos[:] = [300.5, 62.25, 90.75]
    u2.rotateMatrix[:] = vrt.rotate_matrix(-0.2, 2.4)
    o2 = oracle.render(words, 512, 96, u2, 800, 600)
    for tile in (None, None, (8, 16), (8, 16), (32, 4)):
        f = gpu_render(w, u2, 800, 600, kernel=vrt.KERNEL_WORD, debug=False, renderer=r, tile=tile)
        assert np.array_equal(f["rgba"], o2["rgba"]), tile
        assert int(f["stats"][vrt.STAT_RAYS]) == o2["totals"]["rays"], tile
    assert_same_frame(o2, gpu_render(w, u2, 800, 600, kernel=vrt.KERNEL_WORD, renderer=r, tile=(32, 4)))
    r.close()


def test_word_kernel_order_across_worlds_and_host_images(cuda, oracle):
    """One renderer alternating between two depth-field worlds of one size, with images in
    device memory, page-locked host memory and pageable host memory: every frame runs its
    tiles in the order the previous frame (of the other world, or the other image kind)
    recorded, and every frame equals the oracle's."""
    import ctypes as C

    # two worlds of one size: random_case's scene and camera, and sparse random voxels;
    # 160x96 pixels make 120 tiles of 16x8 to order
    words0, W, H, u0, _, _ = random_case(3)
    width, height = 160, 96
    rng = np.random.default_rng(77)
    words1 = np.where(rng.random(W * H * W) < 0.06, 0x01000000 | rng.integers(0, 1 << 24, W * H * W),
                      -1).astype(np.int32)
    worlds = []
    for words in (words0, words1):
        w = make_world(words, W, H)
        w.fix_depth_field()
        worlds.append((w, w.download(np.empty_like(words))))
    u0.aspectRatio = width / height
    expect = [oracle.render(wd, W, H, u0, width, height)["rgba"] for _, wd in worlds]
    r = vrt.Renderer()
    o = vrt.RenderOpts()
    o.kernel = vrt.KERNEL_WORD
    n = width * height * 4
    p = C.c_void_p()
    vrt.check(vrt.lib().vrt_host_alloc(n, C.byref(p)))
    try:
        pinned = np.ctypeslib.as_array((C.c_uint8 * n).from_address(p.value))
        pageable = np.zeros(n, np.uint8)
        for frame in range(9):
            k = frame % 2
            w, _ = worlds[k]
            kind = frame % 3
            if kind == 0:
                f = gpu_render(w, u0, width, height, kernel=vrt.KERNEL_WORD, debug=False, renderer=r)
                img = f["rgba"]
            elif kind == 1:
                pinned[:] = 0
                r.render_to_host(w, u0, width, height, p.value, o)
                img = pinned.reshape(height, width, 4)
            else:
                pageable[:] = 0
                r.render_to_host(w, u0, width, height, pageable.ctypes.data, o)
                img = pageable.reshape(height, width, 4)
            assert np.array_equal(img, expect[k]), (frame, kind)
    finally:
        vrt.check(vrt.lib().vrt_host_free(p))
    r.close()
