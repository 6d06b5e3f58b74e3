"""Parity of the CUDA render kernels (through the C ABI) with the CPU oracle: hit voxel,
cast and occlusion bits and DDA step counts bit-exact, light multipliers bit-exact,
RGBA8 equal (the spec bar is RGB within 1/255)."""
import numpy as np
import pytest

import scenes
import vrt
from helpers import assert_same_frame, gpu_render, load_golden, make_world, fcolor_from_outputs

pytestmark = pytest.mark.gpu

KERNELS = [vrt.KERNEL_WORD, vrt.KERNEL_BITMASK, vrt.KERNEL_MASK_PIXEL]


@pytest.fixture(scope="module")
def small():
    return scenes.small(1)


@pytest.fixture(scope="module")
def full_world():
    sc = scenes.full(2)
    return sc


def _totals_match(o, g):
    t = o["totals"]
    s = g["stats"]
    assert int(s[vrt.STAT_RAYS]) == t["rays"]
    assert int(s[vrt.STAT_STEPS]) == t["steps"]
    assert int(s[vrt.STAT_HITS]) == t["hits"]
    assert int(s[vrt.STAT_PIXELS]) == t["pixels"]


@pytest.mark.parametrize("kernel", KERNELS)
def test_small_scene(cuda, oracle, small, kernel):
    sc = small
    o = oracle.render(sc.words, sc.W, sc.H, sc.uniforms, sc.width, sc.height)
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=kernel)
    assert_same_frame(o, g)
    _totals_match(o, g)
    assert (o["hit"] >= 0).sum() > 0  # camera (32,48,32) over a 64-wide world sees mostly sky


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_small_scene_seeds(cuda, oracle, seed):
    sc = scenes.small(seed)
    u = sc.uniforms
    u.aspectRatio = 160 / 120
    o = oracle.render(sc.words, sc.W, sc.H, u, 160, 120)
    w = make_world(sc.words, sc.W, sc.H)
    for k in KERNELS:
        assert_same_frame(o, gpu_render(w, u, 160, 120, kernel=k))


@pytest.mark.parametrize("kernel", KERNELS)
def test_full_world_reduced_frame(cuda, oracle, full_world, kernel):
    """512x256x512 world, 16 coloured local lights, 1024 steps, at 480x270."""
    sc = full_world
    u = sc.uniforms
    o = oracle.render(sc.words, sc.W, sc.H, u, 480, 270)
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, u, 480, 270, kernel=kernel)
    assert_same_frame(o, g)
    _totals_match(o, g)
    assert (o["cast"] > 1).sum() > 0  # local lights are cast


@pytest.mark.parametrize("kernel", KERNELS)
def test_fast_mode_images_are_exact(cuda, oracle, full_world, kernel):
    """Without step outputs every kernel ends rays that cannot hit early: the image, rays,
    hits and pixels stay exactly the oracle's; with exact_steps the steps do too."""
    sc = full_world
    o = oracle.render(sc.words, sc.W, sc.H, sc.uniforms, 480, 270)
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, 480, 270, kernel=kernel, debug=False)
    assert np.array_equal(g["rgba"], o["rgba"])
    t = o["totals"]
    assert [int(v) for v in g["stats"][[0, 2, 3]]] == [t["rays"], t["hits"], t["pixels"]]
    assert int(g["stats"][vrt.STAT_STEPS]) < t["steps"]  # rays that cannot hit ended early
    e = gpu_render(w, sc.uniforms, 480, 270, kernel=kernel, debug=False, exact_steps=1)
    assert np.array_equal(e["rgba"], o["rgba"]) and int(e["stats"][vrt.STAT_STEPS]) == t["steps"]


def test_full_world_1080p_rows(cuda, oracle, full_world):
    """The full 1920x1080 frame on the GPU; every 24th row checked against the oracle."""
    sc = full_world
    o = oracle.render(sc.words, sc.W, sc.H, sc.uniforms, 1920, 1080, rows=(5, 1080, 24))
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, 1920, 1080, kernel=vrt.KERNEL_BITMASK)
    assert_same_frame(o, g, rows=slice(5, 1080, 24))
    g2 = gpu_render(w, sc.uniforms, 1920, 1080, kernel=vrt.KERNEL_WORD)
    for key in ("rgba", "hit", "cast", "occ", "steps"):
        assert np.array_equal(g[key], g2[key]), key


def test_reference_scene_with_depth_field(cuda, oracle):
    """The reference world (initVoxels + fixDepthField, built on the device), the word
    kernel against the reference shader's own golden outputs and the oracle."""
    gold = load_golden("reference_world.json")
    case = load_golden("shader_reference_scene.npz")
    w = vrt.World(512, 96)
    w.init_reference()
    w.fix_depth_field()
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    import hashlib
    assert hashlib.sha256(words.tobytes()).hexdigest() == gold["depth_field"]["sha256"]
    assert w.info().has_depth_field == 1
    import json
    from helpers import uniforms_from_dict
    u = uniforms_from_dict(json.loads(str(case["uniforms"])))
    g = gpu_render(w, u, 800, 600)  # AUTO picks the word kernel for a depth-field world
    px, py = case["px"], case["py"]
    assert np.array_equal(g["hit"][py, px], case["hit"])
    assert np.array_equal(g["steps"][py, px], case["steps"])
    col = fcolor_from_outputs(words, g["hit"][py, px], g["shade"][py, px])
    assert (col.view(np.uint32) == case["color_bits"][:, :3]).all()
    o = oracle.render(words, 512, 96, u, 800, 600)
    assert_same_frame(o, g)
    with pytest.raises(vrt.VrtError) as e:
        gpu_render(w, u, 64, 48, kernel=vrt.KERNEL_BITMASK)
    assert e.value.status == vrt.ESTATE


def test_reference_world_without_depth_field(cuda, oracle):
    """The reference world before fixDepthField: both kernels, the reference camera."""
    w = vrt.World(512, 96)
    w.init_reference()
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    u = scenes.reference_scene_uniforms(-45.0)
    for i, p in enumerate([(190.0, 45.0, 170.0), (200.0, 44.0, 160.0), (210.0, 50.0, 150.0)]):
        u.localLights[i][:] = [*p, 0.5]
    o = oracle.render(words, 512, 96, u, 400, 300)  # default aspect 800/600 == 400/300
    for k in KERNELS:
        assert_same_frame(o, gpu_render(w, u, 400, 300, kernel=k))


def test_tile_shapes_and_refill_are_invisible(cuda, oracle, small):
    sc = small
    o = oracle.render(sc.words, sc.W, sc.H, sc.uniforms, sc.width, sc.height)
    w = make_world(sc.words, sc.W, sc.H)
    for tile in [(8, 4), (16, 8), (32, 1), (8, 8), (5, 3)]:
        for refill in (1, 8, 24, 32):
            g = gpu_render(w, sc.uniforms, sc.width, sc.height, kernel=vrt.KERNEL_BITMASK, tile=tile,
                           refill_min=refill)
            assert_same_frame(o, g)


def test_tile_kernel_tile_shapes_are_invisible(cuda, oracle, full_world):
    sc = full_world
    u = sc.uniforms
    o = oracle.render(sc.words, sc.W, sc.H, u, 200, 113)
    w = make_world(sc.words, sc.W, sc.H)
    for tile in [(16, 8), (32, 4), (8, 16), (8, 4), (32, 1), (8, 8), (64, 2), (128, 1)]:
        g = gpu_render(w, u, 200, 113, kernel=vrt.KERNEL_MASK_PIXEL, tile=tile)
        assert_same_frame(o, g)
    with pytest.raises(vrt.VrtError):
        gpu_render(w, u, 16, 16, kernel=vrt.KERNEL_MASK_PIXEL, tile=(5, 3))


def test_word_kernel_pixel_tiles_are_invisible(cuda, oracle, full_world):
    sc = full_world
    u = sc.uniforms
    o = oracle.render(sc.words, sc.W, sc.H, u, 200, 113)
    w = make_world(sc.words, sc.W, sc.H)
    for tile in [(16, 8), (8, 4), (32, 1), (1, 32), (16, 4), (64, 2), (96, 1)]:
        assert_same_frame(o, gpu_render(w, u, 200, 113, kernel=vrt.KERNEL_WORD, tile=tile))
    for bad in [(5, 3), (16, 16)]:
        with pytest.raises(vrt.VrtError):
            gpu_render(w, u, 16, 16, kernel=vrt.KERNEL_WORD, tile=bad)


@pytest.mark.parametrize("dims", [(37, 21), (70, 65), (130, 8)])
def test_odd_world_sizes_random_voxels(cuda, oracle, dims):
    """World sizes that are not multiples of the brick/region/super sizes, dense noise."""
    W, H = dims
    rng = np.random.default_rng(W * 1000 + H)
    words = np.where(rng.random(W * H * W) < 0.08, 0x01000000 | rng.integers(0, 1 << 24, W * H * W), -1).astype(np.int32)
    u = vrt.default_uniforms()
    u.camPos[:] = [W * 0.43, H * 0.61, W * 0.37]
    u.rotateMatrix[:] = vrt.rotate_matrix(0.3, 2.2)
    u.lightPos[:] = [W * 0.5, H * 4.0, W * 0.2]
    u.maxSteps = 3 * W
    u.localLightDist = float(W)
    for i in range(5):
        u.localLights[i][:] = [W * (0.1 + 0.17 * i), H * 0.5, W * (0.8 - 0.13 * i), 0.3]
    u.aspectRatio = 97 / 61
    o = oracle.render(words, W, H, u, 97, 61)
    w = make_world(words, W, H)
    for k in KERNELS:
        assert_same_frame(o, gpu_render(w, u, 97, 61, kernel=k))


def test_empty_and_full_worlds(cuda, oracle):
    for fill in (-1, 0x01ABCDEF):
        words = np.full(64 * 64 * 64, fill, np.int32)
        u = vrt.default_uniforms()
        u.camPos[:] = [30.5, 20.5, 10.5]
        u.maxSteps = 100
        o = oracle.render(words, 64, 64, u, 33, 17)
        w = make_world(words, 64, 64)
        for k in KERNELS:
            assert_same_frame(o, gpu_render(w, u, 33, 17, kernel=k))


def test_render_to_host(cuda, small):
    sc = small
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, sc.uniforms, sc.width, sc.height)
    r = vrt.Renderer()
    host = np.zeros(sc.width * sc.height * 4, np.uint8)
    r.render_to_host(w, sc.uniforms, sc.width, sc.height, host.ctypes.data)
    assert np.array_equal(host.reshape(sc.height, sc.width, 4), g["rgba"])


@pytest.mark.parametrize("kernel", KERNELS)
def test_render_to_host_direct(cuda, small, kernel):
    """Page-locked host memory is written by the kernel itself (no staging, no copy): the
    image equals the device render's, also at an offset into the allocation.  A buffer
    that is not 4-byte aligned goes through the staged copy; vrt_render refuses it."""
    import torch
    sc = small
    width, height = 150, 90
    u = sc.uniforms
    u.aspectRatio = width / height
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, u, width, height, kernel=kernel)["rgba"]
    n = width * height * 4
    host = torch.zeros(n + 64, dtype=torch.uint8, pin_memory=True)
    o = vrt.RenderOpts()
    o.kernel = kernel
    r = vrt.Renderer()
    for off in (0, 16, 1, 3):  # 1 and 3: unaligned, staged
        host.fill_(7)
        r.render_to_host(w, u, width, height, host.data_ptr() + off, o)
        out = host.numpy()
        assert np.array_equal(out[off:off + n].reshape(height, width, 4), g), off
        assert (out[:off] == 7).all() and (out[off + n:] == 7).all(), off  # nothing outside the image
    with pytest.raises(vrt.VrtError) as e:
        r.render(w, u, width, height, host.data_ptr() + 2, None, 0, o)
    assert e.value.status == vrt.EINVAL
    host.fill_(0)  # the device stores into page-locked memory through vrt_render too
    r.render(w, u, width, height, host.data_ptr(), None, 0, o)
    torch.cuda.synchronize()
    assert np.array_equal(host.numpy()[:n].reshape(height, width, 4), g)


@pytest.mark.parametrize("bands", [0, 1, 2, 3, 5, 8, 64])
def test_render_to_host_in_bands(cuda, small, bands):
    """The banded host render (each band's copy overlapping the next band's render) gives
    the plain render's image, also when the last ray tile row is partly outside the image."""
    sc = small
    width, height = 200, 250
    u = sc.uniforms
    u.aspectRatio = width / height
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, u, width, height, kernel=vrt.KERNEL_MASK_PIXEL)
    r = vrt.Renderer()
    import torch
    host = torch.zeros(width * height * 4, dtype=torch.uint8, pin_memory=True)
    o = vrt.RenderOpts()
    o.host_bands = bands
    for _ in range(2):  # the renderer's copy stream and events are reused
        host.zero_()
        r.render_to_host(w, u, width, height, host.data_ptr(), o)
        assert np.array_equal(host.numpy().reshape(height, width, 4), g["rgba"])


def test_bad_arguments_fail_loudly(cuda, small):
    sc = small
    w = make_world(sc.words, sc.W, sc.H)
    r = vrt.Renderer()
    with pytest.raises(vrt.VrtError):
        r.render(w, sc.uniforms, 0, 10, 1234)
    with pytest.raises(vrt.VrtError):
        vrt.World(0, 5)
    u = vrt.default_uniforms()
    u.maxSteps = -1
    with pytest.raises(vrt.VrtError):
        gpu_render(w, u, 8, 8)
    u.maxSteps = (1 << 24) + 1  # beyond what the shader's float distance counter can reach
    for k in (vrt.KERNEL_WORD, vrt.KERNEL_MASK_PIXEL):
        with pytest.raises(vrt.VrtError) as e:
            gpu_render(w, u, 8, 8, kernel=k)
        assert e.value.status == vrt.EINVAL


@pytest.mark.parametrize("radius, intensity, limit", [(6.0, 1.0, 1.25), (16.0, 3.0, 1.3), (3.0, 2.0, 1.25)])
def test_local_light_radius_and_overbright(cuda, oracle, radius, intensity, limit):
    """Lights near the surface with small radii: neighbouring pixels see different lights
    in range, and with strong lights the overbright clamp falls after different lights."""
    W, H, seed = 128, 64, 31
    words = vrt.terrain_generate(W, H, seed, 0)
    rng = scenes.SplitMix64(seed)
    u = scenes.base_uniforms(192, 128, 256, 70.0, radius)
    scenes.set_lights(u, scenes.place_lights(rng, W, seed, 16), intensity)
    scenes.aim(u, scenes.surface_camera(rng, W, seed, above=12.0), rng.uniform(0.0, 360.0), -35.0)
    u.lightPos[:] = scenes.sun_position(rng, W, H)
    u.maxOverbright = limit
    u.aspectRatio = 192 / 128
    o = oracle.render(words, W, H, u, 192, 128)
    assert ((o["cast"] >> 1) != 0).sum() > 40
    w = make_world(words, W, H)
    for k in KERNELS:
        assert_same_frame(o, gpu_render(w, u, 192, 128, kernel=k))
        g = gpu_render(w, u, 192, 128, kernel=k, debug=False)  # inexact launch: images and ray counts
        assert np.array_equal(o["rgba"], g["rgba"])
        assert int(g["stats"][vrt.STAT_RAYS]) == o["totals"]["rays"]


def test_host_alloc_and_pageable_bands(cuda, small):
    """vrt_host_alloc gives page-locked memory the banded copies run into; a pageable
    buffer (whose copies block the caller) gets the same image."""
    import ctypes as C
    sc = small
    width, height = 160, 300
    u = sc.uniforms
    u.aspectRatio = width / height
    w = make_world(sc.words, sc.W, sc.H)
    g = gpu_render(w, u, width, height, kernel=vrt.KERNEL_MASK_PIXEL)
    r = vrt.Renderer()
    o = vrt.RenderOpts()
    o.host_bands = 4
    p = C.c_void_p()
    vrt.check(vrt.lib().vrt_host_alloc(width * height * 4, C.byref(p)))
    assert p.value
    try:
        pinned = np.ctypeslib.as_array((C.c_uint8 * (width * height * 4)).from_address(p.value))
        r.render_to_host(w, u, width, height, p.value, o)
        assert np.array_equal(pinned.reshape(height, width, 4), g["rgba"])
    finally:
        vrt.check(vrt.lib().vrt_host_free(p))
    pageable = np.zeros(width * height * 4, np.uint8)
    r.render_to_host(w, u, width, height, pageable.ctypes.data, o)
    assert np.array_equal(pageable.reshape(height, width, 4), g["rgba"])
    q = C.c_void_p(1)
    vrt.check(vrt.lib().vrt_host_alloc(0, C.byref(q)))
    assert not q.value and vrt.lib().vrt_host_free(None) == 0
