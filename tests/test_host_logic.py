"""Host-side logic that needs no GPU: the occupancy-layout model used by the GPU tests,
the uniform helpers of the C ABI, and the seeded scene builders."""
import math
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

from helpers import expected_distances, expected_distances_brute, expected_masks, expected_masks_loops


def test_mask_layout_model_matches_loops():
    rng = np.random.default_rng(3)
    for W, H in [(20, 9), (64, 64), (70, 66)]:
        words = np.where(rng.random(W * H * W) < 0.01, 5, -1).astype(np.int32)
        for a, b in zip(expected_masks(words, W, H), expected_masks_loops(words, W, H)):
            assert np.array_equal(a, b)


def test_distance_field_model_matches_brute_force():
    # a few solid voxels in a tiny world: the summed-area model of the directed brick
    # distances and the region distances equals the pairwise minimum
    rng = np.random.default_rng(8)
    W, H = 24, 12
    words = np.where(rng.random(W * H * W) < 0.0015, 5, -1).astype(np.int32)
    words[0] = 7
    bd, rd = expected_distances(words, W, H)
    bb, rb = expected_distances_brute(words, W, H)
    assert np.array_equal(bd, bb) and np.array_equal(rd, rb)
    assert bd.max() == 15 and (bd == 0).sum() == 8 * (expected_masks(words, W, H)[0] != 0).sum()


def test_uniform_defaults_are_the_reference_constants(vrt_lib):
    u = vrt_lib.default_uniforms()
    assert u.maxSteps == 384 and u.localLightDist == 64.0            # fshader.glsl:5,7
    assert np.float32(u.ambient) == np.float32(0.4)                   # :8
    assert np.float32(u.diffuse) == np.float32(0.8)                   # :9
    assert np.float32(u.maxOverbright) == np.float32(1.25)            # :10
    assert list(u.camPos) == [195.0, 55.0, 155.0]                     # main.cpp:26
    assert u.tanHalfFov == 1.0 and u.viewDepthField == 0
    assert all(list(u.localLights[i]) == [-1.0, -1.0, -1.0, 0.0] for i in range(16))  # render.cpp:304-311
    assert list(u.rotateMatrix) == [float(i % 5 == 0) for i in range(16)]


def test_place_local_light_fills_then_ignores(vrt_lib):
    u = vrt_lib.default_uniforms()
    slots = [vrt_lib.place_local_light(u, float(i), 1.0, 2.0, 0.5) for i in range(18)]
    assert slots == list(range(16)) + [-1, -1]
    u.localLights[5][1] = -3.0  # a slot with any negative coordinate is free again
    assert vrt_lib.place_local_light(u, 9.0, 9.0, 9.0, 0.25) == 5


def test_rotate_matrix_convention(vrt_lib):
    m = np.float32(vrt_lib.rotate_matrix(math.radians(30.0), 0.0)).reshape(4, 4).T  # row-major view
    d = m[:3, :3] @ np.float32([0.0, 0.0, 1.0])
    assert d[1] < 0  # positive camRotation.x looks down (controls.cpp:136-142)


def test_scenes_are_deterministic(vrt_lib):
    import scenes
    a, b = scenes.small(1), scenes.small(1)
    assert np.array_equal(a.words, b.words)
    assert bytes(a.uniforms) == bytes(b.uniforms)
    c = scenes.small(2)
    assert bytes(a.uniforms) != bytes(c.uniforms)
    f = scenes.full(2, W=128, H=64, width=64, height=36, max_steps=64)
    lit = [f.uniforms.localLights[i][0] >= 0 for i in range(16)]
    assert all(lit)
    v = scenes.batch_views(f, 8, seed=3)
    assert len(v) == 8 and all(240 <= h <= 1080 for _, _, h in v)


def test_scene_helpers_in_the_oracle_library_match_libvrt(vrt_lib, oracle):
    """The CPU baseline builds its scenes through the oracle library's copy of the host-only
    helpers (without loading libvrt.so): the same terrain words, uniforms and matrices."""
    import ctypes as C
    import subprocess
    import sys
    vrt = vrt_lib
    L = C.CDLL(oracle.library_path(fast=True))
    for name in vrt.HOST_FUNCTIONS:
        getattr(L, name).restype, getattr(L, name).argtypes = vrt.SIGNATURES[name]
    a = np.empty(96 * 48 * 96, np.int32)
    b = np.empty_like(a)
    assert L.vrt_terrain_generate(a.ctypes.data, 96, 48, 77, 3) == 0
    assert vrt.lib().vrt_terrain_generate(b.ctypes.data, 96, 48, 77, 2) == 0
    assert np.array_equal(a, b)
    assert L.vrt_terrain_height(512, 9, 100, 300) == vrt.lib().vrt_terrain_height(512, 9, 100, 300)
    m1, m2 = (C.c_float * 16)(), (C.c_float * 16)()
    L.vrt_rotate_matrix(0.4, -2.0, m1)
    vrt.lib().vrt_rotate_matrix(0.4, -2.0, m2)
    assert bytes(m1) == bytes(m2)
    u1, u2 = vrt.Uniforms(), vrt.Uniforms()
    L.vrt_uniforms_default(C.byref(u1))
    vrt.lib().vrt_uniforms_default(C.byref(u2))
    assert bytes(u1) == bytes(u2)
    # a fresh process builds the 1080p scene through the oracle library alone
    code = ("import sys; sys.path[:0] = [%r, %r]; import vrt, vrt_oracle, scenes; "
            "vrt.use_host_library(vrt_oracle.library_path(fast=True)); sc = scenes.full(2, W=128, H=64); "
            "import os; maps = open('/proc/self/maps').read(); print(scenes.words_hash(sc.words), "
            "'libvrt.so' in maps)") % (os.path.join(ROOT, "voxel-rt_gb300"), os.path.join(ROOT, "oracle"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120, check=True)
    h, loaded = out.stdout.split()
    import scenes
    assert h == scenes.words_hash(scenes.full(2, W=128, H=64).words) and loaded == "False"


def test_counter_hash_follows_code_not_comments(tmp_path, monkeypatch):
    """bench.py reports the issue-roofline fraction only when profiles/counters.json was
    captured on the current kernel code.  The hash it compares leaves comments and blank
    lines out, so an edited comment keeps the counters, while any change of code drops them;
    and the committed counters match the committed kernels."""
    import json
    import shutil
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import bench
    committed = bench.kernel_source_hash()
    with open(os.path.join(root, "profiles", "counters.json")) as f:
        counters = json.load(f)
    assert all(e["source_sha16"] == committed for e in counters.values())

    src = tmp_path / "voxel-rt_gb300" / "csrc"
    src.mkdir(parents=True)
    for rel in bench.COUNTER_SOURCES:
        shutil.copy(os.path.join(root, rel), tmp_path / rel)
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.kernel_source_hash() == committed
    cu = tmp_path / bench.COUNTER_SOURCES[0]
    text = cu.read_text()
    cu.write_text("// a new comment line\n\n/* and a block\n   comment */\n" + text.replace("\n", "  // note\n", 3))
    assert bench.kernel_source_hash() == committed
    cu.write_text(text.replace("__launch_bounds__(128, 7)", "__launch_bounds__(128, 8)"))
    assert bench.kernel_source_hash() != committed
