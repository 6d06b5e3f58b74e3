"""The oracle against golden vectors made by running the reference's own code
(tests/golden/make_golden.py): the shader compiled as C++ against its vendored GLM,
and level.cpp/render.cpp built with GL stubs.  CPU only."""
import hashlib
import json

import numpy as np
import pytest

from helpers import fcolor_from_outputs, load_golden, uniforms_from_dict


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def ref_gold():
    return load_golden("reference_world.json")


@pytest.fixture(scope="module")
def ref_world(oracle, ref_gold):
    w = oracle.init_reference(512, 96)
    assert sha(w) == ref_gold["init_voxels"]["sha256"]
    return w


@pytest.fixture(scope="module")
def depth_world(oracle, ref_world, ref_gold):
    w = ref_world.copy()
    oracle.fix_depth_field_box(w, 512, 96, (0, 0, 0, 512, 96, 512))
    return w


def test_init_voxels_matches_reference(ref_world, ref_gold):
    g = ref_gold["init_voxels"]
    assert int((ref_world >= 0).sum()) == g["solid"]
    assert int((ref_world == -1).sum()) == g["air"]
    # the relative-coordinate destroyVoxel calls of placeBush/placeTrunk leave the origin
    # corner as air (level.cpp:11,64)
    assert ref_world[0] == -1


def test_depth_field_matches_reference(depth_world, ref_gold):
    g = ref_gold["depth_field"]
    assert sha(depth_world) == g["sha256"]
    assert int((depth_world < -1).sum()) == g["depth_words"]
    vals, counts = np.unique(depth_world[depth_world < -1].view(np.float32), return_counts=True)
    assert {str(float(v)): int(c) for v, c in zip(vals, counts)} == g["hist"]


def test_remove_sphere_sequence_matches_reference(oracle, depth_world, ref_gold):
    w = depth_world.copy()
    for e in ref_gold["remove_sphere"]:
        cx, cy, cz = e["center"]
        oracle.remove_sphere(w, 512, 96, cx, cy, cz, e["radius"], 1)
        assert sha(w) == e["sha256"], f"after removeSphere({e['center']}, {e['radius']})"


def _check_shader_case(oracle, words, case):
    u = uniforms_from_dict(json.loads(str(case["uniforms"])))
    width, height = int(case["width"]), int(case["height"])
    W, H = int(case["W"]), int(case["H"])
    assert sha(words) == str(case["world_sha256"])
    out = oracle.render(words, W, H, u, width, height)
    px, py = case["px"], case["py"]
    hit = out["hit"][py, px]
    steps = out["steps"][py, px]
    assert np.array_equal(hit, case["hit"]), f"{(hit != case['hit']).sum()} hit mismatches"
    assert np.array_equal(steps, case["steps"]), f"{(steps != case['steps']).sum()} step mismatches"
    col = fcolor_from_outputs(words, hit, out["shade"][py, px])
    gold = case["color_bits"][:, :3]
    same = (col.view(np.uint32) == gold).all(1)
    assert same.all(), f"{(~same).sum()} of {same.size} fColor values differ"
    return out


def test_shader_reference_scene_bit_exact(oracle, depth_world):
    """Reference world with its depth field: jumps, 3 local lights, global light."""
    case = load_golden("shader_reference_scene.npz")
    out = _check_shader_case(oracle, depth_world, case)
    assert (out["hit"] >= 0).sum() > 1000 and (out["cast"] > 1).sum() > 100


def test_shader_terrain64_bit_exact(oracle, vrt_lib):
    case = load_golden("shader_terrain64.npz")
    words = vrt_lib.terrain_generate(64, 64, 12345, 4)
    out = _check_shader_case(oracle, words, case)
    assert (out["occ"] != 0).sum() > 100  # shadows are exercised


def test_place_local_light_matches_reference(vrt_lib, ref_gold):
    """The library's placeLocalLight (host) against render.cpp:375-385 run natively."""
    g = ref_gold["place_local_light"]
    u = vrt_lib.default_uniforms()
    for call, table in zip(g["calls"], g["tables"]):
        vrt_lib.place_local_light(u, *call)
        got = [u.localLights[i][c] for i in range(16) for c in range(4)]
        assert np.array_equal(np.float32(got), np.float32(table))


def test_camera_and_light_helpers_match_reference(vrt_lib, ref_gold):
    import scenes
    m = np.float32(vrt_lib.rotate_matrix(0.3, -1.1))
    assert np.allclose(m, np.float32(ref_gold["rotate_matrix_0.3_-1.1"]), atol=2e-6)
    lp = np.float32(list(scenes.reference_scene_uniforms(-45.0).lightPos))
    assert np.allclose(lp, np.float32(ref_gold["light_pos_minus45"]), rtol=2e-6)


def test_terrain_generator_is_deterministic(vrt_lib):
    g = load_golden("terrain.json")
    assert sha(vrt_lib.terrain_generate(64, 64, 12345, 3)) == g["64x64_seed12345_sha256"]
    hs = [vrt_lib.terrain_height(512, 7, x, z) for x, z in [(0, 0), (100, 37), (511, 511), (256, 128), (3, 400)]]
    assert hs == g["heights_512_seed7"]
