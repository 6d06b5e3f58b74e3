"""Device world code against the reference's own CPU code (golden vectors) and the
oracle: initVoxels, fixDepthField, removeSphere, placeVoxel, partial uploads, and the
occupancy hierarchy staying equal to (word >= 0) after every edit."""
import hashlib

import numpy as np
import pytest

import vrt
from helpers import expected_distances, expected_masks, load_golden, make_world

pytestmark = pytest.mark.gpu


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def check_masks(w: vrt.World, words):
    b, r, s = w.masks()
    eb, er, es = expected_masks(words, w.width, w.height)
    assert np.array_equal(s, es), "super masks"
    assert np.array_equal(r, er), "region masks"
    assert np.array_equal(b, eb), "brick masks"


def check_distances(w: vrt.World, words):
    bd, rd = w.distances()
    ebd, erd = expected_distances(words, w.width, w.height)
    assert np.array_equal(rd, erd), "region distances"
    assert np.array_equal(bd, ebd), "directed brick distances"


def test_distance_fields_follow_edits(cuda, vrt_lib):
    # a world wider than twice the distance cap (48 bricks), so an edit refreshes only the
    # bricks around it: every field must still equal a from-scratch computation
    W, H = 192, 64
    rng = np.random.default_rng(12)
    words = np.where(rng.random(W * H * W) < 0.0004, 0x01102030, -1).astype(np.int32)
    w = make_world(words, W, H)
    check_distances(w, words)
    w.remove_sphere(40, 30, 40, 9, 0)
    words = w.download(np.empty_like(words))
    check_distances(w, words)
    for (x, y, z) in [(3, 3, 3), (180, 60, 7), (100, 0, 190), (96, 32, 96)]:
        w.place_voxel(x, y, z, 0x01FFFFFF)
        words[x + W * y + W * H * z] = 0x01FFFFFF
        check_distances(w, words)
    patch = np.full(150, 0x01445566, np.int32)
    first = 20 + W * 10 + W * H * 150
    w.upload(patch, first)
    words[first:first + 150] = patch
    check_distances(w, words)
    empty = make_world(np.full(64 * 64 * 64, -1, np.int32), 64, 64)
    bd, rd = empty.distances()
    assert (bd == 15).all() and (rd == 15).all()


def test_init_reference_matches_reference(cuda):
    gold = load_golden("reference_world.json")
    w = vrt.World(512, 96)
    w.init_reference()
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    assert sha(words) == gold["init_voxels"]["sha256"]
    assert w.info().has_depth_field == 0
    check_masks(w, words)


def test_depth_field_and_remove_sphere_sequence(cuda):
    gold = load_golden("reference_world.json")
    w = vrt.World(512, 96)
    w.init_reference()
    w.fix_depth_field()
    words = w.download(np.empty(512 * 96 * 512, np.int32))
    assert sha(words) == gold["depth_field"]["sha256"]
    for e in gold["remove_sphere"]:
        cx, cy, cz = e["center"]
        w.remove_sphere(cx, cy, cz, e["radius"], 1)
        words = w.download(words)
        assert sha(words) == e["sha256"], f"removeSphere({e['center']}, {e['radius']})"
    check_masks(w, words)


def test_edits_on_generated_world_match_oracle(cuda, oracle, vrt_lib):
    W, H = 128, 64
    words = vrt_lib.terrain_generate(W, H, 99, 4)
    w = make_world(words, W, H)
    ref = words.copy()
    rng = np.random.default_rng(5)
    for _ in range(12):
        cx, cy, cz = int(rng.integers(-5, W + 5)), int(rng.integers(0, H)), int(rng.integers(-5, W + 5))
        r = int(rng.integers(0, 9))
        w.remove_sphere(cx, cy, cz, r, 0)
        oracle.remove_sphere(ref, W, H, cx, cy, cz, r, 0)
    w.place_voxel(3, 4, 5, 0x01123456)
    ref[3 + W * 4 + W * H * 5] = 0x01123456
    w.place_voxel(-1, 4, 5, 0x01123456)  # ignored outside the world
    got = w.download(np.empty_like(ref))
    assert np.array_equal(got, ref)
    assert w.info().has_depth_field == 0
    check_masks(w, got)
    check_distances(w, got)


def test_partial_upload_refreshes_masks(cuda, vrt_lib):
    W, H = 64, 64
    words = vrt_lib.terrain_generate(W, H, 4, 2)
    w = make_world(words, W, H)
    patch = np.full(200, 0x01FF0000, np.int32)
    first = 5 + W * 50 + W * H * 20
    w.upload(patch, first)
    words[first:first + 200] = patch
    got = w.download(np.empty_like(words))
    assert np.array_equal(got, words)
    check_masks(w, words)
    check_distances(w, words)
    # a depth-field word raises the flag, so AUTO renders with the word kernel
    w.upload(np.array([np.float32(-3.0).view(np.int32)], np.int32), 7)
    assert w.info().has_depth_field == 1


def test_probe_save_and_load(cuda, vrt_lib, tmp_path):
    W, H = 64, 64
    words = vrt_lib.terrain_generate(W, H, 21, 2)
    w = make_world(words, W, H)
    rng = np.random.default_rng(2)
    xyz = np.stack([rng.integers(-3, W + 3, 500), rng.integers(-3, H + 3, 500), rng.integers(-3, W + 3, 500)], 1)
    xyz = xyz.astype(np.int32)
    d_xyz = cuda.tensor(xyz.ravel(), device="cuda")
    d_out = cuda.empty(500, dtype=cuda.int32, device="cuda")
    w.probe(d_xyz.data_ptr(), 500, d_out.data_ptr())
    cuda.cuda.synchronize()
    inside = (xyz >= 0).all(1) & (xyz[:, 0] < W) & (xyz[:, 1] < H) & (xyz[:, 2] < W)
    want = np.where(inside, words[np.where(inside, xyz[:, 0] + W * xyz[:, 1] + W * H * xyz[:, 2], 0)], -1)
    assert np.array_equal(d_out.cpu().numpy(), want)
    path = str(tmp_path / "world.vrtw")
    w.save(path)
    w2 = vrt.World.load(path)
    assert (w2.width, w2.height) == (W, H)
    assert np.array_equal(w2.download(np.empty_like(words)), words)
    check_masks(w2, words)
    raw = np.fromfile(path, dtype=np.int32)
    assert list(raw[:4]) == [0x57525456, 1, W, H] and np.array_equal(raw[4:], words)
