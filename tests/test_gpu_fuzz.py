"""Randomised parity: random worlds, cameras, lights, radii, overbright limits and step
caps; every render kernel (and the inexact launches of the tile and word kernels)
against the oracle.

Each case is seeded, so a failure names a reproducible scene."""
import math

import numpy as np
import pytest

import vrt
from helpers import assert_same_frame, gpu_render, make_world

pytestmark = pytest.mark.gpu


def random_world(rng, W, H, kind, seed):
    n = W * H * W
    if kind == 0:  # sparse noise
        density = float(rng.uniform(0.002, 0.1))
        colours = 0x01000000 | rng.integers(0, 1 << 24, n)
        return np.where(rng.random(n) < density, colours, -1).astype(np.int32)
    if kind == 1:  # terrain
        return vrt.terrain_generate(W, H, seed, 0)
    words = np.full((W, H, W), -1, np.int32)  # [z][y][x]: a few axis-aligned slabs
    for _ in range(int(rng.integers(1, 5))):
        a = rng.integers(0, [W, H, W])
        b = a + rng.integers(1, [max(2, W // 2), max(2, H // 2), max(2, W // 2)])
        words[a[2]:b[2], a[1]:b[1], a[0]:b[0]] = 0x01000000 | int(rng.integers(0, 1 << 24))
    return words.reshape(-1)


def random_case(seed):
    rng = np.random.default_rng(1000 + seed)
    W = int(rng.choice([16, 24, 40, 64]))
    H = int(rng.choice([8, 16, 33, 64]))
    words = random_world(rng, W, H, seed % 3, seed)
    u = vrt.default_uniforms()
    if rng.random() < 0.2:  # outside the world: every ray misses at its first step
        u.camPos[:] = [float(rng.uniform(-8, 0)), float(rng.uniform(0, H)), float(rng.uniform(0, W))]
    else:
        u.camPos[:] = [float(rng.uniform(0, W)), float(rng.uniform(0, H)), float(rng.uniform(0, W))]
    solid = np.flatnonzero(words >= 0)
    if rng.random() < 0.25:  # identity camera: odd widths give exactly zero direction components
        u.rotateMatrix[:] = vrt.rotate_matrix(0.0, 0.0)
    elif solid.size and rng.random() < 0.7:  # look at a random solid voxel
        t = int(rng.choice(solid))
        d = np.array([t % W + 0.5, (t // W) % H + 0.5, t // (W * H) + 0.5]) - np.array(list(u.camPos))
        d /= max(np.linalg.norm(d), 1e-6)
        # forward = R_y(yaw) R_x(pitch) (0,0,1) = (sin(yaw) cos(pitch), -sin(pitch), cos(yaw) cos(pitch))
        u.rotateMatrix[:] = vrt.rotate_matrix(float(math.asin(-d[1])), float(math.atan2(d[0], d[2])))
    else:
        u.rotateMatrix[:] = vrt.rotate_matrix(float(rng.uniform(-1.5, 1.5)), float(rng.uniform(0, 2 * math.pi)))
    u.lightPos[:] = [float(rng.uniform(-W, 2 * W)), float(rng.uniform(H, 8 * H)), float(rng.uniform(-W, 2 * W))]
    u.maxSteps = int(rng.integers(0, 3 * W + 1))
    u.localLightDist = float(rng.uniform(1.0, W))
    u.maxOverbright = float(rng.uniform(1.0, 2.0))
    u.diffuse = float(rng.uniform(0.5, 2.0))
    vrt.init_local_lights(u)
    for i in range(int(rng.integers(0, 17))):
        p = [float(rng.uniform(-2, W)), float(rng.uniform(-2, H)), float(rng.uniform(-2, W))]
        u.localLights[i][:] = p + [float(rng.uniform(0.2, 3.0))]
        u.localLightColor[i][:] = [float(c) for c in rng.uniform(0.5, 1.0, 3)]
    width, height = int(rng.integers(17, 65)), int(rng.integers(9, 49))
    u.aspectRatio = width / height
    return words, W, H, u, width, height


@pytest.mark.parametrize("seed", range(24))
def test_random_scene(cuda, oracle, seed):
    words, W, H, u, width, height = random_case(seed)
    o = oracle.render(words, W, H, u, width, height)
    world = make_world(words, W, H)
    for k in (vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD, vrt.KERNEL_BITMASK):
        try:
            assert_same_frame(o, gpu_render(world, u, width, height, kernel=k))
        except AssertionError as e:
            raise AssertionError(f"seed {seed}, kernel {k}: {e}") from None
    for k in (vrt.KERNEL_MASK_PIXEL, vrt.KERNEL_WORD):  # inexact launches: rays that cannot hit end early
        g = gpu_render(world, u, width, height, kernel=k, debug=False)
        assert np.array_equal(o["rgba"], g["rgba"]), f"seed {seed}, kernel {k}: inexact launch"
        assert int(g["stats"][vrt.STAT_RAYS]) == o["totals"]["rays"]
