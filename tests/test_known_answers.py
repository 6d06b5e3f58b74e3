"""Known-answer tests of castRay (fshader.glsl:59-129) and of the shading loop
(fshader.glsl:131-190) on tiny worlds: the oracle (CPU) against hand-derived answers,
and both CUDA kernels against the oracle on the same scenes (gpu)."""
import math

import numpy as np
import pytest

import vrt
from helpers import assert_same_frame, gpu_render, make_world

S = 16  # tiny world: 16 x 16 x 16


def world(solids=()):
    w = np.full(S * S * S, -1, np.int32)
    for (x, y, z) in solids:
        w[x + S * y + S * S * z] = 0x01000000 | 0x808080
    return w


def idx(x, y, z):
    return x + S * y + S * S * z


def nrm(v):
    v = np.float32(v)
    return v * (np.float32(1.0) / np.sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))


def test_hit_single_voxel(oracle):
    d = nrm([1.0, 0.01, 0.02])
    hit, hp, hn, steps = oracle.cast_ray(world([(12, 8, 8)]), S, S, [8.5, 8.5, 8.5], d, 100, 100)
    assert hit == idx(12, 8, 8)
    assert list(hn) == [-1.0, 0.0, 0.0]  # entered through the -x face
    assert steps == 4
    assert abs(hp[0] - 12.0) < 1e-5


def test_start_cell_never_tested(oracle):
    d = nrm([1.0, 0.01, 0.02])
    hit, _, _, steps = oracle.cast_ray(world([(8, 8, 8)]), S, S, [8.5, 8.5, 8.5], d, 100, 100)
    assert hit == -1 and steps == 8  # leaves the world through x = 16


def test_exact_xy_tie_steps_z_only(oracle):
    """tx == ty < tz: neither x nor y is strictly smallest, so z is stepped
    (fshader.glsl:87-104) -- and keeps being stepped, since tx == ty stays true."""
    d = nrm([1.0, 1.0, 0.5])
    hit, _, hn, steps = oracle.cast_ray(world([(0, 0, 5)]), S, S, [0.5, 0.5, 0.5], d, 100, 100)
    assert hit == idx(0, 0, 5) and steps == 5 and list(hn) == [0.0, 0.0, -1.0]


def test_zero_component_gets_stuck(oracle):
    """dir.y == 0 from a non-integer start: ty = -0.5/+0 = -inf is always the smallest,
    the y step is 0, so the ray re-tests its own cell until the cap."""
    hit, _, _, steps = oracle.cast_ray(world(), S, S, [8.5, 8.5, 8.5], [1.0, 0.0, 0.0], 50, 50)
    assert hit == -1 and steps == 50
    hit, _, _, steps = oracle.cast_ray(world([(8, 8, 8)]), S, S, [8.5, 8.5, 8.5], [1.0, 0.0, 0.0], 50, 50)
    assert hit == idx(8, 8, 8) and steps == 1  # ... and a solid start cell is hit at once


def test_nan_intersects_step_z_for_good(oracle):
    """dir = +z exactly from (8, 8, 0.5): tx = ty = (8 - 8.0) / 0 = NaN, so neither x nor y
    is ever strictly smallest (fshader.glsl:87-104) and z is stepped until the voxel.  From
    the voxel's face toward +y, the x and z intersects are NaN and the z step is 0: the
    ray re-tests the voxel it starts in and hits it."""
    hit, _, _, steps = oracle.cast_ray(world([(8, 8, 12)]), S, S, [8.0, 8.0, 0.5], [0.0, 0.0, 1.0], 50, 50)
    assert hit == idx(8, 8, 12) and steps == 12
    hit, _, _, steps = oracle.cast_ray(world([(8, 8, 12)]), S, S, [8.0, 8.001, 12.0], [0.0, 1.0, 0.0], 50, 50)
    assert hit == idx(8, 8, 12) and steps == 1


def test_step_cap_and_dist(oracle):
    d = nrm([0.3, 0.2, 1.0])
    for dist, cap, want in [(100, 3, 3), (2, 100, 2), (0, 100, 0), (100, 0, 0)]:
        hit, _, _, steps = oracle.cast_ray(world(), S, S, [2.5, 2.5, 0.5], d, dist, cap)
        assert hit == -1 and steps == want


def test_leaving_world_counts_the_step(oracle):
    d = nrm([-1.0, 0.001, 0.002])
    hit, _, _, steps = oracle.cast_ray(world(), S, S, [0.5, 8.5, 8.5], d, 100, 100)
    assert hit == -1 and steps == 1


# ---------------------------------------------------------------- whole-pixel scenes

def floor_world():
    return world([(x, 0, z) for x in range(S) for z in range(S)])


def palette_floor_world():
    """The floor with voxel (x, 0, z) coloured by i = x + 16z: red i, green 255 - i, blue
    37i mod 256, so every 8-bit channel value appears (the shader's ch / 255 scale)."""
    w = np.full(S * S * S, -1, np.int32)
    for z in range(S):
        for x in range(S):
            i = x + 16 * z
            w[idx(x, 0, z)] = 0x01000000 | (i << 16) | ((255 - i) << 8) | ((i * 37) & 255)
    return w


def down_uniforms(width=8, height=8):
    u = vrt.default_uniforms()
    u.camPos[:] = [7.3, 10.6, 7.7]
    u.rotateMatrix[:] = vrt.rotate_matrix(1.2, 0.4)  # looking down at the floor
    u.aspectRatio = width / height
    u.lightPos[:] = [8.0, 200.0, 30.0]
    u.maxSteps = 64
    u.localLightDist = 64.0
    return u


def test_overbright_break_stops_casting(oracle):
    u = down_uniforms()
    for i in range(16):
        u.localLights[i][:] = [6.0 + 0.1 * i, 3.0, 7.0, 1.0]
    out = oracle.render(floor_world(), S, S, u, 8, 8)
    hitmask = out["hit"] >= 0
    assert hitmask.sum() > 20
    # the loop clamps at 1.25 and breaks before casting every light
    assert (out["shade"][hitmask] == np.float32(1.25)).all()
    casts = np.vectorize(lambda c: bin(int(c)).count("1"))(out["cast"][hitmask])
    assert casts.max() < 17


def test_overbright_clamp_position_follows_the_shader_loop(oracle):
    # fshader.glsl:159-164: the test runs before each of the 16 iterations, so a multiplier
    # pushed over the limit by light i is clamped only if an iteration i+1 exists
    def run(idx, diffuse=None):
        u = down_uniforms(9, 7)
        for i in idx:
            u.localLights[i][:] = [6.0 + 0.1 * i, 3.0, 7.0, 4.0]
        if diffuse is not None:
            u.diffuse = diffuse
        out = oracle.render(floor_world(), S, S, u, 9, 7)
        h = out["hit"] >= 0
        assert h.sum() > 20
        return out["shade"][h], out["cast"][h]
    shade, cast = run((3, 9, 15))
    assert (shade == np.float32(1.25)).all() and (cast == 1 | (2 << 3)).all()  # 9 and 15 never cast
    shade, cast = run((14,))
    assert (shade == np.float32(1.25)).all() and (cast == 1 | (2 << 14)).all()
    shade, cast = run((15,))
    assert (shade > np.float32(1.25)).all() and (cast == 1 | (2 << 15)).all()  # no test after light 15
    shade, cast = run((), diffuse=2.0)
    assert (shade == np.float32(1.25)).all() and (cast == 1).all()


def test_palette_scene_shows_every_voxel(oracle):
    u = down_uniforms(48, 48)
    u.camPos[:] = [8.0, 12.5, 8.0]
    u.rotateMatrix[:] = vrt.rotate_matrix(1.5707, 0.0)
    out = oracle.render(palette_floor_world(), S, S, u, 48, 48)
    assert len(set(out["hit"][out["hit"] >= 0].tolist())) == 256


def test_inactive_and_far_lights_are_not_cast(oracle):
    u = down_uniforms()
    u.localLights[0][:] = [-1.0, 3.0, 7.0, 1.0]    # x < 0: inactive (fshader.glsl:167)
    u.localLights[1][:] = [6.0, -0.5, 7.0, 1.0]    # y < 0: inactive
    u.localLights[2][:] = [6.0, 3.0, 7.0, 0.5]     # active, near
    u.localLightDist = 4.0
    u.localLights[3][:] = [15.0, 14.0, 15.0, 0.5]  # active, beyond the radius
    out = oracle.render(floor_world(), S, S, u, 8, 8)
    c = out["cast"][out["hit"] >= 0]
    assert ((c & (2 << 0)) == 0).all() and ((c & (2 << 1)) == 0).all() and ((c & (2 << 3)) == 0).all()
    assert ((c & (2 << 2)) != 0).any()


def test_miss_is_background(oracle):
    u = down_uniforms()
    u.rotateMatrix[:] = vrt.rotate_matrix(-1.2, 0.4)  # looking up: nothing to hit
    out = oracle.render(floor_world(), S, S, u, 4, 4)
    assert (out["hit"] == -1).all()
    assert (out["rgba"].reshape(-1, 4) == np.array([153, 179, 204, 255], np.uint8)).all()


def test_camera_outside_world_sees_background(oracle):
    u = down_uniforms()
    u.camPos[:] = [-20.0, 5.0, 5.0]
    out = oracle.render(floor_world(), S, S, u, 4, 4)
    assert (out["hit"] == -1).all() and (out["steps"] == 1).all()


def test_depth_view(oracle):
    u = down_uniforms()
    u.viewDepthField = 1
    out = oracle.render(floor_world(), S, S, u, 4, 4)
    ps = out["primary_steps"]
    assert (out["rgba"][..., 0] == np.minimum(255, np.floor(ps / np.float32(100) * 255 + 0.5))).all()


# ---------------------------------------------------------------- the CUDA kernels on the same scenes

def kat_scenes():
    scenes = []
    u = down_uniforms(9, 7)
    for i in range(16):
        u.localLights[i][:] = [6.0 + 0.1 * i, 3.0, 7.0, 1.0]
    scenes.append(("overbright", floor_world(), u, 9, 7))
    # the overbright clamp with sparse active lights: after light 3 it falls before light 9
    # (only 3 is cast); after light 14 the shader's loop still tests at i = 15 and clamps;
    # after light 15 there is no test left and the multiplier stays above the limit
    for name, idx in (("overbright-sparse", (3, 9, 15)), ("overbright-14", (14,)), ("overbright-15", (15,))):
        u = down_uniforms(9, 7)
        for i in idx:
            u.localLights[i][:] = [6.0 + 0.1 * i, 3.0, 7.0, 4.0]
        scenes.append((name, floor_world(), u, 9, 7))
    u = down_uniforms(9, 7)
    u.diffuse = 2.0  # the global light alone passes the limit: clamped before light 0
    scenes.append(("overbright-global", floor_world(), u, 9, 7))
    u = down_uniforms(8, 8)
    u.localLights[0][:] = [-1.0, 3.0, 7.0, 1.0]
    u.localLights[2][:] = [6.0, 3.0, 7.0, 0.5]
    u.localLights[3][:] = [15.0, 14.0, 15.0, 0.5]
    u.localLightDist = 4.0
    scenes.append(("lights", floor_world(), u, 8, 8))
    u = down_uniforms(5, 5)
    u.camPos[:] = [-20.0, 5.0, 5.0]
    scenes.append(("outside", floor_world(), u, 5, 5))
    u = down_uniforms(6, 6)
    u.viewDepthField = 1
    scenes.append(("depthview", floor_world(), u, 6, 6))
    # odd image width: the centre column has vPos.x == 0, an exact zero direction component
    u = vrt.default_uniforms()
    u.camPos[:] = [8.5, 8.25, 0.5]
    u.aspectRatio = 1.0
    u.maxSteps = 40
    scenes.append(("zero-dir", world([(8, 8, 12), (3, 3, 3), (8, 1, 9)]), u, 17, 9))
    # a start on integer coordinates along zero direction components: (c - start) / 0 = 0/0,
    # NaN intersects, so neither x nor y is ever strictly smallest and z is stepped for good
    # (fshader.glsl:87-104).  The centre pixel's ray runs along +z from (8, 8, 0.5) to the
    # voxel (8, 8, 12); its shadow ray toward (8, 40, 12) has NaN x and z intersects and a
    # zero z step, so it re-tests the hit voxel itself and is occluded.
    u = vrt.default_uniforms()
    u.camPos[:] = [8.0, 8.0, 0.5]
    u.lightPos[:] = [8.0, 40.0, 12.0]
    u.aspectRatio = 17 / 9
    u.maxSteps = 40
    scenes.append(("nan-dir", world([(8, 8, 12), (8, 7, 9), (3, 3, 3)]), u, 17, 9))
    # exact ties on the diagonal
    u = vrt.default_uniforms()
    u.camPos[:] = [0.5, 0.5, 0.5]
    u.rotateMatrix[:] = vrt.rotate_matrix(-math.atan(1.0), math.radians(45.0))
    u.maxSteps = 40
    scenes.append(("ties", world([(0, 0, 5), (6, 6, 6), (4, 4, 9)]), u, 9, 9))
    # every channel value 0..255 on screen, seen from straight above
    u = down_uniforms(48, 48)
    u.camPos[:] = [8.0, 12.5, 8.0]
    u.rotateMatrix[:] = vrt.rotate_matrix(1.5707, 0.0)
    scenes.append(("palette", palette_floor_world(), u, 48, 48))
    # capped and zero-step rays
    u = down_uniforms(4, 4)
    u.maxSteps = 0
    scenes.append(("cap0", floor_world(), u, 4, 4))
    u = down_uniforms(4, 4)
    u.maxSteps = 3
    scenes.append(("cap3", floor_world(), u, 4, 4))
    return scenes


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", [vrt.KERNEL_WORD, vrt.KERNEL_BITMASK, vrt.KERNEL_MASK_PIXEL])
def test_kernels_on_known_answer_scenes(cuda, oracle, kernel):
    for name, words, u, width, height in kat_scenes():
        o = oracle.render(words, S, S, u, width, height)
        w = make_world(words, S, S)
        g = gpu_render(w, u, width, height, kernel=kernel)
        try:
            assert_same_frame(o, g)
        except AssertionError as e:
            raise AssertionError(f"scene {name}: {e}") from None


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", [vrt.KERNEL_BITMASK, vrt.KERNEL_MASK_PIXEL])
def test_fast_mode_on_known_answer_scenes(cuda, oracle, kernel):
    """Images only (rays that cannot hit may end early): still the oracle's pixels."""
    for name, words, u, width, height in kat_scenes():
        if u.viewDepthField == 1:
            continue  # the step view always counts exactly
        o = oracle.render(words, S, S, u, width, height)
        g = gpu_render(make_world(words, S, S), u, width, height, kernel=kernel, debug=False)
        assert np.array_equal(o["rgba"], g["rgba"]), f"scene {name}"
        assert int(g["stats"][vrt.STAT_RAYS]) == o["totals"]["rays"], f"scene {name}"
