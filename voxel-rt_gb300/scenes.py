"""Seeded benchmark scenes over the vrt C ABI (host only; worlds come from the C++
terrain generator, vrt_terrain_generate).

The reference has one scene: its initVoxels world (level.cpp:82-138) seen from
camPos (195,55,155) (main.cpp:26) with the sun at startLightPos rotated by -45 degrees
about +z (main.cpp:33-36, render.cpp:388-402).  The scenes below scale that path up:

  small      64x64x64 terrain, camera (32,48,32), yaw U[0,360), pitch U[-30,0] deg,
             70 deg vertical fov, 256x256, 256 steps, global light only
  full       512x256x512 terrain, 16 local lights at air voxels 2-6 above the surface,
             colours U[0.5,1]^3, radius 32, global light, camera 2 voxels above a
             surface point, 1920x1080, 1024 steps (1 primary + up to 17 shadow rays)
  batch      the full world, 64 cameras, heights log-uniform in [240,1080], aspect 4:3
             or 16:9, 0-16 of the world's lights each
  serving    worlds 256^3, 512x256x512, 1024x256x1024 (x2)
  stress     2048x256x2048, 3840x2160, 4096 steps, camera 1 voxel above the terrain at
             pitch -2 deg (grazing rays)

The global light is a point (the shader's lightPos, fshader.glsl:147) at
centre + 3W * dir, dir uniform on the upper hemisphere.  All draws come from a
splitmix64 stream, so every machine builds the same scene from the same seed.
"""
from __future__ import annotations

import math

import numpy as np

import vrt


class SplitMix64:
    def __init__(self, seed: int):
        self.s = seed & 0xFFFFFFFFFFFFFFFF

    def next(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, a: float = 0.0, b: float = 1.0) -> float:
        return a + (b - a) * ((self.next() >> 11) * (1.0 / 9007199254740992.0))

    def randint(self, a: int, b: int) -> int:
        """Integer in [a, b] inclusive."""
        return a + self.next() % (b - a + 1)


def sun_position(rng: SplitMix64, W: int, H: int):
    y = rng.uniform(0.05, 1.0)  # uniform on the upper hemisphere: y = cos(polar) uniform
    az = rng.uniform(0.0, 2.0 * math.pi)
    r = math.sqrt(max(0.0, 1.0 - y * y))
    d = (r * math.cos(az), y, r * math.sin(az))
    c = (W / 2.0, H / 2.0, W / 2.0)
    return [c[i] + 3.0 * W * d[i] for i in range(3)]


def base_uniforms(width: int, height: int, max_steps: int, fov_deg: float, light_radius: float) -> vrt.Uniforms:
    u = vrt.default_uniforms()
    u.maxSteps = max_steps
    u.localLightDist = light_radius
    u.tanHalfFov = math.tan(math.radians(fov_deg) / 2.0)
    u.aspectRatio = float(width) / float(height)
    return u


def aim(u: vrt.Uniforms, pos, yaw_deg: float, pitch_deg: float):
    """Camera at pos looking along yaw (about +y) and pitch (negative looks down)."""
    pitch_x = math.radians(-pitch_deg)  # R_x(+a) turns +z toward -y (controls.cpp:136-142)
    yaw_y = math.radians(yaw_deg)
    u.camPos[:] = [float(p) for p in pos]
    u.camRotation[:] = [pitch_x, yaw_y]
    u.rotateMatrix[:] = vrt.rotate_matrix(pitch_x, yaw_y)


def place_lights(rng: SplitMix64, W: int, seed: int, n: int = 16):
    out = []
    for _ in range(n):
        x, z = rng.randint(0, W - 1), rng.randint(0, W - 1)
        y = vrt.terrain_height(W, seed, x, z) + rng.randint(2, 6)
        col = [rng.uniform(0.5, 1.0) for _ in range(3)]
        out.append(((x + 0.5, y + 0.5, z + 0.5), col))
    return out


def set_lights(u: vrt.Uniforms, lights, intensity: float = 1.0):
    vrt.init_local_lights(u)
    for i, (p, col) in enumerate(lights[: vrt.MAX_LOCAL_LIGHTS]):
        u.localLights[i][:] = [p[0], p[1], p[2], intensity]
        u.localLightColor[i][:] = col


class Scene:
    def __init__(self, name, W, H, seed, words, uniforms, width, height, lights=None):
        self.name, self.W, self.H, self.seed = name, W, H, seed
        self.words = words
        self.uniforms = uniforms
        self.width, self.height = width, height
        self.lights = lights or []

    @property
    def workload(self) -> str:
        return (f"{self.name}: world {self.W}x{self.H}x{self.W}, {self.width}x{self.height}, "
                f"{self.uniforms.maxSteps} steps, {sum(1 for i in range(16) if self.uniforms.localLights[i][0] >= 0)} "
                f"local lights + global, seed {self.seed}")


def small(seed: int = 1, threads: int = 0) -> Scene:
    W = H = 64
    rng = SplitMix64(seed)
    words = vrt.terrain_generate(W, H, seed, threads)
    u = base_uniforms(256, 256, 256, 70.0, 64.0)
    aim(u, (32.0, 48.0, 32.0), rng.uniform(0.0, 360.0), rng.uniform(-30.0, 0.0))
    u.lightPos[:] = sun_position(rng, W, H)
    return Scene("small", W, H, seed, words, u, 256, 256)


def surface_camera(rng: SplitMix64, W: int, seed: int, above: float = 2.0, margin: float = 0.25):
    lo, hi = int(W * margin), int(W * (1.0 - margin)) - 1
    x, z = rng.randint(lo, hi), rng.randint(lo, hi)
    h = vrt.terrain_height(W, seed, x, z)
    return (x + 0.5, h + above, z + 0.5)


def full(seed: int = 2, W: int = 512, H: int = 256, width: int = 1920, height: int = 1080, max_steps: int = 1024,
         threads: int = 0, words=None) -> Scene:
    rng = SplitMix64(seed)
    if words is None:
        words = vrt.terrain_generate(W, H, seed, threads)
    lights = place_lights(rng, W, seed, 16)
    u = base_uniforms(width, height, max_steps, 70.0, 32.0)
    set_lights(u, lights)
    aim(u, surface_camera(rng, W, seed), rng.uniform(0.0, 360.0), rng.uniform(-30.0, 0.0))
    u.lightPos[:] = sun_position(rng, W, H)
    return Scene("full", W, H, seed, words, u, width, height, lights)


def stress(seed: int = 5, threads: int = 0, W: int = 2048) -> Scene:
    H = 256
    rng = SplitMix64(seed)
    words = vrt.terrain_generate(W, H, seed, threads)
    lights = place_lights(rng, W, seed, 16)
    u = base_uniforms(3840, 2160, 4096, 70.0, 32.0)
    set_lights(u, lights)
    aim(u, surface_camera(rng, W, seed, above=1.0), rng.uniform(0.0, 360.0), -2.0)
    u.lightPos[:] = sun_position(rng, W, H)
    return Scene("stress", W, H, seed, words, u, 3840, 2160, lights)


def batch_views(scene: Scene, count: int = 64, seed: int = 3, max_steps: int | None = None):
    """count cameras over scene's world: (uniforms, width, height) with log-uniform sizes."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        h = int(round(math.exp(rng.uniform(math.log(240.0), math.log(1080.0)))))
        aspect = 4.0 / 3.0 if rng.randint(0, 1) == 0 else 16.0 / 9.0
        w = max(1, int(round(h * aspect)))
        u = base_uniforms(w, h, max_steps or scene.uniforms.maxSteps, 70.0, scene.uniforms.localLightDist)
        k = rng.randint(0, 16)
        set_lights(u, scene.lights[:k])
        aim(u, surface_camera(rng, scene.W, scene.seed), rng.uniform(0.0, 360.0), rng.uniform(-30.0, 0.0))
        u.lightPos[:] = list(scene.uniforms.lightPos)
        out.append((u, w, h))
    return out


def reference_scene_uniforms(light_rotation_deg: float = -45.0) -> vrt.Uniforms:
    """The reference app's first frame: camPos (195,55,155), identity camera, the sun at
    startLightPos = (256, 1536, 256) rotated about +z (render.cpp:388-402), 800x600,
    RENDER_DIST 384."""
    u = vrt.default_uniforms()
    a = math.radians(light_rotation_deg)
    x, y, z = 256.0, 1536.0, 256.0
    u.lightPos[:] = [x * math.cos(a) - y * math.sin(a), x * math.sin(a) + y * math.cos(a), z]
    return u


def words_hash(words: np.ndarray) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(words).tobytes()).hexdigest()
