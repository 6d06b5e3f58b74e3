"""Generate the golden vectors under tests/golden/ from the reference's own code.

Runs only where the reference checkout exists (it builds oracle/_ref/ from it with
oracle/ref/build_ref.sh).  Everything written here comes from executing the
reference's code, never from the oracle:
  - reference_world.json  sha256 and counts of initVoxels (level.cpp:82-138), of the
                          full fixDepthField pass (render.cpp:226-286), and of the world
                          after a sequence of removeSphere edits (level.cpp:30-56);
                          placeLocalLight slot tables (render.cpp:375-385); lightPos
                          and lightRotation after runs of lightUpdate (render.cpp:388-402).
  - shader_reference_scene.npz  the reference fragment shader (src/fshader.glsl compiled
                          as C++ against its vendored GLM) on a pixel subset of the
                          reference scene: 512x96x512 initVoxels world with its depth
                          field, camPos (195,55,155), light startLightPos rotated -45 deg,
                          800x600, RENDER_DIST 384, three local lights.
  - shader_terrain64.npz  the same shader on a 64^3 seeded terrain world (world size,
                          RENDER_DIST 256 and LOCAL_LIGHT_DIST 32 set through the
                          harness), tilted camera, global light plus local lights.
  - terrain.json          not from the reference: a determinism pin of the seeded terrain
                          generator (hash of a 64^3 world, a few column heights), so a
                          build on another CPU that produced other words is caught.
Inputs (uniform floats, pixel lists) are stored with the outputs, so the tests do not
recompute them.  Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "voxel-rt_gb300"))

import vrt_oracle as O  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# the removeSphere sequence applied to the depth-field world (centre, radius)
EDITS = [((195, 40, 170), 7), ((3, 30, 200), 5), ((510, 35, 5), 8), ((100, 94, 100), 4), ((256, 20, 256), 1),
         ((300, 36, 301), 0), ((60, 45, 75), 6)]

# placeLocalLight calls (x, y, z, a); negative coordinates leave a slot free
# lightUpdate runs: (fps, lightRotation at the start, calls).  The app starts at -45
# degrees (main.cpp:36); 170 degrees crosses the fast night branch and wraps past 360.
LIGHT_UPDATES = [(60, -45.0, 1), (60, -45.0, 600), (2, -45.0, 1000), (1, 170.0, 400), (144, 359.9, 50)]
LIGHT_CALLS = [(10.0, 40.0, 10.0, 0.5), (-1.0, 5.0, 5.0, 0.5), (20.0, 41.5, 30.0, 0.7)] + \
              [(float(i), 45.0, float(2 * i), 0.5) for i in range(16)]


def light_cases(L):
    out = []
    L.vrt_ref_init_local_lights()
    buf = np.zeros(64, np.float32)
    for call in LIGHT_CALLS:
        L.vrt_ref_place_local_light(*[C.c_float(v) for v in call])
        L.vrt_ref_get_local_lights(buf.ctypes.data)
        out.append(buf.copy().tolist())
    return out


def uniforms_dict(cam, light, aspect, rot, lights64, render_dist, local_dist):
    return {"camPos": [float(v) for v in cam], "lightPos": [float(v) for v in light], "aspectRatio": float(aspect),
            "rotateMatrix": [float(v) for v in rot], "localLights": np.asarray(lights64, np.float32).reshape(16, 4).tolist(),
            "maxSteps": int(render_dist), "localLightDist": float(local_dist)}


def run_shader_case(words, W, H, u, width, height, px, py, path):
    color, hit, steps = O.ref_shader_run(words, W, H, u["maxSteps"], int(u["localLightDist"]), u["camPos"],
                                         u["lightPos"], np.float32(u["aspectRatio"]), u["rotateMatrix"], 0,
                                         u["localLights"], width, height, px, py)
    np.savez_compressed(path, px=px.astype(np.int32), py=py.astype(np.int32), color_bits=color.view(np.uint32),
                        hit=hit, steps=steps, uniforms=json.dumps(u), width=width, height=height, W=W, H=H,
                        world_sha256=sha(words))
    return color, hit, steps


def main():
    if not O.build_ref():
        print("reference checkout not found: nothing generated", file=sys.stderr)
        return 2
    L = O.ref_world()
    W, H = L.vrt_ref_width(), L.vrt_ref_height()
    gold = {"width": W, "height": H}

    L.vrt_ref_init_world()
    w = O.ref_words_view()
    gold["init_voxels"] = {"sha256": sha(w), "solid": int((w >= 0).sum()), "air": int((w == -1).sum())}
    L.vrt_ref_fix_depth_field_all()
    w = O.ref_words_view()
    depth_world = w.copy()
    gold["depth_field"] = {"sha256": sha(w), "depth_words": int((w < -1).sum()), "plain_air": int((w == -1).sum()),
                           "hist": {str(float(v)): int(c) for v, c in
                                    zip(*np.unique(w[w < -1].view(np.float32), return_counts=True))}}
    seq = []
    for (c, r) in EDITS:
        L.vrt_ref_remove_sphere(c[0], c[1], c[2], r)
        seq.append({"center": list(c), "radius": r, "sha256": sha(O.ref_words_view())})
    gold["remove_sphere"] = seq
    gold["place_local_light"] = {"calls": [list(c) for c in LIGHT_CALLS], "tables": light_cases(L)}
    lp = np.zeros(3, np.float32)
    L.vrt_ref_light_pos(C.c_float(-45.0), lp.ctypes.data)
    gold["light_pos_minus45"] = [float(v) for v in lp]
    # the reference's own lightUpdate (float glm::rotate about +z), from the app's start
    # (-45 degrees) at 60 fps, over many frames, and across the fast night branch and the wrap
    L.vrt_ref_light_update.argtypes = [C.c_longlong, C.c_float, C.c_int, C.c_void_p]
    seq = []
    for (frame_rate, start, calls) in LIGHT_UPDATES:
        out = np.zeros(4, np.float32)
        L.vrt_ref_light_update(frame_rate, start, calls, out.ctypes.data)
        seq.append({"fps": frame_rate, "start_deg": start, "calls": calls,
                    "light_pos_bits": [int(v) for v in out[:3].view(np.uint32)],
                    "rotation_bits": int(out[3:].view(np.uint32)[0])})
    gold["light_update"] = seq
    rot = np.zeros(16, np.float32)
    L.vrt_ref_rotate_matrix(C.c_float(0.3), C.c_float(-1.1), rot.ctypes.data)
    gold["rotate_matrix_0.3_-1.1"] = [float(v) for v in rot]
    with open(os.path.join(HERE, "reference_world.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)

    # ---- shader: the reference scene (depth-field world, word kernel territory)
    lights = np.tile(np.array([-1, -1, -1, 0], np.float32), (16, 1))
    for i, (x, y, z) in enumerate([(190.0, 45.0, 170.0), (200.0, 44.0, 160.0), (210.0, 50.0, 150.0)]):
        lights[i] = [x, y, z, 0.5]
    ident = np.eye(4, dtype=np.float32).reshape(16)
    u = uniforms_dict([195, 55, 155], lp, np.float32(800.0 / 600.0), ident, lights, 384, 64)
    py, px = np.mgrid[0:600:5, 0:800:5]
    run_shader_case(depth_world, W, H, u, 800, 600, px.ravel(), py.ravel(),
                    os.path.join(HERE, "shader_reference_scene.npz"))

    # ---- shader: a 64^3 seeded terrain (mask kernel territory)
    import vrt
    vrt_lib_ok = os.path.exists(vrt.LIB_PATH)
    if not vrt_lib_ok:
        import build as vbuild
        vbuild.build()
    t64 = vrt.terrain_generate(64, 64, 12345, 4)
    lights = np.tile(np.array([-1, -1, -1, 0], np.float32), (16, 1))
    spots = [(20.5, 38.5, 22.5, 0.9), (40.5, 35.5, 30.5, 0.6), (31.5, 42.5, 45.5, 0.75), (10.5, 30.5, 50.5, 0.5)]
    for i, s in enumerate(spots):
        lights[i] = s
    rot = np.array(vrt.rotate_matrix(0.35, math.radians(40.0)), np.float32)
    sun = np.array([32.0, 32.0, 32.0], np.float32) + np.float32(192.0) * np.array([0.3, 0.8, 0.52], np.float32)
    u = uniforms_dict([32.0, 48.0, 32.0], sun, np.float32(1.0), rot, lights, 256, 32)
    py, px = np.mgrid[0:256:2, 0:256:2]
    run_shader_case(t64, 64, 64, u, 256, 256, px.ravel(), py.ravel(), os.path.join(HERE, "shader_terrain64.npz"))
    with open(os.path.join(HERE, "terrain.json"), "w") as f:
        json.dump({"64x64_seed12345_sha256": sha(t64),
                   "heights_512_seed7": [vrt.terrain_height(512, 7, x, z) for x, z in
                                         [(0, 0), (100, 37), (511, 511), (256, 128), (3, 400)]]}, f, indent=1)
    print("golden vectors written to", HERE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
