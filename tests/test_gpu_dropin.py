"""The drop-in render host (voxel-rt_gb300/dropin/, the reference's render.hpp interface on
the C ABI) driven by a headless main.cpp: the reference scene before and after a
removeSphere edit, against the oracle and the reference's own world code."""
import os
import subprocess

import numpy as np
import pytest

import vrt
from helpers import assert_same_frame, load_golden

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_dropin_main_renders_the_reference_scene(cuda, oracle, tmp_path):
    pkg = os.path.join(ROOT, "voxel-rt_gb300")
    exe = str(tmp_path / "dropin_main")
    # no contracted multiply-adds (the reference's x86 build has none; g++ on Arm fuses by default)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(pkg, "dropin"),
                    os.path.join(ROOT, "tests", "dropin_main.cpp"), os.path.join(pkg, "dropin", "render_dropin.cpp"),
                    "-L" + pkg, "-lvrt", "-Wl,-rpath," + pkg, "-o", exe], check=True)
    out = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    W, H, width, height = 512, 96, 400, 300
    params = np.fromfile(tmp_path / "params.f32", np.float32)
    # the world: initVoxels + fixDepthField, then removeSphere in front of the camera
    world = oracle.init_reference(W, H)
    oracle.fix_depth_field_box(world, W, H, (0, 0, 0, W, H, W))
    u = vrt.default_uniforms()
    u.camPos[:] = list(params[0:3])
    # lightUpdate(60) once from -45 degrees: the reference's own lightPos, bit for bit
    first = [c for c in load_golden("reference_world.json")["light_update"] if c["calls"] == 1 and c["fps"] == 60][0]
    assert [int(v) for v in params[3:6].view(np.uint32)] == first["light_pos_bits"]
    u.lightPos[:] = list(params[3:6])
    u.aspectRatio = float(params[6])
    u.maxSteps = int(params[7])
    vrt.place_local_light(u, float(params[0]), float(params[1] - np.float32(1.5)), float(params[2]), 0.5)
    f0 = np.fromfile(tmp_path / "frame0.rgba", np.uint8).reshape(height, width, 4)
    o0 = oracle.render(world, W, H, u, width, height)
    assert np.array_equal(f0, o0["rgba"])
    c = [int(v) for v in params[8:11]]
    oracle.remove_sphere(world, W, H, c[0], c[1], c[2], 7, 1)
    w1 = np.fromfile(tmp_path / "world1.i32", np.int32)
    assert np.array_equal(w1, world)
    f1 = np.fromfile(tmp_path / "frame1.rgba", np.uint8).reshape(height, width, 4)
    o1 = oracle.render(world, W, H, u, width, height)
    assert np.array_equal(f1, o1["rgba"])
    assert not np.array_equal(f0, f1)  # the edit is visible
