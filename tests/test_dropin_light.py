"""The drop-in host's lightUpdate (voxel-rt_gb300/dropin/render_dropin.cpp) against the
reference's own lightUpdate (render.cpp:388-402, float glm::rotate about +z), run through
oracle/_ref when the goldens were made: lightPos and lightRotation bit for bit after runs
of 1 to 1000 frames, across the fast night branch and the wrap at 360 degrees.  No GPU:
lightUpdate only does host arithmetic."""
import os
import subprocess

import numpy as np

from helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include "render_dropin.hpp"
static unsigned bits(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }
int main(int argc, char** argv) {
    for (int i = 1; i + 2 < argc; i += 3) {
        const float fps = (float)std::atoll(argv[i]);
        vrtdrop::lightRotation = std::strtof(argv[i + 1], nullptr);
        const int calls = std::atoi(argv[i + 2]);
        for (int k = 0; k < calls; k++) vrtdrop::lightUpdate(fps);
        std::printf("%u %u %u %u\n", bits(vrtdrop::lightPos.x), bits(vrtdrop::lightPos.y), bits(vrtdrop::lightPos.z),
                    bits(vrtdrop::lightRotation));
    }
    return 0;
}
"""


def test_dropin_light_update_matches_reference(tmp_path, vrt_lib):
    pkg = os.path.join(ROOT, "voxel-rt_gb300")
    src = tmp_path / "light_main.cpp"
    src.write_text(HARNESS)
    exe = str(tmp_path / "light_main")
    # no contracted multiply-adds, as in the reference's own x86 build (compile.bat)
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(pkg, "dropin"), str(src),
                    os.path.join(pkg, "dropin", "render_dropin.cpp"), "-L" + pkg, "-lvrt", "-Wl,-rpath," + pkg,
                    "-o", exe], check=True)
    cases = load_golden("reference_world.json")["light_update"]
    args = []
    for c in cases:
        args += [str(c["fps"]), repr(float(c["start_deg"])), str(c["calls"])]
    out = subprocess.run([exe] + args, capture_output=True, text=True, timeout=60, check=True).stdout.split("\n")
    for c, line in zip(cases, out):
        got = [int(v) for v in line.split()]
        want = c["light_pos_bits"] + [c["rotation_bits"]]
        assert got == want, (c, np.array(got, np.uint32).view(np.float32), np.array(want, np.uint32).view(np.float32))
