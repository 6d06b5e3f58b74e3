// A headless main.cpp on the drop-in render host: the reference's frame loop
// (main.cpp:58-73) with glDrawArrays replaced by drawFrame().  It renders the reference
// scene, then destroys a sphere on the terrain in view (doDestroy, controls.cpp:100-110)
// and renders again, writing both frames and the edited world to the output directory.
#include <cstdio>
#include <cstring>
#include <string>

#include "render_dropin.hpp"

using namespace vrtdrop;

static bool dump(const std::string& path, const void* p, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(p, 1, n, f) == n;
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
    const std::string out = argc > 1 ? argv[1] : ".";
    if (initRender(512, 96, 1) != 0) {
        std::fprintf(stderr, "initRender: %s\n", vrtLastError());
        return 1;
    }
    reshape(400, 300);
    lightUpdate(60.0f);
    placeLocalLight(camPos.x, camPos.y - 1.5f, camPos.z, 0.5f);  // the T key, controls.cpp:46-49
    updateUniforms();
    const uint8_t* f0 = drawFrame();
    if (!f0 || !dump(out + "/frame0.rgba", f0, (size_t)screenWidth * screenHeight * 4)) return 2;
    // doDestroy (removeSphere(center, 7)) aimed at the grass surface 30 voxels ahead
    const ivec3 c{(int)camPos.x, 36, (int)(camPos.z + 30.0f)};
    removeSphere(c, 7);
    updateUniforms();
    const uint8_t* f1 = drawFrame();
    if (!f1 || !dump(out + "/frame1.rgba", f1, (size_t)screenWidth * screenHeight * 4)) return 2;
    if (!dump(out + "/world1.i32", voxels, (size_t)VOXELS_WIDTH * VOXELS_HEIGHT * VOXELS_WIDTH * 4)) return 2;
    float params[11] = {camPos.x, camPos.y, camPos.z, lightPos.x, lightPos.y, lightPos.z, aspectRatio,
                        (float)RENDER_DIST, (float)c.x, (float)c.y, (float)c.z};
    if (!dump(out + "/params.f32", params, sizeof(params))) return 2;
    if (vrtStatus() != 0) {
        std::fprintf(stderr, "vrt: %s\n", vrtLastError());
        return 3;
    }
    std::printf("ok %dx%d\n", screenWidth, screenHeight);
    shutdownRender();
    return 0;
}
