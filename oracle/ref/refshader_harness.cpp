// Test-only harness: runs the reference fragment shader (src/fshader.glsl, turned into
// C++ by glsl_to_cpp.sed at build time) once per pixel on the CPU, with the
// reference's vendored GLM supplying vec/mat arithmetic.  It produces golden vectors
// that pin the oracle (oracle/vrt_oracle.cpp); nothing in the product uses it.
#include <cstdint>
#include <cstring>

#include "glm/glm.hpp"

namespace vrt_refshader {
using namespace glm;
static int g_primaryHit = -1;
#include "fshader_glm.inc"
}  // namespace vrt_refshader

extern "C" {

// Shader constants that the build turned into variables (fshader.glsl:3-7).
int vrt_refshader_set_world(const int32_t* words, int width, int height, int render_dist, int local_light_dist) {
    using namespace vrt_refshader;
    voxels = words;
    VOXELS_WIDTH = width;
    VOXELS_HEIGHT = height;
    RENDER_DIST = render_dist;
    LOCAL_LIGHT_DIST = local_light_dist;
    return 0;
}

// Uniforms of fshader.glsl:20-26.  rot16 is column-major; lights64 is 16 x (x,y,z,w).
int vrt_refshader_set_uniforms(const float* camPos3, const float* lightPos3, float aspect, const float* rot16,
                               int viewDepth, const float* lights64) {
    using namespace vrt_refshader;
    camPos = glm::vec3(camPos3[0], camPos3[1], camPos3[2]);
    lightPos = glm::vec3(lightPos3[0], lightPos3[1], lightPos3[2]);
    aspectRatio = aspect;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) rotateMatrix[c][r] = rot16[4 * c + r];
    viewDepthField = viewDepth;
    for (int i = 0; i < MAX_LOCAL_LIGHTS; i++)
        localLights[i] = glm::vec4(lights64[4 * i], lights64[4 * i + 1], lights64[4 * i + 2], lights64[4 * i + 3]);
    return 0;
}

// One invocation per listed pixel (px[i], py[i]); py counts from the bottom row.
// Outputs per pixel: fColor (4 floats), the primary hit index, and the shader's global
// stepCount after main() (DDA iterations of every ray the pixel cast).
int vrt_refshader_run(const int32_t* px, const int32_t* py, int64_t n, int width, int height, float* color4,
                      int32_t* hit, int32_t* steps) {
    using namespace vrt_refshader;
    for (int64_t i = 0; i < n; i++) {
        hitPos = glm::vec3(0, 0, 0);       // per-invocation globals (fshader.glsl:28-31)
        hitNormal = glm::vec3(0, 0, 0);
        stepCount = 0.0f;
        g_primaryHit = -1;
        float vx = (float)(2 * px[i] + 1) / (float)width - 1.0f;
        float vy = (float)(2 * py[i] + 1) / (float)height - 1.0f;
        vPos = glm::vec4(vx, vy, 0.0f, 1.0f);
        shader_main();
        color4[4 * i + 0] = fColor.r;
        color4[4 * i + 1] = fColor.g;
        color4[4 * i + 2] = fColor.b;
        color4[4 * i + 3] = fColor.a;
        hit[i] = g_primaryHit;
        steps[i] = (int32_t)stepCount;
    }
    return 0;
}

}  // extern "C"
