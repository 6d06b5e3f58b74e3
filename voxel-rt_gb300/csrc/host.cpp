// Host-only entry points of the C ABI, with no CUDA dependency: error reporting, the
// version string, uniform defaults and the helpers that mirror the reference's host-side
// uniform code (render.cpp:304-311, :375-385; controls.cpp:136-142).  The seeded scenes
// are built from these and terrain.cpp alone, so a CPU-only process can build the same
// inputs without loading the CUDA library.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "vrt_host.h"

namespace vrt {

static thread_local char g_err[512] = "";

int set_error(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return status;
}

}  // namespace vrt

extern "C" {

const char* vrt_last_error(void) { return vrt::g_err; }

const char* vrt_version(void) { return "vrt-gb300 0.1 sm_103a"; }

int vrt_init_local_lights(vrt_uniforms* u) {
    if (!u) return vrt::set_error(VRT_EINVAL, "NULL uniforms");
    for (int i = 0; i < VRT_MAX_LOCAL_LIGHTS; i++) {
        u->localLights[i][0] = -1.0f;
        u->localLights[i][1] = -1.0f;
        u->localLights[i][2] = -1.0f;
        u->localLights[i][3] = 0.0f;
        u->localLightColor[i][0] = u->localLightColor[i][1] = u->localLightColor[i][2] = 1.0f;
    }
    return VRT_OK;
}

int vrt_uniforms_default(vrt_uniforms* u) {
    if (!u) return vrt::set_error(VRT_EINVAL, "NULL uniforms");
    std::memset(u, 0, sizeof(*u));
    u->camPos[0] = 195.0f; u->camPos[1] = 55.0f; u->camPos[2] = 155.0f;       // main.cpp:26
    // startLightPos = (W/2, 3W, W/2) for the reference's W = 512 (main.cpp:33-34)
    u->lightPos[0] = 256.0f; u->lightPos[1] = 1536.0f; u->lightPos[2] = 256.0f;
    u->aspectRatio = 800.0f / 600.0f;                                         // main.cpp:11-12,36
    for (int i = 0; i < 16; i++) u->rotateMatrix[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    u->viewDepthField = 0;
    vrt_init_local_lights(u);
    u->tanHalfFov = 1.0f;
    u->maxSteps = 384;          // RENDER_DIST
    u->localLightDist = 64.0f;  // LOCAL_LIGHT_DIST
    u->ambient = 0.4f;          // AMBIENT
    u->diffuse = 0.8f;          // DIFFUSE
    u->maxOverbright = 1.25f;   // MAX_OVERBRIGHT
    return VRT_OK;
}

int vrt_place_local_light(vrt_uniforms* u, float x, float y, float z, float a) {
    if (!u) return vrt::set_error(VRT_EINVAL, "NULL uniforms");
    for (int i = 0; i < VRT_MAX_LOCAL_LIGHTS; i++) {
        if (u->localLights[i][0] < 0 || u->localLights[i][1] < 0 || u->localLights[i][2] < 0) {
            u->localLights[i][0] = x;
            u->localLights[i][1] = y;
            u->localLights[i][2] = z;
            u->localLights[i][3] = a;
            return i;
        }
    }
    return VRT_MAX_LOCAL_LIGHTS;
}

int vrt_rotate_matrix(float pitch_x, float yaw_y, float* m) {
    if (!m) return vrt::set_error(VRT_EINVAL, "NULL matrix");
    // R_x(p) = [1 0 0; 0 c -s; 0 s c], R_y(q) = [c 0 s; 0 1 0; -s 0 c]; M = R_y * R_x
    double cp = std::cos((double)pitch_x), sp = std::sin((double)pitch_x);
    double cq = std::cos((double)yaw_y), sq = std::sin((double)yaw_y);
    double M[3][3] = {{cq, sq * sp, sq * cp}, {0.0, cp, -sp}, {-sq, cq * sp, cq * cp}};  // M[row][col]
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) m[4 * c + r] = (r < 3 && c < 3) ? (float)M[r][c] : (r == c ? 1.0f : 0.0f);
    return VRT_OK;
}

}  // extern "C"
