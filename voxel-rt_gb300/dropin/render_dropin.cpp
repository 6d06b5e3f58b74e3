// Drop-in render host (see render_dropin.hpp), on the C ABI of libvrt.so.
#include "render_dropin.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace vrtdrop {

int32_t* voxels = nullptr;
int VOXELS_WIDTH = 512, VOXELS_HEIGHT = 96;  // render.hpp:4-5
vec3 camPos{195.0f, 55.0f, 155.0f};          // main.cpp:26
vec2 camRotation{0.0f, 0.0f};
mat4 rotateMatrix{{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1}};
vec3 startLightPos{256.0f, 1536.0f, 256.0f};  // (W/2, 3W, W/2) for W = 512, main.cpp:33
vec3 lightPos = startLightPos;
float aspectRatio = 800.0f / 600.0f;
float lightRotation = -45.0f;                 // main.cpp:36
int viewDepthField = 0;
vec4 localLights[VRT_MAX_LOCAL_LIGHTS];
int screenWidth = 800, screenHeight = 600;    // main.cpp:11-12
int RENDER_DIST = 384;

namespace {
vrt_world* g_world = nullptr;
vrt_renderer* g_renderer = nullptr;
vrt_uniforms g_u;
std::vector<int32_t> g_mirror;
uint8_t* g_frame = nullptr;  // page-locked (vrt_host_alloc), so the frame's band copies overlap the render
size_t g_frame_bytes = 0;
int g_status = 0;

inline void note(int st) {
    if (st < 0) g_status = st;
}
}  // namespace

int vrtStatus() { return g_status; }
const char* vrtLastError() { return vrt_last_error(); }

int initRender(int width, int height, int with_reference_world) {
    shutdownRender();
    VOXELS_WIDTH = width;
    VOXELS_HEIGHT = height;
    startLightPos = vec3{width / 2.0f, width * 3.0f, width / 2.0f};
    lightPos = startLightPos;
    int st = vrt_world_create(width, height, &g_world);
    if (st == 0) st = vrt_renderer_create(&g_renderer);
    if (st == 0 && with_reference_world) {
        st = vrt_world_init_reference(g_world, nullptr);                      // initVoxels()
        if (st == 0) st = vrt_fix_depth_field_box(g_world, 0, 0, 0, width, height, width, nullptr);
    }
    g_mirror.assign((size_t)width * height * width, -1);                        // render.cpp:349-351
    if (st == 0) st = vrt_world_download(g_world, g_mirror.data(), 0, g_mirror.size(), nullptr);
    voxels = g_mirror.data();
    initLocalLights();                                                          // render.cpp:343
    vrt_uniforms_default(&g_u);
    updateUniforms();
    note(st);
    return st;
}

void shutdownRender() {
    vrt_host_free(g_frame);
    g_frame = nullptr;
    g_frame_bytes = 0;
    vrt_renderer_destroy(g_renderer);
    vrt_world_destroy(g_world);
    g_renderer = nullptr;
    g_world = nullptr;
    g_mirror.clear();
    voxels = nullptr;
}

int getVoxelIndex(int x, int y, int z) {
    if (x >= 0 && y >= 0 && z >= 0 && x < VOXELS_WIDTH && y < VOXELS_HEIGHT && z < VOXELS_WIDTH)
        return x + VOXELS_WIDTH * y + VOXELS_WIDTH * VOXELS_HEIGHT * z;
    return -1;
}

void updateGeometry() {
    note(vrt_world_upload(g_world, voxels, 0, g_mirror.size(), nullptr));
}

// render.cpp:204-223 uploads one x-row per (z, y) from start to end; rows whose start.x
// is outside the world are skipped there (an edit near x = 0 never reaches the GPU).
// Here each row is clipped to the world instead, so every edited voxel is uploaded.
void updatePartialGeometry(vec3 start, vec3 end) {
    if (getVoxelIndex((int)start.x, (int)start.y, (int)start.z) > getVoxelIndex((int)end.x, (int)end.y, (int)end.z)) {
        vec3 t = start;
        start = end;
        end = t;
    }
    int x0 = std::max(0, (int)start.x), x1 = std::min(VOXELS_WIDTH - 1, (int)start.x + (int)(end.x - start.x));
    if (x0 > x1) return;
    for (float i = start.z; i < end.z; i++)
        for (float j = start.y; j < end.y; j++) {
            const int off = getVoxelIndex(x0, (int)j, (int)i);
            if (off != -1) note(vrt_world_upload(g_world, voxels + off, (uint64_t)off, (uint64_t)(x1 - x0 + 1), nullptr));
        }
}

void placeVoxel(int x, int y, int z, int voxel) {
    const int idx = getVoxelIndex(x, y, z);
    if (idx < 0) return;
    voxels[idx] = voxel;
    note(vrt_place_voxel(g_world, x, y, z, voxel, nullptr));
}

void destroyVoxel(int x, int y, int z) {
    const int idx = getVoxelIndex(x, y, z);
    if (idx < 0) return;
    voxels[idx] = -1;
    note(vrt_place_voxel(g_world, x, y, z, -1, nullptr));
}

void fixDepthField(int x, int y, int z) {
    note(vrt_fix_depth_field_box(g_world, x, y, z, x + 1, y + 1, z + 1, nullptr));
    const int idx = getVoxelIndex(x, y, z);
    if (idx >= 0) note(vrt_world_download(g_world, voxels + idx, (uint64_t)idx, 1, nullptr));
}

// removeSphere runs on the device (scatter + mask refresh + depth-field refresh when the
// world has one); the host mirror of the touched cube is then refreshed.
void removeSphere(ivec3 pos, int radius) {
    vrt_world_info info;
    vrt_world_get_info(g_world, &info);
    note(vrt_remove_sphere(g_world, pos.x, pos.y, pos.z, radius, info.has_depth_field, nullptr));
    const int r2 = radius + (7 >> 1);
    const int x0 = std::max(0, pos.x - r2), x1 = std::min(VOXELS_WIDTH, pos.x + r2);
    if (x0 >= x1) return;
    for (int z = std::max(0, pos.z - r2); z < std::min(VOXELS_WIDTH, pos.z + r2); z++)
        for (int y = std::max(0, pos.y - r2); y < std::min(VOXELS_HEIGHT, pos.y + r2); y++) {
            const int off = getVoxelIndex(x0, y, z);
            note(vrt_world_download(g_world, voxels + off, (uint64_t)off, (uint64_t)(x1 - x0), nullptr));
        }
}

void initLocalLights() {
    for (auto& l : localLights) l = vec4{-1.0f, -1.0f, -1.0f, 0.0f};
}

void placeLocalLight(float x, float y, float z, float diffuse) {
    for (auto& l : localLights)
        if (l.x < 0 || l.y < 0 || l.z < 0) {
            l = vec4{x, y, z, diffuse};
            break;
        }
}

// lightUpdate (render.cpp:388-402): advance lightRotation and rotate startLightPos about +z,
// in float and in the order of the reference's glm::rotate(mat4(1), radians(a), (0,0,1)) *
// vec4(startLightPos, 1).  For the unit z axis that matrix has columns (c, s, 0, 0),
// (-s, c, 0, 0), (0, 0, c + (1 - c), 0) and (0, 0, 0, 1); mat4 * vec4 sums
// (m0*x + m1*y) + (m2*z + m3*w), whose zero terms drop out exactly.  Build this file
// without contracted multiply-adds (-ffp-contract=off), as the reference's x86 build has
// none, or x and y can differ in the last bit.
void lightUpdate(float fps) {
    float increment = 0.3f / fps;
    if (lightRotation >= 360.0f) lightRotation = 0.0f;
    else if (lightRotation >= 180.0f && lightRotation < 270.0f) increment *= 8.0f;
    lightRotation += increment;
    const float a = lightRotation * 0.01745329251994329576923690768489f;  // glm::radians
    const float c = std::cos(a), s = std::sin(a);
    const float czz = c + (1.0f - c);  // Rotate[2][2] = c + (1 - c) * axis.z * axis.z
    const float ns = 0.0f - s;         // Rotate[1][0] = (1 - c) * axis.y * axis.x - s * axis.z
    lightPos = vec3{c * startLightPos.x + ns * startLightPos.y, s * startLightPos.x + c * startLightPos.y,
                    czz * startLightPos.z};
}

void updateUniforms() {
    std::memcpy(g_u.camPos, &camPos, sizeof(g_u.camPos));
    std::memcpy(g_u.camRotation, &camRotation, sizeof(g_u.camRotation));
    std::memcpy(g_u.lightPos, &lightPos, sizeof(g_u.lightPos));
    g_u.aspectRatio = aspectRatio;
    std::memcpy(g_u.rotateMatrix, rotateMatrix.m, sizeof(g_u.rotateMatrix));
    g_u.viewDepthField = viewDepthField;
    for (int i = 0; i < VRT_MAX_LOCAL_LIGHTS; i++) {
        g_u.localLights[i][0] = localLights[i].x;
        g_u.localLights[i][1] = localLights[i].y;
        g_u.localLights[i][2] = localLights[i].z;
        g_u.localLights[i][3] = localLights[i].a;
    }
    g_u.maxSteps = RENDER_DIST;
}

void reshape(int width, int height) {
    screenWidth = width;
    screenHeight = height;
    aspectRatio = (float)width / height;
}

const uint8_t* drawFrame() {
    const size_t bytes = (size_t)screenWidth * screenHeight * 4;
    if (bytes > g_frame_bytes) {
        vrt_host_free(g_frame);
        g_frame = nullptr;
        g_frame_bytes = 0;
        void* p = nullptr;
        const int st = vrt_host_alloc(bytes, &p);
        note(st);
        if (st) return nullptr;
        g_frame = static_cast<uint8_t*>(p);
        g_frame_bytes = bytes;
    }
    note(vrt_render_to_host(g_renderer, g_world, &g_u, screenWidth, screenHeight, g_frame, nullptr, nullptr));
    return g_frame;
}

}  // namespace vrtdrop
