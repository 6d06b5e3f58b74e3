// Test-only link stub: lets the reference's own src/level.cpp and src/render.cpp build
// as a shared library on a machine with no OpenGL.  It supplies the globals that
// src/main.cpp defines, null GLEW function pointers and no-op GL 1.1 entry points (the
// world/edit code never calls GL), and C wrappers over initVoxels, fixDepthField,
// removeSphere, placeLocalLight and initLocalLights for golden-vector generation.
#include <cstdint>
#include <cstring>

#include "render.hpp"
#include "level.hpp"

// ---- globals of src/main.cpp:7-44 ----
long long fps = 60;
int frames;
int mouseX, mouseY;
int screenHeight = 600, screenWidth = 800;
int fullscreen = 0, vsync = 1;
bool keys[KEYS];
int viewDepthField = 0;
glm::vec3 camPos = glm::vec3(195, 55, 155);
glm::vec3 camDir = glm::vec3(0, 0, 1);
glm::vec2 camRotation = glm::vec2(0, 0);
glm::mat4 rotateMatrix = glm::mat4(1.0f);
// Built with -fno-toplevel-reorder: the guard words sit directly before voxels[] so the
// reference's unguarded read of voxels[-1] (render.cpp:237-240, index -1 for a neighbour
// outside the world) sees air.  vrt_ref_check_layout() verifies the placement.
alignas(64) int vrt_ref_guard[16];
int voxels[VOXELS_WIDTH * VOXELS_HEIGHT * VOXELS_WIDTH];
glm::vec3 startLightPos = glm::vec3((float)VOXELS_WIDTH / 2.0f, (float)VOXELS_WIDTH * 3.0f, (float)VOXELS_WIDTH / 2.0f);
glm::vec3 lightPos = startLightPos;
float aspectRatio = 800.0f / 600.0f;
float lightRotation = -45.0f;
glm::vec4 localLights[MAX_LOCAL_LIGHTS];
bool* entityMap = nullptr;

void initLocalLights();  // defined in render.cpp:304, not declared in render.hpp

// ---- GLEW entry points used by render.cpp (never called by the world code) ----
#define VRT_GLEW_NULL(T, n) T __glew##n = nullptr;
VRT_GLEW_NULL(PFNGLATTACHSHADERPROC, AttachShader)
VRT_GLEW_NULL(PFNGLBINDBUFFERPROC, BindBuffer)
VRT_GLEW_NULL(PFNGLBINDBUFFERBASEPROC, BindBufferBase)
VRT_GLEW_NULL(PFNGLBINDVERTEXARRAYPROC, BindVertexArray)
VRT_GLEW_NULL(PFNGLBUFFERDATAPROC, BufferData)
VRT_GLEW_NULL(PFNGLBUFFERSUBDATAPROC, BufferSubData)
VRT_GLEW_NULL(PFNGLCOMPILESHADERPROC, CompileShader)
VRT_GLEW_NULL(PFNGLCREATEPROGRAMPROC, CreateProgram)
VRT_GLEW_NULL(PFNGLCREATESHADERPROC, CreateShader)
VRT_GLEW_NULL(PFNGLENABLEVERTEXATTRIBARRAYPROC, EnableVertexAttribArray)
VRT_GLEW_NULL(PFNGLGENBUFFERSPROC, GenBuffers)
VRT_GLEW_NULL(PFNGLGENVERTEXARRAYSPROC, GenVertexArrays)
VRT_GLEW_NULL(PFNGLGETATTRIBLOCATIONPROC, GetAttribLocation)
VRT_GLEW_NULL(PFNGLGETPROGRAMINFOLOGPROC, GetProgramInfoLog)
VRT_GLEW_NULL(PFNGLGETPROGRAMIVPROC, GetProgramiv)
VRT_GLEW_NULL(PFNGLGETSHADERINFOLOGPROC, GetShaderInfoLog)
VRT_GLEW_NULL(PFNGLGETSHADERIVPROC, GetShaderiv)
VRT_GLEW_NULL(PFNGLGETUNIFORMLOCATIONPROC, GetUniformLocation)
VRT_GLEW_NULL(PFNGLLINKPROGRAMPROC, LinkProgram)
VRT_GLEW_NULL(PFNGLSHADERSOURCEPROC, ShaderSource)
VRT_GLEW_NULL(PFNGLUNIFORM1FPROC, Uniform1f)
VRT_GLEW_NULL(PFNGLUNIFORM1IPROC, Uniform1i)
VRT_GLEW_NULL(PFNGLUNIFORM2FPROC, Uniform2f)
VRT_GLEW_NULL(PFNGLUNIFORM3FPROC, Uniform3f)
VRT_GLEW_NULL(PFNGLUNIFORM4FVPROC, Uniform4fv)
VRT_GLEW_NULL(PFNGLUNIFORMMATRIX4FVPROC, UniformMatrix4fv)
VRT_GLEW_NULL(PFNGLUSEPROGRAMPROC, UseProgram)
VRT_GLEW_NULL(PFNGLVERTEXATTRIBPOINTERPROC, VertexAttribPointer)
extern "C" {
void GLAPIENTRY glShadeModel(GLenum) {}
void GLAPIENTRY glViewport(GLint, GLint, GLsizei, GLsizei) {}
}

extern "C" {

int vrt_ref_width(void) { return VOXELS_WIDTH; }
int vrt_ref_height(void) { return VOXELS_HEIGHT; }
int32_t* vrt_ref_words(void) { return voxels; }

// 0 when voxels[-1] is the last guard word, which then holds air (-1).
int vrt_ref_check_layout(void) {
    for (int i = 0; i < 16; i++) vrt_ref_guard[i] = -1;
    return (&voxels[-1] == &vrt_ref_guard[15]) ? 0 : -1;
}

// initRender's world set-up (render.cpp:349-352): all -1, then initVoxels().
void vrt_ref_init_world(void) {
    for (int i = 0; i < VOXELS_WIDTH * VOXELS_HEIGHT * VOXELS_WIDTH; i++) voxels[i] = -1;
    initVoxels();
}

// The depth-field pass of initRender (render.cpp:354-363 -> :273-286), every z slab,
// split over OpenMP threads instead of the reference's 4 pthreads (the slabs are
// independent: fixDepthField writes only air words and reads only solidity).
void vrt_ref_fix_depth_field_all(void) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int z = 0; z < VOXELS_WIDTH; z++)
        for (int y = 0; y < VOXELS_HEIGHT; y++)
            for (int x = 0; x < VOXELS_WIDTH; x++) fixDepthField(x, y, z);
}

void vrt_ref_remove_sphere(int x, int y, int z, int radius) { removeSphere(glm::ivec3(x, y, z), radius); }

void vrt_ref_init_local_lights(void) { initLocalLights(); }
void vrt_ref_place_local_light(float x, float y, float z, float a) { placeLocalLight(x, y, z, a); }
void vrt_ref_get_local_lights(float* out64) {
    for (int i = 0; i < MAX_LOCAL_LIGHTS; i++)
        for (int c = 0; c < 4; c++) out64[4 * i + c] = localLights[i][c];
}

// lightUpdate's light position for a given rotation in degrees (render.cpp:388-402).
void vrt_ref_light_pos(float rotation_deg, float* out3) {
    glm::mat4 rot = glm::rotate(glm::mat4(1.0f), glm::radians(rotation_deg), glm::vec3(0, 0, 1));
    glm::vec3 p = rot * glm::vec4(startLightPos, 1);
    out3[0] = p.x; out3[1] = p.y; out3[2] = p.z;
}

// The reference's own lightUpdate (render.cpp:388-402) called `calls` times at frame rate
// frame_rate, from lightRotation = start_deg: out4 = lightPos, then lightRotation.
void vrt_ref_light_update(long long frame_rate, float start_deg, int calls, float* out4) {
    fps = frame_rate;
    lightRotation = start_deg;
    for (int i = 0; i < calls; i++) lightUpdate();
    out4[0] = lightPos.x; out4[1] = lightPos.y; out4[2] = lightPos.z; out4[3] = lightRotation;
}

// rotateMatrix of doMouseLook (controls.cpp:136-142) for camRotation (x, y).
void vrt_ref_rotate_matrix(float rx, float ry, float* out16) {
    glm::mat4 rotX = glm::rotate(glm::mat4(1.0f), rx, glm::vec3(1, 0, 0));
    glm::mat4 rotY = glm::rotate(glm::mat4(1.0f), ry, glm::vec3(0, 1, 0));
    glm::mat4 m = rotY * rotX;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) out16[4 * c + r] = m[c][r];
}

}  // extern "C"
