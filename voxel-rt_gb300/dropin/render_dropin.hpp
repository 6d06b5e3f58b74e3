// Drop-in replacement for the reference's render host interface (src/render.hpp:30-41
// and the globals of src/main.cpp:7-44), implemented on the GB300 C ABI (include/vrt.h).
//
// The reference's main loop calls these functions around glDrawArrays (main.cpp:58-73);
// here glDrawArrays becomes drawFrame(), which renders the frame on the GPU into a host
// RGBA8 buffer (row 0 = bottom, as glReadPixels returns it).  Names, argument meanings
// and call order follow the reference; the world size is set at initRender instead of
// by the VOXELS_WIDTH / VOXELS_HEIGHT macros, and errors are reported by return codes
// and vrtLastError() instead of exit().
//
// GLM types are replaced by the small structs below (same member names), so a host
// program can include this header without the vendored GLM.
#pragma once

#include <cstdint>

#include "../../include/vrt.h"

namespace vrtdrop {

struct vec2 { float x, y; };
struct vec3 { float x, y, z; };
struct vec4 { float x, y, z, a; };
struct ivec3 { int x, y, z; };
struct mat4 { float m[16]; };  // column-major, as glm::value_ptr(rotateMatrix)

// ---- the globals of src/main.cpp:7-44 (the shader's uniforms live here) ----
extern int32_t* voxels;         // host mirror of the world, voxels[x + W*y + W*H*z]
extern int VOXELS_WIDTH, VOXELS_HEIGHT;
extern vec3 camPos;
extern vec2 camRotation;
extern mat4 rotateMatrix;
extern vec3 startLightPos;
extern vec3 lightPos;
extern float aspectRatio;
extern float lightRotation;
extern int viewDepthField;
extern vec4 localLights[VRT_MAX_LOCAL_LIGHTS];
extern int screenWidth, screenHeight;
extern int RENDER_DIST;         // fshader.glsl:5, a run-time value here

// ---- render.hpp:30-41 ----
// initRender (render.cpp:313-372): world of width x height x width voxels, all air, then
// initVoxels (level.cpp:82-138) and the depth field (render.cpp:354-363), on the device;
// the host mirror is filled from the device.  with_reference_world = 0 leaves air.
int initRender(int width, int height, int with_reference_world);
void shutdownRender();
void updateGeometry();                                  // render.cpp:199-202
void updatePartialGeometry(vec3 start, vec3 end);       // render.cpp:204-223
int getVoxelIndex(int x, int y, int z);                 // render.cpp:189-196
void placeVoxel(int x, int y, int z, int voxel);        // render.cpp:256-262
void destroyVoxel(int x, int y, int z);                 // render.cpp:265-271
void fixDepthField(int x, int y, int z);                // render.cpp:226-253 (one voxel)
void lightUpdate(float fps);                            // render.cpp:388-402
void updateUniforms();                                  // render.cpp:289-302
void removeSphere(ivec3 pos, int radius);               // level.cpp:30-56
void reshape(int width, int height);                    // render.cpp:404-411
void placeLocalLight(float x, float y, float z, float diffuse);  // render.cpp:375-385
void initLocalLights();                                 // render.cpp:304-311

// glDrawArrays(GL_TRIANGLES, 0, 6) (main.cpp:59): one frame of screenWidth x
// screenHeight into the returned host RGBA8 buffer (page-locked; valid until the next
// call or shutdownRender; NULL if it could not be allocated).
const uint8_t* drawFrame();

int vrtStatus();                 // status of the last failing call, 0 if none
const char* vrtLastError();

}  // namespace vrtdrop
