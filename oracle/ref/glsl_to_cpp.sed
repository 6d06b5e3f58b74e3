# Mechanical GLSL 4.30 -> C++/GLM edits applied to the reference's src/fshader.glsl at
# build time.  The output goes to oracle/_ref/ only; the shader source is never copied
# into the repository.  Every edit keeps the arithmetic of the shader unchanged:
#  - drop the #version line;
#  - world size and ray caps become mutable ints so the harness can set them per world;
#  - the SSBO block becomes a pointer to the caller's words;
#  - in/out/uniform qualifiers become file statics;
#  - ivec3 - vec3 (implicit in GLSL) gets an explicit vec3() conversion;
#  - max(0, float) gets a float literal (GLM's max wants one type);
#  - the .xyz swizzle becomes a vec3() conversion;
#  - main() is renamed, and the primary hit index is copied out for comparison.
/^#version/d
s/^const int \(VOXELS_WIDTH\|VOXELS_HEIGHT\|RENDER_DIST\|LOCAL_LIGHT_DIST\)=/static int \1=/
/^layout(std430/,/^};/c\
static const int* voxels;
s/^in vec4 vPos;/static vec4 vPos;/
s/^out vec4 fColor;/static vec4 fColor;/
s/^uniform /static /
s/(currCheck + forwardSteps - startPosition)/(vec3(currCheck + forwardSteps) - startPosition)/
s/max(0, /max(0.0f, /
s/localLights\[i\]\.xyz/vec3(localLights[i])/g
s/^void main(){/void shader_main(){/
s/int fColorIndex=castRay(camPos, rotatedDir, RENDER_DIST);/& g_primaryHit=fColorIndex;/
