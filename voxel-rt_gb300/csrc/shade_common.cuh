// Device arithmetic of the fragment shader (Berry2460/voxel-rt src/fshader.glsl),
// shared by the render kernels.  Every operation is an explicit round-to-nearest
// intrinsic (1 / x included, as the correctly rounded reciprocal), so no multiply-add is
// ever contracted and the results are the IEEE binary32 values the CPU oracle computes:
//   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z
//   normalize(v) = v * (1 / sqrt(dot(v, v)))          (GLM's form)
//   length(v)    = sqrt(dot(v, v))
//   mat4 * vec4(d, 0): r_i = (m0i*d.x + m1i*d.y) + (m2i*d.z + m3i*0)
//   int(f)       = truncation toward zero, NaN -> 0, saturating
#pragma once

#include <cstdint>

#include "../../include/vrt.h"

namespace vrt {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float fsqrt(float a) { return __fsqrt_rn(a); }
// 1 / a, the IEEE round-to-nearest reciprocal: the same correctly rounded value as
// fdiv(1.0f, a), from a shorter instruction sequence.
__device__ __forceinline__ float frcp(float a) { return __frcp_rn(a); }
__device__ __forceinline__ int f2i(float f) { return __float2int_rz(f); }  // NaN -> 0, saturating
__device__ __forceinline__ int isign(float f) { return f > 0.0f ? 1 : (f < 0.0f ? -1 : 0); }
__device__ __forceinline__ float fmax0(float x) { return x > 0.0f ? x : 0.0f; }

__device__ __forceinline__ float dot3(V3 a, V3 b) { return fadd(fadd(fmul(a.x, b.x), fmul(a.y, b.y)), fmul(a.z, b.z)); }
__device__ __forceinline__ float len3(V3 a) { return fsqrt(dot3(a, a)); }
__device__ __forceinline__ V3 norm3(V3 a) {
    float r = frcp(fsqrt(dot3(a, a)));
    return V3{fmul(a.x, r), fmul(a.y, r), fmul(a.z, r)};
}
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return V3{fsub(a.x, b.x), fsub(a.y, b.y), fsub(a.z, b.z)}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return V3{fadd(a.x, b.x), fadd(a.y, b.y), fadd(a.z, b.z)}; }
__device__ __forceinline__ V3 mul3s(V3 a, float s) { return V3{fmul(a.x, s), fmul(a.y, s), fmul(a.z, s)}; }

// Primary ray direction of pixel (px, py): fshader.glsl:136-137 with the pixel-centre
// NDC of vshader.glsl:6-9 (py counts from the bottom row).
__device__ __forceinline__ V3 primary_dir(const vrt_uniforms& u, int px, int py, int width, int height) {
    float vx = fsub(fdiv((float)(2 * px + 1), (float)width), 1.0f);
    float vy = fsub(fdiv((float)(2 * py + 1), (float)height), 1.0f);
    V3 d = norm3(V3{fmul(fmul(vx, u.aspectRatio), u.tanHalfFov), fmul(vy, u.tanHalfFov), 1.0f});
    const float* m = u.rotateMatrix;
    return V3{fadd(fadd(fmul(m[0], d.x), fmul(m[4], d.y)), fadd(fmul(m[8], d.z), fmul(m[12], 0.0f))),
              fadd(fadd(fmul(m[1], d.x), fmul(m[5], d.y)), fadd(fmul(m[9], d.z), fmul(m[13], 0.0f))),
              fadd(fadd(fmul(m[2], d.x), fmul(m[6], d.y)), fadd(fmul(m[10], d.z), fmul(m[14], 0.0f)))};
}

// hitNormal of a step along `axis` with step sign `s` (fshader.glsl:91,97,103).
__device__ __forceinline__ V3 axis_normal(int axis, int s) {
    float v = (float)(-s);
    return V3{axis == 0 ? v : 0.0f, axis == 1 ? v : 0.0f, axis == 2 ? v : 0.0f};
}

// RGBA8 of a colour channel: (int)(clamp(c, 0, 1) * 255 + 0.5).
__device__ __forceinline__ uint32_t to_u8(float c) {
    float v = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    if (!(v == v)) v = 0.0f;
    return (uint32_t)(int)fadd(fmul(v, 255.0f), 0.5f);
}

// Final colour of fshader.glsl:184-187 (hit) or :133 (miss) / :144 (step view), packed RGBA8.
__device__ __forceinline__ uint32_t pack_color(const vrt_uniforms& u, bool hit, int32_t word, float mr, float mg,
                                               float mb, int primary_steps) {
    float c0, c1, c2, c3 = 1.0f;
    if (u.viewDepthField == 1) {
        c0 = c1 = c2 = fdiv((float)primary_steps, 100.0f);
    } else if (hit) {
        c0 = fmul(fdiv((float)((word & 0x00FF0000) >> 16), 255.0f), mr);
        c1 = fmul(fdiv((float)((word & 0x0000FF00) >> 8), 255.0f), mg);
        c2 = fmul(fdiv((float)(word & 0x000000FF), 255.0f), mb);
    } else {
        c0 = 0.6f; c1 = 0.7f; c2 = 0.8f;
    }
    return to_u8(c0) | (to_u8(c1) << 8) | (to_u8(c2) << 16) | (to_u8(c3) << 24);
}

// A ray's DDA set-up, fshader.glsl:64-79.
struct RaySetup {
    int cx, cy, cz;
    int sx, sy, sz;
    float tx, ty, tz;
    float dx, dy, dz;
};
__device__ __forceinline__ void ray_setup(V3 o, V3 d, RaySetup& r) {
    r.cx = f2i(o.x); r.cy = f2i(o.y); r.cz = f2i(o.z);
    r.sx = isign(d.x); r.sy = isign(d.y); r.sz = isign(d.z);
    r.dx = frcp(fabsf(fadd(d.x, 0.000001f)));
    r.dy = frcp(fabsf(fadd(d.y, 0.000001f)));
    r.dz = frcp(fabsf(fadd(d.z, 0.000001f)));
    r.tx = fdiv(fsub((float)(r.cx + (r.sx > 0)), o.x), d.x);
    r.ty = fdiv(fsub((float)(r.cy + (r.sy > 0)), o.y), d.y);
    r.tz = fdiv(fsub((float)(r.cz + (r.sz > 0)), o.z), d.z);
}

// Per-pixel side outputs and counters.
struct PixelResult {
    uint32_t rgba;
    int32_t hit;
    uint32_t cast, occ;
    int32_t steps, primary_steps;
    float mr, mg, mb;
};

__device__ __forceinline__ void store_pixel(const vrt_debug_out& dbg, uint8_t* rgba, uint64_t i,
                                            const PixelResult& p) {
    reinterpret_cast<uint32_t*>(rgba)[i] = p.rgba;
    if (dbg.hit_index) dbg.hit_index[i] = p.hit;
    if (dbg.cast_mask) dbg.cast_mask[i] = p.cast;
    if (dbg.occ_mask) dbg.occ_mask[i] = p.occ;
    if (dbg.steps) dbg.steps[i] = p.steps;
    if (dbg.primary_steps) dbg.primary_steps[i] = p.primary_steps;
    if (dbg.shade) {
        dbg.shade[3 * i] = p.mr;
        dbg.shade[3 * i + 1] = p.mg;
        dbg.shade[3 * i + 2] = p.mb;
    }
}

}  // namespace vrt
