// CPU oracle for the voxel ray tracer -- TEST INFRASTRUCTURE ONLY.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
// library, and only as the checker or the timed CPU baseline.  The product path
// (voxel-rt_gb300/) never links or calls it.
//
// What it is: a line-for-line scalar C++ restatement of the fragment shader
// src/fshader.glsl of Berry2460/voxel-rt (getVoxelIndex :33-52, vec3ToIntVec3 :54-57,
// castRay :59-129, main :131-190), and of the reference's CPU world code it depends on
// (fixDepthField render.cpp:226-253, computeDepthIndices render.cpp:66-100,
// removeSphere level.cpp:30-56, initVoxels/placeBush/placeTrunk level.cpp:4-138).
//
// Arithmetic contract (shared with the CUDA kernels): IEEE binary32, round to nearest,
// no contraction (build with -ffp-contract=off, no -ffast-math), every expression
// evaluated in the written order:
//   dot(a, b)    = (a.x*b.x + a.y*b.y) + a.z*b.z
//   normalize(v) = v * (1 / sqrt(dot(v, v)))      (GLM's form, glm/detail/func_geometric.inl)
//   length(v)    = sqrt(dot(v, v))
//   mat4 * vec4(d, 0): r_i = (m0i*d.x + m1i*d.y) + (m2i*d.z + m3i*0)   (GLM's association)
//   float -> int conversion truncates toward zero, NaN -> 0, saturates at int range
//   sign(NaN) = 0; max(0, x) = x > 0 ? x : 0
//   RGBA8 = (int)(clamp(c, 0, 1) * 255 + 0.5)
// Pixel (px, py), py counted from the bottom row, sees vPos = ((2px+1)/W - 1, (2py+1)/H - 1).
//
// Parity pins: the shading is checked against the reference shader source compiled as
// C++ against its vendored GLM (oracle/ref/), the world/edit code against the
// reference's own level.cpp/render.cpp compiled with GL stubs (oracle/ref/).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <climits>
#include <vector>
#include <omp.h>

#include "../include/vrt.h"

namespace {

struct V3 { float x, y, z; };
struct I3 { int x, y, z; };

inline int f2i(float f) {  // GLSL int(float): truncation; NaN and overflow pinned
    if (!(f == f)) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f <= -2147483648.0f) return INT_MIN;
    return (int)f;
}
inline int isign(float f) { return f > 0.0f ? 1 : (f < 0.0f ? -1 : 0); }
inline float fmax0(float x) { return x > 0.0f ? x : 0.0f; }
inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float len3(V3 a) { return std::sqrt(dot3(a, a)); }
inline V3 norm3(V3 a) { float r = 1.0f / std::sqrt(dot3(a, a)); return V3{a.x * r, a.y * r, a.z * r}; }
inline V3 sub3(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 add3(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 mul3s(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
inline I3 trunc3(V3 a) { return I3{f2i(a.x), f2i(a.y), f2i(a.z)}; }
inline float as_float(int32_t v) { float f; std::memcpy(&f, &v, 4); return f; }

struct World {
    const int32_t* vox;
    int W, H;
    // getVoxelIndex, fshader.glsl:33-52: -1 outside [0,W)x[0,H)x[0,W).
    inline int64_t index(I3 c) const {
        if (c.x < 0 || c.y < 0 || c.z < 0 || c.x >= W || c.y >= H || c.z >= W) return -1;
        return (int64_t)c.x + (int64_t)W * c.y + (int64_t)W * H * c.z;
    }
};

struct RayOut {
    int64_t hit;   // voxel index or -1
    V3 hitPos;     // written only on a hit (global hitPos of the shader)
    V3 hitNormal;  // normal of the last DDA step (global hitNormal)
    int steps;     // loop iterations (stepCount increments)
};

// castRay, fshader.glsl:59-129.  maxSteps replaces RENDER_DIST.
RayOut cast_ray(const World& w, V3 start, V3 dir, int dist, int maxSteps, V3 prevHitPos, V3 prevNormal) {
    RayOut o{-1, prevHitPos, prevNormal, 0};
    I3 cell = trunc3(start);                                              // :64
    I3 step{isign(dir.x), isign(dir.y), isign(dir.z)};                    // :71
    I3 fwd{step.x > 0, step.y > 0, step.z > 0};                           // :72
    float dx = 1.0f / std::fabs(dir.x + 0.000001f);                       // :74-76
    float dy = 1.0f / std::fabs(dir.y + 0.000001f);
    float dz = 1.0f / std::fabs(dir.z + 0.000001f);
    V3 isect{((float)(cell.x + fwd.x) - start.x) / dir.x,                 // :79
             ((float)(cell.y + fwd.y) - start.y) / dir.y,
             ((float)(cell.z + fwd.z) - start.z) / dir.z};
    float currDist = 0.0f, travelled = 0.0f;
    const float fdist = (float)dist, fcap = (float)maxSteps;
    while (travelled < fdist && travelled < fcap) {                       // :83
        o.steps++;                                                        // :84
        travelled += 1.0f;                                                // :85
        if (isect.x < isect.y && isect.x < isect.z) {                     // :87-92
            currDist = isect.x; cell.x += step.x; isect.x += dx;
            o.hitNormal = V3{(float)(-step.x), 0.0f, 0.0f};
        } else if (isect.y < isect.x && isect.y < isect.z) {              // :93-98
            currDist = isect.y; cell.y += step.y; isect.y += dy;
            o.hitNormal = V3{0.0f, (float)(-step.y), 0.0f};
        } else {                                                          // :99-104 (ties -> z)
            currDist = isect.z; cell.z += step.z; isect.z += dz;
            o.hitNormal = V3{0.0f, 0.0f, (float)(-step.z)};
        }
        int64_t idx = w.index(cell);                                      // :105
        if (idx >= 0 && w.vox[idx] >= 0) {                                // :108-112
            o.hitPos = add3(mul3s(dir, currDist), start);
            o.hit = idx;
            break;
        } else if (idx >= 0 && w.vox[idx] != -1) {                        // :114-121
            float toJump = -as_float(w.vox[idx]);
            travelled += toJump;
            currDist += toJump;
            start = add3(mul3s(dir, currDist), start);
            cell = trunc3(start);
            isect = V3{((float)(cell.x + fwd.x) - start.x) / dir.x,
                       ((float)(cell.y + fwd.y) - start.y) / dir.y,
                       ((float)(cell.z + fwd.z) - start.z) / dir.z};
        } else if (idx < 0) {                                             // :123-125
            break;
        }
    }
    return o;
}

inline uint8_t to_u8(float c) {
    float v = c < 0.0f ? 0.0f : (c > 1.0f ? 1.0f : c);
    if (!(v == v)) v = 0.0f;
    return (uint8_t)(int)(v * 255.0f + 0.5f);
}

struct PixelOut {
    uint8_t rgba[4];
    int32_t hit;
    uint32_t cast, occ;
    int32_t steps, primary_steps;
    float shade[3];
};

// main(), fshader.glsl:131-190 for one pixel.
PixelOut shade_pixel(const World& w, const vrt_uniforms& u, int px, int py, int width, int height) {
    PixelOut p{};
    float col[4] = {0.6f, 0.7f, 0.8f, 1.0f};                              // :133
    float vx = (float)(2 * px + 1) / (float)width - 1.0f;                 // vshader.glsl:6-9
    float vy = (float)(2 * py + 1) / (float)height - 1.0f;
    V3 d0{(vx * u.aspectRatio) * u.tanHalfFov, vy * u.tanHalfFov, 1.0f};
    V3 d = norm3(d0);                                                     // :136
    const float* m = u.rotateMatrix;                                      // :137
    V3 rd{(m[0] * d.x + m[4] * d.y) + (m[8] * d.z + m[12] * 0.0f),
          (m[1] * d.x + m[5] * d.y) + (m[9] * d.z + m[13] * 0.0f),
          (m[2] * d.x + m[6] * d.y) + (m[10] * d.z + m[14] * 0.0f)};
    V3 cam{u.camPos[0], u.camPos[1], u.camPos[2]};
    RayOut pr = cast_ray(w, cam, rd, u.maxSteps, u.maxSteps, V3{0, 0, 0}, V3{0, 0, 0}); // :139
    V3 hp = pr.hitPos, hn = pr.hitNormal;                                 // :140-141
    p.hit = (int32_t)pr.hit;
    p.steps = pr.steps;
    p.primary_steps = pr.steps;
    float mr = u.ambient, mg = u.ambient, mb = u.ambient;
    if (u.viewDepthField == 1) {                                          // :143-145
        float s = (float)pr.steps / 100.0f;
        col[0] = col[1] = col[2] = s; col[3] = 1.0f;
        mr = mg = mb = s;
    } else {
        V3 lp{u.lightPos[0], u.lightPos[1], u.lightPos[2]};
        V3 toLight = norm3(sub3(lp, hp));                                 // :147
        if (pr.hit != -1 && w.vox[pr.hit] >= 0) {                         // :152
            RayOut sr = cast_ray(w, add3(hp, mul3s(toLight, 0.001f)), toLight, u.maxSteps, u.maxSteps, hp, hn); // :154
            p.steps += sr.steps;
            p.cast |= 1u;
            if (sr.hit == -1) {
                float c = u.diffuse * fmax0(dot3(hn, toLight));           // :155
                mr += c; mg += c; mb += c;
            } else {
                p.occ |= 1u;
            }
            for (int i = 0; i < VRT_MAX_LOCAL_LIGHTS; i++) {              // :159
                if (mr >= u.maxOverbright && mg >= u.maxOverbright && mb >= u.maxOverbright) { // :161-164
                    mr = mg = mb = u.maxOverbright;
                    break;
                } else if (u.localLights[i][0] >= 0 && u.localLights[i][1] >= 0 && u.localLights[i][2] >= 0) { // :167
                    V3 L{u.localLights[i][0], u.localLights[i][1], u.localLights[i][2]};
                    float ld = len3(sub3(L, hp));                         // :168
                    if (ld <= u.localLightDist) {                         // :171
                        V3 tl = norm3(sub3(L, hp));                       // :173
                        RayOut lr = cast_ray(w, add3(hp, mul3s(tl, 0.001f)), tl, f2i(ld + 1.0f), u.maxSteps, hp, hn); // :175
                        p.steps += lr.steps;
                        p.cast |= 2u << i;
                        if (lr.hit == -1) {                               // :177
                            float nl = fmax0(dot3(hn, tl));
                            float fall = (u.localLightDist - ld) / u.localLightDist;
                            float a = u.localLights[i][3];
                            mr += ((a * u.localLightColor[i][0]) * nl) * fall;
                            mg += ((a * u.localLightColor[i][1]) * nl) * fall;
                            mb += ((a * u.localLightColor[i][2]) * nl) * fall;
                        } else {
                            p.occ |= 2u << i;
                        }
                    }
                }
            }
            int32_t v = w.vox[pr.hit];                                    // :184-187
            col[0] = (float)((v & 0x00FF0000) >> 16) / 255.0f * mr;
            col[1] = (float)((v & 0x0000FF00) >> 8) / 255.0f * mg;
            col[2] = (float)(v & 0x000000FF) / 255.0f * mb;
            col[3] = 1.0f;
        }
    }
    p.shade[0] = mr; p.shade[1] = mg; p.shade[2] = mb;
    for (int c = 0; c < 4; c++) p.rgba[c] = to_u8(col[c]);
    return p;
}

// ---------------- reference CPU world code ----------------

struct DepthOffset { float dist; int x, y, z; };

// computeDepthIndices, render.cpp:66-100 (DEPTH_FIELD_RADIUS = 7, render.hpp:7).
const std::vector<DepthOffset>& depth_offsets() {
    static std::vector<DepthOffset> offs = [] {
        const int R = 7;
        std::vector<DepthOffset> v;
        for (int z = -R; z <= R; z++)
            for (int y = -R; y <= R; y++)
                for (int x = -R; x <= R; x++) {
                    if (x * x + y * y + z * z <= R * R) {
                        int xd = x - (x > 0) + (x < 0);
                        int yd = y - (y > 0) + (y < 0);
                        int zd = z - (z > 0) + (z < 0);
                        // render.cpp:81: -sqrt(int) is the double sqrt, stored into a float
                        float dist = (float)(-std::sqrt((double)(xd * xd + yd * yd + zd * zd)));
                        if (dist <= (float)R) v.push_back(DepthOffset{dist, x, y, z});
                    }
                }
        return v;
    }();
    return offs;
}

// fixDepthField, render.cpp:226-253.  Neighbours outside the world count as not solid
// (the reference reads voxels[-1] there, render.cpp:237-240).
void fix_depth_field(int32_t* vox, int W, int H, int x, int y, int z) {
    World w{vox, W, H};
    int64_t index = w.index(I3{x, y, z});
    float nearest = (float)(-7 + 1);
    if (index >= 0 && vox[index] < 0) {
        for (const DepthOffset& o : depth_offsets()) {
            int64_t ic = w.index(I3{x + o.x, y + o.y, z + o.z});
            bool solid = ic >= 0 && vox[ic] >= 0;
            if (solid && o.dist > nearest) {
                if (o.dist <= -2.0f) nearest = o.dist;
                else nearest = 0.0f;
            }
        }
        if (nearest < 0.0f) {
            int32_t bits;
            std::memcpy(&bits, &nearest, 4);
            vox[index] = bits;
        }
    }
}

inline void destroy_voxel(int32_t* vox, int W, int H, int x, int y, int z) {
    // destroyVoxel, render.cpp:265-271 (callers only pass in-world coordinates, or
    // relative ones that are >= 0; index -1 only arises for x/y/z beyond W/H/W, skipped).
    World w{vox, W, H};
    int64_t idx = w.index(I3{x, y, z});
    if (x >= 0 && y >= 0 && z >= 0 && idx >= 0) vox[idx] = -1;
}
inline void place_voxel(int32_t* vox, int W, int H, int x, int y, int z, int32_t v) {
    World w{vox, W, H};  // placeVoxel, render.cpp:256-262
    int64_t idx = w.index(I3{x, y, z});
    if (idx >= 0) vox[idx] = v;
}

}  // namespace

extern "C" {

// Renders rows [row_begin, row_end) of a width x height image.  Every output array is
// full-image sized (index py*width + px); any may be NULL.  threads <= 0: OpenMP default.
int vrt_oracle_render(const int32_t* words, int W, int H, const vrt_uniforms* u, int width, int height,
                      int row_begin, int row_end, int row_stride, uint8_t* rgba, int32_t* hit_index,
                      uint32_t* cast_mask, uint32_t* occ_mask, int32_t* steps, int32_t* primary_steps,
                      float* shade, uint64_t* totals, int threads) {
    if (!words || !u || width <= 0 || height <= 0 || row_stride <= 0) return -1;
    World w{words, W, H};
    if (row_begin < 0) row_begin = 0;
    if (row_end > height) row_end = height;
    int nrows = row_end > row_begin ? (row_end - row_begin + row_stride - 1) / row_stride : 0;
    uint64_t t_rays = 0, t_steps = 0, t_hits = 0, t_pix = 0;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads) reduction(+ : t_rays, t_steps, t_hits, t_pix)
    for (int r = 0; r < nrows; r++) {
        int py = row_begin + r * row_stride;
        for (int px = 0; px < width; px++) {
            PixelOut p = shade_pixel(w, *u, px, py, width, height);
            size_t i = (size_t)py * width + px;
            if (rgba) std::memcpy(rgba + 4 * i, p.rgba, 4);
            if (hit_index) hit_index[i] = p.hit;
            if (cast_mask) cast_mask[i] = p.cast;
            if (occ_mask) occ_mask[i] = p.occ;
            if (steps) steps[i] = p.steps;
            if (primary_steps) primary_steps[i] = p.primary_steps;
            if (shade) { shade[3 * i] = p.shade[0]; shade[3 * i + 1] = p.shade[1]; shade[3 * i + 2] = p.shade[2]; }
            t_rays += 1 + (uint64_t)__builtin_popcount(p.cast);
            t_steps += (uint64_t)p.steps;
            t_hits += p.hit >= 0;
            t_pix += 1;
        }
    }
    if (totals) { totals[0] = t_rays; totals[1] = t_steps; totals[2] = t_hits; totals[3] = t_pix; }
    return 0;
}

// One castRay (fshader.glsl:59-129) for known-answer tests.
int vrt_oracle_cast_ray(const int32_t* words, int W, int H, const float* start, const float* dir, int dist,
                        int maxSteps, int64_t* hit, float* hitPos, float* hitNormal, int32_t* steps) {
    World w{words, W, H};
    RayOut o = cast_ray(w, V3{start[0], start[1], start[2]}, V3{dir[0], dir[1], dir[2]}, dist, maxSteps,
                        V3{0, 0, 0}, V3{0, 0, 0});
    if (hit) *hit = o.hit;
    if (hitPos) { hitPos[0] = o.hitPos.x; hitPos[1] = o.hitPos.y; hitPos[2] = o.hitPos.z; }
    if (hitNormal) { hitNormal[0] = o.hitNormal.x; hitNormal[1] = o.hitNormal.y; hitNormal[2] = o.hitNormal.z; }
    if (steps) *steps = o.steps;
    return 0;
}

// fixDepthField over the box [x0,x1)x[y0,y1)x[z0,z1) in z,y,x order (render.cpp:273-286).
int vrt_oracle_fix_depth_field_box(int32_t* words, int W, int H, int x0, int y0, int z0, int x1, int y1, int z1,
                                   int threads) {
    if (threads <= 0) threads = omp_get_max_threads();
    // fixDepthField writes only air words and reads only solidity, so z-slabs are independent.
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
    for (int z = z0; z < z1; z++)
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) fix_depth_field(words, W, H, x, y, z);
    return 0;
}

// removeSphere, level.cpp:30-56 (DEPTH_FIELD_RADIUS>>1 = 3).
int vrt_oracle_remove_sphere(int32_t* words, int W, int H, int cx, int cy, int cz, int radius, int refresh) {
    for (int z = -radius; z < radius; z++)
        for (int y = -radius; y < radius; y++)
            for (int x = -radius; x < radius; x++)
                if (x + cx < W && y + cy < H && z + cz < W && x + cx >= 0 && y + cy >= 0 && z + cz >= 0)
                    if (x * x + y * y + z * z < radius * radius) destroy_voxel(words, W, H, x + cx, y + cy, z + cz);
    if (!refresh) return 0;
    int r2 = radius + (7 >> 1);
    for (int z = -r2; z < r2; z++)
        for (int y = -r2; y < r2; y++)
            for (int x = -r2; x < r2; x++)
                if (x + cx < W && y + cy < H && z + cz < W && x + cx >= 0 && y + cy >= 0 && z + cz >= 0)
                    if (x * x + y * y + z * z < r2 * r2) fix_depth_field(words, W, H, x + cx, y + cy, z + cz);
    return 0;
}

// initVoxels, level.cpp:82-138, with placeBush (:4-27) and placeTrunk (:59-79).
int vrt_oracle_init_reference(int32_t* vox, int W, int H) {
    for (size_t i = 0; i < (size_t)W * H * W; i++) vox[i] = -1;  // render.cpp:349-351
    for (int z = 0; z < W; z++)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                int cv = 5 * ((x + y + z) % 3);
                destroy_voxel(vox, W, H, x, y, z);
                int v;
                if (y <= 25) {
                    v = ((90 + cv) << 16) | ((90 + cv) << 8) | (90 + cv);
                    place_voxel(vox, W, H, x, y, z, v);
                } else if (y <= 33) {
                    v = ((120 + cv) << 16) | ((100 + cv) << 8) | 0;
                    place_voxel(vox, W, H, x, y, z, v);
                } else if (y <= 36) {
                    v = (10 << 16) | ((130 + cv) << 8) | 10;
                    place_voxel(vox, W, H, x, y, z, v);
                }
            }
    for (int z = 10; z < W - 10; z++)
        for (int x = 10; x < W - 10; x++)
            if (x % 30 == 0 && z % 25 == 0) {
                // placeTrunk(ivec3(x + 1 + z%7, 36, z), ivec3(128,100,15), 6)
                {
                    int px = x + 1 + z % 7, py = 36, pz = z, len = 6;
                    for (int dz = -len >> 2; dz < len >> 2; dz++)
                        for (int dy = 0; dy < len; dy++)
                            for (int dx = -len >> 2; dx < len >> 2; dx++)
                                if (dx + px < W && dy + py < H && dz + pz < W) {
                                    destroy_voxel(vox, W, H, dx, dy, dz);
                                    int v = 128 - ((dx + dz) % 2) * 10;
                                    v = (v << 8) + (100 - ((dx + dz) % 2) * 10);
                                    v = (v << 8) + 15;
                                    place_voxel(vox, W, H, dx + px, dy + py, dz + pz, v);
                                }
                }
                // placeBush(ivec3(x + z%7, 36 + 10, z), ivec3(15,128,15), 6)
                {
                    int px = x + z % 7, py = 46, pz = z, r = 6;
                    for (int dz = -r; dz < r; dz++)
                        for (int dy = -r; dy < r; dy++)
                            for (int dx = -r; dx < r; dx++)
                                if (dx + px < W && dy + py < H && dz + pz < W && dx + px >= 0 && dy + py >= 0 &&
                                    dz + pz >= 0)
                                    if (dx * dx + dy * dy + dz * dz < r * r) {
                                        destroy_voxel(vox, W, H, dx, dy, dz);
                                        int v = 15;
                                        v = (v << 8) + (128 - ((dx + dy + dz) % 3) * 20);
                                        v = (v << 8) + 15;
                                        place_voxel(vox, W, H, dx + px, dy + py, dz + pz, v);
                                    }
                }
            }
    return 0;
}

// Number of offsets of the depth-field sphere (computeDepthIndices, render.cpp:66-100).
int vrt_oracle_depth_offset_count(void) { return (int)depth_offsets().size(); }

}  // extern "C"
