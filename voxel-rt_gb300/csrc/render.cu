// Render kernels: the per-pixel path of Berry2460/voxel-rt src/fshader.glsl.
//
// render_word_kernel  one thread per pixel; every DDA step reads the 4-byte voxel word,
//                     follows depth-field jumps (fshader.glsl:114-121).  Exact on every
//                     world, including worlds built by fixDepthField.
// render_mask_kernel  persistent warps over ray tiles; traversal reads the 64-ary
//                     occupancy hierarchy (64^3 -> 16^3 -> 4^3 -> voxel, one uint64
//                     per node) and keeps the current brick's 64 voxel bits in
//                     registers, so a step inside a known box touches no memory; the
//                     colour word is fetched once, at the primary hit.  Lanes whose ray
//                     ends are refilled (next shadow ray of their pixel, or a new
//                     pixel from the warp's tile queue) together, once refill_min lanes
//                     are idle, which keeps the warp's lanes busy although ray lengths
//                     vary from 1 to thousands of steps.
// Both perform every per-cell floating-point add of the shader in its order, so hit
// voxels, step counts and shadow bits are those of the CPU oracle bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include "shade_common.cuh"
#include "vrt_internal.h"

namespace vrt {

// ====================================================================== word kernel

struct WordParams {
    vrt_uniforms u;
    int width, height;
    uint8_t* rgba;
    vrt_debug_out dbg;
    unsigned long long* stats;
};

struct WordRay {
    int32_t hit;   // voxel index or -1
    float cd;      // currDist at the hit
    int axis, s;   // axis and step sign of the last DDA step (hitNormal)
    V3 start;      // start position after depth-field jumps (hitPos uses it)
    int steps;
};

// castRay, fshader.glsl:59-129, over the voxel words.
__device__ WordRay cast_word(const int32_t* __restrict__ words, const Layout& L, V3 start, V3 dir, int dist,
                             int maxSteps) {
    WordRay o;
    o.hit = -1; o.cd = 0.0f; o.axis = 2; o.s = 0; o.steps = 0;
    RaySetup r;
    ray_setup(start, dir, r);
    float cd = 0.0f, travelled = 0.0f;
    const float fdist = (float)dist, fcap = (float)maxSteps;
    int axis = 2, s = 0;
    while (travelled < fdist && travelled < fcap) {
        o.steps++;
        travelled = fadd(travelled, 1.0f);
        if (r.tx < r.ty && r.tx < r.tz) {
            cd = r.tx; r.cx += r.sx; r.tx = fadd(r.tx, r.dx); axis = 0; s = r.sx;
        } else if (r.ty < r.tx && r.ty < r.tz) {
            cd = r.ty; r.cy += r.sy; r.ty = fadd(r.ty, r.dy); axis = 1; s = r.sy;
        } else {
            cd = r.tz; r.cz += r.sz; r.tz = fadd(r.tz, r.dz); axis = 2; s = r.sz;
        }
        if ((unsigned)r.cx >= (unsigned)L.W || (unsigned)r.cy >= (unsigned)L.H || (unsigned)r.cz >= (unsigned)L.W)
            break;  // getVoxelIndex == -1
        int32_t idx = r.cx + L.W * r.cy + L.W * L.H * r.cz;
        int32_t v = __ldg(words + idx);
        if (v >= 0) {
            o.hit = idx;
            break;
        } else if (v != -1) {  // depth-field jump
            float toJump = -__int_as_float(v);
            travelled = fadd(travelled, toJump);
            cd = fadd(cd, toJump);
            start = add3(mul3s(dir, cd), start);
            r.cx = f2i(start.x); r.cy = f2i(start.y); r.cz = f2i(start.z);
            r.tx = fdiv(fsub((float)(r.cx + (r.sx > 0)), start.x), dir.x);
            r.ty = fdiv(fsub((float)(r.cy + (r.sy > 0)), start.y), dir.y);
            r.tz = fdiv(fsub((float)(r.cz + (r.sz > 0)), start.z), dir.z);
        }
    }
    o.cd = cd; o.axis = axis; o.s = s; o.start = start;
    return o;
}

__global__ void __launch_bounds__(128) render_word_kernel(const int32_t* __restrict__ words, Layout L,
                                                          const __grid_constant__ WordParams p) {
    const int px = blockIdx.x * 16 + (threadIdx.x & 15);
    const int py = blockIdx.y * 8 + (threadIdx.x >> 4);
    const bool valid = px < p.width && py < p.height;
    PixelResult res{};
    if (valid) {
        const vrt_uniforms& u = p.u;
        V3 cam{u.camPos[0], u.camPos[1], u.camPos[2]};
        V3 rd = primary_dir(u, px, py, p.width, p.height);
        WordRay pr = cast_word(words, L, cam, rd, u.maxSteps, u.maxSteps);
        res.hit = pr.hit;
        res.steps = pr.steps;
        res.primary_steps = pr.steps;
        float mr = u.ambient, mg = u.ambient, mb = u.ambient;
        int32_t word = 0;
        if (u.viewDepthField == 1) {
            mr = mg = mb = fdiv((float)pr.steps, 100.0f);
        } else if (pr.hit >= 0) {
            V3 hp = add3(mul3s(rd, pr.cd), pr.start);
            V3 hn = axis_normal(pr.axis, pr.s);
            V3 lp{u.lightPos[0], u.lightPos[1], u.lightPos[2]};
            V3 toLight = norm3(sub3(lp, hp));
            WordRay sr = cast_word(words, L, add3(hp, mul3s(toLight, 0.001f)), toLight, u.maxSteps, u.maxSteps);
            res.steps += sr.steps;
            res.cast |= 1u;
            if (sr.hit < 0) {
                float c = fmul(u.diffuse, fmax0(dot3(hn, toLight)));
                mr = fadd(mr, c); mg = fadd(mg, c); mb = fadd(mb, c);
            } else {
                res.occ |= 1u;
            }
            const float ob = u.maxOverbright, R = u.localLightDist;
            for (int i = 0; i < VRT_MAX_LOCAL_LIGHTS; i++) {
                if (mr >= ob && mg >= ob && mb >= ob) {
                    mr = mg = mb = ob;
                    break;
                } else if (u.localLights[i][0] >= 0 && u.localLights[i][1] >= 0 && u.localLights[i][2] >= 0) {
                    V3 Lp{u.localLights[i][0], u.localLights[i][1], u.localLights[i][2]};
                    float ld = len3(sub3(Lp, hp));
                    if (ld <= R) {
                        V3 tl = norm3(sub3(Lp, hp));
                        WordRay lr = cast_word(words, L, add3(hp, mul3s(tl, 0.001f)), tl, f2i(fadd(ld, 1.0f)),
                                               u.maxSteps);
                        res.steps += lr.steps;
                        res.cast |= 2u << i;
                        if (lr.hit < 0) {
                            float nl = fmax0(dot3(hn, tl));
                            float fall = fdiv(fsub(R, ld), R);
                            float a = u.localLights[i][3];
                            mr = fadd(mr, fmul(fmul(fmul(a, u.localLightColor[i][0]), nl), fall));
                            mg = fadd(mg, fmul(fmul(fmul(a, u.localLightColor[i][1]), nl), fall));
                            mb = fadd(mb, fmul(fmul(fmul(a, u.localLightColor[i][2]), nl), fall));
                        } else {
                            res.occ |= 2u << i;
                        }
                    }
                }
            }
            word = __ldg(words + pr.hit);
        }
        res.mr = mr; res.mg = mg; res.mb = mb;
        res.rgba = pack_color(u, pr.hit >= 0, word, mr, mg, mb, pr.steps);
        store_pixel(p.dbg, p.rgba, (uint64_t)py * p.width + px, res);
    }
    if (p.stats) {
        unsigned rays = valid ? 1u + __popc(res.cast) : 0u;
        unsigned steps = valid ? (unsigned)res.steps : 0u;
        unsigned hits = valid && res.hit >= 0 ? 1u : 0u;
        unsigned pix = valid ? 1u : 0u;
        rays = __reduce_add_sync(0xffffffffu, rays);
        unsigned long long s64 = steps;  // a warp's steps can pass 2^32 at large step caps
        for (int off = 16; off > 0; off >>= 1) s64 += __shfl_down_sync(0xffffffffu, s64, off);
        hits = __reduce_add_sync(0xffffffffu, hits);
        pix = __reduce_add_sync(0xffffffffu, pix);
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(p.stats + VRT_STAT_RAYS, (unsigned long long)rays);
            atomicAdd(p.stats + VRT_STAT_STEPS, s64);
            atomicAdd(p.stats + VRT_STAT_HITS, (unsigned long long)hits);
            atomicAdd(p.stats + VRT_STAT_PIXELS, (unsigned long long)pix);
        }
    }
}

// ====================================================================== mask kernel

struct ViewDev {
    vrt_uniforms u;
    int width, height;
    int tiles_x;
    int tile_begin;  // first global tile of this view
    uint8_t* rgba;
    vrt_debug_out dbg;
    unsigned long long* stats;
};

struct MaskParams {
    const int32_t* words;
    const uint64_t* bricks;
    const uint64_t* regions;
    const uint64_t* supers;
    Layout L;
    const ViewDev* views;  // nviews entries (device); NULL when nviews == 1 (v0 is used)
    int nviews;
    int total_tiles;
    int tile_w, tile_h;
    int refill_min;
    unsigned int* tile_counter;
    ViewDev v0;
};

enum { T_LIVE = 0, T_HIT = 1, T_MISS = 2 };
enum { PH_IDLE = -1, PH_PRIMARY = 0, PH_GLOBAL = 1, PH_LOCAL0 = 2 };

struct Trav {
    int cx, cy, cz;
    int sx, sy, sz;
    float tx, ty, tz;
    float dx, dy, dz;
    int rem;         // DDA iterations left
    int ex, ey, ez;  // cell coordinate at which the ray leaves the current box, per axis
    uint64_t m;      // voxel bits of the current brick (0 for an empty box)
    float cd;        // currDist of the last step
    int la;          // axis of the last step
};

// The ray just entered cell c outside its known box: find the largest empty node of
// the hierarchy holding c (super block, region or brick), or load the brick's bits.
__device__ __forceinline__ int refill(Trav& r, const MaskParams& P) {
    const Layout& L = P.L;
    if ((unsigned)r.cx >= (unsigned)L.W || (unsigned)r.cy >= (unsigned)L.H || (unsigned)r.cz >= (unsigned)L.W)
        return T_MISS;  // left the world: getVoxelIndex == -1
    const uint64_t sidx = (uint64_t)(r.cx >> 6) + (uint64_t)L.SW * ((uint64_t)(r.cy >> 6) + (uint64_t)L.SH * (r.cz >> 6));
    const uint64_t sm = __ldg(P.supers + sidx);
    int shift;
    uint64_t m = 0;
    if (sm == 0) {
        shift = 6;
    } else {
        const int rb = ((r.cx >> 4) & 3) + 4 * ((r.cy >> 4) & 3) + 16 * ((r.cz >> 4) & 3);
        if (!((sm >> rb) & 1)) {
            shift = 4;
        } else {
            const uint64_t ridx = sidx * 64 + rb;
            const uint64_t rm = __ldg(P.regions + ridx);
            const int bb = ((r.cx >> 2) & 3) + 4 * ((r.cy >> 2) & 3) + 16 * ((r.cz >> 2) & 3);
            shift = 2;
            if ((rm >> bb) & 1) m = __ldg(P.bricks + ridx * 64 + bb);
        }
    }
    const int lox = (r.cx >> shift) << shift, loy = (r.cy >> shift) << shift, loz = (r.cz >> shift) << shift;
    const int size = 1 << shift;
    const int hix = min(lox + size, L.W), hiy = min(loy + size, L.H), hiz = min(loz + size, L.W);
    r.ex = r.sx > 0 ? hix : (r.sx < 0 ? lox - 1 : INT_MIN);
    r.ey = r.sy > 0 ? hiy : (r.sy < 0 ? loy - 1 : INT_MIN);
    r.ez = r.sz > 0 ? hiz : (r.sz < 0 ? loz - 1 : INT_MIN);
    r.m = m;
    if (m) {
        const int bit = (r.cx & 3) + 4 * (r.cy & 3) + 16 * (r.cz & 3);
        if ((m >> bit) & 1) return T_HIT;
    }
    return T_LIVE;
}

// One iteration of castRay's loop (fshader.glsl:83-126).
__device__ __forceinline__ int dda_step(Trav& r, const MaskParams& P) {
    if (r.rem == 0) return T_MISS;
    r.rem--;
    const bool bx = r.tx < r.ty && r.tx < r.tz;
    const bool by = !bx && r.ty < r.tx && r.ty < r.tz;
    bool out;
    if (bx) {
        r.cd = r.tx; r.tx = fadd(r.tx, r.dx); r.cx += r.sx; out = r.cx == r.ex; r.la = 0;
    } else if (by) {
        r.cd = r.ty; r.ty = fadd(r.ty, r.dy); r.cy += r.sy; out = r.cy == r.ey; r.la = 1;
    } else {
        r.cd = r.tz; r.tz = fadd(r.tz, r.dz); r.cz += r.sz; out = r.cz == r.ez; r.la = 2;
    }
    if (out) return refill(r, P);
    if (r.m) {
        const int bit = (r.cx & 3) + 4 * (r.cy & 3) + 16 * (r.cz & 3);
        if ((r.m >> bit) & 1) return T_HIT;
    }
    return T_LIVE;
}

// Start a ray at o along d with loop bound n; the first step always refills, because
// the known box is empty (each exit coordinate is the first cell the step reaches).
__device__ __forceinline__ void start_ray(Trav& r, V3 o, V3 d, int n, int maxSteps) {
    RaySetup s;
    ray_setup(o, d, s);
    r.cx = s.cx; r.cy = s.cy; r.cz = s.cz;
    r.sx = s.sx; r.sy = s.sy; r.sz = s.sz;
    r.tx = s.tx; r.ty = s.ty; r.tz = s.tz;
    r.dx = s.dx; r.dy = s.dy; r.dz = s.dz;
    r.rem = max(0, min(n, maxSteps));
    r.ex = s.cx + s.sx; r.ey = s.cy + s.sy; r.ez = s.cz + s.sz;
    r.m = 0;
    r.cd = 0.0f;
    r.la = 2;
}

__device__ __forceinline__ const ViewDev& view_of(const MaskParams& P, int v) {
    return P.nviews == 1 ? P.v0 : P.views[v];
}

__global__ void __launch_bounds__(256, 3) render_mask_kernel(const __grid_constant__ MaskParams P) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const unsigned FULL = 0xffffffffu;
    const int tile_px = P.tile_w * P.tile_h;

    // warp tile queue (uniform across the warp)
    int q_pos = 0, q_size = 0, q_vid = 0, q_x0 = 0, q_y0 = 0, q_w = 0, q_h = 0;
    bool q_empty = false;

    // lane state
    int phase = PH_IDLE;
    int vid = 0, pix = 0;
    float hpx = 0.f, hpy = 0.f, hpz = 0.f;
    int hn_axis = 2, hn_s = 0;
    float mr = 0.f, mg = 0.f, mb = 0.f;
    int32_t hit = -1;
    uint32_t cast = 0, occ = 0;
    int steps = 0, psteps = 0;
    bool live = false;
    int status = T_MISS;
    Trav r;
    r.rem = 0; r.m = 0;

    // per-lane counters, flushed when the lane moves to another view and at exit
    int st_vid = -1;
    unsigned long long st_steps = 0;
    unsigned st_rays = 0, st_hits = 0, st_pix = 0;

    while (true) {
        // ---- 1. lanes whose ray ended: fold the result in and pick the pixel's next ray
        bool want = false;
        V3 o{0.f, 0.f, 0.f}, d{0.f, 0.f, 0.f};
        int n = 0;
        if (phase != PH_IDLE && !live) {
            const ViewDev& V = view_of(P, vid);
            const vrt_uniforms& u = V.u;
            steps -= r.rem;  // iterations this ray did not use
            bool done = false;
            V3 hp{hpx, hpy, hpz};
            int next = 16;
            if (phase == PH_PRIMARY) {
                psteps = steps;
                if (status == T_HIT) {
                    hit = r.cx + P.L.W * r.cy + P.L.W * P.L.H * r.cz;
                    const int px = pix % V.width, py = pix / V.width;
                    V3 rd = primary_dir(u, px, py, V.width, V.height);
                    V3 cam{u.camPos[0], u.camPos[1], u.camPos[2]};
                    hp = add3(mul3s(rd, r.cd), cam);
                    hpx = hp.x; hpy = hp.y; hpz = hp.z;
                    hn_axis = r.la;
                    hn_s = r.la == 0 ? r.sx : (r.la == 1 ? r.sy : r.sz);
                }
                if (u.viewDepthField == 1) {
                    mr = mg = mb = fdiv((float)psteps, 100.0f);
                    done = true;
                } else if (hit < 0) {
                    done = true;
                } else {
                    V3 lp{u.lightPos[0], u.lightPos[1], u.lightPos[2]};
                    V3 toLight = norm3(sub3(lp, hp));
                    o = add3(hp, mul3s(toLight, 0.001f));
                    d = toLight;
                    n = u.maxSteps;
                    want = true;
                    phase = PH_GLOBAL;
                }
            } else {
                V3 hn = axis_normal(hn_axis, hn_s);
                if (phase == PH_GLOBAL) {
                    cast |= 1u;
                    if (status == T_HIT) {
                        occ |= 1u;
                    } else {
                        V3 lp{u.lightPos[0], u.lightPos[1], u.lightPos[2]};
                        V3 toLight = norm3(sub3(lp, hp));
                        float c = fmul(u.diffuse, fmax0(dot3(hn, toLight)));
                        mr = fadd(mr, c); mg = fadd(mg, c); mb = fadd(mb, c);
                    }
                    next = 0;
                } else {
                    const int i = phase - PH_LOCAL0;
                    cast |= 2u << i;
                    if (status == T_HIT) {
                        occ |= 2u << i;
                    } else {
                        V3 Lp{u.localLights[i][0], u.localLights[i][1], u.localLights[i][2]};
                        float ld = len3(sub3(Lp, hp));
                        V3 tl = norm3(sub3(Lp, hp));
                        float nl = fmax0(dot3(hn, tl));
                        float fall = fdiv(fsub(u.localLightDist, ld), u.localLightDist);
                        float a = u.localLights[i][3];
                        mr = fadd(mr, fmul(fmul(fmul(a, u.localLightColor[i][0]), nl), fall));
                        mg = fadd(mg, fmul(fmul(fmul(a, u.localLightColor[i][1]), nl), fall));
                        mb = fadd(mb, fmul(fmul(fmul(a, u.localLightColor[i][2]), nl), fall));
                    }
                    next = i + 1;
                }
                // fshader.glsl:159-181: overbright test before each light, then range test
                const float ob = u.maxOverbright;
                for (int i = next; i < VRT_MAX_LOCAL_LIGHTS; i++) {
                    if (mr >= ob && mg >= ob && mb >= ob) {
                        mr = mg = mb = ob;
                        break;
                    }
                    if (u.localLights[i][0] >= 0 && u.localLights[i][1] >= 0 && u.localLights[i][2] >= 0) {
                        V3 Lp{u.localLights[i][0], u.localLights[i][1], u.localLights[i][2]};
                        float ld = len3(sub3(Lp, hp));
                        if (ld <= u.localLightDist) {
                            V3 tl = norm3(sub3(Lp, hp));
                            o = add3(hp, mul3s(tl, 0.001f));
                            d = tl;
                            n = f2i(fadd(ld, 1.0f));
                            want = true;
                            phase = PH_LOCAL0 + i;
                            break;
                        }
                    }
                }
                done = !want;
            }
            if (done) {
                int32_t word = hit >= 0 ? __ldg(P.words + hit) : 0;
                PixelResult res;
                res.rgba = pack_color(u, hit >= 0, word, mr, mg, mb, psteps);
                res.hit = hit; res.cast = cast; res.occ = occ;
                res.steps = steps; res.primary_steps = psteps;
                res.mr = mr; res.mg = mg; res.mb = mb;
                store_pixel(V.dbg, V.rgba, (uint64_t)pix, res);
                if (V.stats) {
                    if (st_vid != vid) {
                        if (st_vid >= 0) {
                            unsigned long long* s = view_of(P, st_vid).stats;
                            atomicAdd(s + VRT_STAT_RAYS, (unsigned long long)st_rays);
                            atomicAdd(s + VRT_STAT_STEPS, st_steps);
                            atomicAdd(s + VRT_STAT_HITS, (unsigned long long)st_hits);
                            atomicAdd(s + VRT_STAT_PIXELS, (unsigned long long)st_pix);
                        }
                        st_vid = vid; st_rays = 0; st_steps = 0; st_hits = 0; st_pix = 0;
                    }
                    st_rays += 1u + __popc(cast);
                    st_steps += (unsigned)steps;
                    st_hits += hit >= 0;
                    st_pix += 1;
                }
                phase = PH_IDLE;
            }
        }

        // ---- 2. hand new pixels to idle lanes from the warp's tile queue
        unsigned need = __ballot_sync(FULL, phase == PH_IDLE);
        while (need && !q_empty) {
            if (q_pos >= q_size) {
                unsigned t = 0;
                if (lane == 0) t = atomicAdd(P.tile_counter, 1u);
                t = __shfl_sync(FULL, t, 0);
                if (t >= (unsigned)P.total_tiles) {
                    q_empty = true;
                    break;
                }
                int v = 0;
                if (P.nviews > 1) {
                    while (v + 1 < P.nviews && P.views[v + 1].tile_begin <= (int)t) v++;
                }
                const ViewDev& V = view_of(P, v);
                const int lt_idx = (int)t - V.tile_begin;
                q_vid = v;
                q_x0 = (lt_idx % V.tiles_x) * P.tile_w;
                q_y0 = (lt_idx / V.tiles_x) * P.tile_h;
                q_w = V.width;
                q_h = V.height;
                q_pos = 0;
                q_size = tile_px;
            }
            const int rank = __popc(need & lt);
            const int take = min(__popc(need), q_size - q_pos);
            if (((need >> lane) & 1) && rank < take) {
                const int pos = q_pos + rank;
                const int px = q_x0 + pos % P.tile_w, py = q_y0 + pos / P.tile_w;
                if (px < q_w && py < q_h) {
                    const vrt_uniforms& u = view_of(P, q_vid).u;
                    vid = q_vid;
                    pix = py * q_w + px;
                    phase = PH_PRIMARY;
                    hit = -1; cast = 0; occ = 0; steps = 0; psteps = 0;
                    mr = mg = mb = u.ambient;
                    hpx = hpy = hpz = 0.0f;
                    hn_axis = 2; hn_s = 0;
                    o = V3{u.camPos[0], u.camPos[1], u.camPos[2]};
                    d = primary_dir(u, px, py, q_w, q_h);
                    n = u.maxSteps;
                    want = true;
                }
            }
            q_pos += take;
            need = __ballot_sync(FULL, phase == PH_IDLE);
        }

        // ---- 3. set up the new rays together
        if (want) {
            const int maxSteps = view_of(P, vid).u.maxSteps;
            start_ray(r, o, d, n, maxSteps);
            steps += r.rem;
            live = true;
        }

        const unsigned act = __ballot_sync(FULL, phase != PH_IDLE);
        if (act == 0) break;

        // ---- 4. traverse until enough lanes need a refill
        const int thr = min(P.refill_min, __popc(act));
        while (true) {
            if (live) {
                int st = dda_step(r, P);
                if (st != T_LIVE) { live = false; status = st; }
            }
            if (live) {
                int st = dda_step(r, P);
                if (st != T_LIVE) { live = false; status = st; }
            }
            const unsigned fin = __ballot_sync(FULL, phase != PH_IDLE && !live);
            if (__popc(fin) >= thr) break;
        }
    }

    if (st_vid >= 0) {
        unsigned long long* s = view_of(P, st_vid).stats;
        atomicAdd(s + VRT_STAT_RAYS, (unsigned long long)st_rays);
        atomicAdd(s + VRT_STAT_STEPS, st_steps);
        atomicAdd(s + VRT_STAT_HITS, (unsigned long long)st_hits);
        atomicAdd(s + VRT_STAT_PIXELS, (unsigned long long)st_pix);
    }
}

// ====================================================================== L2 probe

__global__ void l2_read_kernel(const uint4* __restrict__ buf, size_t n16, int iters, unsigned* sink) {
    unsigned acc = 0;
    size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int it = 0; it < iters; it++)
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
            uint4 v = __ldcg(buf + i);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    if (acc == 0x9e3779b9u) *sink = acc;  // keeps the loads alive
}

}  // namespace vrt

// ====================================================================== host side

using namespace vrt;

struct vrt_renderer {
    int device = 0;
    int num_sms = 0;
    ViewDev* d_views = nullptr;
    int views_cap = 0;
    unsigned int* d_counter = nullptr;
    uint8_t* d_staging = nullptr;
    size_t staging_bytes = 0;
};

struct vrt_batch_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ViewDev* d_views = nullptr;
    unsigned int* d_counter = nullptr;
    cudaStream_t capture_stream = nullptr;
};

static inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static int check_uniforms(const vrt_uniforms* u) {
    if (!u) return set_error(VRT_EINVAL, "NULL uniforms");
    if (u->maxSteps < 0) return set_error(VRT_EINVAL, "maxSteps %d < 0", u->maxSteps);
    return VRT_OK;
}

struct Tuning {
    int tile_w, tile_h, refill_min, blocks_per_sm;
};

static Tuning tuning_of(const vrt_render_opts* o) {
    Tuning t{8, 4, 8, 3};
    if (o) {
        if (o->tile_w > 0) t.tile_w = o->tile_w;
        if (o->tile_h > 0) t.tile_h = o->tile_h;
        if (o->refill_min > 0) t.refill_min = std::min(o->refill_min, 32);
        if (o->blocks_per_sm > 0) t.blocks_per_sm = std::min(o->blocks_per_sm, 3);
    }
    return t;
}

static int launch_mask(vrt_renderer* r, const vrt_world* w, const ViewDev* h_views, int nviews, int total_tiles,
                       const Tuning& t, const ViewDev* d_views, unsigned int* d_counter, cudaStream_t s) {
    MaskParams P;
    std::memset(&P, 0, sizeof(P));
    P.words = w->d_words;
    P.bricks = w->d_bricks;
    P.regions = w->d_regions;
    P.supers = w->d_supers;
    P.L = w->L;
    P.views = nviews == 1 ? nullptr : d_views;
    P.nviews = nviews;
    P.total_tiles = total_tiles;
    P.tile_w = t.tile_w;
    P.tile_h = t.tile_h;
    P.refill_min = t.refill_min;
    P.tile_counter = d_counter;
    P.v0 = h_views[0];
    VRT_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned), s));
    // persistent grid: blocks_per_sm CTAs of 8 warps per SM, never more warps than tiles
    int blocks = std::max(1, std::min(r->num_sms * t.blocks_per_sm, (total_tiles + 7) / 8));
    render_mask_kernel<<<blocks, 256, 0, s>>>(P);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

static void fill_view(ViewDev& v, const vrt_uniforms& u, int width, int height, uint8_t* rgba,
                      const vrt_debug_out* dbg, uint64_t* stats, const Tuning& t, int tile_begin) {
    std::memset(&v, 0, sizeof(v));
    v.u = u;
    v.width = width;
    v.height = height;
    v.tiles_x = (width + t.tile_w - 1) / t.tile_w;
    v.tile_begin = tile_begin;
    v.rgba = rgba;
    if (dbg) v.dbg = *dbg;
    v.stats = reinterpret_cast<unsigned long long*>(stats);
}

static inline int tiles_of(int width, int height, const Tuning& t) {
    return ((width + t.tile_w - 1) / t.tile_w) * ((height + t.tile_h - 1) / t.tile_h);
}

static int ensure_views(vrt_renderer* r, int n) {
    if (n <= r->views_cap) return VRT_OK;
    if (r->d_views) cudaFree(r->d_views);
    r->d_views = nullptr;
    r->views_cap = 0;
    cudaError_t e = cudaMalloc(&r->d_views, sizeof(ViewDev) * (size_t)n);
    if (e != cudaSuccess) return set_error(VRT_ENOMEM, "views: %s", cudaGetErrorString(e));
    r->views_cap = n;
    return VRT_OK;
}

extern "C" {

int vrt_renderer_create(vrt_renderer** out) {
    if (!out) return set_error(VRT_EINVAL, "out is NULL");
    *out = nullptr;
    vrt_renderer* r = new vrt_renderer();
    cudaError_t e = cudaGetDevice(&r->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, r->device);
    if (e == cudaSuccess) e = cudaMalloc(&r->d_counter, 256);
    if (e == cudaSuccess) e = cudaMemset(r->d_counter, 0, 256);
    if (e != cudaSuccess) {
        delete r;
        return cuda_error(e, "vrt_renderer_create");
    }
    *out = r;
    return VRT_OK;
}

int vrt_renderer_destroy(vrt_renderer* r) {
    if (!r) return VRT_OK;
    cudaFree(r->d_views);
    cudaFree(r->d_counter);
    cudaFree(r->d_staging);
    delete r;
    return VRT_OK;
}

int vrt_render(vrt_renderer* r, const vrt_world* w, const vrt_uniforms* u, int32_t width, int32_t height,
               uint8_t* d_rgba, const vrt_debug_out* dbg, uint64_t* d_stats, const vrt_render_opts* opts,
               void* stream) {
    if (!r || !w || !d_rgba) return set_error(VRT_EINVAL, "NULL renderer, world or image");
    int st = check_uniforms(u);
    if (st) return st;
    if (width < 1 || height < 1 || width > 32768 || height > 32768)
        return set_error(VRT_EINVAL, "image %d x %d out of range", width, height);
    int kernel = opts ? opts->kernel : VRT_KERNEL_AUTO;
    if (kernel == VRT_KERNEL_AUTO) kernel = w->has_depth_field ? VRT_KERNEL_WORD : VRT_KERNEL_BITMASK;
    if (kernel == VRT_KERNEL_BITMASK && w->has_depth_field)
        return set_error(VRT_ESTATE, "the world holds depth-field words, which only the word kernel follows");
    if (kernel == VRT_KERNEL_WORD) {
        WordParams p;
        std::memset(&p, 0, sizeof(p));
        p.u = *u;
        p.width = width;
        p.height = height;
        p.rgba = d_rgba;
        if (dbg) p.dbg = *dbg;
        p.stats = reinterpret_cast<unsigned long long*>(d_stats);
        dim3 grid((width + 15) / 16, (height + 7) / 8);
        render_word_kernel<<<grid, 128, 0, S(stream)>>>(w->d_words, w->L, p);
        VRT_CUDA(cudaGetLastError());
        return VRT_OK;
    }
    if (kernel != VRT_KERNEL_BITMASK) return set_error(VRT_EINVAL, "unknown kernel %d", kernel);
    Tuning t = tuning_of(opts);
    ViewDev v;
    fill_view(v, *u, width, height, d_rgba, dbg, d_stats, t, 0);
    return launch_mask(r, w, &v, 1, tiles_of(width, height, t), t, nullptr, r->d_counter, S(stream));
}

int vrt_render_to_host(vrt_renderer* r, const vrt_world* w, const vrt_uniforms* u, int32_t width, int32_t height,
                       uint8_t* host_rgba, const vrt_render_opts* opts, void* stream) {
    if (!r || !host_rgba) return set_error(VRT_EINVAL, "NULL renderer or image");
    if (width < 1 || height < 1 || width > 32768 || height > 32768)
        return set_error(VRT_EINVAL, "image %d x %d out of range", width, height);
    size_t bytes = (size_t)width * height * 4;
    if (bytes > r->staging_bytes) {
        cudaFree(r->d_staging);
        r->d_staging = nullptr;
        r->staging_bytes = 0;
        cudaError_t e = cudaMalloc(&r->d_staging, bytes);
        if (e != cudaSuccess) return set_error(VRT_ENOMEM, "staging image: %s", cudaGetErrorString(e));
        r->staging_bytes = bytes;
    }
    int st = vrt_render(r, w, u, width, height, r->d_staging, nullptr, nullptr, opts, stream);
    if (st) return st;
    VRT_CUDA(cudaMemcpyAsync(host_rgba, r->d_staging, bytes, cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    return VRT_OK;
}

static int build_batch(const vrt_view* views, int32_t count, const Tuning& t, std::vector<ViewDev>& hv,
                       const vrt_world** world_out, int* total_out) {
    if (!views || count < 1) return set_error(VRT_EINVAL, "empty batch");
    const vrt_world* w = views[0].world;
    if (!w) return set_error(VRT_EINVAL, "view 0 has no world");
    if (w->has_depth_field) return set_error(VRT_ESTATE, "batched rendering needs a world without depth-field words");
    hv.resize(count);
    int tiles = 0;
    for (int i = 0; i < count; i++) {
        const vrt_view& v = views[i];
        if (v.world != w) return set_error(VRT_EINVAL, "view %d renders another world; one batch = one world", i);
        if (!v.d_rgba || v.width < 1 || v.height < 1 || v.width > 32768 || v.height > 32768)
            return set_error(VRT_EINVAL, "view %d: bad image", i);
        int st = check_uniforms(&v.uniforms);
        if (st) return st;
        fill_view(hv[i], v.uniforms, v.width, v.height, v.d_rgba, nullptr, v.d_stats, t, tiles);
        tiles += tiles_of(v.width, v.height, t);
    }
    *world_out = w;
    *total_out = tiles;
    return VRT_OK;
}

int vrt_render_batch(vrt_renderer* r, const vrt_view* views, int32_t count, const vrt_render_opts* opts,
                     void* stream) {
    if (!r) return set_error(VRT_EINVAL, "NULL renderer");
    Tuning t = tuning_of(opts);
    std::vector<ViewDev> hv;
    const vrt_world* w = nullptr;
    int total = 0;
    int st = build_batch(views, count, t, hv, &w, &total);
    if (st) return st;
    if (count > 1) {
        st = ensure_views(r, count);
        if (st) return st;
        // pageable source: the copy is staged before the call returns, so hv may go
        VRT_CUDA(cudaMemcpyAsync(r->d_views, hv.data(), sizeof(ViewDev) * count, cudaMemcpyHostToDevice, S(stream)));
    }
    return launch_mask(r, w, hv.data(), count, total, t, r->d_views, r->d_counter, S(stream));
}

int vrt_batch_graph_create(vrt_renderer* r, const vrt_view* views, int32_t count, const vrt_render_opts* opts,
                           void* stream, vrt_batch_graph** out) {
    if (!r || !out) return set_error(VRT_EINVAL, "NULL argument");
    *out = nullptr;
    Tuning t = tuning_of(opts);
    std::vector<ViewDev> hv;
    const vrt_world* w = nullptr;
    int total = 0;
    int st = build_batch(views, count, t, hv, &w, &total);
    if (st) return st;
    vrt_batch_graph* g = new vrt_batch_graph();
    cudaError_t e = cudaMalloc(&g->d_views, sizeof(ViewDev) * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&g->d_counter, 256);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->d_views, hv.data(), sizeof(ViewDev) * count, cudaMemcpyHostToDevice, S(stream));
    if (e == cudaSuccess) e = cudaStreamSynchronize(S(stream));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        vrt_batch_graph_destroy(g);
        return cuda_error(e, "vrt_batch_graph_create");
    }
    e = cudaStreamBeginCapture(g->capture_stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        vrt_batch_graph_destroy(g);
        return cuda_error(e, "cudaStreamBeginCapture");
    }
    st = launch_mask(r, w, hv.data(), count, total, t, g->d_views, g->d_counter, g->capture_stream);
    e = cudaStreamEndCapture(g->capture_stream, &g->graph);
    if (st || e != cudaSuccess) {
        vrt_batch_graph_destroy(g);
        return st ? st : cuda_error(e, "cudaStreamEndCapture");
    }
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        vrt_batch_graph_destroy(g);
        return cuda_error(e, "cudaGraphInstantiate");
    }
    *out = g;
    return VRT_OK;
}

int vrt_batch_graph_launch(vrt_batch_graph* g, void* stream) {
    if (!g || !g->exec) return set_error(VRT_EINVAL, "NULL graph");
    VRT_CUDA(cudaGraphLaunch(g->exec, S(stream)));
    return VRT_OK;
}

int vrt_batch_graph_destroy(vrt_batch_graph* g) {
    if (!g) return VRT_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->capture_stream) cudaStreamDestroy(g->capture_stream);
    cudaFree(g->d_views);
    cudaFree(g->d_counter);
    delete g;
    return VRT_OK;
}

int vrt_probe_l2_read_gbs(uint64_t bytes, int32_t iters, double* gbs_out) {
    if (!gbs_out || bytes < 4096 || iters < 1) return set_error(VRT_EINVAL, "bad probe arguments");
    bytes &= ~(uint64_t)15;
    void* buf = nullptr;
    unsigned* sink = nullptr;
    VRT_CUDA(cudaMalloc(&buf, bytes));
    VRT_CUDA(cudaMalloc(&sink, sizeof(unsigned)));
    VRT_CUDA(cudaMemset(buf, 1, bytes));
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    l2_read_kernel<<<sms * 4, 512>>>(reinterpret_cast<const uint4*>(buf), bytes / 16, 2, sink);  // warm
    cudaEventRecord(a);
    l2_read_kernel<<<sms * 4, 512>>>(reinterpret_cast<const uint4*>(buf), bytes / 16, iters, sink);
    cudaEventRecord(b);
    cudaError_t e = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(buf);
    cudaFree(sink);
    if (e != cudaSuccess) return cuda_error(e, "l2 probe");
    *gbs_out = (double)bytes * iters / (ms * 1e-3) / 1e9;
    return VRT_OK;
}

}  // extern "C"
