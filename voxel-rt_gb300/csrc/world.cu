// Device-resident worlds: the voxel words (the reference's SSBO), the derived occupancy
// hierarchy, and the edit kernels that replace the reference's CPU world code:
//   removeSphere  level.cpp:30-56        -> remove_sphere_kernel + mask refresh + depth refresh
//   fixDepthField render.cpp:226-253     -> fix_depth_field_kernel
//   placeVoxel    render.cpp:256-262     -> place_voxel_kernel
//   initVoxels    level.cpp:82-138       -> init_reference_layers_kernel + init_reference_trees_kernel
//   updateGeometry/updatePartialGeometry render.cpp:199-223 -> vrt_world_upload (+ mask refresh)
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "vrt_internal.h"

namespace vrt {

Layout make_layout(int W, int H) {
    Layout L{};
    L.W = W;
    L.H = H;
    L.RW = (W + 15) / 16;
    L.RH = (H + 15) / 16;
    L.SW = (W + 63) / 64;
    L.SH = (H + 63) / 64;
    L.RWp = 4 * L.SW;
    L.RHp = 4 * L.SH;
    L.BWp = 16 * L.SW;
    L.BHp = 16 * L.SH;
    L.n_words = (uint64_t)W * H * W;
    L.n_supers = (uint64_t)L.SW * L.SH * L.SW;
    L.n_regions = 64 * L.n_supers;
    L.n_bricks = 64 * L.n_regions;
    return L;
}

// ------------------------------------------------------------------ mask kernels

// One thread per brick of the brick box [b0, b1): OR of (word >= 0) over its 4x4x4
// voxels; any word < -1 raises the depth-field flag.
__global__ void brick_mask_kernel(const int32_t* __restrict__ words, uint64_t* __restrict__ bricks, int* flag,
                                  int* aabb, Layout L, int bx0, int by0, int bz0, int nbx, int nby, int nbz) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t total = (uint64_t)nbx * nby * nbz;
    if (t >= total) return;
    int bx = bx0 + (int)(t % nbx);
    int by = by0 + (int)((t / nbx) % nby);
    int bz = bz0 + (int)(t / ((uint64_t)nbx * nby));
    uint64_t m = 0;
    bool depth = false;
    const int x0 = bx * 4;
    const bool vec = (x0 + 4 <= L.W) && ((L.W & 3) == 0);
    for (int dz = 0; dz < 4; dz++) {
        int z = bz * 4 + dz;
        if (z >= L.W) break;
        for (int dy = 0; dy < 4; dy++) {
            int y = by * 4 + dy;
            if (y >= L.H) break;
            const int32_t* row = words + ((uint64_t)z * L.H + y) * L.W;
            int v[4];
            if (vec) {
                int4 q = __ldg(reinterpret_cast<const int4*>(row + x0));
                v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
            } else {
                for (int dx = 0; dx < 4; dx++) v[dx] = (x0 + dx < L.W) ? __ldg(row + x0 + dx) : -1;
            }
            for (int dx = 0; dx < 4; dx++) {
                if (v[dx] >= 0) m |= 1ull << (dx + 4 * dy + 16 * dz);
                depth |= (v[dx] < -1);
            }
        }
    }
    bricks[brick_index(L, bx, by, bz)] = m;
    if (depth) atomicOr(flag, 1);
    // grow the solid bounding box by this brick (one atomic per warp and bound)
    const unsigned mask = __activemask();
    int v[6];
    if (m) {
        v[0] = 4 * bx; v[1] = 4 * by; v[2] = 4 * bz;
        v[3] = 4 * bx + 3; v[4] = 4 * by + 3; v[5] = 4 * bz + 3;
    } else {
        v[0] = v[1] = v[2] = INT_MAX;
        v[3] = v[4] = v[5] = INT_MIN;
    }
    for (int i = 0; i < 3; i++) v[i] = __reduce_min_sync(mask, v[i]);
    for (int i = 3; i < 6; i++) v[i] = __reduce_max_sync(mask, v[i]);
    if ((threadIdx.x & 31) == (__ffs(mask) - 1) && v[0] != INT_MAX) {
        for (int i = 0; i < 3; i++) atomicMin(aabb + i, v[i]);
        for (int i = 3; i < 6; i++) atomicMax(aabb + i, v[i]);
    }
}

__global__ void reset_aabb_kernel(int* aabb) {
    if (threadIdx.x < 3) aabb[threadIdx.x] = INT_MAX;
    else if (threadIdx.x < 6) aabb[threadIdx.x] = INT_MIN;
}

// One thread per node of the parent box: bit i set when child i is non-zero.
// children are stored as 64 consecutive uint64 per parent (region-major / super-major).
__global__ void parent_mask_kernel(const uint64_t* __restrict__ child, uint64_t* __restrict__ parent,
                                   int px0, int py0, int pz0, int npx, int npy, int npz, Layout L, int level) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t total = (uint64_t)npx * npy * npz;
    if (t >= total) return;
    int px = px0 + (int)(t % npx);
    int py = py0 + (int)((t / npx) % npy);
    int pz = pz0 + (int)(t / ((uint64_t)npx * npy));
    uint64_t slot = level == 1 ? region_index(L, px, py, pz) : super_index(L, px, py, pz);
    uint64_t m = 0;
    if (level == 1) {  // the region's 4x4x4 bricks: 16 rows of 4 consecutive slots
        for (int lz = 0; lz < 4; lz++)
            for (int ly = 0; ly < 4; ly++) {
                const uint64_t* row = child + brick_index(L, 4 * px, 4 * py + ly, 4 * pz + lz);
                for (int lx = 0; lx < 4; lx++) m |= (uint64_t)(row[lx] != 0) << (lx + 4 * ly + 16 * lz);
            }
    } else {  // a super block's 64 regions are consecutive
        const uint64_t* c = child + slot * 64;
        for (int i = 0; i < 64; i += 2) {
            ulonglong2 q = *reinterpret_cast<const ulonglong2*>(c + i);
            m |= (uint64_t)(q.x != 0) << i;
            m |= (uint64_t)(q.y != 0) << (i + 1);
        }
    }
    parent[slot] = m;
}

static inline unsigned blocks_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// One 1-D pass of the capped Chebyshev distance transform over the region grid:
//   out(p) = min over |k| <= cap of max(|k|, in(p + k e_axis)),
// where in() of the first pass is 0 for a non-empty region and cap+1 for an empty one, and
// regions outside the padded grid are empty.  Three passes (x, y, z) give the L-inf distance.
__global__ void cheb_pass_kernel(const uint64_t* __restrict__ occ, const uint8_t* __restrict__ in,
                                 uint8_t* __restrict__ out, Layout L, int axis, int first) {
    const int DX = L.RWp, DY = L.RHp;
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)DX * DY * DX) return;
    const int x = (int)(t % DX), y = (int)((t / DX) % DY), z = (int)(t / ((uint64_t)DX * DY));
    const int cap = kDistCap;
    int best = cap + 1;
    for (int k = -cap; k <= cap; k++) {
        int qx = x + (axis == 0 ? k : 0), qy = y + (axis == 1 ? k : 0), qz = z + (axis == 2 ? k : 0);
        if (qx < 0 || qy < 0 || qz < 0 || qx >= DX || qy >= DY || qz >= DX) continue;
        const int v = first ? (occ[region_index(L, qx, qy, qz)] != 0 ? 0 : cap + 1) : in[region_linear(L, qx, qy, qz)];
        int a = k < 0 ? -k : k;
        best = min(best, max(a, v));
    }
    out[region_linear(L, x, y, z)] = (uint8_t)min(best, cap);
}

// One axis pass of the directed brick distances, all eight octants at once (one byte
// each): out_o(b) = min over j in [0, cap] of max(j, in_o(b + sgn_o * j * e_axis)), where
// sgn_o is + for octants with bit `axis` set.  The first pass reads occupancy (0 for a
// non-empty brick, cap otherwise).  Bytes are processed four at a time with the SIMD
// byte min/max intrinsics; values never exceed the cap, which stands for "cap or more".
__global__ void dir_pass_kernel(const uint64_t* __restrict__ occ, const uint64_t* __restrict__ in,
                                uint64_t* __restrict__ out, Layout L, int axis, int x0, int y0, int z0, int nx,
                                int ny, int nz, int first) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)nx * ny * nz) return;
    const int x = x0 + (int)(t % nx), y = y0 + (int)((t / nx) % ny), z = z0 + (int)(t / ((uint64_t)nx * ny));
    const int c = axis == 0 ? x : (axis == 1 ? y : z);
    const int D = axis == 1 ? L.BHp : L.BWp;
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)L.BWp : (int64_t)L.BWp * L.BHp);
    const int64_t self = (int64_t)brick_index(L, x, y, z);
    const uint32_t capb = 0x01010101u * kDistCap;
    uint64_t res[2];
    for (int d = 0; d < 2; d++) {
        const int sg = d == 0 ? 1 : -1;
        uint32_t lo = capb, hi = capb;
        for (int j = 0; j <= kDistCap; j++) {
            const int q = c + sg * j;
            if (q < 0 || q >= D) break;
            const int64_t qi = self + sg * j * stride;
            const uint64_t v = first ? (occ[qi] ? 0ull : ((uint64_t)capb << 32 | capb)) : in[qi];
            const uint32_t jj = 0x01010101u * (uint32_t)j;
            lo = __vminu4(lo, __vmaxu4((uint32_t)v, jj));
            hi = __vminu4(hi, __vmaxu4((uint32_t)(v >> 32), jj));
            if (__vcmpleu4(lo, jj) == 0xFFFFFFFFu && __vcmpleu4(hi, jj) == 0xFFFFFFFFu) break;  // nothing drops below j
        }
        res[d] = (uint64_t)hi << 32 | lo;
    }
    const uint64_t plus = axis == 0 ? 0xFF00FF00FF00FF00ull : (axis == 1 ? 0xFFFF0000FFFF0000ull : 0xFFFFFFFF00000000ull);
    out[self] = (res[0] & plus) | (res[1] & ~plus);
}

// One thread per brick of the whole grid: bit x+4y+16z set when the voxel's word is not
// -1, i.e. the cells where the shader's loop stops to hit (word >= 0) or to jump (a
// depth-field word, fshader.glsl:114-121).  Voxels outside the world are clear.
__global__ void stop_mask_kernel(const int32_t* __restrict__ words, uint64_t* __restrict__ stop, Layout L) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.n_bricks) return;
    const int bx = (int)(t % L.BWp), by = (int)((t / L.BWp) % L.BHp), bz = (int)(t / ((uint64_t)L.BWp * L.BHp));
    uint64_t m = 0;
    for (int dz = 0; dz < 4; dz++) {
        const int z = bz * 4 + dz;
        if (z >= L.W) break;
        for (int dy = 0; dy < 4; dy++) {
            const int y = by * 4 + dy;
            if (y >= L.H) break;
            const int32_t* row = words + ((uint64_t)z * L.H + y) * L.W;
            for (int dx = 0; dx < 4; dx++) {
                const int x = bx * 4 + dx;
                if (x < L.W && __ldg(row + x) != -1) m |= 1ull << (dx + 4 * dy + 16 * dz);
            }
        }
    }
    stop[t] = m;  // t is the linear brick slot bx + BWp*(by + BHp*bz)
}

static int dir_passes(vrt_world* w, const uint64_t* occ, uint8_t* dst8, int bx0, int by0, int bz0, int bx1, int by1,
                      int bz1, cudaStream_t s) {
    const Layout& L = w->L;
    const int cap = kDistCap;
    auto clampbox = [&](int& a0, int& a1, int lim) { a0 = std::max(a0, 0); a1 = std::min(a1, lim); };
    int X0 = bx0, X1 = bx1, Y0 = by0, Y1 = by1, Z0 = bz0, Z1 = bz1;
    clampbox(X0, X1, L.BWp); clampbox(Y0, Y1, L.BHp); clampbox(Z0, Z1, L.BWp);
    if (X0 >= X1 || Y0 >= Y1 || Z0 >= Z1) return VRT_OK;
    int ya0 = Y0 - cap, ya1 = Y1 + cap, za0 = Z0 - cap, za1 = Z1 + cap;
    clampbox(ya0, ya1, L.BHp); clampbox(za0, za1, L.BWp);
    uint64_t* ta = reinterpret_cast<uint64_t*>(w->d_tmp_a);
    uint64_t* tb = reinterpret_cast<uint64_t*>(w->d_tmp_b);
    uint64_t n = (uint64_t)(X1 - X0) * (ya1 - ya0) * (za1 - za0);
    dir_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(occ, nullptr, ta, L, 0, X0, ya0, za0, X1 - X0, ya1 - ya0,
                                                       za1 - za0, 1);
    n = (uint64_t)(X1 - X0) * (Y1 - Y0) * (za1 - za0);
    dir_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(occ, ta, tb, L, 1, X0, Y0, za0, X1 - X0, Y1 - Y0, za1 - za0,
                                                       0);
    n = (uint64_t)(X1 - X0) * (Y1 - Y0) * (Z1 - Z0);
    dir_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(occ, tb, reinterpret_cast<uint64_t*>(dst8), L, 2, X0, Y0, Z0,
                                                       X1 - X0, Y1 - Y0, Z1 - Z0, 0);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

static int region_passes(vrt_world* w, cudaStream_t s) {
    const Layout& L = w->L;
    const uint64_t n = (uint64_t)L.RWp * L.RHp * L.RWp;
    cheb_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w->d_regions, nullptr, w->d_tmp_a, L, 0, 1);
    cheb_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w->d_regions, w->d_tmp_a, w->d_tmp_b, L, 1, 0);
    cheb_pass_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w->d_regions, w->d_tmp_b, w->d_rdist, L, 2, 0);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

// Directed distances of every brick within kDistCap bricks of the changed brick box, and
// the distances of all regions (a few thousand to a few hundred thousand bytes).
static int refresh_distances(vrt_world* w, int bx0, int by0, int bz0, int bx1, int by1, int bz1, cudaStream_t s) {
    const int cap = kDistCap;
    int st = dir_passes(w, w->d_bricks, w->d_bdir, bx0 - cap, by0 - cap, bz0 - cap, bx1 + cap, by1 + cap, bz1 + cap,
                        s);
    if (st) return st;
    return region_passes(w, s);
}

int refresh_stop(vrt_world* w, cudaStream_t s) {
    if (!w->stop_stale) {
        VRT_CUDA(cudaStreamWaitEvent(s, w->stop_ready, 0));  // the last rebuild, on whichever stream
        return VRT_OK;
    }
    const Layout& L = w->L;
    if (!w->d_stop) {
        cudaError_t e = cudaMalloc(&w->d_stop, L.n_bricks * 8);
        if (e == cudaSuccess) e = cudaMalloc(&w->d_sdir, L.n_bricks * 8);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->stop_ready, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaFree(w->d_stop);
            cudaFree(w->d_sdir);
            if (w->stop_ready) cudaEventDestroy(w->stop_ready);
            w->d_stop = nullptr;
            w->d_sdir = nullptr;
            w->stop_ready = nullptr;
            return set_error(VRT_ENOMEM, "stop masks: %s", cudaGetErrorString(e));
        }
        w->device_bytes += L.n_bricks * 16;
    }
    stop_mask_kernel<<<blocks_for(L.n_bricks, 256), 256, 0, s>>>(w->d_words, w->d_stop, L);
    VRT_CUDA(cudaGetLastError());
    const int st = dir_passes(w, w->d_stop, w->d_sdir, 0, 0, 0, L.BWp, L.BHp, L.BWp, s);
    if (st) return st;
    VRT_CUDA(cudaEventRecord(w->stop_ready, s));
    w->stop_stale = false;
    return VRT_OK;
}

// The words of the box [x0,x1)x[y0,y1)x[z0,z1) changed: the z-major copy must follow there.
static void mark_words_z(vrt_world* w, int x0, int y0, int z0, int x1, int y1, int z1) {
    int* b = w->z_dirty;
    if (b[0] >= b[3]) {
        b[0] = x0; b[1] = y0; b[2] = z0; b[3] = x1; b[4] = y1; b[5] = z1;
        return;
    }
    b[0] = std::min(b[0], x0); b[1] = std::min(b[1], y0); b[2] = std::min(b[2], z0);
    b[3] = std::max(b[3], x1); b[4] = std::max(b[4], y1); b[5] = std::max(b[5], z1);
}

// Whole-world copy with x and z swapped, through 32x32 tiles of the (x, z) plane of each y
// so that both the reads (along x) and the writes (along z) are coalesced.
__global__ void words_z_transpose_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, Layout L) {
    __shared__ int32_t tile[32][33];
    const uint64_t W = L.W, WH = (uint64_t)L.W * L.H;
    const int y = blockIdx.z;
    const int x0 = blockIdx.x * 32, z0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += 8) {  // read: x along threadIdx.x
        const int x = x0 + threadIdx.x, z = z0 + j;
        if (x < L.W && z < L.W) tile[j][threadIdx.x] = in[x + W * y + WH * z];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += 8) {  // write: z along threadIdx.x
        const int z = z0 + threadIdx.x, x = x0 + j;
        if (x < L.W && z < L.W) out[z + W * y + WH * x] = tile[threadIdx.x][j];
    }
}

// The same for the words of one box (edit-sized), one thread per word.
__global__ void words_z_box_kernel(const int32_t* __restrict__ in, int32_t* __restrict__ out, Layout L, int x0,
                                   int y0, int z0, int nx, int ny, int nz) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)nx * ny * nz) return;
    const uint64_t W = L.W, WH = (uint64_t)L.W * L.H;
    const uint64_t x = x0 + t % nx, y = y0 + (t / nx) % ny, z = z0 + t / ((uint64_t)nx * ny);
    out[z + W * y + WH * x] = in[x + W * y + WH * z];
}

int refresh_words_z(vrt_world* w, cudaStream_t s) {
    const Layout& L = w->L;
    int* b = w->z_dirty;
    if (w->d_words_z && b[0] >= b[3]) {
        VRT_CUDA(cudaStreamWaitEvent(s, w->z_ready, 0));  // the last update, on whichever stream
        return VRT_OK;
    }
    if (!w->d_words_z) {
        cudaError_t e = cudaMalloc(&w->d_words_z, L.n_words * sizeof(int32_t));
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->z_ready, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            cudaGetLastError();
            cudaFree(w->d_words_z);
            if (w->z_ready) cudaEventDestroy(w->z_ready);
            w->d_words_z = nullptr;
            w->z_ready = nullptr;
            return set_error(VRT_ENOMEM, "z-major words: %s", cudaGetErrorString(e));
        }
        w->device_bytes += L.n_words * sizeof(int32_t);
        dim3 grid((L.W + 31) / 32, (L.W + 31) / 32, L.H);
        words_z_transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(w->d_words, w->d_words_z, L);
    } else {
        const uint64_t n = (uint64_t)(b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2]);
        words_z_box_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w->d_words, w->d_words_z, L, b[0], b[1], b[2],
                                                               b[3] - b[0], b[4] - b[1], b[5] - b[2]);
    }
    VRT_CUDA(cudaGetLastError());
    VRT_CUDA(cudaEventRecord(w->z_ready, s));
    b[0] = b[3] = 0;
    return VRT_OK;
}

int refresh_masks_box(vrt_world* w, int x0, int y0, int z0, int x1, int y1, int z1, cudaStream_t s) {
    const Layout& L = w->L;
    x0 = std::max(x0, 0); y0 = std::max(y0, 0); z0 = std::max(z0, 0);
    x1 = std::min(x1, L.W); y1 = std::min(y1, L.H); z1 = std::min(z1, L.W);
    if (x0 >= x1 || y0 >= y1 || z0 >= z1) return VRT_OK;
    w->stop_stale = true;
    if (w->d_words_z) mark_words_z(w, x0, y0, z0, x1, y1, z1);
    int bx0 = x0 >> 2, by0 = y0 >> 2, bz0 = z0 >> 2;
    int bx1 = (x1 + 3) >> 2, by1 = (y1 + 3) >> 2, bz1 = (z1 + 3) >> 2;
    uint64_t nb = (uint64_t)(bx1 - bx0) * (by1 - by0) * (bz1 - bz0);
    // a refresh of the whole world recomputes the solid bounding box; a partial one only grows it
    if (x0 == 0 && y0 == 0 && z0 == 0 && x1 == L.W && y1 == L.H && z1 == L.W) reset_aabb_kernel<<<1, 32, 0, s>>>(w->d_aabb);
    brick_mask_kernel<<<blocks_for(nb, 256), 256, 0, s>>>(w->d_words, w->d_bricks, w->d_flag, w->d_aabb, L, bx0, by0,
                                                           bz0, bx1 - bx0, by1 - by0, bz1 - bz0);
    int rx0 = bx0 >> 2, ry0 = by0 >> 2, rz0 = bz0 >> 2;
    int rx1 = (bx1 + 3) >> 2, ry1 = (by1 + 3) >> 2, rz1 = (bz1 + 3) >> 2;
    uint64_t nr = (uint64_t)(rx1 - rx0) * (ry1 - ry0) * (rz1 - rz0);
    parent_mask_kernel<<<blocks_for(nr, 256), 256, 0, s>>>(w->d_bricks, w->d_regions, rx0, ry0, rz0, rx1 - rx0,
                                                           ry1 - ry0, rz1 - rz0, L, 1);
    int sx0 = rx0 >> 2, sy0 = ry0 >> 2, sz0 = rz0 >> 2;
    int sx1 = (rx1 + 3) >> 2, sy1 = (ry1 + 3) >> 2, sz1 = (rz1 + 3) >> 2;
    uint64_t ns = (uint64_t)(sx1 - sx0) * (sy1 - sy0) * (sz1 - sz0);
    parent_mask_kernel<<<blocks_for(ns, 256), 256, 0, s>>>(w->d_regions, w->d_supers, sx0, sy0, sz0, sx1 - sx0,
                                                           sy1 - sy0, sz1 - sz0, L, 2);
    VRT_CUDA(cudaGetLastError());
    return refresh_distances(w, bx0, by0, bz0, bx1, by1, bz1, s);
}

int refresh_masks(vrt_world* w, uint64_t first, uint64_t count, cudaStream_t s) {
    if (count == 0) return VRT_OK;
    const Layout& L = w->L;
    uint64_t last = first + count - 1;
    uint64_t plane = (uint64_t)L.W * L.H;
    int z0 = (int)(first / plane), z1 = (int)(last / plane);
    if (z0 != z1) return refresh_masks_box(w, 0, 0, z0, L.W, L.H, z1 + 1, s);
    int y0 = (int)((first % plane) / L.W), y1 = (int)((last % plane) / L.W);
    if (y0 != y1) return refresh_masks_box(w, 0, y0, z0, L.W, y1 + 1, z0 + 1, s);
    int x0 = (int)(first % L.W), x1 = (int)(last % L.W);
    return refresh_masks_box(w, x0, y0, z0, x1 + 1, y0 + 1, z0 + 1, s);
}

// Copy the device solid bounding box to the host copy the render launches pass on
// (synchronises the stream).
static int read_aabb(vrt_world* w, cudaStream_t s) {
    int bb[8];
    VRT_CUDA(cudaMemcpyAsync(bb, w->d_aabb, sizeof(bb), cudaMemcpyDeviceToHost, s));
    VRT_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < 6; i++) w->h_aabb[i] = bb[i];
    return VRT_OK;
}

// ------------------------------------------------------------------ edits

// removeSphere's first loop (level.cpp:31-42): voxels with offsets in [-r,r)^3,
// x*x+y*y+z*z < r*r and inside the world become air.
__global__ void remove_sphere_kernel(int32_t* __restrict__ words, Layout L, int cx, int cy, int cz, int r) {
    int n = 2 * r;
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)n * n * n) return;
    int x = (int)(t % n) - r, y = (int)((t / n) % n) - r, z = (int)(t / ((uint64_t)n * n)) - r;
    int ax = x + cx, ay = y + cy, az = z + cz;
    if (ax < L.W && ay < L.H && az < L.W && ax >= 0 && ay >= 0 && az >= 0 && x * x + y * y + z * z < r * r)
        words[(uint64_t)ax + (uint64_t)L.W * ay + (uint64_t)L.W * L.H * az] = -1;
}

__global__ void place_voxel_kernel(int32_t* words, Layout L, int x, int y, int z, int32_t v) {
    if (x >= 0 && y >= 0 && z >= 0 && x < L.W && y < L.H && z < L.W)
        words[(uint64_t)x + (uint64_t)L.W * y + (uint64_t)L.W * L.H * z] = v;
}

// Depth-field offsets of computeDepthIndices (render.cpp:66-100), reduced to what
// fixDepthField (render.cpp:226-253) can use.  fixDepthField keeps, over the solid
// neighbours in the radius-7 sphere whose shrunk distance d beats the running value
// (start -6), the value (d <= -2 ? d : 0); the running value only grows and that map
// is monotone, so the result is g(max d) over solid neighbours with d > -6, whatever
// the visiting order.  The table therefore holds the sphere offsets with d > -6 sorted
// by decreasing d, and the kernel stops at the first solid neighbour.
struct DepthOff {
    float dist;
    int8_t x, y, z, pad;
};
__constant__ DepthOff c_depth_offs[1536];  // 1413 offsets of the radius-7 sphere have d > -6
__constant__ int c_depth_count;
__device__ DepthOff g_depth_offs[1536];    // the same table, read by the lanes of a warp at once
static std::once_flag g_depth_once;
static int g_depth_count = 0;
static std::vector<DepthOff> g_depth_table;

static void build_depth_table() {
    const int R = 7;  // DEPTH_FIELD_RADIUS, render.hpp:7
    std::vector<DepthOff> v;
    for (int z = -R; z <= R; z++)
        for (int y = -R; y <= R; y++)
            for (int x = -R; x <= R; x++) {
                if (x * x + y * y + z * z > R * R) continue;
                int xd = x - (x > 0) + (x < 0), yd = y - (y > 0) + (y < 0), zd = z - (z > 0) + (z < 0);
                // render.cpp:81: dist = -sqrt(int) through double sqrt, stored as float
                float dist = (float)(-std::sqrt((double)(xd * xd + yd * yd + zd * zd)));
                if (dist > (float)(-R + 1)) v.push_back(DepthOff{dist, (int8_t)x, (int8_t)y, (int8_t)z, 0});
            }
    std::stable_sort(v.begin(), v.end(), [](const DepthOff& a, const DepthOff& b) { return a.dist > b.dist; });
    g_depth_table = v;
    g_depth_count = (int)v.size();
}

static int ensure_depth_table() {
    std::call_once(g_depth_once, build_depth_table);
    // constant memory is per device: upload each time (cheap, 8 KB) to stay correct on any device
    VRT_CUDA(cudaMemcpyToSymbol(c_depth_offs, g_depth_table.data(), g_depth_table.size() * sizeof(DepthOff)));
    VRT_CUDA(cudaMemcpyToSymbol(g_depth_offs, g_depth_table.data(), g_depth_table.size() * sizeof(DepthOff)));
    VRT_CUDA(cudaMemcpyToSymbol(c_depth_count, &g_depth_count, sizeof(int)));
    return VRT_OK;
}

// fixDepthField (render.cpp:226-253) for every voxel of the box, or of the sphere
// x*x+y*y+z*z < r2*r2 around (cx,cy,cz) when r2 > 0 (removeSphere's second loop,
// level.cpp:43-55).  Neighbours outside the world count as not solid (the reference
// reads voxels[-1] there).  Only air words are written and only solidity is read, so
// voxels of one launch do not interact.
__global__ void fix_depth_field_kernel(int32_t* words, Layout L, int x0, int y0, int z0, int nx,
                                       int ny, int nz, int cx, int cy, int cz, int r2) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (uint64_t)nx * ny * nz) return;
    int x = x0 + (int)(t % nx), y = y0 + (int)((t / nx) % ny), z = z0 + (int)(t / ((uint64_t)nx * ny));
    if (x < 0 || y < 0 || z < 0 || x >= L.W || y >= L.H || z >= L.W) return;
    if (r2 > 0) {
        int ox = x - cx, oy = y - cy, oz = z - cz;
        if (ox * ox + oy * oy + oz * oz >= r2 * r2) return;
    }
    uint64_t idx = (uint64_t)x + (uint64_t)L.W * y + (uint64_t)L.W * L.H * z;
    if (words[idx] >= 0) return;
    float nearest = -6.0f;  // -DEPTH_FIELD_RADIUS + 1
    const int n = c_depth_count;
    for (int i = 0; i < n; i++) {
        DepthOff o = c_depth_offs[i];
        int qx = x + o.x, qy = y + o.y, qz = z + o.z;
        if (qx < 0 || qy < 0 || qz < 0 || qx >= L.W || qy >= L.H || qz >= L.W) continue;
        // plain load: this launch writes other air words of the same array
        if (words[(uint64_t)qx + (uint64_t)L.W * qy + (uint64_t)L.W * L.H * qz] >= 0) {
            nearest = o.dist <= -2.0f ? o.dist : 0.0f;
            break;
        }
    }
    if (nearest < 0.0f) words[idx] = __float_as_int(nearest);
}

// fix_depth_field_kernel with one warp per voxel, for edit-sized boxes: one thread per
// voxel leaves most SMs idle there while each thread walks the offset table in turn.  The
// lanes test 32 consecutive table offsets at a time and a ballot picks the first solid
// one in table order -- the offset the one-thread loop stops at -- so the words written
// are the same.
__global__ void fix_depth_field_warp_kernel(int32_t* words, Layout L, int x0, int y0, int z0, int nx, int ny,
                                            int nz, int cx, int cy, int cz, int r2) {
    const uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // this warp's voxel
    const int lane = threadIdx.x & 31;
    if (t >= (uint64_t)nx * ny * nz) return;  // the returns before the ballot are warp-uniform
    const int x = x0 + (int)(t % nx), y = y0 + (int)((t / nx) % ny), z = z0 + (int)(t / ((uint64_t)nx * ny));
    if (x < 0 || y < 0 || z < 0 || x >= L.W || y >= L.H || z >= L.W) return;
    if (r2 > 0) {
        const int ox = x - cx, oy = y - cy, oz = z - cz;
        if (ox * ox + oy * oy + oz * oz >= r2 * r2) return;
    }
    const uint64_t idx = (uint64_t)x + (uint64_t)L.W * y + (uint64_t)L.W * L.H * z;
    if (words[idx] >= 0) return;
    float nearest = -6.0f;  // -DEPTH_FIELD_RADIUS + 1
    const int n = c_depth_count;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        bool solid = false;
        if (i < n) {
            const DepthOff o = g_depth_offs[i];
            const int qx = x + o.x, qy = y + o.y, qz = z + o.z;
            if (qx >= 0 && qy >= 0 && qz >= 0 && qx < L.W && qy < L.H && qz < L.W)
                solid = words[(uint64_t)qx + (uint64_t)L.W * qy + (uint64_t)L.W * L.H * qz] >= 0;  // plain load
        }
        const unsigned hits = __ballot_sync(0xffffffffu, solid);
        if (hits) {
            const float d = g_depth_offs[base + __ffs(hits) - 1].dist;
            nearest = d <= -2.0f ? d : 0.0f;
            break;
        }
    }
    if (lane == 0 && nearest < 0.0f) words[idx] = __float_as_int(nearest);
}

// Boxes of at most this many voxels take the warp-per-voxel kernel (the edit of a
// radius-1024 sphere would otherwise launch 2^38 threads).
constexpr uint64_t kWarpPerVoxelMax = 1ull << 22;

static void launch_fix_depth_field(vrt_world* w, int x0, int y0, int z0, int nx, int ny, int nz, int cx, int cy, int cz,
                                   int r2, cudaStream_t s) {
    const uint64_t n = (uint64_t)nx * ny * nz;
    if (n <= kWarpPerVoxelMax)
        fix_depth_field_warp_kernel<<<blocks_for(n * 32, 256), 256, 0, s>>>(w->d_words, w->L, x0, y0, z0, nx, ny, nz,
                                                                            cx, cy, cz, r2);
    else
        fix_depth_field_kernel<<<blocks_for(n, 256), 256, 0, s>>>(w->d_words, w->L, x0, y0, z0, nx, ny, nz, cx, cy,
                                                                  cz, r2);
}

__global__ void probe_kernel(const int32_t* __restrict__ words, Layout L, const int32_t* __restrict__ xyz, int n,
                             int32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    const bool in = x >= 0 && y >= 0 && z >= 0 && x < L.W && y < L.H && z < L.W;
    out[i] = in ? words[(uint64_t)x + (uint64_t)L.W * y + (uint64_t)L.W * L.H * z] : -1;
}

// ------------------------------------------------------------------ initVoxels

// level.cpp:85-128: stone/dirt/grass layers, then the holes that placeBush/placeTrunk
// punch near the origin by calling destroyVoxel with relative coordinates
// (level.cpp:11,64): (0,0..5,0) from the trunks and the x,y,z >= 0 part of the radius-6
// ball from the bushes.  Both are applied after the layers, as in the reference.
__global__ void init_reference_layers_kernel(int32_t* __restrict__ words, Layout L, int any_tree) {
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L.n_words) return;
    int x = (int)(t % L.W), y = (int)((t / L.W) % L.H), z = (int)(t / ((uint64_t)L.W * L.H));
    int cv = 5 * ((x + y + z) % 3);
    int v = -1;
    if (y <= 25) v = ((90 + cv) << 16) | ((90 + cv) << 8) | (90 + cv);
    else if (y <= 33) v = ((120 + cv) << 16) | ((100 + cv) << 8);
    else if (y <= 36) v = (10 << 16) | ((130 + cv) << 8) | 10;
    if (any_tree) {
        if (x == 0 && z == 0 && y < 6) v = -1;
        if (x < 6 && y < 6 && z < 6 && x * x + y * y + z * z < 36) v = -1;
    }
    words[t] = v;
}

// One tree per blockIdx.y: trunk (placeTrunk, level.cpp:59-79) then bush (placeBush,
// level.cpp:4-27) over the tree's bounding box [-6,6)^3 around the bush centre, which
// contains the trunk; the bush is written last, so it wins where the two overlap.
// Trees are 30 x 25 voxels apart and never overlap each other.
__global__ void init_reference_trees_kernel(int32_t* __restrict__ words, Layout L, int trees_x) {
    int tree = blockIdx.y;
    int tx = 30 * (1 + tree % trees_x);       // x % 30 == 0, x in [10, W-10)
    int tz = 25 * (1 + tree / trees_x);       // z % 25 == 0, z in [10, W-10)
    int bush_x = tx + tz % 7, bush_y = 46, bush_z = tz;      // level.cpp:134
    int trunk_x = tx + 1 + tz % 7, trunk_y = 36, trunk_z = tz; // level.cpp:133
    // box around the bush centre: x in [bush_x-6, bush_x+6) covers the trunk (x offsets [-2,1) from bush_x+1)
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int bw = 12, bh = 16;  // y from 36 (trunk base) to 52 (bush top)
    if (t >= bw * bh * bw) return;
    int ax = bush_x - 6 + t % bw;
    int ay = 36 + (t / bw) % bh;
    int az = bush_z - 6 + t / (bw * bh);
    if (ax < 0 || ay < 0 || az < 0 || ax >= L.W || ay >= L.H || az >= L.W) return;
    int v = 0;
    bool write = false;
    {   // placeTrunk(ivec3(trunk_x, 36, tz), ivec3(128,100,15), 6): x,z in [-2,1), y in [0,6)
        int x = ax - trunk_x, y = ay - trunk_y, z = az - trunk_z;
        if (x >= -2 && x < 1 && z >= -2 && z < 1 && y >= 0 && y < 6) {
            int r = 128 - ((x + z) % 2) * 10, g = 100 - ((x + z) % 2) * 10;
            v = (((r << 8) + g) << 8) + 15;
            write = true;
        }
    }
    {   // placeBush(ivec3(bush_x, 46, tz), ivec3(15,128,15), 6): offsets in [-6,6)^3, |o|^2 < 36
        int x = ax - bush_x, y = ay - bush_y, z = az - bush_z;
        if (x >= -6 && x < 6 && y >= -6 && y < 6 && z >= -6 && z < 6 && x * x + y * y + z * z < 36) {
            int g = 128 - ((x + y + z) % 3) * 20;
            v = (((15 << 8) + g) << 8) + 15;
            write = true;
        }
    }
    if (write) words[(uint64_t)ax + (uint64_t)L.W * ay + (uint64_t)L.W * L.H * az] = v;
}

}  // namespace vrt

using namespace vrt;

static inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

int vrt_world_create(int32_t width, int32_t height, vrt_world** out) {
    if (!out) return set_error(VRT_EINVAL, "out is NULL");
    *out = nullptr;
    if (width < 1 || height < 1 || width > 65536 || height > 65536)
        return set_error(VRT_EINVAL, "world %d x %d x %d out of range", width, height, width);
    uint64_t n = (uint64_t)width * height * width;
    if (n > (1ull << 31)) return set_error(VRT_ERANGE, "world of %llu voxels exceeds 2^31", (unsigned long long)n);
    const Layout L = make_layout(width, height);
    if (L.n_bricks * 8 >= (1ull << 32))  // the render kernels index bricks in 32 bits
        return set_error(VRT_ERANGE, "world %d x %d x %d: brick grid too large", width, height, width);
    vrt_world* w = new vrt_world();
    w->L = L;
    cudaGetDevice(&w->device);
    uint64_t bytes = w->L.n_words * 4 + (w->L.n_bricks + w->L.n_regions + w->L.n_supers) * 8 + 24 * w->L.n_bricks +
                     (uint64_t)w->L.RWp * w->L.RHp * w->L.RWp + 256;
    cudaError_t e = cudaMalloc(&w->d_words, w->L.n_words * 4);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_bricks, w->L.n_bricks * 8);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_regions, w->L.n_regions * 8);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_supers, w->L.n_supers * 8);
    const uint64_t rbytes = ((uint64_t)w->L.RWp * w->L.RHp * w->L.RWp + 15) & ~(uint64_t)15;  // staged as uint4
    if (e == cudaSuccess) e = cudaMalloc(&w->d_rdist, rbytes);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_bdir, w->L.n_bricks * 8);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_tmp_a, w->L.n_bricks * 8);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_tmp_b, w->L.n_bricks * 8);
    if (e == cudaSuccess) e = cudaMalloc(&w->d_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&w->d_aabb, 8 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(w->d_words, 0xFF, w->L.n_words * 4);  // air = -1 (render.cpp:349-351)
    if (e == cudaSuccess) e = cudaMemset(w->d_bricks, 0, w->L.n_bricks * 8);
    if (e == cudaSuccess) e = cudaMemset(w->d_regions, 0, w->L.n_regions * 8);
    if (e == cudaSuccess) e = cudaMemset(w->d_supers, 0, w->L.n_supers * 8);
    if (e == cudaSuccess) e = cudaMemset(w->d_bdir, kDistCap, w->L.n_bricks * 8);  // an all-air world
    if (e == cudaSuccess) e = cudaMemset(w->d_rdist, kDistCap, rbytes);
    if (e == cudaSuccess) e = cudaMemset(w->d_flag, 0, sizeof(int));
    if (e == cudaSuccess) {  // an all-air world: empty box (min > max)
        const int empty[8] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, 0, 0};
        e = cudaMemcpy(w->d_aabb, empty, sizeof(empty), cudaMemcpyHostToDevice);
        for (int i = 0; i < 6; i++) w->h_aabb[i] = empty[i];
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaGetLastError();
        vrt_world_destroy(w);
        return e == cudaErrorMemoryAllocation ? set_error(VRT_ENOMEM, "world allocation: %s", cudaGetErrorString(e))
                                              : cuda_error(e, "vrt_world_create");
    }
    w->device_bytes = bytes;
    *out = w;
    return VRT_OK;
}

int vrt_world_destroy(vrt_world* w) {
    if (!w) return VRT_OK;
    cudaFree(w->d_words);
    cudaFree(w->d_bricks);
    cudaFree(w->d_regions);
    cudaFree(w->d_supers);
    cudaFree(w->d_rdist);
    cudaFree(w->d_bdir);
    cudaFree(w->d_stop);
    cudaFree(w->d_sdir);
    if (w->stop_ready) cudaEventDestroy(w->stop_ready);
    cudaFree(w->d_words_z);
    if (w->z_ready) cudaEventDestroy(w->z_ready);
    cudaFree(w->d_tmp_a);
    cudaFree(w->d_tmp_b);
    cudaFree(w->d_flag);
    cudaFree(w->d_aabb);
    delete w;
    return VRT_OK;
}

int vrt_world_get_info(const vrt_world* w, vrt_world_info* out) {
    if (!w || !out) return set_error(VRT_EINVAL, "NULL argument");
    out->width = w->L.W;
    out->height = w->L.H;
    out->num_words = w->L.n_words;
    out->d_words = w->d_words;
    out->d_brick_mask = w->d_bricks;
    out->d_region_mask = w->d_regions;
    out->has_depth_field = w->has_depth_field;
    out->device_bytes = w->device_bytes;
    return VRT_OK;
}

static int upload_common(vrt_world* w, const int32_t* src, uint64_t first, uint64_t count, void* stream,
                         cudaMemcpyKind kind) {
    if (!w || (!src && count)) return set_error(VRT_EINVAL, "NULL argument");
    if (first > w->L.n_words || count > w->L.n_words - first)
        return set_error(VRT_ERANGE, "words [%llu, %llu) beyond the world's %llu", (unsigned long long)first,
                         (unsigned long long)(first + count), (unsigned long long)w->L.n_words);
    if (count == 0) return VRT_OK;
    VRT_CUDA(cudaMemcpyAsync(w->d_words + first, src, count * 4, kind, S(stream)));
    int st = refresh_masks(w, first, count, S(stream));
    if (st) return st;
    // the kernel choice depends on the depth-field flag: read it back now
    int flag = 0;
    VRT_CUDA(cudaMemcpyAsync(&flag, w->d_flag, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    w->has_depth_field |= flag;
    return read_aabb(w, S(stream));
}

int vrt_world_upload(vrt_world* w, const int32_t* host_words, uint64_t first, uint64_t count, void* stream) {
    return upload_common(w, host_words, first, count, stream, cudaMemcpyHostToDevice);
}

int vrt_world_upload_device(vrt_world* w, const int32_t* d_words, uint64_t first, uint64_t count, void* stream) {
    return upload_common(w, d_words, first, count, stream, cudaMemcpyDeviceToDevice);
}

int vrt_world_download(const vrt_world* w, int32_t* host_words, uint64_t first, uint64_t count, void* stream) {
    if (!w || (!host_words && count)) return set_error(VRT_EINVAL, "NULL argument");
    if (first > w->L.n_words || count > w->L.n_words - first) return set_error(VRT_ERANGE, "range beyond the world");
    if (count == 0) return VRT_OK;
    VRT_CUDA(cudaMemcpyAsync(host_words, w->d_words + first, count * 4, cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    return VRT_OK;
}

int vrt_world_download_masks(const vrt_world* w, uint64_t* bricks, uint64_t* regions, uint64_t* supers,
                             void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    if (bricks)
        VRT_CUDA(cudaMemcpyAsync(bricks, w->d_bricks, w->L.n_bricks * 8, cudaMemcpyDeviceToHost, S(stream)));
    if (regions)
        VRT_CUDA(cudaMemcpyAsync(regions, w->d_regions, w->L.n_regions * 8, cudaMemcpyDeviceToHost, S(stream)));
    if (supers)
        VRT_CUDA(cudaMemcpyAsync(supers, w->d_supers, w->L.n_supers * 8, cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    return VRT_OK;
}

int vrt_world_download_distances(const vrt_world* w, uint8_t* brick_dir, uint8_t* region_dist, void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    if (brick_dir)
        VRT_CUDA(cudaMemcpyAsync(brick_dir, w->d_bdir, w->L.n_bricks * 8, cudaMemcpyDeviceToHost, S(stream)));
    if (region_dist)
        VRT_CUDA(cudaMemcpyAsync(region_dist, w->d_rdist, (uint64_t)w->L.RWp * w->L.RHp * w->L.RWp,
                                 cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    return VRT_OK;
}

// The flag is raised by the brick kernel whenever it sees a word < -1 and never lowered
// by it; a full-world refresh after clearing gives the exact current state.
int vrt_world_sync_flags(vrt_world* w, void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    VRT_CUDA(cudaMemsetAsync(w->d_flag, 0, sizeof(int), S(stream)));
    int st = refresh_masks_box(w, 0, 0, 0, w->L.W, w->L.H, w->L.W, S(stream));
    if (st) return st;
    int flag = 0;
    VRT_CUDA(cudaMemcpyAsync(&flag, w->d_flag, sizeof(int), cudaMemcpyDeviceToHost, S(stream)));
    VRT_CUDA(cudaStreamSynchronize(S(stream)));
    w->has_depth_field = flag;
    return read_aabb(w, S(stream));
}

int vrt_world_probe(const vrt_world* w, const int32_t* d_xyz, int32_t n, int32_t* d_words, void* stream) {
    if (!w || n < 0 || (n > 0 && (!d_xyz || !d_words))) return set_error(VRT_EINVAL, "bad probe arguments");
    if (n == 0) return VRT_OK;
    probe_kernel<<<blocks_for((uint64_t)n, 256), 256, 0, S(stream)>>>(w->d_words, w->L, d_xyz, n, d_words);
    VRT_CUDA(cudaGetLastError());
    return VRT_OK;
}

static const int32_t kWorldMagic = 0x57525456;  // "VRTW" little-endian

int vrt_world_save(const vrt_world* w, const char* path, void* stream) {
    if (!w || !path) return set_error(VRT_EINVAL, "NULL argument");
    std::vector<int32_t> host(w->L.n_words);
    int st = vrt_world_download(w, host.data(), 0, w->L.n_words, stream);
    if (st) return st;
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(VRT_EINVAL, "cannot open %s for writing", path);
    const int32_t head[4] = {kWorldMagic, 1, w->L.W, w->L.H};
    bool ok = std::fwrite(head, sizeof(head), 1, f) == 1 &&
              std::fwrite(host.data(), sizeof(int32_t), host.size(), f) == host.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? VRT_OK : set_error(VRT_EINVAL, "short write to %s", path);
}

int vrt_world_load(const char* path, vrt_world** out, void* stream) {
    if (!path || !out) return set_error(VRT_EINVAL, "NULL argument");
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(VRT_EINVAL, "cannot open %s", path);
    int32_t head[4] = {0, 0, 0, 0};
    if (std::fread(head, sizeof(head), 1, f) != 1 || head[0] != kWorldMagic || head[1] != 1) {
        std::fclose(f);
        return set_error(VRT_EINVAL, "%s is not a version-1 world file", path);
    }
    vrt_world* w = nullptr;
    int st = vrt_world_create(head[2], head[3], &w);
    if (st) {
        std::fclose(f);
        return st;
    }
    std::vector<int32_t> host(w->L.n_words);
    const bool ok = std::fread(host.data(), sizeof(int32_t), host.size(), f) == host.size();
    std::fclose(f);
    if (!ok) {
        vrt_world_destroy(w);
        return set_error(VRT_EINVAL, "%s is truncated", path);
    }
    st = vrt_world_upload(w, host.data(), 0, host.size(), stream);
    if (st) {
        vrt_world_destroy(w);
        return st;
    }
    *out = w;
    return VRT_OK;
}

int vrt_place_voxel(vrt_world* w, int32_t x, int32_t y, int32_t z, int32_t word, void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    if (x < 0 || y < 0 || z < 0 || x >= w->L.W || y >= w->L.H || z >= w->L.W) return VRT_OK;  // render.cpp:259
    place_voxel_kernel<<<1, 1, 0, S(stream)>>>(w->d_words, w->L, x, y, z, word);
    VRT_CUDA(cudaGetLastError());
    if (word < -1) w->has_depth_field = 1;
    if (word >= 0) {  // grow the host copy of the solid box by the voxel's brick
        const int c[3] = {x & ~3, y & ~3, z & ~3};
        for (int i = 0; i < 3; i++) {
            w->h_aabb[i] = std::min(w->h_aabb[i], c[i]);
            w->h_aabb[3 + i] = std::max(w->h_aabb[3 + i], c[i] + 3);
        }
    }
    return refresh_masks_box(w, x, y, z, x + 1, y + 1, z + 1, S(stream));
}

int vrt_fix_depth_field_box(vrt_world* w, int32_t x0, int32_t y0, int32_t z0, int32_t x1, int32_t y1, int32_t z1,
                            void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    x0 = std::max(x0, 0); y0 = std::max(y0, 0); z0 = std::max(z0, 0);
    x1 = std::min(x1, w->L.W); y1 = std::min(y1, w->L.H); z1 = std::min(z1, w->L.W);
    if (x0 >= x1 || y0 >= y1 || z0 >= z1) return VRT_OK;
    int st = ensure_depth_table();
    if (st) return st;
    launch_fix_depth_field(w, x0, y0, z0, x1 - x0, y1 - y0, z1 - z0, 0, 0, 0, 0, S(stream));
    VRT_CUDA(cudaGetLastError());
    w->has_depth_field = 1;
    return refresh_masks_box(w, x0, y0, z0, x1, y1, z1, S(stream));
}

int vrt_remove_sphere(vrt_world* w, int32_t cx, int32_t cy, int32_t cz, int32_t radius, int32_t refresh_depth_field,
                      void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    if (radius < 0 || radius > 1024) return set_error(VRT_ERANGE, "radius %d outside [0, 1024]", radius);
    if (radius > 0) {
        uint64_t n = (uint64_t)(2 * radius) * (2 * radius) * (2 * radius);
        remove_sphere_kernel<<<blocks_for(n, 256), 256, 0, S(stream)>>>(w->d_words, w->L, cx, cy, cz, radius);
        VRT_CUDA(cudaGetLastError());
    }
    int r2 = radius + (7 >> 1);  // DEPTH_FIELD_RADIUS >> 1, level.cpp:43
    if (refresh_depth_field && r2 > 0) {
        int st = ensure_depth_table();
        if (st) return st;
        const int n = 2 * r2;
        launch_fix_depth_field(w, cx - r2, cy - r2, cz - r2, n, n, n, cx, cy, cz, r2, S(stream));
        VRT_CUDA(cudaGetLastError());
        w->has_depth_field = 1;
    }
    int rb = std::max(radius, refresh_depth_field ? r2 : radius);
    return refresh_masks_box(w, cx - rb, cy - rb, cz - rb, cx + rb, cy + rb, cz + rb, S(stream));
}

int vrt_world_init_reference(vrt_world* w, void* stream) {
    if (!w) return set_error(VRT_EINVAL, "NULL world");
    const Layout& L = w->L;
    // trees at x % 30 == 0 and z % 25 == 0 for x, z in [10, W-10) (level.cpp:130-137)
    int trees_x = 0, trees_z = 0;
    for (int x = 10; x < L.W - 10; x++) trees_x += (x % 30 == 0);
    for (int z = 10; z < L.W - 10; z++) trees_z += (z % 25 == 0);
    init_reference_layers_kernel<<<blocks_for(L.n_words, 256), 256, 0, S(stream)>>>(w->d_words, L,
                                                                                    trees_x * trees_z > 0);
    VRT_CUDA(cudaGetLastError());
    if (trees_x * trees_z > 0) {
        dim3 grid(blocks_for(12 * 16 * 12, 256), trees_x * trees_z);
        init_reference_trees_kernel<<<grid, 256, 0, S(stream)>>>(w->d_words, L, trees_x);
        VRT_CUDA(cudaGetLastError());
    }
    VRT_CUDA(cudaMemsetAsync(w->d_flag, 0, sizeof(int), S(stream)));
    w->has_depth_field = 0;
    int st = refresh_masks_box(w, 0, 0, 0, L.W, L.H, L.W, S(stream));
    if (st) return st;
    return read_aabb(w, S(stream));
}

}  // extern "C"
