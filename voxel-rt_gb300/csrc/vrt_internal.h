// Internal declarations shared by the translation units of libvrt.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "vrt_host.h"

namespace vrt {

// ---- error plumbing: every C entry point returns a status and records a message ----
int cuda_error(cudaError_t e, const char* what);

#define VRT_CUDA(call)                                       \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return ::vrt::cuda_error(e_, #call); \
    } while (0)

// ---- occupancy hierarchy ----
// Three levels of 64-bit masks over the voxel words (a 64-ary tree):
//   brick  (4x4x4 voxels):   bit (x&3) + 4*(y&3) + 16*(z&3) set when that voxel is solid
//   region (16x16x16):       bit per brick (bx&3) + 4*(by&3) + 16*(bz&3) set when the brick has a solid voxel
//   super  (64x64x64):       bit per region, same layout, set when the region has a solid voxel
// Bricks are stored linearly, bx + BWp*(by + BHp*bz), so a ray's box lookup computes its
// brick's slot with two multiply-adds; regions are stored super-major (64 regions of a
// super block = 512 contiguous bytes).  Voxels outside the world count as empty.
struct Layout {
    int W, H;           // voxel dims: x,z in [0,W), y in [0,H)
    int RW, RH;         // regions per axis (x/z, y): ceil(W/16), ceil(H/16)
    int SW, SH;         // super blocks per axis: ceil(W/64), ceil(H/64)
    int RWp, RHp;       // regions per axis padded to a multiple of 4 (= 4*SW, 4*SH)
    int BWp, BHp;       // bricks per axis, padded (= 16*SW, 16*SH)
    uint64_t n_words;   // W*H*W
    uint64_t n_bricks;  // 64 * RWp*RHp*RWp
    uint64_t n_regions; // 64 * SW*SH*SW
    uint64_t n_supers;  // SW*SH*SW
};

// Empty-space distance fields (capped Chebyshev distance, in nodes, to the nearest
// non-empty node; 0 = the node itself holds a solid voxel).  Values are capped (never
// larger than the truth) and recomputed whenever solids may be added.
//   region distance: uint8 per region, linear index rx + RWp*(ry + RHp*rz).  A region at
//   distance d >= 1 has every region within Chebyshev radius d-1 empty, so the cube of
//   those regions is a box a ray can cross without reading voxels.
constexpr int kDistCap = 15;

// Directed brick distances: 8 bytes per brick, stored like the brick masks.  Byte o
// (octant o: bit a set = the + direction along axis a, x=0 y=1 z=2) is the capped
// Chebyshev distance from the brick to the nearest non-empty brick n in that octant
// (n_a >= b_a where bit a is set, n_a <= b_a where it is clear).  At distance d >= 1
// the cube of bricks from b to b + (d-1) in the octant's directions is empty: a ray
// moving into that octant leaves its brick only through that cube's far faces, so the
// cube bounds it as well as a centred cube of the same radius would, while solids
// behind or beside the ray no longer shrink it.

__host__ __device__ inline uint64_t region_linear(const Layout& L, int rx, int ry, int rz) {
    return (uint64_t)rx + (uint64_t)L.RWp * ((uint64_t)ry + (uint64_t)L.RHp * rz);
}

__host__ __device__ inline uint64_t super_index(const Layout& L, int sx, int sy, int sz) {
    return (uint64_t)sx + (uint64_t)L.SW * ((uint64_t)sy + (uint64_t)L.SH * sz);
}
// region (rx,ry,rz) -> slot in the region array
__host__ __device__ inline uint64_t region_index(const Layout& L, int rx, int ry, int rz) {
    return super_index(L, rx >> 2, ry >> 2, rz >> 2) * 64 + ((rx & 3) + 4 * (ry & 3) + 16 * (rz & 3));
}
// brick (bx,by,bz) -> slot in the brick array (and the brick distance field)
__host__ __device__ inline uint64_t brick_index(const Layout& L, int bx, int by, int bz) {
    return (uint64_t)bx + (uint64_t)L.BWp * ((uint64_t)by + (uint64_t)L.BHp * bz);
}

Layout make_layout(int W, int H);

}  // namespace vrt

struct vrt_world {
    vrt::Layout L;
    int32_t* d_words = nullptr;
    uint64_t* d_bricks = nullptr;
    uint64_t* d_regions = nullptr;
    uint64_t* d_supers = nullptr;
    uint8_t* d_rdist = nullptr;     // region distance field (linear, RWp*RHp*RWp)
    uint8_t* d_bdir = nullptr;      // directed brick distances (8 bytes per brick, linear)
    uint64_t* d_stop = nullptr;     // depth-field worlds: brick masks of the cells a ray stops at
                                    // (word != -1: solid or depth-field), made on first use
    uint8_t* d_sdir = nullptr;      // directed brick distances over the stop masks
    bool stop_stale = true;         // the stop structures predate the last change of the words
    cudaEvent_t stop_ready = nullptr;  // recorded after each rebuild: renders on other streams wait on it
    int32_t* d_words_z = nullptr;   // the word kernel's second copy of the words with x and z swapped
                                    // (index z + W*y + W*H*x), made on first use
    int z_dirty[6] = {0, 0, 0, 0, 0, 0};  // box [x0,x1)x[y0,y1)x[z0,z1) of words changed since the
                                    // copy was last brought up to date (empty: x0 >= x1)
    cudaEvent_t z_ready = nullptr;  // recorded after each copy update: renders on other streams wait on it
    uint8_t* d_tmp_a = nullptr;     // scratch of the distance passes (8 * n_bricks each)
    uint8_t* d_tmp_b = nullptr;
    int* d_flag = nullptr;          // has-depth-field flag written by the mask kernels
    int* d_aabb = nullptr;          // bounding box of the solid voxels, brick-granular and
                                    // never smaller than the truth: min x,y,z then max x,y,z
    int h_aabb[6] = {0, 0, 0, -1, -1, -1};  // host copy passed to the render kernels; kept a
                                    // superset of the device box (read back after uploads)
    int has_depth_field = 0;        // host copy (as of the last sync)
    uint64_t device_bytes = 0;
    int device = 0;
};

namespace vrt {
// Rebuild the masks of every brick overlapping words [first, first+count).
int refresh_masks(vrt_world* w, uint64_t first, uint64_t count, cudaStream_t s);
// Rebuild the masks of the voxel box [x0,x1)x[y0,y1)x[z0,z1) (clipped).
int refresh_masks_box(vrt_world* w, int x0, int y0, int z0, int x1, int y1, int z1, cudaStream_t s);
// Bring the stop masks and their directed distances up to date (allocated on first use),
// and make stream s wait until they are: the rebuild may have run on another stream.
int refresh_stop(vrt_world* w, cudaStream_t s);
// Bring the z-major copy of the words up to date (allocated and filled on first use, then
// only the box changed since), and make stream s wait until it is: the update may have
// run on another stream.
int refresh_words_z(vrt_world* w, cudaStream_t s);
}  // namespace vrt
