/*
 * vrt.h -- C ABI of the GB300 voxel ray tracer.
 *
 * This is the drop-in boundary for the per-pixel ray tracer of Berry2460/voxel-rt
 * (src/fshader.glsl).  In the reference, the host talks to the GPU through OpenGL:
 *   - the world is an SSBO of int32 voxel words (render.cpp:366-369, :199-223),
 *   - the camera/light state is a set of glUniform* calls (render.cpp:289-296),
 *   - a frame is glDrawArrays(GL_TRIANGLES, 0, 6) over a fullscreen quad (main.cpp:59).
 * Here the world is a device-resident buffer owned by a vrt_world, the uniforms are a
 * plain struct passed by pointer, and a frame is one kernel launch into a caller-owned
 * device RGBA8 buffer.  Block destruction (level.cpp:30-56) and the depth field
 * (render.cpp:226-253) become device-side scatter kernels.
 *
 * Conventions
 *   - Every entry point returns an int status: 0 = ok, negative = error (VRT_E*).
 *     vrt_last_error() returns a message for the calling thread's last failure.
 *   - Streams are passed as void* (a cudaStream_t; NULL = legacy default stream).
 *     All work is stream ordered; no call synchronises unless documented.
 *   - Output buffers are caller-owned device memory unless the name says _host.
 *   - Distinct worlds/renderers may be used from distinct threads; one object is
 *     externally synchronised.
 *
 * Voxel word (fshader.glsl:12-15, README.md:5, render.cpp:189-196)
 *   int32 per voxel at index x + W*y + W*H*z, with x,z in [0,W) and y in [0,H).
 *   v >= 0       solid; colour R = (v>>16)&255, G = (v>>8)&255, B = v&255.
 *   v == -1      empty air.
 *   other v < 0  air carrying a depth-field skip distance: the float whose bits
 *                are v is negative and the ray jumps -asfloat(v) voxels
 *                (fshader.glsl:114-121, written by render.cpp:249-251).
 *   Bit 24 is a free "solid" tag for generated worlds (0x01000000|rgb); it is
 *   never tested: only the sign decides.
 */
#ifndef VRT_H
#define VRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VRT_MAX_LOCAL_LIGHTS 16 /* MAX_LOCAL_LIGHTS, render.hpp:11 / fshader.glsl:6 */

/* status codes */
#define VRT_OK 0
#define VRT_EINVAL -1     /* bad argument */
#define VRT_ECUDA -2      /* a CUDA runtime call failed */
#define VRT_ENOMEM -3     /* device or host allocation failed */
#define VRT_ERANGE -4     /* size beyond a documented maximum */
#define VRT_ETIMEOUT -5   /* a bounded device-side wait gave up */
#define VRT_EBUDGET -6    /* request refused by the memory budget */
#define VRT_ENOTFOUND -7  /* unknown id */
#define VRT_ESTATE -8     /* object in the wrong state for this call */

/* Uniform block of fshader.glsl:20-26 plus the constants of fshader.glsl:3-10 as
 * run-time parameters.  vrt_uniforms_default() fills in the reference values. */
typedef struct vrt_uniforms {
    float camPos[3];           /* uniform vec3 camPos                                */
    float camRotation[2];      /* uniform vec2 camRotation (declared, unused by the shader) */
    float lightPos[3];         /* uniform vec3 lightPos: global light, a POINT position */
    float aspectRatio;         /* uniform float aspectRatio (width/height)          */
    float rotateMatrix[16];    /* uniform mat4 rotateMatrix, column-major (glUniformMatrix4fv, GL_FALSE) */
    int32_t viewDepthField;    /* uniform int viewDepthField: 1 = step-count view    */
    float localLights[VRT_MAX_LOCAL_LIGHTS][4]; /* uniform vec4 localLights[16]: xyz, w = intensity;
                                                   a light is active iff x,y,z >= 0 */
    /* ---- extensions; the defaults reproduce the reference exactly ---- */
    float localLightColor[VRT_MAX_LOCAL_LIGHTS][3]; /* per-channel factor on w; 1,1,1 = reference */
    float tanHalfFov;          /* tan(vertical fov / 2); 1.0 = the reference's 90 degrees */
    int32_t maxSteps;          /* RENDER_DIST (384): DDA iteration cap of every ray, at most 2^24 */
    float localLightDist;      /* LOCAL_LIGHT_DIST (64): local light radius         */
    float ambient;             /* AMBIENT (0.4)                                     */
    float diffuse;             /* DIFFUSE (0.8)                                     */
    float maxOverbright;       /* MAX_OVERBRIGHT (1.25)                             */
} vrt_uniforms;

/* Optional per-pixel side outputs (device pointers, each may be NULL). */
typedef struct vrt_debug_out {
    int32_t* hit_index;     /* primary-ray hit voxel index, -1 on a miss            */
    uint32_t* cast_mask;    /* bit 0: global shadow ray cast; bit 1+i: local light i cast */
    uint32_t* occ_mask;     /* same bits: set when that shadow ray was blocked      */
    int32_t* steps;         /* DDA iterations summed over every ray of the pixel    */
    int32_t* primary_steps; /* DDA iterations of the primary ray (stepCount after castRay #1) */
    float* shade;           /* 3 floats per pixel: the final light multiplier (r,g,b) */
} vrt_debug_out;

/* Optional device counters accumulated by a render (8 x uint64, device memory,
 * caller zeroes): [0] rays cast, [1] DDA iterations, [2] primary hits, [3] pixels;
 * traversal diagnostics of the occupancy-mask kernels: [4] box refills (steps that left
 * a known-empty box or brick), [5] warp slow phases, [6] warp fast batches. */
#define VRT_STAT_RAYS 0
#define VRT_STAT_STEPS 1
#define VRT_STAT_HITS 2
#define VRT_STAT_PIXELS 3
#define VRT_STAT_REFILLS 4
#define VRT_STAT_SLOW 5
#define VRT_STAT_FAST 6
#define VRT_STAT_COUNT 8

/* Render kernel choice.  AUTO picks the tile kernel, or the word kernel for a world that
 * holds depth-field words (both follow the jumps; the word kernel is faster there). */
#define VRT_KERNEL_AUTO 0       /* the tile kernel; the word kernel for worlds with depth-field words */
#define VRT_KERNEL_WORD 1       /* one thread per pixel, one 4-byte word per DDA step     */
#define VRT_KERNEL_BITMASK 2    /* occupancy-mask traversal, persistent ray refill (no depth-field words) */
#define VRT_KERNEL_MASK_PIXEL 3 /* the tile kernel: occupancy-mask traversal, one thread per pixel,
                                   following depth-field jumps too */

/* Step accounting.  The occupancy-mask kernels end a ray as soon as its path provably
 * holds no solid voxel: its cell lies beyond the bounding box of the world's solid voxels
 * along an axis it moves away from (or parallel to).  Such a ray misses whatever path it
 * takes, so every pixel, cast bit and occlusion bit is unchanged; only the number of DDA
 * iterations performed drops.  Those counts (VRT_STAT_STEPS, the steps / primary_steps
 * debug outputs, the viewDepthField step view) equal the shader's exactly whenever they are
 * asked for: exact_steps = 1, a steps or primary_steps debug output, or viewDepthField. */
typedef struct vrt_render_opts {
    int32_t kernel;          /* VRT_KERNEL_*                                        */
    int32_t tile_w, tile_h;  /* ray tile (0 = kernel default: 8x16 tile kernel, 8x4 persistent, 16x8 word
                                kernel); tile and word kernels: tile_w*tile_h a multiple of 32, at most 128 */
    int32_t refill_min;      /* persistent kernel: lanes parked before a slow phase (0 = default) */
    int32_t blocks_per_sm;   /* persistent kernel: resident CTAs per SM it is built for (3 or 4) */
    int32_t exact_steps;     /* 1: count every DDA iteration of the shader, no early miss */
    int32_t host_bands;      /* vrt_render_to_host: 0 = automatic (page-locked memory is written by the
                                kernel directly; other memory gets bands of 128 rows, up to 8); n > 0 =
                                stage in device memory and copy, in n bands of rows with the tile kernel,
                                each band's copy overlapping the next band's render (1 = render then copy) */
} vrt_render_opts;

typedef struct vrt_world vrt_world;
typedef struct vrt_renderer vrt_renderer;

typedef struct vrt_world_info {
    int32_t width, height;          /* VOXELS_WIDTH (x and z), VOXELS_HEIGHT (y)      */
    uint64_t num_words;             /* W*H*W                                          */
    const int32_t* d_words;         /* device voxel words                             */
    const uint64_t* d_brick_mask;   /* device occupancy mask: one uint64 per 4x4x4 brick (linear) */
    const uint64_t* d_region_mask;  /* device: one uint64 per 16x16x16 region, bit per brick */
    int32_t has_depth_field;        /* 1 if any word is < -1 (as of the last sync)    */
    uint64_t device_bytes;          /* device memory held by the world                */
} vrt_world_info;

const char* vrt_last_error(void);
const char* vrt_version(void);

/* ---- uniforms (host only, no GPU) ---- */
/* Reference constants (fshader.glsl:3-10), identity rotateMatrix, camPos (195,55,155)
 * (main.cpp:26), aspect 800/600 (main.cpp:11-12,36), lights cleared as initLocalLights. */
int vrt_uniforms_default(vrt_uniforms* u);
/* initLocalLights, render.cpp:304-311: every slot (-1,-1,-1,0), colour (1,1,1). */
int vrt_init_local_lights(vrt_uniforms* u);
/* placeLocalLight, render.cpp:375-385: the first slot with any coordinate < 0 takes
 * (x,y,z,a).  Returns the slot used (0..15), or VRT_MAX_LOCAL_LIGHTS when all 16 are
 * taken, which the reference also ignores silently. */
int vrt_place_local_light(vrt_uniforms* u, float x, float y, float z, float a);
/* Camera matrix R_y(yaw) * R_x(pitch) (controls.cpp:136-142), angles in radians,
 * column-major into m[16]. */
int vrt_rotate_matrix(float pitch_x, float yaw_y, float* m16);

/* ---- worlds ---- */
/* A W x H x W world of air (-1) on the current device.  W,H in [1, 65536], W*H*W <= 2^31. */
int vrt_world_create(int32_t width, int32_t height, vrt_world** out);
int vrt_world_destroy(vrt_world* w);
int vrt_world_get_info(const vrt_world* w, vrt_world_info* out);
/* glBufferData / glBufferSubData (render.cpp:199-202, :219): copy count words from
 * host memory into words [first, first+count), then refresh the occupancy mask of the
 * bricks touched and read back the depth-field flag (synchronises the stream).
 * Pageable or pinned host memory. */
int vrt_world_upload(vrt_world* w, const int32_t* host_words, uint64_t first, uint64_t count, void* stream);
/* Same from device memory. */
int vrt_world_upload_device(vrt_world* w, const int32_t* d_words, uint64_t first, uint64_t count, void* stream);
/* Copy words [first, first+count) back to host memory. */
int vrt_world_download(const vrt_world* w, int32_t* host_words, uint64_t first, uint64_t count, void* stream);
/* Copy the occupancy hierarchy to host memory (any pointer may be NULL), SW = ceil(W/64),
 * SH = ceil(H/64):
 *   bricks:  64*64*SW*SH*SW words at bx + 16SW*(by + 16SH*bz), voxel bit x+4y+16z (4^3 bricks)
 *   regions: 64*SW*SH*SW words at super*64 + (rx&3)+4(ry&3)+16(rz&3), bit per brick (16^3)
 *   supers:  SW*SH*SW words at sx + SW*(sy + SH*sz), bit per region (64^3)
 * Synchronises the stream. */
int vrt_world_download_masks(const vrt_world* w, uint64_t* bricks, uint64_t* regions, uint64_t* supers,
                             void* stream);
/* Copy the empty-space distance fields to host memory (either pointer may be NULL), a
 * diagnostic with no counterpart in the reference; capped Chebyshev distances, 15 = "15 or more":
 *   brick_dir:   8 bytes per brick (64*64*SW*SH*SW bricks, ordered like the brick masks);
 *                byte o is the distance to the nearest non-empty brick in octant o, where
 *                bit a of o (x=0, y=1, z=2) set means coordinates >= the brick's along a,
 *                clear means <=
 *   region_dist: 1 byte per region at rx + 4SW*(ry + 4SH*rz), distance to the nearest
 *                non-empty region
 * Synchronises the stream. */
int vrt_world_download_distances(const vrt_world* w, uint8_t* brick_dir, uint8_t* region_dist, void* stream);
/* Batched voxel lookups, the query behind the reference's collision and gravity probes
 * (controls.cpp:10-19, :77-98, which read voxels[getVoxelIndex(x,y,z)]): for each of the n
 * device (x,y,z) int32 triples in d_xyz, d_words[i] = the voxel word, or -1 (air) for a
 * cell outside the world (the reference reads voxels[-1] there). */
int vrt_world_probe(const vrt_world* w, const int32_t* d_xyz, int32_t n, int32_t* d_words, void* stream);
/* World file: a 16-byte header ("VRTW", version 1, W, H as little-endian int32) followed by
 * the W*H*W voxel words in the reference's in-memory order (x + W*y + W*H*z).  Save
 * synchronises the stream; load creates the world on the current device. */
int vrt_world_save(const vrt_world* w, const char* path, void* stream);
int vrt_world_load(const char* path, vrt_world** out, void* stream);
/* Recompute has_depth_field (a device reduction; synchronises the stream). */
int vrt_world_sync_flags(vrt_world* w, void* stream);

/* ---- edits (device scatter) ---- */
/* removeSphere, level.cpp:30-56: every voxel (cx+x, cy+y, cz+z) with x,y,z in [-r, r),
 * x*x+y*y+z*z < r*r and inside the world becomes air (-1); the occupancy mask follows.
 * If refresh_depth_field != 0 the depth field is then recomputed, as the reference does,
 * for the voxels of the radius r+3 sphere (render.cpp:226-253). r in [0, 1024]. */
int vrt_remove_sphere(vrt_world* w, int32_t cx, int32_t cy, int32_t cz, int32_t radius,
                      int32_t refresh_depth_field, void* stream);
/* placeVoxel, render.cpp:256-262: set one word (ignored outside the world). */
int vrt_place_voxel(vrt_world* w, int32_t x, int32_t y, int32_t z, int32_t word, void* stream);
/* fixDepthField, render.cpp:226-253, over every voxel of the box [x0,x1)x[y0,y1)x[z0,z1)
 * (clipped to the world).  The whole world: 0,0,0,W,H,W. */
int vrt_fix_depth_field_box(vrt_world* w, int32_t x0, int32_t y0, int32_t z0,
                            int32_t x1, int32_t y1, int32_t z1, void* stream);

/* ---- world generation ---- */
/* initVoxels, level.cpp:82-138 (stone/dirt/grass layers and trees, including the
 * reference's relative-coordinate destroyVoxel calls), run on the device; level.cpp is
 * written for 512 x 96 x 512, other sizes run the same rules.  Synchronises the stream.
 * Depth field not included: call vrt_fix_depth_field_box over the whole world for the
 * app's init state. */
int vrt_world_init_reference(vrt_world* w, void* stream);
/* Seeded terrain of the benchmark scenes (host, multi-threaded, deterministic across
 * CPUs): 2-octave value-noise heightfield in [8,40], grass/dirt/stone bands with +-8
 * colour jitter, caves where 3-D value noise > 0.7.  Solid = 0x01000000|rgb, air = -1.
 * Writes W*H*W words to host memory. */
int vrt_terrain_generate(int32_t* host_words, int32_t width, int32_t height, uint64_t seed, int32_t threads);
/* Height of column (x,z) of that terrain (first air y above the surface). */
int vrt_terrain_height(int32_t width, uint64_t seed, int32_t x, int32_t z);

/* ---- rendering ---- */
/* A renderer owns per-launch scratch: the view table of batches, the persistent kernel's
 * tile counter, the staging image and streams of vrt_render_to_host, and the word
 * kernel's tile order (128 bytes per pixel tile).  Each word-kernel render sorts its tiles
 * into cost classes as they end, and the next word-kernel render of the same tile grid on
 * the same renderer launches them heaviest class first; the order changes no result (and
 * without device memory for it, frames run in row order).
 * Creating the first renderer on a device also fills a 1 KiB table the pixel colour reads
 * (synchronises the device once).  One renderer per concurrently used stream. */
int vrt_renderer_create(vrt_renderer** out);
int vrt_renderer_destroy(vrt_renderer* r);

/* One frame: glDrawArrays(GL_TRIANGLES,0,6) over the fullscreen quad (main.cpp:59) with
 * the uniforms of render.cpp:289-296.  d_rgba: width*height*4 bytes, 4-byte aligned (one
 * 32-bit store per pixel; VRT_EINVAL otherwise), any memory the device can store to, row
 * 0 = bottom row (GL order); pixel (px,py) sees vPos = ((2px+1)/width-1, (2py+1)/height-1).  dbg,
 * d_stats and opts may be NULL.  The tile kernel's first render of a depth-field world
 * after its words changed also rebuilds the world's stop masks on this stream (allocated
 * on first use, 16 bytes per brick).  The word kernel's first render after the words
 * changed brings the world's z-major copy of the words up to date over the changed box
 * on this stream (allocated and filled on first use: as large as the words). */
int vrt_render(vrt_renderer* r, const vrt_world* w, const vrt_uniforms* u, int32_t width,
               int32_t height, uint8_t* d_rgba, const vrt_debug_out* dbg, uint64_t* d_stats,
               const vrt_render_opts* opts, void* stream);
/* vrt_render with the image in host memory (host_rgba: width*height*4 bytes, which the
 * caller guarantees: the kernel may store to every one of them); waits for the image
 * before returning.
 * - Page-locked host memory (vrt_host_alloc, cudaHostAlloc, cudaHostRegister; 4-byte
 *   aligned) with host_bands = 0: the kernel stores each pixel straight into it over the
 *   host link while it renders; nothing is staged or copied afterwards.
 * - Otherwise (pageable memory, or host_bands > 0) the frame renders into the renderer's
 *   staging buffer and is copied.  With the tile kernel it renders in bands of rows
 *   (vrt_render_opts.host_bands), each band's copy running on the renderer's copy stream
 *   while the next band renders. */
int vrt_render_to_host(vrt_renderer* r, const vrt_world* w, const vrt_uniforms* u, int32_t width,
                       int32_t height, uint8_t* host_rgba, const vrt_render_opts* opts, void* stream);
/* Page-locked host memory for images (cudaMallocHost), for callers without CUDA headers:
 * vrt_render_to_host's kernels store into it directly, and copies into it run
 * asynchronously.  No counterpart in the reference.  vrt_host_free(NULL) is a no-op. */
int vrt_host_alloc(size_t bytes, void** out);
int vrt_host_free(void* p);

/* One camera of a batch. */
typedef struct vrt_view {
    const vrt_world* world;
    vrt_uniforms uniforms;
    int32_t width, height;
    uint8_t* d_rgba;        /* width*height*4 device bytes */
    uint64_t* d_stats;      /* optional, as vrt_render     */
    int32_t tile_w, tile_h; /* this view's ray tile (0 = the launch's): in the tile kernel
                               tile_w*tile_h must equal the launch's tile size; the persistent
                               kernel takes any tile of 1 to 1024 pixels */
    int32_t refill_min;     /* persistent kernel: lanes parked before a warp working on this
                               view's tiles runs its refill phase, 1-32 (0 = the launch's) */
} vrt_view;

/* Many cameras of one world, of uneven sizes, in one launch: the tile kernel over every
 * view's ray tiles (each view may pick its own tile shape of the launch's thread count),
 * or with VRT_KERNEL_BITMASK the persistent kernel, which hands tiles out from a counter,
 * lets each view choose its tile and live-ray refill interval, and needs a world without
 * depth-field words. */
int vrt_render_batch(vrt_renderer* r, const vrt_view* views, int32_t count,
                     const vrt_render_opts* opts, void* stream);

/* vrt_render_batch for callers that may not allocate device memory -- for example a
 * plugin whose host application owns every device allocation, or a frame loop that
 * cannot afford cudaMalloc's implicit device synchronisation.  It has no counterpart in
 * the reference.  It takes no renderer: its scratch (the view table, and the tile counter
 * of the persistent kernel) lives in a static device array of the library, about 46 KiB
 * per GPU, so it calls no cudaMalloc or cudaFree.  Limits:
 *   - at most VRT_NOALLOC_MAX_VIEWS views per call (more: VRT_ERANGE);
 *   - worlds without depth-field words only (VRT_ESTATE otherwise: the tile kernel's stop
 *     masks for such worlds are allocated on first use).
 * It checks and lays out views exactly as vrt_render_batch does.  The view table reaches
 * the device inside kernel parameters, so nothing the call queues refers to the caller's
 * views after it returns.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) and fills a 1 KiB table of the library, with that device
 * current; make that first call before any stream capture.  Every call shares the one
 * array and resets its counter, so calls that overlap on the GPU (other streams, other
 * threads) race: order them on one stream. */
#define VRT_NOALLOC_MAX_VIEWS 64
int vrt_render_batch_noalloc(const vrt_view* views, int32_t count, const vrt_render_opts* opts, void* stream);

/* A captured CUDA graph of vrt_render_batch over a fixed view list of a world without
 * depth-field words; replay with vrt_batch_graph_launch.  Uniform or image-pointer changes
 * need a new graph; edits of the world's words do not. */
typedef struct vrt_batch_graph vrt_batch_graph;
int vrt_batch_graph_create(vrt_renderer* r, const vrt_view* views, int32_t count,
                           const vrt_render_opts* opts, void* stream, vrt_batch_graph** out);
int vrt_batch_graph_launch(vrt_batch_graph* g, void* stream);
int vrt_batch_graph_destroy(vrt_batch_graph* g);

/* ---- serving ---- */
typedef struct vrt_server vrt_server;
typedef struct vrt_server_config {
    uint64_t memory_budget_bytes;   /* bytes the server may hold: its resident worlds' device
                                       bytes plus the images of the requests in flight (40 GiB) */
    int32_t slots;                  /* concurrent batches in flight (streams)          */
    int32_t max_batch;              /* requests per launch                            */
    int32_t max_wait_us;            /* how long a partial batch may wait for company (0: none) */
    int32_t image_memory;           /* where images render: 0 = page-locked host memory, stored
                                       by the kernel (the request's own host_rgba when it is
                                       page-locked and 4-byte aligned, else the slot's buffer);
                                       1 = device memory, copied to the slot's host buffer */
    int32_t max_batch_pixels;       /* pixels per launch (0: no cap): a launch gathers requests while
                                       their pixels stay within it (a larger request goes alone),
                                       so that a request arriving under load waits behind less work */
} vrt_server_config;

#define VRT_REQ_RENDER 0
#define VRT_REQ_EDIT 1

typedef struct vrt_request {
    int32_t kind;                   /* VRT_REQ_RENDER or VRT_REQ_EDIT                  */
    int32_t world_id;
    vrt_uniforms uniforms;          /* render                                         */
    int32_t width, height;          /* render                                         */
    uint8_t* host_rgba;             /* render: result destination (host), may be NULL */
    int32_t cx, cy, cz, radius;     /* edit: removeSphere                             */
    uint64_t user_tag;
} vrt_request;

typedef struct vrt_completion {
    uint64_t user_tag;
    int32_t status;                 /* 0 ok, VRT_EBUDGET when refused                 */
    int32_t kind;
    double submit_ms, start_ms, done_ms; /* server clock: arrival, launch, result ready */
    uint64_t rays;                  /* rays cast (render)                              */
} vrt_completion;

int vrt_server_create(const vrt_server_config* cfg, vrt_server** out);
int vrt_server_destroy(vrt_server* s);
/* Register a resident world (not owned).  Returns its id in *id.  Thread-safe, also
 * while another thread submits or polls. */
int vrt_server_add_world(vrt_server* s, vrt_world* w, int32_t* id);
/* Enqueue a request (thread-safe).  Edits of a world run after every earlier render of
 * that world and before every later one. */
int vrt_server_submit(vrt_server* s, const vrt_request* req);
/* Drive the server: admit, batch and launch queued requests, retire finished ones.
 * Returns the number of completions written to out (up to max_out). */
int vrt_server_poll(vrt_server* s, vrt_completion* out, int32_t max_out);
/* Run until every submitted request has completed (completions are kept for poll). */
int vrt_server_drain(vrt_server* s);
/* Wait, spinning on the slots' events, until a launch in flight has finished (returns 1:
 * the next vrt_server_poll retires it), timeout_us passes or nothing is in flight
 * (returns 0).  Call it from the thread that polls. */
int vrt_server_wait(vrt_server* s, int32_t timeout_us);
double vrt_server_now_ms(const vrt_server* s);

/* ---- measurement helpers ---- */
/* Sustained L2 read bandwidth in GB/s over a resident buffer of the given size. */
int vrt_probe_l2_read_gbs(uint64_t bytes, int32_t iters, double* gbs_out);

#ifdef __cplusplus
}
#endif
#endif /* VRT_H */
