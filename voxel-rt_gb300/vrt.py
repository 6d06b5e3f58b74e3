"""Python binding of the C ABI in include/vrt.h (ctypes over libvrt.so).

This is the host-side mirror of the reference's draw-call interface
(Berry2460/voxel-rt src/render.hpp:30-41): a world is created and uploaded once
(initRender / updateGeometry, render.cpp:313-372, :199-202), edits are scatter calls
(removeSphere, level.cpp:30-56; placeLocalLight, render.cpp:375-385), and a frame is
one render call with the shader's uniforms (updateUniforms, render.cpp:289-302;
glDrawArrays, main.cpp:59).

Device buffers are passed as integer addresses (for example ``tensor.data_ptr()``)
and streams as integer handles (``torch.cuda.current_stream().cuda_stream``).
Every call raises VrtError on a non-zero status.  There is no CPU fallback: if the
library is missing, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libvrt.so")

MAX_LOCAL_LIGHTS = 16

OK = 0
EINVAL, ECUDA, ENOMEM, ERANGE, ETIMEOUT, EBUDGET, ENOTFOUND, ESTATE = -1, -2, -3, -4, -5, -6, -7, -8

KERNEL_AUTO, KERNEL_WORD, KERNEL_BITMASK, KERNEL_MASK_PIXEL = 0, 1, 2, 3
STAT_RAYS, STAT_STEPS, STAT_HITS, STAT_PIXELS, STAT_REFILLS, STAT_SLOW, STAT_FAST, STAT_COUNT = 0, 1, 2, 3, 4, 5, 6, 8
REQ_RENDER, REQ_EDIT = 0, 1
NOALLOC_MAX_VIEWS = 64


class VrtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"vrt status {status}: {msg}")
        self.status = status


class Uniforms(C.Structure):
    """vrt_uniforms: the uniform block of fshader.glsl:20-26 plus its constants."""

    _fields_ = [
        ("camPos", C.c_float * 3),
        ("camRotation", C.c_float * 2),
        ("lightPos", C.c_float * 3),
        ("aspectRatio", C.c_float),
        ("rotateMatrix", C.c_float * 16),
        ("viewDepthField", C.c_int32),
        ("localLights", (C.c_float * 4) * MAX_LOCAL_LIGHTS),
        ("localLightColor", (C.c_float * 3) * MAX_LOCAL_LIGHTS),
        ("tanHalfFov", C.c_float),
        ("maxSteps", C.c_int32),
        ("localLightDist", C.c_float),
        ("ambient", C.c_float),
        ("diffuse", C.c_float),
        ("maxOverbright", C.c_float),
    ]


class DebugOut(C.Structure):
    _fields_ = [
        ("hit_index", C.c_void_p),
        ("cast_mask", C.c_void_p),
        ("occ_mask", C.c_void_p),
        ("steps", C.c_void_p),
        ("primary_steps", C.c_void_p),
        ("shade", C.c_void_p),
    ]


class RenderOpts(C.Structure):
    _fields_ = [
        ("kernel", C.c_int32),
        ("tile_w", C.c_int32),
        ("tile_h", C.c_int32),
        ("refill_min", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("exact_steps", C.c_int32),
        ("host_bands", C.c_int32),
    ]


class WorldInfo(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("num_words", C.c_uint64),
        ("d_words", C.c_void_p),
        ("d_brick_mask", C.c_void_p),
        ("d_region_mask", C.c_void_p),
        ("has_depth_field", C.c_int32),
        ("device_bytes", C.c_uint64),
    ]


class View(C.Structure):
    _fields_ = [
        ("world", C.c_void_p),
        ("uniforms", Uniforms),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("d_rgba", C.c_void_p),
        ("d_stats", C.c_void_p),
        ("tile_w", C.c_int32),
        ("tile_h", C.c_int32),
        ("refill_min", C.c_int32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("memory_budget_bytes", C.c_uint64),
        ("slots", C.c_int32),
        ("max_batch", C.c_int32),
        ("max_wait_us", C.c_int32),
        ("image_memory", C.c_int32),
        ("max_batch_pixels", C.c_int32),
    ]


class Request(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("world_id", C.c_int32),
        ("uniforms", Uniforms),
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("host_rgba", C.c_void_p),
        ("cx", C.c_int32),
        ("cy", C.c_int32),
        ("cz", C.c_int32),
        ("radius", C.c_int32),
        ("user_tag", C.c_uint64),
    ]


class Completion(C.Structure):
    _fields_ = [
        ("user_tag", C.c_uint64),
        ("status", C.c_int32),
        ("kind", C.c_int32),
        ("submit_ms", C.c_double),
        ("start_ms", C.c_double),
        ("done_ms", C.c_double),
        ("rays", C.c_uint64),
    ]


_P = C.c_void_p
_I = C.c_int32
_U64 = C.c_uint64
_F = C.c_float

# name -> (restype, argtypes); the full export list of include/vrt.h
SIGNATURES = {
    "vrt_last_error": (C.c_char_p, []),
    "vrt_version": (C.c_char_p, []),
    "vrt_uniforms_default": (_I, [C.POINTER(Uniforms)]),
    "vrt_init_local_lights": (_I, [C.POINTER(Uniforms)]),
    "vrt_place_local_light": (_I, [C.POINTER(Uniforms), _F, _F, _F, _F]),
    "vrt_rotate_matrix": (_I, [_F, _F, C.POINTER(C.c_float)]),
    "vrt_world_create": (_I, [_I, _I, C.POINTER(_P)]),
    "vrt_world_destroy": (_I, [_P]),
    "vrt_world_get_info": (_I, [_P, C.POINTER(WorldInfo)]),
    "vrt_world_upload": (_I, [_P, _P, _U64, _U64, _P]),
    "vrt_world_upload_device": (_I, [_P, _P, _U64, _U64, _P]),
    "vrt_world_download": (_I, [_P, _P, _U64, _U64, _P]),
    "vrt_world_download_masks": (_I, [_P, _P, _P, _P, _P]),
    "vrt_world_download_distances": (_I, [_P, _P, _P, _P]),
    "vrt_world_sync_flags": (_I, [_P, _P]),
    "vrt_world_probe": (_I, [_P, _P, _I, _P, _P]),
    "vrt_world_save": (_I, [_P, C.c_char_p, _P]),
    "vrt_world_load": (_I, [C.c_char_p, C.POINTER(_P), _P]),
    "vrt_remove_sphere": (_I, [_P, _I, _I, _I, _I, _I, _P]),
    "vrt_place_voxel": (_I, [_P, _I, _I, _I, _I, _P]),
    "vrt_fix_depth_field_box": (_I, [_P, _I, _I, _I, _I, _I, _I, _P]),
    "vrt_world_init_reference": (_I, [_P, _P]),
    "vrt_terrain_generate": (_I, [_P, _I, _I, _U64, _I]),
    "vrt_terrain_height": (_I, [_I, _U64, _I, _I]),
    "vrt_renderer_create": (_I, [C.POINTER(_P)]),
    "vrt_renderer_destroy": (_I, [_P]),
    "vrt_render": (_I, [_P, _P, C.POINTER(Uniforms), _I, _I, _P, C.POINTER(DebugOut), _P,
                        C.POINTER(RenderOpts), _P]),
    "vrt_render_to_host": (_I, [_P, _P, C.POINTER(Uniforms), _I, _I, _P, C.POINTER(RenderOpts), _P]),
    "vrt_host_alloc": (_I, [C.c_size_t, C.POINTER(_P)]),
    "vrt_host_free": (_I, [_P]),
    "vrt_render_batch": (_I, [_P, C.POINTER(View), _I, C.POINTER(RenderOpts), _P]),
    "vrt_render_batch_noalloc": (_I, [C.POINTER(View), _I, C.POINTER(RenderOpts), _P]),
    "vrt_batch_graph_create": (_I, [_P, C.POINTER(View), _I, C.POINTER(RenderOpts), _P, C.POINTER(_P)]),
    "vrt_batch_graph_launch": (_I, [_P, _P]),
    "vrt_batch_graph_destroy": (_I, [_P]),
    "vrt_server_create": (_I, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "vrt_server_destroy": (_I, [_P]),
    "vrt_server_add_world": (_I, [_P, _P, C.POINTER(_I)]),
    "vrt_server_submit": (_I, [_P, C.POINTER(Request)]),
    "vrt_server_poll": (_I, [_P, C.POINTER(Completion), _I]),
    "vrt_server_drain": (_I, [_P]),
    "vrt_server_wait": (_I, [_P, _I]),
    "vrt_server_now_ms": (C.c_double, [_P]),
    "vrt_probe_l2_read_gbs": (_I, [_U64, _I, C.POINTER(C.c_double)]),
}

_lib = None


def lib():
    """Load libvrt.so (built by build.py).  Raises if it is missing: no fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run build.py (or __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> int:
    if status < 0:
        msg = lib().vrt_last_error()
        raise VrtError(status, msg.decode() if msg else "")
    return status


# The host-only entry points (csrc/host.cpp, csrc/terrain.cpp: uniform defaults, camera
# matrix, light slots, seeded terrain).  They need no GPU; use_host_library() points them
# at another build of the same sources, so a CPU-only process can build the seeded scenes
# without loading libvrt.so.
HOST_FUNCTIONS = ("vrt_last_error", "vrt_version", "vrt_uniforms_default", "vrt_init_local_lights",
                  "vrt_place_local_light", "vrt_rotate_matrix", "vrt_terrain_generate", "vrt_terrain_height")
_host_lib = None


def use_host_library(path: str) -> None:
    """Call the host-only entry points in the shared library at path (which exports them
    with the signatures of include/vrt.h) instead of libvrt.so."""
    global _host_lib
    L = C.CDLL(path)
    for name in HOST_FUNCTIONS:
        fn = getattr(L, name)
        fn.restype, fn.argtypes = SIGNATURES[name]
    _host_lib = L


def host_lib():
    return _host_lib if _host_lib is not None else lib()


def _hcheck(status: int) -> int:
    if status < 0:
        msg = host_lib().vrt_last_error()
        raise VrtError(status, msg.decode() if msg else "")
    return status


# ---------------------------------------------------------------- uniforms (host only)

def default_uniforms() -> Uniforms:
    """The reference's constants and start state (fshader.glsl:3-10, main.cpp:26-36)."""
    u = Uniforms()
    _hcheck(host_lib().vrt_uniforms_default(C.byref(u)))
    return u


def rotate_matrix(pitch_x: float, yaw_y: float):
    """rotateMatrix = R_y(yaw) * R_x(pitch) (controls.cpp:136-142), column-major list."""
    m = (C.c_float * 16)()
    _hcheck(host_lib().vrt_rotate_matrix(pitch_x, yaw_y, m))
    return list(m)


def place_local_light(u: Uniforms, x: float, y: float, z: float, a: float) -> int:
    """placeLocalLight (render.cpp:375-385): returns the slot used or -1 when all are taken."""
    slot = _hcheck(host_lib().vrt_place_local_light(C.byref(u), x, y, z, a))
    return -1 if slot >= MAX_LOCAL_LIGHTS else slot


def init_local_lights(u: Uniforms) -> None:
    _hcheck(host_lib().vrt_init_local_lights(C.byref(u)))


def set_camera(u: Uniforms, pos, pitch_x: float, yaw_y: float, width: int, height: int,
               fov_deg: float | None = None) -> None:
    u.camPos[:] = [float(p) for p in pos]
    u.camRotation[:] = [pitch_x, yaw_y]
    u.rotateMatrix[:] = rotate_matrix(pitch_x, yaw_y)
    u.aspectRatio = float(width) / float(height)
    if fov_deg is not None:
        u.tanHalfFov = math.tan(math.radians(fov_deg) / 2.0)


# ---------------------------------------------------------------- objects

class World:
    """A device-resident voxel world (the reference's SSBO, render.cpp:366-369)."""

    def __init__(self, width: int, height: int):
        h = C.c_void_p()
        check(lib().vrt_world_create(width, height, C.byref(h)))
        self.handle = h
        self.width, self.height = width, height
        self.num_words = width * height * width

    def close(self):
        if self.handle:
            lib().vrt_world_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> WorldInfo:
        i = WorldInfo()
        check(lib().vrt_world_get_info(self.handle, C.byref(i)))
        return i

    def upload(self, words, first: int = 0, stream: int = 0):
        """words: a C-contiguous int32 numpy array (host)."""
        check(lib().vrt_world_upload(self.handle, words.ctypes.data, first, words.size, stream))

    def upload_device(self, d_ptr: int, first: int, count: int, stream: int = 0):
        check(lib().vrt_world_upload_device(self.handle, d_ptr, first, count, stream))

    def download(self, out, first: int = 0, stream: int = 0):
        check(lib().vrt_world_download(self.handle, out.ctypes.data, first, out.size, stream))
        return out

    def masks(self, stream: int = 0):
        """(bricks, regions, supers) uint64 arrays of the occupancy hierarchy."""
        import numpy as np
        sw, sh = (self.width + 63) // 64, (self.height + 63) // 64
        ns = sw * sh * sw
        b = np.empty(64 * 64 * ns, np.uint64)
        r = np.empty(64 * ns, np.uint64)
        s = np.empty(ns, np.uint64)
        check(lib().vrt_world_download_masks(self.handle, b.ctypes.data, r.ctypes.data, s.ctypes.data, stream))
        return b, r, s

    def distances(self, stream: int = 0):
        """(brick_dir, region_dist) uint8 arrays: directed brick distances, 8 per brick
        (byte o = octant o), and region distances."""
        import numpy as np
        sw, sh = (self.width + 63) // 64, (self.height + 63) // 64
        bd = np.empty(8 * 64 * 64 * sw * sh * sw, np.uint8)
        rd = np.empty(64 * sw * sh * sw, np.uint8)
        check(lib().vrt_world_download_distances(self.handle, bd.ctypes.data, rd.ctypes.data, stream))
        return bd, rd

    def probe(self, d_xyz: int, n: int, d_words: int, stream: int = 0):
        """Voxel words at n device (x,y,z) int32 triples; -1 outside the world."""
        check(lib().vrt_world_probe(self.handle, d_xyz, n, d_words, stream))

    def save(self, path: str, stream: int = 0):
        check(lib().vrt_world_save(self.handle, path.encode(), stream))

    @classmethod
    def load(cls, path: str, stream: int = 0) -> "World":
        h = C.c_void_p()
        check(lib().vrt_world_load(path.encode(), C.byref(h), stream))
        w = cls.__new__(cls)
        w.handle = h
        info = WorldInfo()
        check(lib().vrt_world_get_info(h, C.byref(info)))
        w.width, w.height = info.width, info.height
        w.num_words = w.width * w.height * w.width
        return w

    def sync_flags(self, stream: int = 0) -> int:
        check(lib().vrt_world_sync_flags(self.handle, stream))
        return self.info().has_depth_field

    def remove_sphere(self, cx, cy, cz, radius, refresh_depth_field=1, stream: int = 0):
        check(lib().vrt_remove_sphere(self.handle, cx, cy, cz, radius, refresh_depth_field, stream))

    def place_voxel(self, x, y, z, word, stream: int = 0):
        check(lib().vrt_place_voxel(self.handle, x, y, z, word, stream))

    def fix_depth_field(self, box=None, stream: int = 0):
        if box is None:
            box = (0, 0, 0, self.width, self.height, self.width)
        check(lib().vrt_fix_depth_field_box(self.handle, *box, stream))

    def init_reference(self, stream: int = 0):
        check(lib().vrt_world_init_reference(self.handle, stream))


class Renderer:
    """Owns the device scratch of the render kernels (one per concurrent stream)."""

    def __init__(self):
        h = C.c_void_p()
        check(lib().vrt_renderer_create(C.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            lib().vrt_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, world: World, u: Uniforms, width: int, height: int, d_rgba: int,
               debug: DebugOut | None = None, d_stats: int = 0, opts: RenderOpts | None = None,
               stream: int = 0):
        check(lib().vrt_render(self.handle, world.handle, C.byref(u), width, height, d_rgba,
                               C.byref(debug) if debug is not None else None, d_stats,
                               C.byref(opts) if opts is not None else None, stream))

    def render_to_host(self, world: World, u: Uniforms, width: int, height: int, host_ptr: int,
                       opts: RenderOpts | None = None, stream: int = 0):
        check(lib().vrt_render_to_host(self.handle, world.handle, C.byref(u), width, height, host_ptr,
                                       C.byref(opts) if opts is not None else None, stream))

    def render_batch(self, views, opts: RenderOpts | None = None, stream: int = 0):
        arr = (View * len(views))(*views)
        check(lib().vrt_render_batch(self.handle, arr, len(views),
                                     C.byref(opts) if opts is not None else None, stream))


def make_view(world: World, u: Uniforms, width: int, height: int, d_rgba: int, d_stats: int = 0,
              tile=None, refill_min: int = 0) -> View:
    v = View()
    v.world = world.handle
    v.uniforms = u
    v.width, v.height = width, height
    v.d_rgba = d_rgba
    v.d_stats = d_stats
    if tile:
        v.tile_w, v.tile_h = tile
    v.refill_min = refill_min
    return v


def terrain_generate(width: int, height: int, seed: int, threads: int = 0):
    import numpy as np
    words = np.empty(width * height * width, dtype=np.int32)
    _hcheck(host_lib().vrt_terrain_generate(words.ctypes.data, width, height, seed, threads))
    return words


def terrain_height(width: int, seed: int, x: int, z: int) -> int:
    return _hcheck(host_lib().vrt_terrain_height(width, seed, x, z))


def probe_l2_read_gbs(nbytes: int = 64 << 20, iters: int = 50) -> float:
    out = C.c_double()
    check(lib().vrt_probe_l2_read_gbs(nbytes, iters, C.byref(out)))
    return out.value
