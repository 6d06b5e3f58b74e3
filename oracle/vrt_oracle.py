"""ctypes binding of the CPU oracle (oracle/vrt_oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker
or the timed CPU baseline; the product path never imports it.  Also binds the
reference's own code built by oracle/ref/build_ref.sh into oracle/_ref/ (present only
where the reference checkout exists), used to pin the oracle and make golden vectors.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_libs: dict[str, C.CDLL] = {}

_P = C.c_void_p
_I = C.c_int


def build() -> None:
    subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)


def _load(fast: bool = False) -> C.CDLL:
    name = "libvrt_oracle_fast.so" if fast else "libvrt_oracle.so"
    if name not in _libs:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.vrt_oracle_render.restype = _I
        L.vrt_oracle_render.argtypes = [_P, _I, _I, _P, _I, _I, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _I]
        L.vrt_oracle_cast_ray.restype = _I
        L.vrt_oracle_cast_ray.argtypes = [_P, _I, _I, _P, _P, _I, _I, _P, _P, _P, _P]
        L.vrt_oracle_fix_depth_field_box.restype = _I
        L.vrt_oracle_fix_depth_field_box.argtypes = [_P, _I, _I, _I, _I, _I, _I, _I, _I, _I]
        L.vrt_oracle_remove_sphere.restype = _I
        L.vrt_oracle_remove_sphere.argtypes = [_P, _I, _I, _I, _I, _I, _I, _I]
        L.vrt_oracle_init_reference.restype = _I
        L.vrt_oracle_init_reference.argtypes = [_P, _I, _I]
        L.vrt_oracle_depth_offset_count.restype = _I
        _libs[name] = L
    return _libs[name]


def library_path(fast: bool = False) -> str:
    """The oracle library (built if missing); it also exports the host-only scene helpers
    of include/vrt.h (vrt.use_host_library)."""
    _load(fast)
    return os.path.join(HERE, "libvrt_oracle_fast.so" if fast else "libvrt_oracle.so")


def _ptr(a):
    return None if a is None else a.ctypes.data


def render(words: np.ndarray, W: int, H: int, uniforms, width: int, height: int, rows=None, threads: int = 0,
           fast: bool = False, outputs=True):
    """Render rows of a width x height frame.  rows: None (all), or (begin, end, stride).
    outputs: True (every per-pixel output), False (totals only) or a tuple of names out of
    rgba, hit, cast, occ, steps, primary_steps, shade.
    Returns a dict of full-image arrays (unwritten rows zero) and the totals
    (rays cast, DDA iterations, primary hits, pixels)."""
    L = _load(fast)
    rb, re_, rs = (0, height, 1) if rows is None else rows
    shapes = {
        "rgba": ((height, width, 4), np.uint8),
        "hit": ((height, width), np.int32),
        "cast": ((height, width), np.uint32),
        "occ": ((height, width), np.uint32),
        "steps": ((height, width), np.int32),
        "primary_steps": ((height, width), np.int32),
        "shade": ((height, width, 3), np.float32),
    }
    names = tuple(shapes) if outputs is True else (tuple(outputs) if outputs else ())
    out = {k: np.zeros(*shapes[k]) for k in names}
    totals = np.zeros(4, np.uint64)
    g = out.get
    st = L.vrt_oracle_render(words.ctypes.data, W, H, C.addressof(uniforms), width, height, rb, re_, rs,
                             _ptr(g("rgba")), _ptr(g("hit")), _ptr(g("cast")), _ptr(g("occ")), _ptr(g("steps")),
                             _ptr(g("primary_steps")), _ptr(g("shade")), totals.ctypes.data, threads)
    if st != 0:
        raise RuntimeError(f"oracle render failed: {st}")
    out["totals"] = {"rays": int(totals[0]), "steps": int(totals[1]), "hits": int(totals[2]), "pixels": int(totals[3])}
    return out


def cast_ray(words, W, H, start, direction, dist, max_steps):
    L = _load()
    s = np.asarray(start, np.float32)
    d = np.asarray(direction, np.float32)
    hit = C.c_int64()
    hp = np.zeros(3, np.float32)
    hn = np.zeros(3, np.float32)
    steps = C.c_int32()
    L.vrt_oracle_cast_ray(words.ctypes.data, W, H, s.ctypes.data, d.ctypes.data, dist, max_steps, C.byref(hit),
                          hp.ctypes.data, hn.ctypes.data, C.byref(steps))
    return hit.value, hp, hn, steps.value


def fix_depth_field_box(words, W, H, box, threads: int = 0):
    _load().vrt_oracle_fix_depth_field_box(words.ctypes.data, W, H, *box, threads)


def remove_sphere(words, W, H, cx, cy, cz, r, refresh=1):
    _load().vrt_oracle_remove_sphere(words.ctypes.data, W, H, cx, cy, cz, r, refresh)


def init_reference(W=512, H=96):
    words = np.empty(W * H * W, np.int32)
    _load().vrt_oracle_init_reference(words.ctypes.data, W, H)
    return words


def depth_offset_count() -> int:
    return _load().vrt_oracle_depth_offset_count()


# ---------------------------------------------------------------- the reference's own code

def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "librefworld.so")) and os.path.exists(
        os.path.join(REF_DIR, "librefshader.so"))


def build_ref() -> bool:
    """Build oracle/_ref from the reference checkout; False when it is absent."""
    p = subprocess.run(["sh", os.path.join(HERE, "ref", "build_ref.sh")], capture_output=True, text=True)
    return p.returncode == 0


def ref_world() -> C.CDLL:
    if "refworld" not in _libs:
        L = C.CDLL(os.path.join(REF_DIR, "librefworld.so"))
        L.vrt_ref_words.restype = C.POINTER(C.c_int32)
        L.vrt_ref_check_layout.restype = _I
        L.vrt_ref_width.restype = _I
        L.vrt_ref_height.restype = _I
        L.vrt_ref_remove_sphere.argtypes = [_I, _I, _I, _I]
        L.vrt_ref_place_local_light.argtypes = [C.c_float] * 4
        L.vrt_ref_get_local_lights.argtypes = [_P]
        L.vrt_ref_light_pos.argtypes = [C.c_float, _P]
        L.vrt_ref_rotate_matrix.argtypes = [C.c_float, C.c_float, _P]
        if L.vrt_ref_check_layout() != 0:
            raise RuntimeError("reference world layout check failed: voxels[-1] is not the guard word")
        _libs["refworld"] = L
    return _libs["refworld"]


def ref_words_view() -> np.ndarray:
    """The reference's global voxels[] as a numpy view (512*96*512 int32)."""
    L = ref_world()
    n = L.vrt_ref_width() * L.vrt_ref_height() * L.vrt_ref_width()
    return np.ctypeslib.as_array(L.vrt_ref_words(), shape=(n,))


def ref_shader() -> C.CDLL:
    if "refshader" not in _libs:
        L = C.CDLL(os.path.join(REF_DIR, "librefshader.so"))
        L.vrt_refshader_set_world.argtypes = [_P, _I, _I, _I, _I]
        L.vrt_refshader_set_uniforms.argtypes = [_P, _P, C.c_float, _P, _I, _P]
        L.vrt_refshader_run.argtypes = [_P, _P, C.c_int64, _I, _I, _P, _P, _P]
        _libs["refshader"] = L
    return _libs["refshader"]


def ref_shader_run(words, W, H, render_dist, local_light_dist, cam, light, aspect, rot16, view_depth, lights64,
                   width, height, px, py):
    """Run the reference fragment shader (compiled as C++) on the listed pixels."""
    L = ref_shader()
    L.vrt_refshader_set_world(words.ctypes.data, W, H, render_dist, local_light_dist)
    cam = np.asarray(cam, np.float32)
    light = np.asarray(light, np.float32)
    rot = np.asarray(rot16, np.float32)
    lights = np.asarray(lights64, np.float32).reshape(64)
    L.vrt_refshader_set_uniforms(cam.ctypes.data, light.ctypes.data, float(aspect), rot.ctypes.data, view_depth,
                                 lights.ctypes.data)
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    n = px.size
    color = np.zeros((n, 4), np.float32)
    hit = np.zeros(n, np.int32)
    steps = np.zeros(n, np.int32)
    L.vrt_refshader_run(px.ctypes.data, py.ctypes.data, n, width, height, color.ctypes.data, hit.ctypes.data,
                        steps.ctypes.data)
    return color, hit, steps
