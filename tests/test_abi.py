"""The C ABI library loads without a GPU and exports every function include/*.h declares."""
import ctypes
import glob
import os
import re

import vrt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(vrt_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_api():
    names = declared_functions()
    assert {"vrt_render", "vrt_world_create", "vrt_remove_sphere", "vrt_render_batch", "vrt_server_submit"} <= names


def test_library_exports_every_declared_symbol(vrt_lib):
    lib = ctypes.CDLL(vrt.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_the_header(vrt_lib):
    assert declared_functions() <= set(vrt.SIGNATURES)


def test_version_and_error_string(vrt_lib):
    assert b"sm_103a" in vrt_lib.lib().vrt_version()
    assert vrt_lib.lib().vrt_uniforms_default(None) == vrt.EINVAL
    assert b"NULL" in vrt_lib.lib().vrt_last_error()


def test_struct_sizes_match_the_header(vrt_lib):
    # vrt_uniforms: 3+2+3+1+16 floats, int, 64 floats, 48 floats, float, int, 4 floats
    assert ctypes.sizeof(vrt.Uniforms) == 4 * (3 + 2 + 3 + 1 + 16 + 1 + 64 + 48 + 1 + 1 + 4)
    assert ctypes.sizeof(vrt.DebugOut) == 6 * 8
