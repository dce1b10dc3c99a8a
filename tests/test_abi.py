"""The C ABI library loads without a GPU and exports every entry point its headers declare."""
import ctypes
import os
import re

import numpy as np

from visionaray_gb300 import runtime, types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include", "visionaray_gb300")


def strip_bodies(text):
    """Drops every {...} block (function bodies, struct bodies, extern "C" braces
    excepted by keeping their contents) so that only top-level declarations remain."""
    out, depth, i = [], 0, 0
    text = text.replace('extern "C" {', "").replace("} /* extern \"C\" */", "")
    for ch in text:
        if ch == "{":
            depth += 1
        elif ch == "}":
            depth = max(0, depth - 1)
        elif depth == 0:
            out.append(ch)
    return "".join(out)


def declared_functions():
    names = set()
    for fn in os.listdir(INCLUDE):
        if fn.endswith(".h"):
            text = open(os.path.join(INCLUDE, fn)).read()
            text = strip_bodies(re.sub(r"/\*.*?\*/", "", text, flags=re.S))
            # prototypes only (a declaration ends in ';'); inline helpers are not exports
            names |= set(re.findall(r"\b(gbrt_[a-z0-9_]+)\s*\([^;{}]*\)\s*;", text))
    return names


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "gbrt_trace_closest_hit" in names and "gbrt_bvh_build_lbvh" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = runtime.load_library()
    for name in sorted(declared_functions()):
        assert hasattr(lib, name), f"libgbrt.so does not export {name}"


def test_python_signatures_cover_the_abi():
    assert declared_functions() == set(runtime.SIGNATURES), "runtime.SIGNATURES out of sync with gbrt.h"


def test_abi_version_and_struct_sizes():
    lib = runtime.load_library()
    assert lib.gbrt_abi_version() == 3
    assert types.TRIANGLE.itemsize == 44 and types.RAY.itemsize == 32
    assert types.HIT.itemsize == 16 and types.BVH_NODE.itemsize == 32
    assert types.MATERIAL.itemsize == 64 and types.AREA_LIGHT.itemsize == 60
    assert types.INSTANCE.itemsize == 56 and types.HIT_INST.itemsize == 32
    assert types.LIGHT.itemsize == 108 and types.BATCH_LAUNCH.itemsize == 24


def test_null_context_is_rejected_without_touching_the_gpu():
    lib = runtime.load_library()
    assert lib.gbrt_context_destroy(None) == 1
    assert lib.gbrt_trace_closest_hit(None, None, None, 0, None) == 1
    assert lib.gbrt_bvh_destroy(None) == 1
    assert lib.gbrt_last_error(None) == b"null context"
    out = ctypes.c_void_p()
    assert lib.gbrt_bvh_build_lbvh(None, None, 0, ctypes.byref(out)) == 1
    assert np.uint32(types.NO_HIT) == 0xFFFFFFFF
