"""CPU tests of the C ABI: libkdgb.so builds for sm_103a, loads, exports every
symbol include/kdgb.h declares, and reports errors instead of crashing when
no GPU is present.  No compute call is made here."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kdgb.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"KDGB_API\s+[\w\s\*]*?\b(kdgb_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("kdgb_build", "kdgb_rebuild", "kdgb_tree_upload", "kdgb_tree_destroy", "kdgb_tree_view_get",
                 "kdgb_tree_download", "kdgb_trace", "kdgb_trace_shadow", "kdgb_trace_primary_shadow",
                 "kdgb_trace_brute", "kdgb_status_string", "kdgb_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol(kdgb_lib):
    from kdgb import _lib
    L = C.CDLL(_lib.library_path())
    for name in declared_symbols():
        assert hasattr(L, name), name
    # The Python binding gives every declared symbol a signature.
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_library_is_sm103a(kdgb_lib):
    from kdgb import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.ARCH)
    assert os.path.getsize(_build.LIB_PATH) > 0


def test_defaults_mirror_reference(kdgb_lib):
    p = kdgb_lib.build_params()
    # TriangleMap.cu:46-48, TriangleMapUpperCreator.cu:28-31, KDNode.h:21
    assert p.lower == kdgb_lib.LOWER_BITMAP and p.propagate_aabbs == 1 and p.traversal_cost == 24.0
    assert p.split_empty_space == 1 and abs(p.empty_space_threshold - 0.35) < 1e-7 and p.leaf_size == 32
    t = kdgb_lib.trace_params()
    # IRayTracer.cu:33-34, ShortStack.cu:25
    assert t.leaf_skipping == 1 and t.stack_depth == 4 and t.tie == kdgb_lib.TIE_LOWEST_ID


def test_status_strings(kdgb_lib):
    L = kdgb_lib.lib()
    assert L.kdgb_status_string(0) == b"ok"
    assert L.kdgb_status_string(9) == b"no CUDA device"
    assert L.kdgb_abi_version() == 6


def test_no_device_is_an_error_not_a_crash(kdgb_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = kdgb_lib.lib()
    h = C.c_void_p()
    p = kdgb_lib.build_params()
    buf = (C.c_float * 9)()
    rc = L.kdgb_build(C.cast(buf, C.c_void_p), 1, C.byref(p), C.byref(h), None)
    assert rc == kdgb_lib.ERR_NO_DEVICE and not h.value
    assert b"no CUDA device" in L.kdgb_last_error()


def test_cpp_plugin_header_compiles_and_links(kdgb_lib, tmp_path):
    """include/kdgb_plugin.hpp (reference class names over the C ABI) builds
    with g++ against libkdgb.so (the program is run by the GPU tests)."""
    import shutil
    import subprocess
    cuda_home = "/usr/local/cuda"
    if not shutil.which("g++") or not os.path.isdir(os.path.join(cuda_home, "include")):
        pytest.skip("g++ or the CUDA headers are missing")
    libdir = os.path.dirname(kdgb_lib.library_path())
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), "-I",
                        os.path.join(cuda_home, "include"), os.path.join(ROOT, "tests", "helpers", "plugin_demo.cpp"),
                        "-L", libdir, "-lkdgb", "-L", os.path.join(cuda_home, "lib64"), "-lcudart",
                        "-o", str(tmp_path / "plugin_demo")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_null_arguments_rejected(kdgb_lib):
    L = kdgb_lib.lib()
    assert L.kdgb_build(None, 1, None, None, None) == 1
    assert L.kdgb_tree_destroy(None) == 0
    assert L.kdgb_trace(None, None, None, None, 0, None, None, None, None, None) == 1
