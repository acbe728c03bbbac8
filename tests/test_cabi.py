"""The C ABI library without a GPU: it loads, exports every function that
include/pars_gpu.h declares, and its host-only entry points work."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

HEADER = os.path.join(ROOT, "include", "pars_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pars_gpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "pars_gpu_trace" in names and "pars_gpu_ftle_generate" in names
    assert len(names) >= 30


def test_library_exports_every_declared_function():
    from pars_gb300 import native
    assert os.path.exists(native.LIBRARY_PATH), "build the library first (__graft_entry__.build())"
    lib = ctypes.CDLL(native.LIBRARY_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIBRARY_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (pars_gpu_\w+)", out))
    assert set(declared_functions()) <= exported


def test_binding_signatures_cover_the_header():
    from pars_gb300 import native
    assert set(declared_functions()) == set(native.SIGNATURES)


def test_abi_version():
    from pars_gb300 import native
    assert native.library().pars_gpu_abi_version() == 1


def test_partition_matches_reference_table():
    from pars_gb300 import native
    for row in golden("partition.npz")["table"]:
        info = native.partition(int(row[0]), int(row[1]), row[2:5])
        got = np.concatenate([info["grid"], info["block"], info["multi_rank"], info["offset"], info["ghosted"], info["neighbors"]])
        assert np.array_equal(got, row[5:])


def test_invalid_arguments_are_rejected_without_a_gpu():
    from pars_gb300 import native
    lib = native.library()
    assert lib.pars_gpu_partition(0, 0, None, None) == -1
    assert lib.pars_gpu_destroy(None) == -1
    assert lib.pars_gpu_trace(None, 0, None, 0, 2, 0, ctypes.c_float(0.1), None) == -1
    handle = ctypes.c_void_p()
    # No device here: create must fail with a status, not crash.
    status = lib.pars_gpu_create(ctypes.byref(handle), 0)
    if status == 0:
        lib.pars_gpu_destroy(handle)
        pytest.skip("a CUDA device is present")
    assert status in (-1, -2)


def test_cpp_drop_in_header_compiles_and_links(tmp_path):
    """include/pa_gpu.hpp (the C++ stage classes, ray tracer and data_io
    included) compiles with the pipeline driver and links against the library
    (running it needs a GPU: tests/test_gpu_drop_in.py)."""
    from pars_gb300 import native
    lib_dir = os.path.dirname(native.LIBRARY_PATH)
    exe = str(tmp_path / "drop_in_pipeline")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "drop_in_pipeline.cpp"), "-L" + lib_dir, "-lpars_gpu",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    assert os.path.exists(exe)


# Shapes whose voxel or seed counts overflow 64-bit or 32-bit arithmetic, or
# that exceed the static scratch of the allocation-free entry point: each is
# rejected by the host-side geometry check before any CUDA call, so this runs
# without a GPU.  (The pointers are host buffers that a rejected call never
# touches.)
NO_ALLOC_BAD_GEOMETRY = [
    # (shape, size, spacing, expected status)
    ((1 << 21, 1 << 21, 3 << 20), (float(1 << 21), float(1 << 21), float(3 << 20)), (1.0, 1.0, 1.0), -6),
    (((1 << 21) + 1, (1 << 21) + 1, (1 << 22) + 1), (float(1 << 21), float(1 << 21), float(1 << 22)), (1.0, 1.0, 1.0), -6),
    ((2, 2, (1 << 18) + 1), (2.0, 2.0, float((1 << 18) + 1)), (1.0, 1.0, 1.0), -6),
    ((65, 65, 65), (65.0, 65.0, 65.0), (1.0, 1.0, 1.0), -6),
    ((16, 16, 16), (1e9, 16.0, 16.0), (1.0, 1.0, 1.0), -1),      # seed lattice far beyond the shape
    ((16, 16, 16), (4e9, 4e9, 4e9), (1.0, 1.0, 1.0), -1),        # int(size / spacing) beyond int32
    ((16, 16, 16), (8.0, 16.0, 16.0), (1.0, 1.0, 1.0), -1),      # fewer seeds than vertices
    ((1, 16, 16), (1.0, 16.0, 16.0), (1.0, 1.0, 1.0), -1),
]


@pytest.mark.parametrize("shape,size,spacing,status", NO_ALLOC_BAD_GEOMETRY)
def test_no_alloc_rejects_bad_geometry_before_any_cuda_call(shape, size, spacing, status):
    from pars_gb300 import native
    lib = native.library()
    dummy = np.zeros(16, np.float32)
    shape = np.array(shape, np.int32)
    offset = np.zeros(3, np.float32)
    size = np.array(size, np.float32)
    spacing = np.array(spacing, np.float32)
    got = lib.pars_gpu_ftle_no_alloc(dummy.ctypes.data, shape.ctypes.data, offset.ctypes.data, size.ctypes.data,
                                     spacing.ctypes.data, 11, 2, 1, 0.01, 0.1, 0, dummy.ctypes.data, None, None)
    assert got == status
