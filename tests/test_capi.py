"""The C-ABI library without a GPU: it loads, exports every function that
include/*.h declares, and rejects bad arguments before any CUDA call."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from voxelproj_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\bVP_API\s+[\w\s\*]+?\b(vp_\w+)\s*\(", text)
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ["vp_forward_z0", "vp_backward_z0", "vp_forward_z2", "vp_backward_z2",
                     "vp_forward", "vp_backward", "vp_error_string", "vp_version"]:
        assert required in names


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports_declared_symbol(name):
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_status_strings():
    for code in range(0, 10):
        assert _lib.LIB.vp_error_string(code)
    assert b"unknown" in _lib.LIB.vp_error_string(99)


DUMMY = ctypes.c_void_p(0x1000)  # never dereferenced: validation fails first


@pytest.mark.parametrize("fn", ["vp_forward_z0", "vp_backward_z0", "vp_forward_z2",
                                "vp_backward_z2", "vp_forward_z0_host", "vp_backward_z0_host",
                                "vp_forward_z2_host", "vp_backward_z2_host"])
def test_validation_errors_without_gpu(fn):
    f = getattr(_lib.LIB, fn)
    good = (4, 5, 6)
    # negative dimension
    assert f(DUMMY, -1, 5, 6, DUMMY, *good, DUMMY, 10, 0, None) == _lib.VP_ERR_BAD_SHAPE
    # too few angles for the sinogram's angle extent (7 angles, 6 given)
    y_dims = (7, 5, 6) if "z0" in fn else (6, 7, 5)
    args = (DUMMY, *good, DUMMY, *y_dims) if "forward" in fn else (DUMMY, *y_dims, DUMMY, *good)
    assert f(*args, DUMMY, 6, 0, None) == _lib.VP_ERR_ANGLES
    # unknown flag bits
    assert f(DUMMY, *good, DUMMY, *good, DUMMY, 10, 1 << 7, None) == _lib.VP_ERR_BAD_FLAGS
    # null data pointer for a non-empty array
    assert f(None, *good, DUMMY, *good, DUMMY, 10, 0, None) == _lib.VP_ERR_NULL_POINTER
    assert f(DUMMY, *good, DUMMY, *good, None, 10, 0, None) == _lib.VP_ERR_NULL_POINTER
    # empty problems succeed without touching the device
    assert f(None, 0, 0, 0, None, 0, 0, 0, None, 0, 0, None) == _lib.VP_OK
    assert f(DUMMY, 4, 5, 0, DUMMY, 4, 5, 0, DUMMY, 10, 0, None) == _lib.VP_OK
    # VP_FLAG_OVERWRITE belongs to the host-buffer entry points only
    ow = f(DUMMY, 4, 5, 0, DUMMY, 4, 5, 0, DUMMY, 10, _lib.VP_FLAG_OVERWRITE, None)
    assert ow == (_lib.VP_OK if fn.endswith("_host") else _lib.VP_ERR_BAD_FLAGS)


def test_dispatch_rejects_bad_z_order():
    dims = (ctypes.c_int64 * 3)(4, 5, 6)
    assert _lib.LIB.vp_forward(DUMMY, dims, DUMMY, dims, DUMMY, 10, 1, 0, None) == \
        _lib.VP_ERR_BAD_Z_ORDER
    assert _lib.LIB.vp_backward(DUMMY, dims, DUMMY, dims, DUMMY, 10, 3, 0, None) == \
        _lib.VP_ERR_BAD_Z_ORDER


def test_batch_validation_without_gpu():
    lib = _lib.LIB
    plan = ctypes.c_void_p()
    p = _lib.BatchProblem()
    p.op = 7  # unknown operation
    arr = (_lib.BatchProblem * 1)(p)
    assert lib.vp_batch_create(arr, 1, ctypes.byref(plan)) == _lib.VP_ERR_BATCH
    p.op = _lib.VP_OP_FORWARD
    p.in_, p.out, p.angles = 0x1000, 0x2000, 0x3000
    p.n_angles = 10
    p.in_dims[:] = [8, 8, 6]     # heights not a multiple of 4
    p.out_dims[:] = [10, 8, 6]
    arr = (_lib.BatchProblem * 1)(p)
    assert lib.vp_batch_create(arr, 1, ctypes.byref(plan)) == _lib.VP_ERR_BATCH
    p.in_dims[:] = [8, 8, 8]
    p.out_dims[:] = [12, 8, 8]   # 12 angles, 10 given
    arr = (_lib.BatchProblem * 1)(p)
    assert lib.vp_batch_create(arr, 1, ctypes.byref(plan)) == _lib.VP_ERR_ANGLES
    assert lib.vp_batch_run(None, None) == _lib.VP_ERR_NULL_POINTER
    assert lib.vp_batch_destroy(None) == _lib.VP_OK


def test_batch_forward_default_matches_header():
    from voxelproj_gb300 import batch

    text = (ROOT / "include" / "voxelproj_gb300.h").read_text()
    m = re.search(r"#define VP_BATCH_FORWARD_DEFAULT (\d+)", text)
    assert m and int(m.group(1)) == batch.FORWARD_DEFAULT


def test_batch_problem_layout_matches_header():
    # int op, flags, variant, reserved; 3 pointers; n_angles; 2 x int64[3]
    assert ctypes.sizeof(_lib.BatchProblem) == 16 + 3 * 8 + 8 + 48


@pytest.mark.parametrize("lang", ["c99", "c++17"])
def test_header_is_plain_c(lang, tmp_path):
    """The public header stands alone as strict C99 and as C++ (no CUDA or
    torch headers needed), so a C, cgo or ctypes caller can use it as is."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c99" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "use_header.c"
    # a typed pointer to an entry point also checks its signature
    src.write_text('#include "voxelproj_gb300.h"\n'
                   "int main(void) {\n"
                   "  vp_batch_problem p; (void)p;\n"
                   "  int (*f)(const float*, int64_t, int64_t, int64_t, float*, int64_t, int64_t,\n"
                   "           int64_t, const float*, int64_t, int, void*) = vp_forward_z0;\n"
                   "  (void)f;\n"
                   "  return 0;\n"
                   "}\n")
    cmd = [cc, "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
           "-I", str(ROOT / "include")]
    cmd += ["-std=c99", str(src)] if lang == "c99" else ["-std=c++17", "-x", "c++", str(src)]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
