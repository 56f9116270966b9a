"""C-ABI boundary: the library builds, loads and exports exactly what
include/vorogpu.h declares; host-side argument checks work without a GPU."""
import ctypes
import os
import re

import pytest

import voro_gb300 as vg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vorogpu.h")


def header_symbols():
    txt = open(HEADER).read()
    return set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s*(vgpu_\w+)\s*\(", txt, flags=re.M))


def test_header_matches_python_binding():
    assert header_symbols() == set(vg.EXPORTED)


def test_library_exports_every_declared_symbol():
    lib = vg.load_library()
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_version_string():
    lib = vg.load_library()
    assert b"sm_103a" in lib.vgpu_version()


def test_null_handle_is_an_argument_error():
    lib = vg.load_library()
    assert lib.vgpu_put(None, 1, None, None) == 16
    assert lib.vgpu_compute(None, 1) == 16
    assert lib.vgpu_get_cells(None, None, None, None, None, None, None, None, None) == 16
    assert lib.vgpu_sum_cell_volumes(None, None) == 16
    assert b"null" in lib.vgpu_last_error()


def test_no_device_is_reported_not_faked():
    if vg.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(vg.VoroError) as e:
        vg.container(0, 1, 0, 1, 0, 1, 2, 2, 2, False, False, False, 8)
    assert e.value.code == 22
