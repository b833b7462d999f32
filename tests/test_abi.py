"""C-ABI checks that need no GPU: the library builds, loads, exports every symbol declared in
include/sst.h with the Python prototypes, and fails loudly (no CPU fallback) without a device."""
import ctypes
import os
import re

import pytest

from seesharp_gb300 import _native
from seesharp_gb300 import build as sst_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "sst.h")).read()
    return sorted(set(re.findall(r"^int\s+(sst_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    sst_build.build()
    return _native.load_library()


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s


def test_python_prototypes_cover_the_header():
    assert set(declared_symbols()) == set(_native.SIGNATURES)


def test_struct_layouts_match_header():
    # sizes that the C declarations imply
    assert ctypes.sizeof(_native.SstRay) == 32
    assert ctypes.sizeof(_native.SstHit) == 48
    assert ctypes.sizeof(_native.SstGenericMaterial) == 44
    assert ctypes.sizeof(_native.SstPathTracerParams) == 48
    assert ctypes.sizeof(_native.SstRenderStats) == 104


def test_tuning_struct_matches_header():
    """SstTuning grows with the launch options; the ctypes mirror must list the header's int32
    fields in the header's order."""
    text = open(os.path.join(ROOT, "include", "sst.h")).read()
    body = re.search(r"typedef struct SstTuning \{(.*?)\} SstTuning;", text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"int32_t\s+(\w+)\s*;", body)
    assert [n for n, _ in _native.SstTuning._fields_] == fields
    assert all(t is ctypes.c_int32 for _, t in _native.SstTuning._fields_)
    assert ctypes.sizeof(_native.SstTuning) == 4 * len(fields)


def test_version_and_error_buffer(lib):
    maj, mnr = ctypes.c_int32(), ctypes.c_int32()
    assert lib.sst_version(ctypes.byref(maj), ctypes.byref(mnr)) == 0
    assert (maj.value, mnr.value) >= (0, 1)
    buf = ctypes.create_string_buffer(16)
    assert lib.sst_last_error(buf, 16) == 0
    assert lib.sst_last_error(None, 0) == -1


def test_invalid_arguments_are_rejected_without_a_device(lib):
    # NULL handles never reach the device
    assert lib.sst_scene_create(None, None) == -1
    assert lib.sst_render(None, None, None, 0, None) == -1
    assert lib.sst_trace(None, None, 0, None, 0) == -1


@pytest.mark.skipif(os.path.exists("/dev/nvidia0"), reason="a GPU is present")
def test_no_device_is_an_error_not_a_fallback(lib):
    h = ctypes.c_void_p()
    rc = lib.sst_create(0, ctypes.byref(h))
    assert rc in (-1, -3)
    assert _native.last_error()
