"""CPU checks of the C-ABI library: it loads and exports every symbol that
include/ffengine_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

import ffengine_gb300 as ffe

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "ffengine_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b((?:FluidSimulation|CBindings|ffgpu)_\w+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from ffengine_gb300 import build
    build.build()
    return ffe.load_library()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_loader_would_pick_this_library():
    # the reference's loader takes the longest libffengine*.so in the lib directory
    names = [f for f in os.listdir(ffe.LIB_DIR) if f.startswith("libffengine") and f.endswith(".so")]
    assert sorted(names, key=len, reverse=True)[0] == "libffengine_gb300.so"


def test_error_message_buffer_is_readable(lib):
    f = lib.CBindings_get_error_message
    f.restype = ctypes.c_char_p
    assert isinstance(f(), bytes)
