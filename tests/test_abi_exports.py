"""The C-ABI library loads without a GPU and exports every function that
include/flipgraph.h declares (no compute calls: nothing here needs a device)."""
import ctypes
import os
import re

import pytest

fg = pytest.importorskip("flipgraphgpu_gb300")

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "flipgraph.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)   # block comments
    text = re.sub(r"//[^\n]*", " ", text)                 # line comments
    names = re.findall(r"\b(fg_[a-z0-9_]+)\s*\(", text)
    # typedef'd struct names never appear before "(", so every hit is a function
    return sorted(set(names))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for core in ("fg_create", "fg_destroy", "fg_run", "fg_minimize", "fg_validate", "fg_reducer_create",
                 "fg_reducer_run", "fg_reducer_destroy", "fg_last_error", "fg_version"):
        assert core in names
    assert len(names) >= 20


def test_library_exports_every_declared_function():
    lib = fg.library()          # builds the library from source when only sources are present
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_answers_without_a_device():
    lib = fg.library()
    assert lib.fg_version().decode().strip()
    lib.fg_last_error.restype = ctypes.c_char_p
    assert lib.fg_last_error() is not None
    # argument checks run before any CUDA call
    h = ctypes.c_void_p()
    assert lib.fg_create(None, ctypes.byref(h)) != 0
    assert lib.fg_reducer_create(None, 3, 3, 3, 23, None, ctypes.byref(h)) != 0
