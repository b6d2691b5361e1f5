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


C_TYPES = {"int32_t": ctypes.c_int32, "uint64_t": ctypes.c_uint64, "int64_t": ctypes.c_int64, "double": ctypes.c_double,
           "float": ctypes.c_float, "uint32_t": ctypes.c_uint32}


def declared_structs():
    """{typedef name: [(field, C type or 'pointer')]} for every `typedef struct { ... } name;`."""
    text = re.sub(r"/\*.*?\*/", " ", open(HEADER).read(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.fullmatch(r"([a-z0-9_]+)\s*(\*?)\s*(\w+)", decl)
            assert m, decl
            fields.append((m.group(3), "pointer" if m.group(2) else m.group(1)))
        out[name] = fields
    return out


@pytest.mark.parametrize("c_name,py_name", [("fg_config", "Config"), ("fg_records", "_Records"),
                                            ("fg_stats", "Stats"), ("fg_reducer_config", "ReducerConfig")])
def test_ctypes_structs_mirror_the_header(c_name, py_name):
    """The Python mirror passes these structs by pointer: every field, in order, with the
    header's type (a missing trailing field would let the library read past the struct)."""
    c_fields = declared_structs()[c_name]
    py_fields = getattr(fg, py_name)._fields_
    assert [n for n, _ in py_fields] == [n for n, _ in c_fields]
    for (name, ctype), (_, pytype) in zip(c_fields, py_fields):
        want = ctypes.c_void_p if ctype == "pointer" else C_TYPES[ctype]
        assert pytype == want, (c_name, name, ctype, pytype)


@pytest.mark.parametrize("ring", ["z2", "zt", "zb"])
def test_engine_checks_record_layouts_before_the_library_sees_them(ring):
    """Records are passed to fg_set_records / fg_get_records as raw pointers: the Python
    mirror rejects arrays whose shape, type or contiguity differ from the handle's."""
    import numpy as np
    eng = fg.Engine.__new__(fg.Engine)  # sizes only; no device handle is created
    eng.walks, eng.cap, eng.ring, eng.h = 6, 27, ring, None
    eng._match(fg.Records(6, 27, ring))
    eng._match(fg.Records(6, 27, ring, lists=False))
    bad = [fg.Records(5, 27, ring), fg.Records(6, 28, ring), fg.Records(6, 27, "z2" if ring != "z2" else "zt")]
    r = fg.Records(6, 27, ring)
    r.fac = r.fac[:, :, :20]
    bad.append(r)
    r = fg.Records(6, 27, ring)
    r.m = r.m.astype(np.int64)
    bad.append(r)
    r = fg.Records(6, 27, ring)
    r.best_fac = np.asfortranarray(r.best_fac)
    bad.append(r)
    for rec in bad:
        with pytest.raises(ValueError):
            eng._match(rec)


def test_integration_stub_lists_every_config_field():
    """The ctypes binding a maintainer copies from INTEGRATION.md names every field of fg_config,
    in order, with the types the package's own mirror uses."""
    doc = open(os.path.join(os.path.dirname(HEADER), "..", "INTEGRATION.md")).read()
    block = doc[doc.index("class Config(ctypes.Structure)"):]
    block = block[:block.index("]") + 1]
    stub = [(name, getattr(ctypes, t)) for name, t in re.findall(r'\("([a-z_0-9]+)", ctypes\.(c_[a-z0-9]+)\)', block)]
    assert stub == list(fg.Config._fields_)
