"""The C-ABI library builds for sm_103a, loads, exports every symbol the public
header declares, and rejects bad input before touching a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import gcurval_gb300 as g
from gcurval_gb300 import _lib, build


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    assert os.path.exists(path)
    lib = g.load()
    assert len(_lib.declared_symbols()) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\b(gcv_[a-z0-9_]+)\b", out))
    for header in (_lib.HEADER, _lib.LEARNED_HEADER, _lib.BUNDLE_HEADER):
        declared = _lib.declared_symbols(header)
        assert declared, header
        for name in declared:
            assert hasattr(lib, name), name
            assert name in _lib._SIGS, name  # every declared entry point has a ctypes signature
        assert set(declared) <= exported, header


def test_build_targets_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_status_strings_and_defaults():
    lib = g.load()
    assert lib.gcv_status_string(0) == b"ok"
    assert lib.gcv_status_string(7) == b"no usable CUDA device"
    o = g.default_options(g.GCV_PLAIN_FP64)
    assert o.rtol == 1e-10 and o.max_depth == 30 and o.precision == 0
    m = g.default_options(g.GCV_MIXED)
    assert m.rtol == 1e-8 and m.precision == 1


def test_invalid_options_rejected_without_gpu():
    lib = g.load()
    o = g.default_options()
    o.rtol = 0.0
    h = ctypes.c_void_p()
    a = np.ones(2)
    st = lib.gcv_create_ellipses(ctypes.byref(h), 2, a.ctypes.data_as(ctypes.c_void_p),
                                 a.ctypes.data_as(ctypes.c_void_p), None, None, None, g.GCV_HOST, ctypes.byref(o))
    assert st == _lib.GCV_ERR_INVALID
    assert b"rtol" in lib.gcv_last_error()
    o = g.default_options()
    o.max_depth = 99
    st = lib.gcv_create_ellipses(ctypes.byref(h), 2, a.ctypes.data_as(ctypes.c_void_p),
                                 a.ctypes.data_as(ctypes.c_void_p), None, None, None, g.GCV_HOST, ctypes.byref(o))
    assert st == _lib.GCV_ERR_INVALID


def test_bad_degree_rejected_without_gpu():
    lib = g.load()
    h = ctypes.c_void_p()
    ko = np.array([0, 8], np.int32)
    kv = np.zeros(8)
    cp = np.zeros(8)
    st = lib.gcv_create_bsplines(ctypes.byref(h), 1, 7, 2, ko.ctypes.data_as(ctypes.c_void_p),
                                 kv.ctypes.data_as(ctypes.c_void_p), cp.ctypes.data_as(ctypes.c_void_p), g.GCV_HOST,
                                 None)
    assert st == _lib.GCV_ERR_INVALID


def test_null_handles_rejected():
    lib = g.load()
    assert lib.gcv_destroy(None) == _lib.GCV_ERR_INVALID
    assert lib.gcv_create_arclength_table(None) == _lib.GCV_ERR_INVALID
    assert lib.gcv_free_result(None) == _lib.GCV_ERR_INVALID


def test_bundle_and_f32_arguments_rejected_without_gpu():
    lib = g.load()
    h = ctypes.c_void_p()
    text = b"3 4 8\n0 1 2 3\n0 1 0 1\n0 0 0 0 1 1 1 1\n"
    off = (ctypes.c_int64 * 2)(0, len(text))
    bad_off = (ctypes.c_int64 * 2)(0, len(text) - 1)
    assert lib.gcv_bundle_parse(text, len(text), off, 0, -1, 2, _lib.GCV_HOST, None, ctypes.byref(h)) == \
        _lib.GCV_ERR_INVALID
    assert lib.gcv_bundle_parse(text, len(text), bad_off, 1, -1, 2, _lib.GCV_HOST, None, ctypes.byref(h)) == \
        _lib.GCV_ERR_INVALID
    assert b"n_bytes" in lib.gcv_last_error()
    assert lib.gcv_bundle_parse(text, len(text), off, 1, -1, 4, _lib.GCV_HOST, None, ctypes.byref(h)) == \
        _lib.GCV_ERR_INVALID
    assert lib.gcv_bundle_parse(text, len(text), off, 1, -1, 2, 7, None, ctypes.byref(h)) == _lib.GCV_ERR_INVALID
    assert lib.gcv_bundle_sizes(None, None, None, None) == _lib.GCV_ERR_INVALID
    o = g.default_options()
    kv = np.zeros(8, np.float32)
    cp = np.zeros(8, np.float32)
    ko = np.array([0, 8], np.int32)
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.gcv_create_bsplines_f32(ctypes.byref(h), 1, 7, 2, ptr(ko), ptr(kv), ptr(cp), _lib.GCV_HOST,
                                       ctypes.byref(o)) == _lib.GCV_ERR_INVALID
    assert lib.gcv_create_bsplines_f32(ctypes.byref(h), 1, 3, 4, ptr(ko), ptr(kv), ptr(cp), _lib.GCV_HOST,
                                       ctypes.byref(o)) == _lib.GCV_ERR_INVALID
    assert lib.gcv_create_ellipses_f32(ctypes.byref(h), -1, None, None, None, None, None, _lib.GCV_HOST,
                                       ctypes.byref(o)) == _lib.GCV_ERR_INVALID


def _c_struct_fields(header_text: str, name: str):
    """Field names of `typedef struct name { ... } name;` in the public header."""
    body = re.search(r"typedef struct " + name + r" \{(.*?)\} " + name + ";", header_text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        # "type a, b[N], c": the first declarator carries the type
        for part in decl.split(","):
            fields.append(re.findall(r"([A-Za-z_][A-Za-z0-9_]*)\s*(?:\[[^\]]*\])?\s*$", part.strip())[0])
    return fields


def test_ctypes_structs_mirror_the_header():
    # the Python binding passes these structs by pointer: their fields must be
    # the header's, in the header's order
    text = open(_lib.HEADER).read()
    for py, cname in ((_lib.Options, "gcv_options"), (_lib.Result, "gcv_result"), (_lib.Stats, "gcv_stats")):
        c_fields = _c_struct_fields(text, cname)
        py_fields = [f[0] for f in py._fields_]
        assert py_fields == c_fields, cname


def test_page_locked_allocation_needs_a_gpu():
    # the helpers for page-locked host arrays fail loudly without a device
    lib = g.load()
    if lib.gcv_measure_fma_peak(0, ctypes.byref(ctypes.c_double())) == _lib.GCV_OK:
        pytest.skip("a GPU is present")
    with pytest.raises(g.GcvError):
        g.pinned_empty(16)
    p = ctypes.c_void_p()
    assert lib.gcv_host_alloc(0, ctypes.byref(p)) == _lib.GCV_OK and not p.value
    assert lib.gcv_host_free(None) == _lib.GCV_OK
