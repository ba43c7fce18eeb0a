"""The C-ABI library builds for sm_103a and exports every symbol include/gmm_gb300.h declares.
No compute call is made here (no GPU is needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "gmm_gb300.h")).read()
    return sorted(set(re.findall(r"^\w[\w\s\*]*?\b(gmm_\w+)\(", src, re.M)))


def test_library_exports_header_symbols():
    from gmm_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from gmm_gb300 import _lib
    with pytest.raises(_lib.GMMError):
        _lib.Handle(0)


def handle_entry_points():
    """Declared functions whose first parameter is a handle (gmm_handle or gmm_server)."""
    src = open(os.path.join(ROOT, "include", "gmm_gb300.h")).read()
    return sorted(set(re.findall(r"^[\w\s\*]*?\b(gmm_\w+)\((?:gmm_handle|gmm_server)\s+\w+", src, re.M)))


def test_null_handle_is_an_argument_error():
    """Every entry point that takes a handle checks it before anything else: with a null handle
    (and null / zero for the other arguments) it returns GMM_ERR_ARG and touches no device (this
    runs without a GPU); destroying a null handle is a no-op, and the queries answer for it
    (no error text, no launches, -GMM_ERR_ARG profile entries)."""
    from gmm_gb300 import build, _lib
    lib = ctypes.CDLL(build.build())
    names = handle_entry_points()
    assert len(names) >= 50
    checked = 0
    for name in names:
        res, args = _lib.SIGNATURES[name]
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
        vals = []
        for a in args:
            if a in (ctypes.c_float, ctypes.c_double):
                vals.append(0.0)
            elif a in (ctypes.c_int, ctypes.c_long, ctypes.c_longlong, ctypes.c_size_t, ctypes.c_uint):
                vals.append(0)
            else:
                vals.append(None)
        got = fn(*vals)
        if name in ("gmm_destroy", "gmm_server_destroy"):
            assert got == 0, name
        elif name in ("gmm_last_error", "gmm_server_last_error"):
            assert got is None or isinstance(got, bytes), name
        elif name == "gmm_profile_read":
            assert got == -_lib.ERR_ARG, name
        elif name == "gmm_launch_count":  # a count, not a status
            assert got == 0, name
        else:
            assert got == _lib.ERR_ARG, (name, got)
        checked += 1
    assert checked == len(names)
