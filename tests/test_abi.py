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
