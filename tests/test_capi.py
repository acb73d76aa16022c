"""The C-ABI library builds, loads and exports every symbol the header declares."""
import ctypes
import os
import re

import pytest

import helpers as H


def header_symbols():
    txt = open(os.path.join(H.REPO, 'include', 'ufo_gb300.h')).read()
    return sorted(set(re.findall(r'\b(ufo_[a-z_0-9]+)\s*\(', txt)))


def test_library_exports_header_symbols():
    from ufo_gb300 import build
    so = build.build()
    lib = ctypes.CDLL(so)
    syms = header_symbols()
    assert 'ufo_track' in syms and 'ufo_ctx_create' in syms
    for s in syms:
        assert hasattr(lib, s), s


def test_binding_signatures_cover_header():
    from ufo_gb300 import capi
    assert set(header_symbols()) <= set(capi.SIGNATURES)


def test_errors_are_reported_not_crashed():
    from ufo_gb300 import capi
    lib = capi.load()
    # null arguments are rejected before any CUDA call
    assert lib.ufo_ctx_create(0, None) == -1
    assert b'null' in lib.ufo_last_error()
    assert lib.ufo_track(None, None, None, None, None, 0, 1, 0, 0, 0, 1, None, None, None) == -1


def test_product_path_does_not_import_oracle():
    import ufo_gb300
    root = os.path.dirname(ufo_gb300.__file__)
    for dp, _, files in os.walk(root):
        for f in files:
            if f.endswith('.py'):
                assert 'oracle' not in open(os.path.join(dp, f)).read().split('"""')[-1] \
                    or f == '__init__.py', f
