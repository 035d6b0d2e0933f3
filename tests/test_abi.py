"""CPU checks of the C ABI: libscft.so loads and exports every function that
include/scft.h declares; argument validation that needs no GPU."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "scft.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(scft_[A-Za-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    import scft

    if not os.path.exists(scft.LIB_PATH):
        from scft.build import build

        build()
    return scft.load()


def test_header_and_binding_agree():
    import scft

    assert declared_functions() == sorted(scft.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version_and_error_string(lib):
    assert lib.scft_version() >= 1
    assert isinstance(lib.scft_last_error(), bytes)


def test_null_arguments_are_rejected_without_gpu(lib):
    import scft

    assert lib.scft_create(None, 1, None) == scft.ERR_ARG
    assert lib.scft_calc_poly_density(None) == scft.ERR_ARG
    assert lib.scft_update_1s(None, 1) == scft.ERR_ARG
    assert lib.scft_sync(None) == scft.ERR_ARG
    assert lib.scft_step_fields(None, None, 1, None) == scft.ERR_ARG
    assert lib.scft_iterate_fields(None, None, None, None) == scft.ERR_ARG
    out = ctypes.c_void_p()
    p = scft.make_params()
    assert lib.scft_create(ctypes.byref(p), 0, ctypes.byref(out)) == scft.ERR_ARG
