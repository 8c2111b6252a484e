"""CPU: the C-ABI library builds, loads, and exports every symbol that
include/rmw_gb300.h declares (no compute call is made without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "rmw_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rmw_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_products():
    syms = declared_symbols()
    for s in ("rmw_wall_uf", "rmw_wall_ut", "rmw_wall_wf", "rmw_wall_wt", "rmw_wall_product_host"):
        assert s in syms


def test_library_exports_every_declared_symbol(native_lib):
    missing = [s for s in declared_symbols() if not hasattr(native_lib, s)]
    assert not missing, missing


def test_python_signatures_cover_the_header(native_lib):
    from rigidmultiblobswall_gb300 import _native
    missing = [s for s in declared_symbols() if s not in _native.SIGNATURES]
    assert not missing, missing


def test_version_and_error_string_need_no_gpu(native_lib):
    assert native_lib.rmw_version() >= 1
    assert isinstance(native_lib.rmw_last_error(), bytes)


def test_argument_validation_runs_before_any_device_call(native_lib):
    from rigidmultiblobswall_gb300 import _native
    lib = native_lib
    buf = (ctypes.c_double * 3)()
    # bad kind, bad mode, negative size, non-positive radius: all rejected on the host
    assert lib.rmw_wall_product_host(7, buf, buf, buf, 1, 1.0, 1.0, None, 0) == _native.RMW_ERR_ARG
    assert lib.rmw_wall_product_host(0, buf, buf, buf, 1, 1.0, 1.0, None, 5) == _native.RMW_ERR_ARG
    assert lib.rmw_wall_product_host(0, buf, buf, buf, -1, 1.0, 1.0, None, 0) == _native.RMW_ERR_ARG
    assert lib.rmw_wall_product_host(0, buf, buf, buf, 1, 1.0, 0.0, None, 0) == _native.RMW_ERR_ARG
    assert b"radius" in lib.rmw_last_error()
    # empty input is a no-op
    assert lib.rmw_wall_product_host(0, buf, buf, buf, 0, 1.0, 1.0, None, 0) == _native.RMW_OK
