"""CPU-side checks of the C-ABI boundary: the library builds, loads and
exports every entry point that include/afmib.h declares. No compute calls."""
import ctypes

import pytest

from afmibins_gb300 import build, capi


def test_library_exports_declared_symbols():
    lib = capi.load()
    declared = capi.declared_symbols()
    assert len(declared) >= 27
    missing = [name for name in declared if not hasattr(lib, name)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(capi.declared_symbols()) <= set(capi._SIGS)


def test_error_strings_without_gpu():
    lib = capi.load()
    assert lib.afmib_error_string(capi.AFMIB_OK) == b"ok"
    assert lib.afmib_error_string(capi.AFMIB_ERR_NOCONV) == b"iteration cap reached"
    assert lib.afmib_error_string(99) == b"unknown status"


def test_config_layout_matches_header():
    # the ctypes mirror must agree with the C struct: 9 ints (+pad), 4 doubles, 2 ints, 2 doubles, 1 int (+pad)
    assert ctypes.sizeof(capi.Config) == 9 * 4 + 4 + 4 * 8 + 2 * 4 + 2 * 8 + 8


def test_build_is_in_tree():
    assert capi.library_path().startswith(build.PKG)
