"""CPU checks of the C ABI: the library builds, loads and exports every symbol the
header declares, and argument errors are reported without touching a GPU."""
import ctypes
import re
from pathlib import Path

import pytest

from pyinla_gb300 import _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "pyinla_gb300.h"


def header_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(gbta_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_loads():
    from pyinla_gb300 import build

    build.build()
    lib = _lib.load()
    assert lib.gbta_version() >= 100


def test_every_header_symbol_is_exported_and_bound():
    lib = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 20
    for name in syms:
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert set(_lib.SIGNATURES) == set(syms)


def test_argument_errors_without_gpu():
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.gbta_create(0, 4, 2, ctypes.byref(h)) == _lib.GBTA_ERR_ARG
    assert "b >= 1" in _lib.last_error()
    assert lib.gbta_create(32, 4, 4096, ctypes.byref(h)) == _lib.GBTA_ERR_ARG
    assert lib.gbta_pobtaf(None, None, None, None, None) == _lib.GBTA_ERR_ARG
    assert lib.gbta_status(None) == _lib.GBTA_ERR_ARG
    with pytest.raises(_lib.GBTAError):
        _lib.check(lib.gbta_status(None))


def test_check_maps_pivot_to_linalgerror():
    import numpy as np

    lib = _lib.load()
    lib.gbta_set_error(7, b"not positive definite")
    with pytest.raises(np.linalg.LinAlgError):
        _lib.check(7)
