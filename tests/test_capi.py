"""CPU checks of the C ABI: the library builds, loads, and exports every entry
point declared in include/vmc_gb300.h (no compute calls without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*int\s+(vmc_\w+)\s*\(", src, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    from vmc_torch_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "vmc_slater_sweep" in names and "vmc_hubbard_conn" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lib):
    from vmc_torch_gb300 import _lib
    assert declared_symbols() == set(_lib.SIGNATURES)
    lib.vmc_abi_version.restype = ctypes.c_int
    assert lib.vmc_abi_version() >= 1


def test_argument_validation_without_gpu(lib):
    # invalid sizes are rejected before any launch (status 1), so this is safe on a CPU-only host
    lib.vmc_pack.restype = ctypes.c_int
    assert lib.vmc_pack(None, ctypes.c_int64(4), 65, None, None, None) == 1
    lib.vmc_slater_sweep.restype = ctypes.c_int
    from vmc_torch_gb300 import _lib
    lib.vmc_slater_sweep.argtypes = _lib.SIGNATURES["vmc_slater_sweep"]
    assert lib.vmc_slater_sweep(None, 16, 65, None, 4, 8, None, 10, 1, 0.25, 0, 0, None, None, None, None, None,
                                None, None, None, None) == 1
