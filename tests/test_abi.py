"""The C-ABI library builds, loads and exports every declared entry point.

No CUDA calls are made here (CPU-only environment)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(sbdgb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from sbd_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_abi():
    from sbd_gb300.engine import SYMBOLS
    assert sorted(SYMBOLS) == declared_functions()


def test_host_only_entry_points(lib):
    lib.sbdgb_abi_version.restype = ctypes.c_int
    assert lib.sbdgb_abi_version() == 1
    fp = ctypes.c_size_t(0)
    lib.sbdgb_problem_footprint.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    assert lib.sbdgb_problem_footprint(36, 6000, 6000, 24, 2, 0, ctypes.byref(fp)) == 0
    assert fp.value > 36_000_000 * 8 * 48
    assert lib.sbdgb_problem_footprint(65, 10, 10, 10, 1, 0, ctypes.byref(fp)) != 0


def test_no_oracle_in_product():
    """The product package never imports or links the oracle."""
    pkg = os.path.join(ROOT, "sbd_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.lower(), f
