"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point include/brownian_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    from brownian_gb300 import build as b
    return b.build()


def header_symbols(name):
    src = open(os.path.join(ROOT, "include", name)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mpcd_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    syms = header_symbols("brownian_gb300.h")
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_python_mirror_lists_every_symbol(built):
    import brownian_gb300 as bg
    assert sorted(bg.EXPORTS) == header_symbols("brownian_gb300.h")


def test_build_targets_sm_103a_only():
    from brownian_gb300 import build as b
    gencode = [b.NVCC_FLAGS[i + 1] for i, f in enumerate(b.NVCC_FLAGS) if f == "-gencode"]
    assert gencode == ["arch=compute_103a,code=sm_103a"]
