"""The C-ABI libraries load and export every entry point their headers
declare (no compute call: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from magla_gb300 import _native, build

ROOT = Path(__file__).resolve().parent.parent


def declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(uchol_\w+)\s*\(", text, flags=re.M):
        names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libs():
    build.build_all()
    return _native.host(), _native.gpu()


def test_headers_declare_entry_points():
    assert "uchol_factorize" in declared_functions(ROOT / "include" / "uchol_gpu.h")
    assert "uchol_analyze" in declared_functions(ROOT / "include" / "uchol_host.h")


@pytest.mark.parametrize("header,which", [("uchol_host.h", 0), ("uchol_gpu.h", 1)])
def test_every_declared_symbol_is_exported(libs, header, which):
    lib = libs[which]
    missing = [n for n in declared_functions(ROOT / "include" / header) if not hasattr(lib, n)]
    assert not missing, f"{header}: not exported: {missing}"


def test_default_options_without_gpu(libs):
    o = _native.Options()
    libs[1].uchol_default_options(C.byref(o))
    assert o.pivot_tolerance == 1e-13 and o.diagonal_regularization == 1e-10 and o.panel_width == 32
    assert o.allow_diagonal_regularization == 1 and o.precision == 0


def test_null_arguments_are_rejected_without_gpu(libs):
    host, gpu = libs
    assert gpu.uchol_symbolic_create(None, None) == _native.BAD_ARG
    assert gpu.uchol_factorize(None, 0, 0, None, None, None, None) == _native.BAD_ARG
    assert host.uchol_analyze(-1, 0, None, None, 1, 64, None) == _native.BAD_ARG


def test_host_library_validates_csr(libs):
    host, _ = libs
    import numpy as np
    rp = np.array([0, 1, 2], np.int32)
    col = np.array([1, 0], np.int32)   # row 1 references column 0: outside the upper triangle
    h = C.c_void_p()
    st = host.uchol_analyze(2, 2, _native.ptr(rp), _native.ptr(col), 1, 64, C.byref(h))
    assert st == _native.BAD_ARG
