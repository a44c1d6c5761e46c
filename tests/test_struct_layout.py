"""The ctypes structures of the binding (magla_gb300/_native.py) against the C
declarations of the boundary (include/uchol_gpu.h, include/uchol_host.h): the
same size and the same offset for every field, checked by compiling a probe
with the host C compiler (no GPU needed)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from magla_gb300 import _native

ROOT = Path(__file__).resolve().parent.parent

PAIRS = {
    "uchol_symbolic_desc": _native.SymbolicDesc,
    "uchol_options": _native.Options,
    "uchol_factor_stats": _native.FactorStats,
    "uchol_refine_options": _native.RefineOptions,
    "uchol_refine_stats": _native.RefineStats,
    "uchol_phase_times": _native.PhaseTimes,
    "uchol_autotune_report": _native.AutotuneReport,
    "uchol_cg_options": _native.CgOptions,
    "uchol_cg_result": _native.CgResult,
    "uchol_analysis_info": _native.AnalysisInfo,
}


def _layout_from_c(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "uchol_host.h"', '#include "uchol_gpu.h"',
             "int main(void) {"]
    for cname, cls in PAIRS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, key, val = line.split()
        got[(cname, key)] = int(val)
    return got


def test_ctypes_structures_match_the_headers(tmp_path):
    got = _layout_from_c(tmp_path)
    for cname, cls in PAIRS.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
