"""The tensor-core update kernel finds its tiles with closed-form counts and a grouped
order (common.cuh: tc_job_tiles, tc_decode_tile); the plan sizes every launch with the
same counts.  Compiled for the host and checked exhaustively over a sweep of front shapes."""
import subprocess
from pathlib import Path

import pytest

from magla_gb300 import build

ROOT = Path(__file__).resolve().parent.parent


def test_tile_counts_and_decode_agree(tmp_path):
    exe = tmp_path / "tile_decode_check"
    cmd = ["g++", "-O2", "-std=c++17", f"-I{build._cuda_home() / 'include'}",
           f"-I{ROOT / 'magla_gb300' / 'csrc' / 'device'}", str(ROOT / "tests" / "tile_decode_check.cpp"), "-o", str(exe)]
    c = subprocess.run(cmd, capture_output=True, text=True)
    if c.returncode != 0:
        pytest.fail(f"compile failed:\n{c.stderr[-2000:]}")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
