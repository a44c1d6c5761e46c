"""In-tree build of the native libraries.

* ``_lib/libuchol_host.so`` — host half (matrix construction, symbolic phase), g++.
* ``_lib/libuchol_gpu.so``  — device numeric phase for sm_103a, nvcc.

Both are plain C-ABI shared libraries (``include/uchol_host.h``,
``include/uchol_gpu.h``).  Sources are compiled in parallel and a library
is rebuilt only when one of its sources or headers is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent
REPO = ROOT.parent
LIB_DIR = ROOT / "_lib"
OBJ_DIR = ROOT / "_lib" / "obj"
HOST_SRC = sorted((ROOT / "csrc" / "host").glob("*.cpp"))
HOST_HDR = sorted((ROOT / "csrc" / "host").glob("*.hpp")) + [REPO / "include" / "uchol_host.h"]
DEV_CU = [ROOT / "csrc" / "device" / "capi.cu", ROOT / "csrc" / "device" / "static_scratch.cu"]
DEV_CPP = [ROOT / "csrc" / "device" / "plan.cpp"]
DEV_HDR = sorted((ROOT / "csrc" / "device").glob("*.cuh")) + sorted((ROOT / "csrc" / "device").glob("*.hpp")) + [
    REPO / "include" / "uchol_gpu.h"
]
HOST_LIB = LIB_DIR / "libuchol_host.so"
GPU_LIB = LIB_DIR / "libuchol_gpu.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libuchol_gpu.so")
    return cand


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose: bool):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    proc = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}):\n{' '.join(map(str, cmd))}\n{proc.stdout}\n{proc.stderr}")
    return proc


def build_host(verbose: bool = False) -> Path:
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    if not _stale(HOST_LIB, HOST_SRC + HOST_HDR):
        return HOST_LIB
    objs = []
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        futs = []
        for src in HOST_SRC:
            obj = OBJ_DIR / f"host_{src.stem}.o"
            objs.append(obj)
            futs.append(ex.submit(_run, ["g++", *CXXFLAGS, "-c", src, "-o", obj], verbose))
        for f in futs:
            f.result()
    _run(["g++", "-shared", "-o", HOST_LIB, *objs, "-lpthread"], verbose)
    return HOST_LIB


def build_gpu(verbose: bool = False) -> Path:
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    if not _stale(GPU_LIB, DEV_CU + DEV_CPP + DEV_HDR):
        return GPU_LIB
    nvcc = _nvcc()
    objs = []
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        futs = []
        for src in DEV_CU:
            obj = OBJ_DIR / f"dev_{src.stem}.o"
            objs.append(obj)
            futs.append(ex.submit(_run, [nvcc, "-O3", "-std=c++17", ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                                         "-c", src, "-o", obj], verbose))
        for src in DEV_CPP:
            obj = OBJ_DIR / f"dev_{src.stem}.o"
            objs.append(obj)
            futs.append(ex.submit(_run, ["g++", *CXXFLAGS, f"-I{_cuda_home() / 'include'}", "-c", src, "-o", obj],
                                  verbose))
        for f in futs:
            f.result()
    cuda_lib = _cuda_home() / "lib64"
    if not cuda_lib.exists():
        cuda_lib = _cuda_home() / "lib"
    _run([nvcc, "-shared", ARCH, "-o", GPU_LIB, *objs, f"-L{cuda_lib}", "-lcudart", "-lpthread"], verbose)
    return GPU_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        fh = ex.submit(build_host, verbose)
        fg = ex.submit(build_gpu, verbose)
        fh.result()
        fg.result()


if __name__ == "__main__":
    build_all(verbose=True)
