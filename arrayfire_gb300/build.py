"""Build recipe for libafgb300.so (sm_103a) — plain nvcc, no CMake.

Each translation unit compiles in parallel to an object file under
``arrayfire_gb300/_build/``; the objects link into
``arrayfire_gb300/libafgb300.so`` with the CUDA runtime linked statically,
so the library needs nothing from a Python environment to load.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libafgb300.so"

SOURCES = [
    "afgb_runtime.cpp",
    "afgb_conv_api.cpp",
    "afgb_foreign.cpp",
    "conv_direct.cu",
    "conv_tma.cu",
    "nn_simt.cu",
    "nn_tc.cu",
    "unwrap_wrap.cu",
    "fft_conv.cu",
    "fft_own.cu",
    "image_ops.cu",
    "harris.cu",
    "canny.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists() and shutil.which(cand) is None:
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libafgb300")
    return cand


def _flags(src: str) -> list[str]:
    f = [
        "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
        "-Xcompiler", "-fvisibility=hidden", "-I", str(ROOT / "include"), "-I", str(CSRC),
    ]
    if src.endswith(".cu"):
        f += ARCH + ["--expt-relaxed-constexpr", "-Xptxas", "-O3"]
    else:
        f += ["-x", "cu"] + ARCH
    return f


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD / (Path(src).stem + ".o")
    srcp = CSRC / src
    deps = [srcp] + list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "afgb300.h"]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return obj
    cmd = [_nvcc(), "-c", str(srcp), "-o", str(obj)] + _flags(src)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    cmd = [_nvcc(), "-shared", "-o", str(LIB)] + [str(o) for o in objs] + ARCH + [
        "-cudart", "static", "-Xcompiler", "-fPIC", "-ldl"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
