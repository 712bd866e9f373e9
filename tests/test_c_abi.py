"""The C boundary from C: tests/c/c_caller.c compiles as C99 against
include/afgb300.h, links against libafgb300.so (CPU test), and on a GPU runs
the reference's documented convolution call sequence (GPU test)."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "c" / "c_caller.c"


def _build(tmp_path: Path, lib_dir: Path) -> Path:
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "c_caller"
    cmd = [cc, "-std=c99", "-Wall", "-Werror", "-O1", "-I", str(ROOT / "include"), str(SRC),
           "-L", str(lib_dir), "-lafgb300", "-Wl,-rpath," + str(lib_dir), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_caller_compiles_links_and_loads(aflib_cpu, tmp_path):
    lib_dir = ROOT / "arrayfire_gb300"
    assert (lib_dir / "libafgb300.so").exists()
    exe = _build(tmp_path, lib_dir)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "Invalid input argument"


def test_header_compiles_as_cpp(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "h.cpp"
    src.write_text('#include "afgb300.h"\nint main() { return af_convolve2 == nullptr; }\n')
    r = subprocess.run([cxx, "-std=c++17", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_c_caller_runs_on_gpu(af, tmp_path):
    exe = _build(tmp_path, ROOT / "arrayfire_gb300")
    env = dict(os.environ)
    r = subprocess.run([str(exe), "run"], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok 245"
