"""The serving arena's bookkeeping (libdwt_gb300/csrc/dwt_arena.h), compiled
with the host compiler over host memory and driven by random allocation and
release sequences (tests/c/arena_test.cpp); no GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_arena_bookkeeping(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "arena_test")
    # the header only needs the runtime's declarations: the host backing
    # never calls into CUDA, so the runtime is linked only to resolve them
    libdir = os.path.join(os.path.dirname(inc), "lib64")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", inc, os.path.join(HERE, "c", "arena_test.cpp"), "-o", exe,
                        "-L", libdir, "-lcudart", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "arena: ok" in r.stdout
