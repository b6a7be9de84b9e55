"""Build the CUDA library in tree: libdwt_gb300/_lib/libdwt_gb300.so.

Every .cu under csrc/ is compiled for sm_103a only (one -gencode), in
parallel, then linked into one shared library exporting the C ABI declared in
include/libdwt.h.  Objects go to libdwt_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.environ.get("DWT_GB300_LIB", os.path.join(LIBDIR, "libdwt_gb300.so"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no multiply-add contraction anywhere.  The lifting must round
# the product c*(l + r) before adding it, as the reference's float path does;
# explicit .rn rounding alone did not keep packed f32x2 multiplies and adds
# apart.
# -ffp-contract=off: host code (the harness, the display transform) rounds
# every product too, on both host architectures.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off",
                     "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(os.path.dirname(PKG), "include", "*.h"))


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources() + _headers() + [__file__])


def _compile(src: str, verbose_ptxas: bool, extra_flags=()) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + "".join(extra_flags).replace("-", "_") + ".o")
    cmd = [nvcc()] + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False, extra_flags=()) -> str:
    """Compile and link; returns the library path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas, extra_flags), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-D")]
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, extra_flags=extra))
