"""Drop-in at the link level: the reference's own C example programs
(examples/{simple,simple-double,simple-perf,start,subbands,perf-plot}),
compiled unchanged against the reference's own header, link against this
library instead of libdwt.o with no unresolved symbol.  Runs only where the
reference sources are present ($DWT_REFERENCE_DIR, else a `reference`
directory beside the repository); nothing is copied."""
import glob
import os
import shutil
import subprocess

import pytest

from oracle import oracle as O

REF = O.reference_dir()
EXAMPLES = ["simple", "simple-double", "simple-perf", "start", "subbands", "perf-plot"]


@pytest.fixture(scope="module")
def lib():
    from libdwt_gb300.buildext import build
    return build()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "examples")) or shutil.which("gcc") is None,
                    reason="reference sources or gcc not present")
@pytest.mark.parametrize("name", EXAMPLES)
def test_reference_example_links_unchanged(lib, name, tmp_path):
    srcs = glob.glob(os.path.join(REF, "examples", name, "*.c"))
    assert len(srcs) == 1
    obj = str(tmp_path / f"{name}.o")
    exe = str(tmp_path / name)
    subprocess.run(["gcc", "-std=c99", "-D_GNU_SOURCE", "-I", os.path.join(REF, "src"), "-c", srcs[0], "-o", obj],
                   check=True, capture_output=True)
    libdir = os.path.dirname(lib)
    r = subprocess.run(["gcc", "-o", exe, obj, "-L", libdir, "-ldwt_gb300", f"-Wl,-rpath,{libdir}",
                        "-Wl,--no-undefined", "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)
