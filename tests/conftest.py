import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA GPU")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


class Golden:
    def __init__(self):
        with open(os.path.join(GOLDEN_DIR, "golden.json")) as f:
            self.meta = json.load(f)
        self.arrays = np.load(os.path.join(GOLDEN_DIR, "golden.npz"))

    def cases(self, kind=None):
        return [c for c in self.meta["cases"] if kind is None or c["kind"] == kind]

    def io(self, case):
        return self.arrays[case["id"] + "_in"], self.arrays[case["id"] + "_out"]


def frame_equal(got: np.ndarray, exp: np.ndarray, sx: int, sy: int, ox: int, oy: int) -> bool:
    """Bitwise equality of two byte buffers holding a float frame at byte
    strides (sx, sy), except that two NaNs compare equal whatever their
    payload (x86 and the GPU produce different default NaN bit patterns when
    an overflowed input yields inf - inf).  Bytes outside the frame must be
    identical."""
    if np.array_equal(got, exp):
        return True
    diff = np.flatnonzero(got != exp)
    ys, xs = np.meshgrid(np.arange(oy), np.arange(ox), indexing="ij")
    starts = (ys * sx + xs * sy).ravel()
    owner = {}
    for k, s0 in enumerate(starts):
        for b in range(4):
            owner[int(s0) + b] = int(s0)
    for d in diff:
        s0 = owner.get(int(d))
        if s0 is None:
            return False
        a = np.frombuffer(got[s0:s0 + 4].tobytes(), np.float32)[0]
        b = np.frombuffer(exp[s0:s0 + 4].tobytes(), np.float32)[0]
        if not (np.isnan(a) and np.isnan(b)):
            return False
    return True


@pytest.fixture(scope="session")
def golden():
    return Golden()
