"""The inverse level kernel's wide units (two neighbouring 120-column strips
per warp, 544-byte band rows per copy), on the widths where strips pair up,
leave one strip over, or meet the right border inside a pair: one and several
inverse levels of random coefficients on device frames, both wavelets,
bit-exact against the oracle, with odd and even heights (mirrored rows at the
bottom) and pitched sources."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

WIDTHS = [480, 481, 483, 599, 600, 719, 720, 721, 840, 961, 1023, 1024, 1025, 1500, 2047]
HEIGHTS = [16, 17, 33, 130, 257]


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    D.lib()
    return D, torch


def _check(D, torch, wav):
    rng = np.random.default_rng(17 if wav == "cdf97" else 19)
    bad = []
    for w in WIDTHS:
        for h in HEIGHTS:
            for j in (1, 2):
                coef = rng.uniform(-300, 300, size=(h, w)).astype(np.float32)
                ref, _ = O.transform2_dense(coef, wav, "i", j)
                pw = (w + 3) // 4 * 4 + 4  # pitched source (16-byte rows)
                src = torch.zeros((h, pw), dtype=torch.float32, device="cuda")
                src[:, :w] = torch.from_numpy(coef).cuda()
                dst = torch.full((h, w), float("nan"), dtype=torch.float32, device="cuda")
                D.transform2_dev(src[:, :w], dst, wav, True, j)
                torch.cuda.synchronize()
                if not np.array_equal(dst.cpu().numpy(), ref):
                    bad.append((w, h, j))
    return bad


@pytest.mark.parametrize("wav", ["cdf97", "cdf53"])
def test_inverse_level_matches_oracle(env, wav):
    D, torch = env
    bad = _check(D, torch, wav)
    assert not bad, f"{len(bad)} mismatches, first {bad[:8]}"


def test_wide_units_match_oracle():
    """The same sweep with the wide units switched on (DWT_GPU_WIDE_INV=1, read
    once per process: a child process)."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys; sys.path.insert(0, %r); sys.path.insert(0, %r)\n"
            "import torch, libdwt_gb300 as D, test_gpu_wide_inverse as T\n"
            "bad = T._check(D, torch, 'cdf97') + T._check(D, torch, 'cdf53')\n"
            "print('wide mismatches', len(bad), bad[:8])\n"
            "sys.exit(1 if bad else 0)\n") % (root, os.path.join(root, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=900,
                       env=dict(os.environ, DWT_GPU_WIDE_INV="1"))
    assert r.returncode == 0, r.stdout + r.stderr
