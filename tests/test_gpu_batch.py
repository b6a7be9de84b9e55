"""Batched persistent transforms: every image of a mixed batch (uneven odd
sizes, both wavelets, both directions) equals the per-image device transform
bit for bit, with fixed parameters and with the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    D.lib()
    return D, torch


def _make(torch, rng, n, lo=1, hi=300):
    imgs = []
    for _ in range(n):
        w, h = int(rng.integers(lo, hi)), int(rng.integers(lo, hi))
        pw = (w + 3) // 4 * 4
        src = torch.zeros((h, pw), dtype=torch.float32, device="cuda")
        src[:, :w] = torch.from_numpy(rng.integers(0, 256, size=(h, w)).astype(np.float32)).cuda()
        imgs.append(dict(src=src[:, :w], dst=torch.full((h, w), float("nan"), device="cuda"),
                         wavelet=str(rng.choice(["cdf97", "cdf53"])), inverse=bool(rng.integers(0, 2)),
                         j_levels=int(rng.choice([-1, 1, 4]))))
    return imgs


def _check_all(D, torch, imgs):
    bad = []
    for k, im in enumerate(imgs):
        h, w = im["dst"].shape
        ref = torch.empty((h, w), dtype=torch.float32, device="cuda")
        D.transform2_dev(im["src"], ref, im["wavelet"], im["inverse"], im["j_levels"])
        torch.cuda.synchronize()
        if not torch.equal(ref, im["dst"]):
            bad.append((k, w, h, im["wavelet"], im["inverse"], im["j_levels"]))
    return bad


@pytest.mark.parametrize("params", [(8, 0, 4), (16, 32, 4), (64, 16, 6), (1, 32, 2)])
def test_batch_matches_per_image(env, params):
    D, torch = env
    rng = np.random.default_rng(params[0] * 100 + params[1])
    imgs = _make(torch, rng, 70)
    b = D.Batch(imgs, params)
    b.run()
    torch.cuda.synchronize()
    assert D.lib().dwt_gpu_sync_check() == 0
    bad = _check_all(D, torch, imgs)
    assert not bad, bad[:5]
    # replay: the graph resets its counters every run
    for im in imgs:
        im["dst"].fill_(float("nan"))
    b.run()
    b.run()
    torch.cuda.synchronize()
    assert not _check_all(D, torch, imgs)
    b.close()


def test_batch_autotuned(env, tmp_path, monkeypatch):
    D, torch = env
    monkeypatch.setenv("DWT_GPU_TUNE_CACHE", str(tmp_path / "tune.txt"))
    rng = np.random.default_rng(5)
    imgs = _make(torch, rng, 40, 33, 600)
    b = D.Batch(imgs, None)
    seg, tail, ctas = b.params
    assert seg in (8, 16, 32, 64) and tail in (0, 16, 32) and ctas in (4, 6)
    for im in imgs:
        im["dst"].fill_(float("nan"))
    b.run()
    torch.cuda.synchronize()
    assert not _check_all(D, torch, imgs)
    assert (tmp_path / "tune.txt").read_text().strip()
    b.close()
    # second plan of the same batch reads the cache
    b2 = D.Batch(imgs, None)
    assert b2.params == (seg, tail, ctas)
    b2.close()
