"""Serving loop: each request's result is the same alone and in the mix
(continuous batching with other requests of other sizes, wavelets and
directions in flight), admission respects the memory budget, and the
in-flight memory returns to zero."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    D.lib()
    return D, torch


def test_same_alone_and_in_mix(env):
    D, torch = env
    rng = np.random.default_rng(21)
    src_big = torch.from_numpy(rng.integers(0, 256, size=(2600, 2600)).astype(np.float32)).cuda()
    srv = D.Server(budget_bytes=64 << 30, n_streams=4)
    tracked = []
    for k in range(300):
        if k % 20 == 7:  # large requests take the per-level pipeline inside the server
            w, h = int(rng.integers(1450, 2600)), int(rng.integers(1450, 2600))
        else:
            w, h = int(rng.integers(1, 1100)), int(rng.integers(1, 1100))
        wav = str(rng.choice(["cdf97", "cdf53"]))
        inv = bool(rng.integers(0, 2))
        j = int(rng.integers(1, 7))
        src = src_big[:h, :w]
        if k % 3 == 0:  # tracked: result to a caller buffer
            dst = torch.full((h, w), float("nan"), device="cuda")
            tracked.append((src, dst, wav, inv, j))
            srv.submit(D.Server.request(src, dst, wav, inv, j, tag=k))
        else:  # background load into pooled buffers
            srv.submit(D.Server.request(src, None, wav, inv, j, tag=k, w=w, h=h))
    srv.drain(120)
    torch.cuda.synchronize()
    st = srv.stats()
    assert st["completed"] == 300 and st["bytes_in_use"] == 0 and st["launches"] >= 1
    done = srv.poll(1000)
    assert len(done) == 300 and all(c.status == 0 for c in done)
    assert all(c.t_complete >= c.t_admit >= c.t_submit for c in done)
    bad = []
    for (src, dst, wav, inv, j) in tracked:
        alone = torch.empty_like(dst)
        D.transform2_dev(src, alone, wav, inv, j)
        torch.cuda.synchronize()
        if not torch.equal(alone, dst):
            bad.append((tuple(dst.shape), wav, inv, j))
    assert not bad, bad[:5]
    assert D.lib().dwt_gpu_sync_check() == 0
    srv.close()


def test_admission_budget(env):
    D, torch = env
    src = torch.zeros((512, 512), dtype=torch.float32, device="cuda")
    # a budget that holds about one 512^2 request (output 1 MiB + scratch)
    srv = D.Server(budget_bytes=3 << 20, n_streams=2)
    for k in range(20):
        srv.submit(D.Server.request(src, None, "cdf97", False, 3, tag=k, w=512, h=512))
    srv.drain(60)
    st = srv.stats()
    assert st["completed"] == 20 and st["peak_bytes"] <= (3 << 20) and st["bytes_in_use"] == 0
    # a request larger than the whole budget is refused
    big = torch.zeros((2048, 2048), dtype=torch.float32, device="cuda")
    with pytest.raises(D.DwtError):
        srv.submit(D.Server.request(big, None, "cdf97", False, 3, w=2048, h=2048))
    srv.close()


def test_replay_latencies(env):
    D, torch = env
    rng = np.random.default_rng(3)
    src = torch.zeros((256, 256), dtype=torch.float32, device="cuda")
    srv = D.Server(budget_bytes=1 << 30, n_streams=4)
    n = 2000
    arrival = np.cumsum(rng.exponential(1 / 20000, n))
    reqs = [D.Server.request(src, None, "cdf53", bool(k & 1), 3, tag=k, w=256, h=256) for k in range(n)]
    lat = srv.replay(arrival, reqs)
    assert lat.shape == (n,) and np.all(lat > 0) and np.percentile(lat, 99) < 1.0
    srv.close()


def test_reserved_arena_serves_without_device_allocation(env):
    """After dwt_gpu_server_reserve, a replayed mix of sizes, wavelets and
    directions is served from the reserved arena: no cudaMalloc or
    cudaHostAlloc of the server during the replay, every tracked result equal
    to the same transform alone, and the arena empty afterwards."""
    D, torch = env
    rng = np.random.default_rng(23)
    src_big = torch.from_numpy(rng.integers(0, 256, size=(2600, 2600)).astype(np.float32)).cuda()
    srv = D.Server(budget_bytes=8 << 30, n_streams=4)
    srv.reserve(4 << 30)
    st0 = srv.stats()
    assert st0["arena_bytes"] >= 4 << 30 and st0["completed"] == 0 and st0["bytes_in_use"] == 0
    n = 240
    arrival = np.cumsum(rng.exponential(1 / 2000, n))
    reqs, tracked = [], []
    for k in range(n):
        big = k % 16 == 5
        w = int(rng.integers(1450, 2600)) if big else int(rng.integers(1, 1100))
        h = int(rng.integers(1450, 2600)) if big else int(rng.integers(1, 1100))
        wav = str(rng.choice(["cdf97", "cdf53"]))
        inv = bool(rng.integers(0, 2))
        j = int(rng.integers(1, 7))
        src = src_big[:h, :w]
        if k % 4 == 0:
            dst = torch.full((h, w), float("nan"), device="cuda")
            tracked.append((src, dst, wav, inv, j))
            reqs.append(D.Server.request(src, dst, wav, inv, j, tag=k))
        else:
            reqs.append(D.Server.request(src, None, wav, inv, j, tag=k, w=w, h=h))
    lat = srv.replay(arrival, reqs, timeout_s=120)
    st1 = srv.stats()
    assert lat.shape == (n,) and np.all(lat > 0)
    assert st1["device_allocs"] == st0["device_allocs"], (st0, st1)
    assert st1["completed"] == n and st1["bytes_in_use"] == 0
    bad = []
    for (src, dst, wav, inv, j) in tracked:
        alone = torch.empty_like(dst)
        D.transform2_dev(src, alone, wav, inv, j)
        torch.cuda.synchronize()
        if not torch.equal(alone, dst):
            bad.append((tuple(dst.shape), wav, inv, j))
    assert not bad, bad[:5]
    assert D.lib().dwt_gpu_sync_check() == 0
    srv.close()
