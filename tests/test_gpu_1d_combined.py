"""The strided 1D drop-in called the way the reference's callers call it: one
dwt_cdf{97,53}_{f,i}_ex_stride_s call per signal from 16 host threads at once
(src/libdwt.c:5512-5557), in place on a bank of sample-interleaved signals of
mixed lengths, on pageable host memory and on device memory.  Concurrent
calls are combined into shared launches; every signal must still equal the
oracle bit for bit, and no sample outside the signals may change."""
import ctypes as C
import threading

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

LANES = 8
LENGTHS = [1, 2, 3, 4, 5, 17, 64, 255, 1000, 4097]


@pytest.fixture(scope="module")
def env():
    import torch

    import libdwt_gb300 as D
    L = D.lib()
    for w in ("cdf97", "cdf53"):
        for d in ("f", "i"):
            getattr(L, f"dwt_{w}_{d}_ex_stride_s").argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int]
            getattr(L, f"dwt_{w}_{d}_ex_stride_s").restype = None
    return L, torch


def _bank(rng, groups, nmax):
    return rng.uniform(-100, 300, size=(groups, nmax + 3, LANES)).astype(np.float32)


def _calls(groups, seed):
    rng = np.random.default_rng(seed)
    out = []
    for s in range(groups * LANES):
        out.append((s, int(rng.choice(LENGTHS)), str(rng.choice(["cdf97", "cdf53"]))))
    return out


def _addr(base, s, nmax):
    # signal s: group s // LANES, lane s % LANES; samples 32 bytes apart
    return base + ((s // LANES) * (nmax + 3) * LANES + (s % LANES)) * 4


def _oracle(bank, calls, nmax, direction):
    ref = bank.copy()
    base = ref.ctypes.data
    st = LANES * 4
    for s, n, wav in calls:
        p = _addr(base, s, nmax)
        h = p + ((n + 1) // 2) * st
        if direction == "f":
            O.strided_1d(wav, "f", p, p, h, n, st)
        else:
            O.strided_1d(wav, "i", p, h, p, n, st)
    return ref


def _run_threads(L, base, calls, nmax, direction, threads=16):
    st = LANES * 4

    def work(part):
        for s, n, wav in part:
            p = _addr(base, s, nmax)
            h = p + ((n + 1) // 2) * st
            if direction == "f":
                getattr(L, f"dwt_{wav}_f_ex_stride_s")(p, p, h, None, n, st)
            else:
                getattr(L, f"dwt_{wav}_i_ex_stride_s")(p, h, p, None, n, st)
    ths = [threading.Thread(target=work, args=(calls[t::threads],)) for t in range(threads)]
    for th in ths:
        th.start()
    for th in ths:
        th.join()


@pytest.mark.parametrize("where", ["host", "device"])
def test_per_signal_calls_from_16_threads(env, where):
    L, torch = env
    rng = np.random.default_rng(31 if where == "host" else 37)
    groups, nmax = 96, max(LENGTHS)
    bank = _bank(rng, groups, nmax)
    calls = _calls(groups, 5 if where == "host" else 6)
    ref_f = _oracle(bank, calls, nmax, "f")
    ref_i = _oracle(ref_f, calls, nmax, "i")
    if where == "host":
        buf = bank.copy()
        _run_threads(L, buf.ctypes.data, calls, nmax, "f")
        assert np.array_equal(buf.view(np.uint32), ref_f.view(np.uint32)), "forward differs"
        _run_threads(L, buf.ctypes.data, calls, nmax, "i")
        got_i = buf
    else:
        dev = torch.from_numpy(bank.copy()).cuda()
        _run_threads(L, dev.data_ptr(), calls, nmax, "f")
        torch.cuda.synchronize()
        assert np.array_equal(dev.cpu().numpy().view(np.uint32), ref_f.view(np.uint32)), "forward differs"
        _run_threads(L, dev.data_ptr(), calls, nmax, "i")
        torch.cuda.synchronize()
        got_i = dev.cpu().numpy()
    assert np.array_equal(got_i.view(np.uint32), ref_i.view(np.uint32)), "inverse differs"


@pytest.mark.parametrize("n", [24576, 24577, 30001])
def test_long_signals_from_threads(env, n):
    """Signals longer than the one-launch kernel's shared-memory limit (24576
    samples) take the gather / level / scatter launches: the same bits."""
    L, torch = env
    rng = np.random.default_rng(n)
    groups, lanes = 2, LANES
    bank = rng.uniform(-50, 50, size=(groups, n + 3, lanes)).astype(np.float32)
    calls = [(s, n, ("cdf97", "cdf53")[s % 2]) for s in range(groups * lanes)]
    ref_f = _oracle(bank, calls, n, "f")
    ref_i = _oracle(ref_f, calls, n, "i")
    dev = torch.from_numpy(bank.copy()).cuda()
    _run_threads(L, dev.data_ptr(), calls, n, "f", threads=4)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), ref_f.view(np.uint32)), "forward differs"
    _run_threads(L, dev.data_ptr(), calls, n, "i", threads=4)
    torch.cuda.synchronize()
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), ref_i.view(np.uint32)), "inverse differs"
