"""A bounded device wait that runs out: the kernel gives up, the stream's
error word records it, acc_sync reports ACC_ERR_TIMEOUT and clears it, and
the same stream then scans correctly again.

acc_selftest_timeout runs the library's own wait routines against something
that nothing completes: an mbarrier phase with no arrival (the wait of every
TMA-tiled kernel for its tile) and the look-back of a scan tile whose
predecessor never publishes.  Each wait ends after its limit (a few seconds);
no GPU fault is involved.  The reference has no device-side waits: its scan
runs as separate launches (PTX/Execute.hs:438-468)."""
import ctypes
import time

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TIMEOUT = 6  # ACC_ERR_TIMEOUT


def _scan_again(acc, orc, dev, stream):
    rng = np.random.default_rng(11)
    x = rng.integers(-1000, 1000, size=(1 << 20) + 3).astype(np.int64)
    with torch.cuda.stream(stream):
        got = acc.scanl1("+", torch.from_numpy(x).to(dev))
    acc.sync(stream)
    assert np.array_equal(got.cpu().numpy(), orc.scan("+", None, x, 0, 0))


@pytest.mark.parametrize("which", [0, 1], ids=["mbarrier", "lookback"])
def test_wait_runs_out_and_is_reported(acc, orc, dev, which):
    lib = acc.lib()
    stream = torch.cuda.Stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    _scan_again(acc, orc, dev, stream)  # the stream's workspace exists and is clean
    t0 = time.perf_counter()
    assert lib.acc_selftest_timeout(which, sp) == 0
    assert lib.acc_sync(sp) == TIMEOUT
    waited = time.perf_counter() - t0
    assert waited < 20, f"the wait took {waited:.1f} s to give up"
    # the error word was cleared: the next sync is clean, and the stream works
    assert lib.acc_sync(sp) == 0
    _scan_again(acc, orc, dev, stream)


def test_selftest_rejects_unknown_wait(acc):
    assert acc.lib().acc_selftest_timeout(2, None) == 1  # ACC_ERR_INVALID
