"""acc_scan_noalloc: the scan entry point that performs no device allocation.

It exists for hosts that cannot let the library call cudaMalloc (a stream under
CUDA-graph capture, a fixed device-memory budget, an application-owned pool):
its look-back scratch is a file-scope device array instead of a per-stream
workspace.  These tests call it through the C ABI and compare it with acc_scan,
two calls in a row (the array keeps the previous call's contents, so the
second call checks that the per-call reset works).  Kept in a file that sorts
last so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

I32, I64, F32 = 0, 1, 3


def _call(acc, fn, op, tcode, direction, kind, x, out, sums, outer, inner, seed):
    sp = None
    keep = None
    if seed is not None:
        keep = (ctypes.c_int64 if tcode == I64 else ctypes.c_float if tcode == F32 else ctypes.c_int32)(seed)
        sp = ctypes.cast(ctypes.pointer(keep), ctypes.c_void_p)
    st = fn(op, tcode, 0, direction, kind, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(sums.data_ptr()) if sums is not None else None, outer, inner, sp,
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


CASES = [
    # (dtype, type code, n, direction, kind, seed)
    (torch.int64, I64, (1 << 22) + 3, 0, 0, None),        # scanl1, many look-back tiles
    (torch.int32, I32, (1 << 21) + 17, 0, 1, 5),          # scanl z (n+1 outputs)
    (torch.int32, I32, 100_001, 1, 2, -3),                # scanr' z (+ totals)
    (torch.float32, F32, 1 << 21, 0, 0, None),            # compensated Float32 scanl1
]


@pytest.mark.parametrize("dtype,tcode,n,direction,kind,seed", CASES)
def test_noalloc_matches_acc_scan_on_two_calls(acc, dev, dtype, tcode, n, direction, kind, seed):
    lib = acc.lib()
    g = torch.Generator(device=dev)
    g.manual_seed(n)
    if dtype.is_floating_point:
        x = torch.randn(n, dtype=dtype, device=dev, generator=g)
    else:
        x = torch.randint(-1000, 1000, (n,), dtype=dtype, device=dev, generator=g)
    out_len = n + 1 if kind == 1 else n
    ref = torch.empty(out_len, dtype=dtype, device=dev)
    ref_sums = torch.empty(1, dtype=dtype, device=dev) if kind == 2 else None
    assert _call(acc, lib.acc_scan, 0, tcode, direction, kind, x, ref, ref_sums, 1, n, seed) == 0
    torch.cuda.synchronize()
    for _ in range(2):
        out = torch.full((out_len,), 7, dtype=dtype, device=dev)
        sums = torch.full((1,), 7, dtype=dtype, device=dev) if kind == 2 else None
        assert _call(acc, lib.acc_scan_noalloc, 0, tcode, direction, kind, x, out, sums, 1, n, seed) == 0
        torch.cuda.synchronize()
        if dtype.is_floating_point:
            # the tolerance of the Float32 (+) scan tests: 1e-6 |ref| + 1e-9 sum|x|
            xs = x.double().cpu().numpy()
            ab = np.cumsum(np.abs(xs))
            r = ref.double().cpu().numpy()
            err = np.abs(out.double().cpu().numpy() - r)
            assert np.all(err <= 2 * (1e-6 * np.abs(r) + 1e-9 * ab) + 1e-30)
        else:
            assert torch.equal(out, ref)
            if kind == 2:
                assert torch.equal(sums, ref_sums)


def test_noalloc_rows_and_empty(acc, dev):
    lib = acc.lib()
    x = torch.randint(-50, 50, (3, 1000), dtype=torch.int32, device=dev)
    ref = torch.empty((3, 1001), dtype=torch.int32, device=dev)
    out = torch.empty((3, 1001), dtype=torch.int32, device=dev)
    assert _call(acc, lib.acc_scan, 0, I32, 0, 1, x, ref, None, 3, 1000, 4) == 0
    assert _call(acc, lib.acc_scan_noalloc, 0, I32, 0, 1, x, out, None, 3, 1000, 4) == 0
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    e = torch.empty(0, dtype=torch.int32, device=dev)
    o = torch.empty(1, dtype=torch.int32, device=dev)
    assert _call(acc, lib.acc_scan_noalloc, 0, I32, 0, 1, e, o, None, 1, 0, 9) == 0
    torch.cuda.synchronize()
    assert o.item() == 9


def test_noalloc_rejects_rows_beyond_its_scratch(acc, dev):
    lib = acc.lib()
    x = torch.zeros(16, dtype=torch.int64, device=dev)
    # 2^28 + 1 elements per row exceed the 2 MiB scratch: rejected before any launch
    assert _call(acc, lib.acc_scan_noalloc, 0, I64, 0, 0, x, x, None, 1, (1 << 28) + 1, None) == 8
