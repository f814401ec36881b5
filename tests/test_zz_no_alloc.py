"""acc_scan_noalloc: the scan entry point that performs no device allocation.

It exists for hosts that cannot let the library call cudaMalloc: an
integration with a fixed device-memory budget, a host process that hands out
all device memory from its own pool allocator, a loop that must not stall on
cudaMalloc.  Its look-back scratch is a file-scope device array instead of a
per-stream workspace.  These tests call it through the C ABI, two calls in a
row (the array keeps the previous call's contents, so the second call checks
that the per-call clearing works), and compare each result with the oracle
and with acc_scan, within the tolerances of the scan tests: bit-exact for
integers (and equal to acc_scan's bits); Float32 (+) within
1e-6 |ref| + 1e-9 sum|x| of the FP64 oracle and Float64 (+) within
1e-12 sum|x| + 1e-15 |ref|, for both entry points.  One test checks that a call
leaves the device's free memory unchanged.  Kept in a file that sorts last
so that a failure here cannot hide the other tests.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

I32, I64, F32, F64 = 0, 1, 3, 4
CT = {I32: ctypes.c_int32, I64: ctypes.c_int64, F32: ctypes.c_float, F64: ctypes.c_double}


def _call(acc, fn, op, tcode, direction, kind, x, out, sums, outer, inner, seed, stream=None):
    sp = None
    keep = None
    if seed is not None:
        keep = CT[tcode](seed)
        sp = ctypes.cast(ctypes.pointer(keep), ctypes.c_void_p)
    s = stream if stream is not None else torch.cuda.current_stream()
    st = fn(op, tcode, 0, direction, kind, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(sums.data_ptr()) if sums is not None else None, outer, inner, sp,
            ctypes.c_void_p(s.cuda_stream))
    return st


def _oracle(orc, x, direction, kind, seed):
    xs = x.cpu().numpy()
    z = None if seed is None else xs.dtype.type(seed)
    if xs.dtype.kind in "iu":
        return orc.scan("+", z, xs, direction, kind), None
    r64 = orc.scan_f64("+", None if seed is None else float(seed), xs, direction, kind)
    a64 = orc.scan_f64("+", None if seed is None else abs(float(seed)), np.abs(xs), direction, kind)
    return r64, a64


def _check(got, got_sums, ref, ab, kind, dtype):
    if ab is None:
        if kind == 2:
            assert np.array_equal(got, ref[0])
            assert np.array_equal(np.ravel(got_sums), np.ravel(ref[1]))
        else:
            assert np.array_equal(got, ref)
        return
    pairs = [(got, ref[0], ab[0]), (np.ravel(got_sums), np.ravel(ref[1]), np.ravel(ab[1]))] if kind == 2 else [(got, ref, ab)]
    for g, r, a in pairs:
        err = np.abs(np.asarray(g, dtype=np.float64) - r)
        if dtype == torch.float32:
            tol = 1e-6 * np.abs(r) + 1e-9 * a
        else:
            tol = 1e-12 * a + 1e-15 * np.abs(r)
        assert np.all(err <= tol + 1e-30), f"max excess {(err - tol).max()}"


CASES = [
    # (dtype, type code, n, direction, kind, seed)
    (torch.int64, I64, (1 << 22) + 3, 0, 0, None),        # scanl1, many look-back tiles
    (torch.int64, I64, (1 << 21) + 5, 1, 0, None),        # scanr1: the right-to-left look-back
    (torch.int32, I32, (1 << 21) + 17, 0, 1, 5),          # scanl z (n+1 outputs)
    (torch.int32, I32, 100_001, 1, 2, -3),                # scanr' z (+ totals)
    (torch.float32, F32, 1 << 21, 0, 0, None),            # compensated Float32 scanl1
    (torch.float64, F64, (1 << 20) + 9, 1, 1, 0.25),      # Float64 scanr z
]


@pytest.mark.parametrize("dtype,tcode,n,direction,kind,seed", CASES)
def test_noalloc_matches_oracle_and_acc_scan_on_two_calls(acc, orc, dev, dtype, tcode, n, direction, kind, seed):
    lib = acc.lib()
    g = torch.Generator(device=dev)
    g.manual_seed(n)
    if dtype.is_floating_point:
        x = torch.randn(n, dtype=dtype, device=dev, generator=g)
    else:
        x = torch.randint(-1000, 1000, (n,), dtype=dtype, device=dev, generator=g)
    out_len = n + 1 if kind == 1 else n
    ref_gpu = torch.empty(out_len, dtype=dtype, device=dev)
    ref_gpu_sums = torch.empty(1, dtype=dtype, device=dev) if kind == 2 else None
    assert _call(acc, lib.acc_scan, 0, tcode, direction, kind, x, ref_gpu, ref_gpu_sums, 1, n, seed) == 0
    torch.cuda.synchronize()
    ref, ab = _oracle(orc, x, direction, kind, seed)
    for _ in range(2):
        out = torch.full((out_len,), 7, dtype=dtype, device=dev)
        sums = torch.full((1,), 7, dtype=dtype, device=dev) if kind == 2 else None
        assert _call(acc, lib.acc_scan_noalloc, 0, tcode, direction, kind, x, out, sums, 1, n, seed) == 0
        # no look-back wait of the call ran out
        assert lib.acc_scan_noalloc_status(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        got_sums = sums.cpu().numpy() if sums is not None else None
        _check(got, got_sums, ref, ab, kind, dtype)
        # against the entry point it stands in for: the same bits for
        # integers; for floats both within the tolerance of the FP64 oracle
        # (a look-back combines its predecessors' partial sums in the order
        # the tiles happen to finish, so float bits may differ run to run)
        if dtype.is_floating_point:
            _check(ref_gpu.cpu().numpy(), ref_gpu_sums.cpu().numpy() if kind == 2 else None, ref, ab, kind, dtype)
        else:
            assert torch.equal(out, ref_gpu)
            if kind == 2:
                assert torch.equal(sums, ref_gpu_sums)


def test_noalloc_leaves_free_device_memory_unchanged(acc, orc, dev):
    lib = acc.lib()
    n_small, n_big = 1 << 16, (1 << 24) + 7
    x = torch.randint(-9, 9, (n_big,), dtype=torch.int64, device=dev)
    out = torch.empty(n_big, dtype=torch.int64, device=dev)
    # A first call on this device (looks up the array's address and loads the
    # kernel) on a small input ...
    assert _call(acc, lib.acc_scan_noalloc, 0, I64, 0, 0, x, out, None, 1, n_small, None) == 0
    torch.cuda.synchronize()
    # ... then a call on a stream no library call has used before, with more
    # look-back tiles than any earlier call: acc_scan would create and grow a
    # workspace for it here.
    s = torch.cuda.Stream()
    free0, _ = torch.cuda.mem_get_info()
    assert _call(acc, lib.acc_scan_noalloc, 0, I64, 0, 0, x, out, None, 1, n_big, None, stream=s) == 0
    s.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(out.cpu().numpy(), orc.scan("+", None, x.cpu().numpy(), 0, 0))


def test_noalloc_rows_and_empty(acc, orc, dev):
    lib = acc.lib()
    x = torch.randint(-50, 50, (3, 1000), dtype=torch.int32, device=dev)
    ref = torch.empty((3, 1001), dtype=torch.int32, device=dev)
    out = torch.empty((3, 1001), dtype=torch.int32, device=dev)
    assert _call(acc, lib.acc_scan, 0, I32, 0, 1, x, ref, None, 3, 1000, 4) == 0
    assert _call(acc, lib.acc_scan_noalloc, 0, I32, 0, 1, x, out, None, 3, 1000, 4) == 0
    torch.cuda.synchronize()
    assert torch.equal(out, ref)
    assert np.array_equal(out.cpu().numpy(), orc.scan("+", np.int32(4), x.cpu().numpy(), 0, 1))
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


def test_noalloc_graph_replays_see_new_input(acc, orc, dev):
    """The use the entry point is for: one call captured into a CUDA graph
    (after a first call outside capture), then replayed with new input in
    the same buffer.  Every replay clears its status slots in stream order,
    so no tile takes a prefix left by an earlier replay."""
    lib = acc.lib()
    n = (1 << 22) + 3
    gen = torch.Generator(device=dev)
    gen.manual_seed(17)
    x = torch.randint(-1000, 1000, (n,), dtype=torch.int64, device=dev, generator=gen)
    out = torch.empty_like(x)
    assert _call(acc, lib.acc_scan_noalloc, 0, I64, 0, 0, x, out, None, 1, n, None) == 0
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        st = _call(acc, lib.acc_scan_noalloc, 0, I64, 0, 0, x, out, None, 1, n, None)
    assert st == 0
    for step in range(3):
        x.copy_(torch.randint(-1000, 1000, (n,), dtype=torch.int64, device=dev, generator=gen))
        out.fill_(0)
        g.replay()
        torch.cuda.synchronize()
        assert lib.acc_scan_noalloc_status(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)) == 0
        assert np.array_equal(out.cpu().numpy(), orc.scan("+", None, x.cpu().numpy(), 0, 0)), f"replay {step}"
