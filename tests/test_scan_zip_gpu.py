"""Scans over the fused producer zipWith g xs ys (the reference's delayed scan
input, PTX/CodeGen/Scan.hs:141-439) against the oracle: the zipped array is
formed in the element type (integers wrap, floats round once per element,
float min / max are IEEE fmin / fmax), then scanned by the oracle's scan;
comparison rules as for acc_scan (integers and min / max bit-exact, Float +
within the FP64 oracle's tolerance)."""
import numpy as np
import pytest
import torch

from helpers import TYPES, case_rng, gen, seed_for
from test_fold_zip_gpu import zipped
from test_scan_gpu import FLAVOURS, NAMES, check_scan

pytestmark = pytest.mark.gpu

ZTYPES = ["i32", "i64", "f32", "f64"]
SCAN_OPS = ["+", "min", "max"]
ZIP_OPS = ["+", "*", "min", "max"]


def run_scan_zip(acc, orc, dev, t, f, g, shape, d, k, offset=0, prec=None):
    dt = TYPES[t]
    rng = case_rng("scan_zip", t, f, g, shape, d, k, offset)
    n = int(np.prod(shape))
    src = g if g == "*" else f
    x = gen(dt, src, n, rng)
    y = gen(dt, src, n + offset, rng)
    xs, ys = x.reshape(shape), y[offset:].reshape(shape)
    with np.errstate(over="ignore", invalid="ignore"):
        zs = zipped(g, xs, ys)
    z = seed_for(dt, f)
    tx = torch.from_numpy(x).to(dev).view(shape)
    ty = torch.from_numpy(y).to(dev)[offset:].view(shape)  # offset: a different 16-byte phase
    got = acc.scan_zipwith(NAMES[(d, k)], f, g, z, tx, ty, prec=prec)
    acc.sync()
    got = tuple(v.cpu().numpy() for v in got) if k == 2 else got.cpu().numpy()
    check_scan(orc, got, zs, dt, f, z, d, k)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("f", SCAN_OPS)
@pytest.mark.parametrize("g", ZIP_OPS)
def test_scan_zipwith_grid(acc, orc, dev, t, f, g):
    for d, k in FLAVOURS:
        run_scan_zip(acc, orc, dev, t, f, g, (10_007,), d, k)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("n", [1, 31, 4096, 8193, 100_003, (1 << 20) + 5])
def test_scan_zipwith_sizes(acc, orc, dev, t, n):
    # scanl1 (+) (zipWith (*) xs ys) and scanr' across many look-back tiles
    run_scan_zip(acc, orc, dev, t, "+", "*", (n,), 0, 0)
    run_scan_zip(acc, orc, dev, t, "max", "+", (n,), 1, 2)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("d,k", FLAVOURS)
def test_scan_zipwith_persistent(acc, orc, dev, t, d, k):
    # more than four 32 KiB tiles per SM: the persistent kernel, which zips in
    # its first pass and re-reads the zipped tile from L2 (through the
    # output); the length is not a whole number of 128-byte rows, so the last
    # row is zipped from global memory in both passes
    n = (1 << 23) + 37
    run_scan_zip(acc, orc, dev, t, "+", "*", (n,), d, k)
    run_scan_zip(acc, orc, dev, t, "max", "+", (n,), d, k)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("shape", [(3000, 33), (9728, 40), (5, 10_000)])
def test_scan_zipwith_rows(acc, orc, dev, t, shape):
    # rank 2: one CTA per row, one warp per row (many short rows)
    run_scan_zip(acc, orc, dev, t, "+", "*", shape, 0, 1)
    run_scan_zip(acc, orc, dev, t, "min", "+", shape, 1, 0)


@pytest.mark.parametrize("t", ZTYPES)
def test_scan_zipwith_unaligned_second_input(acc, orc, dev, t):
    # ys one element past a 16-byte boundary: the plain-load look-back kernel
    for n in [4097, 100_003]:
        run_scan_zip(acc, orc, dev, t, "+", "*", (n,), 0, 0, offset=1)
        run_scan_zip(acc, orc, dev, t, "+", "*", (n,), 1, 1, offset=1)


@pytest.mark.parametrize("prec", ["compensated", "fp64"])
def test_scan_zipwith_float32_precisions(acc, orc, dev, prec):
    run_scan_zip(acc, orc, dev, "f32", "+", "*", (3_000_001,), 0, 0, prec=prec)


def test_scan_zipwith_known_answer(acc, dev):
    # scanl (+) 10 (zipWith (+) [0..9] [0..9]) = 10 : running sums of 2i
    xs = torch.arange(10, dtype=torch.int64, device=dev)
    got = acc.scan_zipwith("scanl", "+", "+", 10, xs, xs).cpu().tolist()
    assert got == [10 + sum(2 * j for j in range(i)) for i in range(11)]


def test_scan_zipwith_empty_and_errors(acc, dev):
    e = torch.empty((3, 0), dtype=torch.float32, device=dev)
    assert acc.scan_zipwith("scanl", "+", "*", 2.5, e, e).cpu().tolist() == [[2.5]] * 3
    assert acc.scan_zipwith("scanl1", "+", "*", None, e, e).shape == (3, 0)
    u = torch.zeros(10, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.scan_zipwith("scanl1", "*", "+", None, u, u)
    assert err.value.status == 2  # scan op outside {+, min, max}
    w = torch.zeros(10, dtype=torch.uint32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.scan_zipwith("scanl1", "+", "*", None, w, w)
    assert err.value.status == 2  # Word32 is outside the fused set
    with pytest.raises(ValueError):
        acc.scan_zipwith("scanl1", "+", "*", None, u, u[:5])
