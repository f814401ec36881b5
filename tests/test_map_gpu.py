"""Folds and scans over the fused producer map (\\x -> g x c) xs for a
primitive g and a constant c (the reference's delayed inputs,
PTX/CodeGen/Fold.hs:80-97 and PTX/CodeGen/Scan.hs:141-439) against the
oracle: the mapped array is formed in the element type (integers wrap, floats
round once per element, float min / max are IEEE fmin / fmax), then folded or
scanned by the oracle; comparison rules as for acc_fold / acc_scan
(tests/helpers.py).  The reference's own known answer,
sum (map (+1) [1..10000]) == 50015000, runs through the fused fold."""
import json
import pathlib

import numpy as np
import pytest
import torch

from helpers import TYPES, assert_fold_close, case_rng, gen, seed_for
from test_fold_zip_gpu import zipped
from test_scan_gpu import FLAVOURS, NAMES, check_scan

pytestmark = pytest.mark.gpu

MTYPES = ["i32", "i64", "f32", "f64"]
OPS = ["+", "min", "max"]
MAP_OPS = ["+", "*", "min", "max"]
GOLDEN = json.loads((pathlib.Path(__file__).parent / "golden" / "known_answers.json").read_text())


def constant(dt, g):
    dt = np.dtype(dt)
    if g == "*":
        return dt.type(2 if dt.kind in "iu" else 0.5)
    if g == "+":
        return dt.type(3 if dt.kind in "iu" else 0.25)
    return dt.type(0 if dt.kind in "iu" else 0.1)


def mapped(g, xs, c):
    with np.errstate(over="ignore", invalid="ignore"):
        return zipped(g, xs, np.full_like(xs, c))


def run_fold_map(acc, orc, dev, t, f, g, shape, seeded, offset=0, prec=None):
    dt = TYPES[t]
    rng = case_rng("fold_map", t, f, g, shape, seeded, offset)
    n = int(np.prod(shape))
    x = gen(dt, g if g == "*" else f, n + offset, rng)
    xs = x[offset:].reshape(shape)
    c = constant(dt, g)
    ms = mapped(g, xs, c)
    z = seed_for(dt, f) if seeded else None
    tx = torch.from_numpy(x).to(dev)[offset:].view(shape)
    got = acc.fold_map(f, g, c.item(), z, tx, prec=prec).cpu().numpy()
    ref = orc.fold(f, dt(z) if seeded else None, ms)
    ref64 = absum = None
    if np.dtype(dt).kind == "f" and f == "+":
        ref64 = orc.fold_f64(f, float(z) if seeded else None, ms)
        absum = orc.fold_f64("+", abs(float(z)) if seeded else None, np.abs(ms))
    assert_fold_close(got, ref, ref64, absum, dt, f, prec)


def run_scan_map(acc, orc, dev, t, f, g, shape, d, k, offset=0):
    dt = TYPES[t]
    rng = case_rng("scan_map", t, f, g, shape, d, k, offset)
    n = int(np.prod(shape))
    x = gen(dt, g if g == "*" else f, n + offset, rng)
    xs = x[offset:].reshape(shape)
    c = constant(dt, g)
    ms = mapped(g, xs, c)
    z = seed_for(dt, f)
    tx = torch.from_numpy(x).to(dev)[offset:].view(shape)
    got = acc.scan_map(NAMES[(d, k)], f, g, c.item(), z, tx)
    acc.sync()
    got = tuple(v.cpu().numpy() for v in got) if k == 2 else got.cpu().numpy()
    check_scan(orc, got, ms, dt, f, z, d, k)


def test_sum_map_succ_known_answer(acc, dev):
    """The reference's known answer through the fused map: sum (map (+1) xs)."""
    ka = GOLDEN["sum_map_succ"]
    lo, hi = ka["input_range"]
    xs = torch.arange(lo, hi + 1, dtype=torch.int64, device=dev)
    assert int(acc.fold_map("+", "+", 1, ka["seed"], xs).item()) == ka["expect"]
    # Int32 and the seedless fold1 give the same
    assert int(acc.fold_map("+", "+", 1, None, xs.to(torch.int32)).item()) == ka["expect"]


@pytest.mark.parametrize("t", MTYPES)
@pytest.mark.parametrize("f", OPS)
@pytest.mark.parametrize("g", MAP_OPS)
def test_fold_map_grid(acc, orc, dev, t, f, g):
    for shape in [(1, 1), (5, 17), (3000, 33), (1, 100_003), (2, 1_000_001)]:
        run_fold_map(acc, orc, dev, t, f, g, shape, seeded=True)
    run_fold_map(acc, orc, dev, t, f, g, (7, 50_001), seeded=False)
    run_fold_map(acc, orc, dev, t, f, g, (1, 100_003), seeded=True, offset=1)  # off the 16-byte phase


@pytest.mark.parametrize("prec", ["plain", "compensated", "fp64"])
def test_fold_map_float32_precisions(acc, orc, dev, prec):
    run_fold_map(acc, orc, dev, "f32", "+", "*", (1, 3_000_001), seeded=True, prec=prec)


@pytest.mark.parametrize("t", MTYPES)
@pytest.mark.parametrize("f", OPS)
@pytest.mark.parametrize("g", MAP_OPS)
def test_scan_map_grid(acc, orc, dev, t, f, g):
    for d, k in FLAVOURS:
        run_scan_map(acc, orc, dev, t, f, g, (10_007,), d, k)


@pytest.mark.parametrize("t", MTYPES)
@pytest.mark.parametrize("n", [1, 31, 4097, 100_003, (1 << 20) + 5])
def test_scan_map_sizes(acc, orc, dev, t, n):
    # the TMA tile kernel (aligned), across many look-back tiles
    run_scan_map(acc, orc, dev, t, "+", "+", (n,), 0, 0)
    run_scan_map(acc, orc, dev, t, "max", "*", (n,), 1, 2)
    # one element past a 16-byte boundary: the plain-load look-back kernel
    run_scan_map(acc, orc, dev, t, "+", "+", (n,), 0, 1, offset=1)


@pytest.mark.parametrize("t", MTYPES)
@pytest.mark.parametrize("d,k", FLAVOURS)
def test_scan_map_persistent(acc, orc, dev, t, d, k):
    # more than four 32 KiB tiles per SM: the persistent kernel, which maps
    # each row as it reads it in both passes
    n = (1 << 23) + 37
    run_scan_map(acc, orc, dev, t, "+", "+", (n,), d, k)
    run_scan_map(acc, orc, dev, t, "min", "*", (n,), d, k)


@pytest.mark.parametrize("t", MTYPES)
@pytest.mark.parametrize("shape", [(3000, 33), (9728, 40), (5, 10_000)])
def test_scan_map_rows(acc, orc, dev, t, shape):
    # rank 2: one CTA per row, one warp per row (many short rows)
    run_scan_map(acc, orc, dev, t, "+", "+", shape, 0, 1)
    run_scan_map(acc, orc, dev, t, "min", "*", shape, 1, 0)


def test_map_rejects_unsupported(acc, dev):
    x = torch.ones(8, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError):
        acc.fold_map("+", "xor", 1, 0, x)       # g outside {+, *, min, max}
    with pytest.raises(acc.AccError):
        acc.scan_map("scanl1", "*", "+", 1, None, x)  # f = (*) not in the fused set
