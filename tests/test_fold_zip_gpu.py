"""fold f z (zipWith g xs ys) with the zipWith fused into the fold kernels
(the reference's delayed fold input, PTX/CodeGen/Fold.hs:80-97) against the
oracle: the zipped array is formed in the element type (integers wrap, floats
round once per element, float min / max are IEEE fmin / fmax), then folded by
the oracle's fold; comparison rules as for acc_fold (tests/helpers.py)."""
import numpy as np
import pytest
import torch

from helpers import TYPES, assert_fold_close, case_rng, gen, seed_for

pytestmark = pytest.mark.gpu

ZTYPES = ["i32", "i64", "f32", "f64"]
FOLD_OPS = ["+", "min", "max"]
ZIP_OPS = ["+", "*", "min", "max"]
SHAPES = [(1, 1), (5, 17), (3000, 33), (1, 100_003), (2, 1_000_001)]


def zipped(g, x, y):
    if g == "+":
        return x + y
    if g == "*":
        return x * y
    if np.dtype(x.dtype).kind == "f":
        return np.fmin(x, y) if g == "min" else np.fmax(x, y)
    return np.minimum(x, y) if g == "min" else np.maximum(x, y)


def inputs(dt, f, g, n, rng):
    # Values for the zip: near 1 for *, otherwise as the fold op likes them.
    x = gen(dt, g if g == "*" else f, n, rng)
    y = gen(dt, g if g == "*" else f, n, rng)
    return x, y


def run_zip(acc, orc, dev, t, f, g, shape, seeded, offset=0, prec=None):
    dt = TYPES[t]
    rng = case_rng("fold_zip", t, f, g, shape, seeded, offset)
    n = int(np.prod(shape))
    x, y = inputs(dt, f, g, n + offset, rng)
    xs, ys = x[:n].reshape(shape), y[offset:].reshape(shape)
    with np.errstate(over="ignore", invalid="ignore"):
        zs = zipped(g, xs, ys)
    z = seed_for(dt, f) if seeded else None
    tx = torch.from_numpy(x).to(dev)[:n].view(shape)
    ty = torch.from_numpy(y).to(dev)[offset:].view(shape)  # offset: a different 16-byte phase
    got = acc.fold_zipwith(f, g, z, tx, ty, prec=prec).cpu().numpy()
    ref = orc.fold(f, dt(z) if seeded else None, zs)
    ref64 = absum = None
    if np.dtype(dt).kind == "f" and f == "+":
        ref64 = orc.fold_f64(f, float(z) if seeded else None, zs)
        absum = orc.fold_f64("+", abs(float(z)) if seeded else None, np.abs(zs))
    assert_fold_close(got, ref, ref64, absum, dt, f, prec)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("f", FOLD_OPS)
@pytest.mark.parametrize("g", ZIP_OPS)
def test_fold_zipwith_grid(acc, orc, dev, t, f, g):
    for shape in SHAPES:
        run_zip(acc, orc, dev, t, f, g, shape, seeded=True)
    run_zip(acc, orc, dev, t, f, g, (7, 50_001), seeded=False)


@pytest.mark.parametrize("t", ZTYPES)
def test_fold_zipwith_unaligned_second_input(acc, orc, dev, t):
    # ys starts one element past a 16-byte boundary: the scalar stride path.
    for shape in [(1, 100_003), (3000, 33), (2, 1_000_001)]:
        run_zip(acc, orc, dev, t, "+", "*", shape, seeded=True, offset=1)


@pytest.mark.parametrize("prec", ["plain", "compensated", "fp64"])
def test_dotp_float32_precisions(acc, orc, dev, prec):
    run_zip(acc, orc, dev, "f32", "+", "*", (1, 3_000_001), seeded=True, prec=prec)


def test_dotp_known_answer(acc, dev):
    xs = torch.arange(1, 10001, dtype=torch.int64, device=dev)
    assert int(acc.dotp(xs, torch.ones_like(xs)).item()) == 50005000
    assert int(acc.dotp(xs, xs).item()) == sum(i * i for i in range(1, 10001))


def test_fold_zipwith_empty_and_errors(acc, dev):
    e = torch.empty((3, 0), dtype=torch.float32, device=dev)
    assert acc.fold_zipwith("+", "*", 2.5, e, e).cpu().tolist() == [2.5, 2.5, 2.5]
    with pytest.raises(acc.AccError) as err:
        acc.fold_zipwith("+", "*", None, e, e)
    assert err.value.status == 3  # fold1 of an empty row
    u = torch.zeros(10, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.fold_zipwith("*", "+", 1, u, u)
    assert err.value.status == 2  # fold op outside {+, min, max}
    with pytest.raises(ValueError):
        acc.fold_zipwith("+", "*", 0, u, u[:5])
