"""fold / fold1 on the GPU against the oracle (PTX/Execute.hs:222-340)."""
import numpy as np
import pytest
import torch

from helpers import COMBOS, TYPES, assert_fold_close, case_rng, gen, seed_for

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (1, 5), (1, 17), (3, 100), (1, 100_003), (4096, 1024), (5000, 64), (70_000, 3),
          (2, 3_000_001), (1, 1 << 22), (7, 70_001)]


def run_fold(acc, orc, dev, t, op, shape, seeded, prec=None, offset=0):
    dt = TYPES[t]
    rng = case_rng("fold", t, op, shape, seeded, offset)
    n = int(np.prod(shape))
    x = gen(dt, op, n + offset, rng)
    xs = x[offset:].reshape(shape)
    z = seed_for(dt, op) if seeded else None
    td = torch.from_numpy(x).to(dev)[offset:].view(shape)
    got = (acc.fold(op, z, td, prec=prec) if seeded else acc.fold1(op, td, prec=prec)).cpu().numpy()
    ref = orc.fold(op, dt(z) if seeded else None, xs)
    ref64 = absum = None
    if np.dtype(dt).kind == "f" and op in ("+", "*"):
        ref64 = orc.fold_f64(op, float(z) if seeded else None, xs)
        absum = orc.fold_f64("+", abs(float(z)) if seeded else None, np.abs(xs))
    assert_fold_close(got, ref, ref64, absum, dt, op, prec)


@pytest.mark.parametrize("t,op", COMBOS)
@pytest.mark.parametrize("shape", SHAPES[:8])
def test_fold_grid(acc, orc, dev, t, op, shape):
    run_fold(acc, orc, dev, t, op, shape, seeded=True)


@pytest.mark.parametrize("t,op", COMBOS)
def test_fold1_grid(acc, orc, dev, t, op):
    for shape in [(1, 1), (1, 1000), (3000, 33), (1, 1_000_001)]:
        run_fold(acc, orc, dev, t, op, shape, seeded=False)


@pytest.mark.parametrize("t,op", [("i32", "+"), ("f32", "+"), ("i64", "xor"), ("f64", "max"), ("u32", "*")])
@pytest.mark.parametrize("shape", SHAPES[8:])
def test_fold_large(acc, orc, dev, t, op, shape):
    run_fold(acc, orc, dev, t, op, shape, seeded=True)


@pytest.mark.parametrize("offset", [1, 2, 3])
@pytest.mark.parametrize("t,op", [("i32", "+"), ("f32", "+"), ("i64", "min"), ("f64", "+")])
def test_fold_unaligned(acc, orc, dev, t, op, offset):
    for shape in [(1, 100_000), (1000, 37)]:
        run_fold(acc, orc, dev, t, op, shape, seeded=True, offset=offset)


@pytest.mark.parametrize("prec", ["plain", "compensated", "fp64"])
def test_fold_f32_precisions(acc, orc, dev, prec):
    for shape in [(1, 1 << 20), (64, 4096)]:
        run_fold(acc, orc, dev, "f32", "+", shape, seeded=True, prec=prec)


def test_fold_known_answer(acc, dev):
    # sum (map (+1) [1..10000]) == 50015000 (accelerate-llvm-ptx/test/nofib/.../RunQ.hs:26-31)
    xs = torch.arange(1, 10001, dtype=torch.int64, device=dev) + 1
    assert int(acc.fold("+", 0, xs).item()) == 50015000


def test_fold_empty(acc, dev):
    out = acc.fold("+", 42, torch.empty((5, 0), dtype=torch.int32, device=dev))
    assert out.cpu().tolist() == [42] * 5
    with pytest.raises(acc.AccError) as e:
        acc.fold1("+", torch.empty((5, 0), dtype=torch.int32, device=dev))
    assert e.value.status == 3
    assert acc.fold("+", 1, torch.empty((0, 9), dtype=torch.int32, device=dev)).numel() == 0


def test_fold_repeatable(acc, dev):
    x = torch.randn(1 << 22, device=dev)
    a = acc.fold("+", 0.0, x)
    b = acc.fold("+", 0.0, x)
    assert torch.equal(a, b)
