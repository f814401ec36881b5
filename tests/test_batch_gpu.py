"""Batched persistent launch (acc_batch_*): every request's result against
the oracle -- bit-exact for integers and float min/max (NaN where the oracle
has NaN), within the float (+) tolerance of the FP64 oracle otherwise
(Float32: 1e-6 |ref| + 1e-9 sum|x|; Float64: 1e-12 sum|x| + 1e-15 |ref|) --
for a launch, a captured graph and its replays."""
import json

import numpy as np
import pytest
import torch

from helpers import _diff, case_rng, seed_for

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 255, 256, 1000, 4097, 65_536, 100_003, (1 << 20) + 3]
DT = {"i32": torch.int32, "i64": torch.int64, "f32": torch.float32, "f64": torch.float64}


def make_requests(dev, f, rng):
    reqs = []
    for t, dt in DT.items():
        for n in SIZES:
            for kind in ("fold", "scan"):
                for seeded in (False, True):
                    g = torch.Generator(device=dev)
                    g.manual_seed(int(rng.integers(1 << 30)))
                    if dt.is_floating_point:
                        xs = torch.randn(n, dtype=dt, device=dev, generator=g)
                        if f in ("min", "max") and n > 4:
                            xs[3::97] = float("nan")  # fmin / fmax skip NaN
                    else:
                        xs = torch.randint(-1000, 1000, (n,), dtype=dt, device=dev, generator=g)
                    z = seed_for(np.dtype(str(dt).split(".")[1]), f) if seeded else None
                    out = torch.full((1,) if kind == "fold" else (n,), 123, dtype=dt, device=dev)
                    reqs.append((kind, xs, out, z))
    # fold z [] = z
    e = torch.empty(0, dtype=torch.int32, device=dev)
    reqs.append(("fold", e, torch.zeros(1, dtype=torch.int32, device=dev), 77))
    return reqs


def expected(orc, f, kind, xs, z):
    """The oracle's result of one request: fold z / fold1, or scanl1 with the
    seed (when there is one) on the left of every prefix (scanl z without
    its first element)."""
    x = xs.cpu().numpy()
    zz = None if z is None else x.dtype.type(z)
    if kind == "fold":
        return np.atleast_1d(orc.fold(f, zz, x))
    if z is None:
        return orc.scan(f, None, x, 0, 0)
    return orc.scan(f, zz, x, 0, 1)[1:]


def expected64(orc, f, kind, xs, z):
    """FP64 oracle value and sum|x| per output of a float (+) request."""
    x = xs.cpu().numpy()
    z64 = None if z is None else float(z)
    za = None if z is None else abs(float(z))
    if kind == "fold":
        return np.atleast_1d(orc.fold_f64(f, z64, x)), np.atleast_1d(orc.fold_f64("+", za, np.abs(x)))
    if z is None:
        return orc.scan_f64(f, None, x, 0, 0), orc.scan_f64("+", None, np.abs(x), 0, 0)
    return orc.scan_f64(f, z64, x, 0, 1)[1:], orc.scan_f64("+", za, np.abs(x), 0, 1)[1:]


def check(orc, got, kind, xs, z, f):
    g = got.cpu().numpy()
    if not got.dtype.is_floating_point or f != "+":
        ref = expected(orc, f, kind, xs, z)
        assert g.shape == ref.shape and g.dtype == ref.dtype
        if g.dtype.kind == "f":
            nan = np.isnan(ref)
            assert np.array_equal(np.isnan(g), nan), _diff(g, ref)
            assert np.array_equal(g[~nan], ref[~nan]), _diff(g, ref)
        else:
            assert np.array_equal(g, ref), _diff(g, ref)
        return
    r, ab = expected64(orc, f, kind, xs, z)
    if got.dtype == torch.float32:
        tol = 1e-6 * np.abs(r) + 1e-9 * ab
    else:
        tol = 1e-12 * ab + 1e-15 * np.abs(r)
    err = np.abs(g.astype(np.float64) - r)
    assert g.shape == r.shape and np.all(err <= tol + 1e-30), f"max excess {(err - tol).max()}"


@pytest.mark.parametrize("f", ["+", "min", "max"])
def test_batch_matches_the_oracle(acc, orc, dev, f):
    rng = case_rng("batch", f)
    reqs = make_requests(dev, f, rng)
    b = acc.Batch(f, reqs)
    b.launch()
    b.status()
    torch.cuda.synchronize()
    for kind, xs, out, z in reqs:
        check(orc, out, kind, xs, z, f)
    b.close()


@pytest.mark.parametrize("f", ["+", "max"])
def test_batch_graph_replays(acc, orc, dev, f):
    rng = np.random.default_rng(7)
    reqs = make_requests(dev, f, rng)
    b = acc.Batch(f, reqs)
    b.capture()
    for _ in range(3):
        for _, _, out, _ in reqs:
            out.fill_(55)
        b.launch()
        b.status()
        for kind, xs, out, z in reqs:
            check(orc, out, kind, xs, z, f)
    b.close()


def test_batch_mixed_types_in_any_order(acc, orc, dev):
    # 8-byte requests first, then 4-byte multi-tile folds: every fold tile
    # partial needs its own slot whatever the element size of its neighbours.
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    reqs = []
    for rep in range(6):
        for dt in (torch.float64, torch.int64, torch.float32, torch.int32):
            n = 3000 + 1777 * rep
            if dt.is_floating_point:
                xs = torch.randn(n, dtype=dt, device=dev, generator=g)
            else:
                xs = torch.randint(-100, 100, (n,), dtype=dt, device=dev, generator=g)
            reqs.append(("fold", xs, torch.zeros(1, dtype=dt, device=dev), 0))
    b = acc.Batch("+", reqs)
    for _ in range(2):
        b.launch()
        b.status()
        for kind, xs, out, z in reqs:
            check(orc, out, kind, xs, z, "+")
    b.close()


def test_batch_uses_a_loaded_tuning_table(acc, dev, tmp_path):
    entries = [[k, t, bucket, 2] for k in (0, 1) for t in (0, 1, 3, 4) for bucket in range(8, 23)]
    p = tmp_path / "tune.json"
    p.write_text(json.dumps({"gpu": "test", "threads": 256, "entries": entries}))
    acc.batch_load_tuning(p)
    x = torch.arange(100_000, dtype=torch.int64, device=dev)
    out = torch.empty(100_000, dtype=torch.int64, device=dev)
    s = torch.empty(1, dtype=torch.int64, device=dev)
    b = acc.Batch("+", [("scan", x, out, None), ("fold", x, s, 0)])
    b.launch()
    b.status()
    assert torch.equal(out, torch.cumsum(x, 0))
    assert int(s.item()) == int(x.sum().item())
    b.close()


@pytest.mark.parametrize("nt", [128, 512])
@pytest.mark.parametrize("f", ["+", "max"])
def test_batch_launch_shapes_from_the_table(acc, orc, dev, tmp_path, nt, f):
    """A table whose entries choose 128 or 512 threads per CTA (and tiles of
    the largest and smallest shapes for them): the batch launches with that
    shape and every request matches the oracle."""
    big = 32768 // (nt * 8)  # the largest elements per thread for 8-byte types
    entries = [[k, t, bucket, big if bucket % 2 else 1, nt] for k in (0, 1) for t in (0, 1, 3, 4)
               for bucket in range(0, 40)]
    p = tmp_path / "tune.json"
    p.write_text(json.dumps({"gpu": "test", "entries": entries}))
    acc.batch_load_tuning(p)
    try:
        rng = case_rng("batch_nt", nt, f)
        reqs = make_requests(dev, f, rng)
        b = acc.Batch(f, reqs)
        b.launch()
        b.status()
        torch.cuda.synchronize()
        for kind, xs, out, z in reqs:
            check(orc, out, kind, xs, z, f)
        b.close()
    finally:
        # back to 256 threads for the tests that follow
        reset = [[k, t, bucket, 8, 256] for k in (0, 1) for t in (0, 1, 3, 4) for bucket in range(0, 40)]
        p.write_text(json.dumps({"gpu": "test", "entries": reset}))
        acc.batch_load_tuning(p)


def test_batch_rejects_a_bad_launch_shape_in_the_table(acc, tmp_path):
    p = tmp_path / "tune.json"
    p.write_text(json.dumps({"gpu": "test", "entries": [[0, 0, 10, 4, 300]]}))
    with pytest.raises(acc.AccError):
        acc.batch_load_tuning(p)


def test_batch_rejects_bad_requests(acc, dev):
    e = torch.empty(0, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.Batch("+", [("fold", e, torch.zeros(1, dtype=torch.int32, device=dev), None)])
    assert err.value.status == 3  # fold1 of an empty vector
    x = torch.zeros(10, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.Batch("*", [("fold", x, torch.zeros(1, dtype=torch.int32, device=dev), 1)])
    assert err.value.status == 2  # batches take + / min / max only
