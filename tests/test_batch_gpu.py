"""Batched persistent launch (acc_batch_*): every request's result equals the
per-call entry point's (acc_fold / acc_scan) -- bit-exact for integers and
float min/max, within the Float32 (+) tolerance otherwise -- for a launch, a
captured graph and its replays."""
import json

import numpy as np
import pytest
import torch

from helpers import case_rng, seed_for

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 255, 256, 1000, 4097, 65_536, 100_003, (1 << 20) + 3]
DT = {"i32": torch.int32, "i64": torch.int64, "f32": torch.float32, "f64": torch.float64}


def make_requests(dev, f, rng):
    reqs, refs = [], []
    for t, dt in DT.items():
        for n in SIZES:
            for kind in ("fold", "scan"):
                for seeded in (False, True):
                    g = torch.Generator(device=dev)
                    g.manual_seed(int(rng.integers(1 << 30)))
                    if dt.is_floating_point:
                        xs = torch.randn(n, dtype=dt, device=dev, generator=g)
                    else:
                        xs = torch.randint(-1000, 1000, (n,), dtype=dt, device=dev, generator=g)
                    z = seed_for(np.dtype(str(dt).split(".")[1]), f) if seeded else None
                    out = torch.full((1,) if kind == "fold" else (n,), 123, dtype=dt, device=dev)
                    reqs.append((kind, xs, out, z))
                    refs.append((kind, xs, z))
    # fold z [] = z
    e = torch.empty(0, dtype=torch.int32, device=dev)
    reqs.append(("fold", e, torch.zeros(1, dtype=torch.int32, device=dev), 77))
    refs.append(("fold", e, 77))
    return reqs, refs


def reference(acc, f, kind, xs, z):
    if kind == "fold":
        return (acc.fold(f, z, xs) if z is not None else acc.fold1(f, xs)).reshape(1)
    if z is None:
        return acc.scanl1(f, xs)
    return acc.scanl(f, z, xs)[1:]  # scanl1 with the seed on the left of every prefix


def check(got, ref, xs, f):
    if not got.dtype.is_floating_point or f != "+":
        assert torch.equal(got, ref) or (torch.isnan(got) == torch.isnan(ref)).all()
        return
    g, r = got.double().cpu().numpy(), ref.double().cpu().numpy()
    ab = np.cumsum(np.abs(xs.double().cpu().numpy())) if got.numel() > 1 else np.array([np.abs(xs.double().cpu().numpy()).sum()])
    tol = 2e-6 * np.abs(r) + 2e-9 * ab[-len(r):] + (1e-12 if got.dtype == torch.float64 else 0)
    assert np.all(np.abs(g - r) <= tol + 1e-30)


@pytest.mark.parametrize("f", ["+", "min", "max"])
def test_batch_matches_per_call(acc, dev, f):
    rng = case_rng("batch", f)
    reqs, refs = make_requests(dev, f, rng)
    b = acc.Batch(f, reqs)
    b.launch()
    b.status()
    expect = [reference(acc, f, k, xs, z) for (k, xs, z) in refs]
    torch.cuda.synchronize()
    for (kind, xs, out, z), ref in zip(reqs, expect):
        check(out, ref, xs, f)
    b.close()


def test_batch_graph_replays(acc, dev):
    rng = np.random.default_rng(7)
    reqs, refs = make_requests(dev, "+", rng)
    b = acc.Batch("+", reqs)
    b.capture()
    expect = [reference(acc, "+", k, xs, z) for (k, xs, z) in refs]
    for _ in range(3):
        for _, _, out, _ in reqs:
            out.fill_(55)
        b.launch()
        b.status()
        for (kind, xs, out, z), ref in zip(reqs, expect):
            check(out, ref, xs, "+")
    b.close()


def test_batch_mixed_types_in_any_order(acc, dev):
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
            check(out, acc.fold("+", 0, xs).reshape(1), xs, "+")
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


def test_batch_rejects_bad_requests(acc, dev):
    e = torch.empty(0, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.Batch("+", [("fold", e, torch.zeros(1, dtype=torch.int32, device=dev), None)])
    assert err.value.status == 3  # fold1 of an empty vector
    x = torch.zeros(10, dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.Batch("*", [("fold", x, torch.zeros(1, dtype=torch.int32, device=dev), 1)])
    assert err.value.status == 2  # batches take + / min / max only
