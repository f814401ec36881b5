"""Serving loop (acc_serve_run): every request of a mixed stream gives the same
result served in the mix as run alone through the per-call API -- bit-exact
for integers, foldSeg, permute and stencil, within the Float32 (+)
tolerance for fold / scan (the mix runs them in batched launches)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

W5 = [[0.0, 0.25, 0.0], [0.25, -1.0, 0.25], [0.0, 0.25, 0.0]]


def make_stream(dev, count=240, rate=50_000.0, seed=1):
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    reqs, refs = [], []
    t = 0.0
    kinds = rng.choice(["fold", "scan", "foldseg", "permute", "stencil"], size=count, p=[0.4, 0.25, 0.15, 0.1, 0.1])
    for i, k in enumerate(kinds):
        t += rng.exponential(1.0 / rate)
        n = int(np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 18))))
        if k in ("fold", "scan"):
            dt = [torch.int32, torch.float32, torch.int64, torch.float64][i % 4]
            xs = (torch.randn(n, dtype=dt, device=dev, generator=g) if dt.is_floating_point
                  else torch.randint(-100, 100, (n,), dtype=dt, device=dev, generator=g))
            out = torch.zeros(1 if k == "fold" else n, dtype=dt, device=dev)
            reqs.append((k, xs, None, out, n, 0, t))
        elif k == "foldseg":
            lens = np.minimum(rng.lognormal(np.log(48), 1.5, size=n // 32 + 1), 1 << 12).astype(np.int64)
            off = np.concatenate([[0], np.cumsum(lens)])
            off = off[off <= n]
            xs = torch.randn(n, dtype=torch.float32, device=dev, generator=g)
            offs = torch.from_numpy(off.astype(np.int32)).to(dev)
            out = torch.zeros(len(off) - 1, dtype=torch.float32, device=dev)
            reqs.append((k, xs, offs, out, n, len(off) - 1, t))
        elif k == "permute":
            m = int(2 ** rng.integers(12, 17))
            idx = torch.randint(0, m, (n,), dtype=torch.int32, device=dev, generator=g)
            out = torch.zeros(m, dtype=torch.int32, device=dev)
            reqs.append((k, idx, None, out, n, m, t))
        else:
            h = int(rng.integers(16, 300))
            w = int(rng.integers(16, 300))
            grid = torch.rand((h, w), dtype=torch.float32, device=dev, generator=g)
            out = torch.zeros((h, w), dtype=torch.float32, device=dev)
            reqs.append((k, grid, None, out, h, w, t))
    return reqs


def alone(acc, req):
    k, xs, aux, out, n, m, t = req
    if k == "fold":
        return acc.fold("+", 0, xs).reshape(1)
    if k == "scan":
        return acc.scanl1("+", xs)
    if k == "foldseg":
        return acc.fold_seg("+", 0.0, xs, aux)
    if k == "permute":
        return acc.permute("+", torch.zeros(m, dtype=torch.int32, device=xs.device), xs, 1)
    return acc.stencil(W5, xs, "clamp")


def same(k, got, ref, xs):
    if k in ("fold", "scan") and got.dtype.is_floating_point:
        g, r = got.double().cpu().numpy(), ref.double().cpu().numpy()
        a = np.abs(xs.double().cpu().numpy())
        ab = np.cumsum(a) if k == "scan" else np.array([a.sum()])
        return np.all(np.abs(g - r) <= 2e-6 * np.abs(r) + 2e-9 * ab + 1e-12)
    return torch.equal(got, ref)


@pytest.mark.parametrize("mode", ["batching", "per_call"])
def test_served_results_equal_alone(acc, dev, mode):
    reqs = make_stream(dev)
    lat, stats = acc.serve(reqs, budget_bytes=1 << 30, slots=8, mode=mode)
    acc.sync()
    assert stats["served"] == len(reqs)
    assert all(x >= 0 for x in lat)
    refs = [alone(acc, r) for r in reqs]
    torch.cuda.synchronize()
    bad = [i for i, (r, ref) in enumerate(zip(reqs, refs)) if not same(r[0], r[3], ref, r[1])]
    assert not bad, f"{len(bad)} requests differ, first {reqs[bad[0]][0]} #{bad[0]}"
    if mode == "batching":
        assert stats["batches"] > 0


def test_admission_budget_is_respected(acc, dev):
    reqs = make_stream(dev, count=120, rate=1e9, seed=3)  # everything arrives at once
    budget = 1 << 22
    reqs = [r for r in reqs if r[0] != "stencil" and r[0] != "foldseg"]
    small = []
    for r in reqs:
        k, xs, aux, out, n, m, t = r
        held = (n * xs.element_size() * (2 if k == "scan" else 1)) + out.numel() * out.element_size()
        if held <= budget:
            small.append(r)
    lat, stats = acc.serve(small, budget_bytes=budget, slots=8, mode="batching")
    assert stats["served"] == len(small)
    assert stats["peak_bytes"] <= budget


def test_request_larger_than_budget_is_rejected(acc, dev):
    xs = torch.zeros(1 << 20, dtype=torch.float32, device=dev)
    out = torch.zeros(1, dtype=torch.float32, device=dev)
    with pytest.raises(acc.AccError) as e:
        acc.serve([("fold", xs, None, out, xs.numel(), 0, 0.0)], budget_bytes=1024)
    assert e.value.status == 8


NP = {torch.int32: np.int32, torch.int64: np.int64, torch.float32: np.float32, torch.float64: np.float64}


@pytest.mark.parametrize("mode", ["batching", "per_call"])
def test_results_in_the_arena_copied_back(acc, dev, mode):
    """Results placed by the loop in its device arena (no output buffer),
    each copied back to a host array, under a budget small enough that
    admission waits for arena room; every copied-back result equals the
    request run alone."""
    reqs = make_stream(dev, count=160, rate=1e6, seed=5)
    placed = []
    for k, xs, aux, out, n, m, t in reqs:
        placed.append((k, xs, aux, None, n, m, t, np.full(out.numel(), 7, dtype=NP[out.dtype])))
    budget = 4 << 20
    lat, stats = acc.serve(placed, budget_bytes=budget, slots=8, mode=mode)
    assert stats["served"] == len(placed)
    assert 0 < stats["peak_bytes"] <= budget
    bad = []
    for i, (r, p) in enumerate(zip(reqs, placed)):
        ref = alone(acc, r)
        got = torch.from_numpy(p[7]).to(dev).view(r[3].shape)
        if not same(r[0], got, ref, r[1]):
            bad.append(i)
    assert not bad, f"{len(bad)} requests differ, first {reqs[bad[0]][0]} #{bad[0]}"
