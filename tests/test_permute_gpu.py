"""permute with the fixed primitives on the GPU against the oracle
(PTX/Execute.hs:597-649; Native/CodeGen/Permute.hs:85-118)."""
import numpy as np
import pytest
import torch

from helpers import COMBOS, TYPES, _diff, case_rng, gen

pytestmark = pytest.mark.gpu


def zipf_bins(rng, n, m, s=1.1):
    p = 1.0 / np.arange(1, m + 1) ** s
    cdf = np.cumsum(p / p.sum())
    rank = np.minimum(np.searchsorted(cdf, rng.random(n)), m - 1)
    return rng.permutation(m).astype(np.int32)[rank]


def run_perm(acc, orc, dev, t, op, n, m, const=False, idx_t=np.int32, drop=True):
    dt = TYPES[t]
    rng = case_rng("permute", t, op, n, m, const, str(idx_t))
    idx = rng.integers(-3 if drop else 0, m, size=n).astype(idx_t)
    xs = None if const else gen(dt, op, n, rng)
    defaults = gen(dt, op, m, rng)
    c = 3 if const else None
    got = acc.permute(op, torch.from_numpy(defaults).to(dev), torch.from_numpy(idx).to(dev),
                      c if const else torch.from_numpy(xs).to(dev))
    acc.sync()
    got = got.cpu().numpy()
    ref = orc.permute(op, defaults, idx, xs, cval=c)
    if np.dtype(dt).kind in "iu" or op in ("min", "max", "*"):
        same = (got == ref) | (np.isnan(got.astype(np.float64)) & np.isnan(ref.astype(np.float64)))
        assert same.all(), _diff(got, ref)
    else:
        # float + / *: order-dependent; compare with FP64 accumulation per bin
        keep = idx >= 0
        src = np.full(n, float(c)) if const else xs.astype(np.float64)
        r64 = defaults.astype(np.float64)
        if op == "+":
            np.add.at(r64, idx[keep], src[keep])
            ab = np.abs(defaults.astype(np.float64))
            np.add.at(ab, idx[keep], np.abs(src[keep]))
            eps = np.finfo(dt).eps
            cnt = np.bincount(idx[keep], minlength=m) + 1
            assert np.all(np.abs(got - r64) <= cnt * eps * ab + 1e-30)
        else:
            np.multiply.at(r64, idx[keep], src[keep])
            assert np.allclose(got, r64, rtol=1e-4 if dt == np.float32 else 1e-12)


@pytest.mark.parametrize("t,op", COMBOS)
@pytest.mark.parametrize("m", [1, 100, 4096, 65536])
def test_permute_grid(acc, orc, dev, t, op, m):
    run_perm(acc, orc, dev, t, op, 200_000, m)


@pytest.mark.parametrize("t,op", [("i32", "+"), ("u32", "+"), ("i32", "max"), ("u32", "or"), ("i32", "xor")])
@pytest.mark.parametrize("m", [16, 4096, 50_000, 65536, 100_000, 300_000, 1 << 20])
def test_permute_histogram_paths(acc, orc, dev, t, op, m):
    run_perm(acc, orc, dev, t, op, 1 << 21, m, const=True)


def test_permute_zipf_histogram(acc, orc, dev):
    rng = np.random.default_rng(11)
    idx = zipf_bins(rng, 1 << 22, 1 << 16)
    got = acc.permute("+", torch.zeros(1 << 16, dtype=torch.int32, device=dev), torch.from_numpy(idx).to(dev), 1)
    ref = orc.permute("+", np.zeros(1 << 16, np.int32), idx, cval=1)
    assert np.array_equal(got.cpu().numpy(), ref)
    assert int(got.sum()) == 1 << 22


def test_permute_int64_index_and_source(acc, orc, dev):
    run_perm(acc, orc, dev, "i64", "+", 100_000, 1000, idx_t=np.int64)
    run_perm(acc, orc, dev, "f32", "max", 100_000, 1000, idx_t=np.int64)


def test_permute_out_of_range_raises(acc, dev):
    idx = torch.tensor([0, 1, 5], dtype=torch.int32, device=dev)
    out = acc.permute("+", torch.zeros(4, dtype=torch.int32, device=dev), idx, 1)
    with pytest.raises(acc.AccError) as e:
        acc.sync()
    assert e.value.status == 7
    assert out.cpu().tolist() == [1, 1, 0, 0]
    acc.sync()


def test_permute_empty(acc, dev):
    out = acc.permute("+", torch.arange(5, dtype=torch.int32, device=dev), torch.empty(0, dtype=torch.int32, device=dev), 1)
    assert out.cpu().tolist() == [0, 1, 2, 3, 4]


@pytest.mark.parametrize("c", [1, 7, 2047])
@pytest.mark.parametrize("m,pair", [(1 << 16, (2, 3)), (1 << 16, (5, 5 + (1 << 15))), (65535, (9, 9 + 32768))])
def test_permute_histogram_counter_wrap(acc, orc, dev, c, m, pair):
    # Two hot bins take most of 2^25 updates, so the per-CTA 16-bit counters
    # wrap many times: neighbouring bins (different packed words), and the two
    # bins of one packed word (bin w and bin w + ceil(m / 2)), whose low
    # counter's carries run into the high one concurrently with its own
    # updates; an odd bin count leaves the last word's high half unused.
    rng = np.random.default_rng(c)
    n = 1 << 25
    idx = rng.integers(0, m, size=n).astype(np.int32)
    hot = rng.random(n) < 0.9
    idx[hot] = np.array(pair, dtype=np.int32)[rng.integers(0, 2, size=int(hot.sum()))]
    got = acc.permute("+", torch.zeros(m, dtype=torch.int32, device=dev), torch.from_numpy(idx).to(dev), c)
    acc.sync()
    ref = (np.bincount(idx, minlength=m).astype(np.int64) * c).astype(np.uint32).view(np.int32)
    assert np.array_equal(got.cpu().numpy(), ref)
