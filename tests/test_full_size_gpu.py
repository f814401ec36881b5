"""Parity at the full sizes of the benchmark workloads, each result checked
against the oracle (the C restatement of accelerate-llvm-native):

  * fold (+) 0 along the rows of an Int32 Z:.4096:.1024 array in [-1024, 1024],
    and scanl1 (+) of the same data flattened (2^22): bit-exact;
  * scanl1 (+) Int64, 2^28 elements in [-2^20, 2^20]: bit-exact (also scanr1,
    and scanl1 of a view that starts 8 bytes past an alignment boundary, which
    takes the plain-load look-back kernel);
  * fold (+) 0 Float32, 2^28 elements ~ N(0,1): the compensated result within
    1e-6 relative of the FP64 oracle; the plain and FP64-accumulated results'
    errors are stated;
  * permute (+) histogram of 2^28 Int32 Zipf(1.1) bin indices into 2^16 bins:
    bit-exact;
  * 3x3 Float32 stencil (weights 1/9) on 8192 x 8192 ~ U(0,1), clamp: bit-exact;
  * foldSeg (+) 0 over 2^26 Float32 ~ N(0,1) in 2^20 lognormal segments
    (median 48, sigma 1.5, capped at 2^16, 2 % empty, lengths rescaled to sum
    to 2^26): compensated and FP64-accumulated within 1e-6 |ref| + 1e-9 sum|x|
    per segment, plain within 1e-4 sum|x|, errors stated; and foldSeg max
    minBound over Int32 values on the same segmentation: bit-exact.

The reference ops these replace: accelerate-llvm-ptx/src/Data/Array/
Accelerate/LLVM/PTX/Execute.hs:222-776.  Inputs are seeded and generated on
the device; the oracle runs on all host cores where the result does not
depend on the evaluation order (integer work, stencil outputs, the FP64
reference sums)."""
import os

import numpy as np
import pytest
import torch

from helpers import _diff

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

CORES = os.cpu_count() or 1
SEED = 0xACCE1


def _gen(dev, k):
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + k)
    return g


def _free():
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def _report(record_property, name, value):
    record_property(name, value)
    print(f"{name}: {value}")


def test_c1_fold_rows_and_flat_scan_int32(acc, orc, dev):
    g = _gen(dev, 0)
    x = torch.randint(-1024, 1025, (4096, 1024), dtype=torch.int32, device=dev, generator=g)
    xs = x.cpu().numpy()
    got = acc.fold("+", 0, x).cpu().numpy()
    ref = orc.fold("+", 0, xs)
    assert got.shape == (4096,)
    assert np.array_equal(got, ref), _diff(got, ref)
    got = acc.scanl1("+", x.reshape(-1)).cpu().numpy()
    ref = orc.scan("+", None, xs.reshape(-1), 0, 0, nthreads=CORES)
    assert np.array_equal(got, ref), _diff(got, ref)
    _free()


@pytest.mark.parametrize("flavour", ["scanl1", "scanr1", "scanl1_unaligned"])
def test_c2a_scan_int64_2e28(acc, orc, dev, flavour):
    n = 1 << 28
    off = 1 if flavour == "scanl1_unaligned" else 0
    g = _gen(dev, 1)
    x = torch.randint(-(1 << 20), (1 << 20) + 1, (n + off,), dtype=torch.int64, device=dev, generator=g)[off:]
    if off:
        assert x.data_ptr() % 16 == 8
    got_t = acc.scanr1("+", x) if flavour == "scanr1" else acc.scanl1("+", x)
    acc.sync()
    got = got_t.cpu().numpy()
    del got_t
    xs = x.cpu().numpy()
    del x
    _free()
    ref = orc.scan("+", None, xs, 1 if flavour == "scanr1" else 0, 0, nthreads=CORES)
    assert np.array_equal(got, ref), _diff(got, ref)


def test_c2b_fold_float32_2e28(acc, orc, dev, record_property):
    n = 1 << 28
    x = torch.randn(n, dtype=torch.float32, device=dev, generator=_gen(dev, 2))
    got = {p: float(acc.fold("+", 0.0, x, prec=p).item()) for p in ("compensated", "plain", "fp64")}
    xs = x.cpu().numpy()
    del x
    _free()
    ref = float(orc.fold_f64("+", 0.0, xs))
    abs_sum = float(orc.fold_f64("+", 0.0, np.abs(xs)))
    for p, v in got.items():
        _report(record_property, f"fold_f32_2e28_{p}_rel_err", abs(v - ref) / abs(ref))
    # the workload's stated bound: Float32 sums within 1e-6 relative of FP64
    assert abs(got["compensated"] - ref) <= 1e-6 * abs(ref)
    assert abs(got["fp64"] - ref) <= 1e-6 * abs(ref)
    assert abs(got["plain"] - ref) <= 1e-4 * abs_sum


def _zipf_bins(dev, n, m, s, g):
    """n bin indices in [0, m): ranks ~ Zipf(s) by inverse CDF, rank -> bin
    through a seeded permutation (the hottest rank is not bin 0)."""
    ranks = torch.arange(1, m + 1, dtype=torch.float64, device=dev)
    p = ranks.pow(-s)
    cdf = torch.cumsum(p / p.sum(), 0)
    perm = torch.randperm(m, device=dev, generator=g).to(torch.int32)
    idx = torch.empty(n, dtype=torch.int32, device=dev)
    chunk = 1 << 26
    for st in range(0, n, chunk):
        u = torch.rand(min(chunk, n - st), dtype=torch.float64, device=dev, generator=g)
        r = torch.searchsorted(cdf, u).clamp_(max=m - 1)
        idx[st:st + u.numel()] = perm[r]
    return idx


def test_c2c_permute_histogram_2e28(acc, orc, dev):
    n, m = 1 << 28, 1 << 16
    idx = _zipf_bins(dev, n, m, 1.1, _gen(dev, 3))
    zeros = torch.zeros(m, dtype=torch.int32, device=dev)
    got = acc.permute("+", zeros, idx, 1).cpu().numpy()
    acc.sync()
    ids = idx.cpu().numpy()
    del idx
    _free()
    ref = orc.permute("+", np.zeros(m, np.int32), ids, cval=1, nthreads=CORES)
    assert np.array_equal(got, ref), _diff(got, ref)
    assert int(got.sum()) == n
    # Zipf(1.1): the hottest bin takes about a tenth of all indices
    assert got.max() > n // 20


def test_c2d_stencil_3x3_8192sq_clamp(acc, orc, dev):
    grid = torch.rand((8192, 8192), dtype=torch.float32, device=dev, generator=_gen(dev, 4))
    w = [[1.0 / 9] * 3] * 3
    got = acc.stencil(w, grid, "clamp").cpu().numpy()
    gs = grid.cpu().numpy()
    del grid
    _free()
    ref = orc.stencil2d(w, gs, 0, nthreads=CORES)
    assert np.array_equal(got, ref), _diff(got, ref)


def lognormal_offsets(dev, n_values, nseg, g):
    """Lognormal(median 48, sigma 1.5) lengths capped at 2^16, 2 % forced
    empty, rescaled by largest remainder so that they sum to n_values;
    Int32 offsets (nseg + 1)."""
    lens = torch.empty(nseg, dtype=torch.float64, device=dev).log_normal_(float(np.log(48.0)), 1.5, generator=g)
    lens.clamp_(max=float(1 << 16))
    lens[torch.rand(nseg, device=dev, generator=g) < 0.02] = 0.0
    lens *= n_values / lens.sum()
    fl = torch.floor(lens)
    rem = int(n_values - int(fl.sum().item()))
    order = torch.argsort(lens - fl, descending=True)
    fl[order[:rem]] += 1.0
    off = torch.zeros(nseg + 1, dtype=torch.int64, device=dev)
    off[1:] = torch.cumsum(fl.to(torch.int64), 0)
    return off.to(torch.int32)


def test_c3_foldseg_lognormal(acc, orc, dev, record_property):
    n, nseg = 1 << 26, 1 << 20
    g = _gen(dev, 5)
    off = lognormal_offsets(dev, n, nseg, g)
    vals = torch.randn(n, dtype=torch.float32, device=dev, generator=g)
    ivals = torch.randint(-(1 << 31), (1 << 31) - 1, (n,), dtype=torch.int32, device=dev, generator=g)
    got = {p: acc.fold_seg("+", 0.0, vals, off, prec=p).double().cpu().numpy()
           for p in ("compensated", "plain", "fp64")}
    got_max = acc.fold_seg("max", -(1 << 31), ivals, off).cpu().numpy()
    acc.sync()
    offs, vs, ivs = off.cpu().numpy(), vals.cpu().numpy(), ivals.cpu().numpy()
    del off, vals, ivals
    _free()
    lens = np.diff(offs.astype(np.int64))
    assert offs[-1] == n and (lens == 0).mean() > 0.01 and lens.max() <= 1 << 16
    ref = orc.fold_seg_f64("+", 0.0, vs, offs)
    abs_sum = orc.fold_seg_f64("+", 0.0, np.abs(vs), offs)
    for p, v in got.items():
        err = np.abs(v - ref)
        rel = err / np.maximum(abs_sum, 1e-30)
        _report(record_property, f"foldseg_f32_{p}_max_err_over_seg_sum_abs", float(rel.max()))
        tol = 1e-4 * abs_sum if p == "plain" else 1e-6 * np.abs(ref) + 1e-9 * abs_sum
        assert np.all(err <= tol + 1e-30), f"{p}: max excess {(err - tol).max()}"
    # empty segments give the seed
    assert np.all(got["compensated"][lens == 0] == 0.0)
    ref_max = orc.fold_seg("max", np.int32(-(1 << 31)), ivs, offs, nthreads=CORES)
    assert np.array_equal(got_max, ref_max), _diff(got_max, ref_max)
