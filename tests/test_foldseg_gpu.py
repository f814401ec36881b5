"""foldSeg / fold1Seg on the GPU against the oracle (PTX/Execute.hs:343-374;
Native/CodeGen/FoldSeg.hs:103-141)."""
import numpy as np
import pytest
import torch

from helpers import COMBOS, TYPES, _diff, assert_fold_close, case_rng, gen, seed_for

pytestmark = pytest.mark.gpu


def segmentation(rng, nseg, long_frac=0.01, zero_frac=0.05, maxlen=20_000):
    lens = np.minimum(rng.lognormal(np.log(20.0), 1.5, size=nseg), maxlen).astype(np.int64)
    lens[rng.random(nseg) < zero_frac] = 0
    k = rng.random(nseg) < long_frac
    lens[k] = rng.integers(2049, 9000, size=int(k.sum()))
    return lens


def run_seg(acc, orc, dev, t, op, nseg, seeded, outer=1, off_t=np.int32, prec=None, lengths_api=False):
    dt = TYPES[t]
    rng = case_rng("foldseg", t, op, nseg, seeded, outer, str(off_t), lengths_api)
    lens = segmentation(rng, nseg)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(off_t)
    inner = int(off[-1])
    x = gen(dt, op, outer * inner, rng).reshape((outer, inner) if outer > 1 else (inner,))
    z = seed_for(dt, op) if seeded else None
    seg_arg = torch.from_numpy(lens.astype(off_t) if lengths_api else off).to(dev)
    td = torch.from_numpy(x).to(dev)
    if seeded:
        got = acc.fold_seg(op, z, td, seg_arg, prec=prec, offsets=not lengths_api)
    else:
        got = acc.fold1_seg(op, td, seg_arg, prec=prec, offsets=not lengths_api)
    acc.sync()
    got = got.cpu().numpy()
    ref = orc.fold_seg(op, dt(z) if seeded else None, x, off)
    mask = np.broadcast_to(lens > 0, ref.shape) if not seeded else np.ones(ref.shape, bool)
    ref64 = absum = None
    if np.dtype(dt).kind == "f" and op in ("+", "*"):
        ref64 = orc.fold_seg_f64(op, float(z) if seeded else None, x, off)[mask]
        absum = orc.fold_seg_f64("+", abs(float(z)) if seeded else None, np.abs(x), off)[mask]
    assert_fold_close(got[mask], ref[mask], ref64, absum, dt, op, prec)


@pytest.mark.parametrize("t,op", COMBOS)
@pytest.mark.parametrize("seeded", [True, False])
def test_foldseg_grid(acc, orc, dev, t, op, seeded):
    run_seg(acc, orc, dev, t, op, 3000, seeded)


@pytest.mark.parametrize("t,op", [("i32", "max"), ("f32", "+"), ("i64", "+"), ("f64", "min")])
@pytest.mark.parametrize("nseg", [1, 2, 31, 33, 1000, 100_000])
def test_foldseg_sizes(acc, orc, dev, t, op, nseg):
    run_seg(acc, orc, dev, t, op, nseg, True)


@pytest.mark.parametrize("t,op", [("i32", "+"), ("f32", "+")])
def test_foldseg_rows_and_offset_types(acc, orc, dev, t, op):
    run_seg(acc, orc, dev, t, op, 500, True, outer=3)
    run_seg(acc, orc, dev, t, op, 500, True, off_t=np.int64)
    run_seg(acc, orc, dev, t, op, 500, False, outer=2, off_t=np.int64)


@pytest.mark.parametrize("off_t", [np.int32, np.int64])
def test_foldseg_lengths_api(acc, orc, dev, off_t):
    run_seg(acc, orc, dev, "i32", "+", 5000, True, off_t=off_t, lengths_api=True)
    run_seg(acc, orc, dev, "f32", "+", 5000, True, off_t=off_t, lengths_api=True)


@pytest.mark.parametrize("prec", ["plain", "compensated", "fp64"])
def test_foldseg_f32_precisions(acc, orc, dev, prec):
    run_seg(acc, orc, dev, "f32", "+", 20_000, True, prec=prec)


def test_foldseg_empty_segments(acc, dev):
    xs = torch.arange(10, dtype=torch.int32, device=dev)
    off = torch.tensor([0, 3, 3, 10], dtype=torch.int32, device=dev)
    assert acc.fold_seg("+", 100, xs, off).cpu().tolist() == [103, 100, 142]


def test_foldseg_bad_offsets_raise(acc, dev):
    xs = torch.arange(10, dtype=torch.int32, device=dev)
    off = torch.tensor([0, 5, 11], dtype=torch.int32, device=dev)
    acc.fold_seg("+", 0, xs, off)
    with pytest.raises(acc.AccError) as e:
        acc.sync()
    assert e.value.status == 7
    acc.sync()  # the error word was cleared


def test_per_segment_kernels_on_vectors():
    """The per-segment kernels (selected for 1-D rows by
    ACC_GB300_FOLDSEG=segments, read once per process) give the same results:
    the grid, size, precision and edge-case tests again in a child process."""
    import os
    import pathlib
    import subprocess
    import sys
    env = dict(os.environ, ACC_GB300_FOLDSEG="segments")
    here = pathlib.Path(__file__).resolve()
    r = subprocess.run([sys.executable, "-m", "pytest", str(here), "-q", "-m", "gpu", "-p", "no:cacheprovider",
                        "-k", "not per_segment_kernels"], cwd=here.parent.parent, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-2000:]
