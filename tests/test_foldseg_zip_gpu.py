"""foldSeg f z (zipWith g xs ys) with the zipWith fused into the per-segment
kernels (the reference's delayed foldSeg input, PTX/CodeGen/FoldSeg.hs:56-458)
against the oracle: the zipped array is formed in the element type, then
folded per segment by the oracle; comparison rules as for acc_fold_seg."""
import numpy as np
import pytest
import torch

from helpers import TYPES, assert_fold_close, case_rng, gen, seed_for
from test_fold_zip_gpu import zipped
from test_foldseg_gpu import segmentation

pytestmark = pytest.mark.gpu

ZTYPES = ["i32", "i64", "f32", "f64"]
FOLD_OPS = ["+", "min", "max"]
ZIP_OPS = ["+", "*", "min", "max"]


def run_seg_zip(acc, orc, dev, t, f, g, nseg, seeded, outer=1, off_t=np.int32, offset=0):
    dt = TYPES[t]
    rng = case_rng("foldseg_zip", t, f, g, nseg, seeded, outer, str(off_t), offset)
    lens = segmentation(rng, nseg)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(off_t)
    inner = int(off[-1])
    shape = (outer, inner) if outer > 1 else (inner,)
    src = g if g == "*" else f
    x = gen(dt, src, outer * inner, rng).reshape(shape)
    y = gen(dt, src, outer * inner + offset, rng)
    ys = y[offset:].reshape(shape)
    with np.errstate(over="ignore", invalid="ignore"):
        zs = zipped(g, x, ys)
    z = seed_for(dt, f) if seeded else None
    ty = torch.from_numpy(y).to(dev)[offset:].view(shape)  # offset: a different 16-byte phase
    got = acc.fold_seg_zipwith(f, g, z, torch.from_numpy(x).to(dev), ty, torch.from_numpy(off).to(dev))
    acc.sync()
    got = got.cpu().numpy()
    ref = orc.fold_seg(f, dt(z) if seeded else None, zs, off)
    mask = np.broadcast_to(lens > 0, ref.shape) if not seeded else np.ones(ref.shape, bool)
    ref64 = absum = None
    if np.dtype(dt).kind == "f" and f == "+":
        ref64 = orc.fold_seg_f64(f, float(z) if seeded else None, zs, off)[mask]
        absum = orc.fold_seg_f64("+", abs(float(z)) if seeded else None, np.abs(zs), off)[mask]
    assert_fold_close(got[mask], ref[mask], ref64, absum, dt, f, None)


@pytest.mark.parametrize("t", ZTYPES)
@pytest.mark.parametrize("f", FOLD_OPS)
@pytest.mark.parametrize("g", ZIP_OPS)
def test_foldseg_zipwith_grid(acc, orc, dev, t, f, g):
    run_seg_zip(acc, orc, dev, t, f, g, 3000, True)
    run_seg_zip(acc, orc, dev, t, f, g, 700, False)


@pytest.mark.parametrize("t", ZTYPES)
def test_foldseg_zipwith_rows_offsets_phase(acc, orc, dev, t):
    run_seg_zip(acc, orc, dev, t, "+", "*", 500, True, outer=3)
    run_seg_zip(acc, orc, dev, t, "+", "*", 500, True, off_t=np.int64)
    run_seg_zip(acc, orc, dev, t, "+", "*", 2000, True, offset=1)


def test_foldseg_zipwith_errors(acc, dev):
    u = torch.zeros(10, dtype=torch.int32, device=dev)
    off = torch.tensor([0, 4, 10], dtype=torch.int32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.fold_seg_zipwith("*", "+", 1, u, u, off)
    assert err.value.status == 2  # fold op outside {+, min, max}
    with pytest.raises(ValueError):
        acc.fold_seg_zipwith("+", "*", 0, u, u[:5], off)
