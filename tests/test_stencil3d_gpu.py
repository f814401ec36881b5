"""Rank-3 weighted-sum stencils on the GPU, bit-exact against the oracle's
rank-3 restatement (planes outer, then rows, then columns; every index
component remapped by the boundary: accelerate-llvm/.../CodeGen/
Stencil.hs:126-253; PTX/Execute.hs:652-748)."""
import numpy as np
import pytest
import torch

from helpers import _diff, case_rng

pytestmark = pytest.mark.gpu

STYPES = {"f32": np.float32, "f64": np.float64, "i32": np.int32, "i64": np.int64}
PATTERNS = [(3, 3, 3), (1, 3, 5), (5, 1, 3), (3, 5, 1), (9, 9, 9), (1, 1, 3)]
SHAPES = [(1, 1, 1), (5, 6, 7), (17, 33, 65), (2, 300, 70), (40, 9, 129)]


def data(dt, shape, rng):
    if np.dtype(dt).kind == "f":
        return rng.random(shape).astype(dt)
    return rng.integers(-1000, 1000, size=shape).astype(dt)


def weights(dt, pattern, rng):
    if np.dtype(dt).kind == "f":
        w = rng.uniform(-1, 1, size=pattern).astype(dt)
    else:
        w = rng.integers(-3, 4, size=pattern).astype(dt)
    w[rng.random(w.shape) < 0.2] = 0
    return w


def check(acc, orc, dev, dt, w, x, b, cval):
    got = acc.stencil3d(w.tolist(), torch.from_numpy(np.ascontiguousarray(x)).to(dev), b, cval=cval).cpu().numpy()
    ref = orc.stencil3d(w, x, b, cval=cval)
    assert np.array_equal(got, ref), f"{x.shape} {w.shape}: {_diff(got, ref)}"


@pytest.mark.parametrize("t", list(STYPES))
@pytest.mark.parametrize("b", [0, 1, 2, 3])
@pytest.mark.parametrize("pattern", PATTERNS)
def test_stencil3d_grid(acc, orc, dev, t, b, pattern):
    dt = STYPES[t]
    rng = case_rng("stencil3d", t, b, pattern)
    for shape in SHAPES:
        check(acc, orc, dev, dt, weights(dt, pattern, rng), data(dt, shape, rng), b, dt(7))


@pytest.mark.parametrize("shape", [(70_000, 1, 3), (1, 600_000, 1)])
def test_stencil3d_grid_loops(acc, orc, dev, shape):
    # more planes than gridDim.z and more rows than gridDim.y * 8 cover
    rng = case_rng("stencil3d_loops", shape)
    x = data(np.float32, shape, rng)
    check(acc, orc, dev, np.float32, weights(np.float32, (3, 3, 3), rng), x, 1, np.float32(0.5))


def test_stencil3d_box_clamp(acc, orc, dev):
    rng = np.random.default_rng(5)
    g = rng.random((64, 96, 128), dtype=np.float32)
    w = np.full((3, 3, 3), 1.0 / 27, dtype=np.float32)
    check(acc, orc, dev, np.float32, w, g, 0, np.float32(0))


def dense_or_star(dt, kind, rng):
    w = weights(dt, (3, 3, 3), rng)
    if kind == "dense":
        w[w == 0] = 1
    else:  # the 7-point star: the centre and its six face neighbours
        star = np.zeros((3, 3, 3), dtype=bool)
        star[1, 1, :] = star[1, :, 1] = star[:, 1, 1] = True
        w[~star] = 0
        w[star & (w == 0)] = 2
    return w


@pytest.mark.parametrize("t", list(STYPES))
@pytest.mark.parametrize("b", [0, 1, 2, 3])
@pytest.mark.parametrize("kind", ["dense", "star"])
def test_stencil3d_streaming_patterns(acc, orc, dev, t, b, kind):
    """The 3x3x3 plane-streaming kernel's compile-time tap patterns, over
    rows that are 16-byte aligned (copied in 16-byte pieces) and rows that
    are not, from an array that starts one element past a 16-byte boundary,
    and plane counts that split into several plane ranges."""
    dt = STYPES[t]
    rng = case_rng("stencil3d_stream", t, b, kind)
    for shape in [(1, 1, 1), (5, 6, 7), (9, 40, 64), (33, 35, 96), (3, 70, 200), (300, 4, 8)]:
        w = dense_or_star(dt, kind, rng)
        x = data(dt, shape, rng)
        check(acc, orc, dev, dt, w, x, b, dt(7))
        # the same array one element into its allocation
        flat = torch.zeros(x.size + 1, dtype=torch.from_numpy(x).dtype, device=dev)
        flat[1:] = torch.from_numpy(x.ravel()).to(dev)
        got = acc.stencil3d(w.tolist(), flat[1:].view(shape), b, cval=dt(7)).cpu().numpy()
        ref = orc.stencil3d(w, x, b, cval=dt(7))
        assert np.array_equal(got, ref), f"offset {shape}: {_diff(got, ref)}"


def test_stencil3d_errors(acc, dev):
    x = torch.zeros((4, 4, 4), dtype=torch.float32, device=dev)
    with pytest.raises(ValueError):
        acc.stencil3d([[[1.0, 1.0]]], x)  # even-sized pattern
    with pytest.raises(ValueError):
        acc.stencil3d([[[1.0]]], x[0])  # rank 2
    w11 = [[[0.0] * 11] * 1] * 1
    with pytest.raises(acc.AccError) as err:
        acc.stencil3d(w11, x)
    assert err.value.status == 1  # radius above 4
    u = torch.zeros((4, 4, 4), dtype=torch.uint32, device=dev)
    with pytest.raises(acc.AccError) as err:
        acc.stencil3d([[[1]]], u)
    assert err.value.status == 2  # Word32 stencils are outside the weighted-sum set
