"""Weighted-sum stencils with clamp / mirror / wrap / constant boundaries on the
GPU, bit-exact against the oracle (PTX/Execute.hs:652-776;
accelerate-llvm/.../CodeGen/Stencil.hs:73-253)."""
import numpy as np
import pytest
import torch

from helpers import _diff, case_rng

pytestmark = pytest.mark.gpu

STYPES = {"f32": np.float32, "f64": np.float64, "i32": np.int32, "i64": np.int64}
RADII = [(0, 1), (1, 0), (1, 1), (2, 2), (4, 4), (0, 4), (3, 1)]
SHAPES = [(1, 1), (1, 100), (5, 7), (33, 65), (100, 132), (100, 130), (257, 300)]


def data(dt, shape, rng):
    if np.dtype(dt).kind == "f":
        return rng.random(shape).astype(dt)
    return rng.integers(-1000, 1000, size=shape).astype(dt)


def weights(dt, ry, rx, rng):
    if np.dtype(dt).kind == "f":
        w = rng.uniform(-1, 1, size=(2 * ry + 1, 2 * rx + 1)).astype(dt)
    else:
        w = rng.integers(-3, 4, size=(2 * ry + 1, 2 * rx + 1)).astype(dt)
    w[rng.random(w.shape) < 0.2] = 0
    return w


@pytest.mark.parametrize("t", list(STYPES))
@pytest.mark.parametrize("b", [0, 1, 2, 3])
@pytest.mark.parametrize("ry,rx", RADII)
def test_stencil_grid(acc, orc, dev, t, b, ry, rx):
    dt = STYPES[t]
    rng = case_rng("stencil", t, b, ry, rx)
    for shape in SHAPES:
        if shape[0] == 1 and ry > 0:
            continue
        x = data(dt, shape, rng)
        w = weights(dt, ry, rx, rng)
        xin = x[0] if shape[0] == 1 else x
        got = acc.stencil(w.tolist(), torch.from_numpy(np.ascontiguousarray(xin)).to(dev), b, cval=dt(7)).cpu().numpy()
        ref = orc.stencil2d(w, xin, b, cval=dt(7))
        assert np.array_equal(got, ref), f"{shape}: {_diff(got, ref)}"


def test_stencil_3x3_box_clamp(acc, orc, dev):
    rng = np.random.default_rng(3)
    g = rng.random((1000, 1024), dtype=np.float32)
    w = [[1.0 / 9] * 3] * 3
    got = acc.stencil(w, torch.from_numpy(g).to(dev), "clamp").cpu().numpy()
    assert np.array_equal(got, orc.stencil2d(w, g, 0))


def test_stencil_5point(acc, orc, dev):
    rng = np.random.default_rng(4)
    g = rng.random((777, 513), dtype=np.float32)
    w = [[0, 0.25, 0], [0.25, -1.0, 0.25], [0, 0.25, 0]]
    for b in range(4):
        got = acc.stencil(w, torch.from_numpy(g).to(dev), b, cval=0.5).cpu().numpy()
        assert np.array_equal(got, orc.stencil2d(w, g, b, cval=np.float32(0.5)))


@pytest.mark.parametrize("t", ["f32", "i64"])
def test_stencil2_pair(acc, orc, dev, t):
    dt = STYPES[t]
    rng = np.random.default_rng(9)
    a = data(dt, (70, 90), rng)
    b = data(dt, (64, 100), rng)
    wa, wb = weights(dt, 1, 1, rng), weights(dt, 1, 1, rng)
    got = acc.stencil2(wa.tolist(), wb.tolist(), torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev),
                       "mirror", "wrap").cpu().numpy()
    first = orc.stencil2d(wa, a, 1, out_shape=(64, 90))
    ref = orc.stencil2d(wb, b, 2, accumulate_onto=first, out_shape=(64, 90))
    assert np.array_equal(got, ref), _diff(got, ref)
