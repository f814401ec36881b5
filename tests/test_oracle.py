"""CPU tests of the oracle: pinned to the reference's known answers, and
self-consistent (canonical sequential order vs the OpenMP split order for the
integer primitives, where every order must agree)."""
import json
import pathlib

import numpy as np
import pytest

GOLDEN = json.loads((pathlib.Path(__file__).parent / "golden" / "known_answers.json").read_text())
INT_TYPES = [np.int32, np.int64, np.uint32]
INT_OPS = ["+", "*", "min", "max", "and", "or", "xor"]


def test_known_answer_sum_map_succ(orc):
    g = GOLDEN["sum_map_succ"]
    lo, hi = g["input_range"]
    xs = np.arange(lo, hi + 1, dtype=np.int64) + 1  # A.map (+1)
    assert int(orc.fold(g["op"], g["seed"], xs)) == g["expect"]
    # the parallel (divideWork) order gives the same integer
    assert int(orc.fold(g["op"], g["seed"], xs, nthreads=4)) == g["expect"]


def test_known_answer_scanl_example(orc):
    g = GOLDEN["scanl_example"]
    xs = np.array(g["input"], dtype=np.int64)
    out = orc.scan(g["op"], g["seed"], xs, 0, 1)
    assert out.tolist() == g["expect"] and out.size == g["out_len"]


def test_known_answer_scanl_prime_example(orc):
    # mkScan's example of scanl' (exclusive scan, total returned apart)
    g = GOLDEN["scanl_prime_example"]
    xs = np.array(g["input"], dtype=np.int64)
    out, tot = orc.scan(g["op"], g["seed"], xs, 0, 2)
    assert out.tolist() == g["expect"] and out.size == g["out_len"] and int(tot) == g["expect_total"]


def test_scan_flavours_small(orc):
    xs = np.arange(10, dtype=np.int64)
    # scanr z: out[i] = x_i + ... + x_(n-1) + z, out[n] = z (Native/CodeGen/Scan.hs:190-205)
    assert orc.scan("+", 10, xs, 1, 1).tolist() == [55, 55, 54, 52, 49, 45, 40, 34, 27, 19, 10]
    # scanl' z: exclusive, total separately
    out, tot = orc.scan("+", 10, xs, 0, 2)
    assert out.tolist() == [10, 10, 11, 13, 16, 20, 25, 31, 38, 46] and int(tot) == 55
    # scanr' z: out[i] = x_(i+1) + ... + z
    out, tot = orc.scan("+", 10, xs, 1, 2)
    assert out.tolist() == [55, 54, 52, 49, 45, 40, 34, 27, 19, 10] and int(tot) == 55
    assert orc.scan("+", None, xs, 0, 0).tolist() == np.cumsum(xs).tolist()
    assert orc.scan("+", None, xs, 1, 0).tolist() == np.cumsum(xs[::-1])[::-1].tolist()


def test_divide_work1_covers_range(orc):
    for splits, n in [(0, 100), (3, 10_000), (15, 1 << 20), (7, 4097)]:
        ps = sorted(orc.divide_work1(splits, 4096, 0, n), key=lambda p: p[2])
        assert ps[0][0] == 0 and ps[-1][1] == n
        for a, b in zip(ps, ps[1:]):
            assert a[1] == b[0]
        assert [p[2] for p in ps] == list(range(len(ps)))


@pytest.mark.parametrize("dt", INT_TYPES)
@pytest.mark.parametrize("op", INT_OPS)
def test_integer_orders_agree(orc, dt, op):
    rng = np.random.default_rng(1)
    info = np.iinfo(dt)
    xs = rng.integers(info.min, info.max, size=50_000, dtype=dt, endpoint=True)
    seed = dt(3)
    assert np.array_equal(orc.fold(op, seed, xs), orc.fold(op, seed, xs, nthreads=6))
    assert np.array_equal(orc.scan(op, None, xs, 0, 0), orc.scan(op, None, xs, 0, 0, nthreads=6))
    assert np.array_equal(orc.scan(op, seed, xs, 0, 1), orc.scan(op, seed, xs, 0, 1, nthreads=6))
    idx = rng.integers(-5, 300, size=50_000).astype(np.int32)
    d = rng.integers(0, 100, size=300, dtype=dt)
    assert np.array_equal(orc.permute(op, d, idx, xs), orc.permute(op, d, idx, xs, nthreads=6))


def test_integer_wraparound(orc):
    xs = np.array([np.iinfo(np.int32).max, 1], dtype=np.int32)
    assert int(orc.fold("+", None, xs)) == np.iinfo(np.int32).min
    xs = np.array([1 << 62, 4], dtype=np.int64)
    assert int(orc.fold("*", None, xs)) == 0


def test_float_min_max_ignore_nan(orc):
    xs = np.array([np.nan, 3.0, np.nan, -1.0], dtype=np.float32)
    assert float(orc.fold("min", None, xs)) == -1.0
    assert float(orc.fold("max", None, xs)) == 3.0
    assert np.isnan(orc.fold("min", None, np.array([np.nan, np.nan], np.float32)))


def test_fold_empty(orc):
    with pytest.raises(orc.OracleError):
        orc.fold("+", None, np.zeros((3, 0), np.int32))
    assert orc.fold("+", 7, np.zeros((3, 0), np.int32)).tolist() == [7, 7, 7]


def test_fold_seg_semantics(orc):
    xs = np.arange(10, dtype=np.int32)
    off = np.array([0, 3, 3, 10], dtype=np.int32)
    assert orc.fold_seg("+", 100, xs, off).tolist() == [103, 100, 142]
    out = orc.fold_seg("+", None, xs, off)  # empty segment left unwritten (zeros here)
    assert out[0] == 3 and out[2] == 42
    with pytest.raises(orc.OracleError):
        orc.fold_seg("+", 0, xs, np.array([0, 5, 11], dtype=np.int32))


def test_permute_semantics(orc):
    d = np.zeros(4, dtype=np.int32)
    idx = np.array([0, 1, -1, 1, 3], dtype=np.int32)
    assert orc.permute("+", d, idx, cval=1).tolist() == [1, 2, 0, 1]
    xs = np.array([5, 6, 7, 8, 9], dtype=np.int32)
    assert orc.permute("max", d - 1, idx, xs).tolist() == [5, 8, -1, 9]
    with pytest.raises(orc.OracleError):
        orc.permute("+", d, np.array([4], np.int32), cval=1)


@pytest.mark.parametrize("b,expect", [
    # 1-D [1,2,3], weights [1,10,100]: out[x] = 1*a[x-1] + 10*a[x] + 100*a[x+1]
    (0, [1 + 10 + 200, 1 + 20 + 300, 2 + 30 + 300]),     # clamp: a[-1]=a[0], a[3]=a[2]
    (1, [2 + 10 + 200, 1 + 20 + 300, 2 + 30 + 200]),     # mirror: a[-1]=a[1], a[3]=a[1]
    (2, [3 + 10 + 200, 1 + 20 + 300, 2 + 30 + 100]),     # wrap: a[-1]=a[2], a[3]=a[0]
    (3, [-7 + 10 + 200, 1 + 20 + 300, 2 + 30 - 700]),    # constant -7
])
def test_stencil_boundaries(orc, b, expect):
    a = np.array([1, 2, 3], dtype=np.int32)
    out = orc.stencil2d([[1, 10, 100]], a, boundary=b, cval=-7)
    assert out.tolist() == expect


def test_stencil_zero_weight_taps_not_read(orc):
    a = np.array([[1.0, np.inf, 1.0]], dtype=np.float32)
    w = [[0, 0, 0], [1, 0, 1], [0, 0, 0]]
    out = orc.stencil2d(w, a)
    assert out[0, 1] == 2.0


def test_f64_oracle_is_accurate(orc):
    rng = np.random.default_rng(2)
    xs = rng.standard_normal(1 << 20).astype(np.float32)
    exact = float(np.sum(xs.astype(np.float64)))  # pairwise in f64
    assert abs(float(orc.fold_f64("+", 0.0, xs)) - exact) <= 1e-9 * max(1.0, abs(exact))


# ---- rank-3 stencils (planes outer, then rows, then columns)
PAD_MODE = {0: "edge", 1: "reflect", 2: "wrap", 3: "constant"}  # clamp, mirror, wrap, constant


def stencil3d_numpy(w, x, b, cval):
    """The same weighted sum from numpy's padding modes: Accelerate's mirror
    (i < 0 -> -i, i >= n -> 2n - i - 2) is numpy's 'reflect'."""
    rz, ry, rx = (s // 2 for s in w.shape)
    kw = {"constant_values": cval} if b == 3 else {}
    p = np.pad(x, ((rz, rz), (ry, ry), (rx, rx)), mode=PAD_MODE[b], **kw)
    d, h, wd = x.shape
    out = np.zeros_like(x)
    for dz in range(w.shape[0]):
        for dy in range(w.shape[1]):
            for dx in range(w.shape[2]):
                out += w[dz, dy, dx] * p[dz:dz + d, dy:dy + h, dx:dx + wd]
    return out


@pytest.mark.parametrize("b", [0, 1, 2, 3])
@pytest.mark.parametrize("dt", [np.int32, np.int64, np.float64])
@pytest.mark.parametrize("pattern", [(3, 3, 3), (1, 3, 5), (5, 1, 3), (3, 5, 1)])
def test_stencil3d_against_numpy(orc, b, dt, pattern):
    # small integer values: every sum is exact, so any order must agree
    rng = np.random.default_rng(sum(pattern) * 10 + b)
    x = rng.integers(-50, 50, size=(6, 7, 9)).astype(dt)
    w = rng.integers(-3, 4, size=pattern).astype(dt)
    w.flat[0] = 0  # a tap outside the pattern
    got = orc.stencil3d(w, x, boundary=b, cval=-11)
    assert np.array_equal(got, stencil3d_numpy(w, x, b, dt(-11)))
    assert np.array_equal(orc.stencil3d(w, x, boundary=b, cval=-11, nthreads=4), got)


@pytest.mark.parametrize("b", [0, 1, 2, 3])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_stencil3d_is_planes_of_2d_in_order(orc, b, dt):
    # Float taps with fused multiply-adds: bit-exact against the rank-2 oracle
    # run plane by plane (dz = -rz .. rz), each continuing the accumulator,
    # which pins the planes-outer tap order.
    rng = np.random.default_rng(b)
    x = rng.random((5, 6, 7)).astype(dt)
    w = rng.standard_normal((3, 3, 3)).astype(dt)
    cval = dt(0.25)
    got = orc.stencil3d(w, x, boundary=b, cval=cval)
    d = x.shape[0]
    for z in range(d):
        acc = np.full(x.shape[1:], dt(-0.0))
        for k, dz in enumerate((-1, 0, 1)):
            zz = z + dz
            if 0 <= zz < d:
                plane = x[zz]
            elif b == 3:
                plane = np.full(x.shape[1:], cval)
            else:
                zz = {0: min(max(zz, 0), d - 1), 1: -zz if zz < 0 else 2 * d - zz - 2, 2: zz % d}[b]
                plane = x[zz]
            acc = orc.stencil2d(w[k], plane, boundary=b, cval=cval, accumulate_onto=acc)
        assert np.array_equal(got[z], acc), z


def test_stencil3d_flat_pattern_is_2d(orc):
    rng = np.random.default_rng(7)
    x = rng.random((4, 8, 9)).astype(np.float32)
    w = rng.standard_normal((1, 3, 5)).astype(np.float32)
    got = orc.stencil3d(w, x, boundary=1)
    for z in range(4):
        assert np.array_equal(got[z], orc.stencil2d(w[0], x[z], boundary=1))
