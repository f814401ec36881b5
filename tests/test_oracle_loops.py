"""CPU tests: the C oracle against a second, independent restatement in plain
Python loops, on small inputs, for every (type, primitive) pair.

The loops below follow the native backend's sequential definitions directly:
fold is reduceFromTo from the seed (accelerate-llvm-native/src/Data/Array/
Accelerate/LLVM/Native/CodeGen/Fold.hs:248-260), scans combine `f acc x` left
to right and `f x acc` right to left with the seed first or last
(Native/CodeGen/Scan.hs:136-270), foldSeg folds [seg[s], seg[s+1]) of each row
(Native/CodeGen/FoldSeg.hs:103-141) and permute writes `f new old`
(Native/CodeGen/Permute.hs:85-118).  Integer arithmetic wraps
(LLVM/AST/Type/Instruction.hs:429-473); float min/max are IEEE fmin/fmax
(CodeGen/Arithmetic.hs:456-466).  Every element is a numpy scalar of the
array's type, so each float operation rounds to that type as the oracle's do.
"""
import numpy as np
import pytest

from helpers import case_rng

TYPES = [np.int32, np.int64, np.uint32, np.float32, np.float64]
INT_OPS = ["+", "*", "min", "max", "and", "or", "xor"]
FLOAT_OPS = ["+", "*", "min", "max"]
CASES = [(t, o) for t in TYPES for o in (FLOAT_OPS if np.dtype(t).kind == "f" else INT_OPS)]


def prim(op, dt):
    """The primitive on two numpy scalars of type dt, as Python code."""
    if np.dtype(dt).kind in "iu":
        bits = np.dtype(dt).itemsize * 8
        mask = (1 << bits) - 1

        def wrap(v):
            v &= mask
            if np.dtype(dt).kind == "i" and v >> (bits - 1):
                v -= 1 << bits
            return dt(v)
        return {"+": lambda a, b: wrap(int(a) + int(b)),
                "*": lambda a, b: wrap(int(a) * int(b)),
                "min": lambda a, b: a if a <= b else b,
                "max": lambda a, b: a if a >= b else b,
                "and": lambda a, b: wrap(int(a) & int(b)),
                "or": lambda a, b: wrap(int(a) | int(b)),
                "xor": lambda a, b: wrap(int(a) ^ int(b))}[op]
    return {"+": lambda a, b: dt(a + b), "*": lambda a, b: dt(a * b),
            "min": lambda a, b: dt(np.fmin(a, b)), "max": lambda a, b: dt(np.fmax(a, b))}[op]


def values(dt, op, shape, rng):
    if np.dtype(dt).kind in "iu":
        info = np.iinfo(dt)
        return rng.integers(info.min, info.max, size=shape, dtype=dt, endpoint=True)
    if op == "*":
        return rng.choice(np.array([0.5, 1.0, 1.0, 1.0, 2.0, -1.0], dtype=dt), size=shape)
    x = rng.standard_normal(shape).astype(dt)
    if op in ("min", "max"):
        x[rng.random(shape) < 0.1] = np.nan
    return x


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and a.tobytes() == b.tobytes()


def loop_fold(f, z, row):
    acc = z if z is not None else row[0]
    for x in (row if z is not None else row[1:]):
        acc = f(acc, x)
    return acc


def loop_scan(f, z, row, r2l, kind):
    n = len(row)
    if kind == 1:  # scanl z / scanr z: n+1 outputs, the seed first (left) or last (right)
        out = [None] * (n + 1)
        acc = z
        if not r2l:
            out[0] = acc
            for i in range(n):
                acc = f(acc, row[i])
                out[i + 1] = acc
        else:
            out[n] = acc
            for i in range(n - 1, -1, -1):
                acc = f(row[i], acc)
                out[i] = acc
        return out, None
    if kind == 2:  # scanl' z / scanr' z: the carry-in is written before combining
        out = [None] * n
        acc = z
        for i in (range(n) if not r2l else range(n - 1, -1, -1)):
            out[i] = acc
            acc = f(acc, row[i]) if not r2l else f(row[i], acc)
        return out, acc
    out = [None] * n  # scanl1 / scanr1
    if n:
        order = range(n) if not r2l else range(n - 1, -1, -1)
        acc = None
        for i in order:
            acc = row[i] if acc is None else (f(acc, row[i]) if not r2l else f(row[i], acc))
            out[i] = acc
    return out, None


@pytest.mark.parametrize("dt,op", CASES)
def test_fold_matches_loops(orc, dt, op):
    rng = case_rng("loops_fold", np.dtype(dt).name, op)
    f = prim(op, dt)
    xs = values(dt, op, (3, 37), rng)
    z = values(dt, op, (1,), rng)[0]
    assert same(orc.fold(op, None, xs), np.array([loop_fold(f, None, r) for r in xs], dtype=dt))
    assert same(orc.fold(op, z, xs), np.array([loop_fold(f, z, r) for r in xs], dtype=dt))


@pytest.mark.parametrize("dt,op", CASES)
@pytest.mark.parametrize("r2l", [0, 1])
def test_scans_match_loops(orc, dt, op, r2l):
    rng = case_rng("loops_scan", np.dtype(dt).name, op, r2l)
    f = prim(op, dt)
    xs = values(dt, op, (2, 29), rng)
    z = values(dt, op, (1,), rng)[0]
    got = orc.scan(op, None, xs, r2l, 0)
    assert same(got, np.array([loop_scan(f, None, r, r2l, 0)[0] for r in xs], dtype=dt))
    got = orc.scan(op, z, xs, r2l, 1)
    assert same(got, np.array([loop_scan(f, z, r, r2l, 1)[0] for r in xs], dtype=dt))
    got, sums = orc.scan(op, z, xs, r2l, 2)
    ref = [loop_scan(f, z, r, r2l, 2) for r in xs]
    assert same(got, np.array([o for o, _ in ref], dtype=dt))
    assert same(sums, np.array([t for _, t in ref], dtype=dt))


@pytest.mark.parametrize("dt,op", CASES)
def test_fold_seg_matches_loops(orc, dt, op):
    rng = case_rng("loops_foldseg", np.dtype(dt).name, op)
    f = prim(op, dt)
    lens = rng.integers(0, 9, size=11)
    lens[[2, 7]] = 0  # empty segments
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    xs = values(dt, op, (2, int(off[-1]) + 3), rng)  # a tail no segment covers
    z = values(dt, op, (1,), rng)[0]
    ref = np.array([[loop_fold(f, z, r[off[s]:off[s + 1]]) for s in range(len(lens))] for r in xs], dtype=dt)
    assert same(orc.fold_seg(op, z, xs, off), ref)
    got = orc.fold_seg(op, None, xs, off)  # without a seed an empty segment is left unwritten (zeros here)
    ref = np.zeros_like(got)
    for r in range(xs.shape[0]):
        for s in range(len(lens)):
            if lens[s]:
                ref[r, s] = loop_fold(f, None, xs[r, off[s]:off[s + 1]])
    assert same(got, ref)


@pytest.mark.parametrize("dt,op", [c for c in CASES if np.dtype(c[0]).kind in "iu" or c[1] in ("min", "max")])
def test_permute_matches_loops(orc, dt, op):
    # integers and float min/max: exact in any update order
    rng = case_rng("loops_permute", np.dtype(dt).name, op)
    f = prim(op, dt)
    m = 13
    idx = rng.integers(-3, m, size=200).astype(np.int32)  # negative: Nothing
    xs = values(dt, op, (200,), rng)
    defaults = values(dt, op, (m,), rng)
    ref = list(defaults)
    for i, j in enumerate(idx):
        if j >= 0:
            ref[j] = f(xs[i], ref[j])  # new value first, old value second
    assert same(orc.permute(op, defaults, idx, xs), np.array(ref, dtype=dt))


def loop_bound(i, n, b):
    """Boundary remap of accelerate-llvm/.../CodeGen/Stencil.hs:224-253 (clamp,
    mirror, wrap), kept inside the array when a radius exceeds the extent."""
    if i < 0:
        i = 0 if b == 0 else (-i if b == 1 else n + i)
    elif i >= n:
        i = n - 1 if b == 0 else (n - (i - n + 2) if b == 1 else i - n)
    return min(max(i, 0), n - 1)


def fma_exact(dt, w, v, acc):
    """w*v + acc rounded once to dt (round to nearest, ties to even): the exact
    value in rational arithmetic, then the nearest of the neighbouring values
    of dt.  An exact zero takes the IEEE sign, which the double evaluation of
    the same (then exact) expression gives."""
    from fractions import Fraction
    q = Fraction(float(w)) * Fraction(float(v)) + Fraction(float(acc))
    if q == 0:
        return dt(np.float64(w) * np.float64(v) + np.float64(acc))
    if dt is np.float64:
        return np.float64(float(q))  # int / int division: correctly rounded
    c = np.float32(float(q))
    near = [t for t in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf)))
            if np.isfinite(t)]
    return min(near, key=lambda t: (abs(Fraction(float(t)) - q), int(t.view(np.uint32)) & 1))


def loop_stencil(w, x, b, cval, acc_from=None, out_shape=None):
    """Weighted sum, taps rows outer and -r..r, one fused multiply-add per
    non-zero tap (rounded once), integers wrapping."""
    dt = x.dtype.type
    ky, kx = w.shape
    ry, rx = ky // 2, kx // 2
    ih, iw = x.shape
    h, wd = out_shape if out_shape is not None else x.shape
    out = np.empty((h, wd), dtype=x.dtype)
    f = prim("+", dt)
    for y in range(h):
        for xo in range(wd):
            acc = acc_from[y, xo] if acc_from is not None else (dt(-0.0) if x.dtype.kind == "f" else dt(0))
            for dy in range(-ry, ry + 1):
                for dx in range(-rx, rx + 1):
                    wk = w[dy + ry, dx + rx]
                    if wk == 0:
                        continue
                    yy, xx = y + dy, xo + dx
                    if 0 <= yy < ih and 0 <= xx < iw:
                        v = x[yy, xx]
                    elif b == 3:
                        v = dt(cval)
                    else:
                        v = x[loop_bound(yy, ih, b), loop_bound(xx, iw, b)]
                    if x.dtype.kind == "f":
                        acc = fma_exact(dt, wk, v, acc)
                    else:
                        acc = f(acc, prim("*", dt)(wk, v))
            out[y, xo] = acc
    return out


@pytest.mark.parametrize("dt", [np.float32, np.float64, np.int32, np.int64])
@pytest.mark.parametrize("b", [0, 1, 2, 3])
def test_stencil_matches_loops(orc, dt, b):
    rng = case_rng("loops_stencil", np.dtype(dt).name, b)
    for (ky, kx), shape in [((3, 3), (6, 7)), ((1, 5), (4, 9)), ((5, 3), (7, 5)), ((3, 1), (2, 3)), ((5, 5), (3, 3))]:
        if np.dtype(dt).kind == "f":
            x = rng.random(shape).astype(dt)
            w = rng.uniform(-1, 1, (ky, kx)).astype(dt)
        else:
            x = rng.integers(-1000, 1000, shape).astype(dt)
            w = rng.integers(-3, 4, (ky, kx)).astype(dt)
        w[rng.random(w.shape) < 0.2] = 0
        got = orc.stencil2d(w, x, boundary=b, cval=dt(5))
        assert same(got, loop_stencil(w, x, b, 5)), (ky, kx, shape)
        # stencil2: a second input continues the accumulator over the
        # intersection of the two extents
        x2 = x[: shape[0] - 1, 1:] if shape[0] > 1 and shape[1] > 1 else x
        out_shape = (min(x.shape[0], x2.shape[0]), min(x.shape[1], x2.shape[1]))
        first = orc.stencil2d(w, x, boundary=b, cval=dt(5), out_shape=out_shape)
        got = orc.stencil2d(w, x2, boundary=b, cval=dt(5), accumulate_onto=first, out_shape=out_shape)
        ref = loop_stencil(w, x2, b, 5, acc_from=loop_stencil(w, x, b, 5, out_shape=out_shape), out_shape=out_shape)
        assert same(got, ref), ("pair", ky, kx, shape)
