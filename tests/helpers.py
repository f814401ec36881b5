"""Seeded input generators and the comparison rules of the parity tests.

Comparison rules (the tolerances are written here, once):
  * integer element types, and float min / max: bit-exact;
  * Float32 (+), compensated or FP64-accumulated: |got - ref| <= 1e-6 |ref| + 1e-9 sum|x|,
    ref = the FP64 oracle, sum|x| over the elements the value depends on;
  * Float32 (+), plain: |got - ref| <= 1e-4 sum|x| (stated, not a target);
  * Float64 (+): |got - ref| <= 1e-12 sum|x| + 1e-15 |ref|;
  * Float32 / Float64 (*): bit-exact on inputs that are powers of two (mostly
    1.0, a sparse 0.5 / 2.0), whose products are exact in any order: a
    coverage check that every element is combined exactly once.
"""
import zlib

import numpy as np
import pytest

def case_rng(*parts):
    """A generator seeded from the test case's parameters, the same in every
    run and on every machine (unlike hash(), which Python randomises per
    process), so that a failing case can be rerun on the same data."""
    return np.random.default_rng(zlib.crc32(repr(parts).encode()))

TYPES = {"i32": np.int32, "i64": np.int64, "u32": np.uint32, "f32": np.float32, "f64": np.float64}
INT_OPS = ["+", "*", "min", "max", "and", "or", "xor"]
FLOAT_OPS = ["+", "*", "min", "max"]
COMBOS = [(t, o) for t in TYPES for o in (FLOAT_OPS if t[0] == "f" else INT_OPS)]


def gen(dt, op, n, rng):
    """Values for (type, op): full-range integers (wrap-around exercised),
    N(0,1) floats for +, values near 1 for *, a few NaNs for float min/max."""
    dt = np.dtype(dt)
    if dt.kind in "iu":
        info = np.iinfo(dt)
        if op == "*":
            return rng.integers(-3 if dt.kind == "i" else 0, 4, size=n, dtype=dt)
        return rng.integers(info.min, info.max, size=n, dtype=dt, endpoint=True)
    if op == "*":
        x = np.ones(n, dtype=dt)
        k = rng.random(n) < min(0.05, 100.0 / max(n, 1))
        x[k] = rng.choice(np.array([0.5, 2.0], dtype=dt), size=int(k.sum()))
        return x
    x = rng.standard_normal(n).astype(dt)
    if op in ("min", "max") and n > 4:
        x[rng.integers(0, n, size=max(1, n // 50))] = np.nan
    return x


def seed_for(dt, op):
    dt = np.dtype(dt)
    if dt.kind == "f":
        return {"+": 0.5, "*": 1.0, "min": 7.0, "max": -7.0}[op]
    return {"+": 5, "*": 1, "min": 1000, "max": 3 if dt.kind == "u" else -1000, "and": -1 if dt.kind == "i" else np.iinfo(dt).max,
            "or": 0, "xor": 12345}[op]


def assert_fold_close(got, ref_t, ref64, absum, dt, op, prec=None):
    """got / ref_t: arrays in the element type; ref64: FP64 oracle (floats);
    absum: sum |x| per output (floats, +)."""
    dt = np.dtype(dt)
    got = np.asarray(got)
    if dt.kind in "iu" or op in ("min", "max", "*"):
        assert got.dtype == dt
        if dt.kind == "f":
            both_nan = np.isnan(got) & np.isnan(ref_t)
            assert np.array_equal(got[~both_nan], ref_t[~both_nan]), _diff(got, ref_t)
            assert np.array_equal(np.isnan(got), np.isnan(ref_t))
        else:
            assert np.array_equal(got, ref_t), _diff(got, ref_t)
        return
    g = got.astype(np.float64)
    if op == "+":
        if dt == np.float32:
            tol = (1e-4 * absum) if prec == "plain" else (1e-6 * np.abs(ref64) + 1e-9 * absum)
        else:
            tol = 1e-12 * absum + 1e-15 * np.abs(ref64)
        err = np.abs(g - ref64)
        assert np.all(err <= tol + 1e-30), f"max err {err.max()} tol {tol[np.argmax(err - tol)] if np.ndim(tol) else tol}"
    else:
        rel = 2e-5 if dt == np.float32 else 1e-13
        assert np.allclose(g, ref64, rtol=rel, atol=0), _diff(got, ref64)


def _diff(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.shape != b.shape:
        return f"shape {a.shape} vs {b.shape}"
    bad = np.flatnonzero(~((a == b) | (np.isnan(a.astype(np.float64)) & np.isnan(b.astype(np.float64)))))
    if bad.size == 0:
        return "equal"
    i = bad[0]
    return f"{bad.size} differ; first at flat {i}: got {a.flat[i]} want {b.flat[i]}"
