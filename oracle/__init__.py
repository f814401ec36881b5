"""oracle -- numpy front end of liboracle.so (the C restatement in oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle of tests/ and __graft_entry__.smoke(),
and the timed CPU baseline of bench.py.  The product path never imports it.

Every function takes and returns numpy arrays and mirrors one entry point of
include/acc_gb300.h, with the same enums and the same element semantics
(see oracle.c for the accelerate-llvm-native files each one follows).
`nthreads=1` gives the native backend's single-thread evaluation order (the
canonical order the tests compare against); `nthreads>1` runs the OpenMP
version with the native backend's divideWork split, used for CPU timing.
"""
from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "oracle.c"
LIB = HERE / "liboracle.so"

I32, I64, U32, F32, F64 = range(5)
NP_OF = {I32: np.int32, I64: np.int64, U32: np.uint32, F32: np.float32, F64: np.float64}
CODE_OF = {np.dtype(np.int32): I32, np.dtype(np.int64): I64, np.dtype(np.uint32): U32,
           np.dtype(np.float32): F32, np.dtype(np.float64): F64}
OPS = {"+": 0, "*": 1, "min": 2, "max": 3, "and": 4, "or": 5, "xor": 6}

CFLAGS = ["-O3", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared"]


def build(force: bool = False) -> pathlib.Path:
    """Compile oracle.c into liboracle.so (gcc, OpenMP)."""
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        cc = os.environ.get("CC", "gcc")
        subprocess.run([cc, *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(str(LIB))
        P, I, L = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64
        sig = {
            "orc_threads": ([], I),
            "orc_divide_work1": ([L, L, L, L, P, L], L),
            "orc_fold": ([I, I, P, P, L, L, P, I], I),
            "orc_fold_seg": ([I, I, P, P, I, P, L, L, L, P, I], I),
            "orc_scan": ([I, I, I, I, P, P, P, L, L, P, I], I),
            "orc_permute": ([I, I, P, P, P, I, P, L, L, I], I),
            "orc_fold_f64": ([I, I, P, P, L, L, P], I),
            "orc_fold_seg_f64": ([I, I, P, P, I, P, L, L, L, P], I),
            "orc_scan_f64": ([I, I, I, I, P, P, P, L, L, P], I),
            "orc_stencil2d": ([I, I, I, P, I, P, P, L, L, P, L, L, I, I], I),
            "orc_stencil3d": ([I, I, I, I, P, I, P, P, L, L, L, P, L, L, L, I, I], I),
        }
        for k, (a, r) in sig.items():
            f = getattr(_lib, k)
            f.argtypes, f.restype = a, r
    return _lib


class OracleError(RuntimeError):
    def __init__(self, status):
        self.status = status
        super().__init__(f"oracle status {status}")


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _scalar(dt, v):
    if v is None:
        return None, None
    a = np.array([v], dtype=dt)
    return _p(a), a


def _op(f):
    return f if isinstance(f, int) else OPS[f]


def _chk(st):
    if st != 0:
        raise OracleError(st)


def threads() -> int:
    return lib().orc_threads()


def divide_work1(splits, minsize, frm, to):
    cap = 2 * (splits + 2) + 8
    out = np.zeros(3 * cap, dtype=np.int64)
    k = lib().orc_divide_work1(splits, minsize, frm, to, _p(out), cap)
    return [tuple(int(x) for x in out[3 * i:3 * i + 3]) for i in range(k)]


def fold(f, z, xs: np.ndarray, nthreads: int = 1) -> np.ndarray:
    xs = np.ascontiguousarray(xs)
    tc = CODE_OF[xs.dtype]
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    out = np.empty(xs.shape[:-1], dtype=xs.dtype)
    sp, keep = _scalar(xs.dtype, z)
    _chk(lib().orc_fold(_op(f), tc, _p(xs), _p(out), outer, inner, sp, nthreads))
    return out


def fold_seg(f, z, xs, offsets, nthreads: int = 1) -> np.ndarray:
    xs = np.ascontiguousarray(xs)
    offsets = np.ascontiguousarray(offsets)
    tc = CODE_OF[xs.dtype]
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    nseg = offsets.size - 1
    out = np.zeros(xs.shape[:-1] + (nseg,), dtype=xs.dtype)
    sp, keep = _scalar(xs.dtype, z)
    _chk(lib().orc_fold_seg(_op(f), tc, _p(xs), _p(offsets), CODE_OF[offsets.dtype], _p(out), outer, inner, nseg,
                            sp, nthreads))
    return out


def scan(f, z, xs, direction: int, kind: int, nthreads: int = 1):
    """direction 0 = L2R, 1 = R2L; kind 0 = inclusive, 1 = seeded (n+1), 2 = prime (+ sums)."""
    xs = np.ascontiguousarray(xs)
    tc = CODE_OF[xs.dtype]
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    out = np.zeros(xs.shape[:-1] + (inner + 1 if kind == 1 else inner,), dtype=xs.dtype)
    sums = np.zeros(xs.shape[:-1], dtype=xs.dtype) if kind == 2 else None
    sp, keep = _scalar(xs.dtype, z)
    _chk(lib().orc_scan(_op(f), tc, direction, kind, _p(xs), _p(out), _p(sums), outer, inner, sp, nthreads))
    return (out, sums) if kind == 2 else out


def permute(f, defaults, idx, xs=None, cval=None, nthreads: int = 1) -> np.ndarray:
    out = np.array(defaults, copy=True)
    idx = np.ascontiguousarray(idx)
    tc = CODE_OF[out.dtype]
    n = idx.size
    if xs is not None:
        xs = np.ascontiguousarray(xs, dtype=out.dtype)
        cp, keep = None, None
    else:
        cp, keep = _scalar(out.dtype, 1 if cval is None else cval)
    _chk(lib().orc_permute(_op(f), tc, _p(xs) if xs is not None else None, cp, _p(idx), CODE_OF[idx.dtype],
                           _p(out), n, out.size, nthreads))
    return out


def fold_f64(f, z, xs) -> np.ndarray:
    xs = np.ascontiguousarray(xs)
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    out = np.empty(xs.shape[:-1], dtype=np.float64)
    sp, keep = _scalar(np.float64, z)
    _chk(lib().orc_fold_f64(_op(f), CODE_OF[xs.dtype], _p(xs), _p(out), outer, inner, sp))
    return out


def fold_seg_f64(f, z, xs, offsets) -> np.ndarray:
    xs = np.ascontiguousarray(xs)
    offsets = np.ascontiguousarray(offsets)
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    nseg = offsets.size - 1
    out = np.zeros(xs.shape[:-1] + (nseg,), dtype=np.float64)
    sp, keep = _scalar(np.float64, z)
    _chk(lib().orc_fold_seg_f64(_op(f), CODE_OF[xs.dtype], _p(xs), _p(offsets), CODE_OF[offsets.dtype], _p(out),
                                outer, inner, nseg, sp))
    return out


def scan_f64(f, z, xs, direction: int, kind: int):
    xs = np.ascontiguousarray(xs)
    inner = xs.shape[-1]
    outer = int(np.prod(xs.shape[:-1])) if xs.ndim > 1 else 1
    out = np.zeros(xs.shape[:-1] + (inner + 1 if kind == 1 else inner,), dtype=np.float64)
    sums = np.zeros(xs.shape[:-1], dtype=np.float64) if kind == 2 else None
    sp, keep = _scalar(np.float64, z)
    _chk(lib().orc_scan_f64(_op(f), CODE_OF[xs.dtype], direction, kind, _p(xs), _p(out), _p(sums), outer, inner,
                            sp))
    return (out, sums) if kind == 2 else out


def stencil2d(weights, xs, boundary: int = 0, cval=None, nthreads: int = 1, accumulate_onto=None,
              out_shape=None) -> np.ndarray:
    """Weighted-sum stencil of a rank-1 or rank-2 array.  With accumulate_onto
    the taps continue that array's accumulator (the second input of stencil2);
    out_shape (default: the input's shape) is the output extent."""
    xs = np.ascontiguousarray(xs)
    w2 = np.ascontiguousarray(np.asarray(weights, dtype=xs.dtype).reshape(len(weights), -1))
    ky, kx = w2.shape
    ih, iw = (1, xs.shape[0]) if xs.ndim == 1 else xs.shape
    if out_shape is None:
        out_shape = xs.shape
    h, w = (1, out_shape[0]) if len(out_shape) == 1 else out_shape
    if accumulate_onto is not None:
        out = np.array(accumulate_onto, copy=True)
        acc = 1
    else:
        out = np.empty(out_shape, dtype=xs.dtype)
        acc = 0
    cp, keep = _scalar(xs.dtype, 0 if cval is None else cval)
    _chk(lib().orc_stencil2d(CODE_OF[xs.dtype], ky // 2, kx // 2, _p(w2), boundary, cp, _p(xs), ih, iw, _p(out), h,
                             w, acc, nthreads))
    return out


def stencil3d(weights, xs, boundary: int = 0, cval=None, nthreads: int = 1, accumulate_onto=None,
              out_shape=None) -> np.ndarray:
    """Weighted-sum stencil of a rank-3 array [planes][rows][columns] with a
    (2rz+1) x (2ry+1) x (2rx+1) weight array; taps planes outer, rows, then
    columns, every index component remapped by the boundary.  accumulate_onto
    and out_shape as for stencil2d."""
    xs = np.ascontiguousarray(xs)
    w3 = np.ascontiguousarray(np.asarray(weights, dtype=xs.dtype))
    if xs.ndim != 3 or w3.ndim != 3:
        raise ValueError("stencil3d takes a rank-3 array and a rank-3 weight pattern")
    kz, ky, kx = w3.shape
    if out_shape is None:
        out_shape = xs.shape
    if accumulate_onto is not None:
        out = np.array(accumulate_onto, copy=True)
        acc = 1
    else:
        out = np.empty(out_shape, dtype=xs.dtype)
        acc = 0
    cp, keep = _scalar(xs.dtype, 0 if cval is None else cval)
    _chk(lib().orc_stencil3d(CODE_OF[xs.dtype], kz // 2, ky // 2, kx // 2, _p(w3), boundary, cp, _p(xs), *xs.shape,
                             _p(out), *out_shape, acc, nthreads))
    return out
