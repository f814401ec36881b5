"""accelerate-llvm_gb300 -- host-side mirror of Accelerate's PTX skeleton ops.

Thin Python layer over ``libaccgb.so`` (the C ABI declared in
``include/acc_gb300.h``).  Each function mirrors one `Execute PTX` skeleton op
of accelerate-llvm-ptx (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/
PTX/Execute.hs:83-109) with the Accelerate names and argument meaning:

    fold f z xs, fold1 f xs, fold_seg f z xs seg, fold1_seg f xs seg,
    scanl/scanl1/scanr/scanr1, scanl_ (scanl'), scanr_ (scanr'),
    permute f defaults idx xs, stencil (weighted sum) and stencil2,

plus the host <-> device transfers (``upload`` / ``download``, pokeArrayAsync /
peekArrayAsync) and the memory table (``Table``: useArrayAsync, mallocArray,
pokeArrayAsync, peekArrayAsync, withRemote, freeRemote).

Arrays are CUDA tensors (torch is the device allocator and stream provider
only); results are allocated here, as the reference allocates them with
``allocateRemote``.  The combine function is one of the fixed primitives
``'+' '*' 'min' 'max' 'and' 'or' 'xor'``; anything else raises, as the
reference's shim raises ``internalError "unsupported combine function"``.

There is no CPU fallback: the library is loaded on first use, and that first
call raises on a machine where it cannot be loaded; host (CPU) tensors are
refused with ValueError, never computed on the host.
"""
from __future__ import annotations

import ctypes
import pathlib
from typing import Optional, Sequence, Union

import torch

_HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = _HERE / "libaccgb.so"

# ----------------------------------------------------------------- enums (acc_gb300.h)
I32, I64, U32, F32, F64 = range(5)
ADD, MUL, MIN, MAX, AND, OR, XOR = range(7)
PREC_DEFAULT, PREC_PLAIN, PREC_COMPENSATED, PREC_FP64ACC = range(4)
L2R, R2L = 0, 1
SCAN_INCLUSIVE, SCAN_SEEDED, SCAN_PRIME = range(3)
CLAMP, MIRROR, WRAP, CONSTANT = range(4)

OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "UNSUPPORTED", 3: "EMPTY", 4: "CUDA", 5: "NOMEM",
                6: "TIMEOUT", 7: "INDEX", 8: "TOO_LARGE"}

OPS = {"+": ADD, "add": ADD, "*": MUL, "mul": MUL, "min": MIN, "max": MAX,
       "and": AND, ".&.": AND, "or": OR, ".|.": OR, "xor": XOR}
BOUNDARIES = {"clamp": CLAMP, "mirror": MIRROR, "wrap": WRAP, "constant": CONSTANT}
PRECS = {None: PREC_DEFAULT, "default": PREC_DEFAULT, "plain": PREC_PLAIN,
         "compensated": PREC_COMPENSATED, "fp64": PREC_FP64ACC}

_DTYPES = {torch.int32: I32, torch.int64: I64, torch.float32: F32, torch.float64: F64}
if hasattr(torch, "uint32"):
    _DTYPES[torch.uint32] = U32
_CTYPES = {I32: ctypes.c_int32, I64: ctypes.c_int64, U32: ctypes.c_uint32, F32: ctypes.c_float,
           F64: ctypes.c_double}


class AccError(RuntimeError):
    """A non-zero acc_status from the library."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        text = _lib.acc_strerror(status).decode() if _lib is not None else STATUS_NAMES.get(status, "?")
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)} ({text})" if what else text)


# ----------------------------------------------------------------- loading
_lib: Optional[ctypes.CDLL] = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
SIGNATURES = {
    "acc_version": ([], _I),
    "acc_strerror": ([_I], ctypes.c_char_p),
    "acc_sync": ([_P], _I),
    "acc_release_workspaces": ([], _I),
    "acc_selftest_timeout": ([_I, _P], _I),
    "acc_fold": ([_I, _I, _I, _P, _P, _L, _L, _P, _P], _I),
    "acc_fold_zipwith": ([_I, _I, _I, _I, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_fold_seg": ([_I, _I, _I, _P, _P, _I, _P, _L, _L, _L, _P, _P], _I),
    "acc_fold_seg_zipwith": ([_I, _I, _I, _I, _P, _P, _P, _I, _P, _L, _L, _L, _P, _P], _I),
    "acc_fold_seg_lengths": ([_I, _I, _I, _P, _P, _I, _P, _L, _L, _L, _P, _P], _I),
    "acc_scan": ([_I, _I, _I, _I, _I, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_scan_noalloc": ([_I, _I, _I, _I, _I, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_scan_noalloc_status": ([_P], _I),
    "acc_scan_zipwith": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_scan_map": ([_I, _I, _I, _I, _I, _I, _P, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_fold_map": ([_I, _I, _I, _I, _P, _P, _P, _L, _L, _P, _P], _I),
    "acc_permute": ([_I, _I, _P, _P, _P, _I, _P, _L, _L, _P], _I),
    "acc_permute_clone": ([_I, _I, _P, _P, _P, _P, _I, _P, _L, _L, _P], _I),
    "acc_stencil2d": ([_I, _I, _I, _P, _I, _P, _P, _P, _L, _L, _P], _I),
    "acc_stencil3d": ([_I, _I, _I, _I, _P, _I, _P, _P, _P, _L, _L, _L, _P], _I),
    "acc_stencil2d_pair": ([_I, _I, _I, _P, _P, _I, _P, _I, _P, _P, _L, _L, _P, _L, _L, _P, _P], _I),
    "acc_batch_create": ([_I, _P, _L, _P], _I),
    "acc_batch_capture": ([_P, _P], _I),
    "acc_batch_launch": ([_P, _P], _I),
    "acc_batch_status": ([_P, _P], _I),
    "acc_batch_destroy": ([_P], _I),
    "acc_batch_autotune": ([ctypes.c_char_p, _P], _I),
    "acc_batch_load_tuning": ([ctypes.c_char_p], _I),
    "acc_serve_run": ([_P, _L, _L, _I, _I, _P, _P], _I),
    "acc_upload": ([_P, _P, _L, _P], _I),
    "acc_download": ([_P, _P, _L, _P], _I),
    "acc_table_create": ([_L, _P], _I),
    "acc_table_destroy": ([_P], _I),
    "acc_table_use": ([_P, _P, _L, _P, _P], _I),
    "acc_table_malloc": ([_P, _P, _L, _P, _P], _I),
    "acc_table_poke": ([_P, _P, _P], _I),
    "acc_table_peek": ([_P, _P, _P], _I),
    "acc_table_release": ([_P, _P, _P], _I),
    "acc_table_wait": ([_P, _P], _I),
    "acc_table_join": ([_P, _P], _I),
    "acc_table_free": ([_P, _P], _I),
    "acc_table_get_stats": ([_P, _P], _I),
    "acc_table_trace": ([_P, _I], _I),
    "acc_table_trace_get": ([_P, _P, _P, _L, _P], _I),
}


def load(path: Union[str, pathlib.Path, None] = None) -> ctypes.CDLL:
    """Load libaccgb.so (building it first if it is missing and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        from . import build as _build  # noqa: F401  (only when imported as a package)
        _build.build()
    lib = ctypes.CDLL(str(p))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def lib() -> ctypes.CDLL:
    return _lib if _lib is not None else load()


def _check(status: int, what: str) -> None:
    if status != OK:
        raise AccError(status, what)


# ----------------------------------------------------------------- helpers
def type_of(t: torch.Tensor) -> int:
    try:
        return _DTYPES[t.dtype]
    except KeyError:
        raise TypeError(f"unsupported element type {t.dtype}") from None


def op_of(f) -> int:
    if isinstance(f, int):
        return f
    try:
        return OPS[f]
    except KeyError:
        raise ValueError(f"unsupported combine function {f!r} (fixed primitives only)") from None


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _seed_ptr(type_code: int, value):
    if value is None:
        return None, None
    c = _CTYPES[type_code](value)
    return ctypes.cast(ctypes.pointer(c), ctypes.c_void_p), c


def _ptr(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def _dev(t: torch.Tensor) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError("arrays must be CUDA tensors")
    return t.contiguous()


def _given(t, need: int, what: str, dtype=None):
    """A caller-provided array that the library reads or writes in place (a
    batch or serving request): the library sees only its address, so it must
    be a contiguous CUDA tensor holding at least `need` elements, of `dtype`
    when one is given.  Checked here because a short or host-side buffer would
    otherwise be accessed out of bounds on the device."""
    if not getattr(t, "is_cuda", False):
        raise ValueError(f"{what}: arrays must be CUDA tensors")
    if not t.is_contiguous():
        raise ValueError(f"{what}: arrays must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{what}: element type {t.dtype}, expected {dtype}")
    if t.numel() < need:
        raise ValueError(f"{what}: {t.numel()} elements, at least {need} needed")
    return t


def sync(stream=None) -> None:
    """Wait for the stream and raise any device-side error (acc_sync)."""
    _check(lib().acc_sync(_stream(stream)), "acc_sync")


# ----------------------------------------------------------------- fold
def fold(f, z, xs: torch.Tensor, prec=None, stream=None) -> torch.Tensor:
    """fold f z xs: reduce the innermost dimension from the seed z (PTX/Execute.hs:237-249)."""
    return _fold(f, z, xs, prec, stream)


def fold1(f, xs: torch.Tensor, prec=None, stream=None) -> torch.Tensor:
    """fold1 f xs: reduce the (non-empty) innermost dimension (PTX/Execute.hs:222-235)."""
    return _fold(f, None, xs, prec, stream)


def _fold(f, z, xs, prec, stream):
    xs = _dev(xs)
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1] if shape else 1
    outer_shape = shape[:-1]
    outer = 1
    for d in outer_shape:
        outer *= d
    out = torch.empty(outer_shape, dtype=xs.dtype, device=xs.device)
    sp, _keep = _seed_ptr(tc, z)
    st = lib().acc_fold(op_of(f), tc, PRECS[prec], _ptr(xs), _ptr(out), outer, inner, sp, _stream(stream))
    _check(st, "fold")
    return out


def fold_zipwith(f, g, z, xs: torch.Tensor, ys: torch.Tensor, prec=None, stream=None) -> torch.Tensor:
    """fold f z (zipWith g xs ys) with the zipWith fused into the fold (the
    reference's delayed fold input, PTX/CodeGen/Fold.hs:80-97); z = None gives
    fold1.  dotp xs ys = fold_zipwith("+", "*", 0, xs, ys)."""
    xs, ys = _dev(xs), _dev(ys)
    if xs.shape != ys.shape or xs.dtype != ys.dtype:
        raise ValueError("zipWith of arrays of different shapes or types")
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1] if shape else 1
    outer_shape = shape[:-1]
    outer = 1
    for d in outer_shape:
        outer *= d
    out = torch.empty(outer_shape, dtype=xs.dtype, device=xs.device)
    sp, _keep = _seed_ptr(tc, z)
    st = lib().acc_fold_zipwith(op_of(f), op_of(g), tc, PRECS[prec], _ptr(xs), _ptr(ys), _ptr(out), outer, inner,
                                sp, _stream(stream))
    _check(st, "fold_zipwith")
    return out


def fold_map(f, g, c, z, xs: torch.Tensor, prec=None, stream=None) -> torch.Tensor:
    """fold f z (map (\\x -> g x c) xs) with the map fused into the fold (the
    reference's delayed fold input, PTX/CodeGen/Fold.hs:80-97); z = None gives
    fold1.  The reference's known answer sum (map (+1) xs) is
    fold_map("+", "+", 1, 0, xs)."""
    xs = _dev(xs)
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1] if shape else 1
    outer_shape = shape[:-1]
    outer = 1
    for d in outer_shape:
        outer *= d
    out = torch.empty(outer_shape, dtype=xs.dtype, device=xs.device)
    sp, _keep = _seed_ptr(tc, z)
    cp, _keep_c = _seed_ptr(tc, c)
    st = lib().acc_fold_map(op_of(f), op_of(g), tc, PRECS[prec], _ptr(xs), cp, _ptr(out), outer, inner, sp,
                            _stream(stream))
    _check(st, "fold_map")
    return out


def dotp(xs: torch.Tensor, ys: torch.Tensor, prec=None, stream=None) -> torch.Tensor:
    """dotp xs ys = fold (+) 0 (zipWith (*) xs ys)."""
    return fold_zipwith("+", "*", 0, xs, ys, prec=prec, stream=stream)


# ----------------------------------------------------------------- foldSeg
def fold_seg(f, z, xs: torch.Tensor, seg: torch.Tensor, prec=None, stream=None, offsets: bool = True):
    """foldSeg f z xs seg.  `seg` holds nseg+1 offsets (the reference's input after
    `scanl (+) 0`, PTX/Execute.hs:359) or, with offsets=False, nseg lengths."""
    return _fold_seg(f, z, xs, seg, prec, stream, offsets)


def fold1_seg(f, xs: torch.Tensor, seg: torch.Tensor, prec=None, stream=None, offsets: bool = True):
    return _fold_seg(f, None, xs, seg, prec, stream, offsets)


def _fold_seg(f, z, xs, seg, prec, stream, offsets):
    xs = _dev(xs)
    seg = _dev(seg)
    tc = type_of(xs)
    st_ = type_of(seg)
    shape = tuple(xs.shape)
    inner = shape[-1]
    outer = 1
    for d in shape[:-1]:
        outer *= d
    nseg = seg.numel() - 1 if offsets else seg.numel()
    out = torch.empty(shape[:-1] + (nseg,), dtype=xs.dtype, device=xs.device)
    sp, _keep = _seed_ptr(tc, z)
    fn = lib().acc_fold_seg if offsets else lib().acc_fold_seg_lengths
    _check(fn(op_of(f), tc, PRECS[prec], _ptr(xs), _ptr(seg), st_, _ptr(out), outer, inner, nseg, sp,
              _stream(stream)), "foldSeg")
    return out


def fold_seg_zipwith(f, g, z, xs: torch.Tensor, ys: torch.Tensor, seg: torch.Tensor, prec=None, stream=None):
    """foldSeg f z (zipWith g xs ys) seg with the zipWith fused into the
    segmented fold (acc_fold_seg_zipwith); z = None gives fold1Seg; `seg`
    holds nseg+1 offsets."""
    xs, ys, seg = _dev(xs), _dev(ys), _dev(seg)
    if xs.shape != ys.shape or xs.dtype != ys.dtype:
        raise ValueError("zipWith of arrays of different shapes or types")
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1]
    outer = 1
    for d in shape[:-1]:
        outer *= d
    nseg = seg.numel() - 1
    out = torch.empty(shape[:-1] + (nseg,), dtype=xs.dtype, device=xs.device)
    sp, _keep = _seed_ptr(tc, z)
    _check(lib().acc_fold_seg_zipwith(op_of(f), op_of(g), tc, PRECS[prec], _ptr(xs), _ptr(ys), _ptr(seg),
                                      type_of(seg), _ptr(out), outer, inner, nseg, sp, _stream(stream)),
           "foldSeg_zipwith")
    return out


# ----------------------------------------------------------------- scans
def _scan(f, z, xs, direction, kind, prec, stream):
    xs = _dev(xs)
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1]
    outer = 1
    for d in shape[:-1]:
        outer *= d
    out_inner = inner + 1 if kind == SCAN_SEEDED else inner
    out = torch.empty(shape[:-1] + (out_inner,), dtype=xs.dtype, device=xs.device)
    sums = torch.empty(shape[:-1], dtype=xs.dtype, device=xs.device) if kind == SCAN_PRIME else None
    sp, _keep = _seed_ptr(tc, z)
    st = lib().acc_scan(op_of(f), tc, PRECS[prec], direction, kind, _ptr(xs), _ptr(out),
                        _ptr(sums) if sums is not None else None, outer, inner, sp, _stream(stream))
    _check(st, "scan")
    return (out, sums) if kind == SCAN_PRIME else out


def scanl(f, z, xs, prec=None, stream=None):
    """scanl f z xs (output one longer, z first; PTX/Execute.hs:377-389)."""
    return _scan(f, z, xs, L2R, SCAN_SEEDED, prec, stream)


def scanl1(f, xs, prec=None, stream=None):
    return _scan(f, None, xs, L2R, SCAN_INCLUSIVE, prec, stream)


def scanr(f, z, xs, prec=None, stream=None):
    return _scan(f, z, xs, R2L, SCAN_SEEDED, prec, stream)


def scanr1(f, xs, prec=None, stream=None):
    return _scan(f, None, xs, R2L, SCAN_INCLUSIVE, prec, stream)


def scanl_(f, z, xs, prec=None, stream=None):
    """scanl' f z xs -> (exclusive scan, totals) (PTX/Execute.hs:491-512)."""
    return _scan(f, z, xs, L2R, SCAN_PRIME, prec, stream)


def scanr_(f, z, xs, prec=None, stream=None):
    return _scan(f, z, xs, R2L, SCAN_PRIME, prec, stream)


_SCAN_FLAVOURS = {"scanl": (L2R, SCAN_SEEDED), "scanl1": (L2R, SCAN_INCLUSIVE), "scanr": (R2L, SCAN_SEEDED),
                  "scanr1": (R2L, SCAN_INCLUSIVE), "scanl_": (L2R, SCAN_PRIME), "scanr_": (R2L, SCAN_PRIME)}


def scan_zipwith(flavour, f, g, z, xs: torch.Tensor, ys: torch.Tensor, prec=None, stream=None):
    """A scan of the fused producer zipWith g xs ys, e.g.
    scan_zipwith("scanl1", "+", "*", None, xs, ys) = scanl1 (+) (zipWith (*) xs ys).
    `flavour` names the scan as the functions above do (scanl, scanl1, scanr,
    scanr1, scanl_, scanr_); z is ignored by scanl1 / scanr1.  The zipped array
    is never written (acc_scan_zipwith)."""
    direction, kind = _SCAN_FLAVOURS[flavour]
    xs, ys = _dev(xs), _dev(ys)
    if xs.shape != ys.shape or xs.dtype != ys.dtype:
        raise ValueError("zipWith of arrays of different shapes or types")
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1]
    outer = 1
    for d in shape[:-1]:
        outer *= d
    out_inner = inner + 1 if kind == SCAN_SEEDED else inner
    out = torch.empty(shape[:-1] + (out_inner,), dtype=xs.dtype, device=xs.device)
    sums = torch.empty(shape[:-1], dtype=xs.dtype, device=xs.device) if kind == SCAN_PRIME else None
    sp, _keep = _seed_ptr(tc, None if kind == SCAN_INCLUSIVE else z)
    st = lib().acc_scan_zipwith(op_of(f), op_of(g), tc, PRECS[prec], direction, kind, _ptr(xs), _ptr(ys), _ptr(out),
                                _ptr(sums) if sums is not None else None, outer, inner, sp, _stream(stream))
    _check(st, "scan_zipwith")
    return (out, sums) if kind == SCAN_PRIME else out


def scan_map(flavour, f, g, c, z, xs: torch.Tensor, prec=None, stream=None):
    """A scan of the fused producer map (\\x -> g x c) xs, e.g.
    scan_map("scanl1", "+", "+", 1, None, xs) = scanl1 (+) (map (+1) xs).  The
    mapped array is never written (acc_scan_map)."""
    direction, kind = _SCAN_FLAVOURS[flavour]
    xs = _dev(xs)
    tc = type_of(xs)
    shape = tuple(xs.shape)
    inner = shape[-1]
    outer = 1
    for d in shape[:-1]:
        outer *= d
    out_inner = inner + 1 if kind == SCAN_SEEDED else inner
    out = torch.empty(shape[:-1] + (out_inner,), dtype=xs.dtype, device=xs.device)
    sums = torch.empty(shape[:-1], dtype=xs.dtype, device=xs.device) if kind == SCAN_PRIME else None
    sp, _keep = _seed_ptr(tc, None if kind == SCAN_INCLUSIVE else z)
    cp, _keep_c = _seed_ptr(tc, c)
    st = lib().acc_scan_map(op_of(f), op_of(g), tc, PRECS[prec], direction, kind, _ptr(xs), cp, _ptr(out),
                            _ptr(sums) if sums is not None else None, outer, inner, sp, _stream(stream))
    _check(st, "scan_map")
    return (out, sums) if kind == SCAN_PRIME else out


# ----------------------------------------------------------------- permute
def permute(f, defaults: torch.Tensor, idx: torch.Tensor, xs: Union[torch.Tensor, int, float, None] = None,
            n: Optional[int] = None, stream=None) -> torch.Tensor:
    """permute f defaults p xs with p given as a target-index array (negative =
    Nothing).  `xs` is a source array, or a scalar for a constant (fused fill)
    source of length n (default: len(idx))."""
    defaults = _dev(defaults)
    idx = _dev(idx)
    tc = type_of(defaults)
    it = type_of(idx)
    out = torch.empty_like(defaults)
    n_ = idx.numel() if n is None else n
    if isinstance(xs, torch.Tensor):
        xs = _dev(xs)
        if xs.dtype != defaults.dtype:
            raise TypeError("source and target element types differ")
        srcp, cvp, keep = _ptr(xs), None, None
    else:
        cvp, keep = _seed_ptr(tc, 1 if xs is None else xs)
        srcp = None
    st = lib().acc_permute_clone(op_of(f), tc, _ptr(defaults), srcp, cvp, _ptr(idx), it, _ptr(out), n_,
                                 defaults.numel(), _stream(stream))
    _check(st, "permute")
    return out


# ----------------------------------------------------------------- stencil
def stencil(weights: Sequence[Sequence[float]], xs: torch.Tensor, boundary="clamp", cval=None,
            stream=None) -> torch.Tensor:
    """stencil over a rank-1 or rank-2 array with a weighted-sum stencil
    function; weights is a (2ry+1) x (2rx+1) nested list (rank-1: one row)."""
    xs = _dev(xs)
    tc = type_of(xs)
    rows = [list(r) for r in weights]
    ky, kx = len(rows), len(rows[0])
    if ky % 2 == 0 or kx % 2 == 0 or any(len(r) != kx for r in rows):
        raise ValueError("stencil pattern must be odd-sized and rectangular")
    flat = [v for r in rows for v in r]
    warr = (_CTYPES[tc] * len(flat))(*flat)
    h, w = (1, xs.shape[0]) if xs.dim() == 1 else tuple(xs.shape)
    out = torch.empty_like(xs)
    b = BOUNDARIES[boundary] if isinstance(boundary, str) else boundary
    cvp, keep = _seed_ptr(tc, cval if cval is not None else 0)
    st = lib().acc_stencil2d(tc, ky // 2, kx // 2, ctypes.cast(warr, ctypes.c_void_p), b, cvp, _ptr(xs),
                             _ptr(out), h, w, _stream(stream))
    _check(st, "stencil")
    return out


def stencil3d(weights, xs: torch.Tensor, boundary="clamp", cval=None, stream=None) -> torch.Tensor:
    """stencil over a rank-3 array [planes][rows][columns] with a weighted-sum
    stencil function; weights is a (2rz+1) x (2ry+1) x (2rx+1) nested list
    (planes outer, as the reference's rank-3 patterns)."""
    xs = _dev(xs)
    if xs.dim() != 3:
        raise ValueError("stencil3d takes a rank-3 array")
    tc = type_of(xs)
    planes = [[list(r) for r in p] for p in weights]
    kz, ky, kx = len(planes), len(planes[0]), len(planes[0][0])
    if kz % 2 == 0 or ky % 2 == 0 or kx % 2 == 0 or any(len(p) != ky or any(len(r) != kx for r in p)
                                                         for p in planes):
        raise ValueError("stencil pattern must be odd-sized and rectangular")
    flat = [v for p in planes for r in p for v in r]
    warr = (_CTYPES[tc] * len(flat))(*flat)
    out = torch.empty_like(xs)
    b = BOUNDARIES[boundary] if isinstance(boundary, str) else boundary
    cvp, keep = _seed_ptr(tc, cval if cval is not None else 0)
    d, h, w = xs.shape
    st = lib().acc_stencil3d(tc, kz // 2, ky // 2, kx // 2, ctypes.cast(warr, ctypes.c_void_p), b, cvp, _ptr(xs),
                             _ptr(out), d, h, w, _stream(stream))
    _check(st, "stencil3d")
    return out


def stencil2(wa, wb, a: torch.Tensor, b: torch.Tensor, boundary_a="clamp", boundary_b="clamp", cval_a=None,
             cval_b=None, stream=None) -> torch.Tensor:
    """stencil2: weighted sums of two arrays' neighbourhoods over the
    intersection of their shapes (PTX/Execute.hs:669-684)."""
    a = _dev(a)
    b = _dev(b)
    tc = type_of(a)
    if type_of(b) != tc:
        raise TypeError("stencil2 inputs must share an element type here")
    ra, rb = [list(r) for r in wa], [list(r) for r in wb]
    ky, kx = len(ra), len(ra[0])
    if (len(rb), len(rb[0])) != (ky, kx):
        raise ValueError("both stencil patterns must have the same size")
    fa = (_CTYPES[tc] * (ky * kx))(*[v for r in ra for v in r])
    fb = (_CTYPES[tc] * (ky * kx))(*[v for r in rb for v in r])
    (ha, wa), (hb, wb) = [(1, t.shape[0]) if t.dim() == 1 else tuple(t.shape) for t in (a, b)]
    h, w = min(ha, hb), min(wa, wb)
    out = torch.empty((h, w) if a.dim() == 2 else (w,), dtype=a.dtype, device=a.device)
    ba = BOUNDARIES[boundary_a] if isinstance(boundary_a, str) else boundary_a
    bb = BOUNDARIES[boundary_b] if isinstance(boundary_b, str) else boundary_b
    ca, ka = _seed_ptr(tc, cval_a if cval_a is not None else 0)
    cb, kb = _seed_ptr(tc, cval_b if cval_b is not None else 0)
    st = lib().acc_stencil2d_pair(tc, ky // 2, kx // 2, ctypes.cast(fa, ctypes.c_void_p),
                                  ctypes.cast(fb, ctypes.c_void_p), ba, ca, bb, cb, _ptr(a), ha, wa, _ptr(b), hb, wb,
                                  _ptr(out), _stream(stream))
    _check(st, "stencil2")
    return out


# ----------------------------------------------------------------- batches
REQ_FOLD, REQ_SCAN = 0, 1


class Request(ctypes.Structure):
    """struct acc_request of acc_gb300.h."""
    _fields_ = [("kind", ctypes.c_int), ("type", ctypes.c_int), ("inp", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("n", ctypes.c_int64), ("has_seed", ctypes.c_int), ("seed", ctypes.c_uint64)]


def _seed_bits(type_code: int, value) -> int:
    c = _CTYPES[type_code](value)
    return int.from_bytes(bytes(c), "little")


class Batch:
    """Many fold / scanl1 requests in one persistent launch (acc_batch_*).

    `requests` is a list of (kind, xs, out, seed): kind "fold" (out: one
    element) or "scan" (out: len(xs) elements), seed None for fold1 /
    seedless scanl1.  Every request uses the primitive `f` ('+', 'min' or 'max')."""

    def __init__(self, f, requests):
        self._keep = []
        arr = (Request * max(1, len(requests)))()
        for i, (kind, xs, out, seed) in enumerate(requests):
            if kind not in ("fold", "scan"):
                raise ValueError(f"batch request {i}: kind {kind!r}, expected 'fold' or 'scan'")
            xs = _dev(xs)
            tc = type_of(xs)
            _given(out, 1 if kind == "fold" else xs.numel(), f"batch request {i} output", xs.dtype)
            self._keep += [xs, out]
            arr[i].kind = REQ_FOLD if kind == "fold" else REQ_SCAN
            arr[i].type = tc
            arr[i].inp = xs.data_ptr()
            arr[i].out = out.data_ptr() if out is not None else 0
            arr[i].n = xs.numel()
            arr[i].has_seed = 0 if seed is None else 1
            arr[i].seed = 0 if seed is None else _seed_bits(tc, seed)
        self._reqs = arr
        self._h = ctypes.c_void_p()
        _check(lib().acc_batch_create(op_of(f), ctypes.cast(arr, ctypes.c_void_p), len(requests),
                                      ctypes.byref(self._h)), "acc_batch_create")

    def capture(self, stream=None):
        _check(lib().acc_batch_capture(self._h, _stream(stream)), "acc_batch_capture")

    def launch(self, stream=None):
        _check(lib().acc_batch_launch(self._h, _stream(stream)), "acc_batch_launch")

    def status(self, stream=None):
        _check(lib().acc_batch_status(self._h, _stream(stream)), "acc_batch_status")

    def close(self):
        if self._h:
            lib().acc_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_autotune(table_path=None, stream=None):
    """Run the batch autotuner (acc_batch_autotune): threads per CTA and
    elements per thread per (kind, type, size bucket)."""
    _check(lib().acc_batch_autotune(table_path.encode() if table_path else None, _stream(stream)), "autotune")


def batch_load_tuning(table_path):
    _check(lib().acc_batch_load_tuning(str(table_path).encode()), "load tuning")


# ----------------------------------------------------------------- serving
SK_FOLD, SK_SCAN, SK_FOLDSEG, SK_PERMUTE, SK_STENCIL = range(5)
SKELETONS = {"fold": SK_FOLD, "scan": SK_SCAN, "foldseg": SK_FOLDSEG, "permute": SK_PERMUTE, "stencil": SK_STENCIL}


class ServeReq(ctypes.Structure):
    """struct acc_serve_req of acc_gb300.h."""
    _fields_ = [("skeleton", ctypes.c_int), ("type", ctypes.c_int), ("inp", ctypes.c_void_p),
                ("aux", ctypes.c_void_p), ("out", ctypes.c_void_p), ("n", ctypes.c_int64), ("m", ctypes.c_int64),
                ("arrival", ctypes.c_double), ("host_out", ctypes.c_void_p)]


class ServeStats(ctypes.Structure):
    _fields_ = [("wall_s", ctypes.c_double), ("served", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("max_inflight", ctypes.c_int64), ("peak_bytes", ctypes.c_int64)]


def serve(requests, budget_bytes: int, slots: int = 8, mode: str = "batching"):
    """Serve a request stream (acc_serve_run).  `requests`: list of
    (skeleton name, input tensor, aux tensor or None, output tensor or None,
    n, m, arrival seconds[, host array or None]), sorted by arrival.  A None
    output places the result in the loop's device arena of `budget_bytes`
    (admission waits until it fits); a host array (numpy or CPU tensor)
    receives a copy of the result.  Returns (latencies in seconds as a list,
    stats dict)."""
    arr = (ServeReq * max(1, len(requests)))()
    keep = []
    for i, req in enumerate(requests):
        sk, xs, aux, out, n, m, t = req[:7]
        host_out = req[7] if len(req) > 7 else None
        if sk not in SKELETONS:
            raise ValueError(f"request {i}: skeleton {sk!r}, expected one of {sorted(SKELETONS)}")
        if n < 0 or m < 0:
            raise ValueError(f"request {i}: negative extent")
        what = f"request {i} ({sk})"
        if sk == "permute":
            _given(xs, n, what + " indices", torch.int32)
            if out is not None:
                _given(out, m, what + " bins", torch.int32)
        else:
            _given(xs, n * m if sk == "stencil" else n, what + " input")
            if sk == "stencil" and xs.dtype not in (torch.float32, torch.float64):
                raise TypeError(f"{what}: the 5-point stencil takes Float32 / Float64 grids")
            if out is not None:
                _given(out, {"fold": 1, "scan": n, "foldseg": m, "stencil": n * m}[sk], what + " output", xs.dtype)
        if sk == "foldseg":
            _given(aux, m + 1, what + " offsets", torch.int32)
        esz = 4 if sk == "permute" else xs.element_size()
        nres = {"fold": 1, "scan": n, "foldseg": m, "permute": m, "stencil": n * m}[sk]
        if host_out is not None:
            haddr, hbytes = _host_buf(host_out)
            if hbytes < nres * esz:
                raise ValueError(f"{what}: host_out holds {hbytes} bytes, {nres * esz} needed")
            arr[i].host_out = haddr
        keep += [xs, aux, out, host_out]
        arr[i].skeleton = SKELETONS[sk]
        arr[i].type = type_of(xs) if sk != "permute" else I32
        arr[i].inp = xs.data_ptr()
        arr[i].aux = aux.data_ptr() if aux is not None else 0
        arr[i].out = out.data_ptr() if out is not None else 0
        arr[i].n = n
        arr[i].m = m
        arr[i].arrival = t
    lat = (ctypes.c_double * max(1, len(requests)))()
    stats = ServeStats()
    st = lib().acc_serve_run(ctypes.cast(arr, ctypes.c_void_p), len(requests), int(budget_bytes), slots,
                             0 if mode == "batching" else 1, ctypes.cast(lat, ctypes.c_void_p),
                             ctypes.cast(ctypes.pointer(stats), ctypes.c_void_p))
    _check(st, "acc_serve_run")
    return list(lat)[:len(requests)], {k: getattr(stats, k) for k, _ in ServeStats._fields_}


# ----------------------------------------------------------------- transfers and the memory table
def _host_buf(h):
    """(address, bytes) of a contiguous host array: a numpy array or a CPU
    tensor, pinned or pageable."""
    if isinstance(h, torch.Tensor):
        if h.is_cuda:
            raise ValueError("host arrays must be in host memory")
        if not h.is_contiguous():
            raise ValueError("host arrays must be contiguous")
        return h.data_ptr(), h.numel() * h.element_size()
    import numpy as np
    if not isinstance(h, np.ndarray):
        raise TypeError(f"unsupported host array {type(h).__name__}")
    if not h.flags["C_CONTIGUOUS"]:
        raise ValueError("host arrays must be contiguous")
    return h.ctypes.data, h.nbytes


def upload(dev: torch.Tensor, host, stream=None) -> None:
    """pokeArrayAsync on caller-owned device memory (acc_upload): enqueue the
    copy of the host array into `dev` on the stream."""
    addr, nbytes = _host_buf(host)
    if dev.numel() * dev.element_size() < nbytes or not dev.is_cuda or not dev.is_contiguous():
        raise ValueError("upload: the device array must be contiguous and hold the host array")
    _check(lib().acc_upload(_ptr(dev), ctypes.c_void_p(addr), nbytes, _stream(stream)), "acc_upload")


def download(host, dev: torch.Tensor, stream=None) -> None:
    """peekArrayAsync on caller-owned device memory (acc_download): enqueue the
    copy of `dev` into the host array on the stream (acc_sync before reading)."""
    addr, nbytes = _host_buf(host)
    if dev.numel() * dev.element_size() < nbytes or not dev.is_cuda or not dev.is_contiguous():
        raise ValueError("download: the device array must be contiguous and hold the host array")
    _check(lib().acc_download(ctypes.c_void_p(addr), _ptr(dev), nbytes, _stream(stream)), "acc_download")


class XferRecord(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("bytes", ctypes.c_int64), ("start_ms", ctypes.c_double),
                ("end_ms", ctypes.c_double)]


class TableStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int64) for n in ("budget", "resident_bytes", "arrays", "uploads", "upload_bytes",
                                              "downloads", "download_bytes", "hits", "evictions", "writebacks")]


class _DeviceView:
    """A device range of the table's arena, exposed to torch without a copy."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (ptr, False),
                                         "version": 3, "strides": None}


_TYPESTR = {torch.int32: "<i4", torch.int64: "<i8", torch.float32: "<f4", torch.float64: "<f8"}


def _typestr(h):
    """(typestr, shape) of the device view of a host array: its own element
    type and shape, or raw bytes for an element type outside the skeletons'."""
    if isinstance(h, torch.Tensor):
        if h.dtype in _TYPESTR:
            return _TYPESTR[h.dtype], tuple(h.shape)
        return "|u1", (h.numel() * h.element_size(),)
    return h.dtype.str, tuple(h.shape)


class Table:
    """The memory table (acc_table_*): device copies of host arrays in one
    device arena of `budget_bytes`, least recently used first out.

    Mirrors the reference's memory table and transfers
    (PTX/Array/Table.hs:35-49, PTX/Array/Remote.hs:60-133,
    PTX/Array/Prim.hs:72-195): ``use`` (useArrayAsync: upload unless
    resident), ``malloc`` (mallocArray: space for an output), ``poke`` /
    ``peek`` (pokeArrayAsync / peekArrayAsync), ``release`` (the end of a
    withRemote), ``wait`` and ``free`` (freeRemote).  ``use`` and ``malloc``
    return a CUDA tensor that views the device copy (no allocation, no copy);
    it is valid until the array is evicted, i.e. while held."""

    def __init__(self, budget_bytes: int):
        h = ctypes.c_void_p()
        _check(lib().acc_table_create(int(budget_bytes), ctypes.byref(h)), "acc_table_create")
        self._h = h

    def _view(self, ptr, host):
        typestr, shape = _typestr(host)
        return torch.as_tensor(_DeviceView(ptr.value or 0, shape, typestr), device=torch.device("cuda", torch.cuda.current_device()))

    def use(self, host, stream=None) -> torch.Tensor:
        addr, nbytes = _host_buf(host)
        p = ctypes.c_void_p()
        _check(lib().acc_table_use(self._h, ctypes.c_void_p(addr), nbytes, _stream(stream), ctypes.byref(p)),
               "acc_table_use")
        return self._view(p, host)

    def malloc(self, host, stream=None) -> torch.Tensor:
        addr, nbytes = _host_buf(host)
        p = ctypes.c_void_p()
        _check(lib().acc_table_malloc(self._h, ctypes.c_void_p(addr), nbytes, _stream(stream), ctypes.byref(p)),
               "acc_table_malloc")
        return self._view(p, host)

    def poke(self, host, stream=None) -> None:
        _check(lib().acc_table_poke(self._h, ctypes.c_void_p(_host_buf(host)[0]), _stream(stream)), "acc_table_poke")

    def peek(self, host, stream=None) -> None:
        _check(lib().acc_table_peek(self._h, ctypes.c_void_p(_host_buf(host)[0]), _stream(stream)), "acc_table_peek")

    def release(self, host, stream=None) -> None:
        _check(lib().acc_table_release(self._h, ctypes.c_void_p(_host_buf(host)[0]), _stream(stream)),
               "acc_table_release")

    def wait(self, host) -> None:
        _check(lib().acc_table_wait(self._h, ctypes.c_void_p(_host_buf(host)[0])), "acc_table_wait")

    def join(self, stream=None) -> None:
        """Make the stream wait for every transfer enqueued on the table so far."""
        _check(lib().acc_table_join(self._h, _stream(stream)), "acc_table_join")

    def free(self, host) -> None:
        _check(lib().acc_table_free(self._h, ctypes.c_void_p(_host_buf(host)[0])), "acc_table_free")

    def stats(self) -> dict:
        st = TableStats()
        _check(lib().acc_table_get_stats(self._h, ctypes.byref(st)), "acc_table_get_stats")
        return {n: getattr(st, n) for n, _ in TableStats._fields_}

    def trace(self, enable: bool = True) -> None:
        """Start (or stop) timing every transfer of the table; clears the trace."""
        _check(lib().acc_table_trace(self._h, 1 if enable else 0), "acc_table_trace")

    def trace_records(self, origin) -> list:
        """The traced transfers as (kind, bytes, start ms, end ms) after the
        `origin` event (a torch.cuda.Event with timing, recorded before them)."""
        cnt = ctypes.c_int64()
        _check(lib().acc_table_trace_get(self._h, ctypes.c_void_p(origin.cuda_event), None, 0, ctypes.byref(cnt)),
               "acc_table_trace_get")
        recs = (XferRecord * max(1, cnt.value))()
        _check(lib().acc_table_trace_get(self._h, ctypes.c_void_p(origin.cuda_event), recs, cnt.value,
                                         ctypes.byref(cnt)), "acc_table_trace_get")
        kinds = {0: "upload", 1: "download", 2: "copy back"}
        return [(kinds.get(r.kind, r.kind), r.bytes, r.start_ms, r.end_ms) for r in recs[:cnt.value]]

    def close(self) -> None:
        if getattr(self, "_h", None):
            h, self._h = self._h, None
            _check(lib().acc_table_destroy(h), "acc_table_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
