"""CPU tests of the C ABI: the library loads, exports every entry point the
header declares, and rejects bad arguments before touching the device."""
import ctypes
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "acc_gb300.h"


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    path = ge._load_build().build()
    pkg = ge.load_package()
    return pkg.load(path)


def declared():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(acc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    for n in ["acc_fold", "acc_fold_seg", "acc_scan", "acc_permute", "acc_stencil2d", "acc_sync"]:
        assert n in names


def test_every_declared_symbol_is_exported(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_python_signatures_cover_header(lib):
    import __graft_entry__ as ge
    pkg = ge.load_package()
    assert set(declared()) <= set(pkg.SIGNATURES)


def test_version_and_strerror(lib):
    assert lib.acc_version() == 1
    assert lib.acc_strerror(0) == b"ok"
    assert b"empty" in lib.acc_strerror(3)
    assert lib.acc_strerror(12345) == b"unknown status"


def test_argument_validation_without_device(lib):
    N = None
    # negative extents, bad enums, missing seeds: rejected before any CUDA call
    assert lib.acc_fold(0, 0, 0, N, N, -1, 4, N, N) == 1
    assert lib.acc_fold(0, 0, 0, N, ctypes.c_void_p(16), 2, 0, N, N) == 3  # fold1 of an empty row
    assert lib.acc_scan(0, 0, 0, 7, 0, N, N, N, 1, 4, N, N) == 1           # bad direction
    assert lib.acc_scan(0, 0, 0, 0, 1, N, N, N, 1, 4, N, N) == 1           # scanl without seed
    assert lib.acc_permute(0, 0, N, N, N, 0, N, 4, 4, N) == 1              # no source, no constant
    assert lib.acc_permute(0, 0, N, N, N, 9, N, 4, 4, N) == 1              # bad index type
    one = ctypes.c_void_p(16)
    assert lib.acc_permute_clone(0, 0, one, N, one, one, 9, one, 4, 4, N) == 1  # rejected before the clone
    assert lib.acc_permute_clone(0, 0, one, N, N, one, 0, one, 4, 4, N) == 1   # no source, no constant
    assert lib.acc_permute_clone(9, 0, one, N, one, one, 0, one, 4, 4, N) == 1   # no such primitive
    assert lib.acc_permute_clone(4, 3, one, N, one, one, 0, one, 4, 4, N) == 2   # .&. on Float32
    assert lib.acc_stencil2d(3, 5, 1, N, 0, N, N, N, 4, 4, N) == 1         # radius > 4
    assert lib.acc_stencil2d(2, 1, 1, N, 0, N, N, N, 4, 4, N) == 2         # Word32 stencil unsupported
    assert lib.acc_fold_seg(0, 0, 0, N, N, 3, N, 1, 4, 2, N, N) == 1       # bad offset type
    # the fused zipWith entry points
    out = ctypes.c_void_p(16)
    assert lib.acc_fold_zipwith(0, 9, 0, 0, N, N, out, 1, 4, N, N) == 1    # bad zip primitive
    assert lib.acc_fold_zipwith(0, 1, 0, 0, N, N, out, 2, 0, N, N) == 3    # fold1 of an empty row
    assert lib.acc_fold_zipwith(0, 1, 0, 0, N, N, out, 1, 4, N, N) == 1    # missing inputs
    assert lib.acc_scan_zipwith(0, 9, 0, 0, 0, 0, N, N, out, N, 1, 4, N, N) == 1  # bad zip primitive
    assert lib.acc_scan_zipwith(0, 1, 0, 0, 7, 0, N, N, out, N, 1, 4, N, N) == 1  # bad direction
    assert lib.acc_scan_zipwith(0, 1, 0, 0, 0, 1, N, N, out, N, 1, 4, N, N) == 1  # scanl without seed
    assert lib.acc_scan_zipwith(0, 1, 0, 0, 0, 0, N, N, out, N, 1, 4, N, N) == 1  # missing inputs
    assert lib.acc_scan_zipwith(0, 4, 0, 0, 0, 0, out, out, out, N, 1, 4, N, N) == 2  # zipWith (.&.) unsupported
    assert lib.acc_scan_zipwith(0, 1, 0, 0, 0, 2, out, out, out, N, 1, 4, out, N) == 1  # scanl' without sums
    assert lib.acc_fold_seg_zipwith(0, 9, 0, 0, out, out, out, 0, out, 1, 4, 2, N, N) == 1  # bad zip primitive
    assert lib.acc_fold_seg_zipwith(0, 1, 0, 0, out, out, out, 3, out, 1, 4, 2, N, N) == 1  # bad offset type
    assert lib.acc_fold_seg_zipwith(0, 1, 0, 0, out, N, out, 0, out, 1, 4, 2, N, N) == 1    # missing ys
    assert lib.acc_fold_seg_zipwith(1, 1, 0, 0, out, out, out, 0, out, 1, 4, 2, N, N) == 2  # fold op (*) unsupported
    assert lib.acc_fold_seg_zipwith(0, 5, 0, 0, out, out, out, 0, out, 1, 4, 2, N, N) == 2  # zipWith (.|.) unsupported
    assert lib.acc_fold_seg_zipwith(0, 1, 2, 0, out, out, out, 0, out, 1, 4, 2, N, N) == 2  # Word32 unsupported
    # the fused map entry points
    assert lib.acc_fold_map(0, 0, 0, 0, out, N, out, 1, 4, N, N) == 1      # no constant
    assert lib.acc_fold_map(0, 9, 0, 0, out, out, out, 1, 4, N, N) == 1    # bad map primitive
    assert lib.acc_fold_map(0, 0, 0, 0, out, out, out, 2, 0, N, N) == 3    # fold1 of an empty row
    assert lib.acc_scan_map(0, 0, 0, 0, 7, 0, out, out, out, N, 1, 4, N, N) == 1  # bad direction
    assert lib.acc_scan_map(0, 0, 0, 0, 0, 1, out, out, out, N, 1, 4, N, N) == 1  # scanl without seed
    assert lib.acc_scan_map(0, 0, 0, 0, 0, 0, out, N, out, N, 1, 4, N, N) == 1    # no constant
    assert lib.acc_scan_map(0, 4, 0, 0, 0, 0, out, out, out, N, 1, 4, N, N) == 2  # map (.&. c) unsupported
    # rank-3 stencils
    assert lib.acc_stencil3d(3, 5, 1, 1, out, 0, N, out, out, 4, 4, 4, N) == 1  # radius above 4
    assert lib.acc_stencil3d(3, 1, 1, 1, out, 3, N, out, out, 4, 4, 4, N) == 1  # constant without a value
    assert lib.acc_stencil3d(3, 1, 1, 1, out, 9, N, out, out, 4, 4, 4, N) == 1  # bad boundary
    assert lib.acc_stencil3d(2, 1, 1, 1, out, 0, N, out, out, 4, 4, 4, N) == 2  # Word32 unsupported
    assert lib.acc_stencil3d(3, 1, 1, 1, N, 0, N, out, out, 4, 4, 4, N) == 1   # no weights
    assert lib.acc_stencil3d(3, 1, 1, 1, N, 0, N, N, N, 0, 4, 4, N) == 0      # empty: nothing to do
    # serving requests, checked before the device is touched
    pkg = __import__("__graft_entry__").load_package()
    req = pkg.ServeReq(skeleton=pkg.SK_STENCIL, type=0, n=4, m=4)  # an Int32 grid
    lat = (ctypes.c_double * 1)()
    assert lib.acc_serve_run(ctypes.byref(req), 1, 1 << 20, 4, 0, lat, N) == 2   # 5-point weights need floats
    req.type = 9
    assert lib.acc_serve_run(ctypes.byref(req), 1, 1 << 20, 4, 0, lat, N) == 1   # bad element type
    req = pkg.ServeReq(skeleton=pkg.SK_FOLDSEG, type=3, inp=16, out=16, n=64, m=4)
    assert lib.acc_serve_run(ctypes.byref(req), 1, 1 << 20, 4, 0, lat, N) == 1   # foldSeg without offsets
    req = pkg.ServeReq(skeleton=pkg.SK_SCAN, type=3, out=16, n=64)
    assert lib.acc_serve_run(ctypes.byref(req), 1, 1 << 20, 4, 0, lat, N) == 1   # scan without input
    breq = pkg.Request(kind=pkg.REQ_FOLD, type=0, n=0, has_seed=1)                # fold z [] without output
    h = ctypes.c_void_p()
    assert lib.acc_batch_create(0, ctypes.byref(breq), 1, ctypes.byref(h)) == 1
    # transfers and the memory table
    assert lib.acc_upload(out, out, -1, N) == 1                                   # negative size
    assert lib.acc_upload(N, out, 8, N) == 1                                      # no device buffer
    assert lib.acc_download(out, N, 8, N) == 1                                    # no device buffer
    assert lib.acc_upload(N, N, 0, N) == 0                                        # nothing to copy
    assert lib.acc_table_create(0, ctypes.byref(h)) == 1                          # no budget
    assert lib.acc_table_create(1 << 20, N) == 1                                  # nowhere to put it
    p = ctypes.c_void_p()
    assert lib.acc_table_use(N, out, 8, N, ctypes.byref(p)) == 1                  # no table
    assert lib.acc_table_malloc(N, out, 8, N, ctypes.byref(p)) == 1
    for f in (lib.acc_table_poke, lib.acc_table_peek, lib.acc_table_release):
        assert f(N, out, N) == 1
    assert lib.acc_table_wait(N, out) == 1
    assert lib.acc_table_free(N, out) == 1
    assert lib.acc_table_destroy(N) == 1
    assert lib.acc_table_join(N, N) == 1
    assert lib.acc_table_get_stats(N, N) == 1
    assert lib.acc_table_trace(N, 1) == 1
    assert lib.acc_table_trace_get(N, out, N, 0, N) == 1
    assert lib.acc_selftest_timeout(7, N) == 1                                    # no such wait


def test_batch_tuning_table_loader(lib, tmp_path):
    """The autotuner table's loader (no device work): entries of five numbers
    (elements per thread, threads per CTA) or four (256 threads); a launch
    shape other than 128 / 256 / 512 threads, a file without entries or no
    file are rejected."""
    p = tmp_path / "tune.json"
    p.write_text('{"gpu": "x", "entries": [[0, 0, 10, 4, 128], [1, 3, 12, 8, 512], [1, 4, 9, 2]]}')
    assert lib.acc_batch_load_tuning(str(p).encode()) == 0
    p.write_text('{"gpu": "x", "entries": [[0, 0, 10, 4, 300]]}')
    assert lib.acc_batch_load_tuning(str(p).encode()) == 1
    p.write_text('{"gpu": "x"}')
    assert lib.acc_batch_load_tuning(str(p).encode()) == 1
    assert lib.acc_batch_load_tuning(str(tmp_path / "missing.json").encode()) == 1
    assert lib.acc_batch_load_tuning(None) == 1


def test_c_caller_links_and_validates(lib, tmp_path):
    """The header compiles as strict C99 and a C program linked against the
    library by name gets the same answers as the ctypes calls above (a
    Haskell cbits binding is such a C caller)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    libdir = ROOT / "accelerate-llvm_gb300"
    exe = tmp_path / "abi_from_c"
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "abi_from_c.c"), f"-L{libdir}", "-laccgb", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("0 failed")
