"""scanl / scanl1 / scanr / scanr1 / scanl' / scanr' on the GPU against the
oracle (PTX/Execute.hs:377-594; Native/CodeGen/Scan.hs:136-270)."""
import numpy as np
import pytest
import torch

from helpers import COMBOS, TYPES, _diff, case_rng, gen, seed_for

pytestmark = pytest.mark.gpu

# (direction, kind): 0 L2R / 1 R2L; 0 inclusive, 1 seeded (n+1), 2 prime (+ sums)
FLAVOURS = [(0, 0), (1, 0), (0, 1), (1, 1), (0, 2), (1, 2)]
NAMES = {(0, 0): "scanl1", (1, 0): "scanr1", (0, 1): "scanl", (1, 1): "scanr", (0, 2): "scanl_", (1, 2): "scanr_"}


def gpu_scan(acc, op, z, td, d, k):
    fn = getattr(acc, NAMES[(d, k)])
    return fn(op, td) if k == 0 else fn(op, z, td)


def check_scan(orc, got, xs, dt, op, z, d, k):
    dt = np.dtype(dt)
    ref = orc.scan(op, None if k == 0 else dt.type(z), xs, d, k)
    if k == 2:
        got_out, got_sum = got
        ref_out, ref_sum = ref
    else:
        got_out, ref_out = got, ref
    if dt.kind in "iu" or op in ("min", "max", "*"):
        assert np.array_equal(got_out, ref_out) or (dt.kind == "f" and _nan_equal(got_out, ref_out)), _diff(got_out, ref_out)
        if k == 2:
            assert np.array_equal(got_sum, ref_sum) or _nan_equal(got_sum, ref_sum)
        return
    r64 = orc.scan_f64(op, None if k == 0 else float(z), xs, d, k)
    a64 = orc.scan_f64("+", None if k == 0 else abs(float(z)), np.abs(xs), d, k) if op == "+" else None
    pairs = [(got_out, r64[0] if k == 2 else r64, a64[0] if (k == 2 and a64 is not None) else a64)]
    if k == 2:
        pairs.append((got_sum, r64[1], a64[1] if a64 is not None else None))
    for g, r, a in pairs:
        g = np.asarray(g, dtype=np.float64)
        if op == "+":
            tol = (1e-6 * np.abs(r) + 1e-9 * a) if dt == np.float32 else (1e-12 * a + 1e-15 * np.abs(r))
            err = np.abs(g - r)
            assert np.all(err <= tol + 1e-30), f"max excess {(err - tol).max()}"
        else:
            assert np.allclose(g, r, rtol=2e-5 if dt == np.float32 else 1e-13, atol=0)


def _nan_equal(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def run_scan(acc, orc, dev, t, op, shape, d, k, offset=0):
    dt = TYPES[t]
    rng = case_rng("scan", t, op, shape, d, k, offset)
    n = int(np.prod(shape))
    x = gen(dt, op, n + offset, rng)
    xs = x[offset:].reshape(shape)
    z = seed_for(dt, op)
    td = torch.from_numpy(x).to(dev)[offset:].view(shape)
    got = gpu_scan(acc, op, z, td, d, k)
    acc.sync()
    got = tuple(g.cpu().numpy() for g in got) if k == 2 else got.cpu().numpy()
    check_scan(orc, got, xs, dt, op, z, d, k)


@pytest.mark.parametrize("t,op", COMBOS)
@pytest.mark.parametrize("d,k", FLAVOURS)
def test_scan_grid(acc, orc, dev, t, op, d, k):
    run_scan(acc, orc, dev, t, op, (10_007,), d, k)


SIZES = [1, 2, 31, 4095, 4096, 4097, 8191, 8192, 8193, 100_003, (1 << 20) + 5]


@pytest.mark.parametrize("t,op", [("i32", "+"), ("i64", "+"), ("f32", "+"), ("f64", "max"), ("u32", "xor")])
@pytest.mark.parametrize("n", SIZES)
def test_scan_sizes(acc, orc, dev, t, op, n):
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, (n,), d, k)


# Arrays of hundreds of tiles: look-backs that span several windows, a
# partial last tile, and a tile count that is a multiple of the SM count.
@pytest.mark.parametrize("t,op,n", [("i32", "+", (1 << 23) + 3), ("i32", "+", 608 * 8192), ("u32", "xor", 1 << 23),
                                    ("i64", "+", (1 << 22) + 5), ("f32", "+", (1 << 23) + 1), ("f64", "max", 3 << 20)])
def test_scan_large_sizes(acc, orc, dev, t, op, n):
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, (n,), d, k)


@pytest.mark.parametrize("t,op", [("i32", "+"), ("f32", "+"), ("i64", "max"), ("f64", "+")])
@pytest.mark.parametrize("shape", [(3, 1000), (1000, 3), (2, 9000), (64, 1), (5, 4096)])
def test_scan_rows(acc, orc, dev, t, op, shape):
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, shape, d, k)


@pytest.mark.parametrize("t,op", [("i32", "+"), ("f32", "+"), ("i64", "max"), ("f64", "+"), ("u32", "xor")])
@pytest.mark.parametrize("shape", [(9728, 33), (10_000, 1), (9728, 300), (9728, 512), (12_000, 2048)])
def test_scan_many_short_rows(acc, orc, dev, t, op, shape):
    # Many rows: up to 512 elements one warp per row, longer ones one CTA per row.
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, shape, d, k)


# scanl1 / scanr1 over rows of arrays of at least four 32 KiB tiles per SM:
# one segmented pass of the persistent kernel over the whole array.  Rows
# longer than a tile (look-backs within a row), rows a whole number of tiles
# long (tiles that begin with a row: no look-back), many rows per tile, and
# row lengths that are not a whole number of 128-byte lines (a row start in
# the middle of a thread's line).
@pytest.mark.parametrize("t,op,shape", [("i64", "+", (64, 1 << 18)), ("i64", "+", (1 << 16, 256)),
                                        ("i64", "max", (1024, 1 << 14)), ("i32", "+", (160_000, 37)),
                                        ("f32", "+", (1000, 5003)), ("f64", "min", (4097, 1000)),
                                        ("i32", "*", (2000, 4099)), ("u32", "max", (3, 2_000_003))])
def test_scan_rows_segmented(acc, orc, dev, t, op, shape):
    # scanl1 / scanr1, scanl z / scanr z (every row from the seed, output rows
    # one element longer) and scanl' / scanr' (the row totals in a second array)
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, shape, d, k)


@pytest.mark.parametrize("offset", [1, 3])
@pytest.mark.parametrize("t,op", [("i32", "+"), ("i64", "+"), ("f32", "+")])
def test_scan_unaligned(acc, orc, dev, t, op, offset):
    for d, k in FLAVOURS:
        run_scan(acc, orc, dev, t, op, (50_001,), d, k, offset=offset)


def test_scan_known_answer(acc, dev):
    # scanl (+) 10 [0..9] (Native/CodeGen/Scan.hs:50-56)
    xs = torch.arange(10, dtype=torch.int64, device=dev)
    assert acc.scanl("+", 10, xs).cpu().tolist() == [10, 10, 11, 13, 16, 20, 25, 31, 38, 46, 55]
    # mkScan's scanl' example (Native/CodeGen/Scan.hs:78-85)
    out, tot = acc.scanl_("+", 10, xs)
    assert out.cpu().tolist() == [10, 10, 11, 13, 16, 20, 25, 31, 38, 46] and int(tot.item()) == 55
    out, tot = acc.scanr_("+", 10, xs)
    assert out.cpu().tolist() == [55, 54, 52, 49, 45, 40, 34, 27, 19, 10] and int(tot.item()) == 55


def test_scan_empty(acc, dev):
    e = torch.empty(0, dtype=torch.int32, device=dev)
    assert acc.scanl("+", 4, e).cpu().tolist() == [4]
    assert acc.scanr("+", 4, e).cpu().tolist() == [4]
    assert acc.scanl1("+", e).numel() == 0
    out, tot = acc.scanl_("+", 4, e)
    assert out.numel() == 0 and int(tot.item()) == 4
    e2 = torch.empty((3, 0), dtype=torch.int64, device=dev)
    assert acc.scanl("+", 9, e2).cpu().tolist() == [[9], [9], [9]]


@pytest.mark.parametrize("n", [300_001, (1 << 22) + 1])
def test_scan_in_place(acc, orc, dev, n):
    rng = np.random.default_rng(5)
    x = rng.integers(-100, 100, size=n).astype(np.int64)
    td = torch.from_numpy(x).to(dev)
    st = acc.lib().acc_scan(0, 1, 0, 0, 0, acc._ptr(td), acc._ptr(td), None, 1, td.numel(), None, acc._stream())
    assert st == 0
    acc.sync()
    assert np.array_equal(td.cpu().numpy(), np.cumsum(x))


def test_scan_repeated_calls_reuse_workspace(acc, dev):
    x = torch.randint(-5, 5, (1 << 21,), dtype=torch.int32, device=dev)
    ref = torch.cumsum(x.long(), 0).int().cpu()
    for _ in range(5):
        assert torch.equal(acc.scanl1("+", x).cpu(), ref)
    acc.sync()
