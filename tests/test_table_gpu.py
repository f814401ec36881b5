"""Host <-> device transfers and the memory table on the GPU
(acc_upload / acc_download, acc_table_*), against the host data itself and,
for skeletons run on table arrays, against the oracle.

The reference's counterparts: useArrayAsync / mallocArray / pokeArrayAsync /
peekArrayAsync (PTX/Array/Prim.hs:72-195), the memory table with its LRU
eviction (PTX/Array/Table.hs:35-49, PTX/Array/Remote.hs:60-133) and the copy
back of results (PTX/Array/Data.hs:91-148)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MiB = 1 << 20


def _host(kind, nbytes, rng, offset=0):
    """A host byte array of `nbytes` at `offset` bytes into its allocation:
    pageable numpy memory, or a pinned torch tensor."""
    data = rng.integers(0, 256, size=nbytes + offset, dtype=np.uint8)
    if kind == "pageable":
        return data[offset:]
    t = torch.from_numpy(data).pin_memory()
    return t[offset:]


def _np(h):
    return h.numpy() if isinstance(h, torch.Tensor) else h


@pytest.mark.parametrize("kind", ["pageable", "pinned"])
@pytest.mark.parametrize("nbytes", [1, 15, 16, 17, 4095, MiB + 3, 64 * MiB + 5])
@pytest.mark.parametrize("hoff,doff", [(0, 0), (3, 3), (1, 0), (8, 4)])
def test_upload_download_round_trip(acc, dev, kind, nbytes, hoff, doff):
    rng = np.random.default_rng(nbytes * 31 + hoff * 7 + doff)
    src = _host(kind, nbytes, rng, hoff)
    d = torch.full((nbytes + doff,), 0xAB, dtype=torch.uint8, device=dev)
    dv = d[doff:]
    acc.upload(dv, src)
    acc.sync()
    assert np.array_equal(dv.cpu().numpy(), _np(src))
    assert int(d[:doff].sum()) == 0xAB * doff  # nothing written before the range
    back = _host(kind, nbytes, np.random.default_rng(1), hoff)
    back_np = _np(back)
    back_np[:] = 0
    acc.download(back, dv)
    acc.sync()
    assert np.array_equal(back_np, _np(src))


def test_upload_zero_bytes(acc, dev):
    d = torch.zeros(4, dtype=torch.uint8, device=dev)
    acc.upload(d, np.zeros(0, dtype=np.uint8))
    acc.sync()
    assert int(d.sum()) == 0


@pytest.mark.parametrize("kind", ["pageable", "pinned"])
def test_table_use_is_uploaded_once(acc, dev, kind):
    rng = np.random.default_rng(2)
    h = _host(kind, 3 * MiB + 8, rng)
    tb = acc.Table(16 * MiB)
    try:
        v = tb.use(h)
        assert np.array_equal(v.cpu().numpy(), _np(h))
        tb.release(h)
        v2 = tb.use(h)
        assert v2.data_ptr() == v.data_ptr()
        tb.release(h)
        st = tb.stats()
        assert st["uploads"] == 1 and st["hits"] == 1 and st["arrays"] == 1
        assert st["upload_bytes"] == 3 * MiB + 8
        # the host array changes: poke copies it again
        _np(h)[:] = 7
        tb.poke(h)
        torch.cuda.current_stream().synchronize()
        assert np.array_equal(v.cpu().numpy(), _np(h))
        assert tb.stats()["uploads"] == 2
    finally:
        tb.close()


@pytest.mark.parametrize("kind", ["pageable", "pinned"])
def test_table_malloc_peek_copies_back(acc, dev, kind):
    rng = np.random.default_rng(3)
    h = _host(kind, 2 * MiB, rng)
    want = rng.integers(0, 256, size=2 * MiB, dtype=np.uint8)
    tb = acc.Table(8 * MiB)
    try:
        v = tb.malloc(h)
        v.copy_(torch.from_numpy(want).to(dev))  # the device writes the output
        tb.release(h)
        tb.peek(h)
        tb.wait(h)
        assert np.array_equal(_np(h), want)
        assert tb.stats()["downloads"] == 1
    finally:
        tb.close()


def test_table_lru_eviction_and_write_back(acc, dev):
    rng = np.random.default_rng(4)
    tb = acc.Table(8 * MiB)  # room for two 3 MiB arrays
    try:
        a, b, c = (rng.integers(0, 256, size=3 * MiB, dtype=np.uint8) for _ in range(3))
        out = np.zeros(3 * MiB, dtype=np.uint8)
        va = tb.use(a)
        tb.release(a)
        vo = tb.malloc(out)  # an output the device writes and nobody peeks
        vo.fill_(5)
        tb.release(out)
        # a is the least recently used: c takes its place
        vc = tb.use(c)
        tb.release(c)
        st = tb.stats()
        assert st["evictions"] == 1 and st["writebacks"] == 0
        assert np.array_equal(vc.cpu().numpy(), c)
        # now the written output is the least recently used: evicting it
        # copies it back to its host array first
        vb = tb.use(b)
        tb.release(b)
        st = tb.stats()
        assert st["evictions"] == 2 and st["writebacks"] == 1
        torch.cuda.synchronize()
        assert np.all(out == 5)
        assert np.array_equal(vb.cpu().numpy(), b)
        # a comes back: uploaded again, same bytes
        va = tb.use(a)
        tb.release(a)
        assert np.array_equal(va.cpu().numpy(), a)
        assert tb.stats()["uploads"] == 4
    finally:
        tb.close()


def test_table_held_arrays_are_never_evicted(acc, dev):
    rng = np.random.default_rng(5)
    tb = acc.Table(8 * MiB)
    try:
        a, b, c = (rng.integers(0, 256, size=3 * MiB, dtype=np.uint8) for _ in range(3))
        tb.use(a)
        tb.use(b)
        with pytest.raises(acc.AccError) as ei:
            tb.use(c)
        assert ei.value.status == 5  # ACC_ERR_NOMEM
        with pytest.raises(acc.AccError):
            tb.free(a)  # held
        tb.release(a)
        vc = tb.use(c)  # a is released: it goes
        assert np.array_equal(vc.cpu().numpy(), c)
        tb.release(b)
        tb.release(c)
        with pytest.raises(acc.AccError):
            tb.release(c)  # not held any more
        tb.free(b)
        assert tb.stats()["arrays"] == 1
    finally:
        tb.close()


def test_table_too_large_for_budget(acc, dev):
    tb = acc.Table(2 * MiB)
    try:
        with pytest.raises(acc.AccError) as ei:
            tb.use(np.zeros(3 * MiB, dtype=np.uint8))
        assert ei.value.status == 5
    finally:
        tb.close()


def test_destroy_copies_back_written_arrays(acc, dev):
    out = np.zeros(MiB, dtype=np.int32)
    tb = acc.Table(8 * MiB)
    v = tb.malloc(out)
    v.fill_(-3)
    tb.release(out)
    tb.close()
    assert np.all(out == -3)


@pytest.mark.parametrize("kind", ["pageable", "pinned"])
def test_scan_through_the_table(acc, orc, dev, kind):
    """useArrayAsync -> scanl1 on the device copies -> peekArrayAsync, for
    several steps whose host input changes (poke), against the oracle."""
    lib = acc.lib()
    rng = np.random.default_rng(6)
    n = (1 << 22) + 5
    if kind == "pageable":
        hin, hout = np.zeros(n, dtype=np.int64), np.zeros(n, dtype=np.int64)
        hin_np, hout_np = hin, hout
    else:
        hin, hout = torch.zeros(n, dtype=torch.int64).pin_memory(), torch.zeros(n, dtype=torch.int64).pin_memory()
        hin_np, hout_np = hin.numpy(), hout.numpy()
    tb = acc.Table(256 * MiB)
    stream = torch.cuda.Stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    try:
        for step in range(3):
            hin_np[:] = rng.integers(-(1 << 20), 1 << 20, size=n)
            with torch.cuda.stream(stream):
                vin = tb.use(hin, stream)  # uploaded on the first step, resident after
                if step > 0:
                    tb.poke(hin, stream)  # the host input changed
                vout = tb.malloc(hout, stream)
            st = lib.acc_scan(acc.ADD, acc.I64, 0, 0, 0, ctypes.c_void_p(vin.data_ptr()),
                              ctypes.c_void_p(vout.data_ptr()), None, 1, n, None, sp)
            assert st == 0
            tb.release(hin, stream)
            tb.release(hout, stream)
            tb.peek(hout, stream)
            tb.wait(hout)
            acc.sync(stream)
            assert np.array_equal(hout_np, orc.scan("+", None, hin_np, 0, 0)), f"step {step}"
        s = tb.stats()
        assert s["uploads"] == 3 and s["downloads"] == 3 and s["hits"] == 2
    finally:
        tb.close()
