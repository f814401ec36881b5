"""CPU tests of the host-side mirror (accelerate-llvm_gb300/__init__.py): it
has no CPU fallback.  Every skeleton refuses host tensors with ValueError
before any library call, so nothing is ever computed on the host; combine
functions outside the fixed primitives and unsupported element types are
refused as the reference's shim refuses them (`internalError "unsupported
combine function"`); the buffers a caller hands to a batch or a serving run
are checked for place, layout, type and size before the device sees them."""
import numpy as np
import pytest
import torch


@pytest.fixture(scope="module")
def mirror():
    import __graft_entry__ as ge
    return ge.load_package()


def host(dtype=torch.float32, shape=(4, 8)):
    return torch.zeros(shape, dtype=dtype)


def calls(acc):
    x, i = host(), host(torch.int32, (8,))
    off = torch.tensor([0, 3, 8], dtype=torch.int32)
    x3 = host(shape=(2, 3, 4))
    return {
        "fold": lambda: acc.fold("+", 0.0, x),
        "fold1": lambda: acc.fold1("max", x),
        "fold_zipwith": lambda: acc.fold_zipwith("+", "*", 0.0, x, x),
        "dotp": lambda: acc.dotp(x, x),
        "fold_seg": lambda: acc.fold_seg("+", 0.0, x, off),
        "fold1_seg": lambda: acc.fold1_seg("min", x, off),
        "fold_seg_zipwith": lambda: acc.fold_seg_zipwith("+", "*", 0.0, x, x, off),
        "scanl": lambda: acc.scanl("+", 0.0, x),
        "scanl1": lambda: acc.scanl1("+", x),
        "scanr": lambda: acc.scanr("+", 0.0, x),
        "scanr1": lambda: acc.scanr1("+", x),
        "scanl_": lambda: acc.scanl_("+", 0.0, x),
        "scanr_": lambda: acc.scanr_("+", 0.0, x),
        "scan_zipwith": lambda: acc.scan_zipwith("scanl1", "+", "*", None, x, x),
        "permute": lambda: acc.permute("+", host(torch.int32, (16,)), i),
        "stencil": lambda: acc.stencil([[1.0, 1.0, 1.0]], x),
        "stencil3d": lambda: acc.stencil3d([[[1.0]]], x3),
        "stencil2": lambda: acc.stencil2([[1.0]], [[1.0]], x, x),
    }


SKELETONS = ["fold", "fold1", "fold_zipwith", "dotp", "fold_seg", "fold1_seg", "fold_seg_zipwith", "scanl",
             "scanl1", "scanr", "scanr1", "scanl_", "scanr_", "scan_zipwith", "permute", "stencil", "stencil3d",
             "stencil2"]


def test_every_skeleton_is_covered(mirror):
    assert sorted(calls(mirror)) == sorted(SKELETONS)


@pytest.mark.parametrize("name", SKELETONS)
def test_host_tensors_are_refused(mirror, name):
    with pytest.raises(ValueError, match="CUDA tensors"):
        calls(mirror)[name]()


@pytest.mark.parametrize("f", ["-", "/", "avg", lambda a, b: a + b])
def test_combine_functions_outside_the_primitives_are_refused(mirror, f):
    with pytest.raises(ValueError, match="unsupported combine function"):
        mirror.op_of(f)


def test_primitive_names(mirror):
    assert [mirror.op_of(f) for f in ["+", "*", "min", "max", "and", "or", "xor"]] == list(range(7))
    assert mirror.op_of(".&.") == mirror.AND and mirror.op_of(".|.") == mirror.OR


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16, torch.int8, torch.int16, torch.bool])
def test_element_types_outside_the_set_are_refused(mirror, dtype):
    with pytest.raises(TypeError, match="unsupported element type"):
        mirror.type_of(torch.zeros(2, dtype=dtype))


def test_element_type_codes_match_the_header(mirror):
    # acc_type in include/acc_gb300.h: I32 0, I64 1, U32 2, F32 3, F64 4
    assert [mirror.type_of(torch.zeros(1, dtype=d)) for d in (torch.int32, torch.int64, torch.float32,
                                                              torch.float64)] == [0, 1, 3, 4]
    if hasattr(torch, "uint32"):
        assert mirror.type_of(torch.zeros(1, dtype=torch.uint32)) == 2


def test_seed_is_passed_as_one_host_element(mirror):
    import ctypes
    for code, value in [(mirror.I32, -7), (mirror.I64, 1 << 40), (mirror.F32, 0.5), (mirror.F64, -2.25)]:
        p, keep = mirror._seed_ptr(code, value)
        got = ctypes.cast(p, ctypes.POINTER(mirror._CTYPES[code])).contents.value
        assert got == value and keep is not None
    assert mirror._seed_ptr(mirror.I32, None) == (None, None)
    assert np.float32(mirror._CTYPES[mirror.F32](0.1).value) == np.float32(0.1)


def test_batch_and_serve_refuse_host_tensors(mirror):
    x, out = host(torch.int32, (16,)), host(torch.int32, (1,))
    with pytest.raises(ValueError, match="CUDA tensors"):
        mirror.Batch("+", [("fold", x, out, None)])
    with pytest.raises(ValueError, match="CUDA tensors"):
        mirror.serve([("fold", x, None, out, 16, 0, 0.0)], 1 << 20)
    with pytest.raises(ValueError, match="kind"):
        mirror.Batch("+", [("scanr", x, out, None)])
    with pytest.raises(ValueError, match="skeleton"):
        mirror.serve([("map", x, None, out, 16, 0, 0.0)], 1 << 20)


class DeviceStub:
    """Stands in for a device tensor: the checks of caller-provided batch and
    serving buffers read only these attributes."""

    def __init__(self, numel, dtype=torch.float32, contiguous=True):
        self.is_cuda, self.dtype, self._n, self._c = True, dtype, numel, contiguous

    def numel(self):
        return self._n

    def is_contiguous(self):
        return self._c


def test_caller_buffers_are_checked_before_the_device_sees_them(mirror):
    # the library sees only an address: a short, mistyped or strided buffer
    # would be read or written out of bounds on the device
    g = mirror._given
    assert g(DeviceStub(10), 10, "out", torch.float32).numel() == 10
    with pytest.raises(ValueError, match="at least 11"):
        g(DeviceStub(10), 11, "out")
    with pytest.raises(TypeError, match="element type"):
        g(DeviceStub(10, torch.int32), 1, "out", torch.float32)
    with pytest.raises(ValueError, match="contiguous"):
        g(DeviceStub(10, contiguous=False), 1, "out")
    with pytest.raises(ValueError, match="CUDA tensors"):
        g(torch.zeros(10), 1, "out")


def test_serve_stencil_takes_float_grids(mirror):
    grid, out = DeviceStub(16, torch.int32), DeviceStub(16, torch.int32)
    with pytest.raises(TypeError, match="Float32 / Float64"):
        mirror.serve([("stencil", grid, None, out, 4, 4, 0.0)], 1 << 20)
