"""GPU: the allocation-free product entry point against the regular one.

``tm_perform_op_dev_noalloc`` serves callers that must not allocate device
memory at call time: code inside a framework whose caching allocator owns the
GPU's memory, or a latency-bound loop that cannot afford the synchronisation
an allocation brings.  It runs the FP64 even/odd reduced x-ANNNI product with
its scratch in a fixed device array inside the library.  Here it is called
through the C ABI, twice in a row with different inputs (the array keeps the
previous call's contents), and each result is compared with
``tm_perform_op_dev`` (TM_F64) on the same input, within the 1e-12 relative
bar of the FP64 product tests.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import latttmat_gb300 as lt

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

# (L, extend_cond): flip reduction on/off; L=24 is the largest that fits
CASES = [(12, 0), (16, 2), (20, 2), (24, 2)]


def _noalloc(lib):
    fn = lib.tm_perform_op_dev_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _call(fn, op, x, y):
    code = fn(op._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), None)
    if code != lt.TM_OK:
        raise lt.TMError(code, lt.load_library().tm_last_error().decode(errors="replace"))


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("L,ec", CASES)
def test_noalloc_matches_regular_product(L, ec):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = lt.load_library()
    fn = _noalloc(lib)
    op = lt.TMatOp("A", 2, 5, 0.3, 0.6, 0.0, L, 0.0, ec)
    n = op.rows()
    gen = torch.Generator().manual_seed(1000 + L)
    xs = [(torch.rand(n, generator=gen, dtype=torch.float64) - 0.5).cuda() for _ in range(2)]
    torch.cuda.synchronize()  # the products below run on the library's stream
    refs = []
    for x in xs:
        y = torch.empty_like(x)
        op.perform_op_dev(x.data_ptr(), y.data_ptr(), lt.TM_F64)
        refs.append(y)
    torch.cuda.synchronize()
    outs = [torch.full_like(x, float("nan")) for x in xs]
    torch.cuda.synchronize()
    for x, y in zip(xs, outs):  # two calls in a row, sharing the scratch
        _call(fn, op, x, y)
    torch.cuda.synchronize()
    for y, ref in zip(outs, refs):
        assert bool(torch.isfinite(y).all())
        assert _rel(y, ref) < 1e-12
    # no allocation per call: the library's allocation counter (every device
    # buffer it makes goes through one allocator) does not move, and neither
    # does the device's free memory (this assumes no other process allocates
    # on the same GPU meanwhile)
    allocs0 = lt.alloc_count()
    free0 = torch.cuda.mem_get_info()[0]
    for x, y in zip(xs, outs):
        _call(fn, op, x, y)
    torch.cuda.synchronize()
    assert lt.alloc_count() == allocs0
    assert torch.cuda.mem_get_info()[0] == free0
    for y, ref in zip(outs, refs):
        assert _rel(y, ref) < 1e-12
    op.close()


def test_noalloc_rejects_what_it_cannot_hold():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    fn = _noalloc(lt.load_library())
    big = lt.TMatOp("A", 2, 5, 0.3, 0.6, 0.0, 26, 0.0, 2)
    x = torch.zeros(big.rows(), dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    with pytest.raises(lt.TMError) as e:
        _call(fn, big, x, y)
    assert e.value.code == lt.TM_ERR_LIMIT
    big.close()
    other = lt.TMatOp("A", 2, 1, 0.3, 0.6, 0.0, 10, 0.0, 0)  # full-space operator
    x = torch.zeros(other.rows(), dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    with pytest.raises(lt.TMError) as e:
        _call(fn, other, x, y)
    assert e.value.code == lt.TM_ERR_UNSUPPORTED
    other.close()
