"""The NLBlas function table (nlHostBlas / nlCUDABlas) on the GPU: every
entry -- Dcopy, Dscal, Ddot, Dnrm2, Daxpy, Dmul -- called through the table's
function pointers, with host and with device vectors, unit, strided and
negative increments, against numpy.

Reference callers: src/lib/OGF/scene_graph/NL/blas.cpp:86 (copy), :96 (scal),
:106 (dot), :125 (nrm2), :135 (axpy) forward to these entries of the table
that nlHostBlas() / nlCUDABlas() return.

Tolerances: copy and scal are exact; axpy and mul are one rounding per
element (FMA on the GPU, numpy rounds the product and the sum separately:
within one ulp of |a x| + |y|); dot and nrm2 sum in a different order than
numpy: within 1e-13 relative to sum |x_i y_i|."""
import ctypes
import time

import numpy as np
import pytest

from graphitethree_gb300 import _lib

pytestmark = pytest.mark.gpu

V = ctypes.c_void_p
F = ctypes.CFUNCTYPE
COPY = F(None, V, ctypes.c_int, V, ctypes.c_int, V, ctypes.c_int)
SCAL = F(None, V, ctypes.c_int, ctypes.c_double, V, ctypes.c_int)
DOT = F(ctypes.c_double, V, ctypes.c_int, V, ctypes.c_int, V, ctypes.c_int)
NRM2 = F(ctypes.c_double, V, ctypes.c_int, V, ctypes.c_int)
AXPY = F(None, V, ctypes.c_int, ctypes.c_double, V, ctypes.c_int, V, ctypes.c_int)
MUL = F(None, V, ctypes.c_int, V, V)


class BlasStruct(ctypes.Structure):
    """struct NLBlas (include/nl.h): six function pointers, then the
    unified-memory flag and the flop counter."""
    _fields_ = [("fn", ctypes.c_void_p * 6), ("has_unified_memory", ctypes.c_ubyte),
                ("flops", ctypes.c_double), ("used_ram", ctypes.c_longlong * 2),
                ("max_used_ram", ctypes.c_longlong * 2)]


class Table:
    """The NLBlas struct's leading function pointers, in declaration order."""

    def __init__(self, tbl):
        p = ctypes.cast(tbl, ctypes.POINTER(ctypes.c_void_p))
        self.tbl = tbl
        self.copy, self.scal, self.dot = COPY(p[0]), SCAL(p[1]), DOT(p[2])
        self.nrm2, self.axpy, self.mul = NRM2(p[3]), AXPY(p[4]), MUL(p[5])


@pytest.fixture(scope="module")
def blas(gpu_ok):
    L = _lib.load()
    return Table(L.nlHostBlas())


def logical(buf, n, inc):
    """The n-vector a BLAS routine sees in `buf` with increment `inc`."""
    v = buf[::abs(inc)][:n]
    return v if inc > 0 else v[::-1]


def span(n, inc):
    return 1 + (n - 1) * abs(inc)


class Mem:
    """A host (numpy) or device (torch) buffer, with its address for the table."""

    def __init__(self, arr, where):
        self.where = where
        if where == "host":
            self.a = np.array(arr, dtype=np.float64)
        else:
            import torch
            self.a = torch.tensor(arr, dtype=torch.float64, device="cuda")

    @property
    def ptr(self):
        return V(self.a.ctypes.data if self.where == "host" else self.a.data_ptr())

    def numpy(self):
        return self.a.copy() if self.where == "host" else self.a.cpu().numpy()


CASES = [(1, 1), (3, 2), (-2, 1), (2, -3), (-1, -1)]


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("incx,incy", CASES)
def test_copy_scal_axpy(blas, where, incx, incy):
    rng = np.random.default_rng(abs(incx) * 10 + abs(incy))
    n = 10_007
    xb = rng.standard_normal(span(n, incx))
    yb = rng.standard_normal(span(n, incy))
    # Dcopy: only the strided elements of y change
    x, y = Mem(xb, where), Mem(yb, where)
    blas.copy(blas.tbl, n, x.ptr, incx, y.ptr, incy)
    exp = yb.copy()
    logical(exp, n, incy)[:] = logical(xb, n, incx)
    assert np.array_equal(y.numpy(), exp)
    assert np.array_equal(x.numpy(), xb)
    # Dscal: x_i *= a, exactly one rounding
    x = Mem(xb, where)
    blas.scal(blas.tbl, n, -1.75, x.ptr, incx)
    exp = xb.copy()
    logical(exp, n, incx)[:] *= -1.75
    assert np.array_equal(x.numpy(), exp)
    # Daxpy: y_i += a x_i (one FMA per element)
    x, y = Mem(xb, where), Mem(yb, where)
    a = 0.3
    blas.axpy(blas.tbl, n, a, x.ptr, incx, y.ptr, incy)
    got = y.numpy()
    lx, ly = logical(xb, n, incx), logical(yb, n, incy)
    bound = np.spacing(np.abs(a * lx) + np.abs(ly))
    assert np.all(np.abs(logical(got, n, incy) - (a * lx + ly)) <= bound)
    untouched = np.ones(len(yb), bool)
    logical(untouched, n, incy)[:] = False
    assert np.array_equal(got[untouched], yb[untouched])


@pytest.mark.parametrize("where", ["host", "device"])
@pytest.mark.parametrize("incx,incy", CASES)
def test_dot_nrm2(blas, where, incx, incy):
    rng = np.random.default_rng(100 + abs(incx) * 10 + abs(incy))
    n = 100_003
    xb = rng.standard_normal(span(n, incx))
    yb = rng.standard_normal(span(n, incy))
    x, y = Mem(xb, where), Mem(yb, where)
    lx, ly = logical(xb, n, incx), logical(yb, n, incy)
    d = blas.dot(blas.tbl, n, x.ptr, incx, y.ptr, incy)
    assert abs(d - float(np.dot(lx, ly))) <= 1e-13 * float(np.abs(lx * ly).sum())
    r = blas.nrm2(blas.tbl, n, x.ptr, incx)
    assert abs(r - float(np.linalg.norm(lx))) <= 1e-13 * float(np.linalg.norm(lx))
    # the inputs are left as they were
    assert np.array_equal(x.numpy(), xb) and np.array_equal(y.numpy(), yb)


@pytest.mark.parametrize("where", ["host", "device"])
def test_mul_and_degenerate_sizes(blas, where):
    rng = np.random.default_rng(7)
    n = 4099
    xb, yb = rng.standard_normal(n), rng.standard_normal(n)
    x, y = Mem(xb, where), Mem(yb, where)
    blas.mul(blas.tbl, n, x.ptr, y.ptr)
    assert np.array_equal(y.numpy(), xb * yb)
    # n == 0: nothing is read or written, the reductions are 0
    z = Mem(yb, where)
    blas.copy(blas.tbl, 0, x.ptr, 1, z.ptr, 1)
    blas.scal(blas.tbl, 0, 2.0, z.ptr, 1)
    blas.axpy(blas.tbl, 0, 2.0, x.ptr, 1, z.ptr, 1)
    assert np.array_equal(z.numpy(), yb)
    assert blas.dot(blas.tbl, 0, x.ptr, 1, z.ptr, 1) == 0.0
    assert blas.nrm2(blas.tbl, 0, x.ptr, 1) == 0.0
    # n == 1 and an all-zero vector
    assert blas.nrm2(blas.tbl, 1, x.ptr, 1) == abs(xb[0])
    w = Mem(np.zeros(n), where)
    assert blas.nrm2(blas.tbl, n, w.ptr, 1) == 0.0


def test_zero_increment_is_rejected(blas):
    x = np.arange(8, dtype=np.float64)
    y = np.zeros(8)
    blas.copy(blas.tbl, 8, V(x.ctypes.data), 0, V(y.ctypes.data), 1)
    assert np.array_equal(y, np.zeros(8))
    assert "increment" in _lib.last_error()


def test_flops_counter_and_host_staging_cost(blas, capsys):
    """The table counts flops like the reference's NLBlas (blas.cpp keeps a
    flop counter); the host-vector path stages every call through device
    buffers -- its per-call cost is printed (the device path beside it)."""
    import torch
    L = _lib.load()
    flops = ctypes.cast(blas.tbl, ctypes.POINTER(BlasStruct)).contents
    L.nlBlasResetStats(blas.tbl)
    n = 1 << 20
    xh, yh = np.ones(n), np.ones(n)
    blas.axpy(blas.tbl, n, 2.0, V(xh.ctypes.data), 1, V(yh.ctypes.data), 1)
    assert flops.flops == 2.0 * n
    assert np.array_equal(yh, np.full(n, 3.0))
    xd = torch.ones(n, dtype=torch.float64, device="cuda")
    yd = torch.ones(n, dtype=torch.float64, device="cuda")
    times = {}
    for where, (px, py) in (("host", (V(xh.ctypes.data), V(yh.ctypes.data))),
                            ("device", (V(xd.data_ptr()), V(yd.data_ptr())))):
        blas.dot(blas.tbl, n, px, 1, py, 1)
        t0 = time.perf_counter()
        for _ in range(20):
            blas.dot(blas.tbl, n, px, 1, py, 1)
            blas.axpy(blas.tbl, n, 1e-3, px, 1, py, 1)
        times[where] = (time.perf_counter() - t0) / 40
    with capsys.disabled():
        print(f"\n[NLBlas, 2^20 doubles] per call: host vectors {times['host'] * 1e6:.0f} us, "
              f"device vectors {times['device'] * 1e6:.0f} us")
    assert times["device"] < times["host"]
