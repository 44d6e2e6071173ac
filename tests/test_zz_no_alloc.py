"""nlgb_solve_noalloc: the FP64 solve for callers that cannot allocate GPU
memory (applications that keep a fixed device footprint, or loops that cannot
take the synchronisation of cudaMalloc/cudaFree).  It runs the same tile
procedures, canonical reductions and scalar steps as the allocating entry
point nlgb_solve, so its iterates are bit-identical, call after call, while
its scratch lives in the library's static device array; a call allocates no
device memory.

Kept in a file of its own, collected last, so a failure here cannot hide any
other test's result."""
import ctypes

import numpy as np
import pytest

from graphitethree_gb300 import _lib, solver, systems

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _noalloc(L, n, rp, ci, va, b, x, eps=1e-10, stream=None):
    prm = _lib.NlgbParams(eps, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    rc = L.nlgb_solve_noalloc(n, ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(ci.data_ptr()),
                              ctypes.c_void_p(va.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                              ctypes.c_void_p(x.data_ptr()), ctypes.byref(prm), ctypes.byref(res),
                              None if stream is None else ctypes.c_void_p(stream))
    return rc, res


def _device_system(torch, fs):
    return (_dev(torch, fs.rp, torch.int32), _dev(torch, fs.ci, torch.int32),
            _dev(torch, fs.va, torch.float64))


def test_noalloc_matches_allocating_solve_twice(gpu_ok):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    fs = systems.fairing_system(180, 150, seed=11)          # 27,000 rows
    rp, ci, va = _device_system(torch, fs)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in (0, 2):                                         # two calls in a row
        b = _dev(torch, fs.rhs[k], torch.float64)
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        rc, res = _noalloc(L, fs.n, rp, ci, va, b, x)
        assert rc == 0, _lib.last_error()
        x_ref, info = A.solve(fs.rhs[k])                     # allocating entry point
        assert res.status == 1 and info.status == "converged"
        assert res.iterations == info.iterations
        assert np.array_equal(x.cpu().numpy(), x_ref)
        assert res.true_rel_residual == info.true_rel_residual <= 1e-10


def test_noalloc_allocates_no_device_memory(gpu_ok):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    fs = systems.fairing_system(120, 110, seed=12, n_rhs=1)
    rp, ci, va = _device_system(torch, fs)
    b = _dev(torch, fs.rhs[0], torch.float64)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    assert _noalloc(L, fs.n, rp, ci, va, b, x)[0] == 0      # warm-up (module load, symbol lookup)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    x.zero_()
    rc, res = _noalloc(L, fs.n, rp, ci, va, b, x)
    torch.cuda.synchronize()
    assert rc == 0 and res.status == 1
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_at_its_size_limit_on_a_user_stream(gpu_ok):
    """An odd row count (a tail row in the paired vector loops) near the
    262,144-row limit, on a caller's stream."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    fs = systems.fairing_system(511, 513, seed=13, n_rhs=1)   # 262,143 rows
    assert fs.n == 262143
    rp, ci, va = _device_system(torch, fs)
    b = _dev(torch, fs.rhs[0], torch.float64)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    rc, res = _noalloc(L, fs.n, rp, ci, va, b, x, stream=stream.cuda_stream)
    assert rc == 0, _lib.last_error()
    x_ref, info = solver.Matrix(fs.rp, fs.ci, fs.va).solve(fs.rhs[0])
    assert res.status == 1 and res.iterations == info.iterations
    assert np.array_equal(x.cpu().numpy(), x_ref)


def test_noalloc_rejects_oversized_systems(gpu_ok):
    L = _lib.load()
    prm = _lib.NlgbParams(1e-10, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    rc = L.nlgb_solve_noalloc(262145, None, None, None, None, None, ctypes.byref(prm),
                              ctypes.byref(res), None)
    assert rc != 0 and "262144" in _lib.last_error()


def test_noalloc_empty_system(gpu_ok):
    L = _lib.load()
    prm = _lib.NlgbParams(1e-10, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    assert L.nlgb_solve_noalloc(0, None, None, None, None, None, ctypes.byref(prm), ctypes.byref(res), None) == 0
    assert res.status == 1 and res.iterations == 0
