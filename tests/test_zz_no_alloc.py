"""nlgb_solve_noalloc: the FP64 solve for callers that cannot allocate GPU
memory (applications that keep a fixed device footprint, or loops that cannot
take the synchronisation of cudaMalloc/cudaFree).  It must give the same
answer as the allocating entry point nlgb_solve, call after call, while its
scratch lives in the library's static device array.

Kept in a file of its own, collected last, so a failure here cannot hide any
other test's result."""
import ctypes

import numpy as np
import pytest

from graphitethree_gb300 import _lib, solver, systems

pytestmark = pytest.mark.gpu


def _dev(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _noalloc(L, n, rp, ci, va, b, x, eps=1e-10):
    prm = _lib.NlgbParams(eps, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    rc = L.nlgb_solve_noalloc(n, ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(ci.data_ptr()),
                              ctypes.c_void_p(va.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                              ctypes.c_void_p(x.data_ptr()), ctypes.byref(prm), ctypes.byref(res), None)
    return rc, res


def test_noalloc_matches_allocating_solve_twice(gpu_ok):
    torch = pytest.importorskip("torch")
    L = _lib.load()
    fs = systems.fairing_system(180, 150, seed=11)          # 27,000 rows
    rp = _dev(torch, fs.rp, torch.int32)
    ci = _dev(torch, fs.ci, torch.int32)
    va = _dev(torch, fs.va, torch.float64)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in (0, 2):                                         # two calls in a row
        b = _dev(torch, fs.rhs[k], torch.float64)
        x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
        rc, res = _noalloc(L, fs.n, rp, ci, va, b, x)
        assert rc == 0, _lib.last_error()
        x_ref, info = A.solve(fs.rhs[k])                     # allocating entry point
        x_na = x.cpu().numpy()
        assert res.status == 1 and info.status == "converged"
        # the parity bar of the solver tests: relative difference <= 1e-8
        assert np.linalg.norm(x_na - x_ref) / np.linalg.norm(x_ref) <= 1e-8
        assert abs(res.iterations - info.iterations) <= max(2, 0.02 * info.iterations)
        assert res.true_rel_residual <= 1.5e-10


def test_noalloc_rejects_oversized_systems(gpu_ok):
    L = _lib.load()
    prm = _lib.NlgbParams(1e-10, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    rc = L.nlgb_solve_noalloc(262145, None, None, None, None, None, ctypes.byref(prm),
                              ctypes.byref(res), None)
    assert rc != 0 and "262144" in _lib.last_error()
