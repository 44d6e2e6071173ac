"""The true-residual check at the end of every FP64 / double-float solve, on
the GPU: when the recursive residual meets eps but ||b - A x|| recomputed in
FP64 does not, the iteration continues with a lower recursive threshold
(at most 4 times) or ends as true_residual_stalled.  The check and its
continuation are the same steps in every executor -- the graph solver
(cooperative or three-kernel), the persistent batched kernel, the server
(persistent epochs and graph chunks, a continuation may straddle an epoch
boundary) and the no-alloc entry point -- so results stay bit-identical
across them."""
import ctypes

import numpy as np
import pytest

from graphitethree_gb300 import _lib, solver, systems

pytestmark = pytest.mark.gpu


def continuations(info, n, nnz):
    """Failed checks of an FP64 solve, from its algorithmic bytes (each adds
    a residual pass and a p update: 12 nnz + 48 n)."""
    base = (12 * nnz + 36 * n) + (12 * nnz + 16 * n) + info.iterations * (12 * nnz + 108 * n)
    return int(round((info.algo_bytes - base) / (12 * nnz + 48 * n)))


def _noalloc(torch, fs, b, eps):
    L = _lib.load()
    dev = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device="cuda")
    rp, ci, va = dev(fs.rp, torch.int32), dev(fs.ci, torch.int32), dev(fs.va, torch.float64)
    bd = dev(b, torch.float64)
    x = torch.zeros(fs.n, dtype=torch.float64, device="cuda")
    prm = _lib.NlgbParams(eps, -1, 0, 0.1, 100000)
    res = _lib.NlgbResult()
    rc = L.nlgb_solve_noalloc(fs.n, ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(ci.data_ptr()),
                              ctypes.c_void_p(va.data_ptr()), ctypes.c_void_p(bd.data_ptr()),
                              ctypes.c_void_p(x.data_ptr()), ctypes.byref(prm), ctypes.byref(res), None)
    assert rc == 0, _lib.last_error()
    return x.cpu().numpy(), res


@pytest.mark.parametrize("eps", [1e-13, 1e-14, 1e-15])
def test_check_identical_across_executors(gpu_ok, eps):
    torch = pytest.importorskip("torch")
    fs = systems.fairing_system(96, 80, seed=3, n_rhs=1)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    b = fs.rhs[0]
    x, info = A.solve(b, eps=eps)
    assert info.status in ("converged", "true_residual_stalled")
    if info.status == "converged":
        assert info.true_rel_residual <= eps
    else:
        assert info.true_rel_residual > eps
    c = continuations(info, A.n, A.nnz)
    assert 0 <= c <= 4
    xb, ib, _ = solver.batch_solve([A], [b], eps=eps)
    assert (ib[0].status, ib[0].iterations) == (info.status, info.iterations)
    assert np.array_equal(xb[0], x)
    srv = solver.Server(precision="double", eps=eps, epoch_iters=16)
    xs, isv, _ = srv.wait(srv.submit_square(systems.SquareSystem(fs.n, fs.rp, fs.ci, fs.va, fs.rhs)))
    srv.close()
    assert (isv[0].status, isv[0].iterations) == (info.status, info.iterations)
    assert np.array_equal(xs[0], x)
    xn, rn = _noalloc(torch, fs, b, eps)
    assert (rn.status, rn.iterations) == (solver.K["NL_GB300_STATUS_CONVERGED"] if info.status == "converged"
                                          else solver.K["NL_GB300_STATUS_TRUE_RESIDUAL_STALLED"],
                                          info.iterations)
    assert np.array_equal(xn, x)


def test_some_case_continues(gpu_ok):
    """At least one tolerance of a sweep actually exercises a continuation
    (the recursive residual passes while the true one misses)."""
    fs = systems.fairing_system(96, 80, seed=3, n_rhs=1)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    seen = []
    for eps in (1e-12, 3e-13, 1e-13, 3e-14, 1e-14, 3e-15, 1e-15, 3e-16):
        _, info = A.solve(fs.rhs[0], eps=eps)
        seen.append((eps, info.status, continuations(info, A.n, A.nnz), info.true_rel_residual))
    assert any(c > 0 for _, _, c, _ in seen), seen


def test_graph_chunks_and_persistent_epochs_agree(gpu_ok):
    """A system large enough for the server's graph chunks (>= 384 tiles),
    continued across epochs of 16 iterations: same result as the graph solver."""
    fs = systems.fairing_system(256, 256, seed=9, n_rhs=1)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    x, info = A.solve(fs.rhs[0], eps=1e-15)
    srv = solver.Server(precision="double", eps=1e-15, epoch_iters=16)
    xs, isv, _ = srv.wait(srv.submit_square(systems.SquareSystem(fs.n, fs.rp, fs.ci, fs.va, fs.rhs)))
    st = srv.stats()
    srv.close()
    assert st["graph_epochs"] > 0
    assert (isv[0].status, isv[0].iterations) == (info.status, info.iterations)
    assert np.array_equal(xs[0], x)


def test_double_float_meets_the_true_residual(gpu_ok):
    """Double-float's recursive residual drifts further from the true one;
    with the check, a converged double-float solve meets eps on the true
    residual too, and its graph and batched forms agree bit for bit."""
    M, rhs, _ = solver.assemble(systems.lscm_system(120, 110, seed=2))
    x, info = M.solve(rhs[0], precision="df")
    assert info.precision == "df"
    assert info.status in ("converged", "true_residual_stalled")
    if info.status == "converged":
        assert info.true_rel_residual <= 1e-10
    xb, ib, _ = solver.batch_solve([M], [rhs[0]], precision="df")
    assert (ib[0].status, ib[0].iterations) == (info.status, info.iterations)
    assert np.array_equal(xb[0], x)
