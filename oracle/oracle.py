"""CPU oracle for the OpenNL sparse-solver hot path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module; the library never does.

* ``assemble``: least-squares normal equations / square systems from a row
  stream (C, nl_oracle.c), bit-exact reference for the GPU row-merge.
* ``pcg``: FP64 Jacobi-PCG with OpenMP threads (C), the timed CPU baseline
  and the iterative oracle.
* ``pcg_ssor`` / ``ssor_apply``: CG with the SSOR preconditioner, sequential
  sweeps (C), the oracle of the GPU's level-scheduled sweeps.
* ``direct_solve``: scipy SuperLU, the FP64 direct oracle.
* ``pcg_df``: numpy restatement of the double-float Jacobi-PCG (float pairs
  hi + lo, error-free transformations in float32), for the algorithm's
  numerical behaviour (iteration growth, accuracy), not its bits: its sums
  run in row order, the GPU's in tiles.
* ``dense_normal_equations``: an independent numpy restatement used to pin
  ``assemble`` (no shared code with the C path).

OpenNL's own source is absent from the reference checkout (geogram submodule
not checked out), so parity against OpenNL itself is unpinned; the oracle is
pinned against analytic known-answer tests, numpy dense algebra and scipy's
SuperLU (tests/test_oracle.py, tests/golden/).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libnl_oracle.so"

_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_ll_p = ctypes.POINTER(ctypes.c_longlong)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)

_lib = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        L.nlo_assemble.restype = ctypes.c_void_p
        L.nlo_assemble.argtypes = [ctypes.c_int, ctypes.c_longlong, _c_ll_p, _c_int_p, _c_dbl_p,
                                   _c_dbl_p, _c_dbl_p, ctypes.c_int, ctypes.c_int, _c_dbl_p,
                                   ctypes.c_int]
        L.nlo_system_info.argtypes = [ctypes.c_void_p, _c_int_p, _c_ll_p]
        L.nlo_system_copy.argtypes = [ctypes.c_void_p, _c_int_p, _c_int_p, _c_dbl_p, _c_dbl_p]
        L.nlo_system_free.argtypes = [ctypes.c_void_p]
        L.nlo_spmv.argtypes = [ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p, ctypes.c_int]
        L.nlo_pcg.restype = ctypes.c_int
        L.nlo_pcg.argtypes = [ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p,
                              ctypes.c_double, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                              _c_ll_p, _c_dbl_p]
        L.nlo_pcg_timed.restype = ctypes.c_int
        L.nlo_pcg_timed.argtypes = [ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p,
                                    ctypes.c_double, ctypes.c_longlong, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, _c_ll_p, _c_dbl_p]
        L.nlo_pcg_ssor.restype = ctypes.c_int
        L.nlo_pcg_ssor.argtypes = [ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p, _c_dbl_p, _c_dbl_p,
                                   ctypes.c_double, ctypes.c_longlong, ctypes.c_double, _c_ll_p, _c_dbl_p]
        L.nlo_ssor_apply.argtypes = [ctypes.c_int, _c_int_p, _c_int_p, _c_dbl_p, ctypes.c_double, _c_dbl_p,
                                     _c_dbl_p]
        L.nlo_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(ct) if a is not None else None


def max_threads() -> int:
    return int(lib().nlo_max_threads())


def dedupe_rows(row_ptr, var, val):
    """Merge repeated variables of a row into their first occurrence (the
    nlCoefficient semantics of include/nl.h).  Vectorised: the entries that
    survive keep their first-occurrence order within each row, and the
    repeats of a variable are added left to right (bincount accumulates in
    index order), exactly as a sequential pass over the row would."""
    row_ptr = np.asarray(row_ptr, np.int64)
    var = np.asarray(var, np.int64)
    val = np.asarray(val, np.float64)
    n_rows = row_ptr.shape[0] - 1
    if var.size == 0:
        return (np.zeros(n_rows + 1, np.int64), np.zeros(0, np.int32), np.zeros(0, np.float64))
    row = np.repeat(np.arange(n_rows, dtype=np.int64), np.diff(row_ptr))
    key = row * (int(var.max()) + 1) + var
    _, first, inv = np.unique(key, return_index=True, return_inverse=True)
    sums = np.bincount(inv.ravel(), weights=val, minlength=first.shape[0])
    order = np.argsort(first, kind="stable")
    keep = first[order]
    out_rp = np.zeros(n_rows + 1, np.int64)
    np.cumsum(np.bincount(row[keep], minlength=n_rows), out=out_rp[1:])
    return out_rp, var[keep].astype(np.int32), sums[order]


def assemble(least_squares: bool, row_ptr, col, val, rhs, weight, n_free: int, n_vars: int,
             xl, n_systems: int = 1):
    """Row stream (encoded columns: free index or -(var+1)) -> (rp, ci, va, rhs[k, n])."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int64)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    n_rows = row_ptr.shape[0] - 1
    rhs = None if rhs is None else np.ascontiguousarray(rhs, np.float64).reshape(n_systems, n_rows)
    weight = None if weight is None else np.ascontiguousarray(weight, np.float64)
    xl = np.ascontiguousarray(xl if xl is not None else np.zeros((n_systems, max(1, n_vars))), np.float64)
    L = lib()
    h = L.nlo_assemble(int(least_squares), n_rows, _p(row_ptr, _c_ll_p), _p(col, _c_int_p),
                       _p(val, _c_dbl_p), _p(rhs, _c_dbl_p), _p(weight, _c_dbl_p), n_free, n_vars,
                       _p(xl, _c_dbl_p), n_systems)
    n = ctypes.c_int()
    nnz = ctypes.c_longlong()
    L.nlo_system_info(h, ctypes.byref(n), ctypes.byref(nnz))
    rp = np.empty(n.value + 1, np.int32)
    ci = np.empty(max(1, nnz.value), np.int32)
    va = np.empty(max(1, nnz.value), np.float64)
    rh = np.empty((n_systems, max(1, n.value)), np.float64)
    L.nlo_system_copy(h, _p(rp, _c_int_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(rh, _c_dbl_p))
    L.nlo_system_free(h)
    return rp, ci[: nnz.value], va[: nnz.value], rh[:, : n.value]


def assemble_rowstream(rs):
    """Assemble a graphitethree_gb300.systems.RowStream (after deduping rows)."""
    rp, var, val = dedupe_rows(rs.row_ptr, rs.var, rs.val)
    fidx = np.full(rs.n_vars, -1, np.int64)
    fv = np.flatnonzero(rs.locked == 0)
    fidx[fv] = np.arange(fv.shape[0])
    f = fidx[var]
    col = np.where(f >= 0, f, -(var.astype(np.int64) + 1)).astype(np.int32)
    rhs = np.ascontiguousarray(rs.rhs.T)
    return assemble(rs.least_squares, rp, col, val, rhs, rs.weight, int(fv.shape[0]), rs.n_vars,
                    rs.values, rs.n_systems)


def spmv(rp, ci, va, x, nthreads: int = 0):
    rp = np.ascontiguousarray(rp, np.int32); ci = np.ascontiguousarray(ci, np.int32)
    va = np.ascontiguousarray(va, np.float64); x = np.ascontiguousarray(x, np.float64)
    n = rp.shape[0] - 1
    y = np.empty(n, np.float64)
    lib().nlo_spmv(n, _p(rp, _c_int_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(x, _c_dbl_p),
                   _p(y, _c_dbl_p), nthreads or max_threads())
    return y


def pcg(rp, ci, va, b, x0=None, eps: float = 1e-10, max_iter: int | None = None,
        jacobi: bool = True, nthreads: int = 0, max_seconds: float = 0.0):
    """FP64 (Jacobi-)PCG.  Returns (x, status, iterations, rel_residual);
    status 1 converged, 2 max_iter, 3 breakdown, 4 time limit (max_seconds
    > 0)."""
    rp = np.ascontiguousarray(rp, np.int32); ci = np.ascontiguousarray(ci, np.int32)
    va = np.ascontiguousarray(va, np.float64); b = np.ascontiguousarray(b, np.float64)
    n = rp.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    it = ctypes.c_longlong()
    rr = ctypes.c_double()
    st = lib().nlo_pcg_timed(n, _p(rp, _c_int_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(b, _c_dbl_p),
                             _p(x, _c_dbl_p), eps, 5 * n if max_iter is None else max_iter, int(jacobi),
                             nthreads or max_threads(), float(max_seconds), ctypes.byref(it),
                             ctypes.byref(rr))
    return x, int(st), int(it.value), float(rr.value)


def pcg_ssor(rp, ci, va, b, x0=None, eps: float = 1e-10, max_iter: int | None = None,
             omega: float = 1.5):
    """FP64 CG with the SSOR preconditioner (sequential forward and backward
    sweeps, relaxation omega).  Returns (x, status, iterations, rel_residual)."""
    rp = np.ascontiguousarray(rp, np.int32); ci = np.ascontiguousarray(ci, np.int32)
    va = np.ascontiguousarray(va, np.float64); b = np.ascontiguousarray(b, np.float64)
    n = rp.shape[0] - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    it = ctypes.c_longlong()
    rr = ctypes.c_double()
    st = lib().nlo_pcg_ssor(n, _p(rp, _c_int_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), _p(b, _c_dbl_p),
                            _p(x, _c_dbl_p), eps, 5 * n if max_iter is None else max_iter, float(omega),
                            ctypes.byref(it), ctypes.byref(rr))
    return x, int(st), int(it.value), float(rr.value)


def ssor_apply(rp, ci, va, r, omega: float = 1.5):
    """z = M^-1 r for the SSOR preconditioner (sequential sweeps)."""
    rp = np.ascontiguousarray(rp, np.int32); ci = np.ascontiguousarray(ci, np.int32)
    va = np.ascontiguousarray(va, np.float64); r = np.ascontiguousarray(r, np.float64)
    n = rp.shape[0] - 1
    z = np.empty(n)
    lib().nlo_ssor_apply(n, _p(rp, _c_int_p), _p(ci, _c_int_p), _p(va, _c_dbl_p), float(omega),
                         _p(r, _c_dbl_p), _p(z, _c_dbl_p))
    return z


def direct_solve(rp, ci, va, b):
    """FP64 direct oracle: scipy SuperLU."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = len(rp) - 1
    A = sp.csr_matrix((va, ci, rp), shape=(n, n)).tocsc()
    return spla.spsolve(A, np.asarray(b, np.float64))


def _csr(rp, ci, va):
    import scipy.sparse as sp
    n = len(rp) - 1
    return sp.csr_matrix((np.asarray(va, np.float64), np.asarray(ci), np.asarray(rp)), shape=(n, n))


def bicgstab(rp, ci, va, b, x0=None, eps: float = 1e-10, max_iter: int | None = None,
             jacobi: bool = True):
    """Right-preconditioned BiCGSTAB (van der Vorst 1992), M^-1 = D^-1 (or
    the identity): the algorithm of graphitethree_gb300/csrc/nlgb_krylov.cu,
    restated in numpy.  Stops when ||r|| <= eps ||b|| (recursive r).
    Returns (x, status, iterations) with status 1 converged, 2 max_iter,
    3 breakdown."""
    A = _csr(rp, ci, va)
    n = A.shape[0]
    b = np.asarray(b, np.float64)
    d = A.diagonal()
    dinv = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 1.0) if jacobi else np.ones(n)
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    max_iter = 5 * n if max_iter is None else max_iter
    r = b - A @ x
    rh = r.copy()
    bb = b @ b
    if bb == 0.0:
        return np.zeros(n), 1, 0
    rho, alpha, omega = r @ r, 1.0, 1.0
    beta = rho
    p = np.zeros(n)
    v = np.zeros(n)
    if r @ r <= eps * eps * bb:
        return x, 1, 0
    it = 0
    while True:
        p = r + beta * (p - omega * v)
        y = dinv * p
        v = A @ y
        rv = rh @ v
        if rv == 0.0 or not np.isfinite(rv):
            return x, 3, it
        alpha = rho / rv
        s = r - alpha * v
        z = dinv * s
        t = A @ z
        tt = t @ t
        omega = (t @ s) / tt if tt > 0 else 0.0
        x = x + alpha * y + omega * z
        r = s - omega * t
        it += 1
        rr = r @ r
        if rr <= eps * eps * bb:
            return x, 1, it
        if it >= max_iter:
            return x, 2, it
        rho_new = rh @ r
        if rho_new == 0.0 or omega == 0.0:
            return x, 3, it
        beta = (rho_new / rho) * (alpha / omega)
        rho = rho_new


def gmres(rp, ci, va, b, x0=None, eps: float = 1e-10, restart: int = 30,
          max_iter: int | None = None, jacobi: bool = True):
    """Restarted right-preconditioned GMRES(m) (Saad & Schultz 1986) with
    classical Gram-Schmidt applied twice (CGS2) and Givens rotations,
    M^-1 = D^-1 (or the
    identity): the algorithm of nlgb_krylov.cu in numpy.  Convergence is
    decided on the true residual at the start of a cycle; a cycle ends early
    when its residual estimate reaches eps.  Returns (x, status, inner
    steps)."""
    A = _csr(rp, ci, va)
    n = A.shape[0]
    b = np.asarray(b, np.float64)
    d = A.diagonal()
    dinv = np.where(d != 0, 1.0 / np.where(d != 0, d, 1.0), 1.0) if jacobi else np.ones(n)
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    max_iter = 5 * n if max_iter is None else max_iter
    bb = b @ b
    if bb == 0.0:
        return np.zeros(n), 1, 0
    m = restart
    it = 0
    while True:
        r = b - A @ x
        rr = r @ r
        if rr <= eps * eps * bb:
            return x, 1, it
        if it >= max_iter:
            return x, 2, it
        beta = np.sqrt(rr)
        V = np.zeros((m + 1, n))
        H = np.zeros((m + 1, m))
        cs, sn = np.zeros(m), np.zeros(m)
        g = np.zeros(m + 1)
        g[0] = beta
        V[0] = r / beta
        k = 0
        for j in range(m):
            w = A @ (dinv * V[j])
            h = V[: j + 1] @ w                   # classical Gram-Schmidt, twice (CGS2)
            w = w - V[: j + 1].T @ h
            h2 = V[: j + 1] @ w
            w = w - V[: j + 1].T @ h2
            H[: j + 1, j] = h + h2
            hn = np.sqrt(w @ w)
            H[j + 1, j] = hn
            for i in range(j):
                a_, b_ = H[i, j], H[i + 1, j]
                H[i, j] = cs[i] * a_ + sn[i] * b_
                H[i + 1, j] = -sn[i] * a_ + cs[i] * b_
            den = np.hypot(H[j, j], H[j + 1, j])
            if not den > 0:
                return x, 3, it
            cs[j], sn[j] = H[j, j] / den, H[j + 1, j] / den
            H[j, j], H[j + 1, j] = den, 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            it += 1
            k = j + 1
            if hn > 0:
                V[j + 1] = w / hn
            if g[j + 1] ** 2 <= eps * eps * bb or it >= max_iter or not hn > 0:
                break
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i]
        x = x + dinv * (V[:k].T @ y)


# --- double-float restatement -------------------------------------------
# Float pairs hi + lo with the error-free transformations of the GPU's
# double-float arithmetic: Knuth's TwoSum, Dekker's Fast2Sum and the
# TwoProduct, composed as Dekker's double-length addition / multiplication.
# numpy float32 operations round like the FP32 pipe; the TwoProduct's FMA is
# formed in float64, where the product of two floats is exact, then rounded
# once more to float32 (an exact FMA except for rare double roundings).

_f32, _f64 = np.float32, np.float64


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def _fma32(a, b, c):
    return (a.astype(_f64) * b.astype(_f64) + c.astype(_f64)).astype(_f32)


def _df(d):
    d = np.asarray(d, _f64)
    hi = d.astype(_f32)
    return hi, (d - hi.astype(_f64)).astype(_f32)


def _df_to64(h, l):
    return h.astype(_f64) + l.astype(_f64)


def _df_add(ah, al, bh, bl):
    s, e = _two_sum(ah, bh)
    return _fast_two_sum(s, e + (al + bl))


def _df_mul(ah, al, bh, bl):
    p = ah * bh
    e = _fma32(ah, bh, -p)
    e = _fma32(ah, bl, e)
    e = _fma32(al, bh, e)
    return _fast_two_sum(p, e)


def pcg_df(rp, ci, va, b, eps: float = 1e-10, max_iter: int | None = None):
    """Double-float Jacobi-PCG (OpenNL's recurrence and stopping rule on the
    recursive residual, zero start).  Returns (x, status, iterations,
    true_rel_residual) with status 1 converged, 2 max iterations."""
    rp = np.asarray(rp, np.int64); ci = np.asarray(ci, np.int64)
    va = np.asarray(va, _f64); b = np.asarray(b, _f64)
    n = rp.shape[0] - 1
    max_iter = 5 * n if max_iter is None else max_iter
    lens = np.diff(rp)
    cols = [(np.nonzero(lens > j)[0], None) for j in range(int(lens.max(initial=0)))]
    cols = [(idx, rp[idx] + j) for j, (idx, _) in enumerate(cols)]
    vh, vl = _df(va)
    row = np.repeat(np.arange(n), lens)
    diag = np.zeros(n)
    np.add.at(diag, row[ci == row], va[ci == row])
    dh, dl = _df(np.where(diag != 0.0, 1.0 / np.where(diag != 0.0, diag, 1.0), 1.0))

    def spmv(xh, xl):   # row by row in column order, double-float sums
        sh = np.zeros(n, _f32); sl = np.zeros(n, _f32)
        for idx, k in cols:
            ph, pl = _df_mul(vh[k], vl[k], xh[ci[k]], xl[ci[k]])
            sh[idx], sl[idx] = _df_add(sh[idx], sl[idx], ph, pl)
        return sh, sl

    def dot(ah, al, bh, bl):
        return float(np.sum(_df_to64(*_df_mul(ah, al, bh, bl))))

    xh = np.zeros(n, _f32); xl = np.zeros(n, _f32)
    rh, rl = _df(b)
    ph, pl = _df_mul(dh, dl, rh, rl)
    bb = float(b @ b)
    rho = dot(ph, pl, rh, rl)
    it, status = 0, 2
    if not bb > 0.0:
        return np.zeros(n), 1, 0, 0.0
    while it < max_iter:
        qh, ql = spmv(ph, pl)
        alpha = rho / dot(ph, pl, qh, ql)
        ah, al = _df(alpha)
        xh, xl = _df_add(xh, xl, *_df_mul(ah, al, ph, pl))
        rh, rl = _df_add(rh, rl, *_df_mul(-ah, -al, qh, ql))
        zh, zl = _df_mul(dh, dl, rh, rl)
        rz = dot(zh, zl, rh, rl)
        rr = dot(rh, rl, rh, rl)
        it += 1
        if rr <= eps * eps * bb:
            status = 1
            break
        beta = rz / rho
        rho = rz
        bh_, bl_ = _df(beta)
        ph, pl = _df_add(zh, zl, *_df_mul(bh_, bl_, ph, pl))
    x = _df_to64(xh, xl)
    r = b - spmv_host(rp, ci, va, x)
    return x, status, it, float(np.linalg.norm(r) / np.sqrt(bb))


def spmv_host(rp, ci, va, x):
    """y = A x in numpy (FP64)."""
    rp = np.asarray(rp, np.int64)
    row = np.repeat(np.arange(rp.shape[0] - 1), np.diff(rp))
    y = np.zeros(rp.shape[0] - 1)
    np.add.at(y, row, np.asarray(va, _f64) * np.asarray(x, _f64)[np.asarray(ci, np.int64)])
    return y


def dense_normal_equations(rs):
    """Independent numpy restatement of the least-squares normal equations
    (dense; small systems only)."""
    rp, var, val = dedupe_rows(rs.row_ptr, rs.var, rs.val)
    n_rows = rp.shape[0] - 1
    A = np.zeros((n_rows, rs.n_vars))
    for r in range(n_rows):
        for k in range(rp[r], rp[r + 1]):
            A[r, var[k]] += val[k]
    w = np.ones(n_rows) if rs.weight is None else np.asarray(rs.weight)
    free = rs.locked == 0
    Af, Al = A[:, free], A[:, ~free]
    out_M = (Af * w[:, None]).T @ Af
    rhs = []
    for s in range(rs.n_systems):
        srow = rs.rhs[:, s] - Al @ rs.values[s][~free]
        rhs.append((Af * w[:, None]).T @ srow)
    return out_M, np.array(rhs)
