"""High-level Python API over libnl_gb300: resident matrices, solves and the
full OpenNL context path for a row stream.

* ``Matrix``: a CRS matrix resident in GPU memory (nl_gb300.h
  ``nlgb_matrix``), with ``spmv`` and ``solve`` (plain FP64 or mixed
  FP32-inner / FP64-refined Jacobi-PCG).
* ``assemble``: GPU least-squares / square assembly of a ``RowStream``.
* ``solve_opennl``: the reference's own call sequence (nlNewContext,
  nlSolverParameteri, nlBegin/nlEnd, rows, nlSolve, nlGetVariable) through
  the C ABI -- what geogram's builders do behind Graphite's commands.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .systems import RowStream

K = _lib.header_constants()
PRECISION = {"double": K["NL_GB300_PRECISION_DOUBLE"], "fp64": K["NL_GB300_PRECISION_DOUBLE"],
             "mixed": K["NL_GB300_PRECISION_MIXED"], "auto": K["NL_GB300_PRECISION_AUTO"],
             "df": K["NL_GB300_PRECISION_DOUBLE_FLOAT"],
             "double-float": K["NL_GB300_PRECISION_DOUBLE_FLOAT"]}
PRECISION_NAME = {K["NL_GB300_PRECISION_DOUBLE"]: "double", K["NL_GB300_PRECISION_MIXED"]: "mixed",
                  K["NL_GB300_PRECISION_DOUBLE_FLOAT"]: "df"}
STATUS = {K[n]: n.replace("NL_GB300_STATUS_", "").lower() for n in K if n.startswith("NL_GB300_STATUS_")}


class SolverError(RuntimeError):
    pass


@dataclass
class SolveInfo:
    status: str
    iterations: int
    refinement_steps: int
    rel_residual: float
    true_rel_residual: float
    seconds: float
    algo_bytes: float = 0.0
    precision: str = ""          # precision that ran: "double", "mixed" or "df"


def _info(r) -> SolveInfo:
    return SolveInfo(STATUS.get(r.status, str(r.status)), r.iterations, r.refinement_steps,
                     r.rel_residual, r.true_rel_residual, r.seconds, r.algo_bytes,
                     PRECISION_NAME.get(r.precision, str(r.precision)))


def _ptr(a, t):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _check(rc: int, what: str):
    if rc != 0:
        raise SolverError(f"{what} failed ({rc}): {_lib.last_error()}")


def device_available() -> bool:
    return bool(_lib.load().nlgb_device_available())


class Matrix:
    """CRS matrix resident in HBM (int32 indices, FP64 values)."""

    def __init__(self, rp, ci, va, n_cols: int | None = None, _handle=None):
        L = _lib.load()
        if _handle is not None:
            self._h = _handle
        else:
            rp = np.ascontiguousarray(rp, np.int32)
            ci = np.ascontiguousarray(ci, np.int32)
            va = np.ascontiguousarray(va, np.float64)
            n = rp.shape[0] - 1
            h = L.nlgb_matrix_create(n, n if n_cols is None else n_cols, _ptr(rp, None),
                                     _ptr(ci, None), _ptr(va, None))
            if not h:
                raise SolverError(f"nlgb_matrix_create failed: {_lib.last_error()}")
            self._h = h
        n = ctypes.c_int(); nnz = ctypes.c_longlong(); tpr = ctypes.c_int(); tile = ctypes.c_int()
        _check(L.nlgb_matrix_info(self._h, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(tpr),
                                  ctypes.byref(tile)), "nlgb_matrix_info")
        self.n, self.nnz, self.threads_per_row, self.tile_rows = n.value, nnz.value, tpr.value, tile.value

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().nlgb_matrix_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_layout(self, threads_per_row: int = 0, tile_rows: int = 0):
        _check(_lib.load().nlgb_matrix_set_layout(self._h, threads_per_row, tile_rows), "set_layout")
        self.__init__(None, None, None, _handle=self._h)

    def download(self):
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(max(1, self.nnz), np.int32)
        va = np.empty(max(1, self.nnz), np.float64)
        _check(_lib.load().nlgb_matrix_download(self._h, rp.ctypes.data_as(_lib.i32p),
                                                ci.ctypes.data_as(_lib.i32p),
                                                va.ctypes.data_as(_lib.f64p)), "download")
        return rp, ci[: self.nnz], va[: self.nnz]

    def jacobi(self) -> np.ndarray:
        d = np.empty(self.n, np.float64)
        _check(_lib.load().nlgb_matrix_jacobi(self._h, d.ctypes.data_as(_lib.f64p)), "jacobi")
        return d

    def spmv(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.n, np.float64)
        _check(_lib.load().nlgb_spmv(self._h, _ptr(x, None), _ptr(y, None)), "nlgb_spmv")
        return y

    def solve(self, b, x0=None, eps: float = 1e-10, max_iter: int = -1, precision: str = "double",
              inner_eps: float = 0.1, max_outer: int = 100000):
        """Solve A x = b.  Host numpy arrays in and out.  Returns (x, SolveInfo).

        precision: "double" (OpenNL's FP64 PCG), "mixed" (FP32 inner, FP64
        reliable updates, FP64 fallback), "df" (OpenNL's PCG in double-float
        on the FP32 pipe; FP64 for matrices outside its exponent range) or
        "auto" (mixed for a matrix given directly).  SolveInfo.precision
        says which ran."""
        L = _lib.load()
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64, copy=True)
        p = _lib.NlgbParams(eps, max_iter, PRECISION[precision], inner_eps, max_outer)
        r = _lib.NlgbResult()
        _check(L.nlgb_solve(self._h, _ptr(b, None), _ptr(x, None), ctypes.byref(p), ctypes.byref(r)),
               "nlgb_solve")
        return x, _info(r)

    def solve_krylov(self, b, method: str = "bicgstab", x0=None, eps: float = 1e-10,
                     max_iter: int = -1, restart: int = 30, jacobi: bool = True):
        """General (non-symmetric) systems: BiCGSTAB or GMRES(restart), FP64.
        Returns (x, SolveInfo)."""
        K = _lib.header_constants()
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, np.float64, copy=True)
        r = _lib.NlgbResult()
        code = K["NLGB_KRYLOV_BICGSTAB"] if method == "bicgstab" else K["NLGB_KRYLOV_GMRES"]
        _check(_lib.load().nlgb_solve_krylov(self._h, b.ctypes.data, x.ctypes.data, code, eps, max_iter,
                                             restart, int(jacobi), ctypes.byref(r)), "nlgb_solve_krylov")
        return x, SolveInfo(STATUS.get(r.status, str(r.status)), r.iterations, 0, r.rel_residual,
                            r.true_rel_residual, r.seconds, 0.0)

    def solve_device(self, b_ptr: int, x_ptr: int, eps: float = 1e-10, max_iter: int = -1,
                     precision: str = "double", inner_eps: float = 0.1, max_outer: int = 100000):
        """Solve with device pointers (e.g. torch tensors' data_ptr())."""
        L = _lib.load()
        p = _lib.NlgbParams(eps, max_iter, PRECISION[precision], inner_eps, max_outer)
        r = _lib.NlgbResult()
        _check(L.nlgb_solve(self._h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), ctypes.byref(p),
                            ctypes.byref(r)), "nlgb_solve")
        return _info(r)


def batch_solve(mats, bs, x0s=None, eps: float = 1e-10, max_iter: int = -1,
                precision: str = "double", inner_eps: float = 0.1, max_outer: int = 100000):
    """Solve many systems in one persistent-kernel launch.  mats: list of
    Matrix (may repeat), bs: list of host vectors.  Returns (xs, infos,
    kernel_seconds)."""
    L = _lib.load()
    n = len(mats)
    bs = [np.ascontiguousarray(b, np.float64) for b in bs]
    xs = [np.zeros(m.n) if x0s is None else np.array(x0s[i], np.float64, copy=True)
          for i, m in enumerate(mats)]
    A = (ctypes.c_void_p * n)(*[m.handle for m in mats])
    B = (ctypes.c_void_p * n)(*[b.ctypes.data for b in bs])
    X = (ctypes.c_void_p * n)(*[x.ctypes.data for x in xs])
    p = _lib.NlgbParams(eps, max_iter, PRECISION[precision], inner_eps, max_outer)
    R = (_lib.NlgbResult * n)()
    secs = ctypes.c_double()
    _check(L.nlgb_batch_solve(n, A, B, X, ctypes.byref(p), R, ctypes.byref(secs)), "nlgb_batch_solve")
    infos = [_info(r) for r in R]
    return xs, infos, secs.value


class Server:
    """Continuous-batching solve server (nl_gb300.h nlgb_server_*).

    submit_* copy the inputs and return a ticket; the solution lands in a
    host buffer owned by this object, returned by ``wait``."""

    def __init__(self, budget_bytes: float = 150e9, precision: str = "mixed", mode: str = "batched",
                 eps: float = 1e-10, epoch_iters: int = 256, inner_eps: float = 0.1,
                 max_systems: int = 8192, max_iter: int = -1, schedule: str = "srpt",
                 epoch_ms: float = 10.0, streams: int = 16, eps_least_squares: float = 0.0,
                 min_tile_rows: int = 0, chunk_cta_budget: int = 0):
        L = _lib.load()
        cfg = _lib.NlgbServerConfig()
        L.nlgb_server_default_config(ctypes.byref(cfg))
        cfg.hbm_budget_bytes = int(budget_bytes)
        cfg.mode = K["NLGB_SERVER_BATCHED"] if mode == "batched" else K["NLGB_SERVER_SERIAL"]
        cfg.precision = PRECISION[precision]
        cfg.eps = eps
        cfg.epoch_iters = epoch_iters
        cfg.inner_eps = inner_eps
        cfg.max_systems = max_systems
        cfg.max_iter = max_iter
        cfg.schedule = K["NLGB_SCHEDULE_SRPT"] if schedule == "srpt" else K["NLGB_SCHEDULE_ALL"]
        cfg.epoch_ms = epoch_ms
        cfg.streams = streams
        cfg.eps_least_squares = eps_least_squares
        cfg.min_tile_rows = min_tile_rows
        cfg.chunk_cta_budget = chunk_cta_budget
        h = L.nlgb_server_create(ctypes.byref(cfg))
        if not h:
            raise SolverError(f"nlgb_server_create failed: {_lib.last_error()}")
        self._h = h
        self._out = {}

    def now(self) -> float:
        return _lib.load().nlgb_server_now(self._h)

    def reset_clock(self):
        _lib.load().nlgb_server_reset_clock(self._h)

    def submit_square(self, sq, arrival: float = -1.0, x0=None) -> int:
        rp = np.ascontiguousarray(sq.rp, np.int32); ci = np.ascontiguousarray(sq.ci, np.int32)
        va = np.ascontiguousarray(sq.va, np.float64); b = np.ascontiguousarray(sq.rhs, np.float64)
        k = b.shape[0]
        out = np.empty((k, sq.n), np.float64)
        x0 = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        t = _lib.load().nlgb_server_submit_crs(
            self._h, sq.n, rp.ctypes.data_as(_lib.i32p), ci.ctypes.data_as(_lib.i32p),
            va.ctypes.data_as(_lib.f64p), k, b.ctypes.data_as(_lib.f64p),
            None if x0 is None else x0.ctypes.data_as(_lib.f64p), out.ctypes.data_as(_lib.f64p),
            float(arrival))
        if t < 0:
            raise SolverError(f"submit failed ({t}): {_lib.last_error()}")
        self._out[t] = out
        return t

    def submit_rows(self, rs: RowStream, arrival: float = -1.0) -> int:
        col = rs.encoded_cols()
        n_free = int((rs.locked == 0).sum())
        k = rs.n_systems
        out = np.empty((k, n_free), np.float64)
        rp = np.ascontiguousarray(rs.row_ptr, np.int64)
        val = np.ascontiguousarray(rs.val, np.float64)
        rhs = np.ascontiguousarray(rs.rhs.T, np.float64)
        xl = np.ascontiguousarray(rs.values, np.float64)
        w = None if rs.weight is None else np.ascontiguousarray(rs.weight, np.float64)
        t = _lib.load().nlgb_server_submit_rows(
            self._h, int(rs.least_squares), rs.n_rows, rp.ctypes.data_as(_lib.i64p),
            col.ctypes.data_as(_lib.i32p), val.ctypes.data_as(_lib.f64p),
            rhs.ctypes.data_as(_lib.f64p), None if w is None else w.ctypes.data_as(_lib.f64p),
            n_free, rs.n_vars, xl.ctypes.data_as(_lib.f64p), k, None,
            out.ctypes.data_as(_lib.f64p), float(arrival))
        if t < 0:
            raise SolverError(f"submit failed ({t}): {_lib.last_error()}")
        self._out[t] = out
        return t

    def submit_mesh(self, kind: str, V, F, b=None, lam: float = 1e-2, pins=None, pin_uv=None,
                    arrival: float = -1.0) -> int:
        """A triangle mesh whose system the server builds on the GPU:
        kind "lscm" (b must be None) or "fairing" (b: (n_rhs, nv))."""
        L = _lib.load()
        K = _lib.header_constants()
        V = np.ascontiguousarray(V, np.float64)
        F = np.ascontiguousarray(F, np.int32)
        nv = V.shape[0]
        lscm = kind == "lscm"
        n = 2 * nv - 4 if lscm else nv
        bb = None if b is None else np.ascontiguousarray(np.atleast_2d(b), np.float64)
        k = 1 if lscm else bb.shape[0]
        out = np.empty((k, n), np.float64)
        pins_a = None if pins is None else np.ascontiguousarray(pins, np.int32)
        uv_a = None if pin_uv is None else np.ascontiguousarray(pin_uv, np.float64).reshape(4)
        t = L.nlgb_server_submit_mesh(
            self._h, K["NLGB_MESH_LSCM"] if lscm else K["NLGB_MESH_FAIRING"], nv, V.ctypes.data,
            F.shape[0], F.ctypes.data if F.size else None,
            None if pins_a is None else pins_a.ctypes.data, None if uv_a is None else uv_a.ctypes.data,
            float(lam), k, None if bb is None else bb.ctypes.data, None, out.ctypes.data, float(arrival))
        if t < 0:
            raise SolverError(f"submit failed ({t}): {_lib.last_error()}")
        self._out[t] = out
        return t

    def wait(self, ticket: int):
        """Returns (solutions (n_rhs, n), [SolveInfo], latency_s)."""
        out = self._out[ticket]
        R = (_lib.NlgbResult * out.shape[0])()
        lat = ctypes.c_double()
        rc = _lib.load().nlgb_server_wait(self._h, ticket, R, ctypes.byref(lat))
        infos = [_info(r) for r in R]
        if rc != 0:
            raise SolverError(f"request {ticket} failed: {_lib.last_error()}")
        return out, infos, lat.value

    def wait_result(self, ticket: int):
        """Like wait, without raising: returns (ok, solutions, [SolveInfo],
        latency_s); a failed or aborted request gives ok False and the
        per-system statuses it ended with."""
        out = self._out[ticket]
        R = (_lib.NlgbResult * out.shape[0])()
        lat = ctypes.c_double()
        rc = _lib.load().nlgb_server_wait(self._h, ticket, R, ctypes.byref(lat))
        return rc == 0, out, [_info(r) for r in R], lat.value

    def drain(self) -> int:
        return _lib.load().nlgb_server_drain(self._h)

    def stats(self) -> dict:
        st = _lib.NlgbServerStats()
        _check(_lib.load().nlgb_server_get_stats(self._h, ctypes.byref(st)), "stats")
        return {f: getattr(st, f) for f, _ in st._fields_}

    def abort(self):
        _lib.load().nlgb_server_abort(self._h)

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().nlgb_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def assemble(rs: RowStream):
    """GPU assembly of a row stream.  Returns (Matrix, rhs (n_systems, n_free), seconds)."""
    L = _lib.load()
    col = rs.encoded_cols()
    n_free = int((rs.locked == 0).sum())
    rhs = np.ascontiguousarray(rs.rhs.T, np.float64)
    row_ptr = np.ascontiguousarray(rs.row_ptr, np.int64)
    val = np.ascontiguousarray(rs.val, np.float64)
    weight = None if rs.weight is None else np.ascontiguousarray(rs.weight, np.float64)
    xl = np.ascontiguousarray(rs.values, np.float64)
    out = np.empty((rs.n_systems, max(1, n_free)), np.float64)
    h = ctypes.c_void_p()
    secs = ctypes.c_double()
    _check(L.nlgb_assemble(int(rs.least_squares), rs.n_rows, row_ptr.ctypes.data_as(_lib.i64p),
                           col.ctypes.data_as(_lib.i32p), val.ctypes.data_as(_lib.f64p),
                           rhs.ctypes.data_as(_lib.f64p),
                           None if weight is None else weight.ctypes.data_as(_lib.f64p), n_free,
                           rs.n_vars, xl.ctypes.data_as(_lib.f64p), rs.n_systems, ctypes.byref(h),
                           out.ctypes.data_as(_lib.f64p), ctypes.byref(secs)), "nlgb_assemble")
    return Matrix(None, None, None, _handle=h.value), out[:, :n_free], secs.value


def build_lscm(V, F, pins=None, pin_uv=None):
    """LSCM system of a triangle mesh built on the GPU (nlgb_build_lscm):
    returns (Matrix over the 2 nv - 4 free variables, rhs, seconds)."""
    L = _lib.load()
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    nv = V.shape[0]
    pins_a = None if pins is None else np.ascontiguousarray(pins, np.int32)
    uv_a = None if pin_uv is None else np.ascontiguousarray(pin_uv, np.float64).reshape(4)
    rhs = np.empty(max(1, 2 * nv - 4), np.float64)
    h = ctypes.c_void_p()
    secs = ctypes.c_double()
    _check(L.nlgb_build_lscm(nv, V.ctypes.data, F.shape[0], F.ctypes.data if F.size else None,
                             None if pins_a is None else pins_a.ctypes.data,
                             None if uv_a is None else uv_a.ctypes.data, ctypes.byref(h),
                             rhs.ctypes.data, ctypes.byref(secs)), "nlgb_build_lscm")
    return Matrix(None, None, None, _handle=h.value), rhs[: 2 * nv - 4], secs.value


def build_fairing(V, F, lam: float):
    """Cotangent Laplacian + lam I of a triangle mesh built on the GPU
    (nlgb_build_fairing): returns (Matrix, seconds)."""
    L = _lib.load()
    V = np.ascontiguousarray(V, np.float64)
    F = np.ascontiguousarray(F, np.int32)
    h = ctypes.c_void_p()
    secs = ctypes.c_double()
    _check(L.nlgb_build_fairing(V.shape[0], V.ctypes.data, F.shape[0], F.ctypes.data if F.size else None,
                                float(lam), ctypes.byref(h), ctypes.byref(secs)), "nlgb_build_fairing")
    return Matrix(None, None, None, _handle=h.value), secs.value


def solve_opennl(rs: RowStream, precision: str = "double", eps: float = 1e-10,
                 max_iter: int | None = None, per_call: bool = False, solver: str = "cg",
                 inner_iterations: int | None = None, preconditioner: str = "jacobi"):
    """Run the OpenNL context sequence on a row stream; returns (values
    (n_systems, n_vars), info dict).  per_call=True feeds rows through
    nlBegin(NL_ROW)/nlCoefficient/nlEnd(NL_ROW) one call at a time (slow in
    Python; for small conformance cases), else through nlgb_add_rows."""
    from . import opennl as nl
    ctx = nl.nlNewContext()
    try:
        nl.nlSolverParameteri(nl.NL_NB_VARIABLES, rs.n_vars)
        nl.nlSolverParameteri(nl.NL_NB_SYSTEMS, rs.n_systems)
        nl.nlSolverParameteri(nl.NL_LEAST_SQUARES, nl.NL_TRUE if rs.least_squares else nl.NL_FALSE)
        nl.nlSolverParameteri(nl.NL_SOLVER, {"cg": nl.NL_CG, "bicgstab": nl.NL_BICGSTAB,
                                             "gmres": nl.NL_GMRES}[solver])
        nl.nlSolverParameteri(nl.NL_PRECONDITIONER, {"jacobi": nl.NL_PRECOND_JACOBI,
                                                     "none": nl.NL_PRECOND_NONE,
                                                     "ssor": nl.NL_PRECOND_SSOR}[preconditioner])
        if inner_iterations is not None:
            nl.nlSolverParameteri(nl.NL_INNER_ITERATIONS, int(inner_iterations))
        nl.nlSolverParameterd(nl.NL_THRESHOLD, eps)
        if max_iter is not None:
            nl.nlSolverParameteri(nl.NL_MAX_ITERATIONS, int(max_iter))
        nl.nlSolverParameteri(nl.NL_GB300_PRECISION, PRECISION[precision])
        nl.nlBegin(nl.NL_SYSTEM)
        if per_call:
            for s in range(rs.n_systems):
                for i in range(rs.n_vars):
                    nl.nlMultiSetVariable(i, s, float(rs.values[s, i]))
            for i in np.flatnonzero(rs.locked):
                nl.nlLockVariable(int(i))
        else:
            nl.nlgbSetVariables(rs.values, rs.locked)
        nl.nlBegin(nl.NL_MATRIX)
        if per_call:
            for r in range(rs.n_rows):
                nl.nlBegin(nl.NL_ROW)
                for k in range(rs.row_ptr[r], rs.row_ptr[r + 1]):
                    nl.nlCoefficient(int(rs.var[k]), float(rs.val[k]))
                for s in range(rs.n_systems):
                    nl.nlMultiRightHandSide(s, float(rs.rhs[r, s]))
                if rs.weight is not None:
                    nl.nlRowScaling(float(rs.weight[r]))
                nl.nlEnd(nl.NL_ROW)
        else:
            rc = nl.nlgbAddRows(rs.row_ptr, rs.var, rs.val, rs.rhs, rs.weight)
            if rc != 0:
                raise SolverError(f"nlgb_add_rows failed: {nl.nlGetErrorString()}")
        nl.nlEnd(nl.NL_MATRIX)
        nl.nlEnd(nl.NL_SYSTEM)
        ok = nl.nlSolve()
        info = {
            "ok": bool(ok),
            "status": STATUS.get(nl.nlGetIntegerv(nl.NL_GB300_STATUS), "?"),
            "iterations": nl.nlGetIntegerv(nl.NL_USED_ITERATIONS),
            "refinement_steps": nl.nlGetIntegerv(nl.NL_GB300_REFINEMENT_STEPS),
            "error": nl.nlGetDoublev(nl.NL_ERROR),
            "true_error": nl.nlGetDoublev(nl.NL_GB300_TRUE_RESIDUAL),
            "elapsed": nl.nlGetDoublev(nl.NL_ELAPSED_TIME),
            "assembly_time": nl.nlGetDoublev(nl.NL_GB300_ASSEMBLY_TIME),
            "nnz": nl.nlGetIntegerv(nl.NL_NNZ),
            "error_string": nl.nlGetErrorString() if not ok else "",
        }
        if per_call:
            vals = np.array([[nl.nlMultiGetVariable(i, s) for i in range(rs.n_vars)]
                             for s in range(rs.n_systems)])
        else:
            vals = nl.nlgbGetVariables(rs.n_systems, rs.n_vars)
        return vals, info
    finally:
        nl.nlDeleteContext(ctx)
