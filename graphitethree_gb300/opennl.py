"""Python mirror of the OpenNL C API (include/nl.h), one function per C entry
point, with the reference's names and argument meanings.

The reference binds OpenNL from C++ (plugins/OGF/WarpDrive/commands/
voxel_grob_transport_commands.cpp:231-287) and wraps its matrices for
scripting in OGF::NL (src/lib/OGF/scene_graph/NL/matrix.cpp); this module
lets Python code -- the tests and benchmarks -- drive exactly the same C
calls.  Constants are read from the header, so they cannot drift.

    from graphitethree_gb300.opennl import *
    nlNewContext()
    nlSolverParameteri(NL_LEAST_SQUARES, NL_TRUE)
    nlSolverParameteri(NL_NB_VARIABLES, n)
    nlBegin(NL_SYSTEM) ... nlEnd(NL_SYSTEM)
    nlSolve()
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_CONST = _lib.header_constants()
globals().update({k: v for k, v in _CONST.items() if k.startswith("NL")})

__all__ = sorted(k for k in _CONST if k.startswith("NL_") or k in ("NL_TRUE", "NL_FALSE"))


def _L():
    return _lib.load()


def _export(name):
    def f(*args):
        return getattr(_L(), name)(*args)
    f.__name__ = name
    f.__doc__ = f"C entry point {name} of libnl_gb300 (include/nl.h)."
    globals()[name] = f
    __all__.append(name)


for _name in ("nlNewContext", "nlDeleteContext", "nlMakeCurrent", "nlGetCurrent",
              "nlSolverParameterd", "nlSolverParameteri", "nlEnable", "nlDisable", "nlIsEnabled",
              "nlGetError", "nlSetVariable", "nlMultiSetVariable", "nlGetVariable",
              "nlMultiGetVariable", "nlLockVariable", "nlUnlockVariable", "nlVariableIsLocked",
              "nlBegin", "nlEnd", "nlCoefficient", "nlAddIJCoefficient", "nlAddIRightHandSide",
              "nlMultiAddIRightHandSide", "nlRightHandSide", "nlMultiRightHandSide",
              "nlRowScaling", "nlSolve", "nlSparseMatrixNew", "nlSparseMatrixAdd",
              "nlDeleteMatrix", "nlMatrixNNZ", "nlNewJacobiPreconditioner",
              "nlNewSSORPreconditioner", "nlMatrixFactorize", "nlHostBlas", "nlCUDABlas"):
    _export(_name)


def nlInitExtension(name: str) -> int:
    return _L().nlInitExtension(name.encode())


def nlGetErrorString() -> str:
    s = _L().nlGetErrorString()
    return s.decode() if s else ""


def nlGetIntegerv(pname: int) -> int:
    v = ctypes.c_int()
    _L().nlGetIntegerv(pname, ctypes.byref(v))
    return v.value


def nlGetDoublev(pname: int) -> float:
    v = ctypes.c_double()
    _L().nlGetDoublev(pname, ctypes.byref(v))
    return v.value


def nlMatrixCompress(M: int) -> int:
    """Returns the new (compressed) matrix handle; the old one is freed."""
    h = ctypes.c_void_p(M)
    _L().nlMatrixCompress(ctypes.byref(h))
    return h.value


def _vec_ptr(a, writable: bool):
    """Pointer to an FP64 vector: a numpy array (host) or any CUDA array
    exposing __cuda_array_interface__ (device; passed to the library as is,
    no staging).  Returns (pointer, keep-alive object)."""
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        if cai["typestr"] != "<f8" or len(cai["shape"]) != 1 or cai.get("strides") not in (None, (8,)):
            raise ValueError("device vectors must be contiguous 1-D float64")
        return ctypes.cast(ctypes.c_void_p(cai["data"][0]), _lib.f64p), a
    if writable:
        assert a.dtype == np.float64 and a.flags.c_contiguous
        return a.ctypes.data_as(_lib.f64p), a
    h = np.ascontiguousarray(a, np.float64)
    return h.ctypes.data_as(_lib.f64p), h


def nlMultMatrixVector(M: int, x, y) -> None:
    """y = M x; x and y are host (numpy) or device (CUDA array) vectors."""
    px, kx = _vec_ptr(x, False)
    py, ky = _vec_ptr(y, True)
    _L().nlMultMatrixVector(M, px, py)


def nlSolveSystemIterative(blas, M, P, b, x, solver: int, eps: float,
                           max_iter: int, inner_iter: int = 5) -> int:
    """b and x are host (numpy) or device (CUDA array) vectors."""
    pb, kb = _vec_ptr(b, False)
    px, kx = _vec_ptr(x, True)
    return _L().nlSolveSystemIterative(blas, M, P, pb, px, solver, eps, max_iter, inner_iter)


# ---- bulk helpers (nl_gb300.h) -------------------------------------------
def nlgbAddRows(row_ptr, var, val, rhs=None, weight=None) -> int:
    """Equivalent to nlBegin(NL_ROW)/nlCoefficient/.../nlEnd(NL_ROW) per row."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int64)
    var = np.ascontiguousarray(var, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    rhs = None if rhs is None else np.ascontiguousarray(rhs, np.float64)
    weight = None if weight is None else np.ascontiguousarray(weight, np.float64)
    return _L().nlgb_add_rows(row_ptr.shape[0] - 1, row_ptr.ctypes.data_as(_lib.i64p),
                              var.ctypes.data_as(_lib.i32p), val.ctypes.data_as(_lib.f64p),
                              None if rhs is None else rhs.ctypes.data_as(_lib.f64p),
                              None if weight is None else weight.ctypes.data_as(_lib.f64p))


def nlgbSetVariables(values=None, locked=None) -> int:
    v = None if values is None else np.ascontiguousarray(values, np.float64)
    lk = None if locked is None else np.ascontiguousarray(locked, np.uint8)
    return _L().nlgb_set_variables(None if v is None else v.ctypes.data_as(_lib.f64p),
                                   None if lk is None else lk.ctypes.data_as(_lib.u8p))


def nlgbGetVariables(n_systems: int, n_vars: int) -> np.ndarray:
    out = np.empty((n_systems, n_vars), np.float64)
    _L().nlgb_get_variables(out.ctypes.data_as(_lib.f64p))
    return out


__all__ += ["nlInitExtension", "nlGetErrorString", "nlGetIntegerv", "nlGetDoublev",
            "nlMatrixCompress", "nlMultMatrixVector", "nlSolveSystemIterative", "nlgbAddRows",
            "nlgbSetVariables", "nlgbGetVariables"]
