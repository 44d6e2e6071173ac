"""ctypes bindings of libnl_gb300.so (C ABI in include/nl.h, include/nl_gb300.h).

The library is the product: every numeric call goes to the GPU through it.
Loading fails loudly if it has not been built; there is no Python or CPU
fallback for any solver operation.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

from .build import INCLUDE, lib_path

_lib = None


class LibraryNotBuilt(RuntimeError):
    pass


def header_constants() -> dict[str, int]:
    """#define NAME value constants of the C headers (single source of truth)."""
    out: dict[str, int] = {}
    for h in ("nl.h", "nl_gb300.h"):
        for m in re.finditer(r"^#define\s+(NL\w*|NLGB\w*)\s+(-?0x[0-9a-fA-F]+|-?\d+)\b",
                             (INCLUDE / h).read_text(), re.M):
            out[m.group(1)] = int(m.group(2), 0)
    return out


def header_functions() -> list[str]:
    """Names of the functions declared by the C headers."""
    names: list[str] = []
    for h in ("nl.h", "nl_gb300.h"):
        text = (INCLUDE / h).read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(nl\w+)\s*\(", text, re.M):
            if not m.group(0).lstrip().startswith(("typedef", "#define", "struct")):
                names.append(m.group(1))
    return sorted(set(names))


C = ctypes
i32p = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_longlong)
f64p = C.POINTER(C.c_double)
f32p = C.POINTER(C.c_float)
u8p = C.POINTER(C.c_ubyte)


class NlgbParams(C.Structure):
    _fields_ = [("eps", C.c_double), ("max_iter", C.c_longlong), ("precision", C.c_int),
                ("inner_eps", C.c_double), ("max_outer", C.c_int)]


class NlgbResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_longlong), ("refinement_steps", C.c_int),
                ("rel_residual", C.c_double), ("true_rel_residual", C.c_double),
                ("seconds", C.c_double), ("algo_bytes", C.c_double), ("precision", C.c_int)]


class NlgbServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("mode", C.c_int), ("precision", C.c_int),
                ("eps", C.c_double), ("max_iter", C.c_longlong), ("inner_eps", C.c_double),
                ("epoch_iters", C.c_longlong), ("max_systems", C.c_int), ("schedule", C.c_int),
                ("epoch_ms", C.c_double), ("streams", C.c_int), ("eps_least_squares", C.c_double),
                ("min_tile_rows", C.c_int), ("chunk_cta_budget", C.c_int)]


class NlgbServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("rejected", C.c_longlong), ("p50_latency_s", C.c_double),
                ("p99_latency_s", C.c_double), ("mean_latency_s", C.c_double),
                ("max_latency_s", C.c_double), ("solves_per_s", C.c_double), ("wall_s", C.c_double),
                ("kernel_s", C.c_double), ("epochs", C.c_longlong), ("iterations", C.c_longlong),
                ("algo_bytes", C.c_double), ("peak_bytes", C.c_size_t), ("budget_bytes", C.c_size_t),
                ("graph_s", C.c_double), ("graph_algo_bytes", C.c_double),
                ("graph_epochs", C.c_longlong), ("used_bytes", C.c_size_t),
                ("byte_seconds", C.c_double), ("epoch_algo_bytes", C.c_double)]


_SIGS = {
    # nl.h
    "nlNewContext": (C.c_void_p, []),
    "nlDeleteContext": (None, [C.c_void_p]),
    "nlMakeCurrent": (None, [C.c_void_p]),
    "nlGetCurrent": (C.c_void_p, []),
    "nlInitExtension": (C.c_ubyte, [C.c_char_p]),
    "nlExtensionIsInitialized": (C.c_ubyte, [C.c_char_p]),
    "nlSolverParameterd": (None, [C.c_uint, C.c_double]),
    "nlSolverParameteri": (None, [C.c_uint, C.c_int]),
    "nlGetBooleanv": (None, [C.c_uint, u8p]),
    "nlGetDoublev": (None, [C.c_uint, f64p]),
    "nlGetIntegerv": (None, [C.c_uint, i32p]),
    "nlEnable": (None, [C.c_uint]),
    "nlDisable": (None, [C.c_uint]),
    "nlIsEnabled": (C.c_ubyte, [C.c_uint]),
    "nlGetError": (C.c_uint, []),
    "nlGetErrorString": (C.c_char_p, []),
    "nlSetVariable": (None, [C.c_uint, C.c_double]),
    "nlMultiSetVariable": (None, [C.c_uint, C.c_uint, C.c_double]),
    "nlGetVariable": (C.c_double, [C.c_uint]),
    "nlMultiGetVariable": (C.c_double, [C.c_uint, C.c_uint]),
    "nlLockVariable": (None, [C.c_uint]),
    "nlUnlockVariable": (None, [C.c_uint]),
    "nlVariableIsLocked": (C.c_ubyte, [C.c_uint]),
    "nlBegin": (None, [C.c_uint]),
    "nlEnd": (None, [C.c_uint]),
    "nlCoefficient": (None, [C.c_uint, C.c_double]),
    "nlAddIJCoefficient": (None, [C.c_uint, C.c_uint, C.c_double]),
    "nlAddIRightHandSide": (None, [C.c_uint, C.c_double]),
    "nlMultiAddIRightHandSide": (None, [C.c_uint, C.c_uint, C.c_double]),
    "nlRightHandSide": (None, [C.c_double]),
    "nlMultiRightHandSide": (None, [C.c_uint, C.c_double]),
    "nlRowScaling": (None, [C.c_double]),
    "nlSolve": (C.c_ubyte, []),
    "nlSparseMatrixNew": (C.c_void_p, [C.c_uint, C.c_uint, C.c_uint]),
    "nlSparseMatrixAdd": (None, [C.c_void_p, C.c_uint, C.c_uint, C.c_double]),
    "nlDeleteMatrix": (None, [C.c_void_p]),
    "nlMatrixCompress": (None, [C.POINTER(C.c_void_p)]),
    "nlMultMatrixVector": (None, [C.c_void_p, f64p, f64p]),
    "nlMatrixNNZ": (C.c_uint, [C.c_void_p]),
    "nlNewJacobiPreconditioner": (C.c_void_p, [C.c_void_p]),
    "nlNewSSORPreconditioner": (C.c_void_p, [C.c_void_p, C.c_double]),
    "nlMatrixFactorize": (C.c_void_p, [C.c_void_p, C.c_uint]),
    "nlHostBlas": (C.c_void_p, []),
    "nlCUDABlas": (C.c_void_p, []),
    "nlBlasResetStats": (None, [C.c_void_p]),
    "nlSolveSystemIterative": (C.c_uint, [C.c_void_p, C.c_void_p, C.c_void_p, f64p, f64p, C.c_uint,
                                          C.c_double, C.c_uint, C.c_uint]),
    # nl_gb300.h
    "nlgb_device_available": (C.c_int, []),
    "nlgb_kernel_launches": (C.c_longlong, []),
    "nlgb_last_error": (C.c_char_p, []),
    "nlgb_default_params": (None, [C.POINTER(NlgbParams)]),
    "nlgb_matrix_create": (C.c_void_p, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "nlgb_matrix_destroy": (None, [C.c_void_p]),
    "nlgb_matrix_info": (C.c_int, [C.c_void_p, i32p, i64p, i32p, i32p]),
    "nlgb_matrix_set_layout": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "nlgb_matrix_download": (C.c_int, [C.c_void_p, i32p, i32p, f64p]),
    "nlgb_matrix_jacobi": (C.c_int, [C.c_void_p, f64p]),
    "nlgb_spmv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "nlgb_spmv32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "nlgb_spmv_timed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, f64p]),
    "nlgb_spmv32_timed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, f64p]),
    "nlgb_solve": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(NlgbParams),
                             C.POINTER(NlgbResult)]),
    "nlgb_solve_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.POINTER(NlgbParams), C.POINTER(NlgbResult),
                                     C.c_void_p]),
    "nlgb_batch_solve": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                   C.POINTER(C.c_void_p), C.POINTER(NlgbParams),
                                   C.POINTER(NlgbResult), f64p]),
    "nlgb_assemble": (C.c_int, [C.c_int, C.c_longlong, i64p, i32p, f64p, f64p, f64p, C.c_int,
                                C.c_int, f64p, C.c_int, C.POINTER(C.c_void_p), f64p, f64p]),
    "nlgb_solve_krylov": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double,
                                    C.c_longlong, C.c_int, C.c_int, C.POINTER(NlgbResult)]),
    "nlgb_build_lscm": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_void_p), C.c_void_p, f64p]),
    "nlgb_build_fairing": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double,
                                     C.POINTER(C.c_void_p), f64p]),
    "nlgb_server_submit_mesh": (C.c_longlong, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "nlgb_server_default_config": (None, [C.POINTER(NlgbServerConfig)]),
    "nlgb_server_create": (C.c_void_p, [C.POINTER(NlgbServerConfig)]),
    "nlgb_server_reset_clock": (None, [C.c_void_p]),
    "nlgb_server_now": (C.c_double, [C.c_void_p]),
    "nlgb_server_submit_crs": (C.c_longlong, [C.c_void_p, C.c_int, i32p, i32p, f64p, C.c_int, f64p,
                                              f64p, f64p, C.c_double]),
    "nlgb_server_submit_rows": (C.c_longlong, [C.c_void_p, C.c_int, C.c_longlong, i64p, i32p, f64p,
                                               f64p, f64p, C.c_int, C.c_int, f64p, C.c_int, f64p,
                                               f64p, C.c_double]),
    "nlgb_server_wait": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(NlgbResult), f64p]),
    "nlgb_server_drain": (C.c_int, [C.c_void_p]),
    "nlgb_server_get_stats": (C.c_int, [C.c_void_p, C.POINTER(NlgbServerStats)]),
    "nlgb_server_abort": (None, [C.c_void_p]),
    "nlgb_server_destroy": (None, [C.c_void_p]),
    "nlgb_add_rows": (C.c_int, [C.c_longlong, i64p, i32p, f64p, f64p, f64p]),
    "nlgb_set_variables": (C.c_int, [f64p, u8p]),
    "nlgb_get_variables": (C.c_int, [f64p]),
}


def load():
    """Load the in-tree library (raises LibraryNotBuilt if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not p.exists():
        raise LibraryNotBuilt(f"{p} not found: run graphitethree_gb300.build.build() first")
    L = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        f = getattr(L, name, None)
        if f is None:
            continue
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    s = load().nlgb_last_error()
    return s.decode() if s else ""
