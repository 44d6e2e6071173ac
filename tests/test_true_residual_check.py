"""The true-residual check that ends every FP64 and double-float solve
(scalar_after_check in graphitethree_gb300/csrc/nlgb_core.cuh), on the host:
the same __host__ __device__ function the kernels run, built with nvcc.

OpenNL's CG stops when the recursively updated residual meets eps; the
library then recomputes ||b - A x|| in FP64.  If that misses eps, the
recursive threshold is lowered by the observed ratio (0.9 margin in norm)
and the same recurrence continues; after 4 continuations, or when the gap
exceeds 1e4 in norm, or when the iteration cannot continue, the status is
NL_GB300_STATUS_TRUE_RESIDUAL_STALLED.  Mixed-precision solves stop on the
true residual already and are not touched."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
RUNNING, CONVERGED, MAX_ITER, STALLED = 0, 1, 2, 8


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc is missing")
    out = tmp_path_factory.mktemp("chk") / "libcheckshim.so"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC",
                    "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", str(ROOT / "graphitethree_gb300" / "csrc"), str(ROOT / "tests" / "check_shim.cu"),
                    "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    d, i, ll = ctypes.c_double, ctypes.c_int, ctypes.c_longlong
    L.shim_after_check.argtypes = [d, d, d, d, d, i, i, ll, ll, i, i, i, ctypes.POINTER(d),
                                   ctypes.POINTER(i), ctypes.POINTER(i)]
    L.shim_after_check.restype = i
    return L


def check(L, *, thresh2=1e-20, rthresh2=None, bb=1.0, rr, rr_true, checks=0, cont_ok=1, it=100,
          max_iter=10**6, precision=0, zero_rhs=0, status=CONVERGED):
    rt = ctypes.c_double()
    ck = ctypes.c_int()
    stt = ctypes.c_int()
    cont = L.shim_after_check(thresh2, thresh2 if rthresh2 is None else rthresh2, bb, rr, rr_true, checks,
                              cont_ok, it, max_iter, precision, zero_rhs, status, ctypes.byref(rt),
                              ctypes.byref(ck), ctypes.byref(stt))
    return bool(cont), rt.value, ck.value, stt.value


def test_true_residual_within_eps_is_accepted(shim):
    assert check(shim, rr=0.9e-20, rr_true=0.99e-20) == (False, 1e-20, 0, CONVERGED)


def test_small_gap_continues_with_a_lower_recursive_threshold(shim):
    cont, rt, ck, st = check(shim, rr=0.9e-20, rr_true=1.21e-20)
    assert cont and st == RUNNING and ck == 1
    assert rt == pytest.approx(1e-20 * (0.9 / 1.21) * 0.81, rel=1e-15)


def test_continuations_are_bounded(shim):
    assert check(shim, rr=0.5e-22, rr_true=2e-20, rthresh2=1e-22, checks=3)[0]
    cont, _, ck, st = check(shim, rr=0.5e-24, rr_true=2e-20, rthresh2=1e-24, checks=4)
    assert not cont and st == STALLED and ck == 4


def test_a_gap_beyond_1e4_in_norm_stalls_at_once(shim):
    # recursive 1e-10 (relative) vs true 1.45e-6: config 5's FP64 floor
    cont, _, ck, st = check(shim, rr=1e-20, rr_true=(1.45e-6) ** 2)
    assert not cont and st == STALLED and ck == 0


@pytest.mark.parametrize("kw", [dict(cont_ok=0), dict(it=500, max_iter=500), dict(rr=0.0)])
def test_no_continuation_possible_stalls(shim, kw):
    args = dict(rr=0.9e-20, rr_true=1.21e-20)
    args.update(kw)
    cont, _, _, st = check(shim, **args)
    assert not cont and st == STALLED


@pytest.mark.parametrize("kw", [dict(precision=1), dict(zero_rhs=1), dict(status=MAX_ITER)])
def test_mixed_zero_rhs_and_other_stops_are_left_alone(shim, kw):
    st0 = kw.get("status", CONVERGED)
    cont, rt, ck, st = check(shim, rr=0.9e-20, rr_true=4e-20, **kw)
    assert (cont, rt, ck, st) == (False, 1e-20, 0, st0)
