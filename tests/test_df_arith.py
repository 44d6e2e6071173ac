"""Double-float arithmetic (graphitethree_gb300/csrc/nlgb_df.cuh) on the host:
the same inline primitives the double-float PCG kernels use, built with g++
(-ffp-contract=off) and checked against exact rational arithmetic.

Checked: TwoSum is error-free; Dekker's addition and the product are
accurate to a few units of 2^-48 relative to the operands (the format's
~48-bit significand); addition is commutative bit for bit (the kernels'
butterfly reductions rely on it); conversions to and from FP64 round-trip
to 2^-48."""
import ctypes
import shutil
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
U = 2.0 ** -48


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    cxx = shutil.which("g++")
    cuda_inc = Path("/usr/local/cuda/include")
    if cxx is None or not (cuda_inc / "vector_types.h").exists():
        pytest.skip("g++ or the CUDA headers are missing")
    out = tmp_path_factory.mktemp("df") / "libdfshim.so"
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-std=c++17",
                    "-I", str(ROOT / "graphitethree_gb300" / "csrc"), "-I", str(cuda_inc),
                    str(ROOT / "tests" / "df_shim.cpp"), "-o", str(out)], check=True)
    L = ctypes.CDLL(str(out))
    fp = ctypes.POINTER(ctypes.c_float)
    L.df_two_sum.argtypes = [ctypes.c_float, ctypes.c_float, fp]
    for n in ("df_add", "df_mul"):
        getattr(L, n).argtypes = [fp, fp, fp]
    L.df_mac.argtypes = [fp, fp, fp, fp]
    L.df_from_double.argtypes = [ctypes.c_double, fp]
    L.df_to_double.argtypes = [fp]
    L.df_to_double.restype = ctypes.c_double
    return L


def _f2():
    return (ctypes.c_float * 2)()


def _mk(v):
    a = _f2()
    a[0], a[1] = float(v[0]), float(v[1])
    return a


def _val(a):
    return Fraction(float(np.float32(a[0]))) + Fraction(float(np.float32(a[1])))


def _rand_df(rng, n):
    """n random normalised double-float values (hi, lo) over many binades."""
    d = rng.standard_normal(n) * np.exp2(rng.integers(-30, 30, n))
    hi = d.astype(np.float32)
    lo = (d - hi.astype(np.float64)).astype(np.float32)
    return list(zip(hi, lo))


def test_two_sum_is_exact(shim):
    rng = np.random.default_rng(1)
    a = (rng.standard_normal(2000) * np.exp2(rng.integers(-20, 20, 2000))).astype(np.float32)
    b = (rng.standard_normal(2000) * np.exp2(rng.integers(-20, 20, 2000))).astype(np.float32)
    out = _f2()
    for x, y in zip(a, b):
        shim.df_two_sum(float(x), float(y), out)
        assert Fraction(float(out[0])) + Fraction(float(out[1])) == Fraction(float(x)) + Fraction(float(y))
        assert out[0] == np.float32(np.float32(x) + np.float32(y))


def test_add_mul_mac_accuracy(shim):
    rng = np.random.default_rng(2)
    A, B, C = _rand_df(rng, 1500), _rand_df(rng, 1500), _rand_df(rng, 1500)
    out, out2 = _f2(), _f2()
    for a, b, c in zip(A, B, C):
        fa, fb, fc = _mk(a), _mk(b), _mk(c)
        ea, eb, ec = _val(fa), _val(fb), _val(fc)
        shim.df_add(fa, fb, out)
        assert abs(_val(out) - (ea + eb)) <= 4 * U * (abs(ea) + abs(eb))
        shim.df_add(fb, fa, out2)                       # commutative, bit for bit
        assert (out[0], out[1]) == (out2[0], out2[1])
        shim.df_mul(fa, fb, out)
        assert abs(_val(out) - ea * eb) <= 4 * U * abs(ea * eb)
        shim.df_mac(fc, fa, fb, out)
        assert abs(_val(out) - (ec + ea * eb)) <= 8 * U * (abs(ec) + abs(ea * eb))
        # results are normalised: |lo| <= ulp(hi)
        assert abs(float(out[1])) <= float(np.spacing(np.float32(abs(out[0])))) or out[0] == 0


def test_cancellation_and_zero(shim):
    out = _f2()
    a = _mk((np.float32(1.5), np.float32(3e-8)))
    b = _mk((np.float32(-1.5), np.float32(1e-8)))
    shim.df_add(a, b, out)
    # the heads cancel exactly; the tails' float sum rounds (Dekker's
    # addition is accurate relative to the operands, not to the result)
    assert abs(_val(out) - (_val(a) + _val(b))) <= 4 * U * (abs(_val(a)) + abs(_val(b)))
    z = _mk((0.0, 0.0))
    shim.df_add(z, z, out)
    assert (out[0], out[1]) == (0.0, 0.0)
    shim.df_mac(z, a, z, out)
    assert _val(out) == 0


def test_double_round_trip(shim):
    rng = np.random.default_rng(3)
    # the range the solver admits for double-float, [2^-100, 2^100]: below
    # it the low half becomes a subnormal float and precision is lost
    d = rng.uniform(1.0, 2.0, 3000) * rng.choice([-1.0, 1.0], 3000) * np.exp2(rng.integers(-100, 100, 3000))
    out = _f2()
    for v in d:
        shim.df_from_double(float(v), out)
        back = shim.df_to_double(out)
        assert abs(back - v) <= U * abs(v)
        assert abs(float(out[1])) <= float(np.spacing(np.float32(abs(out[0]))))
    for v in (0.0, 1.0, -2.5, 2.0 ** 60, 2.0 ** -60):
        shim.df_from_double(v, out)
        assert shim.df_to_double(out) == v
