"""A compiled C++ caller (tests/caller/opennl_caller.cpp) that includes the
library through geogram's OpenNL header paths -- <geogram/NL/nl.h>,
nl_matrix.h, nl_iterative_solvers.h, nl_preconditioners.h, nl_blas.h, the
lines Graphite's sources use (src/lib/OGF/scene_graph/NL/matrix.cpp:40-42,
blas.cpp:40, plugins/OGF/WarpDrive/commands/voxel_grob_transport_commands.
cpp:41) -- and makes their call shapes: the WarpDrive least-squares context
sequence, the OGF::NL::Matrix sequence (including the (NLSparseMatrix*)
cast before nlSparseMatrixAdd) and the NLBlas table.

CPU: the translation unit compiles against include/ and links against
libnl_gb300.so.  GPU: the program runs and its results match the oracle."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from graphitethree_gb300 import systems

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "caller" / "opennl_caller.cpp"
LIBDIR = ROOT / "graphitethree_gb300" / "lib"


def _cxx():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is missing")
    return cxx


def test_compiles_against_geogram_header_paths():
    subprocess.run([_cxx(), "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I",
                    str(ROOT / "include"), str(SRC)], check=True)


@pytest.fixture(scope="module")
def caller(nllib, tmp_path_factory):
    exe = tmp_path_factory.mktemp("caller") / "opennl_caller"
    subprocess.run([_cxx(), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(SRC), "-o", str(exe),
                    "-L", str(LIBDIR), "-lnl_gb300", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


def test_links_against_the_library(caller):
    assert caller.exists()


@pytest.mark.gpu
def test_voxel_context_sequence_matches_oracle(gpu_ok, caller, oracle_mod, tmp_path):
    nu, nv, nw = 24, 20, 16
    rs = systems.voxel_rows(nu, nv, nw, seed=3)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([nu, nv, nw], np.int32).tofile(f)
        rs.locked.astype(np.uint8).tofile(f)
        rs.values[0].astype(np.float64).tofile(f)
    subprocess.run([str(caller), "voxel", str(inp), str(out)], check=True, timeout=120)
    raw = out.read_bytes()
    n = nu * nv * nw
    x = np.frombuffer(raw[: 8 * n], np.float64)
    ok, used = np.frombuffer(raw[8 * n:], np.int32)
    assert ok == 1 and used > 0
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    ref = oracle_mod.direct_solve(rp, ci, va, rhs[0])
    free = rs.locked == 0
    assert np.array_equal(x[~free], rs.values[0][~free])
    assert np.linalg.norm(x[free] - ref) / np.linalg.norm(ref) <= 1e-8


@pytest.mark.gpu
def test_matrix_and_blas_sequence_matches_numpy(gpu_ok, caller, oracle_mod, tmp_path):
    fs = systems.fairing_system(64, 60, seed=6, n_rhs=1)
    n = fs.n
    rows = np.repeat(np.arange(n), np.diff(fs.rp))
    b = fs.rhs[0] / np.abs(fs.rhs[0]).max()
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([n, fs.nnz], np.int32).tofile(f)
        rows.astype(np.int32).tofile(f)
        fs.ci.astype(np.int32).tofile(f)
        fs.va.astype(np.float64).tofile(f)
        b.astype(np.float64).tofile(f)
    subprocess.run([str(caller), "matrix", str(inp), str(out)], check=True, timeout=120)
    v = np.frombuffer(out.read_bytes(), np.float64)
    y_dyn, y_crs, x, c, e = (v[k * n:(k + 1) * n] for k in range(5))
    s2 = v[5 * n: 7 * n]
    dot, nrm, dot_rev, iters = v[7 * n:]
    import scipy.sparse as sp
    A = sp.csr_matrix((fs.va, fs.ci, fs.rp), shape=(n, n))
    y = A @ b
    for yy in (y_dyn, y_crs):
        assert np.linalg.norm(yy - y) <= 1e-14 * np.linalg.norm(y)
    ref = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, b)
    assert iters > 0
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-8
    assert np.array_equal(c, 2.0 * b)
    assert np.allclose(e, 0.5 * b, rtol=0, atol=1e-15)
    assert dot == pytest.approx(2.0 * b @ b, rel=1e-13)
    assert nrm == pytest.approx(np.linalg.norm(b), rel=1e-13)
    assert np.array_equal(s2[0::2], 3.0 * b) and np.all(s2[1::2] == -1.0)
    assert dot_rev == pytest.approx(float(b @ (3.0 * b[::-1])), rel=1e-12)
