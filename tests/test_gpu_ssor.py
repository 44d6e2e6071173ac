"""The SSOR preconditioner on the GPU (nlNewSSORPreconditioner, which
OGF::NL::Matrix::solve_iterative creates with omega = 1.5 at
src/lib/OGF/scene_graph/NL/matrix.cpp:366-368): level-scheduled forward and
backward sweeps that compute every row as the sequential sweep does.
Checked against the oracle's sequential SSOR (application and SSOR-PCG) and
the direct solution, through the matrix API (CG, BiCGSTAB, GMRES) and the
context API (NL_PRECOND_SSOR)."""
import numpy as np
import pytest

from graphitethree_gb300 import opennl as nl
from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _matrix(fs):
    M = nl.nlSparseMatrixNew(fs.n, fs.n, nl.NL_MATRIX_STORE_ROWS)
    for i in range(fs.n):
        for k in range(fs.rp[i], fs.rp[i + 1]):
            nl.nlSparseMatrixAdd(M, i, int(fs.ci[k]), float(fs.va[k]))
    return nl.nlMatrixCompress(M)


@pytest.fixture(scope="module")
def fairing():
    return systems.fairing_system(40, 36, seed=3, n_rhs=1)


def test_ssor_application_matches_sequential_sweeps(gpu_ok, oracle_mod, fairing):
    fs = fairing
    M = _matrix(fs)
    P = nl.nlNewSSORPreconditioner(M, 1.5)
    assert P
    r = np.random.default_rng(4).standard_normal(fs.n)
    z = np.zeros(fs.n)
    nl.nlMultMatrixVector(P, r, z)          # the preconditioner as a matrix: z = M^-1 r
    z_ref = oracle_mod.ssor_apply(fs.rp, fs.ci, fs.va, r, 1.5)
    assert rel(z, z_ref) <= 1e-13
    nl.nlDeleteMatrix(P)
    nl.nlDeleteMatrix(M)


@pytest.mark.parametrize("omega", [1.0, 1.5])
def test_ssor_cg_matches_oracle(gpu_ok, oracle_mod, fairing, omega):
    fs = fairing
    M = _matrix(fs)
    P = nl.nlNewSSORPreconditioner(M, omega)
    x = np.zeros(fs.n)
    its = nl.nlSolveSystemIterative(nl.nlHostBlas(), M, P, fs.rhs[0], x, nl.NL_CG, 1e-10, 5 * fs.n, 5)
    xo, st, it_o, _ = oracle_mod.pcg_ssor(fs.rp, fs.ci, fs.va, fs.rhs[0], eps=1e-10, omega=omega)
    xd = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[0])
    assert st == 1 and its > 0
    assert abs(its - it_o) <= max(2, 0.05 * it_o)
    assert rel(x, xo) <= 1e-8 and rel(x, xd) <= 1e-8
    # SSOR cuts the iterations of Jacobi-PCG on this Laplacian
    xj, stj, it_j, _ = oracle_mod.pcg(fs.rp, fs.ci, fs.va, fs.rhs[0], eps=1e-10)
    assert its < it_j
    nl.nlDeleteMatrix(P)
    nl.nlDeleteMatrix(M)


@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_ssor_with_bicgstab_and_gmres(gpu_ok, oracle_mod, fairing, method):
    fs = fairing
    M = _matrix(fs)
    P = nl.nlNewSSORPreconditioner(M, 1.5)
    x = np.zeros(fs.n)
    code = nl.NL_BICGSTAB if method == "bicgstab" else nl.NL_GMRES
    its = nl.nlSolveSystemIterative(nl.nlHostBlas(), M, P, fs.rhs[0], x, code, 1e-10, 5 * fs.n, 30)
    xd = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[0])
    assert its > 0 and rel(x, xd) <= 1e-8
    nl.nlDeleteMatrix(P)
    nl.nlDeleteMatrix(M)


def test_ssor_through_the_context_api(gpu_ok, oracle_mod):
    rs = systems.lscm_system(30, 28, seed=5)
    vals, info = solver.solve_opennl(rs, preconditioner="ssor", eps=1e-12)
    assert info["ok"] and info["status"] in ("converged", "true_residual_stalled")
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    xd = oracle_mod.direct_solve(rp, ci, va, rhs[0])
    x = vals[0][rs.locked == 0]
    assert rel(x, xd) <= 1e-8
    _, info_j = solver.solve_opennl(rs, preconditioner="jacobi", eps=1e-12)
    assert info["iterations"] < info_j["iterations"]


def test_ssor_rejects_bad_relaxation(gpu_ok, fairing):
    M = _matrix(fairing)
    assert not nl.nlNewSSORPreconditioner(M, 2.5)
    nl.nlDeleteMatrix(M)
