"""BiCGSTAB and restarted GMRES(m) on the GPU (nlgb_krylov.cu), through
OpenNL's two entry points: nlSolveSystemIterative on an NLMatrix (the
OGF::NL::Matrix path) and nlSolve with NL_SOLVER on a context.  Checked on a
non-symmetric convection-diffusion system against SuperLU and against the
oracle's numpy restatement of the same algorithms (iteration counts agree
up to rounding), and on an SPD system against the CG solution."""
import numpy as np
import pytest

from graphitethree_gb300 import opennl as nl
from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def nl_matrix(sq):
    M = nl.nlSparseMatrixNew(sq.n, sq.n, nl.NL_MATRIX_STORE_ROWS)
    for i in range(sq.n):
        for k in range(sq.rp[i], sq.rp[i + 1]):
            nl.nlSparseMatrixAdd(M, i, int(sq.ci[k]), float(sq.va[k]))
    return nl.nlMatrixCompress(M)


@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
@pytest.mark.parametrize("jacobi", [True, False])
def test_matrix_api_krylov_nonsymmetric(gpu_ok, oracle_mod, method, jacobi):
    cd = systems.convection_diffusion(40, 30, seed=1)
    M = nl_matrix(cd)
    P = nl.nlNewJacobiPreconditioner(M) if jacobi else None
    x = np.zeros(cd.n)
    code = nl.NL_BICGSTAB if method == "bicgstab" else nl.NL_GMRES
    its = nl.nlSolveSystemIterative(nl.nlHostBlas(), M, P, cd.rhs[0], x, code, 1e-12, 5 * cd.n, 20)
    xd = oracle_mod.direct_solve(cd.rp, cd.ci, cd.va, cd.rhs[0])
    assert its > 0 and rel(x, xd) <= 1e-9
    if method == "bicgstab":
        _, st, its_o = oracle_mod.bicgstab(cd.rp, cd.ci, cd.va, cd.rhs[0], eps=1e-12, jacobi=jacobi)
    else:
        _, st, its_o = oracle_mod.gmres(cd.rp, cd.ci, cd.va, cd.rhs[0], eps=1e-12, restart=20,
                                        jacobi=jacobi)
    assert st == 1 and abs(its - its_o) <= max(3, its_o // 10), (its, its_o)
    if P:
        nl.nlDeleteMatrix(P)
    nl.nlDeleteMatrix(M)


@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_context_krylov(gpu_ok, oracle_mod, method):
    cd = systems.convection_diffusion(33, 29, seed=2)
    vals, info = solver.solve_opennl(cd.to_rows(), eps=1e-12, solver=method, inner_iterations=15)
    assert info["status"] == "converged", info
    xd = oracle_mod.direct_solve(cd.rp, cd.ci, cd.va, cd.rhs[0])
    assert rel(vals[0], xd) <= 1e-9


def test_gmres_restart_length(gpu_ok):
    cd = systems.convection_diffusion(36, 30, seed=4)
    its = {}
    for m in (4, 40):
        vals, info = solver.solve_opennl(cd.to_rows(), eps=1e-11, solver="gmres", inner_iterations=m)
        assert info["status"] == "converged"
        its[m] = info["iterations"]
    assert its[4] != its[40]


def test_krylov_on_spd_matches_cg(gpu_ok):
    fs = systems.fairing_system(40, 36, seed=5, n_rhs=1)
    x_cg, info = solver.solve_opennl(fs.to_rows(), eps=1e-12)
    for method in ("bicgstab", "gmres"):
        x, i2 = solver.solve_opennl(fs.to_rows(), eps=1e-12, solver=method, inner_iterations=30)
        assert i2["status"] == "converged" and rel(x[0], x_cg[0]) <= 1e-8


def test_krylov_edge_cases(gpu_ok):
    cd = systems.convection_diffusion(20, 18, seed=6)
    zero = systems.SquareSystem(n=cd.n, rp=cd.rp, ci=cd.ci, va=cd.va, rhs=np.zeros((1, cd.n)))
    for method in ("bicgstab", "gmres"):
        vals, info = solver.solve_opennl(zero.to_rows(), solver=method)
        assert info["status"] == "converged" and info["iterations"] == 0 and not vals.any()
        vals, info = solver.solve_opennl(cd.to_rows(), eps=1e-14, max_iter=6, solver=method,
                                         inner_iterations=4)
        assert info["status"] == "max_iter" and info["iterations"] == 6


@pytest.mark.parametrize("method", ["bicgstab", "gmres"])
def test_handle_api_equals_matrix_api(gpu_ok, method):
    """nlgb_solve_krylov on a matrix handle and nlSolveSystemIterative on an
    NLMatrix run the same solver on the same CRS: identical results."""
    cd = systems.convection_diffusion(34, 31, seed=7)
    A = solver.Matrix(cd.rp, cd.ci, cd.va)
    xh, ih = A.solve_krylov(cd.rhs[0], method=method, eps=1e-11, restart=25)
    assert ih.status == "converged" and ih.true_rel_residual <= 1.5e-11 and ih.seconds > 0
    M = nl_matrix(cd)
    P = nl.nlNewJacobiPreconditioner(M)
    x = np.zeros(cd.n)
    code = nl.NL_BICGSTAB if method == "bicgstab" else nl.NL_GMRES
    its = nl.nlSolveSystemIterative(nl.nlHostBlas(), M, P, cd.rhs[0], x, code, 1e-11, 5 * cd.n, 25)
    assert its == ih.iterations and np.array_equal(x, xh)
    nl.nlDeleteMatrix(P)
    nl.nlDeleteMatrix(M)
