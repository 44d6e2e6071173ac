"""The benchmark configurations at their full sizes, checked through
size-independent properties: the true FP64 residual, agreement with the CPU
oracle's FP64 PCG run to a tighter tolerance, and, for mixed precision, the
FP64 fallback rule on the ill-conditioned systems.

* config 1: LSCM on a 256 x 256 bumpy grid (131,068 unknowns);
* config 2: cotangent Laplacian + 1e-2 I on a 2048 x 2048 grid (4.2M
  unknowns, ~29M nonzeros), 3 right-hand sides;
* config 3 (reduced): uneven charts in one batched launch;
* config 5: cotangent Laplacian + 1e-4 I on a 1024 x 1024 grid with x
  stretched per row band by log-uniform [1, 1e3], one N(0,1) right-hand side.
"""
import numpy as np
import pytest

from graphitethree_gb300 import meshes, solver, systems

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_config1_lscm_256(gpu_ok, oracle_mod):
    rs = systems.lscm_system(256, 256, seed=1)
    assert rs.n_rows == 260100 and rs.n_vars == 131072
    M, rhs, secs = solver.assemble(rs)
    assert M.n == 131068
    # converged means the TRUE residual met eps (the recursive one may have
    # needed a continuation)
    x64, i64 = M.solve(rhs[0], eps=1e-10)
    assert i64.status == "converged" and i64.true_rel_residual <= 1e-10
    xmx, imx = M.solve(rhs[0], eps=1e-10, precision="mixed")
    assert imx.status == "converged" and imx.true_rel_residual <= 1e-10
    # error against the FP64 direct oracle: at a relative residual of 1e-10
    # the LSCM normal equations (kappa ~ 1e6 after Jacobi scaling) leave an
    # error of a few 1e-8 in any CG solution, the reference's own included
    rp, ci, va, orhs = oracle_mod.assemble_rowstream(rs)
    xd = oracle_mod.direct_solve(rp, ci, va, orhs[0])
    assert rel(x64, xd) <= 1e-7 and rel(xmx, xd) <= 1e-7
    # at 1e-12 the true residual of the FP64 recurrence may stall above eps
    # (the status says so); the iterate is still within 1e-8 of the
    # oracle's own PCG
    xo, st, it, rr = oracle_mod.pcg(rp, ci, va, orhs[0], eps=1e-12)
    assert st == 1
    x12, i12 = M.solve(rhs[0], eps=1e-12)
    assert i12.status in ("converged", "true_residual_stalled")
    assert (i12.status == "converged") == (i12.true_rel_residual <= 1e-12)
    assert rel(x12, xo) <= 1e-8


def test_config2_fairing_2048(gpu_ok, oracle_mod):
    fs = systems.fairing_system(2048, 2048, seed=2)
    assert fs.n == 4194304
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in range(3):
        x64, i64 = A.solve(fs.rhs[k], eps=1e-10)
        xmx, imx = A.solve(fs.rhs[k], eps=1e-10, precision="mixed")
        assert i64.status == "converged" and imx.status == "converged"
        assert imx.true_rel_residual <= 1e-10          # mixed stops on the true FP64 residual
        assert i64.true_rel_residual <= 1e-10          # FP64: checked after the recursive stop
        # per coordinate, both forms against the oracle's FP64 PCG run to
        # 1e-14 (kappa ~ 1e3; a direct factorisation of 4.2M unknowns is
        # beyond a test's time)
        xo, st, it, rr = oracle_mod.pcg(fs.rp, fs.ci, fs.va, fs.rhs[k], eps=1e-14)
        assert st == 1
        assert rel(x64, xo) <= 1e-8 and rel(xmx, xo) <= 1e-8


def test_config3_batched_charts_reduced(gpu_ok):
    """Uneven charts (long side log-uniform, aspect log-uniform in [1, 4]) in
    one persistent-kernel launch: every chart converges and equals its own
    single-system solve bit for bit."""
    nx, ny = meshes.chart_sizes(48, seed=3, side_min=16, side_max=160)
    mats, bs = [], []
    for c in range(48):
        M, rhs, _ = solver.assemble(systems.lscm_system(int(nx[c]), int(ny[c]), seed=100 + c))
        mats.append(M)
        bs.append(rhs[0])
    for precision in ("double", "mixed"):
        xs, infos, secs = solver.batch_solve(mats, bs, precision=precision)
        assert all(i.status == "converged" for i in infos)
        for c in (0, 17, 47):
            x1, i1 = mats[c].solve(bs[c], precision=precision)
            assert np.array_equal(xs[c], x1)


def test_config5_stretched_illconditioned(gpu_ok):
    """kappa ~ 1e8 at 1e-12.  Plain FP64 PCG meets eps on its recursive
    residual, but the true one has drifted far above it (the attainable
    accuracy of the recurrence): the solve reports true_residual_stalled,
    not converged.  FP32 cannot track this system, so the mixed form falls
    back to that same FP64 PCG from its current x: it must end like the
    plain form, not claim more."""
    fs = systems.fairing_system(1024, 1024, seed=5, lam=1e-4, n_rhs=1, stretch_bands=16,
                                rhs_normal=True)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    x64, i64 = A.solve(fs.rhs[0], eps=1e-12)
    assert i64.rel_residual <= 1e-12
    assert i64.status in ("converged", "true_residual_stalled")
    assert (i64.status == "converged") == (i64.true_rel_residual <= 1e-12)
    # a cap well above plain FP64's iteration count, so that a regression of
    # the fallback fails in seconds instead of running to 5n iterations
    cap = 3 * i64.iterations
    xmx, imx = A.solve(fs.rhs[0], eps=1e-12, precision="mixed", max_iter=cap)
    assert imx.status in ("converged", "true_residual_stalled") and imx.rel_residual <= 1e-12, imx
    assert (imx.status == "converged") == (imx.true_rel_residual <= 1e-12)
    assert imx.refinement_steps >= 1
    # the drift of the recursive residual is of the same size in both runs
    assert imx.true_rel_residual <= 4.0 * i64.true_rel_residual
    xs, infos, _ = solver.batch_solve([A], [fs.rhs[0]], eps=1e-12, precision="mixed",
                                      max_iter=cap)
    assert np.array_equal(xs[0], xmx) and infos[0].status == imx.status
