"""Batched persistent-kernel solver: every system's result must be
bit-identical to the single-system solver on the same system (same tiles,
same canonical reductions, same scalar steps), whatever the team layout and
the rest of the batch; and correct against the oracle."""
import numpy as np
import pytest

from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu


def _mix():
    """Uneven systems: tiny and small (queue workers) and larger (teams)."""
    out = []
    for nx, ny, seed in [(12, 9, 1), (40, 33, 2), (90, 70, 3)]:
        fs = systems.fairing_system(nx, ny, seed=seed)
        out.append((solver.Matrix(fs.rp, fs.ci, fs.va), fs.rhs[0]))
        out.append((out[-1][0], fs.rhs[2]))            # second RHS, same matrix
    for side, seed in [(10, 4), (24, 5), (64, 6)]:
        M, rhs, _ = solver.assemble(systems.lscm_system(side, side + 3, seed=seed))
        out.append((M, rhs[0]))
    return out


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_batch_bit_identical_to_single(gpu_ok, precision):
    items = _mix()
    xs, infos, secs = solver.batch_solve([m for m, _ in items], [b for _, b in items],
                                         precision=precision)
    assert secs > 0
    for (M, b), x, info in zip(items, xs, infos):
        x1, i1 = M.solve(b, precision=precision)
        assert info.status == "converged", info
        assert info.iterations == i1.iterations, (info, i1)
        assert np.array_equal(x, x1)


def test_batch_matches_oracle(gpu_ok, oracle_mod):
    rs = systems.lscm_system(50, 41, seed=9)
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    M, grhs, _ = solver.assemble(rs)
    fs = systems.fairing_system(80, 80, seed=3)
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    # The LSCM normal equations are ill-conditioned: two CG runs stopped at
    # relative residual 1e-10 can differ from the direct solution by more than
    # 1e-8, so this comparison runs at 1e-12.
    for precision in ("double", "mixed"):
        xs, infos, _ = solver.batch_solve([M, F, F, F], [grhs[0], *fs.rhs], precision=precision,
                                          eps=1e-12)
        xd = oracle_mod.direct_solve(rp, ci, va, rhs[0])
        assert infos[0].status == "converged"
        assert np.linalg.norm(xs[0] - xd) / np.linalg.norm(xd) <= 1e-8
        for k in range(3):
            xf = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[k])
            assert np.linalg.norm(xs[1 + k] - xf) / np.linalg.norm(xf) <= 1e-8
            if precision == "mixed":
                assert infos[1 + k].true_rel_residual <= 1e-12


def test_mixed_falls_back_to_fp64_on_lscm(gpu_ok, oracle_mod):
    """FP32 values cannot represent the LSCM normal equations well enough
    (kappa * u32 ~ 1); the mixed solver detects it at a reliable update and
    finishes the system in FP64, in both the graph and the batched solver."""
    M, rhs, _ = solver.assemble(systems.lscm_system(96, 96, seed=3))
    x1, i1 = M.solve(rhs[0], precision="mixed")
    xs, infos, _ = solver.batch_solve([M], [rhs[0]], precision="mixed")
    assert i1.status == "converged" and infos[0].status == "converged"
    assert i1.true_rel_residual <= 1.5e-10
    assert np.array_equal(x1, xs[0]) and i1.iterations == infos[0].iterations


def test_batch_edge_cases(gpu_ok):
    fs = systems.fairing_system(30, 30, seed=1)
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    xs, infos, _ = solver.batch_solve([F, F], [np.zeros(fs.n), fs.rhs[0]], max_iter=5)
    assert infos[0].status == "converged" and infos[0].iterations == 0 and not xs[0].any()
    assert infos[1].status == "max_iter" and infos[1].iterations == 5
    xs, infos, _ = solver.batch_solve([], [])
    assert xs == [] and infos == []


@pytest.mark.parametrize("precision", ["double", "mixed"])
def test_team_queue_more_large_systems_than_teams(gpu_ok, precision):
    """More multi-tile systems than the grid has two-CTA teams for: the ones
    left over are drawn from the shared team queue by whichever team finishes
    first.  Every system still converges, bit-identical to its own solve."""
    mats, bs = [], []
    for c in range(400):
        nx = 48 + (c % 5) * 8
        fs = systems.fairing_system(nx, 48, seed=500 + c, n_rhs=1)
        assert fs.n >= 2048                      # at least 16 tiles of 128 rows
        mats.append(solver.Matrix(fs.rp, fs.ci, fs.va))
        bs.append(fs.rhs[0])
    xs, infos, secs = solver.batch_solve(mats, bs, precision=precision)
    assert all(i.status == "converged" for i in infos)
    for c in (0, 1, 250, 399):
        x1, i1 = mats[c].solve(bs[c], precision=precision)
        assert i1.iterations == infos[c].iterations and np.array_equal(xs[c], x1)
    for M in mats:
        M.close()
