"""The CPU oracle pinned against golden vectors made by independent methods
(numpy dense normal equations, scipy SuperLU, analytic known answers)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from graphitethree_gb300 import meshes, systems


@pytest.mark.parametrize("name", golden_names())
def test_oracle_assembly_matches_dense_algebra(oracle_mod, name):
    rs, exp = load_golden(name)
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    n = rp.shape[0] - 1
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(rp[i], rp[i + 1]):
            A[i, ci[k]] += va[k]
    scale = max(1.0, np.abs(exp["normal_dense"]).max())
    assert np.abs(A - exp["normal_dense"]).max() <= 1e-13 * scale
    assert np.abs(rhs - exp["normal_rhs"]).max() <= 1e-13 * max(1.0, np.abs(exp["normal_rhs"]).max())
    # CRS invariants: monotone row pointers, in-range sorted unique columns (LS mode)
    assert np.all(np.diff(rp) >= 0) and np.all((ci >= 0) & (ci < n))
    if rs.least_squares:
        for i in range(n):
            row = ci[rp[i]:rp[i + 1]]
            assert np.all(np.diff(row) > 0)


@pytest.mark.parametrize("name", golden_names())
def test_oracle_pcg_matches_direct_solution(oracle_mod, name):
    rs, exp = load_golden(name)
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    for s in range(rs.n_systems):
        x, st, it, rr = oracle_mod.pcg(rp, ci, va, rhs[s], eps=1e-13)
        assert st == 1, (name, st, it, rr)
        ref = exp["solution"][s]
        assert np.linalg.norm(x - ref) <= 1e-8 * max(1e-300, np.linalg.norm(ref)) + 1e-14


def test_oracle_flat_lscm_is_identity_map(oracle_mod):
    rs, exp = load_golden("lscm_flat_9x8")
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    x, st, it, rr = oracle_mod.pcg(rp, ci, va, rhs[0], eps=1e-14)
    assert st == 1
    exact = exp["exact"][rs.free_vars()]
    assert np.abs(x - exact).max() < 1e-11


def test_oracle_constant_fairing_closed_form(oracle_mod):
    rs, exp = load_golden("fairing_const")
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    x, st, it, rr = oracle_mod.pcg(rp, ci, va, rhs[0], eps=1e-14)
    assert st == 1 and np.abs(x - exp["exact"]).max() < 1e-11


def test_oracle_hand_systems(oracle_mod):
    rs, exp = load_golden("hand_spd_2x2")
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    x, st, it, rr = oracle_mod.pcg(rp, ci, va, rhs[0], eps=1e-15)
    assert st == 1 and np.abs(x - exp["exact"]).max() < 1e-14
    # hand_ls_3var: minimise 2(x0+x1-3)^2 + (x0-x1-1)^2 + (2 x1 + 4 - 5)^2, x2 = 4 locked.
    rs, exp = load_golden("hand_ls_3var")
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    A = np.array([[2.0 + 1.0, 2.0 - 1.0], [2.0 - 1.0, 2.0 + 1.0 + 4.0]])
    b = np.array([2 * 3.0 + 1.0, 2 * 3.0 - 1.0 + 2 * 1.0])
    dense = np.zeros((2, 2))
    for i in range(2):
        for k in range(rp[i], rp[i + 1]):
            dense[i, ci[k]] = va[k]
    assert np.array_equal(dense, A) and np.array_equal(rhs[0], b)


def test_oracle_edge_cases(oracle_mod):
    # b == 0: x = 0, converged after 0 iterations, whatever the start
    fs = systems.fairing_system(6, 6, seed=1)
    x, st, it, rr = oracle_mod.pcg(fs.rp, fs.ci, fs.va, np.zeros(fs.n), x0=np.ones(fs.n))
    assert st == 1 and it == 0 and not x.any()
    # start at the solution: 0 iterations
    xs = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[0])
    x, st, it, rr = oracle_mod.pcg(fs.rp, fs.ci, fs.va, fs.rhs[0], x0=xs, eps=1e-8)
    assert st == 1 and it == 0
    # max_iter = 0 with a nonzero residual
    x, st, it, rr = oracle_mod.pcg(fs.rp, fs.ci, fs.va, fs.rhs[0], max_iter=0)
    assert st == 2 and it == 0
    # indefinite matrix: breakdown reported, not a hang
    rp = np.array([0, 1, 2], np.int32); ci = np.array([0, 1], np.int32); va = np.array([1.0, -1.0])
    x, st, it, rr = oracle_mod.pcg(rp, ci, va, np.array([1.0, 1.0]), jacobi=False)
    assert st == 3


def test_generators_have_config_sizes():
    V, F = meshes.height_field(256, 256, seed=1)
    assert V.shape == (65536, 3) and F.shape == (130050, 3)
    rs = systems.lscm_rows(V, F)
    assert rs.n_rows == 260100 and rs.n_vars == 131072 and int(rs.locked.sum()) == 4
    # every triangle is counter-clockwise in the xy plane (positive LSCM area)
    p = V[F]
    cross = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - \
            (p[:, 1, 1] - p[:, 0, 1]) * (p[:, 2, 0] - p[:, 0, 0])
    assert np.all(cross > 0)


def test_generators_are_seeded():
    a = systems.fairing_system(16, 16, seed=9)
    b = systems.fairing_system(16, 16, seed=9)
    c = systems.fairing_system(16, 16, seed=10)
    assert np.array_equal(a.va, b.va) and np.array_equal(a.rhs, b.rhs)
    assert not np.array_equal(a.va, c.va)
    # cotangent Laplacian + lam I is symmetric and diagonally weighted
    import scipy.sparse as sp
    A = sp.csr_matrix((a.va, a.ci, a.rp), shape=(a.n, a.n))
    assert abs(A - A.T).max() < 1e-14
    assert np.allclose(A @ np.ones(a.n), 1e-2)


def test_oracle_bicgstab_gmres_pinned_to_direct_solve(oracle_mod):
    """The numpy restatements of BiCGSTAB and GMRES(m) (checkers of the GPU
    Krylov solvers) converge on a non-symmetric convection-diffusion system
    to the SuperLU solution."""
    from graphitethree_gb300 import systems
    cd = systems.convection_diffusion(30, 24, seed=3)
    xd = oracle_mod.direct_solve(cd.rp, cd.ci, cd.va, cd.rhs[0])
    for jac in (True, False):
        x, st, it = oracle_mod.bicgstab(cd.rp, cd.ci, cd.va, cd.rhs[0], eps=1e-12, jacobi=jac)
        assert st == 1 and it > 5
        assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)
        for m in (5, 30):
            x, st, it = oracle_mod.gmres(cd.rp, cd.ci, cd.va, cd.rhs[0], eps=1e-12, restart=m, jacobi=jac)
            assert st == 1 and it > 5
            assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)
    x, st, it = oracle_mod.bicgstab(cd.rp, cd.ci, cd.va, np.zeros(cd.n))
    assert st == 1 and it == 0 and not x.any()
    x, st, it = oracle_mod.gmres(cd.rp, cd.ci, cd.va, cd.rhs[0], eps=1e-14, restart=5, max_iter=7)
    assert st == 2 and it == 7                    # stops inside the second cycle


def test_double_float_pcg_restatement(oracle_mod):
    """The double-float PCG (float pairs on float32 arithmetic) behaves like
    FP64 CG on LSCM normal equations and a fairing system: converged on the
    recursive residual, iterations within 15 % of FP64's, true residual
    near the threshold down to its rounding floor (~5e-12 relative here:
    the recursive residual drifts from the true one at 2^-48 rounding),
    solution within 1e-8 of the direct solve at 1e-12."""
    for rs_or_sq in (systems.lscm_system(24, 20, seed=7), systems.fairing_system(30, 28, seed=3)):
        if hasattr(rs_or_sq, "rp"):
            rp, ci, va, b = rs_or_sq.rp, rs_or_sq.ci, rs_or_sq.va, rs_or_sq.rhs[0]
        else:
            rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs_or_sq)
            b = rhs[0]
        xd = oracle_mod.direct_solve(rp, ci, va, b)
        for eps in (1e-10, 1e-12):
            x, st, it, true_rel = oracle_mod.pcg_df(rp, ci, va, b, eps=eps)
            _, st64, it64, _ = oracle_mod.pcg(rp, ci, va, b, eps=eps)
            assert st == 1 and st64 == 1
            assert abs(it - it64) <= max(3, 0.15 * it64)
            assert true_rel <= max(3 * eps, 1e-11)
            if eps == 1e-12:
                assert np.linalg.norm(x - xd) / np.linalg.norm(xd) <= 1e-8
