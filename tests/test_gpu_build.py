"""GPU mesh builders (nlgb_build_lscm / nlgb_build_fairing): one thread per
triangle writes the LSCM or cotangent-Laplacian rows on the device, then the
normal-equation assembly builds the system.  Checked against the host
builders of graphitethree_gb300.systems (the published formulas in numpy,
assembled by the bit-exact GPU assembly or as CRS directly): the sparsity
must be identical; values may differ in the last bits where numpy's norms
and dot products round differently (the GPU restatement uses no FMA), so
they are compared at 1e-13 of the largest entry.  The solutions are checked
against the oracle's direct solve and, for a planar grid, against the exact
LSCM map."""
import numpy as np
import pytest

from graphitethree_gb300 import meshes, solver, systems

pytestmark = pytest.mark.gpu


def close(a, b, rtol=1e-13):
    scale = max(float(np.abs(b).max()), 1e-300)
    return float(np.abs(np.asarray(a) - np.asarray(b)).max()) <= rtol * scale


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_lscm_builder_matches_host_rows(gpu_ok):
    V, F = meshes.height_field(48, 40, seed=3)
    Mg, rhs_g, secs = solver.build_lscm(V, F)
    Mh, rhs_h, _ = solver.assemble(systems.lscm_rows(V, F))
    assert Mg.n == Mh.n == 2 * V.shape[0] - 4 and secs > 0
    rpg, cig, vag = Mg.download()
    rph, cih, vah = Mh.download()
    assert np.array_equal(rpg, rph) and np.array_equal(cig, cih)
    assert close(vag, vah)
    assert close(rhs_g, rhs_h[0])


def test_lscm_builder_custom_pins(gpu_ok):
    V, F = meshes.height_field(20, 17, seed=8)
    pins, uv = (37, 5), ((0.25, -1.0), (2.0, 0.5))
    Mg, rhs_g, _ = solver.build_lscm(V, F, pins=pins, pin_uv=np.array(uv).reshape(-1))
    Mh, rhs_h, _ = solver.assemble(systems.lscm_rows(V, F, pins=pins, pin_uv=uv))
    rpg, cig, vag = Mg.download()
    rph, cih, vah = Mh.download()
    assert np.array_equal(rpg, rph) and np.array_equal(cig, cih)
    assert close(vag, vah) and close(rhs_g, rhs_h[0])


def test_lscm_builder_solution_matches_oracle(gpu_ok, oracle_mod):
    V, F = meshes.height_field(40, 36, seed=5)
    Mg, rhs, _ = solver.build_lscm(V, F)
    x, info = Mg.solve(rhs, eps=1e-12)
    assert info.status == "converged"
    rp, ci, va, orhs = oracle_mod.assemble_rowstream(systems.lscm_rows(V, F))
    xd = oracle_mod.direct_solve(rp, ci, va, orhs[0])
    assert rel(x, xd) <= 1e-8


def test_flat_grid_lscm_is_identity_map(gpu_ok):
    """Known answer: a planar grid on [0,1]^2 pinned at (0,0) -> (0,0) and
    (1,1) -> (1,1) is mapped to itself (u = x, v = y)."""
    V, F = meshes.height_field(17, 13, seed=2, flat=True)
    Mg, rhs, _ = solver.build_lscm(V, F)
    x, info = Mg.solve(rhs, eps=1e-13)
    assert info.status == "converged"
    free = np.ones(2 * V.shape[0], bool)
    free[[0, 1, 2 * V.shape[0] - 2, 2 * V.shape[0] - 1]] = False
    expect = V[:, :2].reshape(-1)[free]
    assert np.abs(x - expect).max() <= 1e-9


def test_fairing_builder_matches_host_crs(gpu_ok):
    V, F = meshes.height_field(64, 50, seed=4)
    Mg, secs = solver.build_fairing(V, F, 1e-2)
    rp, ci, va = systems.cotan_laplacian(V, F, 1e-2)
    rpg, cig, vag = Mg.download()
    assert np.array_equal(rpg, rp) and np.array_equal(cig, ci)
    assert close(vag, va)


def test_fairing_builder_solution_matches_oracle(gpu_ok, oracle_mod):
    fs = systems.fairing_system(50, 47, seed=6, n_rhs=1)
    V, F = meshes.height_field(50, 47, seed=6)
    Mg, _ = solver.build_fairing(V, F, 1e-2)
    x, info = Mg.solve(fs.rhs[0], eps=1e-12)
    xd = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[0])
    assert info.status == "converged" and rel(x, xd) <= 1e-8


def test_degenerate_triangle_gives_finite_system(gpu_ok):
    """A zero-area triangle (two coincident vertices) contributes zero LSCM
    coefficients and a zero cotangent weight, as in the host builders."""
    V, F = meshes.height_field(6, 5, seed=9)
    V = V.copy()
    V[7] = V[8]                      # collapse an edge
    Mg, rhs_g, _ = solver.build_lscm(V, F)
    Mh, rhs_h, _ = solver.assemble(systems.lscm_rows(V, F))
    vag, vah = Mg.download()[2], Mh.download()[2]
    assert np.isfinite(vag).all() and close(vag, vah)
    Lg, _ = solver.build_fairing(V, F, 1e-2)
    rp, ci, va = systems.cotan_laplacian(V, F, 1e-2)
    assert np.isfinite(Lg.download()[2]).all() and close(Lg.download()[2], va)


def test_builders_reject_bad_input(gpu_ok):
    V, F = meshes.height_field(8, 8, seed=1)
    bad = F.copy()
    bad[3, 1] = V.shape[0]
    with pytest.raises(solver.SolverError):
        solver.build_lscm(V, bad)
    with pytest.raises(solver.SolverError):
        solver.build_fairing(V, bad, 1e-2)
    with pytest.raises(solver.SolverError):
        solver.build_lscm(V, F, pins=(4, 4))


@pytest.mark.parametrize("precision", ["auto", "mixed"])
def test_server_mesh_requests(gpu_ok, precision):
    """Mesh submissions: the server builds the systems on the GPU at
    admission; the results equal the builder + single-system solve, bit for
    bit (same matrix bits, same iterates), LSCM in FP64 under AUTO."""
    V1, F1 = meshes.height_field(36, 30, seed=11)
    V2, F2 = meshes.height_field(44, 40, seed=12)
    fs = systems.fairing_system(44, 40, seed=12, n_rhs=2)
    srv = solver.Server(precision=precision, epoch_iters=64)
    t1 = srv.submit_mesh("lscm", V1, F1)
    t2 = srv.submit_mesh("fairing", V2, F2, b=fs.rhs, lam=1e-2)
    x1, i1, _ = srv.wait(t1)
    x2, i2, _ = srv.wait(t2)
    srv.close()
    M1, rhs1, _ = solver.build_lscm(V1, F1)
    M2, _ = solver.build_fairing(V2, F2, 1e-2)
    p1 = "double" if precision == "auto" else "mixed"
    xs1, is1 = M1.solve(rhs1, precision=p1)
    assert i1[0].status == "converged" and np.array_equal(x1[0], xs1)
    if precision == "auto":
        assert i1[0].refinement_steps == 0
    for k in range(2):
        xs2, is2 = M2.solve(fs.rhs[k], precision="mixed")
        assert i2[k].status == "converged" and np.array_equal(x2[k], xs2)
    with pytest.raises(solver.SolverError):
        srv2 = solver.Server(precision=precision)
        bad = F1.copy()
        bad[0, 0] = -1
        try:
            srv2.submit_mesh("lscm", V1, bad)
        finally:
            srv2.close()
