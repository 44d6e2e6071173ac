"""Double-float precision (NL_GB300_PRECISION_DOUBLE_FLOAT): the FP64
Jacobi-PCG with its vectors, matrix and 1/diag held as float pairs and
computed on the FP32 pipe.

Checked: convergence with OpenNL's stopping rule and a true FP64 residual
near the threshold; the solution against the oracle's direct solve; the
iteration count close to FP64's; bit-identical results on every executor
(cooperative single-kernel graph, three-kernel graph, persistent batched
kernel, server epochs and graph chunks, serial server); the FP64 fallback
for a matrix outside double-float's exponent range; the OpenNL context API
with NL_GB300_PRECISION_DOUBLE_FLOAT."""
import numpy as np
import pytest

from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def lscm_small():
    M, rhs, _ = solver.assemble(systems.lscm_system(60, 52, seed=3))
    return M, rhs[0]


def test_df_solve_matches_oracle(gpu_ok, oracle_mod, lscm_small):
    M, b = lscm_small
    rs = systems.lscm_system(60, 52, seed=3)
    rp, ci, va, orhs = oracle_mod.assemble_rowstream(rs)
    xd = oracle_mod.direct_solve(rp, ci, va, orhs[0])
    for eps in (1e-10, 1e-12):
        x, info = M.solve(b, eps=eps, precision="df")
        x64, i64 = M.solve(b, eps=eps, precision="double")
        assert info.precision == "df" and info.refinement_steps == 0
        assert i64.precision == "double"
        # same stopping rule as FP64 (the recursive residual, then the true
        # one checked in FP64 and the iteration continued while it misses);
        # double-float's recurrence drifts further (rounding at ~2^-48), so
        # its true residual may stall a little above eps -- the status says so
        assert info.status in ("converged", "true_residual_stalled")
        assert (info.status == "converged") == (info.true_rel_residual <= eps)
        assert info.rel_residual <= eps and info.true_rel_residual <= 3 * eps
        # iterations close to FP64's (the continuations add some)
        assert abs(info.iterations - i64.iterations) <= 0.6 * i64.iterations
        if eps == 1e-12:
            assert rel(x, xd) <= 1e-8 and rel(x64, xd) <= 1e-8


def test_df_fairing_matches_fp64(gpu_ok):
    fs = systems.fairing_system(150, 140, seed=9, n_rhs=2)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in range(2):
        x, info = A.solve(fs.rhs[k], precision="df")
        x64, i64 = A.solve(fs.rhs[k], precision="double")
        assert info.status == "converged" and info.precision == "df"
        assert rel(x, x64) <= 1e-8
        assert abs(info.iterations - i64.iterations) <= max(3, 0.1 * i64.iterations)


def test_df_same_on_every_executor(gpu_ok):
    """Small system (single-kernel cooperative iteration) and large system
    (three kernels per iteration, > 640 tiles; graph chunks in the server):
    graph solver == persistent batched kernel == batched server == serial
    server, bit for bit."""
    small = systems.fairing_system(70, 66, seed=13, n_rhs=1)
    large = systems.fairing_system(520, 510, seed=14, n_rhs=1)
    for fs in (small, large):
        A = solver.Matrix(fs.rp, fs.ci, fs.va)
        x1, i1 = A.solve(fs.rhs[0], precision="df")
        xs, infos, _ = solver.batch_solve([A], [fs.rhs[0]], precision="df")
        assert i1.precision == infos[0].precision == "df"
        assert infos[0].iterations == i1.iterations and np.array_equal(xs[0], x1)
        for mode in ("batched", "serial"):
            srv = solver.Server(precision="df", mode=mode, epoch_iters=32)
            x, infs, _ = srv.wait(srv.submit_square(fs))
            st = srv.stats()
            srv.close()
            assert infs[0].status == "converged" and infs[0].precision == "df"
            assert infs[0].iterations == i1.iterations
            assert np.array_equal(x[0], x1)
            if mode == "batched" and fs is large:
                assert A.n // A.tile_rows > 640 and st["graph_epochs"] >= 1


def test_df_in_mix_equals_alone(gpu_ok):
    """Double-float least-squares and square systems side by side in one
    batched server: each equals its own solve alone."""
    reqs = [("rows", systems.lscm_system(50, 47, seed=21)),
            ("square", systems.fairing_system(80, 75, seed=22)),
            ("rows", systems.lscm_system(90, 80, seed=23))]
    alone = []
    for kind, obj in reqs:
        srv = solver.Server(precision="df")
        t = srv.submit_rows(obj) if kind == "rows" else srv.submit_square(obj)
        x, infs, _ = srv.wait(t)
        alone.append((x.copy(), [i.iterations for i in infs], [i.precision for i in infs]))
        srv.close()
    assert alone[0][2] == ["df"] and alone[1][2][0] == "df"
    srv = solver.Server(precision="df", epoch_iters=48)
    ts = [srv.submit_rows(o, 0.001 * i) if k == "rows" else srv.submit_square(o, 0.001 * i)
          for i, (k, o) in enumerate(reqs)]
    for t, (xa, ia, pa) in zip(ts, alone):
        x, infs, _ = srv.wait(t)
        assert [i.iterations for i in infs] == ia and [i.precision for i in infs] == pa
        assert np.array_equal(x, xa)
    srv.close()


def test_df_with_initial_guess(gpu_ok, lscm_small):
    """x0 is packed into float pairs before the initial residual: the same
    result from the graph solver and the batched kernel, and a start at the
    solution converges at once."""
    M, b = lscm_small
    rng = np.random.default_rng(5)
    x0 = rng.standard_normal(M.n)
    x1, i1 = M.solve(b, x0=x0, precision="df")
    xs, infos, _ = solver.batch_solve([M], [b], x0s=[x0], precision="df")
    assert i1.status == "converged" and np.array_equal(xs[0], x1)
    assert infos[0].iterations == i1.iterations
    x2, i2 = M.solve(b, x0=x1, precision="df", eps=1e-6)
    assert i2.iterations <= 2 and rel(x2, x1) <= 1e-9


def test_df_out_of_range_runs_fp64(gpu_ok):
    """A matrix with entries below 2^-100 has no usable double-float copy:
    the solve runs (and reports) FP64, identical to the FP64 solve."""
    fs = systems.fairing_system(40, 40, seed=31, n_rhs=1)
    s = 2.0 ** -110
    A = solver.Matrix(fs.rp, fs.ci, fs.va * s)
    b = fs.rhs[0] * s
    x, info = A.solve(b, precision="df")
    x64, i64 = A.solve(b, precision="double")
    assert info.precision == "double" and info.status == "converged"
    assert np.array_equal(x, x64) and info.iterations == i64.iterations


def test_opennl_context_double_float(gpu_ok):
    """OpenNL context API: NL_GB300_PRECISION_DOUBLE_FLOAT on a
    least-squares system is within 1e-8 of FP64's solution at eps = 1e-12,
    and AUTO stays FP64 for least-squares systems (bit-identical to it)."""
    rs = systems.lscm_system(40, 36, seed=41)
    xa, ia = solver.solve_opennl(rs, precision="auto", eps=1e-12)
    xf, if_ = solver.solve_opennl(rs, precision="df", eps=1e-12)
    xd, id_ = solver.solve_opennl(rs, precision="double", eps=1e-12)
    # nlSolve succeeds when OpenNL's own rule (the recursive residual) is met;
    # NL_GB300_STATUS tells whether the true residual met eps too
    assert if_["ok"] and if_["status"] in ("converged", "true_residual_stalled")
    assert (if_["status"] == "converged") == (if_["true_error"] <= 1e-12)
    assert np.array_equal(xa, xd) and ia["iterations"] == id_["iterations"]
    assert rel(xf, xd) <= 1e-8
