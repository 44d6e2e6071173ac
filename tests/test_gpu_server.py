"""Solve server: continuous batching under an HBM budget.  Each result must
be the same alone and in the mix (bit-identical here, which is stronger than
the 1e-8 solution tolerance the solver guarantees), admission must respect
the budget, and failures must be reported, not hung."""
import numpy as np
import pytest

from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu


def _requests():
    reqs = []
    for side, seed in [(40, 1), (18, 2), (70, 3)]:
        reqs.append(("rows", systems.lscm_system(side, side - 3, seed=seed)))
    for side, seed in [(50, 4), (25, 5), (90, 6)]:
        reqs.append(("square", systems.fairing_system(side, side + 7, seed=seed)))
    return reqs


def _submit(srv, kind, obj, arrival=-1.0):
    return srv.submit_rows(obj, arrival) if kind == "rows" else srv.submit_square(obj, arrival)


@pytest.mark.parametrize("schedule", ["srpt", "all"])
@pytest.mark.parametrize("precision", ["mixed", "double", "auto"])
def test_result_same_alone_and_in_mix(gpu_ok, precision, schedule):
    reqs = _requests()
    alone = []
    for kind, obj in reqs:
        srv = solver.Server(precision=precision, budget_bytes=2e9)
        t = _submit(srv, kind, obj)
        x, infos, lat = srv.wait(t)
        alone.append((x.copy(), [i.iterations for i in infos]))
        srv.close()
    # short epochs (0.5 ms time box, or 64 iterations), so that every
    # system crosses several epoch boundaries in the mix
    srv = solver.Server(precision=precision, budget_bytes=2e9, epoch_iters=64, schedule=schedule,
                        epoch_ms=0.5)
    tickets = [_submit(srv, kind, obj, arrival=0.002 * i) for i, (kind, obj) in enumerate(reqs)]
    for t, (xa, ia) in zip(tickets, alone):
        x, infos, lat = srv.wait(t)
        assert all(i.status == "converged" for i in infos), infos
        assert [i.iterations for i in infos] == ia
        assert np.array_equal(x, xa)
        assert lat >= 0
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["epochs"] >= 2 and st["solves_per_s"] > 0
    srv.close()


def test_server_matches_oracle_and_single_solver(gpu_ok, oracle_mod):
    # LSCM normal equations are ill-conditioned: compare with the direct
    # solution at relative residual 1e-12 (at 1e-10 two correct CG runs can
    # differ from it by more than 1e-8).
    rs = systems.lscm_system(45, 40, seed=7)
    fs = systems.fairing_system(60, 60, seed=8)
    srv = solver.Server(precision="mixed", eps=1e-12)
    t1 = srv.submit_rows(rs)
    t2 = srv.submit_square(fs)
    x1, i1, _ = srv.wait(t1)
    x2, i2, _ = srv.wait(t2)
    rp, ci, va, rhs = oracle_mod.assemble_rowstream(rs)
    xd = oracle_mod.direct_solve(rp, ci, va, rhs[0])
    assert np.linalg.norm(x1[0] - xd) / np.linalg.norm(xd) <= 1e-8
    for k in range(3):
        xf = oracle_mod.direct_solve(fs.rp, fs.ci, fs.va, fs.rhs[k])
        assert np.linalg.norm(x2[k] - xf) / np.linalg.norm(xf) <= 1e-8
        assert i2[k].true_rel_residual <= 1e-12
    # the mixed server equals the single-system mixed solver bit for bit
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    xs, info = F.solve(fs.rhs[1], precision="mixed", eps=1e-12)
    assert np.array_equal(xs, x2[1])
    srv.close()


@pytest.mark.parametrize("mode", ["batched", "serial"])
def test_least_squares_tolerance_applies_to_lscm_only(gpu_ok, mode):
    """eps_least_squares: the LSCM (least-squares) request stops at its own
    threshold, the square one at eps; each result equals the single-system
    solver's at that threshold bit for bit."""
    rs = systems.lscm_system(40, 36, seed=21)
    fs = systems.fairing_system(50, 44, seed=22)
    srv = solver.Server(precision="auto", mode=mode, eps=1e-10, eps_least_squares=3e-11)
    t1, t2 = srv.submit_rows(rs), srv.submit_square(fs)
    x1, i1, _ = srv.wait(t1)
    x2, i2, _ = srv.wait(t2)
    srv.close()
    assert i1[0].status == "converged" and i1[0].true_rel_residual <= 3e-11
    assert all(i.status == "converged" and i.true_rel_residual <= 1e-10 for i in i2)
    M, rhs, _ = solver.assemble(rs)
    x_ref, inf = M.solve(rhs[0], eps=3e-11)
    assert inf.iterations == i1[0].iterations and np.array_equal(x_ref, x1[0])
    x_loose, inf_loose = M.solve(rhs[0], eps=1e-10)
    assert inf_loose.iterations < i1[0].iterations
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in range(3):
        assert F.solve(fs.rhs[k], precision="mixed", eps=1e-10)[1].iterations == i2[k].iterations


@pytest.mark.parametrize("schedule", ["srpt", "all"])
def test_min_tile_rows_changes_only_the_layout(gpu_ok, schedule):
    """min_tile_rows: the batched server cuts each system into tiles of at
    least that many rows; chunk_cta_budget holds back chunks that would not
    fit the budget.  Results are bit-identical alone and in the mix,
    and equal the single-system solver's on a matrix given the same layout;
    a system smaller than one tile runs as a single tile."""
    reqs = _requests()
    alone = []
    for kind, obj in reqs:
        srv = solver.Server(precision="auto", budget_bytes=2e9, min_tile_rows=1000)   # -> 1024
        x, infos, _ = srv.wait(_submit(srv, kind, obj))
        alone.append((x.copy(), [i.iterations for i in infos]))
        srv.close()
    # a CTA budget of 8 lets only a few of these 1-10-tile systems run at once
    srv = solver.Server(precision="auto", budget_bytes=2e9, min_tile_rows=1024, epoch_iters=64,
                        schedule=schedule, epoch_ms=0.5, chunk_cta_budget=8)
    tickets = [_submit(srv, kind, obj, arrival=0.002 * i) for i, (kind, obj) in enumerate(reqs)]
    for t, (xa, ia) in zip(tickets, alone):
        x, infos, _ = srv.wait(t)
        assert all(i.status == "converged" for i in infos)
        assert [i.iterations for i in infos] == ia and np.array_equal(x, xa)
    srv.close()
    for (kind, obj), (xa, ia) in zip(reqs, alone):
        if kind == "rows":
            M, rhs, _ = solver.assemble(obj)
            bs, prec = [rhs[0]], "double"
        else:
            M, bs, prec = solver.Matrix(obj.rp, obj.ci, obj.va), list(obj.rhs), "mixed"
        if M.tile_rows < 1024:
            M.set_layout(0, 1024)
        for k, b in enumerate(bs):
            xs, inf = M.solve(b, precision=prec)
            assert inf.iterations == ia[k] and np.array_equal(xs, xa[k])
        M.close()


def test_budget_admission_queues_and_rejects(gpu_ok):
    fs = [systems.fairing_system(64, 64, seed=s) for s in range(6)]
    one = solver.Server(budget_bytes=1e9)
    t = one.submit_square(fs[0])
    one.wait(t)
    foot = one.stats()["peak_bytes"]
    one.close()
    # room for about two requests at a time: all complete, peak stays in budget
    srv = solver.Server(budget_bytes=int(2.5 * foot))
    ts = [srv.submit_square(f) for f in fs]
    for t in ts:
        x, infos, _ = srv.wait(t)
        assert all(i.status == "converged" for i in infos)
    st = srv.stats()
    assert st["peak_bytes"] <= 2.5 * foot and st["completed"] == 6
    # a request larger than the whole budget is rejected up front
    with pytest.raises(solver.SolverError):
        srv.submit_square(systems.fairing_system(400, 400, seed=1))
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_serial_mode_equals_graph_solver(gpu_ok):
    fs = systems.fairing_system(70, 50, seed=3)
    srv = solver.Server(mode="serial", precision="double")
    x, infos, _ = srv.wait(srv.submit_square(fs))
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    for k in range(3):
        xk, ik = F.solve(fs.rhs[k])
        assert np.array_equal(xk, x[k]) and ik.iterations == infos[k].iterations
    srv.close()


def test_abort_fails_waiting_requests(gpu_ok):
    srv = solver.Server()
    t = srv.submit_square(systems.fairing_system(30, 30, seed=1), arrival=3600.0)
    srv.abort()
    with pytest.raises(solver.SolverError):
        srv.wait(t)
    assert srv.stats()["failed"] == 1
    srv.close()


def test_auto_precision_least_squares_in_fp64(gpu_ok):
    """AUTO: least-squares row submissions start in FP64 (no FP32 phase, no
    reliable update; iterates identical to the FP64 server), square systems
    run in mixed precision (reliable updates, same result as the mixed
    server)."""
    rs = systems.lscm_system(44, 41, seed=11)
    fs = systems.fairing_system(64, 60, seed=12)
    out = {}
    for precision in ("auto", "double", "mixed"):
        srv = solver.Server(precision=precision)
        t1, t2 = srv.submit_rows(rs), srv.submit_square(fs)
        out[precision] = (srv.wait(t1), srv.wait(t2))
        srv.close()
    (xa1, ia1, _), (xa2, ia2, _) = out["auto"]
    (xd1, id1, _), _ = out["double"]
    _, (xm2, im2, _) = out["mixed"]
    assert ia1[0].status == "converged" and ia1[0].refinement_steps == 0
    assert ia1[0].precision == id1[0].precision == "double"
    assert np.array_equal(xa1, xd1) and ia1[0].iterations == id1[0].iterations
    assert all(i.status == "converged" and i.refinement_steps >= 1 for i in ia2)
    assert all(i.precision == "mixed" for i in ia2)
    assert np.array_equal(xa2, xm2)


def test_lone_large_system_continues_on_graph(gpu_ok):
    """A large FP64 system alone in the server runs its first epoch in the
    persistent kernel, then continues in CUDA-graph chunks: the result is the
    same as the graph solver's and the persistent kernel's, bit for bit."""
    fs = systems.fairing_system(420, 400, seed=21, n_rhs=1)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    assert A.n // A.tile_rows >= 384
    x1, i1 = A.solve(fs.rhs[0])
    xs, infos, _ = solver.batch_solve([A], [fs.rhs[0]])
    srv = solver.Server(precision="double", epoch_iters=32, schedule="all")
    t = srv.submit_square(fs)
    x, infs, _ = srv.wait(t)
    st = srv.stats()
    srv.close()
    assert infs[0].status == "converged" and st["epochs"] >= 3
    assert infs[0].iterations == i1.iterations == infos[0].iterations
    assert np.array_equal(x[0], x1) and np.array_equal(x[0], xs[0])


def test_switch_back_from_graph_when_requests_arrive(gpu_ok):
    """A large least-squares system runs alone (graph chunks) until a small
    request arrives; both then share persistent-kernel epochs.  Each result
    equals its solve alone."""
    big = systems.lscm_system(200, 190, seed=31)
    small = systems.fairing_system(40, 37, seed=32)
    alone = []
    for kind, obj in (("rows", big), ("square", small)):
        srv = solver.Server(precision="auto", epoch_iters=64, schedule="all")
        x, infs, _ = srv.wait(_submit(srv, kind, obj))
        alone.append((x.copy(), [i.iterations for i in infs]))
        srv.close()
    srv = solver.Server(precision="auto", epoch_iters=64, schedule="all")
    t1 = _submit(srv, "rows", big, arrival=0.0)
    t2 = _submit(srv, "square", small, arrival=0.05)
    for t, (xa, ia) in zip((t1, t2), alone):
        x, infs, _ = srv.wait(t)
        assert all(i.status == "converged" for i in infs)
        assert [i.iterations for i in infs] == ia
        assert np.array_equal(x, xa)
    srv.close()


def test_large_systems_share_graph_epochs(gpu_ok):
    """Two large FP64 systems and nothing else: after their first epoch both
    continue as graph chunks within the same epochs; each result equals its
    own single-system solve bit for bit."""
    fa = systems.fairing_system(420, 400, seed=41, n_rhs=1)
    fb = systems.fairing_system(400, 410, seed=42, n_rhs=1)
    alone = []
    for fs in (fa, fb):
        A = solver.Matrix(fs.rp, fs.ci, fs.va)
        assert A.n // A.tile_rows >= 384
        alone.append(A.solve(fs.rhs[0]))
    srv = solver.Server(precision="double", epoch_iters=32, schedule="all")
    ta, tb = srv.submit_square(fa), srv.submit_square(fb)
    for t, (x1, i1) in zip((ta, tb), alone):
        x, infs, _ = srv.wait(t)
        assert infs[0].status == "converged" and infs[0].iterations == i1.iterations
        assert np.array_equal(x[0], x1)
    st = srv.stats()
    srv.close()
    assert st["graph_epochs"] >= 2 and st["graph_s"] > 0


def test_graph_continuation_after_slot_reuse(gpu_ok):
    """Two different large systems of the same size, one after the other in
    one server: the second's slot may come back at the first's addresses
    (stream-ordered pool); its graph chunks must run on its own matrix."""
    fa = systems.fairing_system(420, 400, seed=51, n_rhs=1)
    fb = systems.fairing_system(420, 400, seed=52, n_rhs=1, lam=3e-2)
    srv = solver.Server(precision="double", epoch_iters=32, schedule="all")
    for fs in (fa, fb):
        A = solver.Matrix(fs.rp, fs.ci, fs.va)
        x1, i1 = A.solve(fs.rhs[0])
        x, infs, _ = srv.wait(srv.submit_square(fs))
        assert infs[0].status == "converged" and infs[0].iterations == i1.iterations
        assert np.array_equal(x[0], x1)
    assert srv.stats()["graph_epochs"] >= 2
    srv.close()


def test_srpt_serves_light_requests_first(gpu_ok):
    """SRPT epochs: a large least-squares request submitted first does not
    hold back light requests that arrive after it; every result is still
    bit-identical to its solve alone."""
    big = systems.lscm_system(260, 250, seed=61)
    lights = [systems.fairing_system(50 + 7 * i, 45, seed=62 + i) for i in range(4)]
    srv = solver.Server(precision="auto")
    x_big_alone, i_big_alone, _ = srv.wait(srv.submit_rows(big))
    alone = [srv.wait(srv.submit_square(f))[:2] for f in lights]
    srv.close()
    srv = solver.Server(precision="auto")
    t_big = srv.submit_rows(big, arrival=0.0)
    t_l = [srv.submit_square(f, arrival=0.01) for f in lights]
    lat_l = []
    for t, (xa, ia) in zip(t_l, alone):
        x, infs, lat = srv.wait(t)
        assert all(i.status == "converged" for i in infs)
        assert [i.iterations for i in infs] == [i.iterations for i in ia]
        assert np.array_equal(x, xa)
        lat_l.append(lat)
    x, infs, lat_big = srv.wait(t_big)
    srv.close()
    assert infs[0].iterations == i_big_alone[0].iterations and np.array_equal(x, x_big_alone)
    assert max(lat_l) < lat_big


def test_srpt_chunks_follow_their_target_length(gpu_ok, tmp_path, monkeypatch):
    """SRPT executor: after a system's 16-iteration probe, its chunks are
    sized from its measured time per iteration to last about epoch_ms
    (trace of the chunks, NLGB_SERVER_TRACE)."""
    trace = tmp_path / "trace.csv"
    monkeypatch.setenv("NLGB_SERVER_TRACE", str(trace))
    reqs = [systems.lscm_system(120 + 3 * i, 110, seed=71 + i) for i in range(6)]
    srv = solver.Server(precision="double", epoch_ms=5.0)
    tickets = [srv.submit_rows(r) for r in reqs]
    for t in tickets:
        x, infs, _ = srv.wait(t)
        assert infs[0].status == "converged"
    srv.close()
    rows = [l.split(",") for l in trace.read_text().splitlines() if l.startswith("C,")]
    iters = np.array([int(r[6]) - int(r[5]) for r in rows])
    ms = np.array([float(r[7]) for r in rows])
    assert (iters <= 16).sum() >= len(reqs)                 # one probe per system
    long_ = ms[iters > 16]
    assert len(long_) >= 6
    assert 1.0 <= float(np.median(long_)) <= 15.0, ms
