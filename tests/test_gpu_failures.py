"""Failure paths that a running kernel can reach, exercised without faulting
the GPU:

* a team barrier of the persistent kernel whose wait runs out: with a test
  limit of 50 ms and a first team planned for one CTA more than it is given
  (test hooks NLGB_BARRIER_TIMEOUT_MS / NLGB_TEST_TEAM_SHORTFALL, read when
  a batch runner starts), the barrier gives up, the kernel flags the error
  and returns, the call reports a device error, and the GPU stays usable;
* the solve server's abort, raised while a graph solve (serial mode) or a
  persistent epoch (batched mode) is running: the host-mapped abort flag
  (polled by the graph's guard kernel once per while-loop pass) or the next
  epoch boundary stops the work, the request ends as aborted with the
  iterations it ran."""
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np
import pytest

from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

BARRIER_SCRIPT = r"""
import json, sys, time
sys.path.insert(0, sys.argv[1])
from graphitethree_gb300 import solver, systems
M, rhs, _ = solver.assemble(systems.lscm_system(40, 40, seed=4))
out = {}
t0 = time.perf_counter()
try:
    solver.batch_solve([M], [rhs[0]])
    out["batch"] = "ok"
except solver.SolverError as e:
    out["batch"] = str(e)
out["batch_s"] = time.perf_counter() - t0
x, info = M.solve(rhs[0])          # graph executor: the context is still usable
out["after"] = info.status
out["after_true"] = info.true_rel_residual
print(json.dumps(out))
"""


def test_team_barrier_timeout_is_reported_and_the_gpu_stays_usable(gpu_ok):
    env = dict(os.environ, NLGB_BARRIER_TIMEOUT_MS="50", NLGB_TEST_TEAM_SHORTFALL="1")
    p = subprocess.run([sys.executable, "-c", BARRIER_SCRIPT, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    out = json.loads(p.stdout.strip().splitlines()[-1])
    assert "barrier timed out" in out["batch"], out
    assert out["batch_s"] < 10.0
    assert out["after"] == "converged" and out["after_true"] <= 1e-10


def _lscm_square(side, seed):
    M, rhs, _ = solver.assemble(systems.lscm_system(side, side, seed=seed))
    rp, ci, va = M.download()
    return systems.SquareSystem(M.n, rp, ci, va, rhs[:1].copy())


def test_abort_stops_a_running_serial_graph_solve(gpu_ok):
    big = _lscm_square(600, 7)                      # ~720k unknowns: ~60k iterations, seconds
    srv = solver.Server(precision="double", mode="serial")
    t = srv.submit_square(big)
    time.sleep(0.5)                                  # the graph solve is running
    t_abort = time.perf_counter()
    srv.abort()
    ok, x, infos, lat = srv.wait_result(t)
    waited = time.perf_counter() - t_abort
    srv.close()
    assert not ok and infos[0].status == "aborted"
    assert 0 < infos[0].iterations < 5 * big.n
    assert waited < 2.0


def test_abort_stops_batched_epochs(gpu_ok):
    big = _lscm_square(600, 8)
    small = systems.fairing_system(60, 50, seed=9)
    srv = solver.Server(precision="double", mode="batched")
    t_big = srv.submit_square(big)
    t_small = srv.submit_square(small)
    _, info_small, _ = srv.wait(t_small)             # the small request completes normally
    assert all(i.status == "converged" for i in info_small)
    time.sleep(0.5)
    t_abort = time.perf_counter()
    srv.abort()
    ok, x, infos, lat = srv.wait_result(t_big)
    waited = time.perf_counter() - t_abort
    st = srv.stats()
    srv.close()
    assert not ok and infos[0].status == "aborted"
    assert 0 < infos[0].iterations < 5 * big.n      # the iterations run before the abort
    assert waited < 2.0
    assert st["completed"] == 1 and st["failed"] == 1
