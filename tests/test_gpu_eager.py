"""Eager mode (NLGB_EAGER_SOLVE=1, read once per process): the solver's
kernels launched one by one instead of through conditional CUDA graphs, so
that a profiler sees each of them.  Same kernels, same order: results must
be bit-identical to the graph path, in every precision (FP64, mixed,
double-float)."""
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from graphitethree_gb300 import solver, systems

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from graphitethree_gb300 import solver, systems
M, rhs, _ = solver.assemble(systems.lscm_system(40, 37, seed=4))
fs = systems.fairing_system(70, 60, seed=5, n_rhs=1)
F = solver.Matrix(fs.rp, fs.ci, fs.va)
out = {}
for name, A, b in (("lscm", M, rhs[0]), ("fair", F, fs.rhs[0])):
    for prec in ("double", "mixed", "df"):
        x, info = A.solve(b, precision=prec)
        out[f"{name}_{prec}"] = {"x": x.tolist(), "it": info.iterations, "status": info.status}
big = systems.fairing_system(420, 400, seed=21, n_rhs=1)
srv = solver.Server(precision="double", epoch_iters=32)
xb, ib, _ = srv.wait(srv.submit_square(big))
srv.close()
out["server_graph_chunks"] = {"x": xb[0].tolist(), "it": ib[0].iterations, "status": ib[0].status}
np.save(sys.argv[2], np.array([json.dumps(out)]))
"""


def test_eager_mode_bit_identical(gpu_ok, tmp_path):
    target = tmp_path / "eager.npy"
    env = dict(os.environ, NLGB_EAGER_SOLVE="1")
    subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT), str(target)], env=env, check=True,
                   timeout=300)
    eager = json.loads(str(np.load(target)[0]))
    M, rhs, _ = solver.assemble(systems.lscm_system(40, 37, seed=4))
    fs = systems.fairing_system(70, 60, seed=5, n_rhs=1)
    F = solver.Matrix(fs.rp, fs.ci, fs.va)
    for name, A, b in (("lscm", M, rhs[0]), ("fair", F, fs.rhs[0])):
        for prec in ("double", "mixed", "df"):
            x, info = A.solve(b, precision=prec)
            e = eager[f"{name}_{prec}"]
            assert e["status"] == info.status == "converged"
            assert e["it"] == info.iterations
            assert np.array_equal(np.array(e["x"]), x)
    # the server's lone-large-system graph chunks, eager vs graph
    big = systems.fairing_system(420, 400, seed=21, n_rhs=1)
    srv = solver.Server(precision="double", epoch_iters=32)
    xb, ib, _ = srv.wait(srv.submit_square(big))
    srv.close()
    e = eager["server_graph_chunks"]
    assert e["status"] == ib[0].status == "converged" and e["it"] == ib[0].iterations
    assert np.array_equal(np.array(e["x"]), xb[0])
