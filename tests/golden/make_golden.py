"""Generate the golden fixtures of tests/golden/ (run from the repo root:
``python tests/golden/make_golden.py``).

OpenNL's source is not part of the reference checkout, so these vectors are
produced by methods independent of both the GPU library and the C oracle:

* normal equations by dense numpy algebra (A_f^T W A_f, A_f^T W (b - A_l x_l));
* solutions by scipy's SuperLU direct solver;
* analytic known answers: a flat grid's LSCM map is the identity u = x,
  v = y (pins (0,0) and (1,1)); (L + lam I)(c 1) = lam c 1 for the cotangent
  Laplacian; hand-checkable 2x2 / 3x3 systems.

Every fixture is a small .npz holding the row stream (the inputs of the
OpenNL call sequence) and the expected outputs.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from graphitethree_gb300 import meshes, systems  # noqa: E402


def dense_normal(rs):
    n_rows = rs.n_rows
    A = np.zeros((n_rows, rs.n_vars))
    for r in range(n_rows):
        for k in range(rs.row_ptr[r], rs.row_ptr[r + 1]):
            A[r, rs.var[k]] += rs.val[k]
    w = np.ones(n_rows) if rs.weight is None else rs.weight
    free = rs.locked == 0
    Af, Al = A[:, free], A[:, ~free]
    if rs.least_squares:
        M = (Af * w[:, None]).T @ Af
        rhs = np.array([(Af * w[:, None]).T @ (rs.rhs[:, s] - Al @ rs.values[s][~free])
                        for s in range(rs.n_systems)])
    else:
        M = Af
        rhs = np.array([rs.rhs[:, s] - Al @ rs.values[s][~free] for s in range(rs.n_systems)])
    return M, rhs


def save(name, rs, extra=None):
    import scipy.linalg as la
    M, rhs = dense_normal(rs)
    sol = np.array([la.solve(M, rhs[s], assume_a="sym") for s in range(rs.n_systems)])
    d = dict(n_vars=rs.n_vars, row_ptr=rs.row_ptr, var=rs.var, val=rs.val, rhs=rs.rhs,
             locked=rs.locked, values=rs.values, least_squares=int(rs.least_squares),
             weight=rs.weight if rs.weight is not None else np.zeros(0),
             has_weight=int(rs.weight is not None), normal_dense=M, normal_rhs=rhs, solution=sol)
    if extra:
        d.update(extra)
    np.savez_compressed(Path(__file__).parent / f"{name}.npz", **d)
    print(name, "n_free", M.shape[0], "rows", rs.n_rows)


def main():
    # 1. LSCM on a small bumpy grid (the config-1 shape, reduced).
    save("lscm_bumps_12x10", systems.lscm_system(12, 10, seed=11))
    # 2. LSCM on a flat grid: analytic answer u = x, v = y.
    V, F = meshes.height_field(9, 8, seed=2, flat=True)
    rs = systems.lscm_rows(V, F)
    save("lscm_flat_9x8", rs, {"exact": V[:, :2].ravel()})
    # 3. WarpDrive-style periodic 7-point voxel rows, locked data voxels.
    save("voxel_6x5x4", systems.voxel_rows(6, 5, 4, seed=4, locked_fraction=0.35))
    # 4. Cotangent Laplacian + lam I, square mode, three right-hand sides.
    fs = systems.fairing_system(9, 9, seed=3, lam=1e-2)
    save("fairing_9x9", fs.to_rows())
    # 5. Constant right-hand side: (L + lam I)(c 1) = lam c 1.
    fs = systems.fairing_system(8, 11, seed=5, lam=0.5, n_rhs=1)
    fs.rhs[:] = 0.5 * 2.5
    save("fairing_const", fs.to_rows(), {"exact": np.full(fs.n, 2.5)})
    # 6. Hand-checkable least squares with weights, duplicates and a lock:
    #    rows: x0 + x1 = 3 (w=2), x0 - x1 = 1, x1 + x1 + x2 = 5 (dup), x2 = 4 (x2 locked = 4)
    rs = systems.RowStream(
        n_vars=3, row_ptr=np.array([0, 2, 4, 7, 8], np.int64),
        var=np.array([0, 1, 0, 1, 1, 1, 2, 2], np.int32),
        val=np.array([1.0, 1.0, 1.0, -1.0, 1.0, 1.0, 1.0, 1.0]),
        rhs=np.array([[3.0], [1.0], [5.0], [4.0]]), locked=np.array([0, 0, 1], np.uint8),
        values=np.array([[0.0, 0.0, 4.0]]), least_squares=True, weight=np.array([2.0, 1.0, 1.0, 1.0]))
    save("hand_ls_3var", rs)
    # 7. Hand-checkable square SPD system (2x2): [[4,1],[1,3]] x = [1,2].
    rs = systems.RowStream(
        n_vars=2, row_ptr=np.array([0, 2, 4], np.int64), var=np.array([0, 1, 0, 1], np.int32),
        val=np.array([4.0, 1.0, 1.0, 3.0]), rhs=np.array([[1.0], [2.0]]),
        locked=np.zeros(2, np.uint8), values=np.zeros((1, 2)), least_squares=False)
    save("hand_spd_2x2", rs, {"exact": np.array([1.0 / 11.0, 7.0 / 11.0])})


if __name__ == "__main__":
    main()
