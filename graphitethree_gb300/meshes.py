"""Seeded synthetic surface meshes for the solver workloads.

Graphite's LSCM and fairing commands run on user meshes
(``MeshGrobSurfaceCommands::parameterize_chart`` / ``smooth`` in
src/lib/OGF/mesh/commands/mesh_grob_surface_commands.cpp:687-779).  The
benchmarks use seeded grid surfaces instead:

* a height field over [0,1]^2: z = sum of Gaussian bumps with amplitude
  U(-0.1, 0.1), centre U(0,1)^2 and sigma U(0.03, 0.15);
* an nx x ny vertex grid whose quads are split along a seeded random
  diagonal (2 (nx-1)(ny-1) counter-clockwise triangles);
* optional per-row-band stretching of x (ill-conditioned fairing stress).

Vertex (i, j) (column i, row j) has index j * nx + i.
"""
from __future__ import annotations

import numpy as np


def bump_field(rng: np.random.Generator, n_bumps: int = 8):
    """Return (amp, cx, cy, sigma) arrays of a seeded bump model."""
    amp = rng.uniform(-0.1, 0.1, n_bumps)
    cx = rng.uniform(0.0, 1.0, n_bumps)
    cy = rng.uniform(0.0, 1.0, n_bumps)
    sig = rng.uniform(0.03, 0.15, n_bumps)
    return amp, cx, cy, sig


def eval_bumps(bumps, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    amp, cx, cy, sig = bumps
    z = np.zeros_like(x, dtype=np.float64)
    for a, u, v, s in zip(amp, cx, cy, sig):
        z += a * np.exp(-((x - u) ** 2 + (y - v) ** 2) / (2.0 * s * s))
    return z


def grid_faces(nx: int, ny: int, rng: np.random.Generator) -> np.ndarray:
    """Triangles of an nx x ny vertex grid, one seeded diagonal per quad."""
    i, j = np.meshgrid(np.arange(nx - 1, dtype=np.int32), np.arange(ny - 1, dtype=np.int32), indexing="xy")
    v00 = (j * np.int32(nx) + i).ravel()
    v10 = v00 + 1
    v01 = v00 + np.int32(nx)
    v11 = v01 + 1
    diag = rng.integers(0, 2, size=v00.shape[0]).astype(bool)
    # diag False: (v00,v10,v11), (v00,v11,v01); True: (v00,v10,v01), (v10,v11,v01)
    faces = np.empty((2 * v00.shape[0], 3), dtype=np.int32)
    faces[0::2, 0] = v00
    faces[0::2, 1] = v10
    faces[0::2, 2] = np.where(diag, v01, v11)
    faces[1::2, 0] = np.where(diag, v10, v00)
    faces[1::2, 1] = v11
    faces[1::2, 2] = v01
    return faces


def height_field(nx: int, ny: int, seed: int, n_bumps: int = 8, flat: bool = False,
                 stretch_bands: int = 0, stretch_max: float = 1.0e3,
                 extent: tuple[float, float] = (1.0, 1.0)):
    """Seeded height-field grid surface.  Returns (V (N,3) float64, F (M,3) int32).

    ``stretch_bands > 0`` multiplies the x coordinate of each horizontal band
    of rows by a factor drawn log-uniform in [1, stretch_max].
    """
    rng = np.random.default_rng(seed)
    bumps = bump_field(rng, n_bumps)
    xs = np.linspace(0.0, extent[0], nx)
    ys = np.linspace(0.0, extent[1], ny)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    Z = np.zeros_like(X) if flat else eval_bumps(bumps, X / max(extent[0], 1e-300), Y / max(extent[1], 1e-300))
    if stretch_bands > 0:
        f = np.exp(rng.uniform(0.0, np.log(stretch_max), stretch_bands))
        band = np.minimum((np.arange(ny) * stretch_bands) // ny, stretch_bands - 1)
        X = X * f[band][:, None]
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    F = grid_faces(nx, ny, rng)
    return V, F


def chart_sizes(n_charts: int, seed: int, side_min: int = 16, side_max: int = 512,
                aspect_max: float = 4.0):
    """Batched-atlas chart grid sizes (nx, ny).

    The long side is drawn log-uniform in [side_min, side_max] and the aspect
    ratio log-uniform in [1, aspect_max]; the short side is long/aspect
    (at least 4 vertices).
    """
    rng = np.random.default_rng(seed)
    long_side = np.exp(rng.uniform(np.log(side_min), np.log(side_max), n_charts))
    aspect = np.exp(rng.uniform(0.0, np.log(aspect_max), n_charts))
    nx = np.maximum(4, np.rint(long_side)).astype(np.int64)
    ny = np.maximum(4, np.rint(long_side / aspect)).astype(np.int64)
    return nx, ny
