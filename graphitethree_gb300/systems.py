"""System builders on top of the seeded meshes: LSCM rows, cotangent
Laplacian fairing, the WarpDrive voxel-interpolation fixture, and the
request streams of the batched / serving workloads.

These restate, from the published mathematics, what geogram's builders hand
to OpenNL behind Graphite's commands:

* LSCM (Levy, Petitjean, Ray, Maillot, SIGGRAPH 2002), called through
  ``mesh_compute_LSCM`` at src/lib/OGF/mesh/commands/
  mesh_grob_surface_commands.cpp:759: per triangle, the complex conformality
  equation  sum_j E_j U_j = 0  (E_j = q_{j+2} - q_{j+1}, the edge opposite
  vertex j in the triangle's own orthonormal frame, U_j = u_j + i v_j),
  weighted by 1/sqrt(2 area), gives one real and one imaginary row of six
  coefficients; two pinned vertices are locked.  Solved in NL_LEAST_SQUARES
  mode.
* Fairing (``mesh_smooth`` behind mesh_grob_surface_commands.cpp:703): the
  cotangent Laplacian L (Pinkall-Polthier) plus lambda I, an SPD matrix
  given row by row in square (non least-squares) mode, one right-hand side
  lambda * p~ per coordinate.
* The periodic 7-point voxel rows of plugins/OGF/WarpDrive/commands/
  voxel_grob_transport_commands.cpp:256-276 (least squares, locked data
  voxels).

Variable numbering: LSCM u of vertex v is 2v, its v is 2v+1.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import meshes


@dataclass
class RowStream:
    """OpenNL rows: row r = coefficients (var[k], val[k]) for k in
    [row_ptr[r], row_ptr[r+1]), right-hand side rhs[r, s] for system s."""
    n_vars: int
    row_ptr: np.ndarray          # int64 (n_rows + 1)
    var: np.ndarray              # int32 variable indices
    val: np.ndarray              # float64
    rhs: np.ndarray              # float64 (n_rows, n_systems)
    locked: np.ndarray           # uint8 (n_vars,)
    values: np.ndarray           # float64 (n_systems, n_vars): locked values / initial guess
    least_squares: bool = True
    weight: np.ndarray | None = None

    @property
    def n_rows(self) -> int:
        return int(self.row_ptr.shape[0] - 1)

    @property
    def n_systems(self) -> int:
        return int(self.rhs.shape[1])

    def free_vars(self) -> np.ndarray:
        return np.flatnonzero(self.locked == 0).astype(np.int32)

    def encoded_cols(self) -> np.ndarray:
        """Column encoding of the device row stream: free index >= 0, or
        -(var+1) for a locked variable."""
        fidx = np.full(self.n_vars, -1, dtype=np.int64)
        fv = self.free_vars()
        fidx[fv] = np.arange(fv.shape[0])
        f = fidx[self.var]
        return np.where(f >= 0, f, -(self.var.astype(np.int64) + 1)).astype(np.int32)


@dataclass
class SquareSystem:
    """An SPD system given directly in CRS form (int32 indices, FP64 values)."""
    n: int
    rp: np.ndarray
    ci: np.ndarray
    va: np.ndarray
    rhs: np.ndarray              # (n_systems, n)
    meta: dict = field(default_factory=dict)

    @property
    def nnz(self) -> int:
        return int(self.rp[-1])

    def to_rows(self) -> RowStream:
        n = self.n
        return RowStream(
            n_vars=n, row_ptr=self.rp.astype(np.int64), var=self.ci.astype(np.int32),
            val=self.va.astype(np.float64), rhs=np.ascontiguousarray(self.rhs.T),
            locked=np.zeros(n, np.uint8), values=np.zeros((self.rhs.shape[0], n)),
            least_squares=False)


# ---------------------------------------------------------------------------
# LSCM
# ---------------------------------------------------------------------------
def lscm_coefficients(V: np.ndarray, F: np.ndarray):
    """Per triangle: (a_j, b_j) = (Re, Im) of E_j / sqrt(2 area), j = 0..2."""
    p0, p1, p2 = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    e1 = p1 - p0
    e2 = p2 - p0
    l1 = np.linalg.norm(e1, axis=1)
    X = e1 / np.where(l1 > 0, l1, 1.0)[:, None]
    N = np.cross(e1, e2)
    nN = np.linalg.norm(N, axis=1)
    Y = np.cross(N / np.where(nN > 0, nN, 1.0)[:, None], X)
    x1 = l1
    x2 = np.einsum("ij,ij->i", e2, X)
    y2 = np.einsum("ij,ij->i", e2, Y)
    d = x1 * y2                          # twice the area (> 0 for valid triangles)
    s = np.where(d > 0, 1.0 / np.sqrt(np.where(d > 0, d, 1.0)), 0.0)
    # E_0 = q2 - q1, E_1 = q0 - q2, E_2 = q1 - q0 with q0 = 0, q1 = (x1, 0), q2 = (x2, y2)
    a = np.stack([(x2 - x1) * s, -x2 * s, x1 * s], axis=1)
    b = np.stack([y2 * s, -y2 * s, np.zeros_like(x1)], axis=1)
    return a, b


def lscm_rows(V: np.ndarray, F: np.ndarray, pins: tuple[int, int] | None = None,
              pin_uv=((0.0, 0.0), (1.0, 1.0))) -> RowStream:
    """LSCM least-squares rows with two locked pinned vertices."""
    nv = V.shape[0]
    T = F.shape[0]
    a, b = lscm_coefficients(V, F)
    vu = 2 * F.astype(np.int64)          # u variables
    vv = vu + 1                          # v variables
    var = np.empty((T, 2, 6), dtype=np.int64)
    val = np.empty((T, 2, 6), dtype=np.float64)
    for j in range(3):
        var[:, 0, 2 * j] = vu[:, j]
        var[:, 0, 2 * j + 1] = vv[:, j]
        var[:, 1, 2 * j] = vu[:, j]
        var[:, 1, 2 * j + 1] = vv[:, j]
        val[:, 0, 2 * j] = a[:, j]        # real row: a u - b v
        val[:, 0, 2 * j + 1] = -b[:, j]
        val[:, 1, 2 * j] = b[:, j]        # imaginary row: b u + a v
        val[:, 1, 2 * j + 1] = a[:, j]
    n_rows = 2 * T
    if pins is None:
        pins = (0, nv - 1)
    locked = np.zeros(2 * nv, np.uint8)
    values = np.zeros((1, 2 * nv))
    for p, (pu, pv) in zip(pins, pin_uv):
        locked[2 * p] = locked[2 * p + 1] = 1
        values[0, 2 * p] = pu
        values[0, 2 * p + 1] = pv
    return RowStream(
        n_vars=2 * nv, row_ptr=np.arange(0, 6 * n_rows + 1, 6, dtype=np.int64),
        var=var.reshape(-1).astype(np.int32), val=val.reshape(-1),
        rhs=np.zeros((n_rows, 1)), locked=locked, values=values, least_squares=True)


# ---------------------------------------------------------------------------
# Cotangent Laplacian
# ---------------------------------------------------------------------------
def cotan_weights(V: np.ndarray, F: np.ndarray):
    """Edge list (i, j, w_ij) with w_ij = (cot alpha + cot beta) / 2 summed
    over the triangles sharing the edge."""
    I, J, W = [], [], []
    for k in range(3):
        i = F[:, (k + 1) % 3]
        j = F[:, (k + 2) % 3]
        u = V[i] - V[F[:, k]]
        v = V[j] - V[F[:, k]]
        cr = np.linalg.norm(np.cross(u, v), axis=1)
        cot = np.einsum("ij,ij->i", u, v) / np.where(cr > 0, cr, 1.0)
        cot = np.where(cr > 0, cot, 0.0)
        I.append(i); J.append(j); W.append(0.5 * cot)
    return np.concatenate(I), np.concatenate(J), np.concatenate(W)


def csr_from_coo(n: int, I: np.ndarray, J: np.ndarray, W: np.ndarray):
    """Sum duplicates; columns sorted within each row (deterministic order)."""
    I = I.astype(np.int64)
    J = J.astype(np.int64)
    key = I * n + J
    order = np.argsort(key, kind="stable")
    key = key[order]
    W = W[order]
    uniq, start = np.unique(key, return_index=True)
    vals = np.add.reduceat(W, start) if W.size else W
    rows = uniq // n
    cols = uniq % n
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    return rp.astype(np.int32), cols.astype(np.int32), vals.astype(np.float64)


def cotan_laplacian(V: np.ndarray, F: np.ndarray, lam: float):
    """CRS of L + lam I (L_ij = -w_ij, L_ii = sum_j w_ij)."""
    n = V.shape[0]
    i, j, w = cotan_weights(V, F)
    I = np.concatenate([i, j, i, j, np.arange(n)])
    J = np.concatenate([j, i, i, j, np.arange(n)])
    W = np.concatenate([-w, -w, w, w, np.full(n, lam)])
    return csr_from_coo(n, I, J, W)


def fairing_system(nx: int, ny: int, seed: int, lam: float = 1e-2, noise: float = 1e-3,
                   n_rhs: int = 3, stretch_bands: int = 0, rhs_normal: bool = False) -> SquareSystem:
    """(L + lam I) x = lam (p + noise) per coordinate (or N(0,1) entries)."""
    V, F = meshes.height_field(nx, ny, seed, stretch_bands=stretch_bands)
    rp, ci, va = cotan_laplacian(V, F, lam)
    rng = np.random.default_rng(seed + 7919)
    if rhs_normal:
        rhs = rng.standard_normal((n_rhs, V.shape[0]))
    else:
        P = V[:, :n_rhs].T.copy()
        rhs = lam * (P + rng.normal(0.0, noise, P.shape))
    return SquareSystem(n=V.shape[0], rp=rp, ci=ci, va=va, rhs=np.ascontiguousarray(rhs),
                        meta={"kind": "fairing", "nx": nx, "ny": ny, "seed": seed, "lam": lam})


def lscm_system(nx: int, ny: int, seed: int, flat: bool = False) -> RowStream:
    V, F = meshes.height_field(nx, ny, seed, flat=flat)
    return lscm_rows(V, F)


# ---------------------------------------------------------------------------
# Non-symmetric test system (BiCGSTAB / GMRES)
# ---------------------------------------------------------------------------
def convection_diffusion(nx: int, ny: int, seed: int, wind=(40.0, 25.0), reaction: float = 2e4,
                         n_rhs: int = 1) -> SquareSystem:
    """-lap u + w . grad u + c u on the unit square, Dirichlet boundary,
    first-order upwind differences on an nx x ny interior grid, c(x) seeded
    uniform in [0, reaction]: a non-symmetric M-matrix with a varying
    diagonal (the structure of a linearised transport step).  Right-hand
    sides N(0, 1), seeded."""
    hx, hy = 1.0 / (nx + 1), 1.0 / (ny + 1)
    wx, wy = wind
    n = nx * ny
    I, J, W = [], [], []
    k = np.arange(n)
    i, j = k % nx, k // nx
    rng = np.random.default_rng(seed)
    diag = 2.0 / hx**2 + 2.0 / hy**2 + abs(wx) / hx + abs(wy) / hy + rng.uniform(0.0, reaction, n)
    I.append(k); J.append(k); W.append(diag)
    for di, dj, c in ((-1, 0, -1.0 / hx**2 - max(wx, 0.0) / hx), (1, 0, -1.0 / hx**2 + min(wx, 0.0) / hx),
                      (0, -1, -1.0 / hy**2 - max(wy, 0.0) / hy), (0, 1, -1.0 / hy**2 + min(wy, 0.0) / hy)):
        ok = (i + di >= 0) & (i + di < nx) & (j + dj >= 0) & (j + dj < ny)
        I.append(k[ok]); J.append((k + di + dj * nx)[ok]); W.append(np.full(int(ok.sum()), c))
    rp, ci, va = csr_from_coo(n, np.concatenate(I), np.concatenate(J), np.concatenate(W))
    rhs = rng.standard_normal((n_rhs, n))
    return SquareSystem(n=n, rp=rp, ci=ci, va=va, rhs=rhs,
                        meta={"kind": "convection-diffusion", "nx": nx, "ny": ny, "seed": seed})


# ---------------------------------------------------------------------------
# WarpDrive voxel interpolation fixture (least squares, locked data voxels)
# ---------------------------------------------------------------------------
def voxel_rows(nu: int, nv: int, nw: int, seed: int, locked_fraction: float = 0.3) -> RowStream:
    rng = np.random.default_rng(seed)
    n = nu * nv * nw
    u, v, w = np.meshgrid(np.arange(nu), np.arange(nv), np.arange(nw), indexing="ij")
    u = u.transpose(2, 1, 0).ravel(); v = v.transpose(2, 1, 0).ravel(); w = w.transpose(2, 1, 0).ravel()
    lin = lambda a, b, c: (c * nv + b) * nu + a
    cols = np.stack([lin(u, v, w), lin((u + nu - 1) % nu, v, w), lin((u + 1) % nu, v, w),
                     lin(u, (v + nv - 1) % nv, w), lin(u, (v + 1) % nv, w),
                     lin(u, v, (w + nw - 1) % nw), lin(u, v, (w + 1) % nw)], axis=1)
    vals = np.tile(np.array([-6.0, 1, 1, 1, 1, 1, 1]), (n, 1))
    locked = (rng.random(n) < locked_fraction).astype(np.uint8)
    values = np.where(locked == 1, rng.random(n), 0.0)[None, :]
    return RowStream(n_vars=n, row_ptr=np.arange(0, 7 * n + 1, 7, dtype=np.int64),
                     var=cols.reshape(-1).astype(np.int32), val=vals.reshape(-1),
                     rhs=np.zeros((n, 1)), locked=locked, values=values, least_squares=True)


# ---------------------------------------------------------------------------
# Request streams (batched atlas / serving)
# ---------------------------------------------------------------------------
@dataclass
class Request:
    rid: int
    kind: str           # "lscm" or "fairing"
    nx: int
    ny: int
    seed: int
    arrival: float      # seconds after stream start


def request_stream(n_requests: int, seed: int, rate: float, vmin: int = 1_000,
                   vmax: int = 1_000_000) -> list[Request]:
    """Poisson arrivals at `rate`/s; vertex counts log-uniform [vmin, vmax];
    LSCM or fairing with probability 1/2 each; square-ish grid patches."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests)
    t = np.cumsum(gaps) - gaps[0]
    nverts = np.exp(rng.uniform(np.log(vmin), np.log(vmax), n_requests))
    kinds = rng.integers(0, 2, n_requests)
    out = []
    for k in range(n_requests):
        side = max(4, int(round(np.sqrt(nverts[k]))))
        out.append(Request(rid=k, kind="lscm" if kinds[k] == 0 else "fairing", nx=side, ny=side,
                           seed=int(rng.integers(0, 2**31 - 1)), arrival=float(t[k])))
    return out


def serving_sample(n_requests: int, seed: int, rate: float, vmin: int = 1_000,
                   vmax: int = 1_000_000):
    """The requests of request_stream() with their systems: ("rows", RowStream)
    for LSCM (least-squares rows, one right-hand side) and ("square",
    SquareSystem) for fairing (L + 1e-2 I, three right-hand sides)."""
    reqs = request_stream(n_requests, seed, rate, vmin, vmax)
    objs = []
    for r in reqs:
        if r.kind == "lscm":
            objs.append(("rows", lscm_system(r.nx, r.ny, r.seed)))
        else:
            objs.append(("square", fairing_system(r.nx, r.ny, r.seed, lam=1e-2, n_rhs=3)))
    return reqs, objs


@dataclass
class StreamRequest:
    """One request of the serving stream with its mesh: LSCM (one system
    over the 2 nv - 4 free variables, pins at vertices 0 and nv - 1) or
    cotangent fairing (L + lam I, right-hand sides b (3, nv))."""
    rid: int
    kind: str            # "lscm" or "fairing"
    nx: int
    ny: int
    seed: int
    arrival: float       # seconds after the stream starts
    V: np.ndarray
    F: np.ndarray
    b: np.ndarray | None = None
    lam: float = 1e-2

    @property
    def n_verts(self) -> int:
        return int(self.V.shape[0])

    @property
    def unknowns(self) -> int:
        return 2 * self.n_verts - 4 if self.kind == "lscm" else self.n_verts

    def host_system(self):
        """The same system built on the host from the published formulas
        (rows / CRS of systems.py): (rp, ci, va, rhs (n_rhs, n)) -- the
        oracle's input."""
        if self.kind == "lscm":
            from oracle import oracle   # test infrastructure, imported only by its callers
            rp, ci, va, rhs = oracle.assemble_rowstream(lscm_rows(self.V, self.F))
            return rp, ci, va, rhs
        rp, ci, va = cotan_laplacian(self.V, self.F, self.lam)
        return rp, ci, va, self.b


def stream_window(rate: float, window: float, seed: int, vmin: int = 1_000, vmax: int = 1_000_000,
                  lam: float = 1e-2, noise: float = 1e-3) -> list[StreamRequest]:
    """The serving stream over [0, window): Poisson arrivals at `rate`/s;
    each request is LSCM or cotangent-Laplacian fairing (3 right-hand sides:
    the x, y, z positions + N(0, noise) times lam) with probability 1/2,
    vertex count log-uniform in [vmin, vmax], a square-ish seeded grid patch
    with the bump model of config 1.  Requests are drawn one after the
    other from one seeded generator, so a longer window extends a shorter
    one."""
    rng = np.random.default_rng(seed)
    out: list[StreamRequest] = []
    t = 0.0
    while True:
        gap = float(rng.exponential(1.0 / rate))
        t = gap if not out else t + gap
        if t >= window:
            break
        nv = float(np.exp(rng.uniform(np.log(vmin), np.log(vmax))))
        kind = "lscm" if int(rng.integers(0, 2)) == 0 else "fairing"
        s = int(rng.integers(0, 2**31 - 1))
        side = max(4, int(round(np.sqrt(nv))))
        V, F = meshes.height_field(side, side, s)
        b = None
        if kind == "fairing":
            r2 = np.random.default_rng(s + 7919)
            P = V.T.copy()
            b = np.ascontiguousarray(lam * (P + r2.normal(0.0, noise, P.shape)))
        out.append(StreamRequest(rid=len(out), kind=kind, nx=side, ny=side, seed=s, arrival=t, V=V,
                                 F=F, b=b, lam=lam))
    return out
