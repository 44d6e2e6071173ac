#!/usr/bin/env python3
"""Benchmark: solves/s and p99 latency at relative residual 1e-10 on the
serving stream (batched mixed-precision server vs plain FP64 GPU PCG).

Workload (one "step"): a window of the serving stream of the configuration
"serving stream" -- Poisson arrivals at `--rate` per second during `--window`
seconds, each request an LSCM parameterisation or a cotangent-Laplacian
fairing (3 right-hand sides) with probability 1/2, vertex count log-uniform
in [1e3, 1e6], a seeded square-ish grid patch with the bump model -- replayed
in real time through the C ABI (nlgb_server_submit_mesh with host buffers:
the server uploads the mesh, builds the system on the GPU, solves, and
copies the solution back to the host) to the continuous-batching server
(HBM budget 150 GB, shortest-work-first admission, `--streams` concurrent
CUDA streams running chunks of the PCG iteration graph, the system with the
least estimated remaining work first; precision AUTO: mixed FP32/FP64 for
the square fairing systems, FP64 for the least-squares LSCM normal
equations).  The step ends `--drain` seconds after the window; the server is
then aborted.  Every step replays the same seeded stream from scratch
(upload, build, solve, download: nothing is cached).

Reported:
  e2e         completed requests / (window + drain): a request counts when
              its solution is on the host before the step ends;
  value       completed requests / time during which the server had
              at least one chunk in flight (the GPU-side throughput);
  latency     p50 / p99 from arrival to solution on the host over every
              request of the window, an unfinished one counted as censored
              at the end of the step (p50 / p99 of the completed ones
              beside it);
  plain_fp64  the same stream through the serial FP64 server (graph-captured
              single-system PCG, one request at a time, first come first
              served);
  roofline    achieved algorithmic GB/s of the step's chunk kernels (bytes
              from the iteration counts, over the time with a chunk in
              flight) vs the measured HBM peak;
  spmv_fp64   the FP64 CRS SpMV on the 2048^2 cotangent Laplacian (4.2M
              rows, 29.3M nonzeros) vs the measured HBM peak;
  parity      statuses and true residuals of the completed requests, and
              each checked result's relative error against the FP64 direct
              oracle (SuperLU on the system built on the host);
  cpu_baseline  the CPU oracle (C, OpenMP, FP64 Jacobi-PCG on all host
              cores; host row builder + assembly) on the same stream window,
              first come first served, bounded by the same window + drain:
              completions / (window + drain); cpu_baseline_1thread likewise;
  hbm         peak and mean device footprint admitted by the server.
`--impl reference` runs only the CPU reference arm (the oracle port: the
reference's own OpenNL source is not in the checkout) and prints its line.
`--workload sweep` runs the stream at several arrival rates (both arms),
`--workload configs` the other benchmark configurations.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
os.environ.setdefault("NLGB_QUIET", "1")
# one hardware work queue per server stream (read at CUDA context creation)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

METRIC = "solves/s & p99 latency at rel-residual 1e-10: batched mixed vs plain FP64 GPU"
# DRAM bytes (read + write) per algorithmic byte of one PCG iteration (the
# three phase kernels), from one ncu capture on the 1.3M-unknown LSCM system
# (808^2 grid): 252.6 + 52.6 + 20.9 MB of DRAM traffic for 360.1 MB
# algorithmic (0.906; vectors written by one phase are partly read back
# from L2 by the next).  The 4.2M-unknown fairing system measured 0.953.
# The serving workload is too large to capture whole; its traffic grows in
# proportion to the iterations run.
GRAPH_DRAM_PER_ALGO_BYTE = 0.906
HBM_FALLBACK_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--seed", type=int, default=20261203)
    p.add_argument("--rate", type=float, default=100.0, help="Poisson arrival rate (requests/s)")
    p.add_argument("--window", type=float, default=4.0, help="arrival window of one step (s)")
    p.add_argument("--drain", type=float, default=2.0, help="time after the window before the step ends (s)")
    p.add_argument("--lead", type=float, default=1.5,
                   help="submission lead time before the window opens (s; not timed)")
    p.add_argument("--eps", type=float, default=1e-10)
    p.add_argument("--eps-lsq", type=float, default=1e-11,
                   help="relative residual of the least-squares (LSCM) requests, every arm: the "
                        "normal equations square kappa; at 1e-10 (and at 3e-11 for the larger "
                        "ones) a few LSCM solutions of the stream sit just above 1e-8 from the "
                        "direct solve")
    p.add_argument("--budget-gb", type=float, default=150.0)
    p.add_argument("--plain-steps", type=int, default=2, help="steps of the serial plain-FP64 arm")
    p.add_argument("--streams", type=int, default=32, help="concurrent chunk streams of the batched server")
    p.add_argument("--min-tile-rows", type=int, default=2048,
                   help="batched server: minimum rows per tile (fewer, fuller CTAs per system when "
                        "many streams share the GPU; the serial arm keeps the single-system tiling)")
    p.add_argument("--cta-budget", type=int, default=-1,
                   help="batched server: CTA budget of the chunks in flight (-1: one resident wave of "
                        "the phase kernels, SMs x 8; 0: no limit)")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-spmv", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-parity", action="store_true")
    p.add_argument("--parity-max-unknowns", type=int, default=300_000,
                   help="largest completed request checked against the direct oracle")
    p.add_argument("--profile-case", choices=["spmv", "batch", "batch_small", "batch_lscm", "stream_mid", "mid_systems",
                                              "plain", "mixed", "plain_lscm", "mixed_lscm", "df_lscm",
                                              "kernels"], default=None,
                   help="run one small case for an ncu capture and exit")
    p.add_argument("--workload", choices=["stream", "configs", "sweep"], default="stream",
                   help="configs: measure the other benchmark configurations and exit; sweep: the "
                        "serving stream at several arrival rates (--rates, --windows), both arms")
    p.add_argument("--charts", type=int, default=256, help="configs: charts of the batched uneven LSCM case")
    p.add_argument("--rates", type=str, default="100,1000,10000", help="sweep: arrival rates (requests/s)")
    p.add_argument("--windows", type=str, default="60,6,0.6", help="sweep: arrival window per rate (s)")
    return p.parse_args()


def measure_configs(args):
    """Configs 1, 2, 3 (`--charts` charts) and 5 -- plain FP64 vs mixed,
    serial vs batched, errors against the FP64 oracles -- one JSON line
    (device times from CUDA events); --charts 0 leaves config 3 out."""
    from graphitethree_gb300 import solver, systems
    from oracle import oracle
    out = {"workload": "configs"}
    t_start = time.perf_counter()

    def progress(msg):
        print(f"[configs {time.perf_counter() - t_start:8.1f}s] {msg}", file=sys.stderr, flush=True)

    def rec(info, n, z):
        return {"status": info.status, "iterations": info.iterations,
                "reliable_updates": info.refinement_steps, "ms": info.seconds * 1e3,
                "true_rel_residual": info.true_rel_residual,
                "GBs": info.algo_bytes / info.seconds / 1e9 if info.seconds > 0 else 0.0,
                "us_per_iteration": 1e6 * info.seconds / max(1, info.iterations), "n": n, "nnz": z}

    progress("config 1")
    M1, rhs1, asm = solver.assemble(systems.lscm_system(256, 256, seed=1))
    out["config1_lscm256"] = {"assembly_s": asm,
                              "plain": rec(M1.solve(rhs1[0])[1], M1.n, M1.nnz),
                              "mixed": rec(M1.solve(rhs1[0], precision="mixed")[1], M1.n, M1.nnz)}
    progress("SSOR vs Jacobi (context API)")
    rs_s = systems.lscm_system(128, 128, seed=4)
    ssor = {"system": "LSCM 128^2 (32,764 unknowns), nlSolve with NL_PRECONDITIONER"}
    for pc in ("jacobi", "ssor"):
        solver.solve_opennl(rs_s, preconditioner=pc, max_iter=8)          # warm-up
        _, inf = solver.solve_opennl(rs_s, preconditioner=pc)
        ssor[pc] = {k: inf[k] for k in ("status", "iterations", "elapsed", "true_error")}
        ssor[pc]["us_per_iteration"] = 1e6 * inf["elapsed"] / max(1, inf["iterations"])
    out["ssor"] = ssor

    def errors(x, ref):
        d = np.abs(x - ref)
        return {"max_abs_over_max": float(d.max() / max(np.abs(ref).max(), 1e-300)),
                "rel_2norm": float(np.linalg.norm(x - ref) / max(np.linalg.norm(ref), 1e-300))}

    progress("config 2")
    fs = systems.fairing_system(2048, 2048, seed=2)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    c2 = {}
    for k in range(3):
        # per coordinate: both forms against the oracle's FP64 Jacobi-PCG run
        # to 1e-14 (kappa ~ 1e3; the C oracle, all host threads)
        t0 = time.perf_counter()
        xo, st, it, rr = oracle.pcg(fs.rp, fs.ci, fs.va, fs.rhs[k], eps=1e-14)
        c2[f"rhs{k}_oracle"] = {"iterations": int(it), "converged": int(st) == 1,
                                "seconds": time.perf_counter() - t0}
        for p in ("double", "mixed"):
            x, inf = A.solve(fs.rhs[k], precision=p)
            c2[f"rhs{k}_{p}"] = rec(inf, A.n, A.nnz)
            c2[f"rhs{k}_{p}"]["error_vs_oracle_pcg_1e-14"] = errors(x, xo)
    out["config2_fairing2048"] = c2
    A.close()
    if args.charts > 0:
        out["config3_charts"] = measure_config3(args, progress)
    progress("mesh builders")
    measure_builders_krylov_config5(args, out, progress, rec, errors)
    print(json.dumps(out))


def measure_config3(args, progress):
    """Config 3: `--charts` uneven LSCM charts built on the GPU, batched
    (one persistent launch, FP64 and mixed) against one after another."""
    from graphitethree_gb300 import meshes, solver
    progress(f"config 3: building {args.charts} charts on the GPU")
    nx, ny = meshes.chart_sizes(args.charts, seed=3, side_min=16, side_max=512)
    mats, bs, unknowns, build_s = [], [], 0, 0.0
    for c in range(args.charts):
        V, F = meshes.height_field(int(nx[c]), int(ny[c]), 1000 + c)
        M, rhs, secs = solver.build_lscm(V, F)
        mats.append(M); bs.append(rhs); unknowns += M.n; build_s += secs
    c3 = {"charts": args.charts, "unknowns": unknowns, "gpu_build_s": build_s,
          "sides": "long side log-uniform [16,512], aspect log-uniform [1,4]; LSCM systems built on "
                   "the GPU from each chart's mesh (nlgb_build_lscm, pins 0 and nv-1)"}
    for p in ("double", "mixed"):
        progress(f"config 3: batched {p} ({unknowns} unknowns)")
        xs, infos, ks = solver.batch_solve(mats, bs, precision=p)
        progress(f"config 3: batched {p} kernel {ks:.3f}s, max iterations "
                 f"{max(i.iterations for i in infos)}")
        c3[f"batched_{p}_s"] = ks
        c3[f"batched_{p}_converged"] = sum(i.status == "converged" for i in infos)
    progress("config 3: serial plain")
    serial, serial_iters = 0.0, 0
    for M, b in zip(mats, bs):
        inf = M.solve(b)[1]
        serial += inf.seconds
        serial_iters += inf.iterations
    c3["serial_plain_s"] = serial
    c3["serial_plain_iterations"] = serial_iters
    c3["batched_speedup_double"] = serial / c3["batched_double_s"] if c3["batched_double_s"] > 0 else None
    c3["batched_speedup_mixed"] = serial / c3["batched_mixed_s"] if c3["batched_mixed_s"] > 0 else None
    statuses = {}
    for i in infos:
        statuses[i.status] = statuses.get(i.status, 0) + 1
    c3["batched_mixed_statuses"] = statuses
    c3["batched_mixed_not_converged"] = [
        {"chart": c, "n": mats[c].n, "status": i.status, "iterations": i.iterations,
         "reliable_updates": i.refinement_steps, "true_rel_residual": i.true_rel_residual}
        for c, i in enumerate(infos) if i.status != "converged"][:16]
    for M in mats:
        M.close()
    return c3


def measure_builders_krylov_config5(args, out, progress, rec, errors):
    """Mesh builders, BiCGSTAB / GMRES and config 5 (stretched fairing at
    1e-12, FP64 and mixed, against SuperLU)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from graphitethree_gb300 import meshes, solver, systems
    V1, F1 = meshes.height_field(256, 256, seed=1)
    V2, F2 = meshes.height_field(2048, 2048, seed=2)
    solver.build_lscm(V1, F1)                       # warm-up (context, kernels)
    t0 = time.perf_counter()
    rs1 = systems.lscm_rows(V1, F1)
    host_lscm = time.perf_counter() - t0
    _, _, asm1 = solver.assemble(rs1)
    gl_best = min(solver.build_lscm(V1, F1)[2] for _ in range(3))
    t0 = time.perf_counter()
    systems.cotan_laplacian(V2, F2, 1e-2)
    host_fair = time.perf_counter() - t0
    gf_best = min(solver.build_fairing(V2, F2, 1e-2)[1] for _ in range(3))
    out["mesh_builders"] = {
        "lscm_256": {"gpu_build_s": gl_best, "host_rows_s": host_lscm, "gpu_assembly_of_host_rows_s": asm1,
                     "triangles": int(F1.shape[0])},
        "fairing_2048": {"gpu_build_s": gf_best, "host_crs_s": host_fair, "triangles": int(F2.shape[0])},
        "note": "gpu_build_s: nlgb_build_* on the host clock, mesh upload + rows + assembly; host: numpy "
                "builders of graphitethree_gb300.systems (single thread)"}
    progress("krylov (non-symmetric)")
    cd = systems.convection_diffusion(1024, 1024, seed=8)
    Ak = solver.Matrix(cd.rp, cd.ci, cd.va)
    kr = {"system": "upwind convection-diffusion 1024^2 (1,048,576 unknowns, non-symmetric)", "nnz": Ak.nnz}
    for method in ("bicgstab", "gmres"):
        Ak.solve_krylov(cd.rhs[0], method=method, eps=1e-10, max_iter=20)          # warm-up
        x, inf = Ak.solve_krylov(cd.rhs[0], method=method, eps=1e-10, restart=30)
        kr[method] = {"status": inf.status, "iterations": inf.iterations, "ms": inf.seconds * 1e3,
                      "us_per_iteration": 1e6 * inf.seconds / max(1, inf.iterations),
                      "true_rel_residual": inf.true_rel_residual}
    # BiCGSTAB algorithmic bytes per iteration: two SpMVs (12 nnz + 28 n
    # each) and the three vector passes (p, y: 48 n; s, z: 40 n; x, r: 64 n)
    b_it = 2 * (12 * Ak.nnz + 28 * Ak.n) + 152 * Ak.n
    kr["bicgstab"]["algo_GBs"] = b_it / (kr["bicgstab"]["us_per_iteration"] * 1e-6) / 1e9
    out["krylov"] = kr
    Ak.close()
    progress("config 5")
    f5 = systems.fairing_system(1024, 1024, seed=5, lam=1e-4, n_rhs=1, stretch_bands=16, rhs_normal=True)
    A5 = solver.Matrix(f5.rp, f5.ci, f5.va)
    x5, i5 = A5.solve(f5.rhs[0], eps=1e-12)
    x5m, i5m = A5.solve(f5.rhs[0], eps=1e-12, precision="mixed")
    # the configuration's own split: FP32 inner iteration until its residual
    # fell by 1e-5 between FP64 reliable updates, FP64 outer to 1e-12
    x5i, i5i = A5.solve(f5.rhs[0], eps=1e-12, precision="mixed", inner_eps=1e-5)
    c5 = {"plain_1e-12": rec(i5, A5.n, A5.nnz), "mixed_1e-12": rec(i5m, A5.n, A5.nnz),
          "mixed_inner_1e-5_outer_1e-12": rec(i5i, A5.n, A5.nnz)}
    A5.close()
    progress("config 5: FP64 direct oracle (SuperLU)")
    t0 = time.perf_counter()
    Ah = sp.csr_matrix((f5.va, f5.ci, f5.rp), shape=(f5.n, f5.n)).tocsc()
    xd = spla.spsolve(Ah, f5.rhs[0])
    c5["direct_oracle"] = {"seconds": time.perf_counter() - t0,
                           "rel_residual": float(np.linalg.norm(Ah @ xd - f5.rhs[0]) / np.linalg.norm(f5.rhs[0])),
                           "note": "backward stable: its own forward error is up to ~kappa x 1e-16 ~ 1e-8"}
    c5["plain_1e-12"]["error_vs_direct"] = errors(x5, xd)
    c5["mixed_1e-12"]["error_vs_direct"] = errors(x5m, xd)
    c5["mixed_inner_1e-5_outer_1e-12"]["error_vs_direct"] = errors(x5i, xd)
    out["config5_stretched"] = c5


def run_sweep(args):
    """The serving stream at each rate of --rates over the matching window of
    --windows, through the batched server (AUTO precision) and the serial
    plain-FP64 server.  Requests are drawn cyclically from the seeded 4-s
    window at 100/s (405 meshes; every request is uploaded, built and solved
    from scratch, nothing is shared between requests on the device) and
    submitted in real time by a submitter thread.  One JSON line."""
    import dataclasses
    from graphitethree_gb300 import solver, systems
    pool = systems.stream_window(100.0, 4.0, args.seed)
    rates = [float(v) for v in args.rates.split(",")]
    windows = [float(v) for v in args.windows.split(",")]
    out = {"workload": "sweep", "pool_requests": len(pool), "drain_s": args.drain, "rows": []}
    for rate, window in zip(rates, windows):
        rng = np.random.default_rng(args.seed + int(rate))
        t, reqs = 0.0, []
        while True:
            t += float(rng.exponential(1.0 / rate))
            if t >= window:
                break
            reqs.append(dataclasses.replace(pool[len(reqs) % len(pool)], rid=len(reqs), arrival=t))
        row = {"rate_per_s": rate, "window_s": window, "requests": len(reqs)}
        for arm, mode, prec in (("batched_auto", "batched", "auto"), ("serial_fp64", "serial", "double")):
            srv = solver.Server(budget_bytes=args.budget_gb * 1e9, precision=prec, mode=mode, eps=args.eps,
                                streams=args.streams, eps_least_squares=args.eps_lsq,
                                min_tile_rows=args.min_tile_rows if mode == "batched" else 0,
                                chunk_cta_budget=args.cta_budget if mode == "batched" else 0)
            srv.reset_clock()
            T0 = 0.5
            tickets = [None] * len(reqs)
            lag = [0.0]

            t_end = T0 + window + args.drain

            def submitter():
                # a request not submitted by the end of the step (the host
                # copies fell behind the arrivals) counts as not completed
                for i, r in enumerate(reqs):
                    dt = T0 + r.arrival - srv.now()
                    if dt > 0:
                        time.sleep(dt)
                    if srv.now() >= t_end:
                        break
                    lag[0] = max(lag[0], srv.now() - (T0 + r.arrival))
                    try:
                        tickets[i] = srv.submit_mesh(r.kind, r.V, r.F, b=r.b, lam=r.lam,
                                                     arrival=T0 + r.arrival)
                    except solver.SolverError:
                        break

            th = threading.Thread(target=submitter)
            th.start()
            while srv.now() < t_end:
                time.sleep(min(0.05, max(0.0, t_end - srv.now())))
            srv.abort()
            th.join()
            lat_all, lat_done = [], []
            for r, tk in zip(reqs, tickets):
                arr = T0 + r.arrival
                ok = False
                if tk is not None:
                    try:
                        x, inf, lat = srv.wait(tk)
                        ok = arr + lat <= t_end
                    except solver.SolverError:
                        ok = False
                if ok:
                    lat_all.append(lat)
                    lat_done.append(lat)
                else:
                    lat_all.append(max(0.0, t_end - arr))
            st = srv.stats()
            srv.close()
            span = window + args.drain
            row[arm] = {"completed": len(lat_done), "solves_per_s": len(lat_done) / span,
                        "submitted": sum(tk is not None for tk in tickets),
                        "p50_s": pct(lat_all, 50), "p99_s": pct(lat_all, 99),
                        "completed_p50_s": pct(lat_done, 50), "completed_p99_s": pct(lat_done, 99),
                        "censored_fraction": 1.0 - len(lat_done) / max(1, len(reqs)),
                        "peak_admitted_gb": st["peak_bytes"] / 1e9,
                        "mean_admitted_gb": st["byte_seconds"] / t_end / 1e9,
                        "max_submit_lag_s": lag[0]}
            print(f"[sweep] rate {rate} window {window}: {arm} {row[arm]}", file=sys.stderr, flush=True)
        b, s = row["batched_auto"]["solves_per_s"], row["serial_fp64"]["solves_per_s"]
        row["speedup"] = b / s if s > 0 else None
        out["rows"].append(row)
    print(json.dumps(out))


def profile_case(which):
    """Small, bounded cases for ncu captures (a few hundred MB on the device).
    spmv:  3 FP64 SpMVs on the 2048^2 cotangent Laplacian (k_spmv);
    batch: one persistent-kernel launch over 8 mid-size systems, 300
           iterations each (k_batch);
    kernels: every kernel family once at sizes beyond L2 (assembly, mesh
           builders, FP64 / mixed PCG kernels one by one, BiCGSTAB, GMRES,
           SpMV);
    plain_lscm / mixed_lscm / df_lscm: 40 iterations on the 1.3M-unknown
           LSCM normal equations (808^2 grid), graph path, in FP64, mixed or
           double-float;
    batch_lscm: the 1.3M-unknown LSCM system alone in the persistent kernel,
           200 FP64 iterations;
    batch_small: one 4,604-unknown LSCM system in the persistent kernel,
           1000 iterations (k_batch, latency-bound);
    plain: 20 FP64 PCG iterations on the 2048^2 Laplacian (graph kernels);
    mixed: 20 FP32/FP64 iterations on the same system."""
    import ctypes
    from graphitethree_gb300 import _lib, solver, systems
    L = _lib.load()
    if which in ("spmv", "plain", "mixed"):
        fs = systems.fairing_system(2048, 2048, seed=2)
        A = solver.Matrix(fs.rp, fs.ci, fs.va)
        if which == "spmv":
            import torch
            x = torch.randn(A.n, dtype=torch.float64, device="cuda")
            y = torch.empty_like(x)
            ms = ctypes.c_double()
            L.nlgb_spmv_timed(A.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 3,
                              ctypes.byref(ms))
            print(json.dumps({"case": "spmv", "us": ms.value * 1e3, "tpr": A.threads_per_row,
                              "tile_rows": A.tile_rows}))
        else:
            x, info = A.solve(fs.rhs[0], max_iter=20, precision="double" if which == "plain" else "mixed")
            print(json.dumps({"case": which, "iterations": info.iterations, "ms": info.seconds * 1e3}))
        return
    if which == "kernels":
        # every kernel family once, at sizes beyond L2: least-squares assembly
        # (LSCM 808^2 rows), the GPU mesh builders, FP64 and mixed PCG
        # iterations (kernels launched one by one), BiCGSTAB and GMRES on a
        # non-symmetric 1M-unknown system, the standalone SpMV
        from graphitethree_gb300 import meshes
        os.environ["NLGB_EAGER_SOLVE"] = "1"
        M, rhs, _ = solver.assemble(systems.lscm_system(808, 808, seed=1))
        M.close()
        V, F = meshes.height_field(1024, 1024, seed=2)
        solver.build_lscm(V, F)[0].close()
        solver.build_fairing(V, F, 1e-2)[0].close()
        fs = systems.fairing_system(2048, 2048, seed=2, n_rhs=1)
        A = solver.Matrix(fs.rp, fs.ci, fs.va)
        A.solve(fs.rhs[0], max_iter=8, eps=1e-30)
        A.solve(fs.rhs[0], max_iter=8, eps=1e-30, precision="mixed")
        A.spmv(fs.rhs[0])
        A.close()
        cd = systems.convection_diffusion(1024, 1024, seed=8)
        K = solver.Matrix(cd.rp, cd.ci, cd.va)
        K.solve_krylov(cd.rhs[0], method="bicgstab", max_iter=4, eps=1e-30)
        K.solve_krylov(cd.rhs[0], method="gmres", max_iter=4, restart=4, eps=1e-30)
        K.close()
        print(json.dumps({"case": which, "done": True}))
        return
    if which in ("plain_lscm", "mixed_lscm", "df_lscm"):
        # 40 iterations on the LSCM normal equations of an 808 x 808 grid
        # (1,305,724 unknowns): graph-captured single-system PCG
        M, rhs, _ = solver.assemble(systems.lscm_system(808, 808, seed=1))
        prec = {"plain_lscm": "double", "mixed_lscm": "mixed", "df_lscm": "df"}[which]
        x, info = M.solve(rhs[0], max_iter=40, eps=1e-30, precision=prec)
        print(json.dumps({"case": which, "iterations": info.iterations, "ms": info.seconds * 1e3,
                          "n": M.n, "nnz": M.nnz, "tile_rows": M.tile_rows, "tpr": M.threads_per_row}))
        return
    if which == "batch_lscm":
        # the 1.3M-unknown LSCM system alone in the persistent kernel, 200
        # FP64 iterations (one team over the whole grid)
        M, rhs, _ = solver.assemble(systems.lscm_system(808, 808, seed=1))
        xs, infos, ks = solver.batch_solve([M], [rhs[0]], max_iter=200, eps=1e-30)
        print(json.dumps({"case": which, "kernel_ms": ks * 1e3, "iterations": infos[0].iterations,
                          "us_per_iteration": 1e3 * ks * 1e3 / max(1, infos[0].iterations)}))
        return
    if which == "stream_mid":
        # mid-size requests of the serving stream through the server's
        # stream executor (chunk kernels launched one by one; tiles of at
        # least 1,024 rows, as the serving bench's batched arm): an LSCM mesh
        # of 150^2 vertices (44,996 unknowns) and a fairing mesh of 300^2
        # (90,000 unknowns, 3 right-hand sides), 48 FP64 iterations each
        from graphitethree_gb300 import meshes
        os.environ["NLGB_EAGER_SOLVE"] = "1"
        srv = solver.Server(precision="double", eps=1e-30, max_iter=48, budget_bytes=4e9, min_tile_rows=1024)
        V1, F1 = meshes.height_field(150, 150, 11)
        V2, F2 = meshes.height_field(300, 300, 12)
        b2 = np.ascontiguousarray(1e-2 * V2.T)
        t1 = srv.submit_mesh("lscm", V1, F1)
        t2 = srv.submit_mesh("fairing", V2, F2, b=b2, lam=1e-2)
        i1, i2 = srv.wait(t1)[1], srv.wait(t2)[1]
        srv.close()
        print(json.dumps({"case": which, "iterations": [i.iterations for i in i1 + i2]}))
        return
    if which == "mid_systems":
        # the mid-size requests of the serving stream as the batched server
        # runs them (tiles of at least 2,048 rows, AUTO precision: FP64 for
        # LSCM, mixed for fairing), through the single-system solver with
        # its kernels launched one by one: an LSCM mesh of 150^2 vertices
        # (44,996 unknowns) and a fairing mesh of 300^2 (90,000 unknowns),
        # 48 iterations each
        from graphitethree_gb300 import meshes
        os.environ["NLGB_EAGER_SOLVE"] = "1"
        V1, F1 = meshes.height_field(150, 150, 11)
        V2, F2 = meshes.height_field(300, 300, 12)
        M1, rhs1, _ = solver.build_lscm(V1, F1)
        M2, _ = solver.build_fairing(V2, F2, 1e-2)
        its = []
        for M, b, prec in ((M1, rhs1, "double"), (M2, np.ascontiguousarray(1e-2 * V2[:, 0]), "mixed")):
            if M.tile_rows < 2048:
                M.set_layout(0, 2048)
            its.append(M.solve(b, max_iter=48, eps=1e-30, precision=prec)[1].iterations)
            M.close()
        print(json.dumps({"case": which, "iterations": its}))
        return
    if which == "batch_small":
        # one small LSCM system (4,604 unknowns, 35 tiles) in the persistent
        # kernel: a latency-bound team of 35 CTAs, 1000 FP64 iterations
        M, rhs, _ = solver.assemble(systems.lscm_system(48, 48, seed=1))
        xs, infos, ks = solver.batch_solve([M], [rhs[0]], max_iter=1000, eps=1e-30)
        print(json.dumps({"case": which, "kernel_ms": ks * 1e3, "iterations": infos[0].iterations,
                          "us_per_iteration": 1e3 * ks * 1e3 / max(1, infos[0].iterations)}))
        return
    mats, bs = [], []
    for s, side in enumerate((180, 150, 120, 90)):
        M, rhs, _ = solver.assemble(systems.lscm_system(side, side, seed=s))
        mats.append(M); bs.append(rhs[0])
        fs = systems.fairing_system(side * 2, side * 2, seed=s)
        F = solver.Matrix(fs.rp, fs.ci, fs.va)
        mats.append(F); bs.append(fs.rhs[0])
    xs, infos, ks = solver.batch_solve(mats, bs, precision="mixed", max_iter=300)
    print(json.dumps({"case": "batch", "kernel_ms": ks * 1e3, "iterations": [i.iterations for i in infos],
                      "algo_bytes": sum(i.algo_bytes for i in infos)}))


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            d = json.loads(f.read_text())
            return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
        except Exception:
            pass
    return HBM_FALLBACK_GBS, "fallback 6.8 TB/s (of fallback)"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                                "sw_power_cap"], f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def spmv_roofline(peak):
    import ctypes
    from graphitethree_gb300 import _lib, solver, systems
    fs = systems.fairing_system(2048, 2048, seed=2)
    A = solver.Matrix(fs.rp, fs.ci, fs.va)
    L = _lib.load()
    import torch
    x = torch.randn(A.n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    ms = ctypes.c_double()
    L.nlgb_spmv_timed(A.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 10, ctypes.byref(ms))
    L.nlgb_spmv_timed(A.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 100, ctypes.byref(ms))
    algo = 12 * A.nnz + 20 * A.n + 4
    gbs = algo / (ms.value * 1e-3) / 1e9
    out = {"kernel": "k_spmv<1,double,double>", "matrix": "cotangent Laplacian + 1e-2 I, 2048^2 grid",
           "rows": A.n, "nnz": A.nnz, "threads_per_row": A.threads_per_row, "tile_rows": A.tile_rows,
           "algo_bytes_per_launch": algo, "us_per_launch": ms.value * 1e3, "achieved": gbs,
           "peak": peak, "unit": "GB/s", "frac": gbs / peak,
           "note": "x (33.5 MB) is gathered through L2; matrix (352 MB) > L2 (129 MB)"}
    A.close()
    return out




# ---------------------------------------------------------------------------
# Serving stream
# ---------------------------------------------------------------------------
def make_stream(args, rank=0):
    from graphitethree_gb300 import systems
    return systems.stream_window(args.rate, args.window, args.seed + 7919 * rank)


def run_stream(stream, args, mode: str, precision: str, keep_x: bool = False):
    """One step: replay the window in real time through the C ABI, end it
    `drain` seconds after the window, abort what is left.  Returns a dict."""
    from graphitethree_gb300 import solver
    srv = solver.Server(budget_bytes=args.budget_gb * 1e9, precision=precision, mode=mode, eps=args.eps,
                        streams=args.streams, eps_least_squares=args.eps_lsq,
                        min_tile_rows=args.min_tile_rows if mode == "batched" else 0,
                        chunk_cta_budget=args.cta_budget if mode == "batched" else 0)
    srv.reset_clock()
    T0 = args.lead
    tickets = [srv.submit_mesh(r.kind, r.V, r.F, b=r.b, lam=r.lam, arrival=T0 + r.arrival) for r in stream]
    t_submitted = srv.now()
    t_end = T0 + args.window + args.drain
    while srv.now() < t_end:
        time.sleep(min(0.01, max(0.0, t_end - srv.now())))
    srv.abort()
    lat_all, lat_done, done, xs, infos = [], [], [], {}, {}
    for r, t in zip(stream, tickets):
        arr = T0 + r.arrival
        try:
            x, inf, lat = srv.wait(t)
            ok = arr + lat <= t_end
        except solver.SolverError:
            ok, lat, x, inf = False, None, None, None
        if ok:
            done.append(r.rid)
            lat_all.append(lat)
            lat_done.append(lat)
            infos[r.rid] = inf
            if keep_x:
                xs[r.rid] = x.copy()
        else:
            lat_all.append(t_end - arr)   # censored
    st = srv.stats()
    srv.close()
    span = args.window + args.drain
    return {"completed": len(done), "done_ids": done, "e2e": len(done) / span,
            "kernel_s": st["kernel_s"], "value": len(done) / st["kernel_s"] if st["kernel_s"] > 0 else 0.0,
            "lat_all": lat_all, "lat_done": lat_done, "stats": st, "infos": infos, "xs": xs,
            "submit_s": t_submitted, "t_end": t_end}


def pct(v, q):
    return float(np.percentile(v, q)) if len(v) else None


def _oracle_error(job):
    """One GPU result against the oracles, on the system built on the host
    from the same mesh: relative error against the FP64 direct solution
    (SuperLU), and relative difference from the oracle's own FP64 Jacobi-PCG
    (the restated OpenNL CPU solve, one thread) run to the same threshold,
    when pcg_max >= n.  Runs in a worker process."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from graphitethree_gb300.systems import StreamRequest
    from oracle import oracle
    kind, V, F, b, lam, xs, eps, pcg_max = job
    r = StreamRequest(rid=0, kind=kind, nx=0, ny=0, seed=0, arrival=0.0, V=V, F=F, b=b, lam=lam)
    rp, ci, va, rhs = r.host_system()
    n = len(rp) - 1
    lu = spla.splu(sp.csr_matrix((va, ci, rp), shape=(n, n)).tocsc())
    direct, pcg = [], []
    for k in range(xs.shape[0]):
        ref = lu.solve(np.asarray(rhs[k], np.float64))
        direct.append(float(np.linalg.norm(xs[k] - ref) / max(np.linalg.norm(ref), 1e-300)))
        if n <= pcg_max:
            xo = oracle.pcg(rp, ci, va, rhs[k], eps=eps, nthreads=1)[0]
            pcg.append(float(np.linalg.norm(xs[k] - xo) / max(np.linalg.norm(xo), 1e-300)))
    return kind, n, direct, pcg


def oracle_errors(stream, res, args):
    """Every completed request up to --parity-max-unknowns against the
    direct oracle, and up to a third of that against the oracle's PCG
    (process pool started with spawn)."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    by_id = {r.rid: r for r in stream}
    pcg_max = args.parity_max_unknowns // 3
    jobs = []
    for rid in res["done_ids"]:
        r = by_id[rid]
        if r.unknowns <= args.parity_max_unknowns and rid in res["xs"]:
            eps = args.eps_lsq if r.kind == "lscm" else args.eps
            jobs.append((r.unknowns, (r.kind, r.V, r.F, r.b, r.lam, res["xs"][rid], eps, pcg_max)))
    jobs.sort(key=lambda j: -j[0])
    workers = max(1, min(16, (os.cpu_count() or 2) - 1))
    t0 = time.perf_counter()
    out = {"lscm": {"direct": [], "pcg": []}, "fairing": {"direct": [], "pcg": []}}
    if jobs:
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            for kind, n, d, p in ex.map(_oracle_error, [j[1] for j in jobs]):
                out[kind]["direct"].extend(d)
                out[kind]["pcg"].extend(p)
    summary = {"method": "each completed request's system rebuilt on the host from its mesh; "
                         "direct = relative error against scipy SuperLU (FP64 direct), pcg = relative "
                         "difference from the oracle's FP64 Jacobi-PCG (the restated OpenNL CPU solve) "
                         f"run to the same threshold (systems up to {pcg_max} unknowns)",
               "requests_checked": len(jobs), "requests_completed": len(res["done_ids"]),
               "max_unknowns_checked": max([j[0] for j in jobs], default=0),
               "seconds": time.perf_counter() - t0}
    above = 0
    for kind in ("lscm", "fairing"):
        for what in ("direct", "pcg"):
            v = out[kind][what]
            summary[f"{kind}_{what}"] = {"systems": len(v), "max": max(v, default=None),
                                        "above_1e-8": int(sum(e > 1e-8 for e in v))}
            above += summary[f"{kind}_{what}"]["above_1e-8"]
    # the benchmark spec's bar, stated as pass / fail over every checked system
    summary["all_within_1e-8"] = above == 0
    summary["note"] = ("at a relative residual of 1e-10 the error of any solution, the oracle's own PCG "
                       "included, is bounded only by kappa x 1e-10; the LSCM normal equations have "
                       "kappa up to ~1e6 after Jacobi scaling")
    return summary


def cpu_stream(stream, args, threads):
    """The CPU oracle on the same stream window, first come first served:
    host row builder + C assembly (LSCM) or host CRS (fairing), then FP64
    Jacobi-PCG with OpenMP on `threads` cores, bounded by window + drain."""
    from oracle import oracle
    span = args.window + args.drain
    t0 = time.perf_counter()
    done = 0
    lat = []
    for r in stream:
        now = time.perf_counter() - t0
        if now >= span:
            break
        if now < r.arrival:
            time.sleep(r.arrival - now)
        rp, ci, va, rhs = r.host_system()
        ok = True
        for k in range(rhs.shape[0]):
            left = span - (time.perf_counter() - t0)
            if left <= 0:
                ok = False
                break
            eps = args.eps_lsq if r.kind == "lscm" else args.eps
            _, status, _, _ = oracle.pcg(rp, ci, va, rhs[k], eps=eps, nthreads=threads, max_seconds=left)
            if status != 1:
                ok = False
                break
        t_done = time.perf_counter() - t0
        if ok and t_done <= span:
            done += 1
            lat.append(t_done - r.arrival)
    return {"value": done / span, "unit": "solves/s", "cores": threads, "kind": "port",
            "completed": done, "p50_latency_s": pct(lat, 50),
            "sample": f"the same stream window ({len(stream)} requests arriving in {args.window:g} s, "
                      f"+{args.drain:g} s drain): host LSCM rows + C normal-equation assembly or host "
                      f"cotangent CRS, FP64 Jacobi-PCG to {args.eps:g} ({args.eps_lsq:g} for LSCM; C, OpenMP), first come first "
                      f"served, each step bounded by window + drain ({span:g} s); completions / {span:g} s"}


def config(args, stream):
    n_l = sum(r.kind == "lscm" for r in stream)
    return {"workload": f"serving stream (Poisson arrivals {args.rate:g}/s during a {args.window:g} s window "
                        f"+ {args.drain:g} s drain; LSCM / cotangent fairing with 3 RHS 50/50; vertices "
                        f"log-uniform [1e3,1e6]; seed {args.seed}): {len(stream)} requests "
                        f"({n_l} LSCM, {len(stream) - n_l} fairing), "
                        f"{sum(r.unknowns for r in stream)} unknowns",
            "requests": len(stream), "rate_per_s": args.rate, "window_s": args.window, "drain_s": args.drain,
            "rel_residual": args.eps, "rel_residual_least_squares": args.eps_lsq,
            "hbm_budget_gb": args.budget_gb,
            "precision": "auto: mixed FP32/FP64 (with FP64 fallback) for the square fairing "
                        "systems, FP64 for the least-squares LSCM normal equations",
            "schedule": "shortest estimated remaining work first, epochs time-boxed to 10 ms",
            "min_tile_rows": args.min_tile_rows, "chunk_cta_budget": args.cta_budget,
            "l2": "inputs larger than L2 for the large requests; every step re-uploads, rebuilds and "
                  "re-solves every request (no cached data)"}


def run_reference(args):
    from oracle import oracle
    stream = make_stream(args)
    vals, res = [], None
    for i in range(args.warmup + args.steps):
        r = cpu_stream(stream, args, threads=oracle.max_threads())
        if i >= args.warmup:
            vals.append(r["value"])
            res = r
    v = float(statistics.median(vals)) if vals else 0.0
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * (args.window + args.drain),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded serving stream; no public dataset)",
            "config": config(args, stream),
            "cpu_baseline": {**res, "value": v},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def io_bytes(stream, done_ids):
    """Host<->device bytes of one step: every mesh (and fairing right-hand
    side) is uploaded, every completed solution downloaded."""
    h2d = sum(r.V.nbytes + r.F.nbytes + (r.b.nbytes if r.b is not None else 0) for r in stream)
    ids = set(done_ids)
    d2h = sum(8 * r.unknowns * (1 if r.kind == "lscm" else 3) for r in stream if r.rid in ids)
    return int(h2d), int(d2h)


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.workload == "configs":
        measure_configs(args)
        return
    if args.workload == "sweep":
        run_sweep(args)
        return
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    from graphitethree_gb300 import _lib, solver
    if not solver.device_available():
        raise SystemExit("bench.py: no CUDA device")
    dist = None
    if world > 1:
        # replicas only: each rank serves its own seeded stream on its GPU; no
        # data-path collective, only a barrier and max-over-ranks timing
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    L = _lib.load()
    peak, peak_src = measured_peak()
    stream = make_stream(args, rank)
    span = args.window + args.drain

    for _ in range(args.warmup):
        run_stream(stream, args, "batched", "auto")
    if dist is not None:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    launches0 = L.nlgb_kernel_launches()
    steps = []
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        steps.append(run_stream(stream, args, "batched", "auto", keep_x=(i == args.steps - 1)))
    t_wall = time.perf_counter() - t_wall0
    launches = L.nlgb_kernel_launches() - launches0
    clk = clocks.stop()

    e2e = statistics.median([s["e2e"] for s in steps])
    value = statistics.median([s["value"] for s in steps])
    if dist is not None:
        from graphitethree_gb300.replicas import max_over_ranks
        # slowest replica: the smallest completion rate, as the largest time
        inv = max_over_ranks([1.0 / max(e2e, 1e-12), 1.0 / max(value, 1e-12), t_wall], dist, device="cuda")
        e2e, value, t_wall = world / inv[0], world / inv[1], inv[2]
        dist.barrier()
    lat_all = [l for s in steps for l in s["lat_all"]]
    lat_done = [l for s in steps for l in s["lat_done"]]
    last = steps[-1]
    st_last = last["stats"]
    h2d, d2h = io_bytes(stream, last["done_ids"])

    # Device work of the step: the server's executor runs every system as
    # CUDA-graph chunks of the PCG iteration kernels (k_spmv_pq + k_update_xr
    # + k_update_p, or the mixed-precision k_mx_* kernels) on --streams
    # concurrent streams; achieved = algorithmic bytes of all iterations run (finished
    # requests or not) / wall time during which at least one chunk was in
    # flight.
    busy = st_last["kernel_s"]
    algo = st_last["epoch_algo_bytes"]
    chunks = max(1, st_last["epochs"])
    ach = algo / busy / 1e9 if busy > 0 else 0.0
    roofline = {"bound": "hbm",
                "kernel": "PCG iteration kernels in CUDA-graph chunks (k_spmv_pq, k_update_xr, k_update_p; "
                          "k_mx_spmv_pq, k_mx_update_cr, k_mx_update_p for mixed systems), "
                          f"{args.streams} concurrent streams",
                "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                "traffic": GRAPH_DRAM_PER_ALGO_BYTE * algo / chunks,
                "algo_bytes_per_launch": algo / chunks, "launches_per_step": chunks,
                "busy_s_per_step": busy, "peak_source": peak_src,
                "traffic_note": "dram read+write per chunk: 0.906 DRAM byte per algorithmic byte of a PCG "
                                "iteration (k_spmv_pq + k_update_xr + k_update_p), from one ncu capture on "
                                "the 1.3M-unknown LSCM system, times this workload's algorithmic bytes per "
                                "chunk",
                "fp64_note": "the FP64 phases are co-limited by GB300's FP64 pipe, not only by HBM"}

    infos = [i for infs in last["infos"].values() for i in infs]
    statuses = {}
    for i in infos:
        statuses[i.status] = statuses.get(i.status, 0) + 1
    parity = {"completed_requests": last["completed"], "statuses": statuses,
              "all_converged": all(i.status == "converged" for i in infos),
              "max_true_rel_residual": max((i.true_rel_residual for i in infos), default=None),
              "iterations_per_step": st_last["iterations"]}
    if not args.no_parity and rank == 0:
        parity["oracle_error"] = oracle_errors(stream, last, args)

    plain = None
    if not args.no_plain:
        pr = [run_stream(stream, args, "serial", "double") for _ in range(max(1, args.plain_steps))]
        p_e2e = statistics.median([r["e2e"] for r in pr])
        p_val = statistics.median([r["value"] for r in pr])
        p_all = [l for r in pr for l in r["lat_all"]]
        plain = {"solves_per_s_e2e": p_e2e, "solves_per_s_device": p_val,
                 "completed": [r["completed"] for r in pr],
                 "p50_latency_s": pct(p_all, 50), "p99_latency_s": pct(p_all, 99),
                 "achieved_GBs": (pr[-1]["stats"]["algo_bytes"] / pr[-1]["stats"]["kernel_s"] / 1e9
                                  if pr[-1]["stats"]["kernel_s"] > 0 else 0.0),
                 "speedup_e2e_batched_mixed_over_plain": e2e / p_e2e if p_e2e > 0 else None,
                 "speedup_device": value / p_val if p_val > 0 else None,
                 "note": "one request at a time, first come first served, graph-captured FP64 PCG; "
                         "censored latencies as for the batched arm"}
    spmv = None if args.no_spmv else spmv_roofline(peak)
    cpu = cpu1 = None
    if not args.no_cpu and rank == 0:
        from oracle import oracle
        cpu = cpu_stream(stream, args, oracle.max_threads())
        cpu1 = cpu_stream(stream, args, 1)

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
        "data": "synthetic (seeded serving stream; no public dataset)",
        "config": config(args, stream),
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "completed_per_step": [s["completed"] for s in steps],
        "latency": {"p50_s": pct(lat_all, 50), "p99_s": pct(lat_all, 99),
                    "completed_p50_s": pct(lat_done, 50), "completed_p99_s": pct(lat_done, 99),
                    "censored_fraction": 1.0 - len(lat_done) / max(1, len(lat_all)), "unit": "s"},
        "plain_fp64": plain,
        "roofline": roofline,
        "spmv_fp64": spmv,
        "cpu_baseline": cpu,
        "cpu_baseline_1thread": None if cpu1 is None else {k: cpu1[k] for k in ("value", "unit", "cores",
                                                                                 "completed")},
        "hbm": {"peak_admitted_gb": st_last["peak_bytes"] / 1e9,
                "mean_admitted_gb": st_last["byte_seconds"] / max(1e-9, last["t_end"]) / 1e9,
                "budget_gb": st_last["budget_bytes"] / 1e9},
        "clocks": clk,
        "gpu_launches": int(launches),
        "parity": parity,
        "submit_s": last["submit_s"],
    }
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
