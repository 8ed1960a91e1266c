"""Repeatable single-kernel workloads for profiling (ncu) and bandwidth sweeps.

    python -m mycode_gb300.profile_case --path residual64 --cells 1000000 --reps 3
    python -m mycode_gb300.profile_case --path krylov_stream --workload laminar_plate --reps 8
    python -m mycode_gb300.profile_case --path krylov_stream --cells 4000000 --gmres-m 20 --gmres-tol 0

Workloads: the bump channel (3 x 1, Gaussian bump) triangulated at ``--cells`` with
HLLC, second-order limited reconstruction and the viscous flux, from a perturbed
free-stream state; or the laminar plate of the benchmark (240 x 120, Roe, central, from
its free-stream start).  Paths, each ``--reps`` times:
  residual64     the FP64 residual (prim, grad + limiter, flux, gather)
  residual32     the FP32 residual
  jv64 / jv32    the exact J v (dual-number kernels) in FP64 / FP32
  vjp64          the adjoint (VJP) of the FP64 residual
  krylov_stream  mixed-precision Newton steps whose GMRES runs the graph driver's fused
                 kernels from the stream driver (outside a graph, so ncu sees them)
printing the per-kernel CUDA-event times (average over the evaluations).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def build(cells: int, seed: int = 0):
    from mycode_gb300 import api, meshgen
    spec = meshgen.bump(cells, seed=seed)
    m = api.Mesh.from_spec(spec)
    return api, spec, m


def perturbed(U0: np.ndarray, xyc: np.ndarray, seed: int = 1, amp: float = 0.05) -> np.ndarray:
    from mycode_gb300 import meshgen
    p = meshgen.smooth_perturbation(xyc, seed, amp)
    U = U0.copy()
    U[:, 0] *= 1 + p[:, 0]
    U[:, 1] *= 1 + p[:, 1]
    U[:, 2] += 0.05 * U0[:, 1] * p[:, 2]
    U[:, 3] *= 1 + p[:, 3]
    return U


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--path", default="residual64",
                    choices=["residual64", "residual32", "jv64", "jv32", "vjp64", "krylov_stream"])
    ap.add_argument("--workload", default="bump", choices=["bump", "laminar_plate"])
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--flux", default="HLLC")
    ap.add_argument("--spatial", default="SECOND_ORDER_LIMITED")
    ap.add_argument("--inviscid", action="store_true")
    ap.add_argument("--gmres-m", type=int, default=None, help="Krylov dimension (krylov_stream)")
    ap.add_argument("--gmres-tol", type=float, default=None, help="GMRES tolerance; 0 runs m iterations")
    a = ap.parse_args(argv)
    gm = {}
    if a.gmres_m is not None:
        gm["gmres_m"] = a.gmres_m
    if a.gmres_tol is not None:
        gm["gmres_tol"] = a.gmres_tol
    from mycode_gb300 import api, meshgen
    if a.workload == "laminar_plate":
        m = api.Mesh.from_spec(meshgen.laminar_plate(240, 120, ratio=1.08))
        s = api.Solver(m, bcset="plate", init="freestream", viscous=1, flux="ROE", spatial="SECOND_ORDER_CENTRAL",
                       precision="mixed", jv="exact", krylov=2, **gm)
        s.setFreestreamStatic(0.2, 101325.0, 300.0)
        s.setKinematicViscosity(1e5, 1.0)
        s.initialize()
        U = s.getSolution()
    else:
        api, spec, m = build(a.cells)
        cfg = dict(bcset="bump", init="bump", viscous=0 if a.inviscid else 1, flux=a.flux, spatial=a.spatial,
                   precision="mixed", jv="exact", krylov=2, **gm)
        s = api.Solver(m, **cfg)
        s.setFlowConditions(0.5, 101325.0, 300.0)
        s.setKinematicViscosity(3e6, 1.0)
        s.initialize()
        U = perturbed(s.getSolution(), m.cells()[:, 1:])
        s.set_state(U)
    s.set_timing(True)
    s.residual_device(True)
    s.set_dt(s.local_timestep(100.0))
    v = np.random.default_rng(3).standard_normal(U.shape) * np.abs(U).mean(axis=0)
    lam = np.random.default_rng(4).standard_normal(U.shape)
    run = {
        "residual64": (lambda: s.residual_device(True), "residual."),
        "residual32": (lambda: s.residual32(), "residual."),
        "jv64": (lambda: s.apply_jacobian(U, None, v, mode="exact"), "jv."),
        "jv32": (lambda: s.apply_jacobian32(U, v), "jv."),
        "vjp64": (lambda: s.vjp(lam, U), "vjp."),
        "krylov_stream": (lambda: s.newton_step(0.0), "krylov."),
    }[a.path]
    s.synchronize()
    s.kernel_stats(reset=True)
    t0 = time.perf_counter()
    iters = []
    for _ in range(a.reps):
        r = run[0]()
        if a.path == "krylov_stream":
            iters.append(r[0].gmres_iters)
    s.synchronize()
    st = s.kernel_stats(reset=True)
    out = {k: round(v[0] / max(v[1], 1), 5) for k, v in st.items() if k.startswith(run[1]) and v[1]}
    line = {"path": a.path, "workload": a.workload, "cells": m.n_cells, "faces": m.n_faces,
            "ms_per_launch": out, "wall_s": time.perf_counter() - t0}
    if iters:
        # Arnoldi iterations per solve and the mean basis index j over them (iteration j
        # reads j + 1 stored vectors)
        line["gmres_iters"] = iters
        line["mean_j"] = sum(i * (i - 1) / 2 for i in iters) / max(1, sum(iters))
        line["launches"] = {k: v[1] for k, v in st.items() if k.startswith(run[1]) and v[1]}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
