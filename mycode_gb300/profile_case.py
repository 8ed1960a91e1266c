"""Repeatable single-kernel workloads for profiling (ncu) and bandwidth sweeps.

    python -m mycode_gb300.profile_case --path residual64 --cells 1000000 --reps 3

Builds the bump channel (3 x 1, Gaussian bump) triangulated at ``--cells``, sets a
perturbed free-stream state and evaluates ``--reps`` times one of
  residual64   the FP64 residual (prim, grad + limiter, flux, gather)
  jv64         the exact J v (dual-number kernels) in FP64
with HLLC, second-order limited reconstruction and the viscous flux, printing the
per-kernel CUDA-event times of the last evaluation.
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
    ap.add_argument("--path", default="residual64", choices=["residual64", "jv64"])
    ap.add_argument("--cells", type=int, default=1_000_000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--flux", default="HLLC")
    ap.add_argument("--spatial", default="SECOND_ORDER_LIMITED")
    ap.add_argument("--inviscid", action="store_true")
    a = ap.parse_args(argv)
    api, spec, m = build(a.cells)
    cfg = dict(bcset="bump", init="bump", viscous=0 if a.inviscid else 1, flux=a.flux, spatial=a.spatial)
    s = api.Solver(m, **cfg)
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.setKinematicViscosity(3e6, 1.0)
    s.initialize()
    U = perturbed(s.getSolution(), m.cells()[:, 1:])
    s.set_state(U)
    s.set_timing(True)
    s.residual_device(True)
    s.local_timestep(100.0)
    t0 = time.perf_counter()
    out = {}
    if a.path == "residual64":
        for _ in range(a.reps):
            s.residual_device(True)
        out = s.kernel_times()
    else:
        v = np.random.default_rng(3).standard_normal(U.shape) * np.abs(U).mean(axis=0)
        for _ in range(a.reps):
            s.apply_jacobian(U, None, v, mode="exact")
        st = s.kernel_stats()
        out = {k: v[0] / max(v[1], 1) for k, v in st.items() if k.startswith("jv")}
    s.synchronize()
    print(json.dumps({"path": a.path, "cells": m.n_cells, "faces": m.n_faces, "ms_last": out,
                      "wall_s": time.perf_counter() - t0}))


if __name__ == "__main__":
    main()
