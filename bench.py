#!/usr/bin/env python3
"""Benchmark of the residual-and-Newton path: cell-residuals per second.

Workload (one GPU): the laminar flat plate — Navier-Stokes, M = 0.2, Re_L = 1e5,
Pr = 0.72, adiabatic no-slip plate from x = 0 behind a 0.2 symmetry lead-in, 240 x 120
quads (28,800 cells, 57,960 faces) with wall-normal stretching 1.08; Roe flux plus the
viscous flux, second-order central reconstruction; pseudo-transient JFNK.  Synthetic
mesh and state (seeded recipe, no dataset).

A step is one pseudo-transient Newton step of the solve: local time step, residual,
one right-preconditioned GMRES solve (each Krylov iteration one J v product) and the
clamped update.  The unit of work is one cell-residual: one cell of one residual or
J v evaluation, so a step processes n_cells * (1 + GMRES iterations) cell-residuals.

  value  mixed precision (FP32 Krylov basis, FP32 exact J v and preconditioner; FP64
         residual, update, Hessenberg/Givens and norms), state resident in HBM; device
         time from CUDA events on the solver's stream; L2 flushed between steps
  e2e    the same step through the C ABI with the state uploaded from pinned host
         memory before and read back after every step (wall clock)
  fp64   the plain FP64 path (FD J v as the reference) on the same workload

``--impl reference`` times the reference's algorithm on the host cores instead: the
reference built from its sources (oracle/_ref) when present, else the plain-C
restatement (oracle/), one independent copy per host core.
"""
from __future__ import annotations

import argparse
import atexit
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-residuals/s; JFNK time-to-1e-10 mixed vs FP64 GPU; adjoint/primal cost"
UNIT = "cell-residuals/s"
L2_FLUSH_BYTES = 256 << 20


def workload_spec():
    from mycode_gb300 import meshgen
    return meshgen.laminar_plate(240, 120, ratio=1.08)


WORKLOAD = {
    "workload": "laminar flat plate 240x120 quads (28,800 cells, 57,960 faces), stretching 1.08, "
                "Navier-Stokes M=0.2 Re_L=1e5 Pr=0.72, Roe + viscous flux, 2nd-order central, "
                "pseudo-transient JFNK-GMRES(40), one Newton step per step",
    "n_cells": 28800,
    "n_faces": 57960,
}


def setup_flow(s):
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(1e5, 1.0)
    s.initialize()
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")


# ---------------------------------------------------------------- roofline helpers

def algorithmic_bytes(kind: str, nc: int, nf: int, nv: int, s: int, spatial: str, viscous: bool, dual: bool) -> float:
    """Compulsory DRAM bytes of one launch: every distinct input read once and every
    output written once.  s = bytes per real; dual kernels move value + derivative.
    With SST (nv = 6) the primitives carry k, w (7 planes), the gradients 14 planes, and
    the cell terms (mu_t, F1, S_k vol, S_w vol) are written by the gradient stage (its
    SST kernel, which also reads the wall distance) and read by the flux and gather."""
    k = 2 if dual else 1
    sst = nv == 6
    nq = 7 if sst else 5
    ng = 2 * nq
    second = spatial != "FIRST_ORDER"
    limited = spatial == "SECOND_ORDER_LIMITED"
    if kind == "prim":
        return nc * (nv * s * k + nq * s * k)
    if kind == "grad":
        # U (ghost faces) is negligible; W of every cell, gradients written, limiter written
        b = nc * (nq * s * k + ng * s * k + (s if limited and not dual else 0)) + nc * 4 * 4
        if sst:
            b += nc * (nq * s * k + ng * s * k + s + 4 * s * k)  # the SST cell kernel: W, G, d in, T out
        return b
    if kind == "flux":
        per_face = 8 + 9 * s + nv * s  # indices, geometry, F*A (derivative only for dual)
        per_cell = nv * s * k + 3 * s * k
        if second or viscous:
            per_cell += ng * s * k
        if limited:
            per_cell += s
        if sst:
            per_cell += 2 * s * k  # mu_t, F1
        return nf * per_face + nc * per_cell
    if kind == "gather":
        b = nc * 16 + nf * nv * s + nc * nv * s + (nc * (nv * s + s + s) if dual else 0)
        if sst:
            b += nc * 2 * s  # the source planes
        return b
    raise ValueError(kind)


def krylov_bytes(stage: str, nc: int, nf: int, nv: int, s: int, jbar: float) -> float:
    """Compulsory bytes of one fused Arnoldi stage (FP32 basis: s = 4) at the mean number
    of basis vectors jbar + 1 that the iterations read."""
    L = nv * nc
    nb = jbar + 1.0
    if stage == "prim_z":
        # second pass of the pending vector and first pass of the last product (the pending
        # vector, the product and j basis vectors in; the finished basis vector and the new
        # pending vector out), then U and 1/D in, z and the dual primitives out
        return nc * (nv * s + s + nv * s + 2 * (7 if nv == 6 else 5) * s) + L * s * (jbar + 4)
    if stage in ("grad", "flux"):
        return algorithmic_bytes(stage, nc, nf, nv, s, "SECOND_ORDER_CENTRAL", True, True)
    if stage == "gather_dot":
        return nc * 16 + nf * nv * s + nc * (nv * s + 2 * s + nv * s) + nb * L * s
    if stage in ("update_dot", "update_final"):  # FD J v body only
        return L * s * (2 + nb)
    raise ValueError(stage)


def vjp_algorithmic_bytes(nc: int, nf: int, nv: int, spatial: str) -> float:
    """Compulsory FP64 bytes of one VJP: the forward recomputation (prim, gradients,
    limiter, SST terms), then the face kernel (state, primitives, gradients, limiter of
    both cells, lambda, geometry in; 2 x slots out) and the two cell kernels (slots in,
    gU out).  Slots per face side: nv + gradients + phi (+ mu_t, F1 with SST)."""
    s = 8
    ng = 14 if nv == 6 else 10
    slots = nv + ng + 1 + (2 if nv == 6 else 0)
    fwd = sum(algorithmic_bytes(kd, nc, nf, nv, s, spatial, True, False) for kd in ("prim", "grad"))
    face = nf * (8 + 9 * s + 2 * slots * s) + nc * (nv * s + (ng + 7) * s + s + nv * s)
    cells = nf * 2 * slots * s + nc * (ng * s + 2 * s + 8 + nv * s) + nc * (ng * s + nv * s + nv * s)
    return fwd + face + cells


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            j = json.load(fh)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_fp64_pipe():
    """FP64 pipe fraction and FP64 flops per unit of the FP64 residual's kernels from the
    committed ncu summary (profiles/fp64_pipe.txt)."""
    path = os.path.join(ROOT, "profiles", "fp64_pipe.txt")
    out = {}
    if os.path.exists(path):
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) == 4 and not parts[0].startswith("#"):
                    try:
                        out[parts[0]] = {"fp64_pipe_frac": float(parts[1]), "fp64_flops_per_unit": float(parts[2]),
                                         "unit": parts[3]}
                    except ValueError:
                        pass
    return out


def profile_traffic(kernel_class: str, jbar: float = 0.0):
    """DRAM bytes per launch of a kernel class from the committed ncu summary
    (profiles/traffic.txt: bytes at Arnoldi iteration 0 and per further basis vector),
    evaluated at the mean iteration jbar; None when the class is not listed."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) >= 2 and not parts[0].startswith("#") and parts[0] == kernel_class:
                try:
                    base = float(parts[1])
                    per = float(parts[2]) if len(parts) > 2 else 0.0
                except ValueError:
                    return None
                return round(base + per * jbar)
    return None


# ---------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        atexit.register(self._kill)  # no sampler outlives the benchmark (an error mid-run)

    def _kill(self):
        if self.proc is not None and self.proc.poll() is None:
            self.proc.kill()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout: float = 5.0):
        """Blocks until the sampler has printed its first line (it is live), at most timeout s."""
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- distributed

def dist_setup(gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def all_sum(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- our arm

def run_steps(s, steps, flush=True):
    """Timed Newton steps; returns (device seconds, cell-residual evaluations, per-step records)."""
    tot_ms, evals, recs = 0.0, 0, []
    for _ in range(steps):
        if flush:
            s.flush_l2(L2_FLUSH_BYTES)
        rec, _ = s.newton_step(0.0)
        tot_ms += rec.device_ms
        evals += 1 + rec.gmres_iters
        recs.append((rec.res_vm, rec.gmres_iters, rec.device_ms, rec.cfl, rec.krylov_ms))
    return tot_ms / 1e3, evals, recs


def make_solver(api, mesh, device, precision):
    cfg = dict(bcset="plate", init="freestream", viscous=1, flux="ROE", spatial="SECOND_ORDER_CENTRAL",
               device=device)
    if precision == "mixed":
        cfg.update(precision="mixed", jv="exact")
    else:
        cfg.update(precision="fp64", jv="fd")
    s = api.Solver(mesh, **cfg)
    setup_flow(s)
    return s


def ours(args):
    world, rank, local = dist_setup(args.gpus)
    from mycode_gb300 import api
    import numpy as np
    spec = workload_spec()
    mesh = api.Mesh.from_spec(spec)
    nc, nf = mesh.n_cells, mesh.n_faces

    # ---- primary: mixed precision, state resident in HBM
    s = make_solver(api, mesh, local, "mixed")
    # the timed steps carry CUDA events around each step and its GMRES graph only; the
    # per-kernel times come from the replay below
    s.set_timing("steps")
    # the clock sampler (50 ms period) is live before the warm-up and runs through the
    # timed steps, the kernel replay and the e2e steps, so that it has samples under load
    # although the timed region itself lasts only ~30 ms
    clk = ClockSampler(local)
    clk.start()
    clk.wait_first()
    for _ in range(args.warmup):
        s.newton_step(0.0)
    s.kernel_stats(reset=True)
    l0 = s.launch_count()
    s.synchronize()
    barrier(world)
    t_dev, evals, recs = run_steps(s, args.steps)
    s.synchronize()
    barrier(world)
    launches = s.launch_count() - l0
    kinfo = s.krylov_info()
    # Per-kernel times: event nodes are not allowed inside the graph's WHILE body, and
    # events between the timed steps' kernels would add to their time, so a few steps are
    # replayed with the stream driver (the graph's kernels launched one iteration at a
    # time) and every kernel timed with events there.
    Usnap = s.getSolution()
    s.set_timing(True)
    s.set_krylov("stream")
    run_steps(s, 1)  # one untimed stream-driven step first
    s.kernel_stats(reset=True)
    _, _, rrecs = run_steps(s, min(args.steps, 10))
    s.synchronize()
    stats = s.kernel_stats(reset=True)
    s.set_krylov("graph")
    s.set_state(Usnap)
    # mean number of basis vectors read per iteration in the replay (j + 1 at iteration j)
    jits = [r[1] for r in rrecs]
    jbar = (sum(i * (i + 1) / 2 for i in jits) / max(1, sum(jits))) - 1.0
    t_max = all_max(world, t_dev)
    units = all_sum(world, float(evals * nc))
    value = units / t_max

    # ---- roofline of the dominant kernel class
    # The timed steps' GMRES graphs are timed whole (CUDA events around each graph launch:
    # krylov_ms).  The replay times every Arnoldi kernel alone (its events add ~2-3 us per
    # launch and it runs without programmatic dependent launch), so the graph time is
    # attributed to the kernel classes in proportion to their replay averages.
    iters = evals - args.steps
    t_kry_ms = sum(r[4] for r in recs)
    replay_sum = sum(ms / n for k, (ms, n) in stats.items() if k.startswith("krylov.") and n)
    attr = t_kry_ms / (replay_sum * iters) if replay_sum > 0 and iters > 0 else 1.0
    peak, peak_kind = measured_peak()
    kern = {}
    for k, (ms, n) in stats.items():
        if n == 0:
            continue
        grp, name = k.split(".")
        if grp == "krylov":
            b = krylov_bytes(name, nc, nf, 4, 4, jbar)
        else:
            dual = grp == "jv"
            b = algorithmic_bytes(name, nc, nf, 4, 4 if dual else 8, "SECOND_ORDER_CENTRAL", True, dual)
        avg = ms / n
        kern[k] = {"replay_launches": n, "avg_us": round(avg * 1e3, 3), "algorithmic_bytes": int(b)}
        if grp == "residual":
            kern[k]["timed_launches"] = args.steps
            kern[k]["est_total_ms"] = round(avg * args.steps, 4)
            kern[k]["source"] = "stream-driver replay (CUDA events around the kernel)"
        elif grp != "krylov":
            kern[k]["est_total_ms"] = round(ms, 4)
        if grp == "krylov":
            # replayed launches: their averages scaled to the graph's measured time, times
            # the Arnoldi iterations of the timed steps
            kern[k]["replay_avg_us"] = kern[k].pop("avg_us")
            avg = avg * attr
            kern[k]["avg_us"] = round(avg * 1e3, 3)
            kern[k]["timed_launches"] = iters
            kern[k]["est_total_ms"] = round(avg * iters, 4)
            kern[k]["source"] = ("stream-driver replay of the graph's kernels, scaled by the graph time "
                                 f"(factor {attr:.3f})")
        kern[k]["achieved_gbs"] = round(b / (avg * 1e-3) / 1e9, 1)
        kern[k]["share_of_step"] = round(kern[k]["est_total_ms"] / (t_dev * 1e3), 4)
    dom = max(kern, key=lambda k: kern[k]["est_total_ms"])
    d = kern[dom]
    traffic = profile_traffic(dom, jbar)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": d["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": round(d["achieved_gbs"] / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "traffic": traffic}

    # ---- the FP64 residual: HBM fraction (live) beside the FP64-pipe fraction (ncu)
    pipe = profile_fp64_pipe()
    fp64_residual = {}
    for k in ("residual.prim", "residual.grad", "residual.flux", "residual.gather"):
        if k in kern:
            e = {"avg_us": kern[k]["avg_us"], "hbm_frac": round(kern[k]["achieved_gbs"] / peak, 4)}
            e.update(pipe.get(k, {}))
            fp64_residual[k.split(".")[1]] = e
    fp64_residual["source"] = "hbm_frac: this run; fp64_pipe_frac, flops: profiles/fp64_pipe.txt (ncu)"

    # ---- e2e through the C ABI with pinned host buffers (per-kernel timing off: the
    # production call)
    import torch
    Uh = torch.empty((nc, 6), dtype=torch.float64, pin_memory=True).numpy()
    s.getSolution(out=Uh)
    s.set_timing(False)
    s.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    e_evals = 0
    for _ in range(args.steps):
        s.set_state(Uh)
        rec, _ = s.newton_step(0.0)
        s.getSolution(out=Uh)
        e_evals += 1 + rec.gmres_iters
    s.synchronize()
    barrier(world)
    t_e2e = all_max(world, time.perf_counter() - t0)
    clocks = clk.stop()
    clocks["window"] = "warm-up, timed steps, kernel replay and e2e steps"
    e_units = all_sum(world, float(e_evals * nc))
    e2e = {"value": e_units / t_e2e, "unit": UNIT, "h2d_bytes_per_step": nc * 6 * 8, "d2h_bytes_per_step": nc * 6 * 8,
           "api": "cfdg_set_state + cfdg_newton_step + cfdg_get_state"}

    # ---- the plain FP64 path (FD J v), same protocol
    s64 = make_solver(api, mesh, local, "fp64")
    s64.set_timing(True)
    for _ in range(args.warmup):
        s64.newton_step(0.0)
    s64.synchronize()
    t64, ev64, recs64 = run_steps(s64, args.steps)
    fp64 = {"value": ev64 * nc / t64, "unit": UNIT, "ms_per_step": 1e3 * t64 / args.steps,
            "gmres_iters": [r[1] for r in recs64], "jv": "one-sided FD (reference)"}

    # ---- adjoint / primal cost: FP64 VJP (gradients and limiter recomputed) over one FP64
    # residual, CUDA-event kernel time on the same state, L2 flushed before each
    s64.set_timing(True)
    s64.kernel_stats(reset=True)
    reps = 20
    for _ in range(reps):
        s64.flush_l2(L2_FLUSH_BYTES)
        s64.residual_device(True)
        s64.flush_l2(L2_FLUSH_BYTES)
        s64.vjp_device()
    st64 = s64.kernel_stats(reset=True)
    t_res = sum(st64[k][0] for k in st64 if k.startswith("residual.")) / reps
    t_vjp = sum(st64[k][0] for k in st64 if k.startswith("vjp.")) / reps
    adjoint = {"ratio": t_vjp / t_res, "residual_ms": t_res, "vjp_ms": t_vjp,
               "note": "FP64 VJP of the full residual (forward recomputation included) / FP64 residual"}

    # ---- time to a density residual of 1e-10: mixed vs the FP64 paths on the supersonic
    # wedge (the reference's own CPU case, which converges under the reference's CFL control)
    t2c = time_to_converge(api) if (rank == 0 and not args.no_t2c) else None
    others = other_configs(api) if (rank == 0 and not args.no_t2c) else None

    # ---- CPU baseline: the oracle port on this host, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(args.cpu_steps)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 Krylov/J v + f64 residual/update",
            "data": "synthetic (seeded mesh recipe, free-stream start)",
            "config": dict(WORKLOAD, precision="mixed", jv="exact (dual numbers, FP32)",
                           l2="flushed between timed steps (256 MiB write)", parallelism="replicas" if world > 1 else "1 GPU"),
            "gmres_iters": [r[1] for r in recs],
            "res_vm": [r[0] for r in recs],
            "gpu_launches": launches,
            "krylov_driver": kinfo,
            "roofline": roofline,
            "kernels": kern,
            "fp64_residual": fp64_residual,
            "e2e": e2e,
            "fp64": fp64,
            "adjoint_over_primal": adjoint,
            "time_to_1e-10": t2c,
            "other_configs": others,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))


def other_configs(api, steps=20, warmup=3):
    """The mixed-precision Newton step on the SST configurations at full size, from the
    free stream, CUDA events around each step (secondary measurements, not the headline):
    the turbulent flat plate 480 x 240 (115,200 cells, Roe, central) and the shock/boundary-
    layer interaction box 800 x 640 with its outer half split (768,000 cells, HLLC + BJ
    limiter, 8-degree shock inflow)."""
    from mycode_gb300 import meshgen
    out = {}
    cases = (
        ("turbulent_plate_sst", meshgen.turb_plate(), dict(flux="ROE", spatial="SECOND_ORDER_CENTRAL"),
         (0.2, 5e6), {}),
        ("swbli_sst", meshgen.swbli(), dict(flux="HLLC", spatial="SECOND_ORDER_LIMITED"), (2.0, 1e7),
         dict(shock_deflection_deg=8.0)),
    )
    for name, spec, method, (mach, re), extra in cases:
        mesh = api.Mesh.from_spec(spec)
        s = api.Solver(mesh, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision="mixed",
                       jv="exact", **method, **extra)
        s.setFreestreamStatic(mach, 101325.0, 300.0)
        s.setKinematicViscosity(re, 1.0)
        s.initialize()
        s.set_timing("steps")
        try:
            for _ in range(warmup):
                s.newton_step(0.0)
            t, evals, recs = run_steps(s, steps)
            out[name] = {"n_cells": mesh.n_cells, "n_faces": mesh.n_faces, "value": evals * mesh.n_cells / t,
                         "unit": UNIT, "ms_per_step": 1e3 * t / steps, "steps": steps, "warmup": warmup,
                         "gmres_iters": [r[1] for r in recs], "res_vm_first_last": [recs[0][0], recs[-1][0]]}
        except api.CfdgError as e:
            # a diverging start-up (no start-up strategy beyond the reference's CFL control)
            out[name] = {"n_cells": mesh.n_cells, "n_faces": mesh.n_faces, "error": str(e)}
        s.close()
    return out


def time_to_converge(api, max_steps=1500):
    """Wall time of full solves from the free stream to a volume-weighted density residual
    of 1e-10: the wedge 120 x 80 x 2 triangles (19,200 cells, 10 % jitter), M 2.5, HLLC with
    the Barth-Jespersen limiter, GMRES(30), CFL from 10, for the mixed path (FP32 Krylov and
    exact J v, FP64 residual and update), the FP64 path with exact J v and the FP64 path
    with the reference's FD J v.  Also the relative L2 difference of the converged states and
    of their wall pressure coefficients (the slip wall, tag 3).  The limited scheme freezes
    its limiter early (src/Solver.cpp:1714), at slightly different values in each run, so
    its converged states solve slightly different discrete problems; the first-order pair
    (same wedge, no limiter) shows the mixed path converging to the FP64 solution itself."""
    from mycode_gb300 import meshgen
    import numpy as np
    mesh = api.Mesh.from_spec(meshgen.wedge(120, 80, jitter=0.10, seed=0))

    def solve(prec, jv, spatial):
        s = api.Solver(mesh, bcset="supersonic", init="freestream", viscous=0, precision=prec, jv=jv, gmres_m=30,
                       cfl0=10.0, flux="HLLC", spatial=spatial)
        s.setFlowConditions(2.5, 101325.0, 300.0)
        s.initialize()
        s.synchronize()
        t0 = time.perf_counter()
        n, reached, its = 0, False, 0
        while n < max_steps:
            rec, _ = s.newton_step(0.0)
            n += 1
            its += rec.gmres_iters
            if rec.res_rho <= 1e-10 and n > 5:
                reached = True
                break
        s.synchronize()
        t = time.perf_counter() - t0
        res = {"seconds": round(t, 4), "newton_steps": n, "gmres_iters": its, "reached": reached,
               "final_res_rho": rec.res_rho}
        U, cp = s.getSolution(), s.wall_coefficients(3)[1]
        s.close()
        return res, U, cp

    out, states, cps = {}, {}, {}
    for name, prec, jv in (("mixed", "mixed", "exact"), ("fp64_exact", "fp64", "exact"), ("fp64_fd", "fp64", "fd")):
        out[name], states[name], cps[name] = solve(prec, jv, "SECOND_ORDER_LIMITED")
    ref = states["fp64_fd"]
    for name in ("mixed", "fp64_exact"):
        out[name]["state_rel_l2_vs_fp64_fd"] = float(np.linalg.norm(states[name] - ref) / np.linalg.norm(ref))
        out[name]["wall_cp_max_abs_diff_vs_fp64_fd"] = float(np.abs(cps[name] - cps["fp64_fd"]).max())
    out["speedup_mixed_vs_fp64_fd"] = out["fp64_fd"]["seconds"] / out["mixed"]["seconds"]
    out["speedup_mixed_vs_fp64_exact"] = out["fp64_exact"]["seconds"] / out["mixed"]["seconds"]
    out["workload"] = "supersonic wedge 120x80x2 (19,200 cells), M 2.5, HLLC + BJ limiter, GMRES(30), CFL0 10"
    m1, Um, cpm = solve("mixed", "exact", "FIRST_ORDER")
    f1, Uf, cpf = solve("fp64", "exact", "FIRST_ORDER")
    out["first_order"] = {
        "mixed": m1, "fp64_exact": f1, "speedup_mixed_vs_fp64_exact": f1["seconds"] / m1["seconds"],
        "state_rel_l2_mixed_vs_fp64": float(np.linalg.norm(Um - Uf) / np.linalg.norm(Uf)),
        "wall_cp_max_abs_diff_mixed_vs_fp64": float(np.abs(cpm - cpf).max()),
        "wall_cp_range": [float(cpf.min()), float(cpf.max())],
        "workload": "the same wedge, HLLC first order (no limiter), to a density residual of 1e-10"}
    return out


# ---------------------------------------------------------------- CPU side

def _cpu_worker(args):
    """One independent copy of the CPU path: untimed warm-up Newton steps, then a timed
    solveImplicit of `steps` steps continuing from that state."""
    warm, steps, kind = args
    sys.path.insert(0, ROOT)
    from oracle.oracle import OracleSolver, RefSolver
    spec = workload_spec()
    if kind == "reference":
        s = RefSolver(spec, "plate_visc")
    else:
        s = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    setup_flow(s)
    if warm:
        s.solveImplicit(0.0, warm)
    t0 = time.perf_counter()
    tr = s.solveImplicit(0.0, steps)
    t = time.perf_counter() - t0
    evals = int(len(tr["res_vm"]) + tr["gmres_iters"].sum())
    return evals, t, len(tr["res_vm"])


def cpu_kind():
    from oracle.oracle import ref_available
    return "reference" if ref_available("plate_visc") else "port"


def cpu_baseline_sample(steps: int):
    """The first `steps` Newton steps of the workload on one host core (the GMRES
    iterations per step grow along the solve: 150 steps are about 2,400 evaluations,
    15-35 s of FP64 FD work on one core)."""
    from oracle.oracle import build_oracle
    build_oracle()
    kind = cpu_kind()
    evals, t, n = _cpu_worker((0, steps, kind))
    nc = WORKLOAD["n_cells"]
    return {"value": evals * nc / t, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": f"{n} Newton steps ({evals} residual/J v evaluations, FD J v, FP64) of the same workload "
                      f"from the free-stream start on 1 host core, {t:.1f} s"}


def reference_arm(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import build_oracle
    build_oracle()
    kind = cpu_kind()
    cores = os.cpu_count() or 1
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(args.warmup, args.steps, kind)] * cores)
    nc = WORKLOAD["n_cells"]
    evals = sum(r[0] for r in res)
    t = max(r[1] for r in res)
    value = evals * nc / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded mesh recipe, free-stream start)",
        "config": dict(WORKLOAD, precision="fp64", jv="one-sided FD (reference)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{cores} independent copies x {args.steps} Newton steps after {args.warmup} "
                                   f"warm-up steps ({evals} evaluations in {t:.1f} s)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- bandwidth sweep

SWEEP_SIZES = (64_000, 256_000, 1_000_000, 4_000_000)


def sweep(args):
    """Per-kernel throughput of the residual, the exact J v and the VJP in FP64 and FP32
    on the Gaussian-bump channel (3 x 1, height 0.05, width 0.2, triangles, 10 % seeded
    jitter) at M = 0.5, Re = 3e6 with SST, HLLC, second-order limited; one JSON line."""
    from mycode_gb300 import api, meshgen
    import numpy as np
    peak, peak_kind = measured_peak()
    sizes = [int(x) for x in args.sweep_sizes.split(",")] if args.sweep_sizes else SWEEP_SIZES
    out = []
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clk.start()
    for target in sizes:
        spec = meshgen.bump(target, jitter=0.10, seed=0)
        mesh = api.Mesh.from_spec(spec)
        nc, nf = mesh.n_cells, mesh.n_faces
        s = api.Solver(mesh, bcset="bump", init="bump", viscous=1, turbulence="sst", precision="mixed", jv="exact",
                       flux="HLLC", spatial="SECOND_ORDER_LIMITED")
        s.setFlowConditions(0.5, 101325.0, 300.0)
        s.setKinematicViscosity(3e6, 1.0)
        s.initialize()
        U0 = s.getSolution()
        cells = mesh.cells()
        pert = meshgen.smooth_perturbation(cells[:, 1:], 7, 0.05)
        U = U0.copy()
        for c in range(4):
            U[:, c] *= 1.0 + pert[:, c]
        U[:, 4] *= 1.0 + 0.5 * pert[:, 0]
        U[:, 5] *= 1.0 + 0.5 * pert[:, 1]
        s.set_state(U)
        s.residual_device(True)
        s.set_dt(s.local_timestep(10.0))
        v = np.random.default_rng(1).standard_normal(U.shape) * np.abs(U).mean(axis=0)
        lam = np.random.default_rng(2).standard_normal(U.shape)
        s.set_timing(True)
        ops = {
            "residual_fp64": (lambda: s.residual_device(True), "residual.", 8, False),
            "residual_fp32": (lambda: s.residual32(), "residual.", 4, False),
            "jv_fp64": (lambda: s.apply_jacobian(U, None, v, mode="exact"), "jv.", 8, True),
            "jv_fp32": (lambda: s.apply_jacobian32(U, v), "jv.", 4, True),
            "vjp_fp64": (lambda: s.vjp(lam, U), "vjp.", 8, None),
        }
        res = {"n_cells": nc, "n_faces": nf}
        for name, (fn, cls, sz, dual) in ops.items():
            for _ in range(2):
                fn()
            s.synchronize()
            s.kernel_stats(reset=True)
            for _ in range(args.sweep_reps):
                s.flush_l2(L2_FLUSH_BYTES)
                fn()
            s.synchronize()
            st = s.kernel_stats(reset=True)
            kern, tot = {}, 0.0
            for k, (ms, n) in st.items():
                if not k.startswith(cls) or n == 0:
                    continue
                avg = ms / n
                tot += avg
                entry = {"avg_us": round(avg * 1e3, 2)}
                if dual is not None:
                    b = algorithmic_bytes(k.split(".")[1], nc, nf, 6, sz, "SECOND_ORDER_LIMITED", True, dual)
                    entry.update(algorithmic_bytes=int(b), gbs=round(b / (avg * 1e-3) / 1e9, 1),
                                 hbm_frac=round(b / (avg * 1e-3) / 1e9 / peak, 4))
                kern[k.split(".")[1]] = entry
            r = {"ms": round(tot, 4), "cell_residuals_per_s": nc / (tot * 1e-3), "kernels": kern}
            if dual is None:
                b = vjp_algorithmic_bytes(nc, nf, 6, "SECOND_ORDER_LIMITED")
                r.update(algorithmic_bytes=int(b), gbs=round(b / (tot * 1e-3) / 1e9, 1),
                         hbm_frac=round(b / (tot * 1e-3) / 1e9 / peak, 4))
            res[name] = r
        res["vjp_fp32"] = None  # the adjoint runs in FP64 only
        res["vjp_over_residual_fp64"] = res["vjp_fp64"]["ms"] / res["residual_fp64"]["ms"]
        out.append(res)
        s.close()
        del mesh
    clocks = clk.stop()
    cpu = None
    if not args.no_cpu_baseline:
        cpu = sweep_cpu_sample(SWEEP_SIZES[0])
    line = {"metric": "bandwidth sweep: cell-residuals/s per kernel", "unit": UNIT,
            "config": {"workload": "Gaussian bump channel 3x1 (height 0.05, width 0.2), triangles, 10% seeded jitter, "
                                   "M=0.5 Re=3e6, SST, HLLC, 2nd-order limited; seeded smooth perturbation of the "
                                   "initial state", "l2": "flushed before every evaluation"},
            "peak_gbs": peak, "peak_source": peak_kind, "sizes": out, "clocks": clocks, "cpu_baseline": cpu}
    print(json.dumps(line))


def sweep_cpu_sample(target: int):
    """The oracle's FP64 SST residual on one host core at the smallest sweep size."""
    from oracle.oracle import build_oracle, OracleSolver
    from mycode_gb300 import meshgen
    build_oracle()
    spec = meshgen.bump(target, jitter=0.10, seed=0)
    o = OracleSolver(spec, bcset="bump", viscous=True, init="bump")
    o.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    o.setFlowConditions(0.5, 101325.0, 300.0)
    o.setKinematicViscosity(3e6, 1.0)
    o.initialize()
    U = o.get_state()
    k, w = o.sst_freestream()
    U[:, 4] = U[:, 0] * k
    U[:, 5] = U[:, 0] * w
    o.residual_sst(U)
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < 5.0:
        o.residual_sst(U)
        n += 1
    t = time.perf_counter() - t0
    return {"value": n * o.n_cells / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} FP64 SST residual evaluations of the {o.n_cells}-cell bump on 1 host core, {t:.1f} s"}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=150)
    ap.add_argument("--no-t2c", action="store_true", help="skip the time-to-1e-10 solves")
    ap.add_argument("--sweep", action="store_true", help="bandwidth sweep on the bump channel instead")
    ap.add_argument("--sweep-sizes", default="", help="comma-separated target cell counts")
    ap.add_argument("--sweep-reps", type=int, default=10)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.sweep:
        sweep(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
