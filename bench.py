#!/usr/bin/env python3
"""Benchmark of the residual-and-Newton path: cell-residuals per second.

Workload (one GPU): the Gaussian-bump channel at its largest size — a 3 x 1 channel with a
bump of height 0.05 and width 0.2, 2448 x 816 quads split into 3,995,136 triangles
(5,995,968 faces) with 10 % seeded jitter; M = 0.5, Re = 3e6, the SST k-omega model (six
conserved variables), HLLC, second-order reconstruction with the Barth-Jespersen limiter,
the viscous flux; the initial state with a seeded smooth perturbation.  Synthetic mesh and
state (seeded recipe, no dataset).

A step is one evaluation of the FP64 residual R(U) (computeResiduals with the limiter
recomputed) over the whole mesh, in the reference's floating-point operation order.  The
unit of work is one cell-residual, so a step is n_cells cell-residuals.

  value  state resident in HBM; device time from CUDA events on the solver's stream;
         inputs larger than L2 (U alone is 192 MB) and L2 flushed between steps
  e2e    the same evaluations through the C ABI (cfdg_residual) with the state in pinned
         host memory, in the reference's AoS layout and numbering: the host-to-device
         copy, the renumbering, the residual, the renumbering back and the device-to-host
         copy of R inside the timed region (wall clock)

Beside it, at the same size: the FP32 residual, the exact J v in FP32 and FP64 and the
FP64 adjoint (VJP); the mixed-precision Newton step on the laminar flat plate; the time
to a density residual of 1e-10 (mixed vs FP64) with its wall-Cp error against the FP64
CPU oracle; the other full-size configurations.

``--impl reference`` times the CPU path instead: the plain-C restatement of the
reference's residual with the SST terms (oracle/; the reference itself has no SST), one
independent copy per host core on the same mesh, state and scheme.
``--sweep`` runs the bandwidth sweep over 64k-4M cells; ``--profile-case`` one kernel
path on a chosen case for ncu captures.
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
HEADLINE_CELLS = 4_000_000


def headline_spec(target: int = HEADLINE_CELLS):
    from mycode_gb300 import meshgen
    return meshgen.bump(target, jitter=0.10, seed=0)


def headline_workload(spec) -> dict:
    return {
        "workload": f"Gaussian-bump channel 3x1 (bump height 0.05, width 0.2), {spec.n_cells:,} triangles "
                    f"({spec.expected_faces():,} faces), 10% seeded jitter; M=0.5 Re=3e6, SST k-omega (6 conserved "
                    "variables), HLLC, 2nd-order Barth-Jespersen-limited reconstruction, viscous flux; one FP64 "
                    "residual evaluation R(U) per step (limiter recomputed), seeded smooth perturbation of the "
                    "initial state",
        "n_cells": spec.n_cells,
        "n_faces": spec.expected_faces(),
        "precision": "fp64, the reference's operation order (bit-exact residual path)",
        "l2": f"inputs larger than L2 (U alone {spec.n_cells * 48 / 1e6:.0f} MB) and L2 flushed (256 MiB write) "
              "between steps",
    }


def perturb_state(U0, xyc):
    """The benchmark state: the initial state times a seeded smooth perturbation (5 %) of
    rho, rho u, rho v, rho E and (half as strong) of rho k, rho w."""
    from mycode_gb300 import meshgen
    pert = meshgen.smooth_perturbation(xyc, 7, 0.05)
    U = U0.copy()
    for c in range(4):
        U[:, c] *= 1.0 + pert[:, c]
    U[:, 4] *= 1.0 + 0.5 * pert[:, 0]
    U[:, 5] *= 1.0 + 0.5 * pert[:, 1]
    return U


def bump_solver(api, mesh, device=0, precision="mixed", sst=True):
    s = api.Solver(mesh, bcset="bump", init="bump", viscous=1, turbulence="sst" if sst else "none",
                   precision=precision, jv="exact", flux="HLLC", spatial="SECOND_ORDER_LIMITED", device=device)
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.setKinematicViscosity(3e6, 1.0)
    s.initialize()
    return s


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


def krylov_bytes(stage: str, nc: int, nf: int, nv: int, s: int, jbar: float,
                 spatial: str = "SECOND_ORDER_CENTRAL") -> float:
    """Compulsory bytes of one fused Arnoldi stage (FP32 basis: s = 4) at the mean number
    of basis vectors jbar + 1 that the iterations read.  The value planes of the
    linearisation point (primitives, gradients, SST cell terms) are formed once per solve,
    so the body writes derivative planes only."""
    L = nv * nc
    nb = jbar + 1.0
    nq = 7 if nv == 6 else 5
    ng = 2 * nq
    if stage == "prim_z":
        # second pass of the pending vector and first pass of the last product (the pending
        # vector, the product and j basis vectors in; the finished basis vector and the new
        # pending vector out), then U and 1/D in, z and the primitives' derivatives out
        return nc * (nv * s + s + nv * s + nq * s) + L * s * (jbar + 4)
    if stage == "grad":
        # the primitives' derivatives in, the gradients' derivatives out, the face list, each
        # face's two cells, normal and area once; the SST cell kernel: primitives and
        # gradients (value + derivative) and d in, the cell terms' derivatives out
        b = nc * (nq * s + ng * s + 16) + nf * (8 + 3 * s)
        if nv == 6:
            b += nc * (2 * nq * s + 2 * ng * s + s + 4 * s)
        return b
    if stage == "flux":
        return algorithmic_bytes(stage, nc, nf, nv, s, spatial, True, True)
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


def _profile_table(name: str) -> dict:
    """Rows of a committed ncu summary under profiles/: `class value...` per line, `#`
    comments; the values as floats."""
    path = os.path.join(ROOT, "profiles", name)
    out = {}
    if os.path.exists(path):
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) >= 2 and not parts[0].startswith("#"):
                    try:
                        out[parts[0]] = [float(x) for x in parts[1:]]
                    except ValueError:
                        pass
    return out


def profile_fp64_pipe() -> dict:
    """FP64 pipe of the FP64 residual's kernels on the headline workload, from ncu
    (profiles/fp64_pipe.txt): per class the pipe's busy fraction, its warp instructions
    and DRAM bytes per unit (per face for the flux, per cell otherwise)."""
    out = {}
    for k, v in _profile_table("fp64_pipe.txt").items():
        if len(v) >= 3:
            out[k] = {"pipe_frac_ncu": v[0], "fp64_warp_inst_per_unit": v[1], "dram_bytes_per_unit": v[2]}
    return out


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

def timed_kernels(s, fn, prefix, reps, warm=1):
    """Per-class CUDA-event kernel times of `reps` calls of fn (L2 flushed before each):
    {class: (total ms, launches)} for the classes starting with prefix."""
    for _ in range(warm):
        fn()
    s.synchronize()
    s.kernel_stats(reset=True)
    for _ in range(reps):
        s.flush_l2(L2_FLUSH_BYTES)
        fn()
    s.synchronize()
    st = s.kernel_stats(reset=True)
    return {k: v for k, v in st.items() if k.startswith(prefix) and v[1]}


def fp64_roofline_row(cls, avg_ms, nc, nf, peak_gbs, pipe_peak_warp, pipe_prof):
    """One FP64 residual kernel class: its time, HBM fraction of algorithmic bytes and FP64
    pipe fraction (the pipe's warp instructions per unit from ncu over the live time,
    against the live FP64 pipe rate).  Bound: the FP64 pipe."""
    kind = cls.split(".")[1]
    b = algorithmic_bytes(kind, nc, nf, 6, 8, "SECOND_ORDER_LIMITED", True, False)
    units = nf if kind == "flux" else nc
    row = {"avg_us": round(avg_ms * 1e3, 2), "algorithmic_bytes": int(b),
           "hbm_gbs": round(b / (avg_ms * 1e-3) / 1e9, 1), "hbm_frac": round(b / (avg_ms * 1e-3) / 1e9 / peak_gbs, 4),
           # every class of the FP64 residual is bound by the FP64 pipe (ncu: 79-89 % busy)
           "bound": "fp64_pipe"}
    p = pipe_prof.get(cls)
    if p:
        inst = p["fp64_warp_inst_per_unit"] * units
        ach = inst / (avg_ms * 1e-3)
        row.update(fp64_warp_inst_per_launch=int(inst), fp64_pipe_ginst_s=round(ach / 1e9, 3),
                   fp64_pipe_frac=round(ach / pipe_peak_warp, 4), fp64_pipe_frac_ncu=p["pipe_frac_ncu"],
                   traffic=int(p["dram_bytes_per_unit"] * units))
    return row


def kernel_paths(s, U, nc, nf, peak_gbs, reps, pipe_peak_warp=None, pipe_prof=None):
    """The residual, exact J v and VJP kernel paths on one state: per path its time per
    evaluation, cell-residuals/s and per-kernel fractions (FP32 and dual kernels against
    HBM, FP64 kernels against the FP64 pipe where ncu counts exist)."""
    import numpy as np
    s.set_timing(True)
    s.residual_device(True)          # the limiter the J v products freeze
    s.set_dt(s.local_timestep(10.0))  # the time term of J v
    v = np.random.default_rng(1).standard_normal(U.shape) * np.abs(U).mean(axis=0)
    lam = np.random.default_rng(2).standard_normal(U.shape)
    ops = {
        "residual_fp64": (lambda: s.residual_device(True), "residual.", 8, False),
        "residual_fp32": (lambda: s.residual32(), "residual.", 4, False),
        "jv_fp64": (lambda: s.apply_jacobian(U, None, v, mode="exact"), "jv.", 8, True),
        "jv_fp32": (lambda: s.apply_jacobian32(U, v), "jv.", 4, True),
        "vjp_fp64": (lambda: s.vjp(lam, U), "vjp.", 8, None),
    }
    out = {}
    for name, (fn, prefix, sz, dual) in ops.items():
        st = timed_kernels(s, fn, prefix, reps)
        kern, tot = {}, 0.0
        for k, (ms, n) in st.items():
            avg = ms / n
            tot += avg
            if dual is None:
                kern[k.split(".")[1]] = {"avg_us": round(avg * 1e3, 2)}
            elif sz == 8 and not dual and pipe_prof is not None:
                kern[k.split(".")[1]] = fp64_roofline_row(k, avg, nc, nf, peak_gbs, pipe_peak_warp, pipe_prof)
            else:
                b = algorithmic_bytes(k.split(".")[1], nc, nf, 6, sz, "SECOND_ORDER_LIMITED", True, dual)
                kern[k.split(".")[1]] = {"avg_us": round(avg * 1e3, 2), "algorithmic_bytes": int(b),
                                         "hbm_gbs": round(b / (avg * 1e-3) / 1e9, 1),
                                         "hbm_frac": round(b / (avg * 1e-3) / 1e9 / peak_gbs, 4),
                                         "bound": "fp64_pipe" if sz == 8 else "hbm"}
        r = {"ms": round(tot, 4), "cell_residuals_per_s": nc / (tot * 1e-3), "kernels": kern}
        if dual is None:
            b = vjp_algorithmic_bytes(nc, nf, 6, "SECOND_ORDER_LIMITED")
            r.update(algorithmic_bytes=int(b), hbm_gbs=round(b / (tot * 1e-3) / 1e9, 1),
                     hbm_frac=round(b / (tot * 1e-3) / 1e9 / peak_gbs, 4), bound="fp64_pipe")
        out[name] = r
    out["vjp_over_residual_fp64"] = out["vjp_fp64"]["ms"] / out["residual_fp64"]["ms"]
    return out


def ours(args):
    world, rank, local = dist_setup(args.gpus)
    from mycode_gb300 import api
    import numpy as np
    import torch
    spec = headline_spec(args.cells)
    # mesh ingest (connectivity, geometry, Hilbert renumbering, device layout) on the host
    # and with the GPU kernels (the same mesh bit for bit); the solver uses the GPU-built one
    t0 = time.perf_counter()
    mesh_h = api.Mesh.from_spec(spec)
    t_mesh_host = time.perf_counter() - t0
    del mesh_h
    t0 = time.perf_counter()
    mesh = api.Mesh.from_spec(spec, gpu=local)
    t_mesh = time.perf_counter() - t0
    nc, nf = mesh.n_cells, mesh.n_faces
    s = bump_solver(api, mesh, local)
    U = perturb_state(s.getSolution(), mesh.cells()[:, 1:])
    s.set_state(U)
    peak, peak_kind = measured_peak()
    pipe_fma = api.fp64_pipe_rate(local)  # thread FMAs per second, measured now
    pipe_peak_warp = pipe_fma / 32.0
    pipe_prof = profile_fp64_pipe()

    # the clock sampler (50 ms period) is live before the warm-up and runs through the
    # timed steps and the e2e steps
    clk = ClockSampler(local)
    clk.start()
    clk.wait_first()

    # ---- value: FP64 residual, state resident in HBM, CUDA events around every kernel
    s.set_timing(True)
    for _ in range(args.warmup):
        s.flush_l2(L2_FLUSH_BYTES)
        s.residual_device(True)
    s.synchronize()
    s.kernel_stats(reset=True)
    l0 = s.launch_count()
    barrier(world)
    for _ in range(args.steps):
        s.flush_l2(L2_FLUSH_BYTES)
        s.residual_device(True)
    s.synchronize()
    barrier(world)
    launches = s.launch_count() - l0
    st = {k: v for k, v in s.kernel_stats(reset=True).items() if k.startswith("residual.") and v[1]}
    t_dev = sum(v[0] for v in st.values()) / 1e3
    t_max = all_max(world, t_dev)
    value = all_sum(world, float(args.steps * nc)) / t_max

    # ---- e2e: the same evaluations through cfdg_residual with pinned host buffers
    Uh = torch.empty((nc, 6), dtype=torch.float64, pin_memory=True).numpy()
    Rh = torch.empty((nc, 6), dtype=torch.float64, pin_memory=True).numpy()
    Uh[:] = U
    s.set_timing(False)
    for _ in range(args.warmup):
        s.computeResiduals(Uh, True, out=Rh)
    s.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.computeResiduals(Uh, True, out=Rh)
    t_e2e = all_max(world, time.perf_counter() - t0)
    clocks = clk.stop()
    clocks["window"] = "warm-up, timed steps and e2e steps"
    e2e = {"value": all_sum(world, float(args.steps * nc)) / t_e2e, "unit": UNIT,
           "h2d_bytes_per_step": int(Uh.nbytes), "d2h_bytes_per_step": int(Rh.nbytes),
           "api": "cfdg_residual (host AoS state in pinned memory -> host AoS residual)", "ms_per_step":
           1e3 * t_e2e / args.steps}

    # ---- per-kernel roofline: every class of the FP64 residual is bound by the FP64 pipe
    kern = {}
    for k, (ms, n) in st.items():
        kern[k] = fp64_roofline_row(k, ms / n, nc, nf, peak, pipe_peak_warp, pipe_prof)
        kern[k].update(launches=n, share_of_step=round(ms / (t_dev * 1e3), 4))
    dom = max(kern, key=lambda k: kern[k]["share_of_step"])
    d = kern[dom]
    roofline = {"bound": "fp64_pipe", "kernel": dom, "unit": "G FP64-pipe warp instructions/s",
                "achieved": d.get("fp64_pipe_ginst_s"), "peak": round(pipe_peak_warp / 1e9, 3),
                "frac": d.get("fp64_pipe_frac"),
                "peak_source": "measured live in this run (cfdg_fp64_pipe_rate: an FP64 FMA stream over all SMs); "
                               "instructions per launch from ncu (profiles/fp64_pipe.txt) scaled to this mesh",
                "traffic": d.get("traffic"), "algorithmic_bytes": d["algorithmic_bytes"],
                "hbm": {"achieved": d["hbm_gbs"], "peak": peak, "unit": "GB/s", "frac": d["hbm_frac"],
                        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                        else "fallback 6.8 TB/s"},
                "fp64_pipe_frac_ncu": d.get("fp64_pipe_frac_ncu")}

    # ---- the other kernel paths at the same size (FP32 residual, exact J v, VJP)
    paths = kernel_paths(s, U, nc, nf, peak, min(args.steps, 5), pipe_peak_warp, pipe_prof) \
        if not args.quick else None
    s.close()
    del mesh
    # the bandwidth sweep's smaller sizes (the 4M-cell size is kernel_paths above)
    sweep_sizes = None
    if rank == 0 and not args.quick:
        sweep_sizes = []
        for target in SWEEP_SIZES[:-1]:
            spec_t = headline_spec(target)
            mesh_t = api.Mesh.from_spec(spec_t)
            st_ = bump_solver(api, mesh_t, local)
            Ut = perturb_state(st_.getSolution(), mesh_t.cells()[:, 1:])
            st_.set_state(Ut)
            r = {"n_cells": mesh_t.n_cells, "n_faces": mesh_t.n_faces}
            r.update(kernel_paths(st_, Ut, mesh_t.n_cells, mesh_t.n_faces, peak, 5, pipe_peak_warp, pipe_prof))
            sweep_sizes.append(r)
            st_.close()
            del mesh_t

    extra = {}
    if rank == 0 and not args.quick:
        extra["newton_laminar_plate"] = newton_plate(api, args, local)
        extra["time_to_1e-10"] = time_to_converge(api)
        extra["other_configs"] = other_configs(api)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(args.cells, args.cpu_seconds)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded mesh recipe and seeded smooth perturbation of the initial state)",
            "config": dict(headline_workload(spec), parallelism="replicas" if world > 1 else "1 GPU"),
            "gpu_launches": launches,
            "roofline": roofline,
            "kernels": kern,
            "e2e": e2e,
            "mesh_build_s": {"gpu": round(t_mesh, 3), "host": round(t_mesh_host, 3),
                             "note": "cfdg_mesh_create_gpu / cfdg_mesh_create wall time of the headline mesh"},
            "fp64_pipe_fma_per_s": pipe_fma,
            "kernel_paths": paths,
            "bandwidth_sweep": None if sweep_sizes is None else {
                "workload": "the same channel, case and state recipe at smaller sizes (the 4M-cell size is "
                            "kernel_paths); per path ms per evaluation, cell-residuals/s and per-kernel fractions",
                "sizes": sweep_sizes},
            "adjoint_over_primal": None if paths is None else {
                "ratio": paths["vjp_over_residual_fp64"], "residual_ms": paths["residual_fp64"]["ms"],
                "vjp_ms": paths["vjp_fp64"]["ms"],
                "note": "FP64 VJP of the full residual (forward recomputation included) / FP64 residual, same mesh"},
            **extra,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))


def run_newton_steps(s, steps, flush=True):
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


PLATE = ("laminar flat plate 240x120 quads (28,800 cells, 57,960 faces), stretching 1.08, Navier-Stokes M=0.2 "
         "Re_L=1e5 Pr=0.72, Roe + viscous flux, 2nd-order central, pseudo-transient JFNK-GMRES(40) from the free "
         "stream; one Newton step per step")


def plate_solver(api, mesh, device, precision):
    cfg = dict(bcset="plate", init="freestream", viscous=1, flux="ROE", spatial="SECOND_ORDER_CENTRAL", device=device)
    if precision == "mixed":
        cfg.update(precision="mixed", jv="exact")
    else:
        cfg.update(precision="fp64", jv="fd")
    s = api.Solver(mesh, **cfg)
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(1e5, 1.0)
    s.initialize()
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    return s


def newton_plate(api, args, device, steps=20, warmup=5):
    """The mixed-precision Newton step (FP32 Krylov basis and exact J v, FP64 residual and
    update) on the laminar flat plate: device time of `steps` steps after `warmup`, the same
    steps end to end through the C ABI (state restored with its CFL and step counter, then
    uploaded from and read back to pinned host memory every step), and the plain FP64
    path with the reference's FD J v on the same steps."""
    from mycode_gb300 import meshgen
    import torch
    mesh = api.Mesh.from_spec(meshgen.laminar_plate(240, 120, ratio=1.08))
    nc = mesh.n_cells
    s = plate_solver(api, mesh, device, "mixed")
    s.set_timing("steps")
    for _ in range(warmup):
        s.newton_step(0.0)
    Usnap = s.getSolution()
    cfl, step = s.newton_state()
    s.synchronize()
    t_dev, evals, recs = run_newton_steps(s, steps)
    # e2e: the same steps again (same state, CFL and step counter)
    Uh = torch.empty((nc, 6), dtype=torch.float64, pin_memory=True).numpy()
    Uh[:] = Usnap
    s.set_newton_state(cfl, step)
    s.set_timing(False)
    s.synchronize()
    t0 = time.perf_counter()
    e_evals, e_iters = 0, []
    for _ in range(steps):
        s.set_state(Uh)
        rec, _ = s.newton_step(0.0)
        s.getSolution(out=Uh)
        e_evals += 1 + rec.gmres_iters
        e_iters.append(rec.gmres_iters)
    s.synchronize()
    t_e2e = time.perf_counter() - t0
    s.close()
    s64 = plate_solver(api, mesh, device, "fp64")
    s64.set_timing("steps")
    for _ in range(warmup):
        s64.newton_step(0.0)
    s64.synchronize()
    t64, ev64, recs64 = run_newton_steps(s64, steps)
    s64.close()
    return {"workload": PLATE, "steps": steps, "warmup": warmup, "value": evals * nc / t_dev, "unit": UNIT,
            "ms_per_step": 1e3 * t_dev / steps, "gmres_iters": [r[1] for r in recs],
            "precision": "mixed (FP32 Krylov basis and exact J v; FP64 residual, update, Hessenberg, norms)",
            "e2e": {"value": e_evals * nc / t_e2e, "unit": UNIT, "gmres_iters": e_iters,
                    "h2d_bytes_per_step": nc * 6 * 8, "d2h_bytes_per_step": nc * 6 * 8,
                    "api": "cfdg_set_state + cfdg_newton_step + cfdg_get_state"},
            "fp64": {"value": ev64 * nc / t64, "unit": UNIT, "ms_per_step": 1e3 * t64 / steps,
                     "gmres_iters": [r[1] for r in recs64], "jv": "one-sided FD (reference)"}}


def other_configs(api, steps=20, warmup=3):
    """The mixed-precision Newton step on the SST configurations at full size, from the
    free stream, CUDA events around each step (secondary measurements, not the headline):
    the turbulent flat plate 480 x 240 (115,200 cells, Roe, central) and the shock/boundary-
    layer interaction box 800 x 640 with its outer half split (768,000 cells, HLLC + BJ
    limiter, 8-degree shock inflow).  Then the plate converged and its skin-friction-drag
    VJP; the interaction's wall-pressure VJP (x in [0.3, 0.7]) at the state the timed steps
    reached, and the interaction converged at full size with its wall-pressure VJP there."""
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
            t, evals, recs = run_newton_steps(s, steps)
            out[name] = {"n_cells": mesh.n_cells, "n_faces": mesh.n_faces, "value": evals * mesh.n_cells / t,
                         "unit": UNIT, "ms_per_step": 1e3 * t / steps, "steps": steps, "warmup": warmup,
                         "gmres_iters": [r[1] for r in recs], "res_vm_first_last": [recs[0][0], recs[-1][0]]}
            if name == "swbli_sst":
                s.set_timing(False)
                out[name]["wall_pressure_vjp"] = vjp_fd_check(s, s.getSolution(), "wall_pressure", 0.3, 0.7, seed=37,
                                                              steps=(1e-9, 1e-8))
                out[name]["wall_pressure_vjp"]["state"] = f"after {warmup + steps} Newton steps from the free stream"
        except api.CfdgError as e:
            out[name] = {"n_cells": mesh.n_cells, "n_faces": mesh.n_faces, "error": str(e)}
        s.close()
        if name == "turbulent_plate_sst":
            out[name].update(converged_plate_vjp(api, mesh, method, mach, re))
        if name == "swbli_sst":
            out[name]["converged_full_size"] = converged_swbli_vjp(api, mesh, method, mach, re, extra)
    return out


def vjp_fd_check(s, U, kind, x0=-1e300, x1=1e300, seed=29, directions=16, steps=(1e-7, 1e-8)):
    """The VJP of a wall objective at state U against central differences: lambda = dJ/dU
    (itself checked against differences of J), then lambda^T (dR/dU) v by the VJP against
    central differences of lambda^T R along seeded directions v scaled per component.  A
    direction whose two step sizes disagree crossed a branch (a min / max / clip of the
    scheme, a limiter switch) and is counted, not compared."""
    import numpy as np
    J, lam = s.objective(kind, x0, x1)
    gU = s.vjp(lam, U)
    rng = np.random.default_rng(seed)
    scale = np.abs(U).mean(axis=0)
    worst, worst_dj, switched = 0.0, 0.0, 0
    for _ in range(directions):
        v = rng.standard_normal(U.shape) * scale
        s.set_state(U + 1e-6 * v)
        jp = s.objective(kind, x0, x1, gradient=False)
        s.set_state(U - 1e-6 * v)
        jm = s.objective(kind, x0, x1, gradient=False)
        lv = float(np.sum(lam * v))
        worst_dj = max(worst_dj, abs((jp - jm) / 2e-6 - lv) / max(abs(lv), 1e-300))
        fd = [float(np.sum(lam * (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)))) / (2 * h)
              for h in steps]
        a = float(np.sum(gU * v))
        err = abs(fd[0] - a) / abs(a)
        if err > 1e-6 and abs(fd[0] - fd[1]) > 1e-7 * abs(a):
            switched += 1
        else:
            worst = max(worst, err)
    s.set_state(U)
    return {"objective": kind, "range": [x0, x1] if x0 > -1e300 else None, "J": J, "directions": directions,
            "steps": list(steps), "worst_rel_err": worst, "dJdU_worst_rel_err": worst_dj,
            "branch_switches": switched, "seed": seed}


def _converge(api, mesh, method, mach, re, extra, orders, max_steps):
    """A mixed-precision solver on `mesh` from the free stream to `orders` orders of
    volume-weighted residual reduction under the reference's CFL control (chains of 64
    Newton steps): the solver and the run's record."""
    s = api.Solver(mesh, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision="mixed",
                   jv="exact", **method, **extra)
    s.setFreestreamStatic(mach, 101325.0, 300.0)
    s.setKinematicViscosity(re, 1.0)
    s.initialize()
    s.reset_newton()
    s.synchronize()
    t0 = time.perf_counter()
    recs = []
    while len(recs) < max_steps:
        r, _ = s.newton_steps(64)
        recs += r
        if recs[-1].res_vm <= 10.0 ** -orders * recs[0].res_vm:
            break
    s.synchronize()
    t = time.perf_counter() - t0
    return s, {"n_cells": mesh.n_cells, "newton_steps": len(recs), "seconds": round(t, 3),
               "res_vm_first_last": [recs[0].res_vm, recs[-1].res_vm],
               "res_rho_first_last": [recs[0].res_rho, recs[-1].res_rho],
               "orders": math.log10(recs[0].res_vm / recs[-1].res_vm),
               "gmres_iters": int(sum(x.gmres_iters for x in recs))}


def converged_plate_vjp(api, mesh, method, mach, re, orders=6.0, max_steps=8000):
    """The turbulent flat plate converged `orders` orders, then the skin-friction-drag VJP at
    that state against central differences along 16 seeded directions."""
    s, conv = _converge(api, mesh, method, mach, re, {}, orders, max_steps)
    chk = vjp_fd_check(s, s.getSolution(), "skin_friction_drag")
    s.close()
    return {"converged": conv, "skin_friction_drag_vjp": chk}


def converged_swbli_vjp(api, mesh, method, mach, re, extra, orders=6.0, max_steps=40000, lift_at=16384):
    """The shock/boundary-layer interaction at full size converged `orders` orders under the
    reference's pseudo-transient control with a continuation schedule for the CFL cap: 1.5
    through the start-up transient (the first `lift_at` steps; a cap of 2.5 or more goes
    non-finite there with the reference's scalar diagonal preconditioner), then 10
    (cfdg_set_cfl_max); then the wall-pressure VJP (x in [0.3, 0.7]) at that state against
    central differences along 16 seeded directions."""
    s = api.Solver(mesh, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision="mixed",
                   jv="exact", cfl_max=1.5, **method, **extra)
    s.setFreestreamStatic(mach, 101325.0, 300.0)
    s.setKinematicViscosity(re, 1.0)
    s.initialize()
    s.reset_newton()
    s.synchronize()
    t0 = time.perf_counter()
    recs = []
    while len(recs) < max_steps:
        if len(recs) == lift_at:
            s.set_cfl_max(10.0)
        r, _ = s.newton_steps(64)
        recs += r
        if recs[-1].res_vm <= 10.0 ** -orders * recs[0].res_vm:
            break
    s.synchronize()
    conv = {"n_cells": mesh.n_cells, "newton_steps": len(recs), "seconds": round(time.perf_counter() - t0, 3),
            "res_vm_first_last": [recs[0].res_vm, recs[-1].res_vm],
            "res_rho_first_last": [recs[0].res_rho, recs[-1].res_rho],
            "orders": math.log10(recs[0].res_vm / recs[-1].res_vm),
            "gmres_iters": int(sum(x.gmres_iters for x in recs)),
            "cfl_cap": f"1.5 for the first {lift_at} steps, then 10"}
    chk = vjp_fd_check(s, s.getSolution(), "wall_pressure", 0.3, 0.7, seed=37, steps=(1e-9, 1e-8))
    s.close()
    return {"converged": conv, "wall_pressure_vjp": chk}


def _golden(name):
    """A converged FP64 CPU-oracle solution (tests/golden/make_converged.py) and its mesh."""
    import numpy as np
    from mycode_gb300 import meshgen
    d = np.load(os.path.join(ROOT, "tests", "golden", name))
    return d, meshgen.MeshSpec(str(d["name"]), d["nodes"], d["cells"], d["bedges"])


def _solve_to(s, max_steps, tol_rho=1e-10, chain=16):
    """Newton steps from the current state until the density residual is at or below
    tol_rho (after step 5): wall time, steps, GMRES iterations.  The steps run in chains
    (cfdg_newton_steps: with the graph driver one host synchronisation per chain, the CFL
    control and the density test on the device)."""
    s.synchronize()
    t0 = time.perf_counter()
    n, reached, its, rec = 0, False, 0, None
    while n < max_steps and not reached:
        recs, reached = s.newton_steps(min(chain, max_steps - n), 0.0, tol_rho)
        n += len(recs)
        its += sum(r.gmres_iters for r in recs)
        rec = recs[-1]
    s.synchronize()
    return {"seconds": round(time.perf_counter() - t0, 4), "newton_steps": n, "gmres_iters": its,
            "reached": reached, "final_res_rho": rec.res_rho}


def time_to_converge(api, max_steps=1500):
    """Wall time of full solves from the free stream to a volume-weighted density residual
    of 1e-10, mixed precision (FP32 Krylov basis and exact J v, FP64 residual and update)
    against the FP64 paths, with the errors of the converged solutions against the FP64
    CPU oracle's converged solution (tests/golden/, made by tests/golden/make_converged.py
    and checked bit for bit against the compiled reference):
      wedge   120 x 80 x 2 (19,200 cells, 10 % jitter), M 2.5, HLLC + BJ limiter, GMRES(30),
              first CFL 10.  The reference freezes its limiter at the state step 7 reached
              (src/Solver.cpp:1714); every run here keeps the oracle's frozen limiter from the
              start, so all of them solve the oracle's discrete problem.  Error: the wall Cp
              (slip wall, tag 3) and the state.
      plate   the laminar flat plate 60 x 30 (Roe + viscous, central, the reference's
              GMRES(40) and first CFL 0.1).  Error: wall Cf and Cp (tag 4) and the state.
    Also the first-order wedge pair (no limiter) against each other."""
    import numpy as np
    dw, spec_w = _golden("wedge_converged.npz")
    mesh_w = api.Mesh.from_spec(spec_w)

    def wedge(prec, jv, spatial="SECOND_ORDER_LIMITED"):
        limited = spatial == "SECOND_ORDER_LIMITED"
        s = api.Solver(mesh_w, bcset="supersonic", init="freestream", viscous=0, precision=prec, jv=jv, gmres_m=30,
                       cfl0=10.0, flux="HLLC", spatial=spatial, limiter_freeze_step=-1 if limited else 150)
        s.setFlowConditions(2.5, 101325.0, 300.0)
        s.initialize()
        if limited:
            s.set_limiters(dw["phi"])
        res = _solve_to(s, max_steps)
        U, cp = s.getSolution()[:, :4], s.wall_coefficients(3)[1]
        s.close()
        return res, U, cp

    out = {"workload": "supersonic wedge 120x80x2 (19,200 cells), M 2.5, HLLC + BJ limiter (the FP64 oracle's frozen "
                       "limiter in every run), GMRES(30), first CFL 10"}
    for name, prec, jv in (("mixed", "mixed", "exact"), ("fp64_exact", "fp64", "exact"), ("fp64_fd", "fp64", "fd")):
        r, U, cp = wedge(prec, jv)
        r["state_rel_l2_vs_fp64_oracle"] = float(np.linalg.norm(U - dw["U"]) / np.linalg.norm(dw["U"]))
        r["wall_cp_max_abs_diff_vs_fp64_oracle"] = float(np.abs(cp - dw["cp_wall"]).max())
        out[name] = r
    out["oracle_steps_to_1e-10"] = int(dw["n_reach"])
    out["speedup_mixed_vs_fp64_fd"] = out["fp64_fd"]["seconds"] / out["mixed"]["seconds"]
    out["speedup_mixed_vs_fp64_exact"] = out["fp64_exact"]["seconds"] / out["mixed"]["seconds"]

    dp, spec_p = _golden("plate_converged.npz")
    mesh_p = api.Mesh.from_spec(spec_p)
    plate = {"workload": "laminar flat plate 60x30 quads (1,800 cells), stretching 1.08, M 0.2, Re_L 1e5, Roe + "
                         "viscous, 2nd-order central, GMRES(40), first CFL 0.1",
             "oracle_steps_to_1e-10": int(dp["n_reach"])}
    for name, prec, jv in (("mixed", "mixed", "exact"), ("fp64_fd", "fp64", "fd")):
        s = api.Solver(mesh_p, bcset="plate", init="freestream", viscous=1, precision=prec, jv=jv, flux="ROE",
                       spatial="SECOND_ORDER_CENTRAL")
        s.setFreestreamStatic(0.2, 101325.0, 300.0)
        s.setKinematicViscosity(1e5, 1.0)
        s.initialize()
        r = _solve_to(s, 4 * max_steps)
        _, cp, cf = s.wall_coefficients(4)
        U = s.getSolution()[:, :4]
        s.close()
        r["state_rel_l2_vs_fp64_oracle"] = float(np.linalg.norm(U - dp["U"]) / np.linalg.norm(dp["U"]))
        r["wall_cf_max_abs_diff_vs_fp64_oracle"] = float(np.abs(cf - dp["cf_wall"]).max())
        r["wall_cp_max_abs_diff_vs_fp64_oracle"] = float(np.abs(cp - dp["cp_wall"]).max())
        plate[name] = r
    plate["speedup_mixed_vs_fp64_fd"] = plate["fp64_fd"]["seconds"] / plate["mixed"]["seconds"]
    out["laminar_plate"] = plate

    m1, Um, cpm = wedge("mixed", "exact", "FIRST_ORDER")
    f1, Uf, cpf = wedge("fp64", "exact", "FIRST_ORDER")
    out["first_order"] = {
        "mixed": m1, "fp64_exact": f1, "speedup_mixed_vs_fp64_exact": f1["seconds"] / m1["seconds"],
        "state_rel_l2_mixed_vs_fp64": float(np.linalg.norm(Um - Uf) / np.linalg.norm(Uf)),
        "wall_cp_max_abs_diff_mixed_vs_fp64": float(np.abs(cpm - cpf).max()),
        "workload": "the same wedge, HLLC first order (no limiter), to a density residual of 1e-10"}
    return out


# ---------------------------------------------------------------- CPU side

def _oracle_headline(target: int):
    """The CPU restatement (oracle/) on the headline mesh, scheme and state."""
    from oracle.oracle import OracleSolver
    spec = headline_spec(target)
    o = OracleSolver(spec, bcset="bump", viscous=True, init="bump")
    o.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    o.setFlowConditions(0.5, 101325.0, 300.0)
    o.setKinematicViscosity(3e6, 1.0)
    o.initialize()
    U = o.get_state()
    k, w = o.sst_freestream()
    U[:, 4] = U[:, 0] * k
    U[:, 5] = U[:, 0] * w
    return spec, o, perturb_state(U, o.cells()[:, 1:])


def _cpu_worker(args):
    """One independent copy of the CPU path: `warm` untimed FP64 SST residual evaluations of
    the headline case, then `steps` timed ones (or as many as fit in `seconds` when steps is
    0)."""
    target, warm, steps, seconds = args
    sys.path.insert(0, ROOT)
    spec, o, U = _oracle_headline(target)
    for _ in range(warm):
        o.residual_sst(U)
    n, t0 = 0, time.perf_counter()
    while (steps and n < steps) or (not steps and time.perf_counter() - t0 < seconds):
        o.residual_sst(U)
        n += 1
    return n, time.perf_counter() - t0, o.n_cells


def cpu_baseline_sample(target: int, seconds: float):
    """The CPU path on one host core: FP64 SST residual evaluations of the headline case for
    about `seconds` after one untimed evaluation."""
    from oracle.oracle import build_oracle
    build_oracle()
    n, t, nc = _cpu_worker((target, 1, 0, seconds))
    return {"value": n * nc / t, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{n} FP64 residual evaluations (SST, HLLC, BJ limiter, viscous) of the same {nc:,}-cell "
                      f"mesh and state on 1 host core after one untimed evaluation, {t:.1f} s (oracle/ restatement; "
                      "the reference has no SST)"}


def reference_copies(per_copy_bytes: float = 3.2e9) -> int:
    """One copy per host core, capped by the memory available (a copy of the 4M-cell case
    holds about 2.5 GB)."""
    cores = os.cpu_count() or 1
    try:
        avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
        return max(1, min(cores, int(avail // per_copy_bytes)))
    except (ValueError, OSError, AttributeError):
        return cores


def reference_arm(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.oracle import build_oracle
    build_oracle()
    copies = reference_copies()
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(copies) as pool:
        res = pool.map(_cpu_worker, [(args.cells, args.warmup, args.steps, 0.0)] * copies)
    nc = res[0][2]
    evals = sum(r[0] for r in res)
    t = max(r[1] for r in res)
    value = evals * nc / t
    spec = headline_spec(args.cells)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mesh recipe and seeded smooth perturbation of the initial state)",
        "config": dict(headline_workload(spec), parallelism="1 GPU"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": copies, "kind": "port",
                         "sample": f"{copies} independent copies (one per host core{' the memory allows' if copies < (os.cpu_count() or 1) else ''}) "
                                   f"x {args.steps} FP64 residual evaluations of the same {nc:,}-cell mesh and state "
                                   f"after {args.warmup} untimed ones ({evals} evaluations in {t:.1f} s); the plain-C "
                                   "restatement of the reference's residual with the SST terms (oracle/; the "
                                   "reference has no SST)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- bandwidth sweep

SWEEP_SIZES = (64_000, 256_000, 1_000_000, 4_000_000)


def sweep(args):
    """Per-kernel throughput of the residual, the exact J v and the VJP in FP64 and FP32 on
    the headline's Gaussian-bump channel at 64k-4M cells; one JSON line."""
    from mycode_gb300 import api
    peak, peak_kind = measured_peak()
    sizes = [int(x) for x in args.sweep_sizes.split(",")] if args.sweep_sizes else SWEEP_SIZES
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pipe_peak_warp = api.fp64_pipe_rate(local) / 32.0
    pipe_prof = profile_fp64_pipe()
    out = []
    clk = ClockSampler(local)
    clk.start()
    for target in sizes:
        spec = headline_spec(target)
        mesh = api.Mesh.from_spec(spec)
        s = bump_solver(api, mesh, local)
        U = perturb_state(s.getSolution(), mesh.cells()[:, 1:])
        s.set_state(U)
        res = {"n_cells": mesh.n_cells, "n_faces": mesh.n_faces}
        res.update(kernel_paths(s, U, mesh.n_cells, mesh.n_faces, peak, args.sweep_reps, pipe_peak_warp, pipe_prof))
        res["vjp_fp32"] = None  # the adjoint runs in FP64 only
        out.append(res)
        s.close()
        del mesh
    clocks = clk.stop()
    cpu = None if args.no_cpu_baseline else cpu_baseline_sample(sizes[0], 5.0)
    line = {"metric": "bandwidth sweep: cell-residuals/s per kernel", "unit": UNIT,
            "config": {"workload": "Gaussian bump channel 3x1 (height 0.05, width 0.2), triangles, 10% seeded jitter, "
                                   "M=0.5 Re=3e6, SST, HLLC, 2nd-order limited; seeded smooth perturbation of the "
                                   "initial state", "l2": "flushed before every evaluation"},
            "peak_gbs": peak, "peak_source": peak_kind, "fp64_pipe_warp_inst_per_s": pipe_peak_warp, "sizes": out,
            "clocks": clocks, "cpu_baseline": cpu}
    print(json.dumps(line))


# ---------------------------------------------------------------- profiling cases

def profile_case(args):
    """One kernel path, `--reps` times, on a chosen case, printing per-kernel CUDA-event
    times: the workload for ncu captures (profiles/ gives the exact commands).
    Paths: residual64 / residual32 (the FP64 / FP32 residual), jv64 / jv32 (exact J v),
    vjp64 (the adjoint), krylov_stream (mixed Newton steps whose GMRES runs the graph
    driver's kernels from the stream driver, outside a graph, so ncu sees them).
    Workloads: the headline's bump channel at --cells (SST unless --no-sst) or the laminar
    plate of the Newton-step measurement."""
    import numpy as np
    from mycode_gb300 import api, meshgen
    gm = {}
    if args.gmres_m is not None:
        gm["gmres_m"] = args.gmres_m
    if args.gmres_tol is not None:
        gm["gmres_tol"] = args.gmres_tol
    if args.gather_split_cells is not None:
        gm["gather_split_cells"] = args.gather_split_cells
    if args.profile_workload == "laminar_plate":
        m = api.Mesh.from_spec(meshgen.laminar_plate(240, 120, ratio=1.08))
        s = api.Solver(m, bcset="plate", init="freestream", viscous=1, flux="ROE", spatial="SECOND_ORDER_CENTRAL",
                       precision="mixed", jv="exact", krylov=2, **gm)
        s.setFreestreamStatic(0.2, 101325.0, 300.0)
        s.setKinematicViscosity(1e5, 1.0)
        s.initialize()
        U = s.getSolution()
    else:
        m = api.Mesh.from_spec(headline_spec(args.cells))
        s = api.Solver(m, bcset="bump", init="bump", viscous=1, turbulence="none" if args.no_sst else "sst",
                       flux="HLLC", spatial="SECOND_ORDER_LIMITED", precision="mixed", jv="exact", krylov=2, **gm)
        s.setFlowConditions(0.5, 101325.0, 300.0)
        s.setKinematicViscosity(3e6, 1.0)
        s.initialize()
        U = perturb_state(s.getSolution(), m.cells()[:, 1:])
        s.set_state(U)
    s.set_timing(True)
    s.residual_device(True)
    s.set_dt(s.local_timestep(100.0))
    v = np.random.default_rng(3).standard_normal(U.shape) * np.abs(U).mean(axis=0)
    lam = np.random.default_rng(4).standard_normal(U.shape)
    run, prefix = {
        "residual64": (lambda: s.residual_device(True), "residual."),
        "residual32": (lambda: s.residual32(), "residual."),
        "jv64": (lambda: s.apply_jacobian(U, None, v, mode="exact"), "jv."),
        "jv32": (lambda: s.apply_jacobian32(U, v), "jv."),
        "vjp64": (lambda: s.vjp(lam, U), "vjp."),
        "krylov_stream": (lambda: s.newton_step(0.0), "krylov."),
    }[args.profile_case]
    run()  # warm-up: every kernel of the path launched once (module loading) before the stats
    s.synchronize()
    s.kernel_stats(reset=True)
    t0 = time.perf_counter()
    iters = []
    for _ in range(args.reps):
        r = run()
        if args.profile_case == "krylov_stream":
            iters.append(r[0].gmres_iters)
    s.synchronize()
    st = s.kernel_stats(reset=True)
    line = {"path": args.profile_case, "workload": args.profile_workload, "cells": m.n_cells, "faces": m.n_faces,
            "ms_per_launch": {k: round(v[0] / v[1], 5) for k, v in st.items() if k.startswith(prefix) and v[1]},
            "wall_s": time.perf_counter() - t0}
    if iters:
        # Arnoldi iterations per solve and the mean basis index j over them (iteration j
        # reads j + 1 stored vectors)
        line["gmres_iters"] = iters
        line["mean_j"] = sum(i * (i - 1) / 2 for i in iters) / max(1, sum(iters))
        line["launches"] = {k: v[1] for k, v in st.items() if k.startswith(prefix) and v[1]}
        # algorithmic bytes of each stage at the mean j, per launch, and the bandwidth
        nv = 4 if args.profile_workload == "laminar_plate" or args.no_sst else 6
        spatial = "SECOND_ORDER_CENTRAL" if args.profile_workload == "laminar_plate" else "SECOND_ORDER_LIMITED"
        peak, _ = measured_peak()
        line["algorithmic"] = {}
        for k, ms in line["ms_per_launch"].items():
            b = krylov_bytes(k.split(".")[1], m.n_cells, m.n_faces, nv, 4, line["mean_j"], spatial)
            line["algorithmic"][k] = {"MB": round(b / 1e6, 1), "GBs": round(b / (ms * 1e-3) / 1e9, 1),
                                      "hbm_frac": round(b / (ms * 1e-3) / 1e9 / peak, 3)}
    print(json.dumps(line))


def profile_krylov_iteration(args):
    """Time of one Arnoldi iteration of the graph GMRES (the WHILE body, mixed precision,
    exact J v) on a small mesh: Newton steps at GMRES tolerance 0 with Krylov dimensions
    10 and 30 (every solve runs all of them); the slope of the step time over the
    iterations is the iteration time.  Workloads: the limited supersonic wedge of
    time_to_1e-10 (the FP64 oracle's frozen limiter) and the 240 x 120 laminar plate."""
    import numpy as np
    from mycode_gb300 import api, meshgen
    if args.profile_workload == "laminar_plate":
        mesh = api.Mesh.from_spec(meshgen.laminar_plate(240, 120, ratio=1.08))

        def make(m, prec):
            s = api.Solver(mesh, bcset="plate", init="freestream", viscous=1, flux="ROE",
                           spatial="SECOND_ORDER_CENTRAL", precision=prec, jv="exact", gmres_m=m, gmres_tol=0.0)
            s.setFreestreamStatic(0.2, 101325.0, 300.0)
            s.setKinematicViscosity(1e5, 1.0)
            s.initialize()
            return s
    else:
        dw, spec = _golden("wedge_converged.npz")
        mesh = api.Mesh.from_spec(spec)

        def make(m, prec):
            s = api.Solver(mesh, bcset="supersonic", init="freestream", viscous=0, precision=prec, jv="exact",
                           gmres_m=m, gmres_tol=0.0, cfl0=10.0, flux="HLLC", spatial="SECOND_ORDER_LIMITED",
                           limiter_freeze_step=-1)
            s.setFlowConditions(2.5, 101325.0, 300.0)
            s.initialize()
            s.set_limiters(dw["phi"])
            return s
    line = {"path": "krylov_iteration", "workload": args.profile_workload, "cells": mesh.n_cells}
    for prec in ("mixed", "fp64"):
        t = {}
        for m in (10, 30):
            s = make(m, prec)
            for _ in range(3):
                s.newton_step(0.0)
            s.synchronize()
            t0 = time.perf_counter()
            its = [s.newton_step(0.0)[0].gmres_iters for _ in range(args.reps)]
            s.synchronize()
            t[m] = ((time.perf_counter() - t0) / args.reps, float(np.mean(its)))
            s.close()
        line[prec] = {"ms_per_step": {m: round(v[0] * 1e3, 4) for m, v in t.items()},
                      "us_per_iteration": round((t[30][0] - t[10][0]) / (t[30][1] - t[10][1]) * 1e6, 2)}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=HEADLINE_CELLS, help="target cells of the bump channel")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--quick", action="store_true", help="the headline only (no secondary measurements)")
    ap.add_argument("--sweep", action="store_true", help="bandwidth sweep on the bump channel instead")
    ap.add_argument("--sweep-sizes", default="", help="comma-separated target cell counts")
    ap.add_argument("--sweep-reps", type=int, default=10)
    ap.add_argument("--profile-case", default=None,
                    choices=["residual64", "residual32", "jv64", "jv32", "vjp64", "krylov_stream",
                             "krylov_iteration"],
                    help="run one kernel path --reps times (ncu workload) instead")
    ap.add_argument("--profile-workload", default="bump", choices=["bump", "laminar_plate", "wedge"])
    ap.add_argument("--no-sst", action="store_true", help="profile case: the bump without SST")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--gmres-m", type=int, default=None, help="profile case: Krylov dimension")
    ap.add_argument("--gmres-tol", type=float, default=None, help="profile case: GMRES tolerance (0: m iterations)")
    ap.add_argument("--gather-split-cells", type=int, default=None,
                    help="profile case: cfdg_config.gather_split_cells (-1: the fused gather/dot kernel at any size)")
    args = ap.parse_args()
    if args.warmup < 3 and not args.profile_case:
        ap.error("--warmup must be at least 3")
    if args.profile_workload == "wedge" and args.profile_case != "krylov_iteration":
        ap.error("--profile-workload wedge is for --profile-case krylov_iteration")
    if args.profile_case == "krylov_iteration":
        profile_krylov_iteration(args)
    elif args.profile_case:
        profile_case(args)
    elif args.sweep:
        sweep(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
