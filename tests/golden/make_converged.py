"""Converged FP64 solutions of the CPU path: the accuracy fixtures of the GPU solves.

    python tests/golden/make_converged.py

Writes
  wedge_converged.npz   the supersonic wedge 120 x 80 x 2 (19,200 cells, 10 % seeded
                        jitter), M 2.5, HLLC, Barth-Jespersen limiter, GMRES(30), first
                        CFL 10.  (1) The solve from the free stream with the reference's own
                        limiter freeze (src/Solver.cpp:1714: step > 150 or CFL > 10, here
                        reached at step 7) gives the frozen limiter phi.  (2) The solve from
                        the free stream with that phi frozen from the start, to a
                        volume-weighted density residual of 1e-10 and then EXTRA steps more
                        (the residual reaches its round-off floor): per-step res_vm, res_rho,
                        CFL and GMRES iterations, the final state and the wall Cp (tag 3).
  plate_converged.npz   the laminar flat plate 60 x 30 quads (stretching 1.08), M 0.2,
                        Re_L 1e5, Roe + viscous flux, second-order central, GMRES(40), first
                        CFL 0.1 (the reference's settings), to a density residual of 1e-10
                        and EXTRA steps more: the same trace, the final state and the wall Cp
                        and Cf (tag 4).
Both carry their meshes (node coordinates can differ in the last bit between machines).

The runs are the plain-C restatement (oracle/cfd_oracle.c).  Where the reference itself
is compiled (oracle/build_ref.py; its GMRES size, first CFL and limiter-freeze rule set
at compile time for the wedge), every run is repeated with it first and must agree bit
for bit: state, limiter and per-step residuals.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from mycode_gb300 import meshgen as mg  # noqa: E402
from oracle.oracle import OracleSolver, RefSolver, build_oracle, ref_available  # noqa: E402

EXTRA = 40
STOP_RHO = 1e-10


def _mesh(spec):
    return dict(nodes=spec.nodes, cells=spec.cells, bedges=spec.bedges, name=np.array(spec.name))


def _check_same(what, a, b):
    if not np.array_equal(a, b):
        raise SystemExit(f"{what}: the oracle differs from the compiled reference "
                         f"(max {np.abs(np.asarray(a) - np.asarray(b)).max():.3e})")


def wedge():
    spec = mg.wedge(120, 80, jitter=0.10, seed=0)

    def oracle(frozen_phi=None):
        o = OracleSolver(spec, bcset="supersonic", viscous=False, init="freestream")
        o.setGMRES(30)
        o.setCFL0(10.0)
        o.setFlowConditions(2.5, 101325.0, 300.0)
        o.initialize()
        o.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
        if frozen_phi is not None:
            o.set_limiters(frozen_phi)
            o.setLimiterFreeze(-1)
        return o

    # (1) the reference's own freeze: the limiter stops changing after step 7
    o = oracle()
    tr1 = o.solveImplicit(0.0, 20)
    phi = o.get_limiters()
    freeze_step = int(np.flatnonzero(tr1["cfl"] > 10.0)[0])
    # (2) phi frozen from the start, to the density tolerance, then EXTRA steps more
    o = oracle(phi)
    o.setStopRho(STOP_RHO)
    n_reach = len(o.solveImplicit(0.0, 3000)["res_rho"]) - 1  # index of the step that reached it
    o = oracle(phi)
    tr = o.solveImplicit(0.0, n_reach + EXTRA)
    U = o.get_state()
    x, cp, _ = o.wall_coefficients(3)
    if ref_available("supersonic_m30_cfl10"):
        r = RefSolver(spec, "supersonic_m30_cfl10")
        r.setFlowConditions(2.5, 101325.0, 300.0)
        r.initialize()
        r.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
        rt = r.solveImplicit(0.0, 20)
        _check_same("wedge natural-freeze limiter", r.get_limiters(), phi)
        _check_same("wedge natural-freeze trace", rt["res_vm"], tr1["res_vm"])
        r = RefSolver(spec, "supersonic_m30_cfl10_frozen")
        r.setFlowConditions(2.5, 101325.0, 300.0)
        r.initialize()
        r.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
        r.set_limiters(phi)
        rt = r.solveImplicit(0.0, n_reach + EXTRA)
        _check_same("wedge frozen-limiter trace", rt["res_vm"], tr["res_vm"])
        _check_same("wedge frozen-limiter gmres", rt["gmres_iters"], tr["gmres_iters"])
        _check_same("wedge frozen-limiter state", r.get_state(), U)
        print("wedge: compiled reference agrees bit for bit")
    np.savez_compressed(os.path.join(HERE, "wedge_converged.npz"), **_mesh(spec), phi=phi,
                        freeze_step=freeze_step, n_reach=n_reach, extra=EXTRA,
                        res_vm=tr["res_vm"], res_rho=tr["res_rho"], cfl=tr["cfl"], gmres_iters=tr["gmres_iters"],
                        U=U[:, :4], x_wall=x, cp_wall=cp)
    print(f"wedge: freeze at step {freeze_step}, density residual {STOP_RHO:g} at step {n_reach}, "
          f"final res_rho {tr['res_rho'][-1]:.3e}")


def plate():
    spec = mg.laminar_plate(60, 30, ratio=1.08)

    def oracle():
        o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
        o.setFreestreamStatic(0.2, 101325.0, 300.0)
        o.setKinematicViscosity(1e5, 1.0)
        o.initialize()
        o.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
        return o

    o = oracle()
    o.setStopRho(STOP_RHO)
    n_reach = len(o.solveImplicit(0.0, 5000)["res_rho"]) - 1
    o = oracle()
    tr = o.solveImplicit(0.0, n_reach + EXTRA)
    U = o.get_state()
    x, cp, cf = o.wall_coefficients(4)
    if ref_available("plate_visc"):
        r = RefSolver(spec, "plate_visc")
        r.setFreestreamStatic(0.2, 101325.0, 300.0)
        r.setKinematicViscosity(1e5, 1.0)
        r.initialize()
        r.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
        rt = r.solveImplicit(0.0, n_reach + EXTRA)
        _check_same("plate trace", rt["res_vm"], tr["res_vm"])
        _check_same("plate state", r.get_state(), U)
        print("plate: compiled reference agrees bit for bit")
    np.savez_compressed(os.path.join(HERE, "plate_converged.npz"), **_mesh(spec), n_reach=n_reach, extra=EXTRA,
                        res_vm=tr["res_vm"], res_rho=tr["res_rho"], cfl=tr["cfl"], gmres_iters=tr["gmres_iters"],
                        U=U[:, :4], x_wall=x, cp_wall=cp, cf_wall=cf)
    print(f"plate: density residual {STOP_RHO:g} at step {n_reach}, final res_rho {tr['res_rho'][-1]:.3e}")


if __name__ == "__main__":
    build_oracle()
    wedge()
    plate()
