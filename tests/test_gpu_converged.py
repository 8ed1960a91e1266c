"""Converged solutions on the GPU against the FP64 CPU path (fixtures made by
tests/golden/make_converged.py from the oracle, checked bit for bit against the compiled
reference where it exists).

The supersonic wedge (19,200 cells, HLLC, Barth-Jespersen limiter, GMRES(30), first CFL
10): the reference freezes its limiter at whatever state step 7 reached
(src/Solver.cpp:1714), so two runs whose transients differ by round-off converge to the
steady states of slightly different frozen-limiter residuals.  Every run here therefore
takes the oracle's frozen limiter phi (cfdg_set_limiters) and keeps it from the start
(limiter_freeze_step = -1), as the fixture's own solve did: all of them solve
R(U; phi) = 0.

* The reference's algorithm (FP64, finite-difference J v, host-driven modified
  Gram-Schmidt) follows the oracle's 300-step Newton trace (to round-off over the first
  steps, within the transient's GMRES-count jitter after) and converges to its state.
* Mixed precision (FP32 Krylov basis and exact J v, FP64 residual and update) and FP64
  with exact J v reach a density residual of 1e-10 with the wall Cp within 1e-6 of the
  oracle's (the target), and the converged states agree with the oracle's to 1e-10.
* The laminar flat plate (60 x 30, Roe + viscous, the reference's GMRES(40) and first CFL
  0.1) does the same for the wall Cf and Cp (no limiter)."""
import os

import numpy as np
import pytest

from mycode_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
STATE_REL = 1e-10   # converged states, relative L2 over the four conserved variables
WALL_ABS = 1e-6     # wall Cp / Cf, absolute (the path's stated target)


def fixture(name):
    d = np.load(os.path.join(GOLDEN, name))
    spec = mg.MeshSpec(str(d["name"]), d["nodes"], d["cells"], d["bedges"])
    return d, spec


def wedge_solver(api, spec, phi, **cfg):
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset="supersonic", init="freestream", viscous=0, gmres_m=30, cfl0=10.0,
                   limiter_freeze_step=-1, **cfg)
    s.setFlowConditions(2.5, 101325.0, 300.0)
    s.initialize()
    s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    s.set_limiters(phi)
    return s


def plate_solver(api, spec, **cfg):
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset="plate", init="freestream", viscous=1, **cfg)
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(1e5, 1.0)
    s.initialize()
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    return s


def run_to(s, tol_rho, extra, max_steps):
    """Newton steps until the density residual is at or below tol_rho (after step 5),
    then `extra` steps more; returns the per-step records and the index of the step that
    reached tol_rho."""
    recs, reached = [], None
    while len(recs) < max_steps:
        rec, _ = s.newton_step(0.0)
        recs.append(rec)
        if reached is None and rec.res_rho <= tol_rho and len(recs) > 5:
            reached = len(recs) - 1
        if reached is not None and len(recs) > reached + extra:
            break
    return recs, reached


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_wedge_reference_algorithm_follows_the_oracle_300_steps_and_converges_to_its_state(cuda_lib):
    d, spec = fixture("wedge_converged.npz")
    s = wedge_solver(cuda_lib, spec, d["phi"], precision="fp64", jv="fd", krylov=0)
    recs, reached = run_to(s, 1e-10, int(d["extra"]), len(d["res_vm"]) + 200)
    rg = np.array([r.res_vm for r in recs])
    ro = d["res_vm"]
    n = min(300, len(rg), len(ro))
    rel = np.abs(rg[:n] - ro[:n]) / ro[:n]
    iters_g = np.array([r.gmres_iters for r in recs[:n]])
    dU = rel_l2(s.getSolution()[:, :4], d["U"])
    dcp = float(np.abs(s.wall_coefficients(3)[1] - d["cp_wall"]).max())
    msg = (f"300-step trace: max rel res diff {rel.max():.2e} (first 50: {rel[:50].max():.2e}), GMRES iteration "
           f"differences {int(np.abs(iters_g - d['gmres_iters'][:n]).sum())}; density 1e-10 at step {reached} "
           f"(oracle {int(d['n_reach'])}); final state rel diff {dU:.2e}; wall Cp max diff {dcp:.2e}")
    print(msg)
    # The first steps agree to round-off; after that the two runs' reductions (the FD
    # epsilon's norms, the Gram-Schmidt dots) sum in different orders, a GMRES solve now and
    # then takes one iteration more or less, and the CFL control follows it, so single steps'
    # residuals differ by up to an order of magnitude mid-transient; both runs reach the
    # density residual of 1e-10 within a few steps of each other, at the same state.
    ratio = np.abs(np.log10(rg[:n] / ro[:n]))
    msg += f"; max |log10 ratio| over 300 steps {ratio.max():.2f}"
    assert n == 300 and reached is not None, msg
    assert rel[:10].max() <= 1e-6, msg
    assert ratio.max() <= 2.0, msg
    assert abs(reached - int(d["n_reach"])) <= 30, msg
    assert dU <= STATE_REL, msg
    assert dcp <= WALL_ABS, msg


@pytest.mark.parametrize("precision,jv", [("mixed", "exact"), ("fp64", "exact")])
def test_wedge_reaches_1e10_with_wall_cp_of_the_oracle(cuda_lib, precision, jv):
    d, spec = fixture("wedge_converged.npz")
    s = wedge_solver(cuda_lib, spec, d["phi"], precision=precision, jv=jv)
    recs, reached = run_to(s, 1e-10, int(d["extra"]), 3000)
    dU = rel_l2(s.getSolution()[:, :4], d["U"])
    dcp = float(np.abs(s.wall_coefficients(3)[1] - d["cp_wall"]).max())
    msg = (f"{precision}/{jv}: density 1e-10 at step {reached} (oracle {int(d['n_reach'])}), final res_rho "
           f"{recs[-1].res_rho:.2e}; state rel diff {dU:.2e}; wall Cp max diff {dcp:.2e}")
    print(msg)
    assert reached is not None, msg
    assert dcp <= WALL_ABS, msg
    assert dU <= STATE_REL, msg


@pytest.mark.parametrize("precision,jv", [("mixed", "exact"), ("fp64", "fd")])
def test_plate_wall_cf_cp_of_the_oracle(cuda_lib, precision, jv):
    d, spec = fixture("plate_converged.npz")
    s = plate_solver(cuda_lib, spec, precision=precision, jv=jv)
    recs, reached = run_to(s, 1e-10, int(d["extra"]), 6000)
    x, cp, cf = s.wall_coefficients(4)
    np.testing.assert_array_equal(x, d["x_wall"])
    dU = rel_l2(s.getSolution()[:, :4], d["U"])
    dcf = float(np.abs(cf - d["cf_wall"]).max())
    dcp = float(np.abs(cp - d["cp_wall"]).max())
    msg = (f"{precision}/{jv}: density 1e-10 at step {reached} (oracle {int(d['n_reach'])}); state rel diff "
           f"{dU:.2e}; wall Cf max diff {dcf:.2e} (Cf range {d['cf_wall'].min():.3e}..{d['cf_wall'].max():.3e}); "
           f"wall Cp max diff {dcp:.2e}")
    print(msg)
    assert reached is not None, msg
    assert dcf <= WALL_ABS and dcp <= WALL_ABS, msg
    assert dU <= STATE_REL, msg
