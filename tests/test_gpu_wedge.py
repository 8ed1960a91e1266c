"""The supersonic wedge (120 x 80 quads split into 19,200 triangles, 10 % seeded jitter;
M 2.5, HLLC, Barth-Jespersen limiter, GMRES(30), CFL from 10): the reference's
pseudo-transient algorithm (FP64, FD J v) on the GPU against the CPU oracle, which is
bit-identical to the compiled reference on this path, from the free stream to a
volume-weighted residual of 1e-3 (about 420 Newton steps).
The GPU's reductions (FD epsilon, GMRES dot products) sum in a different order, so the
traces agree to round-off growth rather than bit for bit: closely over the first steps,
then both converge (see the assertions' comment for why not to the same state)."""
import numpy as np
import pytest

from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def test_wedge_converges_with_the_cpu_path(cuda_lib):
    spec = mg.wedge(120, 80, jitter=0.10, seed=0)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="supersonic", init="freestream", viscous=0, precision="fp64", jv="fd", gmres_m=30,
                        krylov=0, cfl0=10.0)
    o = OracleSolver(spec, bcset="supersonic", viscous=False, init="freestream")
    o.setGMRES(30)
    o.setCFL0(10.0)
    for x in (s, o):
        x.setFlowConditions(2.5, 101325.0, 300.0)
        x.initialize()
        x.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    tg = s.solveImplicit(1e-3, 600)
    to = o.solveImplicit(1e-3, 600)
    rg, ro = tg["res_vm"], to["res_vm"]
    n = min(len(rg), len(ro))
    rel = np.abs(rg[:n] - ro[:n]) / ro[:n]
    Ug, Uo = s.getSolution()[:, :4], o.get_state()[:, :4]
    dU = np.linalg.norm(Ug - Uo) / np.linalg.norm(Uo)
    print("steps", len(rg), len(ro), "max rel res diff first 10 / 300:", rel[:10].max(), rel[:300].max(),
          "final state rel L2 diff:", dU, "final res", rg[-1], ro[-1])
    # The first steps agree to round-off.  The transient then drifts apart: the limiter
    # and the CFL control amplify round-off, and the reference freezes the limiter at
    # whatever state step 150 (or the last step with CFL <= 10) reached, so the two
    # converged states are steady states of slightly different frozen-limiter residuals.
    assert rel[:10].max() <= 1e-6
    assert len(rg) < 600 and len(ro) < 600
    assert abs(len(rg) - len(ro)) <= 40
    assert dU <= 1e-2
