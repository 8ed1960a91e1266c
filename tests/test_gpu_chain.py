"""Chained Newton steps (graph driver): the steps of solveImplicit enqueued back to back
with the reference's CFL control (src/Solver.cpp:1747-1750, :1780-1796) and limiter-freeze
decision (:1714) taken on the device between them.  The trace must be the one of single
steps bit for bit, across the limiter freeze and up to a convergence in mid-chain, and
cfdg_newton_steps must continue a solve exactly where the last call left it."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

CASES = [("supersonic", "mixed", "exact", "HLLC"), ("plate_visc", "fp64", "exact", "ROE"),
         ("bump", "fp64", "fd", "LLF")]


def _solver(api, name, precision, jv, flux, chain):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], precision=precision,
                   jv=jv, krylov=1, newton_chain=chain, cfl0=2.0)
    C.setup(s, case)
    s.setNumericalMethod(flux, "SECOND_ORDER_LIMITED")
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    s.set_state(C.perturbed_state(o.get_state(), o.cells(), seed=21))
    return s


def _same(a, b):
    for k in ("res_vm", "res_abs", "res_rho", "cfl", "gmres_iters"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("name,precision,jv,flux", CASES)
def test_chained_solve_has_the_single_step_trace(cuda_lib, name, precision, jv, flux):
    one = _solver(cuda_lib, name, precision, jv, flux, 1)
    ten = _solver(cuda_lib, name, precision, jv, flux, 10)
    a = one.solveImplicit(0.0, 25)
    b = ten.solveImplicit(0.0, 25)
    _same(a, b)
    # the limiter freeze (CFL > 10) falls inside the run
    assert a["cfl"].max() > 10.0 and a["cfl"].min() < 10.0, a["cfl"]
    np.testing.assert_array_equal(one.getSolution(), ten.getSolution())


def test_chained_solve_stops_at_convergence_in_mid_chain(cuda_lib):
    ref = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1)
    tr = ref.solveImplicit(0.0, 20)
    tol = float(tr["res_vm"][13]) * (1.0 + 1e-12)   # reached at step 13 (first below: <= 13)
    first = int(np.flatnonzero(tr["res_vm"] < tol)[0])
    a = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1).solveImplicit(tol, 40)
    b = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 8).solveImplicit(tol, 40)
    assert a["converged"] and b["converged"]
    assert len(a["res_vm"]) == len(b["res_vm"]) == first + 1
    _same(a, b)


def test_chained_steps_stop_at_the_density_tolerance(cuda_lib):
    ref = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1)
    tr = ref.solveImplicit(0.0, 20)
    tol_rho = float(tr["res_rho"][12]) * (1.0 + 1e-12)
    first = 6 + int(np.flatnonzero(tr["res_rho"][6:] <= tol_rho)[0])
    s = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1)
    s.reset_newton()
    recs, cv = s.newton_steps(40, 0.0, tol_rho)
    assert cv and len(recs) == first + 1
    np.testing.assert_array_equal([r.res_vm for r in recs], tr["res_vm"][: first + 1])
    np.testing.assert_array_equal([r.cfl for r in recs], tr["cfl"][: first + 1])


def test_newton_steps_continue_the_solve(cuda_lib):
    whole = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1)
    w = whole.solveImplicit(0.0, 25)
    parts = _solver(cuda_lib, "supersonic", "mixed", "exact", "HLLC", 1)
    parts.reset_newton()
    r1, c1 = parts.newton_steps(13)
    r2, c2 = parts.newton_steps(12)
    assert not c1 and not c2 and len(r1) == 13 and len(r2) == 12
    recs = r1 + r2
    np.testing.assert_array_equal([r.res_vm for r in recs], w["res_vm"])
    np.testing.assert_array_equal([r.cfl for r in recs], w["cfl"])
    np.testing.assert_array_equal([r.gmres_iters for r in recs], w["gmres_iters"])
    np.testing.assert_array_equal(parts.getSolution(), whole.getSolution())
