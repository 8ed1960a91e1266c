"""CUDA residual path against the CPU oracle and the reference's fixtures.

The FP64 kernels are compiled without FMA contraction and sum every cell in the
reference's face order, so R(U), the gradients, the limiter, the local time step and
the preconditioner must agree bit for bit with the oracle; the only exception is the
bump set's subsonic inlet, whose ghost state goes through pow() (CUDA's and glibc's
may differ in the last bit), where the bar is 1e-12 relative.  Quantities that pass
through global reductions (FD J v's epsilon, GMRES) are compared with tolerances.
"""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

REL = 1e-12  # bar for the FP64 residual path


def _make(api, name, renumber="hilbert", spec=None, **cfg):
    case = C.CASES[name]
    spec = case["spec"]() if spec is None else spec
    m = api.Mesh.from_spec(spec, renumber=renumber)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], **cfg)
    C.setup(s, case)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    return case, s, o


def _assert_match(got, want, exact, what):
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(got - want).max()
    if exact:
        assert np.array_equal(got, want), f"{what}: max abs diff {err:.3e} (scale {scale:.3e})"
    else:
        assert err <= REL * scale, f"{what}: rel err {err / scale:.3e}"


@pytest.mark.parametrize("name", list(C.CASES))
def test_initial_state_and_params(cuda_lib, name):
    case, s, o = _make(cuda_lib, name)
    assert s.params() == pytest.approx(o.params(), rel=0, abs=0)
    np.testing.assert_array_equal(s.getSolution(), o.get_state())


@pytest.mark.parametrize("renumber", ["hilbert", "none", "rcm"])
@pytest.mark.parametrize("name", list(C.CASES))
def test_residual_all_schemes(cuda_lib, name, renumber):
    case, s, o = _make(cuda_lib, name, renumber=renumber)
    exact = case["bcset"] != "bump"
    U = C.perturbed_state(o.get_state(), o.cells(), seed=3, amplitude=0.08)
    _assert_match(s.gradients(U), o.gradients(U), exact, "gradients")
    _assert_match(s.limiters(U), o.limiters(U), exact, "limiters")
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            o.setNumericalMethod(fl, sp)
            _assert_match(s.computeResiduals(U), o.residual(U), exact, f"R {fl} {sp}")
            # frozen limiter: both keep the values of the last update
            _assert_match(s.computeResiduals(U, False), o.residual(U, False), exact, f"R frozen {fl} {sp}")


@pytest.mark.parametrize("name,spec", [("supersonic", lambda: mg.wedge(260, 200, jitter=0.1, seed=4)),
                                       ("plate_visc", lambda: mg.laminar_plate(300, 180, ratio=1.02))])
def test_residual_bit_exact_with_per_face_gradient_terms(cuda_lib, name, spec):
    """Meshes with more than 100,000 interior faces, where the FP64 residual forms each
    interior face's Green-Gauss terms once (k_grad_faces64) and the gradient kernel adds
    them: the gradients, limiter and residual still equal the oracle's bit for bit."""
    case, s, o = _make(cuda_lib, name, spec=spec())
    assert s.mesh.n_faces - s.mesh.n_boundary_faces >= 100_000
    U = C.perturbed_state(o.get_state(), o.cells(), seed=7, amplitude=0.08)
    _assert_match(s.gradients(U), o.gradients(U), True, "gradients")
    _assert_match(s.limiters(U), o.limiters(U), True, "limiters")
    for fl in C.FLUXES:
        for sp in ("SECOND_ORDER_CENTRAL", "SECOND_ORDER_LIMITED"):
            s.setNumericalMethod(fl, sp)
            o.setNumericalMethod(fl, sp)
            _assert_match(s.computeResiduals(U), o.residual(U), True, f"R {fl} {sp}")


@pytest.mark.parametrize("name", list(C.CASES))
def test_against_reference_fixtures(cuda_lib, name):
    import os
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cases.npz"))
    case, s, o = _make(cuda_lib, name, spec=C.golden_spec(gold, name))
    exact = case["bcset"] != "bump"
    U = np.zeros((s.n_cells, 6))
    U[:, :4] = gold[f"{name}/U"]
    _assert_match(s.gradients(U), gold[f"{name}/G"], exact, "gradients vs reference")
    _assert_match(s.limiters(U), gold[f"{name}/phi"], exact, "limiter vs reference")
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            _assert_match(s.computeResiduals(U)[:, :4], gold[f"{name}/{fl}/{sp}/R"], exact, f"R vs reference {fl} {sp}")
    s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    s.set_state(U)
    _assert_match(s.local_timestep(5.0), gold[f"{name}/dt"], True, "dt vs reference")
    _assert_match(s.preconditioner(), gold[f"{name}/D"], exact, "D vs reference")


@pytest.mark.parametrize("name", list(C.CASES))
def test_pseudo_time_jv_gmres(cuda_lib, name):
    case, s, o = _make(cuda_lib, name)
    exact = case["bcset"] != "bump"
    U = C.perturbed_state(o.get_state(), o.cells(), seed=4)
    for x in (s, o):
        x.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    Rs, Ro = s.computeResiduals(U), o.residual(U)
    s.set_state(U)
    o.set_state(U)
    _assert_match(s.local_timestep(5.0), o.local_timestep(5.0), True, "dt")
    _assert_match(s.preconditioner(), o.preconditioner(), exact, "D")
    v = C.random_direction(U.shape[0], seed=8)
    Jo = o.apply_jacobian(U, Ro, v)
    Js = s.apply_jacobian(U, Ro, v, mode="fd")
    assert np.linalg.norm(Js - Jo) <= 1e-6 * np.linalg.norm(Jo)
    it_s, xs = s.gmres(U, Ro, -Ro)
    it_o, xo = o.gmres(U, Ro, -Ro)
    assert abs(it_s - it_o) <= 1
    if it_s == it_o:
        assert np.linalg.norm(xs - xo) <= 1e-6 * np.linalg.norm(xo)


def test_residual_is_deterministic(cuda_lib):
    case, s, o = _make(cuda_lib, "supersonic")
    U = C.perturbed_state(o.get_state(), o.cells(), seed=5)
    a = s.computeResiduals(U)
    b = s.computeResiduals(U)
    np.testing.assert_array_equal(a, b)
    s.set_state(U)
    x1 = s.gmres(U, a, -a)[1]
    x2 = s.gmres(U, a, -a)[1]
    np.testing.assert_array_equal(x1, x2)


@pytest.mark.parametrize("name", list(C.CASES))
def test_newton_trace_against_reference(cuda_lib, name):
    import os
    from golden.make_golden import TRACE_METHOD
    gold = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_cases.npz"))
    case, s, o = _make(cuda_lib, name, spec=C.golden_spec(gold, name))
    s.setNumericalMethod(*TRACE_METHOD[name])
    tr = s.solveImplicit(0.0, 25)
    g = gold[f"{name}/trace_res_vm"]
    np.testing.assert_allclose(tr["res_vm"], g, rtol=1e-7)
    np.testing.assert_array_equal(tr["cfl"], gold[f"{name}/trace_cfl"])
    np.testing.assert_array_equal(tr["gmres_iters"], gold[f"{name}/trace_iters"])
    Ug = gold[f"{name}/trace_U"]
    assert np.abs(s.getSolution()[:, :4] - Ug).max() <= 1e-7 * np.abs(Ug).max()
