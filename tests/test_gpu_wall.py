"""Wall quantities on the GPU against the oracle (itself pinned to the reference's
calculateDrag, extractSkinFriction, calculateEntropyError and computeWallDistances).

The kernels evaluate the reference's expressions in its IEEE order (no FMA
contraction), so the wall distance, Cp, Cf and the drag (summed in reference face
order) are compared bit for bit.  The entropy error sums over cells through a
deterministic tree reduction and a device pow(), so its bar is 1e-13 relative.
"""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def _pair(api, name, seed=21, renumber="hilbert", **cfg):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec, renumber=renumber)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], **cfg)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    for x in (s, o):
        C.setup(x, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=seed, amplitude=0.08)
    s.set_state(U)
    o.set_state(U)
    return s, o


@pytest.mark.parametrize("renumber", ["hilbert", "rcm"])
@pytest.mark.parametrize("name", ["plate_visc", "bump"])
def test_wall_distance_bit_exact(cuda_lib, name, renumber):
    s, o = _pair(cuda_lib, name, renumber=renumber)
    np.testing.assert_array_equal(s.wall_distance(), o.wall_distance())


def test_wall_distance_of_sst_solver(cuda_lib):
    spec = mg.turb_plate(40, 24)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst")
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    np.testing.assert_array_equal(s.wall_distance(), o.wall_distance())


@pytest.mark.parametrize("tag", [4, 3, 1])
def test_wall_coefficients_bit_exact(cuda_lib, tag):
    s, o = _pair(cuda_lib, "plate_visc")
    xs, cps, cfs = s.wall_coefficients(tag)
    xo, cpo, cfo = o.wall_coefficients(tag)
    assert len(xs) == len(xo) > 0
    np.testing.assert_array_equal(xs, xo)
    np.testing.assert_array_equal(cps, cpo)
    np.testing.assert_array_equal(cfs, cfo)


@pytest.mark.parametrize("name", ["supersonic", "bump", "plate"])
def test_drag_bit_exact(cuda_lib, name):
    s, o = _pair(cuda_lib, name)
    assert s.drag() == o.drag()


@pytest.mark.parametrize("name", ["bump", "supersonic", "plate_visc"])
def test_entropy_error(cuda_lib, name):
    s, o = _pair(cuda_lib, name)
    assert s.entropy_error() == pytest.approx(o.entropy_error(), rel=1e-13, abs=0)


def test_wall_quantities_follow_the_solve(cuda_lib):
    """After Newton steps the QoIs read the solver's current state."""
    s, o = _pair(cuda_lib, "plate_visc")
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    s.solveImplicit(tol=1e-30, max_steps=5)
    o.set_state(s.getSolution())
    np.testing.assert_array_equal(s.wall_coefficients(4)[2], o.wall_coefficients(4)[2])


@pytest.mark.parametrize("kind,name", [("pressure_drag", "supersonic"), ("skin_friction_drag", "plate_visc"),
                                       ("wall_pressure", "plate_visc")])
def test_objective_and_gradient_bit_exact(cuda_lib, kind, name):
    s, o = _pair(cuda_lib, name)
    Js, gs = s.objective(kind, 0.1, 0.6)
    Jo, go = o.objective(kind, 0.1, 0.6)
    assert Js == Jo and Js != 0.0
    np.testing.assert_array_equal(gs, go)
    if kind == "pressure_drag":
        assert Js == s.drag()
