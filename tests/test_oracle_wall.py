"""The oracle's wall quantities against the compiled reference: wall distance
(computeWallDistances), pressure drag (calculateDrag), the L2 entropy error
(calculateEntropyError) and the skin-friction distribution (extractSkinFriction,
which the reference writes with six significant digits)."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver, RefSolver, ref_available, ref_variant

needs_ref = pytest.mark.skipif(not ref_available("bump"), reason="reference build oracle/_ref absent")


def _pair(name, seed=21):
    case = C.CASES[name]
    spec = case["spec"]()
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    r = RefSolver(spec, variant=ref_variant(case["bcset"], case["viscous"]))
    for x in (o, r):
        C.setup(x, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=seed, amplitude=0.08)
    o.set_state(U)
    r.set_state(U)
    return o, r, U


@needs_ref
@pytest.mark.parametrize("name", ["plate_visc", "bump"])
def test_wall_distance_bit_exact(name):
    o, r, _ = _pair(name)
    np.testing.assert_array_equal(o.wall_distance(), r.wall_distance())


@needs_ref
@pytest.mark.parametrize("name", ["bump", "supersonic"])
def test_drag_bit_exact(name):
    o, r, _ = _pair(name)
    assert o.drag() == r.drag()
    if name == "supersonic":  # the ramp carries pressure drag; the bump case's box walls are flat
        assert o.drag() != 0.0


@needs_ref
@pytest.mark.parametrize("name", ["bump", "plate_visc"])
def test_entropy_error_bit_exact(name):
    o, r, _ = _pair(name)
    assert o.entropy_error() == r.entropy_error()


@needs_ref
def test_skin_friction_matches_reference_csv(tmp_path):
    o, r, _ = _pair("plate_visc")
    x_ref, cf_ref = r.skin_friction(tmp_path / "cf.csv")
    x, cp, cf = o.wall_coefficients(4)
    assert len(x) == len(x_ref) > 0
    order = np.argsort(x, kind="stable")
    np.testing.assert_allclose(x[order], x_ref, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(cf[order], cf_ref, rtol=1e-5, atol=1e-12)
    assert np.isfinite(cp).all()


def test_wall_coefficients_count_and_cp_definition():
    case = C.CASES["plate_visc"]
    o = OracleSolver(case["spec"](), bcset="plate", viscous=True, init="freestream")
    C.setup(o, case)
    x, cp, cf = o.wall_coefficients(4)
    assert len(x) > 0
    # the free stream itself: p = p_exit, so Cp = 0; u_t of the owner > 0 gives Cf > 0
    np.testing.assert_allclose(cp, 0.0, atol=1e-12)
    assert (cf > 0).all()
    assert len(o.wall_coefficients(1)[0]) > 0
    assert len(o.wall_coefficients(7)[0]) == 0


@pytest.mark.parametrize("kind", ["pressure_drag", "skin_friction_drag", "wall_pressure"])
def test_objective_gradient_matches_central_differences(kind):
    name = "supersonic" if kind == "pressure_drag" else "plate_visc"
    case = C.CASES[name]
    o = OracleSolver(case["spec"](), bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=4, amplitude=0.08)
    o.set_state(U)
    J, g = o.objective(kind, 0.1, 0.6)
    assert J != 0.0 and np.abs(g).max() > 0
    rng = np.random.default_rng(1)
    for _ in range(4):
        v = rng.standard_normal(U.shape) * np.abs(U).mean(axis=0)
        v[:, 4:] = 0
        h = 1e-6
        o.set_state(U + h * v)
        jp = o.objective(kind, 0.1, 0.6, gradient=False)
        o.set_state(U - h * v)
        jm = o.objective(kind, 0.1, 0.6, gradient=False)
        fd = (jp - jm) / (2 * h)
        assert fd == pytest.approx(float(np.sum(g * v)), rel=1e-6, abs=1e-12 * abs(J))


@needs_ref
def test_pressure_drag_objective_is_calculate_drag():
    o, r, _ = _pair("supersonic")
    assert o.objective("pressure_drag", gradient=False) == r.drag()
