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


def test_nasa_plate_fixture_wall_and_blasius_columns(tmp_path):
    """The reference's NASA laminar flat plate (its mesh and shipped results/data/cf_profile.csv,
    tests/golden/make_golden.py): the profile's x column is the tag-4 face midpoints of the
    mesh as this project ingests it, and its Blasius column 0.664 / sqrt(Re_x) follows from
    the flow set up as the reference's plate case does (setFlowConditions(0.1, 41368.5,
    388.89), setKinematicViscosity(2e5, 0.3048); src/Solver.cpp:34-43, :1899-1979)."""
    import gzip
    import os

    from mycode_gb300 import meshgen as mg

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    p = tmp_path / "plate_nasa.msh"
    with gzip.open(os.path.join(gold, "plate_nasa.msh.gz"), "rb") as fh:
        p.write_bytes(fh.read())
    spec = mg.read_gmsh(str(p))
    assert spec.n_cells == 6962
    prof = np.loadtxt(os.path.join(gold, "plate_cf_profile.csv"), delimiter=",", skiprows=1)
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    o.setFlowConditions(0.1, 41368.5, 388.89)
    o.setKinematicViscosity(200000.0, 0.3048)
    o.initialize()
    x, cp, cf = o.wall_coefficients(4)
    order = np.argsort(x, kind="stable")
    assert len(x) == len(prof) == 79
    np.testing.assert_allclose(x[order], prof[:, 0], rtol=5e-6)
    par = o.params()
    gam = 1.4
    u_inf = par["M_inf"] * np.sqrt(gam * par["R_gas"] * par["T0"] / (1.0 + 0.5 * (gam - 1.0) * par["M_inf"] ** 2))
    blasius = 0.664 / np.sqrt(u_inf * prof[:, 0] / par["nu"])
    np.testing.assert_allclose(blasius, prof[:, 2], rtol=1e-5)
