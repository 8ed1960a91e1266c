"""The known-answer properties of tests/test_oracle_known_answers.py on the GPU path:
free-stream preservation of the FP64 residual (every scheme and order, inviscid and
viscous) and of the FP32 residual, Green-Gauss exactness for linear fields on a uniform
grid, the Barth-Jespersen limiter's bounds and its value 1 for a linear pressure, and
plane Couette flow (zero mass and momentum residual, the energy residual the viscous
heating), plane Poiseuille flow (zero mass and momentum residual), discrete
conservation in a box closed by slip walls and the residual's rotation with the mesh."""
import numpy as np
import pytest

import cases as C
import test_oracle_known_answers as K
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver, normal_flux

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,spec", [("supersonic", lambda: mg.wedge(24, 16, jitter=0.1, seed=3)),
                                       ("plate_visc", lambda: mg.laminar_plate(24, 16, ratio=1.1))])
def test_free_stream_preservation(cuda_lib, name, spec):
    spec = spec()
    case = C.CASES[name]
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], precision="mixed")
    C.setup(s, case)
    U = s.getSolution()
    assert np.ptp(U[:, :4], axis=0).max() == 0.0
    keep = K._layers_from_boundary(spec, 2)
    scale = np.abs(normal_flux(U[0], 1.0, 0.0)).max() * m.faces()[1][:, 2].max()
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            R = s.computeResiduals(U)
            assert np.abs(R[keep, :4]).max() <= 1e-11 * scale, (name, fl, sp)
            R32 = s.residual32(U)
            assert np.abs(R32[keep, :4]).max() <= 2e-5 * scale, (name, fl, sp, "fp32")


def test_green_gauss_exact_for_linear_fields(cuda_lib):
    spec, o, xc = K._linear_box()
    x, y = xc[:, 0], xc[:, 1]
    coef = ((1.1, 0.2, -0.1), (80.0, 30.0, -20.0), (-10.0, 15.0, 25.0), (1e5, 3e3, -2e3))
    prim = np.stack([a + b * x + c * y for a, b, c in coef], axis=1)
    U = o.state_from_primitives(prim)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="bump", viscous=0, init="bump")
    s.setFlowConditions(0.3, 101325.0, 300.0)
    s.initialize()
    G = s.gradients(U)
    keep = K._layers_from_boundary(spec, 1)
    for q, (a, b, c) in enumerate(coef):
        for d, want in enumerate((b, c)):
            assert np.abs(G[keep, 2 * q + d] - want).max() <= 1e-10 * max(abs(b), abs(c)), (q, d)


def test_limiter_bounds_and_linear_pressure(cuda_lib):
    spec = mg.wedge(24, 16, jitter=0.1, seed=5)
    o = OracleSolver(spec, bcset="supersonic", viscous=False, init="freestream")
    o.setFlowConditions(2.5, 101325.0, 300.0)
    o.initialize()
    U = C.perturbed_state(o.get_state(), o.cells(), seed=9, amplitude=0.15)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="supersonic", viscous=0, init="freestream")
    s.setFlowConditions(2.5, 101325.0, 300.0)
    s.initialize()
    phi = s.limiters(U)
    assert (phi >= 0.0).all() and (phi <= 1.0).all() and (phi < 1.0).any()
    spec, o, xc = K._linear_box()
    x, y = xc[:, 0], xc[:, 1]
    prim = np.stack([np.full_like(x, 1.2), 50.0 + 10.0 * x, 5.0 - 3.0 * y, 1e5 * (1.0 + 0.05 * x - 0.03 * y)], axis=1)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="bump", viscous=0, init="bump")
    s.setFlowConditions(0.3, 101325.0, 300.0)
    s.initialize()
    phi = s.limiters(o.state_from_primitives(prim))
    assert (phi[K._layers_from_boundary(spec, 2)] == 1.0).all()


def test_plane_couette_flow(cuda_lib):
    spec = mg.box(10, 8)
    _, U, keep, vol, tau, heat = K.couette(spec)
    s = cuda_lib.Solver(cuda_lib.Mesh.from_spec(spec), bcset="plate", viscous=1, init="freestream")
    K.couette_setup(s)
    K.check_couette(s, U, keep, vol, tau, heat, s.computeResiduals)


def test_plane_poiseuille_flow(cuda_lib):
    spec = mg.box(10, 8)
    _, U, keep, scale = K.poiseuille(spec)
    s = cuda_lib.Solver(cuda_lib.Mesh.from_spec(spec), bcset="plate", viscous=1, init="freestream")
    K.couette_setup(s)
    K.check_poiseuille(s, U, keep, scale, s.computeResiduals)


def test_discrete_conservation_in_a_closed_box(cuda_lib):
    for spec, bc, visc, _, U, scale in K.closed_box_cases():
        s = cuda_lib.Solver(cuda_lib.Mesh.from_spec(spec), bcset=bc, viscous=int(visc), init="freestream")
        K.closed_box_setup(s)
        K.check_closed_box(s, U, visc, scale, s.computeResiduals)


def test_residual_rotates_with_the_mesh(cuda_lib):
    for spec, rspec, visc, U, Ur, keep, cs in K.rotated_cases():
        a = cuda_lib.Solver(cuda_lib.Mesh.from_spec(spec), bcset="plate", viscous=int(visc), init="freestream")
        b = cuda_lib.Solver(cuda_lib.Mesh.from_spec(rspec), bcset="plate", viscous=int(visc), init="freestream")
        for x in (a, b):
            K.closed_box_setup(x)
        K.check_rotated(a, b, U, Ur, keep, cs, a.computeResiduals, b.computeResiduals)
