"""Known-answer tests of the reference's discretisation on the CPU oracle: properties that
hold whatever the floating-point operation order, so they pin the restatement (and, through
the bit-exact parity tests, the GPU path) to the mathematics as well as to the reference.

  consistency           F(U, U, n) = F.n(U) for LLF, Roe and HLLC (include/Flux.hpp:36-213)
  rotational invariance rotating both states' velocities and the normal by one angle rotates
                        the momentum flux by it and leaves mass and energy fluxes unchanged
  free-stream           R(U_inf) = 0 on cells two layers or more from the boundary, every
  preservation          scheme and order, inviscid and viscous (src/Solver.cpp:529-801)
  Green-Gauss           exact gradients of linear rho, u, v, p on interior cells of a uniform
                        quad grid (src/Solver.cpp:81-149)
  Barth-Jespersen       phi in [0, 1] for any state, and phi = 1 on interior cells for a linear
                        pressure field (src/Solver.cpp:152-253)
  plane Couette flow    u = a y, v = 0, constant rho and p: the stress mu a is uniform, so the
                        mass and momentum residuals vanish on interior cells for every scheme
                        and order, and the energy residual is the viscous heating
                        -mu a^2 vol wherever the scheme adds no dissipation of its own (HLLC,
                        which resolves the shear wave, and every flux with the limited
                        reconstruction, exact for a linear field) (src/Solver.cpp:543-800)
  rotated residual     rotating the mesh and every cell's velocity by one angle rotates the
                        momentum rows of the whole residual (reconstruction, limiter, Riemann
                        and viscous fluxes) on cells three layers from the boundary and leaves
                        mass and energy unchanged, every scheme and order
  discrete             in a box closed by slip walls the interior face fluxes telescope: the
  conservation         cells' mass residuals sum to zero (and, inviscid, their energy
                        residuals) for any state, scheme, order and BC set
  oblique shock        the converged supersonic wedge (M 2.5, 15 degree ramp from x = 0.5,
                        tests/golden/wedge_converged.npz, the oracle's solution, bit for bit
                        the compiled reference's): wall Cp 0 upstream of the ramp and, past the
                        shock foot, the theta-beta-M relation's weak-shock value
  plane Poiseuille flow u = u0 + b y (y - 1) with mu u'' = dp/dx, p linear in x, constant rho:
                        with the limited reconstruction (exact at the faces for the linear p and
                        the quadratic u, phi = 1) the interior mass and momentum residuals
                        vanish for every flux: the Green-Gauss gradients, their face average
                        and its correction are exact for quadratics on a uniform grid
"""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver, inviscid_flux, normal_flux

GAMMA = 1.4


def _cons(r, u, v, p):
    return np.array([r, r * u, r * v, p / (GAMMA - 1.0) + 0.5 * r * (u * u + v * v), 0.0, 0.0])


def _random_states(rng, n, mach_max):
    out = []
    for _ in range(n):
        r = rng.uniform(0.3, 3.0)
        p = rng.uniform(2e4, 3e5)
        c = np.sqrt(GAMMA * p / r)
        speed = rng.uniform(0.0, mach_max) * c
        th = rng.uniform(0.0, 2 * np.pi)
        out.append(_cons(r, speed * np.cos(th), speed * np.sin(th), p))
    return out


@pytest.mark.parametrize("scheme", ["LLF", "ROE", "HLLC"])
def test_flux_consistency(scheme):
    rng = np.random.default_rng(11)
    for U in _random_states(rng, 400, 3.0):
        th = rng.uniform(0.0, 2 * np.pi)
        nx, ny = np.cos(th), np.sin(th)
        F = inviscid_flux(U, U, nx, ny, scheme)
        Fn = normal_flux(U, nx, ny)
        scale = np.abs(Fn).max()
        assert np.abs(F[:4] - Fn[:4]).max() <= 1e-13 * scale, (scheme, U, F, Fn)


def _rotate(U, a):
    c, s = np.cos(a), np.sin(a)
    R = U.copy()
    R[1] = c * U[1] - s * U[2]
    R[2] = s * U[1] + c * U[2]
    return R


@pytest.mark.parametrize("scheme", ["LLF", "ROE", "HLLC"])
def test_flux_rotational_invariance(scheme):
    rng = np.random.default_rng(12)
    states = _random_states(rng, 600, 2.5)
    for k in range(0, len(states), 2):
        UL, UR = states[k], states[k + 1]
        th = rng.uniform(0.0, 2 * np.pi)
        nx, ny = np.cos(th), np.sin(th)
        F = inviscid_flux(UL, UR, nx, ny, scheme)
        a = rng.uniform(0.0, 2 * np.pi)
        Fr = inviscid_flux(_rotate(UL, a), _rotate(UR, a), np.cos(th + a), np.sin(th + a), scheme)
        scale = np.abs(F).max()
        want = _rotate(F, a)
        assert np.abs(Fr[:4] - want[:4]).max() <= 1e-11 * scale, (scheme, UL, UR, F, Fr)


def _layers_from_boundary(spec, depth):
    """Cells at least `depth` face-neighbour layers away from every boundary face."""
    o = OracleSolver(spec, bcset="supersonic", viscous=False, init="freestream")
    ints, _ = o.faces()
    owner, nbr = ints[:, 2], ints[:, 3]
    nc = spec.n_cells
    near = np.zeros(nc, bool)
    near[owner[nbr < 0]] = True
    inner = nbr >= 0
    for _ in range(depth - 1):
        grow = near.copy()
        a, b = owner[inner], nbr[inner]
        grow[a[near[b]]] = True
        grow[b[near[a]]] = True
        near = grow
    return ~near


@pytest.mark.parametrize("name,spec", [("supersonic", lambda: mg.wedge(24, 16, jitter=0.1, seed=3)),
                                       ("plate_visc", lambda: mg.laminar_plate(24, 16, ratio=1.1))])
def test_free_stream_preservation(name, spec):
    spec = spec()
    case = C.CASES[name]
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    U = o.get_state()
    assert np.ptp(U[:, :4], axis=0).max() == 0.0  # a uniform free stream
    keep = _layers_from_boundary(spec, 2)
    assert keep.sum() > 50
    areas = o.faces()[1][:, 2]
    scale = np.abs(normal_flux(U[0], 1.0, 0.0)).max() * areas.max()
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            o.setNumericalMethod(fl, sp)
            R = o.residual(U)
            assert np.abs(R[keep, :4]).max() <= 1e-11 * scale, (name, fl, sp)


def _linear_box(nx=10, ny=8):
    spec = mg.box(nx, ny)
    o = OracleSolver(spec, bcset="bump", viscous=False, init="bump")
    o.setFlowConditions(0.3, 101325.0, 300.0)
    o.initialize()
    xc = o.cells()[:, 1:]
    return spec, o, xc


def test_green_gauss_exact_for_linear_fields():
    spec, o, xc = _linear_box()
    x, y = xc[:, 0], xc[:, 1]
    coef = {"rho": (1.1, 0.2, -0.1), "u": (80.0, 30.0, -20.0), "v": (-10.0, 15.0, 25.0), "p": (1e5, 3e3, -2e3)}
    prim = np.stack([a + b * x + c * y for a, b, c in coef.values()], axis=1)
    U = o.state_from_primitives(prim)
    G = o.gradients(U)
    keep = _layers_from_boundary(spec, 1)
    assert keep.sum() >= 40
    for q, (a, b, c) in enumerate(coef.values()):
        for d, want in enumerate((b, c)):
            got = G[keep, 2 * q + d]
            assert np.abs(got - want).max() <= 1e-10 * max(abs(b), abs(c)), (list(coef)[q], d)


def test_limiter_bounds_and_linear_pressure():
    # any state: 0 <= phi <= 1
    o = OracleSolver(mg.wedge(24, 16, jitter=0.1, seed=5), bcset="supersonic", viscous=False, init="freestream")
    o.setFlowConditions(2.5, 101325.0, 300.0)
    o.initialize()
    U = C.perturbed_state(o.get_state(), o.cells(), seed=9, amplitude=0.15)
    phi = o.limiters(U)
    assert (phi >= 0.0).all() and (phi <= 1.0).all() and (phi < 1.0).any()
    # a linear pressure (constant density, linear temperature) on a uniform grid: every
    # reconstructed face pressure lies between the cell's and its neighbour's, so phi = 1
    spec, o, xc = _linear_box()
    x, y = xc[:, 0], xc[:, 1]
    prim = np.stack([np.full_like(x, 1.2), 50.0 + 10.0 * x, 5.0 - 3.0 * y, 1e5 * (1.0 + 0.05 * x - 0.03 * y)], axis=1)
    phi = o.limiters(o.state_from_primitives(prim))
    keep = _layers_from_boundary(spec, 2)
    assert (phi[keep] == 1.0).all()


def couette(spec):
    """The plane Couette state on `spec` (cells in the spec's numbering), from an oracle set
    up with the reference's setters: the oracle, the state, interior cells, cell volumes, the
    stress scale mu a A and the heating mu a^2."""
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    couette_setup(o)
    cells = o.cells()
    y = cells[:, 2]
    a, rho = 400.0, 1.2
    U = np.stack([_cons(rho, 30.0 + a * yc, 0.0, 1e5) for yc in y])
    mu = rho * o.params()["nu"]
    keep = _layers_from_boundary(spec, 2)
    return o, U, keep, cells[:, 0], mu * a * o.faces()[1][:, 2].max(), mu * a * a


def couette_setup(s):
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(1e3, 1.0)
    s.initialize()


COUETTE_EXACT_ENERGY = [(fl, sp) for fl in C.FLUXES for sp in C.SPATIALS if fl == "HLLC" or sp == "SECOND_ORDER_LIMITED"]


def check_couette(s, U, keep, vol, tau, heat, residual):
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            R = residual(U)
            assert np.abs(R[keep, 0]).max() <= 1e-11 * tau, (fl, sp)
            assert np.abs(R[keep, 1:3]).max() <= 1e-11 * tau, (fl, sp)
            if (fl, sp) in COUETTE_EXACT_ENERGY:
                want = -heat * vol[keep]
                assert np.abs(R[keep, 3] / want - 1.0).max() <= 1e-10, (fl, sp)


def test_plane_couette_flow():
    o, U, keep, vol, tau, heat = couette(mg.box(10, 8))
    assert keep.sum() >= 20
    check_couette(o, U, keep, vol, tau, heat, o.residual)


def poiseuille(spec):
    """The plane Poiseuille state on `spec` (u from 37 to 60 m/s, dp/dx = -20 Pa/m): the
    oracle, the state, interior cells and the scale |dp/dx| vol."""
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    couette_setup(o)
    cells = o.cells()
    x, y = cells[:, 1], cells[:, 2]
    rho, dpdx = 1.2, -20.0
    b = dpdx / (2.0 * rho * o.params()["nu"])
    U = np.stack([_cons(rho, 30.0 + b * yc * (yc - 1.0), 0.0, 1e5 + dpdx * xc) for xc, yc in zip(x, y)])
    return o, U, _layers_from_boundary(spec, 2), abs(dpdx) * cells[:, 0].max()


def check_poiseuille(s, U, keep, scale, residual):
    for fl in C.FLUXES:
        s.setNumericalMethod(fl, "SECOND_ORDER_LIMITED")
        R = residual(U)
        assert np.abs(R[keep, :3]).max() <= 1e-10 * scale, fl


def test_plane_poiseuille_flow():
    o, U, keep, scale = poiseuille(mg.box(10, 8))
    check_poiseuille(o, U, keep, scale, o.residual)


def oblique_shock_cp(mach, theta_deg, gamma=GAMMA):
    """Wall Cp behind the weak attached oblique shock of a wedge (the theta-beta-M relation
    tan theta = 2 cot beta (M^2 sin^2 beta - 1) / (M^2 (gamma + cos 2 beta) + 2), then the
    normal-shock pressure ratio of M sin beta)."""
    from scipy.optimize import brentq
    th = np.radians(theta_deg)

    def f(b):
        m2s = mach * mach * np.sin(b) ** 2
        return np.tan(th) - 2.0 / np.tan(b) * (m2s - 1.0) / (mach * mach * (gamma + np.cos(2.0 * b)) + 2.0)

    beta = brentq(f, np.arcsin(1.0 / mach) + 1e-9, np.radians(64.0))  # the weak root
    p21 = 1.0 + 2.0 * gamma / (gamma + 1.0) * (mach * mach * np.sin(beta) ** 2 - 1.0)
    return (p21 - 1.0) / (0.5 * gamma * mach * mach), np.degrees(beta)


def test_wedge_ramp_pressure_is_the_oblique_shock_value():
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "wedge_converged.npz"))
    x, cp = d["x_wall"], d["cp_wall"]
    cp_th, beta = oblique_shock_cp(2.5, 15.0)
    assert abs(beta - 36.945) < 1e-2 and abs(cp_th - 0.33543) < 1e-4
    assert np.abs(cp[x < 0.45]).max() <= 1e-12
    ramp = x > 0.65
    assert ramp.sum() >= 10
    assert np.abs(cp[ramp] / cp_th - 1.0).max() <= 1e-2


def closed_box_cases():
    """(solver arguments, perturbed state, mass scale) for a jittered triangulated box
    closed by slip walls, every BC set, inviscid and viscous."""
    ts = mg.TAG_SLIP
    spec = mg.box(12, 9, split=True, jitter=0.15, seed=4, tags=(ts, ts, ts, ts))
    out = []
    for bc in ("bump", "plate", "supersonic"):
        for visc in (False, True):
            o = OracleSolver(spec, bcset=bc, viscous=visc, init="freestream")
            closed_box_setup(o)
            U = C.perturbed_state(o.get_state(), o.cells(), seed=3, amplitude=0.1)
            scale = np.abs(U[:, 0]).max() * 100.0 * o.faces()[1][:, 2].max()
            out.append((spec, bc, visc, o, U, scale))
    return out


def closed_box_setup(s):
    s.setFreestreamStatic(0.3, 101325.0, 300.0)
    s.setKinematicViscosity(1e3, 1.0)
    s.initialize()


def check_closed_box(s, U, visc, scale, residual):
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            R = residual(U)
            assert abs(R[:, 0].sum()) <= 1e-13 * scale, (fl, sp, visc)
            if not visc:  # slip walls do no pressure work; the viscous wall terms do
                assert abs(R[:, 3].sum()) <= 1e-13 * scale * 3e5, (fl, sp)


def test_discrete_conservation_in_a_closed_box():
    for spec, bc, visc, o, U, scale in closed_box_cases():
        check_closed_box(o, U, visc, scale, o.residual)


def rotated_cases(angle=0.7):
    """(mesh, rotated mesh, viscous, state, rotated state, interior cells, rotation) for a
    jittered triangulated box, inviscid and viscous."""
    import copy
    spec = mg.box(14, 10, split=True, jitter=0.15, seed=7)
    c, s = np.cos(angle), np.sin(angle)
    rspec = copy.deepcopy(spec)
    rspec.nodes = spec.nodes @ np.array([[c, s], [-s, c]])
    keep = _layers_from_boundary(spec, 3)
    out = []
    for visc in (False, True):
        o = OracleSolver(spec, bcset="plate", viscous=visc, init="freestream")
        closed_box_setup(o)
        U = C.perturbed_state(o.get_state(), o.cells(), seed=3, amplitude=0.1)
        Ur = U.copy()
        Ur[:, 1] = c * U[:, 1] - s * U[:, 2]
        Ur[:, 2] = s * U[:, 1] + c * U[:, 2]
        out.append((spec, rspec, visc, U, Ur, keep, (c, s)))
    return out


def check_rotated(a, b, U, Ur, keep, cs, residual_a, residual_b):
    c, s = cs
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            a.setNumericalMethod(fl, sp)
            b.setNumericalMethod(fl, sp)
            R, Rr = residual_a(U), residual_b(Ur)
            back = Rr.copy()
            back[:, 1] = c * Rr[:, 1] + s * Rr[:, 2]
            back[:, 2] = -s * Rr[:, 1] + c * Rr[:, 2]
            scale = np.abs(R[keep, :4]).max(axis=0)
            assert (np.abs(back[keep, :4] - R[keep, :4]).max(axis=0) <= 1e-12 * scale).all(), (fl, sp)


def test_residual_rotates_with_the_mesh():
    for spec, rspec, visc, U, Ur, keep, cs in rotated_cases():
        a = OracleSolver(spec, bcset="plate", viscous=visc, init="freestream")
        b = OracleSolver(rspec, bcset="plate", viscous=visc, init="freestream")
        for x in (a, b):
            closed_box_setup(x)
        check_rotated(a, b, U, Ur, keep, cs, a.residual, b.residual)
