"""SST residual (nv = 6) on the GPU against the oracle's SST restatement, the exact
(dual-number) J v of the SST residual against central differences, and a short
mixed-precision solve of a turbulent plate.

The SST terms have no reference counterpart, so their parity is to the oracle's
independent restatement of the model, within round-off (the two order their
floating-point operations differently): 1e-10 of each row's largest entry.
"""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

REL_SST = 1e-10

SST_CASES = {
    "plate": dict(C.CASES["plate_visc"]),
    "bump": dict(C.CASES["bump_visc"]),
    "supersonic": dict(C.CASES["supersonic"], viscous=True, re=(1e5, 1.0)),
}


def _make(api, name, **cfg):
    case = SST_CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=1, init=case["init"], turbulence="sst", **cfg)
    C.setup(s, case)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=True, init=case["init"])
    C.setup(o, case)
    return spec, s, o


def _turbulent_state(o, seed):
    """Perturbed mean flow with k of a few percent turbulence and nu_t of 5-25 nu."""
    U = C.perturbed_state(o.get_state(), o.cells(), seed=seed, amplitude=0.06)
    xc = o.cells()[:, 1:]
    pert = mg.smooth_perturbation(xc, seed + 101, 1.0)
    r = U[:, 0]
    speed = np.sqrt(U[:, 1] ** 2 + U[:, 2] ** 2) / r
    nu = o.params()["nu"]
    k = (0.03 * speed.mean()) ** 2 * (1.0 + 0.5 * pert[:, 0])
    nut = nu * (15.0 + 10.0 * pert[:, 1])
    U[:, 4] = r * k
    U[:, 5] = r * k / nut
    return U


def _rows_match(got, want, what):
    for c in range(6):
        scale = max(np.abs(want[:, c]).max(), 1e-300)
        err = np.abs(got[:, c] - want[:, c]).max()
        assert err <= REL_SST * scale, f"{what} row {c}: rel err {err / scale:.3e}"


@pytest.mark.parametrize("name", list(SST_CASES))
def test_sst_residual_against_oracle(cuda_lib, name):
    spec, s, o = _make(cuda_lib, name)
    U = _turbulent_state(o, seed=5)
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            s.setNumericalMethod(fl, sp)
            o.setNumericalMethod(fl, sp)
            _rows_match(s.computeResiduals(U), o.residual_sst(U), f"{name} {fl} {sp}")


def test_sst_initial_state_is_freestream_k_w(cuda_lib):
    spec, s, o = _make(cuda_lib, "plate")
    k_inf, w_inf = o.sst_freestream()
    U = s.getSolution()
    np.testing.assert_allclose(U[:, 4], U[:, 0] * k_inf, rtol=1e-15)
    np.testing.assert_allclose(U[:, 5], U[:, 0] * w_inf, rtol=1e-15)


@pytest.mark.parametrize("flux", ["ROE", "HLLC"])
def test_sst_exact_jv_matches_central_differences(cuda_lib, flux):
    spec, s, o = _make(cuda_lib, "plate")
    s.setNumericalMethod(flux, "SECOND_ORDER_CENTRAL")
    U = _turbulent_state(o, seed=7)
    n = U.shape[0]
    s.set_dt(np.full(n, 1e300))  # time term vol / dt vanishes
    rng = np.random.default_rng(3)
    v = rng.standard_normal(U.shape) * np.abs(U).mean(axis=0)
    J = s.apply_jacobian(U, None, v, mode="exact")
    h = 1e-6
    Jfd = (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)) / (2 * h)
    for c in range(6):
        err = np.linalg.norm(J[:, c] - Jfd[:, c])
        assert err <= 1e-6 * np.linalg.norm(Jfd[:, c]), f"row {c}: {err / np.linalg.norm(Jfd[:, c]):.3e}"


@pytest.mark.parametrize("name", list(SST_CASES))
@pytest.mark.parametrize("flux", C.FLUXES)
def test_sst_vjp_is_the_transpose_of_exact_jv(cuda_lib, name, flux):
    """<lambda, J v> = <J^T lambda, v> to round-off (no limiter: both differentiate the
    same operation sequence along the same branches)."""
    spec, s, o = _make(cuda_lib, name)
    s.setNumericalMethod(flux, "SECOND_ORDER_CENTRAL")
    U = _turbulent_state(o, seed=9)
    n = U.shape[0]
    s.set_dt(np.full(n, 1e300))
    rng = np.random.default_rng(5)
    scale = np.abs(U).mean(axis=0)
    for trial in range(3):
        v = rng.standard_normal(U.shape) * scale
        lam = rng.standard_normal(U.shape) / scale
        J = s.apply_jacobian(U, None, v, mode="exact")
        gU = s.vjp(lam, U)
        a, b = float(np.sum(lam * J)), float(np.sum(gU * v))
        mag = float(np.sum(np.abs(lam * J)))
        assert abs(a - b) <= 1e-11 * mag, (a, b, mag)


@pytest.mark.parametrize("spatial", C.SPATIALS)
def test_sst_vjp_matches_central_differences(cuda_lib, spatial):
    """lambda^T dR/dU v from the VJP against central differences of lambda^T R along 16
    seeded directions (limited scheme included: the VJP differentiates the limiter)."""
    spec, s, o = _make(cuda_lib, "plate")
    s.setNumericalMethod("ROE", spatial)
    U = _turbulent_state(o, seed=13)
    rng = np.random.default_rng(17)
    scale = np.abs(U).mean(axis=0)
    lam = rng.standard_normal(U.shape) / scale
    gU = s.vjp(lam, U)
    bad = 0
    for d in range(16):
        v = rng.standard_normal(U.shape) * scale
        fd = {}
        for h in (1e-7, 1e-8):
            fd[h] = float(np.sum(lam * (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)))) / (2 * h)
        a = float(np.sum(gU * v))
        err = abs(fd[1e-7] - a) / max(abs(a), 1e-300)
        if err > 1e-6:
            # a limiter or model branch inside the stencil switches: the two steps disagree
            assert abs(fd[1e-7] - fd[1e-8]) > 1e-7 * abs(a), (d, err)
            bad += 1
    assert bad <= 3


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_turbulent_plate_solve_reduces_residual(cuda_lib, precision):
    spec = mg.turb_plate(48, 40)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision=precision,
                        jv="exact", gmres_m=30)
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(5e6, 1.0)
    s.initialize()
    h = s.solveImplicit(tol=1e-8, max_steps=300)
    U = s.getSolution()
    assert np.isfinite(U).all()
    assert (U[:, 4] >= 0).all() and (U[:, 5] > 0).all()
    r = h["res_vm"]
    assert r[-1] <= 1e-4 * r[0], r[-10:]


def test_turbulent_plate_skin_friction_adjoint_vjp(cuda_lib):
    """Skin-friction drag J on a turbulent plate: lambda = dJ/dU drives the SST VJP, checked
    against central differences of lambda^T R along 16 seeded directions; dJ/dU itself
    against central differences of J."""
    spec = mg.turb_plate(40, 24)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst")
    s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(5e6, 1.0)
    s.initialize()
    s.solveImplicit(tol=1e-30, max_steps=40)  # a developing boundary layer, not the free stream
    U = s.getSolution()
    J, lam = s.objective("skin_friction_drag")
    assert J > 0
    rng = np.random.default_rng(23)
    scale = np.abs(U).mean(axis=0)
    gU = s.vjp(lam, U)
    bad = 0
    for d in range(16):
        v = rng.standard_normal(U.shape) * scale
        s.set_state(U + 1e-6 * v)
        jp = s.objective("skin_friction_drag", gradient=False)
        s.set_state(U - 1e-6 * v)
        jm = s.objective("skin_friction_drag", gradient=False)
        assert (jp - jm) / 2e-6 == pytest.approx(float(np.sum(lam * v)), rel=1e-6)
        fd = {h: float(np.sum(lam * (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)))) / (2 * h)
              for h in (1e-7, 1e-8)}
        a = float(np.sum(gU * v))
        if abs(fd[1e-7] - a) > 1e-6 * abs(a):
            assert abs(fd[1e-7] - fd[1e-8]) > 1e-7 * abs(a), (d, fd, a)
            bad += 1
    assert bad <= 3


def _fp32_pair(api, spec, flow, method, sst=True, **cfg):
    m = api.Mesh.from_spec(spec)
    extra = dict(turbulence="sst") if sst else {}
    s = api.Solver(m, bcset="plate", viscous=1, init="freestream", precision="mixed", jv="exact", **extra, **cfg)
    s.setNumericalMethod(*method)
    s.setFreestreamStatic(flow[0], 101325.0, 300.0)
    s.setKinematicViscosity(flow[1], 1.0)
    s.initialize()
    return s


@pytest.mark.parametrize("sst", [False, True])
@pytest.mark.parametrize("spatial", ["FIRST_ORDER", "SECOND_ORDER_CENTRAL", "SECOND_ORDER_LIMITED"])
def test_fp32_residual_and_jv_track_fp64(cuda_lib, sst, spatial):
    s = _fp32_pair(cuda_lib, mg.laminar_plate(24, 16, ratio=1.2), (0.3, 1e4), ("ROE", spatial), sst=sst)
    o = OracleSolver(mg.laminar_plate(24, 16, ratio=1.2), bcset="plate", viscous=True, init="freestream")
    o.setFreestreamStatic(0.3, 101325.0, 300.0)
    o.setKinematicViscosity(1e4, 1.0)
    o.initialize()
    U = _turbulent_state(o, seed=3) if sst else C.perturbed_state(o.get_state(), o.cells(), seed=3)
    nv = 6 if sst else 4
    R64, R32 = s.computeResiduals(U), s.residual32(U)
    for c in range(nv):
        scale = np.abs(R64[:, c]).max()
        assert np.abs(R32[:, c] - R64[:, c]).max() <= 1e-4 * scale, c
    s.set_dt(s.local_timestep(5.0))
    v = np.random.default_rng(2).standard_normal(U.shape) * np.abs(U).mean(axis=0)
    v[:, nv:] = 0
    J64, J32 = s.apply_jacobian(U, None, v, mode="exact"), s.apply_jacobian32(U, v)
    for c in range(nv):
        scale = np.abs(J64[:, c]).max()
        assert np.abs(J32[:, c] - J64[:, c]).max() <= 1e-3 * scale, c


def test_fp32_sst_jv_finite_at_the_omega_floor(cuda_lib):
    """Next to a wall with the first cell at y+ < 1 and w at its floor, arg1^4 of F1
    reaches 1e45: FP32 must stay finite (the blending arguments are capped where tanh is
    already 1), and the mixed-precision Newton step on the full SWBLI grid must too."""
    spec = mg.swbli(80, 64)
    s = _fp32_pair(cuda_lib, spec, (2.0, 1e7), ("HLLC", "FIRST_ORDER"))
    U = s.getSolution()
    U[:, 5] = U[:, 0] * 1.0  # w = 1, below the w_inf * 1e-6 floor of this flow
    s.set_dt(s.local_timestep(0.1))
    v = np.random.default_rng(4).standard_normal(U.shape) * np.abs(U).mean(axis=0)
    J32 = s.apply_jacobian32(U, v)
    J64 = s.apply_jacobian(U, None, v, mode="exact")
    # finiteness is the point here: this state (free stream against a y+ < 1 wall with w
    # at its floor) is far outside where FP32 derivatives keep their relative accuracy
    assert np.isfinite(J32).all() and np.isfinite(J64).all()


def test_swbli_submesh_wall_pressure_adjoint_gradcheck(cuda_lib):
    """The SWBLI recipe on a 1,920-cell sub-mesh (40 x 32, outer half in triangles): M 2,
    Re 1e7, SST, HLLC with the Barth-Jespersen limiter, 8-degree shock inflow.  The wall-
    pressure integral over the interaction region drives the VJP (lambda = dJ/dU), which is
    checked against central differences of lambda^T R along 16 seeded directions (limiter
    switches detected by a second step size), and dJ/dU against differences of J."""
    spec = mg.swbli(40, 32)
    m = cuda_lib.Mesh.from_spec(spec)
    assert m.n_cells == 1920
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst", shock_deflection_deg=8.0)
    s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    s.setFreestreamStatic(2.0, 101325.0, 300.0)
    s.setKinematicViscosity(1e7, 1.0)
    s.initialize()
    s.solveImplicit(tol=1e-30, max_steps=30)
    U = s.getSolution()
    assert np.isfinite(U).all()
    J, lam = s.objective("wall_pressure", 0.3, 0.7)
    assert J > 0 and np.abs(lam).max() > 0
    gU = s.vjp(lam, U)
    rng = np.random.default_rng(31)
    scale = np.abs(U).mean(axis=0)
    bad = 0
    for d in range(16):
        v = rng.standard_normal(U.shape) * scale
        s.set_state(U + 1e-6 * v)
        jp = s.objective("wall_pressure", 0.3, 0.7, gradient=False)
        s.set_state(U - 1e-6 * v)
        jm = s.objective("wall_pressure", 0.3, 0.7, gradient=False)
        assert (jp - jm) / 2e-6 == pytest.approx(float(np.sum(lam * v)), rel=1e-6)
        # limiter and model kinks are everywhere on this grid: steps of 1e-7 of the state
        # cross some of them, 1e-9 rarely does
        fd = {h: float(np.sum(lam * (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)))) / (2 * h)
              for h in (1e-8, 1e-9)}
        a = float(np.sum(gU * v))
        if abs(fd[1e-9] - a) > 1e-6 * abs(a):
            assert abs(fd[1e-8] - fd[1e-9]) > 1e-7 * abs(a), (d, fd, a)
            bad += 1
    assert bad <= 3
