"""The shock/boundary-layer interaction (M 2, Re 1e7 per unit length, 8-degree shock inflow,
SST, HLLC with the Barth-Jespersen limiter, mixed-precision JFNK under the reference's
pseudo-transient control, src/Solver.cpp:1696-1799).

At full size (800 x 640 rows, the outer half split: 768,000 cells) the wall-pressure
integral over the interaction region drives the VJP, checked against central differences
of lambda^T R along 16 seeded directions, and dJ/dU against differences of J: at the state
of 24 Newton steps from the free stream (a developing boundary layer and shock), and at the
converged state.  The full mesh converges six orders of the volume-weighted residual from
the free stream under the reference's pseudo-transient control with a continuation
schedule for the CFL cap: 1.5 through the start-up transient (the first 16,384 steps; with
a cap of 2.5 or more the transient goes non-finite with the reference's scalar diagonal
preconditioner, and at 2 it survives or not depending on the FP32 Krylov solutions'
last bits), then 10 (cfdg_set_cfl_max).  The 200 x 160 mesh converges six orders
with the reference's cap.  (No reference counterpart: the reference has no SST and no adjoint.)"""
import numpy as np
import pytest

from mycode_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _solver(api, spec, **extra):
    m = api.Mesh.from_spec(spec, gpu=0)
    s = api.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision="mixed", jv="exact",
                   flux="HLLC", spatial="SECOND_ORDER_LIMITED", shock_deflection_deg=8.0, **extra)
    s.setFreestreamStatic(2.0, 101325.0, 300.0)
    s.setKinematicViscosity(1e7, 1.0)
    s.initialize()
    s.reset_newton()
    return m, s


def _wall_pressure_vjp_check(s, U, label):
    """lambda = dJ/dU of the wall-pressure integral over x in [0.3, 0.7] and the VJP
    lambda^T dR/dU at U, against central differences along 16 seeded directions; returns
    the directions that crossed a branch (limiter and model kinks: a step of 1e-8 of the
    state crosses some, 1e-9 rarely)."""
    J, lam = s.objective("wall_pressure", 0.3, 0.7)
    assert J > 0 and np.abs(lam).max() > 0
    gU = s.vjp(lam, U)
    rng = np.random.default_rng(37)
    scale = np.abs(U).mean(axis=0)
    bad, worst = 0, 0.0
    for d in range(16):
        v = rng.standard_normal(U.shape) * scale
        s.set_state(U + 1e-6 * v)
        jp = s.objective("wall_pressure", 0.3, 0.7, gradient=False)
        s.set_state(U - 1e-6 * v)
        jm = s.objective("wall_pressure", 0.3, 0.7, gradient=False)
        assert (jp - jm) / 2e-6 == pytest.approx(float(np.sum(lam * v)), rel=1e-6)
        fd = {h: float(np.sum(lam * (s.computeResiduals(U + h * v) - s.computeResiduals(U - h * v)))) / (2 * h)
              for h in (1e-8, 1e-9)}
        a = float(np.sum(gU * v))
        err = abs(fd[1e-9] - a) / abs(a)
        if err > 1e-6:
            assert abs(fd[1e-8] - fd[1e-9]) > 1e-7 * abs(a), (d, fd, a)
            bad += 1
        else:
            worst = max(worst, err)
    s.set_state(U)
    print(f"{label}: wall-pressure J = {J:.6e}; VJP vs central differences: worst {worst:.2e} over "
          f"{16 - bad} directions, {bad} with a branch switch")
    return bad


def test_swbli_full_size_wall_pressure_vjp_matches_fd(cuda_lib):
    m, s = _solver(cuda_lib, mg.swbli())
    assert m.n_cells == 768_000
    recs, _ = s.newton_steps(24)
    assert len(recs) == 24 and recs[-1].res_vm < 0.1 * recs[0].res_vm
    U = s.getSolution()
    assert np.isfinite(U).all() and (U[:, 4] >= 0).all() and (U[:, 5] > 0).all()
    assert _wall_pressure_vjp_check(s, U, "SWBLI 768,000 cells, 24 steps") <= 3


def test_swbli_200x160_converges_six_orders(cuda_lib):
    m, s = _solver(cuda_lib, mg.swbli(200, 160))
    assert m.n_cells == 48_000
    recs = []
    while len(recs) < 14_000:
        r, _ = s.newton_steps(64)
        recs += r
        if recs[-1].res_vm <= 1e-6 * recs[0].res_vm:
            break
    orders = np.log10(recs[0].res_vm / recs[-1].res_vm)
    print(f"SWBLI 48,000 cells: {len(recs)} Newton steps, res_vm {recs[0].res_vm:.3e} -> {recs[-1].res_vm:.3e} "
          f"({orders:.2f} orders), res_rho {recs[0].res_rho:.3e} -> {recs[-1].res_rho:.3e}")
    assert orders >= 6.0
    U = s.getSolution()
    assert np.isfinite(U).all()


def test_swbli_full_size_converges_six_orders_then_wall_pressure_vjp(cuda_lib):
    m, s = _solver(cuda_lib, mg.swbli(), cfl_max=1.5)
    assert m.n_cells == 768_000
    recs = []
    while len(recs) < 40_000:
        if len(recs) == 16_384:
            s.set_cfl_max(10.0)  # the start-up transient is over: the CFL may grow again
        r, _ = s.newton_steps(64)
        recs += r
        if recs[-1].res_vm <= 1e-6 * recs[0].res_vm:
            break
    orders = np.log10(recs[0].res_vm / recs[-1].res_vm)
    print(f"SWBLI 768,000 cells, CFL cap 1.5 then 10: {len(recs)} Newton steps, res_vm {recs[0].res_vm:.3e} -> "
          f"{recs[-1].res_vm:.3e} ({orders:.2f} orders), res_rho {recs[0].res_rho:.3e} -> {recs[-1].res_rho:.3e}")
    assert orders >= 6.0
    U = s.getSolution()
    assert np.isfinite(U).all() and (U[:, 4] >= 0).all() and (U[:, 5] > 0).all()
    assert _wall_pressure_vjp_check(s, U, "SWBLI 768,000 cells, converged") <= 3
