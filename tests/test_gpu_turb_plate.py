"""The turbulent flat plate at full size (480 x 240 quads, 115,200 cells, first cell at
y+ < 1, stretching 1.12): SST, Roe, second-order central, mixed-precision JFNK from the
free stream under the reference's pseudo-transient control (src/Solver.cpp:1696-1799).
The volume-weighted residual falls six orders; at that state the skin-friction drag's
dJ/dU drives the adjoint (VJP), checked against central differences of lambda^T R along
16 seeded directions, and dJ/dU itself against central differences of J (no reference
counterpart: the reference has no SST and no adjoint)."""
import numpy as np
import pytest

from mycode_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def test_turbulent_plate_full_size_converges_and_skin_friction_vjp_matches_fd(cuda_lib):
    spec = mg.turb_plate()
    m = cuda_lib.Mesh.from_spec(spec, gpu=0)
    assert m.n_cells == 115_200
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", turbulence="sst", precision="mixed",
                        jv="exact", flux="ROE", spatial="SECOND_ORDER_CENTRAL")
    s.setFreestreamStatic(0.2, 101325.0, 300.0)
    s.setKinematicViscosity(5e6, 1.0)
    s.initialize()
    s.reset_newton()
    recs = []
    while len(recs) < 8000:
        r, _ = s.newton_steps(64)
        recs += r
        if recs[-1].res_vm <= 1e-6 * recs[0].res_vm:
            break
    orders = np.log10(recs[0].res_vm / recs[-1].res_vm)
    print(f"turbulent plate: {len(recs)} Newton steps, res_vm {recs[0].res_vm:.3e} -> {recs[-1].res_vm:.3e} "
          f"({orders:.2f} orders)")
    assert orders >= 6.0, (len(recs), recs[-1].res_vm)
    U = s.getSolution()
    assert np.isfinite(U).all() and (U[:, 4] >= 0).all() and (U[:, 5] > 0).all()
    J, lam = s.objective("skin_friction_drag")
    assert J > 0
    gU = s.vjp(lam, U)
    rng = np.random.default_rng(29)
    scale = np.abs(U).mean(axis=0)
    bad, worst = 0, 0.0
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
        err = abs(fd[1e-7] - a) / abs(a)
        if err > 1e-6:
            # a branch (min / max / clip) switched inside the step: the two step sizes disagree
            assert abs(fd[1e-7] - fd[1e-8]) > 1e-7 * abs(a), (d, fd, a)
            bad += 1
        else:
            worst = max(worst, err)
    print(f"skin-friction drag J = {J:.6e}; VJP vs central differences: worst {worst:.2e} over "
          f"{16 - bad} directions, {bad} with a branch switch")
    assert bad <= 3
