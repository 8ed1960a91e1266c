"""The device-resident GMRES (one CUDA graph per solve: WHILE node, device Givens,
CGS2) against the host-driven modified Gram-Schmidt loop of the reference
(src/Solver.cpp:1472-1618): both must solve (vol/dt + dR/dU) x = -R to the GMRES
tolerance, the empty solve must return zero iterations, and with tolerance 0 the loop
must stop after exactly m iterations."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def _solver(api, name, **cfg):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], **cfg)
    C.setup(s, case)
    return s, spec, case


def _linear_residual(s_exact, U, R, x):
    r = s_exact.apply_jacobian(U, None, x, mode="exact") + R
    return np.linalg.norm(r) / np.linalg.norm(R)


@pytest.mark.parametrize("name", ["bump", "supersonic", "plate_visc"])
@pytest.mark.parametrize("precision,jv", [("fp64", "exact"), ("mixed", "exact"), ("fp64", "fd")])
def test_graph_gmres_solves_system(cuda_lib, name, precision, jv):
    s_ref, spec, case = _solver(cuda_lib, name, jv="exact", krylov=0)       # host MGS, exact J v
    s_g, _, _ = _solver(cuda_lib, name, precision=precision, jv=jv, krylov=1)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=12)
    for s in (s_ref, s_g):
        s.setNumericalMethod("ROE", "SECOND_ORDER_LIMITED")
        R = s.computeResiduals(U)
        s.set_state(U)
        s.local_timestep(50.0)
    it_h, x_h = s_ref.gmres(U, R, -R)
    it_g, x_g = s_g.gmres(U, R, -R)
    tol = 1.05e-2 if precision == "fp64" and jv == "exact" else 3e-2
    assert _linear_residual(s_ref, U, R, x_h) <= 1.05e-2
    assert _linear_residual(s_ref, U, R, x_g) <= tol
    assert abs(it_g - it_h) <= 2


def test_graph_gmres_runs_exactly_m_iterations_at_zero_tolerance(cuda_lib):
    s, spec, case = _solver(cuda_lib, "supersonic", precision="mixed", gmres_m=7, gmres_tol=0.0)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=13)
    R = s.computeResiduals(U)
    s.set_state(U)
    s.local_timestep(5.0)
    for _ in range(2):  # the second launch reuses the instantiated graph
        it, x = s.gmres(U, R, -R)
        assert it == 7
        assert np.isfinite(x).all()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_gmres_long_basis(cuda_lib, precision):
    """m = 80 at tolerance 0: 80 iterations (the back substitution's triangle then exceeds
    its shared-memory stage and is read from global memory); the solution still solves
    the system better than the 40-iteration one."""
    s, spec, case = _solver(cuda_lib, "supersonic", precision=precision, jv="exact", gmres_m=80, gmres_tol=0.0)
    s_ref, _, _ = _solver(cuda_lib, "supersonic", jv="exact", krylov=0)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=17)
    for t in (s, s_ref):
        t.setNumericalMethod("ROE", "SECOND_ORDER_LIMITED")
        R = t.computeResiduals(U)
        t.set_state(U)
        t.local_timestep(50.0)
    it, x = s.gmres(U, R, -R)
    assert it == 80
    assert np.isfinite(x).all()
    assert _linear_residual(s_ref, U, R, x) <= (1e-3 if precision == "fp64" else 1e-2)


def test_graph_gmres_empty_solve(cuda_lib):
    s, spec, case = _solver(cuda_lib, "bump", precision="mixed")
    U = s.getSolution()
    s.local_timestep(1.0)
    it, x = s.gmres(U, np.zeros_like(U), np.zeros_like(U))
    assert it == 0
    assert not x.any()


def test_graph_newton_solve_matches_host_driver(cuda_lib):
    """A mixed-precision solve with the graph driver follows the host-driven one."""
    out = {}
    for kry in (0, 1):
        s, _, _ = _solver(cuda_lib, "supersonic", precision="mixed", krylov=kry)
        s.setNumericalMethod("HLLC", "FIRST_ORDER")
        tr = s.solveImplicit(0.0, 20)
        out[kry] = tr
    a, b = out[0]["res_vm"], out[1]["res_vm"]
    np.testing.assert_allclose(b, a, rtol=1e-3)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_newton_step_norm_and_update(cuda_lib, precision):
    """One graph Newton step: the norm that its fused reduction kernel takes of R (with
    |R|^2 and rhs = -R in the same pass) is the volume-weighted norm of R bit for bit, and
    its update (the mixed path's time step and preconditioner computed in FP32 inside the
    graph) follows the host-driven step to the GMRES tolerance."""
    out = {}
    for kry in (0, 1):
        s, spec, case = _solver(cuda_lib, "supersonic", precision=precision, jv="exact", krylov=kry)
        o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
        C.setup(o, case)
        U = C.perturbed_state(o.get_state(), o.cells(), seed=16)
        s.setNumericalMethod("ROE", "SECOND_ORDER_LIMITED")
        s.set_state(U)
        ref = s.norm_vm(s.computeResiduals(U))
        s.set_state(U)
        rec, _ = s.newton_step(0.0)
        assert rec.res_vm == ref
        out[kry] = s.getSolution() - U
    d0, d1 = out[0], out[1]
    assert np.linalg.norm(d1 - d0) <= 5e-2 * np.linalg.norm(d0)


@pytest.mark.parametrize("name", ["supersonic", "plate_visc"])
@pytest.mark.parametrize("precision,jv", [("mixed", "exact"), ("fp64", "exact"), ("fp64", "fd")])
def test_stream_driver_is_the_graph_bit_for_bit(cuda_lib, name, precision, jv):
    """The stream driver launches the graph's kernels one iteration at a time: the same
    arithmetic in the same order, so the same solution bit for bit, and with timing on
    every stage of the fused body is timed."""
    out = {}
    for kry in (1, 2):
        s, spec, case = _solver(cuda_lib, name, precision=precision, jv=jv, krylov=kry, gmres_m=12, persistent=0)
        o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
        C.setup(o, case)
        U = C.perturbed_state(o.get_state(), o.cells(), seed=14)
        s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
        R = s.computeResiduals(U)
        s.set_state(U)
        s.local_timestep(20.0)
        s.set_timing(True)
        s.kernel_stats(reset=True)
        out[kry] = s.gmres(U, R, -R)
        st = s.kernel_stats(reset=True)
        if kry == 2 and (precision == "mixed" or jv == "exact"):
            # the exact J v body (delayed CGS2) finishes column j after the product of
            # iteration j + 1 and runs its Givens step in the first kernel of iteration
            # j + 2, so the body runs twice more than the iterations (in the last run the
            # first kernel ends the solve and the others return at once)
            k = out[kry][0]
            for cls in ("krylov.prim_z", "krylov.grad", "krylov.flux", "krylov.gather_dot"):
                assert st[cls][1] == k + 2
            assert st["krylov.update_dot"][1] == st["krylov.update_final"][1] == 0
    assert out[1][0] == out[2][0]
    np.testing.assert_array_equal(out[1][1], out[2][1])


@pytest.mark.parametrize("name", ["supersonic", "plate_visc", "bump_visc"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_persistent_arnoldi_kernel_matches_the_four_kernel_body(cuda_lib, name, precision):
    """One persistent kernel per Arnoldi iteration (grid barriers between the phases)
    (two-reduction CGS2) against the four-kernel body (delayed one-reduction CGS2): the
    same Krylov space and Hessenberg matrix in exact arithmetic, with norms by Pythagoras
    here and reductions partitioned over a different number of blocks, so the same
    iterations and the same solution to the basis precision."""
    out = {}
    for pers in (0, 1):
        s, spec, case = _solver(cuda_lib, name, precision=precision, jv="exact", krylov=1, gmres_m=20, persistent=pers)
        o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
        C.setup(o, case)
        U = C.perturbed_state(o.get_state(), o.cells(), seed=15)
        s.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
        R = s.computeResiduals(U)
        s.set_state(U)
        s.local_timestep(20.0)
        out[pers] = s.gmres(U, R, -R)
    assert abs(out[0][0] - out[1][0]) <= 1
    x0, x1 = out[0][1], out[1][1]
    tol = 1e-4 if precision == "mixed" else 1e-10
    if out[0][0] == out[1][0]:
        assert np.linalg.norm(x1 - x0) <= tol * np.linalg.norm(x0)


def test_persistent_arnoldi_newton_solve(cuda_lib):
    """Newton steps with the persistent kernel follow the four-kernel driver."""
    tr = {}
    for pers in (0, 1):
        s, _, _ = _solver(cuda_lib, "supersonic", precision="mixed", krylov=1, persistent=pers)
        s.setNumericalMethod("HLLC", "FIRST_ORDER")
        tr[pers] = s.solveImplicit(0.0, 15)
    np.testing.assert_allclose(tr[1]["res_vm"], tr[0]["res_vm"], rtol=1e-4)


@pytest.mark.parametrize("name", ["supersonic", "plate_visc"])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_split_gather_is_the_fused_kernel_bit_for_bit(cuda_lib, name, precision):
    """The exact J v body's gather and dots as two kernels (k_gmres_gather_w, then the dots
    alone: large meshes, forced here with gather_split_cells = 1) against the fused kernel
    (gather_split_cells = -1): the same arithmetic and the same block partials, so the same
    GMRES solve and the same Newton steps bit for bit, through the graph and the stream
    drivers."""
    for kry in (1, 2):
        out = {}
        for split in (-1, 1):
            s, spec, case = _solver(cuda_lib, name, precision=precision, jv="exact", krylov=kry, gmres_m=12,
                                    gather_split_cells=split)
            o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
            C.setup(o, case)
            U = C.perturbed_state(o.get_state(), o.cells(), seed=21)
            s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
            R = s.computeResiduals(U)
            s.set_state(U)
            s.local_timestep(20.0)
            its, x = s.gmres(U, R, -R)
            s.set_state(U)
            recs = [s.newton_step(0.0)[0] for _ in range(4)]
            out[split] = (its, x, [(r.res_vm, r.gmres_iters) for r in recs], s.getSolution())
        a, b = out[-1], out[1]
        assert a[0] == b[0] and a[2] == b[2], (kry, a[0], b[0], a[2], b[2])
        np.testing.assert_array_equal(a[1], b[1])
        np.testing.assert_array_equal(a[3], b[3])
