"""Exact linearisation, mixed precision and whole Newton solves on the GPU.

* exact J v (dual-number kernels, limiter frozen) against central differences of the
  oracle's FP64 residual, the oracle for a path the reference only approximates by a
  one-sided difference (src/Solver.cpp:1331-1386)
* mixed precision: the FP32-Krylov / FP32-J v GMRES step solves the FP64-exact system
  to its tolerance
* the reference's own bump case (mesh/bump_1230, LLF, first order, tol 1e-5) on the GPU
  against the shipped trace results/residual_history.csv
"""
import gzip
import os

import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _make(api, name, **cfg):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], **cfg)
    C.setup(s, case)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    return case, s, o


def _scaled_direction(U, seed):
    v = C.random_direction(U.shape[0], seed)
    return v * np.abs(U).mean(axis=0)


def central_jv(o, U, v, dt, h=1e-6):
    """(R(U + h v) - R(U - h v)) / 2h + (vol/dt) v with the oracle's limiter frozen."""
    phi = o.get_limiters()
    o.set_limiters(phi)
    Rp = o.residual(U + h * v, False)
    o.set_limiters(phi)
    Rm = o.residual(U - h * v, False)
    vol = o.cells()[:, 0]
    return (Rp - Rm) / (2 * h) + v * (vol / (dt + 1e-30))[:, None]


@pytest.mark.parametrize("name", list(C.CASES))
@pytest.mark.parametrize("flux,spatial", [("LLF", "FIRST_ORDER"), ("ROE", "SECOND_ORDER_CENTRAL"),
                                          ("HLLC", "SECOND_ORDER_LIMITED")])
def test_exact_jv_matches_central_differences(cuda_lib, name, flux, spatial):
    case, s, o = _make(cuda_lib, name)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=6)
    for x in (s, o):
        x.setNumericalMethod(flux, spatial)
    R = o.residual(U)        # sets the oracle's limiter at U
    s.computeResiduals(U)    # and the GPU's
    s.set_state(U)
    o.set_state(U)
    dt = o.local_timestep(10.0)
    s.local_timestep(10.0)
    v = _scaled_direction(U, 9)
    J = s.apply_jacobian(U, None, v, mode="exact")
    Jc = central_jv(o, U, v, dt)
    err = np.linalg.norm(J - Jc) / np.linalg.norm(Jc)
    assert err < 2e-6, err


@pytest.mark.parametrize("name", ["bump", "supersonic", "plate_visc"])
def test_mixed_precision_gmres_solves_exact_system(cuda_lib, name):
    case, s64, o = _make(cuda_lib, name, jv=1)
    _, s32, _ = _make(cuda_lib, name, precision=1)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=7)
    for s in (s64, s32):
        s.setNumericalMethod("ROE", "SECOND_ORDER_LIMITED")
        R = s.computeResiduals(U)
        s.set_state(U)
        s.local_timestep(20.0)
    it32, x32 = s32.gmres(U, R, -R)
    it64, x64 = s64.gmres(U, R, -R)
    # residual of the linear system measured with the FP64 exact operator
    r32 = s64.apply_jacobian(U, None, x32, mode="exact") + R
    r64 = s64.apply_jacobian(U, None, x64, mode="exact") + R
    nR = np.linalg.norm(R)
    assert np.linalg.norm(r64) <= 1.05e-2 * nR
    assert np.linalg.norm(r32) <= 2e-2 * nR
    assert abs(it32 - it64) <= 2


def _bump_mesh(api, tmp_path):
    p = tmp_path / "bump_1230.msh"
    with gzip.open(os.path.join(GOLD, "bump_1230.msh.gz"), "rb") as fh:
        p.write_bytes(fh.read())
    return api.Mesh.load(str(p))


def test_bump_case_against_shipped_trace(cuda_lib, tmp_path):
    """The reference's default case end to end on the GPU (FP64, FD J v)."""
    m = _bump_mesh(cuda_lib, tmp_path)
    s = cuda_lib.Solver(m, bcset="bump", init="bump")
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.initialize()
    s.setNumericalMethod("LLF", "FIRST_ORDER")
    tr = s.solveImplicit(1e-5, 2500)
    gold = np.loadtxt(os.path.join(GOLD, "bump_residual_history.csv"), delimiter=",", skiprows=1)
    six = np.array([float("%.6g" % x) for x in tr["res_vm"]])
    same = six[:130] == gold[:130, 1]
    assert same[:60].all(), np.nonzero(~same)[0][:5]
    assert tr["converged"] and tr["res_vm"][-1] < 1e-5
    assert abs(len(tr["res_vm"]) - len(gold)) <= 25
    g = np.load(os.path.join(GOLD, "ref_bump_full.npz"))
    U = s.getSolution()[:, :4]
    assert np.abs(U - g["U"]).max() <= 1e-6 * np.abs(g["U"]).max()


def test_nasa_laminar_plate_against_shipped_skin_friction(cuda_lib, tmp_path):
    """The reference's NASA laminar flat plate end to end on the GPU with its settings (the
    plate case of src/main.cpp: mesh/new_laminar_flat_plate, 6,962 quads; HLLC, second-order
    central, M 0.1, Re 2e5 on 0.3048 m; the reference's pseudo-transient control to
    res_vm < 1e-4) through the mixed-precision driver: the wall Cf against the reference's
    shipped profile (results/data/cf_profile.csv), and downstream of x = 0.2 against
    Blasius 0.664 / sqrt(Re_x), which the shipped profile itself exceeds by 4-12 % there.
    The shipped profile was written by an earlier build of the reference: its current
    sources, compiled, stop after 39,807 steps, 0.77 % from it at most, with the CPU oracle's
    state bit for bit (tests/golden/plate_nasa_ref.npz, the Cf of that run); hence 2 %
    against the shipped profile and a tighter bound against the current reference's Cf."""
    p = tmp_path / "plate_nasa.msh"
    with gzip.open(os.path.join(GOLD, "plate_nasa.msh.gz"), "rb") as fh:
        p.write_bytes(fh.read())
    m = cuda_lib.Mesh.load(str(p))
    s = cuda_lib.Solver(m, bcset="plate", viscous=1, init="freestream", precision=1)
    s.setNumericalMethod("HLLC", "SECOND_ORDER_CENTRAL")
    s.setFlowConditions(0.1, 41368.5, 388.89)
    s.setKinematicViscosity(200000.0, 0.3048)
    s.initialize()
    tr = s.solveImplicit(1e-4, 50000)
    assert tr["converged"]
    x, cp, cf = s.wall_coefficients(4)
    gold = np.loadtxt(os.path.join(GOLD, "plate_cf_profile.csv"), delimiter=",", skiprows=1)
    o = np.argsort(x, kind="stable")
    x, cf = x[o], cf[o]
    np.testing.assert_allclose(x, gold[:, 0], rtol=5e-6)
    rel = np.abs(cf - gold[:, 1]) / np.abs(gold[:, 1])
    keep = x > 0.2
    blas = np.abs(cf[keep] / gold[keep, 2] - 1.0)
    ref = np.load(os.path.join(GOLD, "plate_nasa_ref.npz"))
    np.testing.assert_allclose(x, ref["x"], rtol=1e-12)
    rel_ref = np.abs(cf - ref["cf"]) / np.abs(ref["cf"])
    print(f"NASA plate: {len(tr['res_vm'])} Newton steps (reference {int(ref['steps'])}), Cf vs the reference's run "
          f"max rel {rel_ref.max():.3e}, vs shipped profile {rel.max():.3e}, vs Blasius (x > 0.2) {blas.max():.3f}")
    assert abs(len(tr["res_vm"]) - int(ref["steps"])) <= 50
    assert rel_ref.max() <= 1e-8  # 8.1e-10 measured (mixed driver; a deterministic solve)
    assert rel.max() <= 2e-2
    assert blas.max() <= 0.16


def test_bump_case_mixed_precision_exact_jv(cuda_lib, tmp_path):
    m = _bump_mesh(cuda_lib, tmp_path)
    s = cuda_lib.Solver(m, bcset="bump", init="bump", precision=1)
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.initialize()
    s.setNumericalMethod("LLF", "FIRST_ORDER")
    tr = s.solveImplicit(1e-5, 2500)
    assert tr["converged"]
    g = np.load(os.path.join(GOLD, "ref_bump_full.npz"))
    U = s.getSolution()[:, :4]
    assert np.abs(U - g["U"]).max() <= 1e-6 * np.abs(g["U"]).max()
