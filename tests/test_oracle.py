"""The CPU oracle (oracle/cfd_oracle.c) pinned against the reference.

* against fixtures produced by the reference's own Solver compiled from its sources
  (tests/golden/ref_cases.npz, ref_bump_full.npz; see tests/golden/make_golden.py)
* against the reference's shipped artefacts: results/residual_history.csv (first 130
  rows at the printed 6 digits, the rows that reproduce across compilers) and
  results/sol_9999.vtk (6-digit Mach, pressure, density)
* against the live reference build (oracle/_ref) when it exists (not on the GPU host)
"""
import gzip
import os

import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver, RefSolver, ref_available, ref_variant

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gold():
    return np.load(os.path.join(GOLD, "ref_cases.npz"))


def _oracle(name, gold):
    case = C.CASES[name]
    o = OracleSolver(C.golden_spec(gold, name), bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    return o


def _full(U4):
    U = np.zeros((U4.shape[0], 6))
    U[:, :4] = U4
    return U


@pytest.mark.parametrize("name", list(C.CASES))
def test_oracle_matches_reference_fixtures(gold, name):
    o = _oracle(name, gold)
    U = _full(gold[f"{name}/U"])
    np.testing.assert_array_equal(o.gradients(U), gold[f"{name}/G"])
    np.testing.assert_array_equal(o.limiters(U), gold[f"{name}/phi"])
    for fl in C.FLUXES:
        for sp in C.SPATIALS:
            o.setNumericalMethod(fl, sp)
            np.testing.assert_array_equal(o.residual(U)[:, :4], gold[f"{name}/{fl}/{sp}/R"], err_msg=f"{fl} {sp}")
    o.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    R = o.residual(U)
    o.set_state(U)
    np.testing.assert_array_equal(o.local_timestep(5.0), gold[f"{name}/dt"])
    np.testing.assert_array_equal(o.preconditioner(), gold[f"{name}/D"])
    v = _full(gold[f"{name}/v"])
    np.testing.assert_array_equal(o.apply_jacobian(U, R, v)[:, :4], gold[f"{name}/Jv"])
    it, x = o.gmres(U, R, -R)
    assert it == int(gold[f"{name}/gmres_iters"])
    np.testing.assert_array_equal(x[:, :4], gold[f"{name}/gmres_x"])


@pytest.mark.parametrize("name", list(C.CASES))
def test_oracle_newton_trace_matches_reference(gold, name):
    from golden.make_golden import TRACE_METHOD  # noqa: E402
    o = _oracle(name, gold)
    o.setNumericalMethod(*TRACE_METHOD[name])
    tr = o.solveImplicit(0.0, 25)
    np.testing.assert_array_equal(tr["res_vm"], gold[f"{name}/trace_res_vm"])
    np.testing.assert_array_equal(tr["cfl"], gold[f"{name}/trace_cfl"])
    np.testing.assert_array_equal(tr["gmres_iters"], gold[f"{name}/trace_iters"])
    np.testing.assert_array_equal(o.get_state()[:, :4], gold[f"{name}/trace_U"])


def bump_mesh(tmp_path_factory=None):
    with gzip.open(os.path.join(GOLD, "bump_1230.msh.gz"), "rb") as fh:
        text = fh.read()
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), f"bump_1230_{os.getpid()}.msh")
    with open(path, "wb") as fh:
        fh.write(text)
    return path


@pytest.fixture(scope="module")
def bump_run():
    path = bump_mesh()
    spec = mg.read_gmsh(path)
    o = OracleSolver(spec, bcset="bump", init="bump")
    o.setFlowConditions(0.5, 101325.0, 300.0)
    o.initialize()
    o.setNumericalMethod("LLF", "FIRST_ORDER")
    tr = o.solveImplicit(1e-5, 2500)
    os.unlink(path)
    return o, tr


def test_oracle_bump_against_shipped_trace(bump_run):
    """results/residual_history.csv: rows 0-129 reproduce exactly at 6 digits; the
    whole run converges near step 623 like the shipped one."""
    o, tr = bump_run
    gold = np.loadtxt(os.path.join(GOLD, "bump_residual_history.csv"), delimiter=",", skiprows=1)
    six = np.array([float("%.6g" % x) for x in tr["res_vm"]])
    np.testing.assert_array_equal(six[:130], gold[:130, 1])
    assert abs(len(tr["res_vm"]) - len(gold)) <= 5
    assert tr["res_vm"][-1] < 1e-5


def test_oracle_bump_against_reference_full_run(bump_run):
    o, tr = bump_run
    g = np.load(os.path.join(GOLD, "ref_bump_full.npz"))
    np.testing.assert_array_equal(tr["res_vm"], g["res_vm"])
    np.testing.assert_array_equal(tr["gmres_iters"], g["gmres_iters"])
    np.testing.assert_array_equal(o.get_state()[:, :4], g["U"])
    assert int(tr["gmres_iters"].sum()) == 12854
    assert abs(o.drag() - (-804.738)) < 1e-3
    assert abs(o.entropy_error() - 0.00291055) < 1e-8


def test_oracle_bump_against_shipped_field(bump_run):
    """results/sol_9999.vtk holds Mach, pressure, density at ~6 significant digits."""
    o, _ = bump_run
    U = o.get_state()
    g = np.load(os.path.join(GOLD, "bump_sol_9999.npz"))
    r = U[:, 0]
    p = 0.4 * (U[:, 3] - 0.5 * (U[:, 1] ** 2 + U[:, 2] ** 2) / r)
    mach = np.sqrt(U[:, 1] ** 2 + U[:, 2] ** 2) / r / np.sqrt(1.4 * p / r)
    for name, val in (("Density", r), ("Pressure", p), ("Mach", mach)):
        np.testing.assert_allclose(val, g[name], rtol=6e-6, err_msg=name)


needs_ref = pytest.mark.skipif(not ref_available("bump"), reason="reference build oracle/_ref absent")


@needs_ref
@pytest.mark.parametrize("name", list(C.CASES))
@pytest.mark.parametrize("flux", C.FLUXES)
def test_oracle_bit_exact_with_live_reference(name, flux):
    case = C.CASES[name]
    spec = case["spec"]()
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    r = RefSolver(spec, ref_variant(case["bcset"], case["viscous"]))
    fi, fd = o.faces()
    ri, rd = r.faces()
    np.testing.assert_array_equal(fi, ri)
    np.testing.assert_array_equal(fd, rd)
    np.testing.assert_array_equal(o.cells(), r.cells())
    for s in (o, r):
        C.setup(s, case)
    assert o.params() == r.params()
    for seed in (1, 2):
        U = C.perturbed_state(o.get_state(), o.cells(), seed=seed, amplitude=0.08)
        for sp in C.SPATIALS:
            o.setNumericalMethod(flux, sp)
            r.setNumericalMethod(flux, sp)
            np.testing.assert_array_equal(o.residual(U), r.residual(U))
            np.testing.assert_array_equal(o.residual(U, False), r.residual(U, False))
        o.set_state(U)
        r.set_state(U)
        np.testing.assert_array_equal(o.local_timestep(7.0), r.local_timestep(7.0))
        R = o.residual(U)
        r.residual(U)
        v = C.random_direction(U.shape[0], seed + 10)
        np.testing.assert_array_equal(o.apply_jacobian(U, R, v), r.apply_jacobian(U, R, v))
        i1, x1 = o.gmres(U, R, -R)
        i2, x2 = r.gmres(U, R, -R)
        assert i1 == i2
        np.testing.assert_array_equal(x1, x2)


@needs_ref
def test_oracle_bit_exact_with_live_reference_larger_mesh():
    spec = mg.bump(6000, seed=4)
    o = OracleSolver(spec, bcset="bump")
    r = RefSolver(spec, "bump")
    for s in (o, r):
        s.setFlowConditions(0.5, 101325.0, 300.0)
        s.initialize()
        s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    tr_o = o.solveImplicit(0.0, 12)
    tr_r = r.solveImplicit(0.0, 12)
    np.testing.assert_array_equal(tr_o["res_vm"], tr_r["res_vm"])
    np.testing.assert_array_equal(o.get_state(), r.get_state())
