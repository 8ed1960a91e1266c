"""Explicit (timeStepExplicit) and dual-time (solveUnsteady) stepping on the GPU against
the oracle (itself bit-identical to the compiled reference): the explicit update is
bit-exact (the bump set's inlet pow() aside), the dual-time steps pass through GMRES
reductions summed in another order, so they agree to round-off."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def _pair(api, name, method, **cfg):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"], **cfg)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    for x in (s, o):
        C.setup(x, case)
        x.setNumericalMethod(*method)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=41, amplitude=0.03)
    o.set_state(U)
    s.set_state(U)
    return s, o, case


@pytest.mark.parametrize("name", ["bump", "supersonic", "plate_visc"])
def test_explicit_steps(cuda_lib, name):
    s, o, case = _pair(cuda_lib, name, ("HLLC", "SECOND_ORDER_LIMITED"))
    for _ in range(5):
        rs = s.timeStepExplicit(1e-6)
        ro = o.timeStepExplicit(1e-6)
        assert rs == pytest.approx(ro, rel=1e-12)
    Us, Uo = s.getSolution(), o.get_state()
    if case["bcset"] == "bump":
        assert np.abs(Us - Uo).max() <= 1e-12 * np.abs(Uo).max()
    else:
        np.testing.assert_array_equal(Us, Uo)


@pytest.mark.parametrize("name", ["bump", "plate_visc"])
def test_dual_time_steps(cuda_lib, name):
    s, o, _ = _pair(cuda_lib, name, ("ROE", "SECOND_ORDER_CENTRAL"), jv="fd", krylov=0)
    ts = s.solveUnsteady(1e-4, 3)
    to = o.solveUnsteady(1e-4, 3)
    assert np.abs(ts["newton_steps"] - to["newton_steps"]).max() <= 1
    Us, Uo = s.getSolution(), o.get_state()
    assert np.abs(Us - Uo).max() <= 1e-7 * np.abs(Uo).max()


def test_dual_time_with_mixed_precision_tracks_fp64(cuda_lib):
    """The mixed-precision Krylov solver in the dual-time loop: the inner Newton converges
    to the same physical step as the FP64 path (both to the 1e-6 inner tolerance)."""
    s64, _, _ = _pair(cuda_lib, "plate_visc", ("ROE", "SECOND_ORDER_CENTRAL"), jv="exact")
    smx, _, _ = _pair(cuda_lib, "plate_visc", ("ROE", "SECOND_ORDER_CENTRAL"), precision="mixed", jv="exact")
    a = s64.solveUnsteady(1e-4, 2)
    b = smx.solveUnsteady(1e-4, 2)
    U64, Umx = s64.getSolution(), smx.getSolution()
    assert np.abs(U64 - Umx).max() <= 1e-5 * np.abs(U64).max()
    assert (b["newton_steps"] <= 15).all() and (a["newton_steps"] <= 15).all()
