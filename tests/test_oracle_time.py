"""The oracle's explicit (timeStepExplicit) and dual-time (solveUnsteady) stepping
against the compiled reference, bit for bit."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver, RefSolver, ref_available, ref_variant

needs_ref = pytest.mark.skipif(not ref_available("bump"), reason="reference build oracle/_ref absent")


def _pair(name, method):
    case = C.CASES[name]
    spec = case["spec"]()
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    r = RefSolver(spec, variant=ref_variant(case["bcset"], case["viscous"]))
    for x in (o, r):
        C.setup(x, case)
        x.setNumericalMethod(*method)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=41, amplitude=0.03)
    o.set_state(U)
    r.set_state(U)
    return o, r


@needs_ref
@pytest.mark.parametrize("name", ["bump", "supersonic", "plate_visc"])
def test_explicit_steps_bit_exact(name):
    o, r = _pair(name, ("HLLC", "SECOND_ORDER_LIMITED"))
    for _ in range(5):
        o.timeStepExplicit(1e-6)
        r.timeStepExplicit(1e-6)
    np.testing.assert_array_equal(o.get_state(), r.get_state())


@needs_ref
@pytest.mark.parametrize("name", ["bump", "plate_visc"])
def test_dual_time_steps_bit_exact(name):
    o, r = _pair(name, ("ROE", "SECOND_ORDER_CENTRAL"))
    out = o.solveUnsteady(1e-4, 2)
    r.solveUnsteady(1e-4, 2)
    np.testing.assert_array_equal(o.get_state(), r.get_state())
    assert (out["newton_steps"] >= 1).all()
