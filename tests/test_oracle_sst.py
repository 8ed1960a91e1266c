"""The oracle's SST residual (parity unpinned: the reference has no SST terms).

What can be pinned is pinned: with k = 0 in every cell the eddy viscosity vanishes,
so the mean-flow rows of the SST residual must equal the oracle's laminar viscous
residual, which is itself pinned bit for bit to the compiled reference.  The k and w
rows are checked for the structure of the model: a uniform free stream with the
free-stream k and w has zero k and w fluxes, so those rows are the sources alone.
"""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver


def _plate(n=(12, 8)):
    from mycode_gb300 import meshgen as mg

    spec = mg.laminar_plate(*n, ratio=1.2)
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    C.setup(o, C.CASES["plate_visc"])
    return spec, o


@pytest.mark.parametrize("flux", C.FLUXES)
@pytest.mark.parametrize("spatial", ["FIRST_ORDER", "SECOND_ORDER_CENTRAL"])
def test_sst_mean_flow_reduces_to_laminar_at_zero_k(flux, spatial):
    spec, o = _plate()
    o.setNumericalMethod(flux, spatial)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=11, amplitude=0.08)
    U[:, 4] = 0.0
    U[:, 5] = U[:, 0] * 50.0
    R_lam = o.residual(U)[:, :4]
    R_sst = o.residual_sst(U)[:, :4]
    scale = np.abs(R_lam).max(axis=0)
    err = np.abs(R_sst - R_lam).max(axis=0)
    assert np.all(err <= 1e-12 * scale), err / scale


def test_sst_uniform_freestream_rows_are_sources():
    spec, o = _plate()
    o.setNumericalMethod("ROE", "SECOND_ORDER_CENTRAL")
    k_inf, w_inf = o.sst_freestream()
    assert k_inf > 0 and w_inf > 0
    U = o.get_state().copy()
    U[:, 4] = U[:, 0] * k_inf
    U[:, 5] = U[:, 0] * w_inf
    R = o.residual_sst(U)
    vol = o.cells()[:, 0]
    # away from the no-slip wall the gradients of the uniform state vanish: S = 0, so
    # mu_t = rho k / w, P = 0, and the sources are the destruction terms only
    r = U[:, 0]
    far = R[:, 4] != 0.0
    assert far.any()
    Sk = -0.09 * r * w_inf * k_inf
    # cells whose faces all see the uniform state: residual k row = -S_k vol
    ok = np.isclose(R[:, 4], -Sk * vol, rtol=1e-9, atol=0)
    assert ok.mean() > 0.3
    # the destruction of w is bounded by the two model constants
    lo = 0.075 * r * w_inf * w_inf * vol
    hi = 0.0828 * r * w_inf * w_inf * vol
    sel = ok
    assert np.all(R[sel, 5] >= lo[sel] * (1 - 1e-9)) and np.all(R[sel, 5] <= hi[sel] * (1 + 1e-9))


def test_sst_freestream_values():
    spec, o = _plate()
    p = o.params()
    g, Rg = 1.4, p["R_gas"]
    fT = 1.0 + 0.5 * (g - 1.0) * p["M_inf"] ** 2
    U = p["M_inf"] * np.sqrt(g * Rg * p["T0"] / fT)
    k, w = o.sst_freestream(0.001, 0.01)
    assert k == pytest.approx(1.5 * (0.001 * U) ** 2, rel=1e-14)
    assert w == pytest.approx(k / (0.01 * p["nu"]), rel=1e-14)
