"""Adjoint VJP of the full residual (gradients and limiter recomputed and differentiated
along the forward branches) against central differences of the CPU oracle's FP64
residual (oracle/cfd_oracle.c, the reference's computeResiduals with the limiter updated)
in 16 seeded random directions:  <gU, d>  vs  lambda . (R(U + h d) - R(U - h d)) / 2h,
to 1e-6 relative.  The reference has no adjoint; this is the oracle the build plan names.
The limiter's min/max selections and the HLLC wave regions are not differentiable at
their switch points; a direction whose difference quotient changes between h = 1e-7 and
h = 1e-8 by more than 1e-6 crosses one within the step and is reported as
branch-switched instead of compared (at most 3 of 16 allowed).

Also: a torch.autograd.Function over cfdg_residual / cfdg_vjp (used only by this test
harness), checked with torch.autograd.gradcheck."""
import numpy as np
import pytest

import cases as C
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

REL = 1e-6


def _make(api, name):
    case = C.CASES[name]
    spec = case["spec"]()
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset=case["bcset"], viscous=int(case["viscous"]), init=case["init"])
    C.setup(s, case)
    o = OracleSolver(spec, bcset=case["bcset"], viscous=case["viscous"], init=case["init"])
    C.setup(o, case)
    return case, s, o


def _fd_dir(o, U, d, lam, h):
    def f(t):
        return float(np.sum(lam * o.residual(U + t * d, True)))
    d1 = (f(h) - f(-h)) / (2 * h)
    d2 = (f(h / 2) - f(-h / 2)) / h
    return (4 * d2 - d1) / 3


@pytest.mark.parametrize("name", list(C.CASES))
@pytest.mark.parametrize("flux,spatial", [("LLF", "FIRST_ORDER"), ("ROE", "SECOND_ORDER_CENTRAL"),
                                          ("HLLC", "SECOND_ORDER_LIMITED")])
def test_vjp_matches_central_differences(cuda_lib, name, flux, spatial):
    case, s, o = _make(cuda_lib, name)
    for x in (s, o):
        x.setNumericalMethod(flux, spatial)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=21, amplitude=0.06)
    rng = np.random.default_rng(5)
    scale = np.abs(U).mean(axis=0)
    lam = rng.standard_normal(U.shape)
    lam[:, 4:] = 0
    gU = s.vjp(lam, U)
    assert np.isfinite(gU).all()
    bad, switched = [], []
    for k in range(16):
        d = rng.standard_normal(U.shape) * scale
        d[:, 4:] = 0
        fd = _fd_dir(o, U, d, lam, 1e-7)
        fd_small = _fd_dir(o, U, d, lam, 1e-8)
        ad = float(np.sum(gU * d))
        if abs(fd - fd_small) > 1e-6 * abs(fd):
            switched.append(k)
            continue
        if abs(ad - fd) > REL * max(abs(fd), abs(ad)):
            bad.append((k, ad, fd))
    print(f"{name} {flux} {spatial}: branch-switched directions {switched}")
    assert len(switched) <= 3, switched
    assert not bad, bad


def test_vjp_leaves_the_frozen_limiter_alone(cuda_lib):
    case, s, o = _make(cuda_lib, "supersonic")
    s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    U = C.perturbed_state(o.get_state(), o.cells(), seed=3)
    s.computeResiduals(U)
    phi0 = s.get_limiters()
    s.vjp(np.ones_like(U), C.perturbed_state(o.get_state(), o.cells(), seed=4))
    np.testing.assert_array_equal(s.get_limiters(), phi0)


def test_torch_autograd_shim_gradcheck(cuda_lib):
    torch = pytest.importorskip("torch")
    case, s, o = _make(cuda_lib, "plate_visc")
    s.setNumericalMethod("ROE", "SECOND_ORDER_LIMITED")
    U0 = C.perturbed_state(o.get_state(), o.cells(), seed=9, amplitude=0.05)
    U0t = torch.tensor(U0)

    class Residual(torch.autograd.Function):
        """R(U) through cfdg_residual; backward through cfdg_vjp."""

        @staticmethod
        def forward(ctx, U):
            ctx.save_for_backward(U)
            return torch.from_numpy(s.computeResiduals(U.detach().numpy(), True))

        @staticmethod
        def backward(ctx, gR):
            (U,) = ctx.saved_tensors
            return torch.from_numpy(s.vjp(gR.detach().numpy(), U.detach().numpy()))

    # relative perturbation variables on 4 conservative components, scaled to O(1)
    x = torch.zeros(U0.shape[0], 4, dtype=torch.float64, requires_grad=True)

    def f(x):
        U = U0t.clone()
        U[:, :4] = U0t[:, :4] * (1 + 1e-3 * x)
        return Residual.apply(U)[:, :4] / 1e3

    assert torch.autograd.gradcheck(f, (x,), eps=1e-4, atol=1e-6, rtol=1e-5, fast_mode=True)
