"""Pinned host buffers: the library reads and writes the caller's page-locked AoS arrays in
place over the CPU-GPU link (row kernels staging whole blocks of rows in shared memory; the
residual's primitive and gather stages take and give the rows themselves), with no staging
copy.  The results must be the same bits as through pageable buffers (the copy-engine
path)."""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg

pytestmark = pytest.mark.gpu


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64).pin_memory().numpy()


@pytest.mark.parametrize("turbulence", ["none", "sst"])
def test_pinned_buffers_match_pageable(cuda_lib, turbulence):
    spec = mg.bump(20_000, seed=4)
    m = cuda_lib.Mesh.from_spec(spec)
    s = cuda_lib.Solver(m, bcset="bump", init="bump", viscous=1, turbulence=turbulence, flux="HLLC",
                        spatial="SECOND_ORDER_LIMITED")
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.setKinematicViscosity(3e6, 1.0)
    s.initialize()
    U = C.perturbed_state(s.getSolution(), m.cells(), seed=5)
    if turbulence == "sst":
        U[:, 4:] = s.getSolution()[:, 4:] * 1.05
    R_pageable = s.computeResiduals(U)
    Uh = _pinned((m.n_cells, 6))
    Rh = _pinned((m.n_cells, 6))
    Uh[:] = U
    Rh[:] = np.nan
    for _ in range(2):
        s.computeResiduals(Uh, out=Rh)
        np.testing.assert_array_equal(Rh, R_pageable)
    s.set_state(Uh)
    Ug = _pinned((m.n_cells, 6))
    Ug[:] = np.nan
    s.getSolution(out=Ug)
    nv = 6 if turbulence == "sst" else 4
    np.testing.assert_array_equal(Ug[:, :nv], U[:, :nv])
    np.testing.assert_array_equal(Ug, s.getSolution())
