"""cfdg_norm_vm_noalloc: the residual norm for callers that cannot allocate device
memory (an application whose GPU memory belongs to its own pool, or a latency-bound
caller that cannot afford cudaMalloc's synchronisation).  It must give the same norm as
cfdg_norm_vm, the entry point it is a variant of, and as the CPU oracle's
norm_L2_VolumeWeighted (src/Solver.cpp:1280-1303), on two calls in a row (the second
call reuses the static scratch the first one left behind), for the four-variable and the
six-variable (SST) state, and refuse sizes beyond its static scratch.  This file is
collected last so that a run stopping at the first failure has run everything else
first; it also passes alone in a fresh process."""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

REL = 1e-12  # the FP64 bar of the parity tests


@pytest.mark.parametrize("turbulence", ["none", "sst"])
def test_norm_vm_noalloc_matches_norm_vm_and_oracle_twice(cuda_lib, turbulence):
    import torch
    api = cuda_lib
    spec = mg.bump(30_000, seed=5)
    m = api.Mesh.from_spec(spec)
    s = api.Solver(m, bcset="bump", init="bump", viscous=1, turbulence=turbulence)
    s.setFlowConditions(0.5, 101325.0, 300.0)
    s.setKinematicViscosity(3e6, 1.0)
    s.initialize()
    cells = m.cells()
    U = C.perturbed_state(s.getSolution(), cells, seed=2, amplitude=0.1)
    if turbulence == "sst":
        U0 = s.getSolution()
        U[:, 4:] = U0[:, 4:] * (1.0 + 0.1 * np.sin(np.arange(len(U)))[:, None])
    R = s.computeResiduals(U)
    nv = 6 if turbulence == "sst" else 4
    assert np.abs(R[:, 4:]).max() > 0 if nv == 6 else np.abs(R[:, 4:]).max() == 0
    want = s.norm_vm(R)
    o = OracleSolver(spec, bcset="bump", viscous=True, init="bump")
    want_oracle = o.norm_vm(R)  # all six components; the last two are zero without SST
    assert want > 0 and abs(want - want_oracle) <= REL * want_oracle
    nc = m.n_cells
    Rd = torch.tensor(np.ascontiguousarray(R[:, :nv].T), dtype=torch.float64, device="cuda")
    vd = torch.tensor(cells[:, 0], dtype=torch.float64, device="cuda")
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    lib = api.lib()
    for call in range(2):
        out.fill_(float("nan"))
        st = lib.cfdg_norm_vm_noalloc(Rd.data_ptr(), vd.data_ptr(), nc, nv, out.data_ptr(), stream)
        assert st == 0, lib.cfdg_last_error().decode()
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - want) <= REL * want, (call, got, want)
        assert abs(got - want_oracle) <= REL * want_oracle, (call, got, want_oracle)


def test_norm_vm_noalloc_rejects_sizes_beyond_its_scratch(cuda_lib):
    import torch
    lib = cuda_lib.lib()
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = lib.cfdg_norm_vm_noalloc(buf.data_ptr(), buf.data_ptr(), 8_388_609, 4, buf.data_ptr(), None)
    assert st == 1
    assert "8388608" in lib.cfdg_last_error().decode()
    st = lib.cfdg_norm_vm_noalloc(buf.data_ptr(), buf.data_ptr(), 0, 4, buf.data_ptr(), None)
    assert st == 1
