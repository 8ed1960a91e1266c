"""Failure detection without faulting the GPU: every failure is made on the host (a bad
state, a degenerate mesh, a corrupt file) or by a device wait whose limit runs out, and
each must come back as a status code with the context still usable.

The reference has no error paths here: NaNs propagate silently, a degenerate cell divides
by a zero volume, and an unreadable mesh exits the process (src/Mesh.cpp:32-35)."""
import numpy as np
import pytest

import cases as C
from mycode_gb300 import api, meshgen as mg


def _status(excinfo):
    return excinfo.value.status


def test_zero_area_cell_is_rejected_at_ingest():
    """A triangle whose three nodes are collinear has zero area: the mesh is refused
    (CFDG_ERR_MESH) before any solver divides by its volume."""
    spec = mg.box(3, 2, split=True)
    cells = spec.cells.copy()
    tri = int(np.flatnonzero(cells[:, 3] < 0)[0])
    a, b = cells[tri, 0], cells[tri, 1]
    xy = spec.nodes.copy()
    # move the third node onto the line through the first two
    xy[cells[tri, 2]] = xy[a] + 0.5 * (xy[b] - xy[a])
    bad = mg.MeshSpec(spec.name + "_degenerate", xy, cells, spec.bedges)
    with pytest.raises(api.CfdgError) as e:
        api.Mesh.from_spec(bad)
    assert _status(e) == 6
    assert "area" in str(e.value)


def test_corrupt_gmsh_file_is_rejected(tmp_path):
    """A Gmsh file cut off inside its element list is an error status, not an exit."""
    p = tmp_path / "cut.msh"
    mg.write_gmsh(mg.box(3, 2), str(p))
    text = p.read_text()
    p.write_text(text[: text.index("$Elements") + 20])
    with pytest.raises(api.CfdgError) as e:
        api.Mesh.load(str(p))
    assert _status(e) == 6


def test_missing_gmsh_file_is_rejected(tmp_path):
    with pytest.raises(api.CfdgError) as e:
        api.Mesh.load(str(tmp_path / "absent.msh"))
    assert _status(e) == 6


def _supersonic(cuda_lib, **cfg):
    case = C.CASES["supersonic"]
    m = cuda_lib.Mesh.from_spec(case["spec"]())
    s = cuda_lib.Solver(m, bcset=case["bcset"], viscous=0, init=case["init"], **cfg)
    C.setup(s, case)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [dict(precision="fp64", jv="fd", krylov=0),
                                 dict(precision="mixed", jv="exact", krylov=1)],
                         ids=["host_gmres_fd", "graph_gmres_mixed"])
def test_nan_in_state_reports_err_nan_and_solver_recovers(cuda_lib, cfg):
    """A NaN planted in one cell's density (host-side injection) makes the Newton step
    return CFDG_ERR_NAN; the same solver then steps normally from a good state."""
    s = _supersonic(cuda_lib, **cfg)
    U0 = s.getSolution()
    U = U0.copy()
    U[len(U) // 2, 0] = np.nan
    s.set_state(U)
    with pytest.raises(cuda_lib.CfdgError) as e:
        s.newton_step(0.0)
    assert _status(e) == 3
    s.set_state(U0)
    s.reset_newton()
    rec, _ = s.newton_step(0.0)
    assert np.isfinite(rec.res_vm) and rec.gmres_iters >= 1
    assert np.isfinite(s.getSolution()).all()


@pytest.mark.gpu
def test_negative_density_after_update_reports_err_nan(cuda_lib):
    """A state whose density is negative in one cell gives a non-finite sound speed in the
    residual: the step reports CFDG_ERR_NAN instead of carrying NaNs forward."""
    s = _supersonic(cuda_lib, precision="mixed", jv="exact", krylov=1)
    U = s.getSolution()
    U[3, 0] = -U[3, 0]
    s.set_state(U)
    with pytest.raises(cuda_lib.CfdgError) as e:
        s.newton_step(0.0)
    assert _status(e) == 3


@pytest.mark.gpu
def test_persistent_kernel_barrier_wait_runs_out_and_reports_timeout(cuda_lib):
    """The persistent Arnoldi kernel's grid barrier gives up after barrier_poll_limit polls:
    with a limit of one poll the blocks that arrive before the last one stop waiting, the
    kernel finishes (every wait bounded, every access in bounds) and the step reports
    CFDG_ERR_TIMEOUT; the barrier words are reset, and a solver with the default limit
    then runs the same step normally."""
    s = _supersonic(cuda_lib, precision="mixed", jv="exact", krylov=1, persistent=1, barrier_poll_limit=1)
    assert s.krylov_info()["persistent"]
    U0 = s.getSolution()
    with pytest.raises(cuda_lib.CfdgError) as e:
        for _ in range(3):
            s.newton_step(0.0)
    assert _status(e) == 5
    s.close()
    ok = _supersonic(cuda_lib, precision="mixed", jv="exact", krylov=1, persistent=1)
    ok.set_state(U0)
    rec, _ = ok.newton_step(0.0)
    assert np.isfinite(rec.res_vm) and rec.gmres_iters >= 1
