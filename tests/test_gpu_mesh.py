"""Mesh ingest on the GPU (cfdg_mesh_create_gpu) against the host build: the same faces in
the reference's order (src/Mesh.cpp:102-143), the same geometry (:148-201) bit for bit,
the same renumbering, and a device layout that gives bit-identical residuals and wall
distances; the same errors for a degenerate cell or an edge of three cells."""
import time

import numpy as np
import pytest

import cases as C
from mycode_gb300 import meshgen as mg
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu

SPECS = {
    "mixed_box": lambda: mg.mixed_box(8, 6),
    "wedge": lambda: mg.wedge(24, 16, jitter=0.1, seed=3),
    "plate": lambda: mg.laminar_plate(30, 16, ratio=1.1),
    "bump": lambda: mg.bump(20_000, seed=2),
}


@pytest.mark.parametrize("name", list(SPECS))
@pytest.mark.parametrize("renumber", ["none", "hilbert", "rcm"])
def test_gpu_mesh_equals_host_mesh(cuda_lib, name, renumber):
    spec = SPECS[name]()
    mh = cuda_lib.Mesh.from_spec(spec, renumber=renumber)
    mgpu = cuda_lib.Mesh.from_spec(spec, renumber=renumber, gpu=0)
    assert (mh.n_cells, mh.n_faces, mh.n_boundary_faces) == (mgpu.n_cells, mgpu.n_faces, mgpu.n_boundary_faces)
    for a, b in zip(mh.faces(), mgpu.faces()):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(mh.cells(), mgpu.cells())
    for a, b in zip(mh.permutation(), mgpu.permutation()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("case", ["supersonic", "plate_visc"])
def test_gpu_mesh_gives_the_same_residual_and_wall_distance(cuda_lib, case):
    c = C.CASES[case]
    spec = c["spec"]()
    o = OracleSolver(spec, bcset=c["bcset"], viscous=c["viscous"], init=c["init"])
    C.setup(o, c)
    U = C.perturbed_state(o.get_state(), o.cells(), seed=31)
    out = []
    for gpu in (None, 0):
        m = cuda_lib.Mesh.from_spec(spec, gpu=gpu)
        s = cuda_lib.Solver(m, bcset=c["bcset"], viscous=int(c["viscous"]), init=c["init"])
        C.setup(s, c)
        s.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
        out.append((s.computeResiduals(U), s.wall_distance()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    o.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
    np.testing.assert_array_equal(out[1][0], o.residual(U))


def test_gpu_mesh_reports_the_host_errors(cuda_lib):
    spec = mg.box(3, 2, split=True)
    cells = spec.cells.copy()
    tri = int(np.flatnonzero(cells[:, 3] < 0)[0])
    xy = spec.nodes.copy()
    xy[cells[tri, 2]] = xy[cells[tri, 0]] + 0.5 * (xy[cells[tri, 1]] - xy[cells[tri, 0]])
    bad = mg.MeshSpec("degenerate", xy, cells, spec.bedges)
    msgs = []
    for gpu in (None, 0):
        with pytest.raises(cuda_lib.CfdgError) as e:
            cuda_lib.Mesh.from_spec(bad, gpu=gpu)
        assert e.value.status == 6
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1]
    # a third cell on the edge the two quads of a 2 x 1 box share
    base = mg.box(2, 1)
    a, b = sorted(set(base.cells[0, :4].tolist()) & set(base.cells[1, :4].tolist()))
    extra = np.array([[a, b, len(base.nodes), -1]], np.int32)
    nodes = np.vstack([base.nodes, [[0.37, 1.9]]])
    three = mg.MeshSpec("three", nodes, np.vstack([base.cells, extra]).astype(np.int32), base.bedges)
    msgs = []
    for gpu in (None, 0):
        with pytest.raises(cuda_lib.CfdgError) as e:
            cuda_lib.Mesh.from_spec(three, gpu=gpu)
        assert e.value.status == 6
        msgs.append(str(e.value))
    assert msgs[0] == msgs[1], msgs


def test_gpu_mesh_at_one_million_cells(cuda_lib):
    spec = mg.bump(1_000_000, jitter=0.10, seed=0)
    t0 = time.perf_counter()
    mh = cuda_lib.Mesh.from_spec(spec)
    th = time.perf_counter() - t0
    t0 = time.perf_counter()
    mgpu = cuda_lib.Mesh.from_spec(spec, gpu=0)
    tg = time.perf_counter() - t0
    print(f"1M-cell bump: host build {th:.3f} s, GPU build {tg:.3f} s")
    for a, b in zip(mh.faces(), mgpu.faces()):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(mh.permutation(), mgpu.permutation()):
        np.testing.assert_array_equal(a, b)
