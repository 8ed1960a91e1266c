"""libcfdgpu on the host: it loads, exports every entry point include/cfdg.h declares,
ingests meshes with the reference's face order and geometry bit for bit, and refuses to
compute without a GPU (there is no CPU path)."""
import ctypes
import os
import re

import numpy as np
import pytest

import cases as C
from mycode_gb300 import api, meshgen as mg
from oracle.oracle import OracleSolver

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "cfdg.h")).read()
    decl = r"^\s*(?:cfdg_status|void|const char\s*\*)\s+(cfdg_[a-z0-9_]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = api.lib()
    names = declared_symbols()
    assert len(names) >= 40
    for n in names:
        assert hasattr(lib, n), n
    assert set(api.SIGNATURES) == set(names)


def test_config_defaults_follow_reference():
    c = api.default_config()
    assert c.flux == api.FLUX["HLLC"] and c.spatial == api.SPATIAL["SECOND_ORDER_LIMITED"]
    assert c.gmres_m == 40 and c.gmres_tol == 1e-2
    assert c.gamma == 1.4 and c.R_gas == 287.0 and c.Pr == 0.72 and c.nu == 0.01
    assert c.cfl0 == 0.1 and c.cfl_max == 1e4 and c.limiter_freeze_step == 150 and c.limiter_freeze_cfl == 10.0


def test_config_defaults_leave_the_reference_algorithm_untouched():
    """Off by default: the start-up aids (no reference counterpart) and the persistent
    Arnoldi kernel; automatic (0): the Krylov driver, the barrier poll limit and the size
    from which the Arnoldi body splits its gather and dots (results the same either way)."""
    c = api.default_config()
    assert c.precision == 0 and c.jv == 0  # FP64 with the reference's FD J v
    assert c.startup_first_order == 0 and c.update_limit == 0.0
    assert c.persistent == 0 and c.barrier_poll_limit == 0 and c.gather_split_cells == 0
    assert c.krylov == -1 and c.pdl == 1 and c.newton_chain == 8


@pytest.mark.parametrize("spec_fn", [lambda: mg.mixed_box(8, 6), lambda: mg.wedge(12, 8),
                                     lambda: mg.laminar_plate(12, 8, ratio=1.2), lambda: mg.bump(3000, seed=1)])
@pytest.mark.parametrize("renumber", ["none", "hilbert", "rcm"])
def test_mesh_ingest_bit_exact_with_oracle(spec_fn, renumber):
    spec = spec_fn()
    m = api.Mesh.from_spec(spec, renumber=renumber)
    o = OracleSolver(spec)
    assert (m.n_cells, m.n_faces) == (o.n_cells, o.n_faces) == (spec.n_cells, spec.expected_faces())
    mi, md = m.faces()
    oi, od = o.faces()
    np.testing.assert_array_equal(mi, oi)
    np.testing.assert_array_equal(md, od)
    np.testing.assert_array_equal(m.cells(), o.cells())
    cp, fp = m.permutation()
    assert sorted(cp) == list(range(m.n_cells)) and sorted(fp) == list(range(m.n_faces))
    if renumber == "none":
        np.testing.assert_array_equal(cp, np.arange(m.n_cells))


def test_gmsh_loader_accepts_crlf_and_lf(tmp_path):
    spec = mg.mixed_box(5, 4)
    a, b = tmp_path / "lf.msh", tmp_path / "crlf.msh"
    mg.write_gmsh(spec, str(a))
    mg.write_gmsh(spec, str(b), crlf=True)
    ma, mb = api.Mesh.load(str(a)), api.Mesh.load(str(b))
    ms = api.Mesh.from_spec(spec)
    for m in (ma, mb):
        np.testing.assert_array_equal(m.faces()[0], ms.faces()[0])
        np.testing.assert_array_equal(m.faces()[1], ms.faces()[1])


@pytest.mark.parametrize("renumber", ["none", "hilbert"])
def test_reference_plate_mesh_file_ingest_bit_exact_with_oracle(tmp_path, renumber):
    """The reference's own NASA laminar plate mesh (Gmsh 2.2, 6,962 quads) through the
    library's C++ reader and host connectivity against the oracle's ingest of the same file."""
    import gzip

    gold = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    p = tmp_path / "plate_nasa.msh"
    with gzip.open(os.path.join(gold, "plate_nasa.msh.gz"), "rb") as fh:
        p.write_bytes(fh.read())
    m = api.Mesh.load(str(p), renumber=renumber)
    o = OracleSolver(mg.read_gmsh(str(p)))
    assert (m.n_cells, m.n_faces) == (o.n_cells, o.n_faces) and m.n_cells == 6962
    mi, md = m.faces()
    oi, od = o.faces()
    np.testing.assert_array_equal(mi, oi)
    np.testing.assert_array_equal(md, od)
    np.testing.assert_array_equal(m.cells(), o.cells())


def test_mesh_errors_are_reported(tmp_path):
    with pytest.raises(api.CfdgError) as e:
        api.Mesh.load(str(tmp_path / "missing.msh"))
    assert e.value.status == 6
    spec = mg.mixed_box(3, 2)
    bad = spec.cells.copy()
    bad[0, 0] = 10 ** 6
    with pytest.raises(api.CfdgError):
        api.Mesh.from_spec(mg.MeshSpec("bad", spec.nodes, bad, spec.bedges))


@pytest.mark.skipif(api.device_count() > 0, reason="a GPU is visible")
def test_no_cpu_fallback_without_gpu():
    m = api.Mesh.from_spec(mg.mixed_box(3, 2))
    with pytest.raises(api.CfdgError) as e:
        api.Solver(m)
    assert e.value.status == 2 and "no CUDA device" in str(e.value)


def test_solver_entry_points_reject_a_null_handle():
    """Entry points taking a solver return CFDG_ERR_ARG (1) with a message for a null handle
    (no GPU needed: the check comes before any device work)."""
    lib = api.lib()
    cfl, step = ctypes.c_double(), ctypes.c_int()
    calls = {
        "cfdg_set_cfl_max": (None, 2.0),
        "cfdg_set_newton_state": (None, 1.0, 0),
        "cfdg_get_newton_state": (None, ctypes.byref(cfl), ctypes.byref(step)),
        "cfdg_reset_newton": (None,),
        "cfdg_set_krylov": (None, 1),
    }
    for name, args in calls.items():
        assert getattr(lib, name)(*args) == 1, name
        assert lib.cfdg_last_error().decode(), name
