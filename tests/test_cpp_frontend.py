"""The C++ front-end (include/cfdg_solver.hpp) as a reference driver would use it:
the reference's default bump case (src/main.cpp:53-100) built with g++ against
libcfdgpu.so, its printed residual history against the reference's shipped trace."""
import gzip
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def _build(tmp_path):
    exe = tmp_path / "bump_main"
    lib = os.path.join(ROOT, "mycode_gb300", "_lib")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "mycode_gb300", "examples", "bump_main.cpp"),
                           "-L", lib, "-lcfdgpu", f"-Wl,-rpath,{lib}", "-o", str(exe)])
    return exe


def test_cpp_driver_compiles(tmp_path):
    assert _build(tmp_path).exists()


@pytest.mark.gpu
def test_cpp_driver_runs_reference_case(cuda_lib, tmp_path):
    exe = _build(tmp_path)
    mesh = tmp_path / "bump_1230.msh"
    with gzip.open(os.path.join(GOLD, "bump_1230.msh.gz"), "rb") as fh:
        mesh.write_bytes(fh.read())
    out = subprocess.run([str(exe), str(mesh), "80"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    rows = [l.split(",") for l in out.stdout.strip().splitlines()[1:] if re.match(r"^\d+, ", l)]
    got = np.array([float(r[1]) for r in rows])
    gold = np.loadtxt(os.path.join(GOLD, "bump_residual_history.csv"), delimiter=",", skiprows=1)
    assert len(got) == 80
    np.testing.assert_array_equal(got[:60], gold[:60, 1])


@pytest.mark.gpu
def test_cpp_driver_converges_to_the_reference_drag_and_entropy_error(cuda_lib, tmp_path):
    """The full default case: the reference's run printed L2 entropy error 0.00291055 and
    drag -804.738 (its default 6-digit stream output)."""
    exe = _build(tmp_path)
    mesh = tmp_path / "bump_1230.msh"
    with gzip.open(os.path.join(GOLD, "bump_1230.msh.gz"), "rb") as fh:
        mesh.write_bytes(fh.read())
    out = subprocess.run([str(exe), str(mesh), "2500"], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stderr
    ent = float(re.search(r"L2 Entropy Error: (\S+)", out.stdout).group(1))
    drag = float(re.search(r"Drag :(\S+)", out.stdout).group(1))
    assert ent == pytest.approx(0.00291055, rel=2e-6)
    assert drag == pytest.approx(-804.738, rel=2e-6)
