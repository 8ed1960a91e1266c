"""Build the reference solver as shared-library oracles: oracle/_ref/libref_<variant>.so.

Test infrastructure only.  The reference (AmberMond/mycode) selects its boundary
condition set, initial condition and the viscous term by commenting whole function
bodies in and out of src/Solver.cpp (see the variants at src/Solver.cpp:806-863,
:973-1011, :1088-1139 and the initialisers at :46-65, :905-920; the viscous toggle
is :787 vs :792).  This script writes one source variant per case into a temporary
directory OUTSIDE the repository (checking every edited line's text first), compiles
it with the reference's own flags (``g++ -O2 -std=c++17``, makefile:2) together with
oracle/ref_harness.cpp, and keeps only the shared objects in oracle/_ref/.

The one edit that is not a variant switch: with the viscous term enabled, a boundary
face that is not a no-slip wall reads ``mesh.cells[f.neighbor]`` with neighbor = -1
(src/Solver.cpp:729-730), which is undefined behaviour.  The variants with the viscous
term replace that index by the owner, which makes the non-orthogonal correction
vanish (dist2 = 0) on those faces; the CPU restatement and the CUDA kernels define
the same behaviour.

Where the reference checkout is: ``--src``, else the CFD_REFERENCE environment variable,
else the read-only checkout this recipe was written against (REFERENCE_CHECKOUT); this
file is the only one that names that location.  Where none exists (e.g. on a machine
that has only this repository) nothing is built and the tests that need these objects
skip; the committed fixtures under tests/golden/ still pin the restatement.

Usage: python oracle/build_ref.py [--src PATH]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REFERENCE_CHECKOUT = "/root/reference"


def reference_source():
    """The reference checkout to build from, or None when there is none here."""
    for cand in (os.environ.get("CFD_REFERENCE"), REFERENCE_CHECKOUT):
        if cand and os.path.isdir(os.path.join(cand, "src")):
            return cand
    return None

# (first line, last line) ranges of src/Solver.cpp, 1-based inclusive
ACTIVE_INIT = (46, 65)
ACTIVE_BC = (806, 863)
BC_SUPERSONIC = (973, 1011)
BC_PLATE = (1088, 1139)
INIT_FREESTREAM = (905, 920)

VARIANTS = {
    # name: (bc range to enable or None, init range to enable or None, viscous[, knobs])
    "bump": (None, None, False),
    "bump_visc": (None, None, True),
    "supersonic": (BC_SUPERSONIC, INIT_FREESTREAM, False),
    "plate": (BC_PLATE, INIT_FREESTREAM, False),
    "plate_visc": (BC_PLATE, INIT_FREESTREAM, True),
    # the supersonic wedge of the converged-solution fixtures: GMRES(30) and a first CFL of
    # 10, with the reference's limiter freeze and with the limiter frozen from the start
    "supersonic_m30_cfl10": (BC_SUPERSONIC, INIT_FREESTREAM, False, dict(REF_GMRES_M=30, REF_CFL0=10.0)),
    "supersonic_m30_cfl10_frozen": (BC_SUPERSONIC, INIT_FREESTREAM, False,
                                    dict(REF_GMRES_M=30, REF_CFL0=10.0, REF_FREEZE_STEP=-1)),
}

# Hard-coded constants of solveGMRES / solveImplicit made compile-time knobs; their
# defaults are the reference's own values, so a variant without knobs compiles to the
# reference's code.  (line, original text, replacement)
KNOBS = (
    (1479, "int m = 40;", "int m = REF_GMRES_M;"),
    (1701, "double CFL = 0.1;", "double CFL = REF_CFL0;"),
    (1714, "if (step > 150 || CFL > 10.0)", "if (step > REF_FREEZE_STEP || CFL > REF_FREEZE_CFL)"),
)
KNOB_DEFAULTS = dict(REF_GMRES_M=40, REF_CFL0=0.1, REF_FREEZE_STEP=150, REF_FREEZE_CFL=10.0)


def _expect(lines, no, needle):
    got = lines[no - 1]
    if needle not in got:
        raise SystemExit(f"src/Solver.cpp:{no}: expected {needle!r}, found {got!r}")


def _comment(lines, rng):
    a, b = rng
    for i in range(a - 1, b):
        lines[i] = "// " + lines[i]


def _uncomment(lines, rng):
    a, b = rng
    for i in range(a - 1, b):
        s = lines[i]
        k = s.find("//")
        if k < 0 or s[:k].strip():
            if s.strip():
                raise SystemExit(f"src/Solver.cpp:{i + 1}: not a comment line: {s!r}")
            continue
        lines[i] = s[:k] + s[k + 2:]


def make_variant(src_lines, bc, init, viscous):
    lines = list(src_lines)
    for no, old, new in KNOBS:
        _expect(lines, no, old)
        lines[no - 1] = lines[no - 1].replace(old, new)
    _expect(lines, 46, "void Solver::initialize()")
    _expect(lines, 806, "State Solver::getBoundaryGhostState")
    _expect(lines, 863, "}")
    _expect(lines, 787, "// State TotalFlux = FluxEuler - FluxVisc;")
    _expect(lines, 792, "State TotalFlux = FluxEuler;")
    _expect(lines, 729, "double dx_LR = mesh.cells[f.neighbor].x_c - mesh.cells[f.owner].x_c;")
    _expect(lines, 730, "double dy_LR = mesh.cells[f.neighbor].y_c - mesh.cells[f.owner].y_c;")
    if bc is not None:
        _expect(lines, bc[0], "State Solver::getBoundaryGhostState")
        _comment(lines, ACTIVE_BC)
        _uncomment(lines, bc)
    if init is not None:
        _expect(lines, init[0], "void Solver::initialize()")
        _comment(lines, ACTIVE_INIT)
        _uncomment(lines, init)
    if viscous:
        lines[786] = lines[786].replace("// State TotalFlux", "State TotalFlux")
        lines[791] = lines[791].replace("State TotalFlux = FluxEuler;", "// State TotalFlux = FluxEuler;")
        nb = "mesh.cells[f.neighbor >= 0 ? f.neighbor : f.owner]"
        lines[728] = lines[728].replace("mesh.cells[f.neighbor]", nb)
        lines[729] = lines[729].replace("mesh.cells[f.neighbor]", nb)
    # the knobs' defaults, prepended last so the line numbers above are the reference's
    defaults = "".join(f"#ifndef {k}\n#define {k} {v}\n#endif\n" for k, v in KNOB_DEFAULTS.items())
    return [defaults + lines[0]] + lines[1:]


def build(src_root: str, jobs: int = 4) -> list[str]:
    solver = os.path.join(src_root, "src", "Solver.cpp")
    mesh = os.path.join(src_root, "src", "Mesh.cpp")
    inc = os.path.join(src_root, "include")
    if not (os.path.isfile(solver) and os.path.isfile(mesh)):
        raise FileNotFoundError(f"reference sources not found under {src_root}")
    with open(solver, "r", newline="") as fh:
        src_lines = fh.read().split("\n")
    os.makedirs(OUT, exist_ok=True)
    tmp = tempfile.mkdtemp(prefix="cfd_ref_")
    procs, outs = [], []
    try:
        for name, spec in VARIANTS.items():
            bc, init, visc = spec[:3]
            knobs = spec[3] if len(spec) > 3 else {}
            gen = os.path.join(tmp, f"Solver_{name}.cpp")
            with open(gen, "w", newline="") as fh:
                fh.write("\n".join(make_variant(src_lines, bc, init, visc)))
            so = os.path.join(OUT, f"libref_{name}.so")
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                   f"-I{inc}", f'-DREF_SOLVER_CPP="{gen}"', f'-DREF_MESH_CPP="{mesh}"',
                   *[f"-D{k}={v}" for k, v in knobs.items()],
                   os.path.join(HERE, "ref_harness.cpp"), "-o", so]
            procs.append((name, subprocess.Popen(cmd, stderr=subprocess.PIPE, text=True)))
            outs.append(so)
            if len(procs) >= jobs:
                _wait(procs.pop(0))
        for p in procs:
            _wait(p)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return outs


def _wait(item):
    name, p = item
    _, err = p.communicate()
    if p.returncode != 0:
        raise SystemExit(f"building reference variant {name} failed:\n{err}")


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=None)
    a = ap.parse_args(argv)
    src = a.src or reference_source()
    if src is None:
        raise SystemExit("no reference checkout: pass --src or set CFD_REFERENCE")
    for so in build(src):
        print(so)


if __name__ == "__main__":
    sys.exit(main())
