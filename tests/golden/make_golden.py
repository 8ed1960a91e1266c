"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference sources exist (they are not on the GPU host):

    python oracle/build_ref.py            # compiles oracle/_ref/libref_*.so
    python tests/golden/make_golden.py

Writes
  ref_cases.npz            outputs of the reference's own Solver (compiled from its
                           sources) on the small cases of tests/cases.py: residual
                           for every flux x spatial scheme, gradients and limiter; local time
                           step, preconditioner, FD J v and one GMRES solve; 25-step
                           Newton traces
  ref_bump_full.npz        the reference's full bump solve (mesh/bump_1230, LLF, first
                           order, tol 1e-5): trace at 17 digits, GMRES counts, CFL and
                           the final state
  bump_1230.msh.gz         the reference's mesh/bump_1230 with LF line ends
  bump_residual_history.csv  the reference's shipped trace results/residual_history.csv
  bump_sol_9999.npz        Mach, Pressure, Density of the reference's shipped
                           results/sol_9999.vtk
  plate_nasa.msh.gz        the reference's mesh/new_laminar_flat_plate (its NASA laminar
                           flat plate, 6,962 quads) with LF line ends
  plate_cf_profile.csv     the reference's shipped skin-friction profile of that case
                           (results/data/cf_profile.csv: x, Cf, Blasius Cf)
  plate_nasa_ref.npz       the reference's own run of that case (compiled from its current
                           sources; src/main.cpp's settings, solveImplicit(1e-4, 50000)):
                           Newton steps, last res_vm, and x, Cf of the tag-4 faces at full
                           precision (about 45 minutes of one core)
"""
import gzip
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from mycode_gb300 import meshgen as mg  # noqa: E402
from oracle.oracle import RefSolver, ref_variant  # noqa: E402
import cases as C  # noqa: E402

from oracle.build_ref import reference_source  # noqa: E402

REF_SRC = reference_source()


def gen_cases():
    out = {}
    for name, case in C.CASES.items():
        spec = case["spec"]()
        # the mesh itself is stored: regenerating it elsewhere can differ in the last bit
        # (numpy's pow and cumsum are not the same on every machine)
        out[f"{name}/nodes"] = spec.nodes
        out[f"{name}/cells"] = spec.cells
        out[f"{name}/bedges"] = spec.bedges
        variant = ref_variant(case["bcset"], case["viscous"])
        r = RefSolver(spec, variant)
        C.setup(r, case)
        U0 = r.get_state()
        U = C.perturbed_state(U0, r.cells(), seed=11)
        out[f"{name}/U"] = U[:, :4]
        # gradients and limiter do not depend on the flux scheme
        out[f"{name}/G"] = r.gradients(U)
        out[f"{name}/phi"] = r.limiters(U)
        for fl in C.FLUXES:
            for sp in C.SPATIALS:
                r.setNumericalMethod(fl, sp)
                out[f"{name}/{fl}/{sp}/R"] = r.residual(U)[:, :4]
        # pseudo-time pieces and one Krylov solve with HLLC, limited
        r.setNumericalMethod("HLLC", "SECOND_ORDER_LIMITED")
        R = r.residual(U)
        r.set_state(U)
        out[f"{name}/dt"] = r.local_timestep(5.0)
        out[f"{name}/D"] = r.preconditioner()
        v = C.random_direction(U.shape[0], seed=5)
        out[f"{name}/v"] = v[:, :4]
        out[f"{name}/Jv"] = r.apply_jacobian(U, R, v)[:, :4]
        it, x = r.gmres(U, R, -R)
        out[f"{name}/gmres_iters"] = np.array(it)
        out[f"{name}/gmres_x"] = x[:, :4]
        # a 25-step Newton trace from the initial state
        r2 = RefSolver(spec, variant)
        C.setup(r2, case)
        r2.setNumericalMethod(*TRACE_METHOD[name])
        tr = r2.solveImplicit(0.0, 25)
        out[f"{name}/trace_res_vm"] = tr["res_vm"]
        out[f"{name}/trace_cfl"] = tr["cfl"]
        out[f"{name}/trace_iters"] = tr["gmres_iters"]
        out[f"{name}/trace_U"] = r2.get_state()[:, :4]
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **out)


TRACE_METHOD = {
    "bump": ("LLF", "FIRST_ORDER"),
    "bump_visc": ("ROE", "SECOND_ORDER_CENTRAL"),
    "supersonic": ("HLLC", "SECOND_ORDER_LIMITED"),
    "plate": ("HLLC", "FIRST_ORDER"),
    "plate_visc": ("ROE", "SECOND_ORDER_LIMITED"),
}


def gen_bump():
    src = os.path.join(REF_SRC, "mesh", "bump_1230")
    with open(src, "rb") as fh:
        text = fh.read().replace(b"\r", b"")
    with gzip.open(os.path.join(HERE, "bump_1230.msh.gz"), "wb", compresslevel=9) as fh:
        fh.write(text)
    with open(os.path.join(REF_SRC, "results", "residual_history.csv"), "rb") as fh:
        csv = fh.read().replace(b"\r", b"")
    with open(os.path.join(HERE, "bump_residual_history.csv"), "wb") as fh:
        fh.write(csv)
    fields = parse_vtk_cell_scalars(os.path.join(REF_SRC, "results", "sol_9999.vtk"))
    np.savez_compressed(os.path.join(HERE, "bump_sol_9999.npz"), **fields)
    spec = mg.read_gmsh(src)
    r = RefSolver(spec, "bump")
    r.setFlowConditions(0.5, 101325.0, 300.0)
    r.initialize()
    r.setNumericalMethod("LLF", "FIRST_ORDER")
    tr = r.solveImplicit(1e-5, 2500)
    U = r.get_state()
    np.savez_compressed(os.path.join(HERE, "ref_bump_full.npz"), res_vm=tr["res_vm"], res_abs=tr["res_abs"],
                        cfl=tr["cfl"], gmres_iters=tr["gmres_iters"], U=U[:, :4])


def gen_plate():
    for name, out in (("new_laminar_flat_plate", "plate_nasa.msh.gz"),):
        with open(os.path.join(REF_SRC, "mesh", name), "rb") as fh:
            text = fh.read().replace(b"\r", b"")
        with gzip.open(os.path.join(HERE, out), "wb", compresslevel=9) as fh:
            fh.write(text)
    with open(os.path.join(REF_SRC, "results", "data", "cf_profile.csv"), "rb") as fh:
        csv = fh.read().replace(b"\r", b"")
    with open(os.path.join(HERE, "plate_cf_profile.csv"), "wb") as fh:
        fh.write(csv)
    from oracle.oracle import OracleSolver
    spec = mg.read_gmsh(os.path.join(REF_SRC, "mesh", "new_laminar_flat_plate"))
    runs = []
    for cls, kw in ((RefSolver, dict(variant="plate_visc")),
                    (OracleSolver, dict(bcset="plate", viscous=True, init="freestream"))):
        r = cls(spec, **kw)
        r.setNumericalMethod("HLLC", "SECOND_ORDER_CENTRAL")
        r.setFlowConditions(0.1, 41368.5, 388.89)
        r.setKinematicViscosity(200000.0, 0.3048)
        r.initialize()
        tr = r.solveImplicit(1e-4, 50000)
        runs.append((tr["res_vm"], r.get_state()))
    (rv, U), (ov, Uo) = runs
    assert len(rv) == len(ov) and np.array_equal(U, Uo), "oracle and reference disagree on the plate"
    # the oracle's wall coefficients at the reference's final state (the same state bit for bit)
    o = OracleSolver(spec, bcset="plate", viscous=True, init="freestream")
    o.setFlowConditions(0.1, 41368.5, 388.89)
    o.setKinematicViscosity(200000.0, 0.3048)
    o.initialize()
    o.set_state(U)
    x, cp, cf = o.wall_coefficients(4)
    order = np.argsort(x, kind="stable")
    np.savez_compressed(os.path.join(HERE, "plate_nasa_ref.npz"), steps=len(rv), res_vm_last=rv[-1],
                        x=x[order], cf=cf[order])


def parse_vtk_cell_scalars(path):
    with open(path, "r", newline="") as fh:
        lines = [l.strip() for l in fh]
    out = {}
    i = 0
    while i < len(lines):
        if lines[i].startswith("SCALARS"):
            name = lines[i].split()[1]
            n = int(next(l for l in lines if l.startswith("CELL_DATA")).split()[1])
            vals = np.array([float(x) for x in lines[i + 2:i + 2 + n]])
            out[name] = vals
            i += 2 + n
        else:
            i += 1
    return out


if __name__ == "__main__":
    if REF_SRC is None:
        raise SystemExit("no reference checkout: set CFD_REFERENCE (see oracle/build_ref.py)")
    gen_cases()
    gen_bump()
    gen_plate()
    for f in sorted(os.listdir(HERE)):
        print(f, os.path.getsize(os.path.join(HERE, f)))
