"""Small parity cases shared by the CPU and GPU tests.

Each case is a synthetic mesh plus one of the reference's boundary-condition sets
(src/Solver.cpp:806-863 bump, :973-1011 supersonic, :1088-1139 flat plate), its
initialiser and flow conditions, and optionally the viscous term.
"""
import numpy as np

from mycode_gb300 import meshgen as mg

CASES = {
    "bump": dict(spec=lambda: mg.mixed_box(8, 6), bcset="bump", viscous=False, init="bump",
                 flow=("cond", 0.3, 101325.0, 300.0), re=None),
    "bump_visc": dict(spec=lambda: mg.mixed_box(8, 6, seed=3), bcset="bump", viscous=True, init="bump",
                      flow=("cond", 0.3, 101325.0, 300.0), re=(2e3, 1.0)),
    "supersonic": dict(spec=lambda: mg.wedge(12, 8, jitter=0.1, seed=2), bcset="supersonic", viscous=False,
                       init="freestream", flow=("cond", 2.5, 101325.0, 300.0), re=None),
    "plate": dict(spec=lambda: mg.laminar_plate(12, 8, ratio=1.2), bcset="plate", viscous=False,
                  init="freestream", flow=("static", 0.3, 101325.0, 300.0), re=None),
    "plate_visc": dict(spec=lambda: mg.laminar_plate(12, 8, ratio=1.2), bcset="plate", viscous=True,
                       init="freestream", flow=("static", 0.3, 101325.0, 300.0), re=(1e3, 1.0)),
}
FLUXES = ["LLF", "ROE", "HLLC"]
SPATIALS = ["FIRST_ORDER", "SECOND_ORDER_CENTRAL", "SECOND_ORDER_LIMITED"]


def setup(solver, case):
    """Apply a case's flow conditions and initialiser to any object with the reference
    Solver's setter names (GPU solver, C oracle or compiled reference)."""
    kind, M, P, T = case["flow"]
    if kind == "cond":
        solver.setFlowConditions(M, P, T)
    else:
        solver.setFreestreamStatic(M, P, T)
    if case["re"] is not None:
        solver.setKinematicViscosity(*case["re"])
    solver.initialize()


def perturbed_state(U0, cells_vol_xc_yc, seed, amplitude=0.05, gamma=1.4):
    """Initial state times a seeded smooth perturbation of rho, u, v, p (<= amplitude),
    plus a cross-flow component so every face sees non-trivial velocity."""
    xc = cells_vol_xc_yc[:, 1:]
    pert = mg.smooth_perturbation(xc, seed, amplitude)
    r = U0[:, 0]
    u = U0[:, 1] / r
    v = U0[:, 2] / r
    p = (gamma - 1.0) * (U0[:, 3] - 0.5 * (U0[:, 1] ** 2 + U0[:, 2] ** 2) / r)
    c = np.sqrt(gamma * p / r)
    r = r * (1 + pert[:, 0])
    u = u * (1 + pert[:, 1]) + amplitude * c * pert[:, 1]
    v = v * (1 + pert[:, 2]) + amplitude * c * pert[:, 2]
    p = p * (1 + pert[:, 3])
    U = np.zeros_like(U0)
    U[:, 0] = r
    U[:, 1] = r * u
    U[:, 2] = r * v
    U[:, 3] = p / (gamma - 1.0) + 0.5 * r * (u * u + v * v)
    return U


def random_direction(n_cells, seed, nv=4):
    v = np.random.default_rng(seed).standard_normal((n_cells, 6))
    v[:, nv:] = 0.0
    return v


def golden_spec(gold, name):
    """The case's mesh exactly as stored with the reference fixtures."""
    return mg.MeshSpec(name, gold[f"{name}/nodes"], gold[f"{name}/cells"], gold[f"{name}/bedges"])
