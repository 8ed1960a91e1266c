"""ctypes front-ends for the two CPU checkers — TEST INFRASTRUCTURE ONLY.

* :class:`OracleSolver` drives oracle/cfd_oracle.c, the plain-C restatement of the
  reference's residual-and-Newton path (built here and on the GPU host by
  :func:`build_oracle`).
* :class:`RefSolver` drives the reference solver itself, compiled from its own
  sources into oracle/_ref/libref_<variant>.so by oracle/build_ref.py (only where
  the reference sources exist; absent elsewhere).

Both take a :class:`mycode_gb300.meshgen.MeshSpec` and use the reference's AoS
state layout (6 doubles per cell) and numbering.  Only tests, the smoke check and
the benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(BUILD, "liboracle.so")

FLUX = {"LLF": 0, "ROE": 1, "HLLC": 2, "AUSM": 3}
SPATIAL = {"FIRST_ORDER": 0, "SECOND_ORDER_CENTRAL": 1, "SECOND_ORDER_LIMITED": 2}
BCSET = {"bump": 0, "supersonic": 1, "plate": 2}
INIT = {"bump": 0, "freestream": 1}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_oracle(force: bool = False) -> str:
    """Compile oracle/cfd_oracle.c (no FMA contraction, so results match x86 g++ -O2)."""
    src = os.path.join(HERE, "cfd_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                           src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def _oracle_lib():
    global _lib
    if _lib is None:
        lib = C.CDLL(build_oracle())
        vp = C.c_void_p
        sig = {
            "om_mesh_build": (vp, [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip]),
            "om_mesh_free": (None, [vp]),
            "om_mesh_n_cells": (C.c_int, [vp]),
            "om_mesh_n_faces": (C.c_int, [vp]),
            "om_mesh_faces": (None, [vp, _ip, _dp]),
            "om_mesh_cells": (None, [vp, _dp]),
            "om_solver_create": (vp, [vp]),
            "om_solver_free": (None, [vp]),
            "om_set_method": (None, [vp, C.c_int, C.c_int]),
            "om_set_case": (None, [vp, C.c_int, C.c_int, C.c_int]),
            "om_set_gmres": (None, [vp, C.c_int, C.c_double]),
            "om_set_nu": (None, [vp, C.c_double]),
            "om_set_cfl0": (None, [vp, C.c_double]),
            "om_time_step_explicit": (C.c_double, [vp, C.c_double]),
            "om_solve_unsteady": (None, [vp, C.c_double, C.c_int, _ip, _dp]),
            "om_set_flow_conditions": (None, [vp, C.c_double, C.c_double, C.c_double]),
            "om_set_freestream_static": (None, [vp, C.c_double, C.c_double, C.c_double]),
            "om_set_kinematic_viscosity": (None, [vp, C.c_double, C.c_double]),
            "om_get_params": (None, [vp, _dp]),
            "om_initialize": (None, [vp]),
            "om_set_state": (None, [vp, _dp]),
            "om_get_state": (None, [vp, _dp]),
            "om_gradients": (None, [vp, _dp]),
            "om_limiters": (None, [vp, _dp]),
            "om_get_gradients": (None, [vp, _dp]),
            "om_get_limiters": (None, [vp, _dp]),
            "om_set_limiters": (None, [vp, _dp]),
            "om_residual": (None, [vp, _dp, _dp, C.c_int]),
            "om_norm": (C.c_double, [C.c_int, _dp]),
            "om_dot": (C.c_double, [C.c_int, _dp, _dp]),
            "om_norm_vm": (C.c_double, [vp, _dp]),
            "om_local_timestep": (None, [vp, C.c_double]),
            "om_get_dt": (None, [vp, _dp]),
            "om_set_dt": (None, [vp, _dp]),
            "om_preconditioner": (None, [vp, _dp]),
            "om_apply_jacobian": (None, [vp, _dp, _dp, _dp, _dp]),
            "om_gmres": (C.c_int, [vp, _dp, _dp, _dp, _dp]),
            "om_solve_implicit": (C.c_int, [vp, C.c_double, C.c_int, _dp, _dp, _dp, _ip, _dp]),
            "om_set_freeze": (None, [vp, C.c_int, C.c_double]),
            "om_set_stop_rho": (None, [vp, C.c_double]),
            "om_norm_vm_rho": (C.c_double, [vp, _dp]),
            "om_drag": (C.c_double, [vp]),
            "om_entropy_error": (C.c_double, [vp]),
            "om_residual_sst": (None, [vp, _dp, _dp, C.c_double, C.c_double]),
            "om_sst_freestream": (None, [vp, C.c_double, C.c_double, _dp]),
            "om_sst_reset": (None, []),
            "om_wall_coefficients": (C.c_int, [vp, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
            "om_wall_distance": (None, [vp, _dp]),
            "om_objective": (C.c_double, [vp, C.c_int, C.c_double, C.c_double, C.c_void_p]),
            "om_inviscid_flux": (None, [_dp, _dp, C.c_double, C.c_double, C.c_int, _dp]),
            "om_normal_flux": (None, [_dp, C.c_double, C.c_double, _dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _mesh_arrays(spec):
    xy = np.ascontiguousarray(spec.nodes, dtype=np.float64).ravel()
    cells = np.ascontiguousarray(spec.cells, dtype=np.int32).ravel()
    bed = np.ascontiguousarray(spec.bedges, dtype=np.int32).ravel()
    return xy, cells, bed


class _Base:
    n_cells: int
    n_faces: int

    def state_from_primitives(self, prim: np.ndarray, gamma: float = 1.4) -> np.ndarray:
        """AoS conservative state from per-cell primitives [rho, u, v, p] (k = w = 0)."""
        r, u, v, p = prim.T
        U = np.zeros((prim.shape[0], 6))
        U[:, 0] = r
        U[:, 1] = r * u
        U[:, 2] = r * v
        U[:, 3] = p / (gamma - 1.0) + 0.5 * r * (u * u + v * v)
        return U


FLUX_CODES = {"LLF": 0, "ROE": 1, "HLLC": 2}


def inviscid_flux(UL, UR, nx, ny, scheme):
    """computeInviscidFlux (include/Flux.hpp:216-227) of one face: 6 components."""
    F = np.zeros(6)
    _oracle_lib().om_inviscid_flux(np.ascontiguousarray(UL, np.float64), np.ascontiguousarray(UR, np.float64),
                                   float(nx), float(ny), FLUX_CODES[scheme], F)
    return F


def normal_flux(U, nx, ny):
    """computeNormalFlux (include/Flux.hpp:23-34): 6 components, k and w zero."""
    F = np.zeros(6)
    _oracle_lib().om_normal_flux(np.ascontiguousarray(U, np.float64), float(nx), float(ny), F)
    return F


class OracleSolver(_Base):
    """The C restatement (oracle/cfd_oracle.c) with the reference's Solver surface."""

    def __init__(self, spec, bcset="bump", viscous=False, init="bump"):
        L = _oracle_lib()
        self._L = L
        self._arrays = _mesh_arrays(spec)
        xy, cells, bed = self._arrays
        self._mesh = L.om_mesh_build(spec.n_nodes, xy, spec.n_cells, cells, spec.bedges.shape[0], bed)
        self._s = L.om_solver_create(self._mesh)
        self.n_cells = L.om_mesh_n_cells(self._mesh)
        self.n_faces = L.om_mesh_n_faces(self._mesh)
        L.om_set_case(self._s, BCSET[bcset], int(bool(viscous)), INIT[init])

    def __del__(self):
        try:
            self._L.om_solver_free(self._s)
            self._L.om_mesh_free(self._mesh)
        except Exception:
            pass

    def faces(self):
        i5 = np.zeros(5 * self.n_faces, np.int32)
        d5 = np.zeros(5 * self.n_faces)
        self._L.om_mesh_faces(self._mesh, i5, d5)
        return i5.reshape(-1, 5), d5.reshape(-1, 5)

    def cells(self):
        d = np.zeros(3 * self.n_cells)
        self._L.om_mesh_cells(self._mesh, d)
        return d.reshape(-1, 3)

    def setNumericalMethod(self, flux, spatial):
        self._L.om_set_method(self._s, FLUX[flux], SPATIAL[spatial])

    def setGMRES(self, m, tol=1e-2):
        self._L.om_set_gmres(self._s, int(m), float(tol))

    def setNu(self, nu):
        self._L.om_set_nu(self._s, float(nu))

    def setCFL0(self, cfl0):
        self._L.om_set_cfl0(self._s, float(cfl0))

    def timeStepExplicit(self, dt):
        return self._L.om_time_step_explicit(self._s, float(dt))

    def solveUnsteady(self, dt_phy, max_time_steps):
        n = int(max_time_steps)
        it, res = np.zeros(max(n, 1), np.int32), np.zeros(max(n, 1))
        self._L.om_solve_unsteady(self._s, float(dt_phy), n, it, res)
        return {"newton_steps": it[:n], "res_vm": res[:n]}

    def setFlowConditions(self, M, P, T):
        self._L.om_set_flow_conditions(self._s, M, P, T)

    def setFreestreamStatic(self, M, P, T):
        self._L.om_set_freestream_static(self._s, M, P, T)

    def setKinematicViscosity(self, Re, L):
        self._L.om_set_kinematic_viscosity(self._s, Re, L)

    def params(self):
        o = np.zeros(6)
        self._L.om_get_params(self._s, o)
        return dict(zip(["M_inf", "P0", "T0", "Pexit", "nu", "R_gas"], o))

    def initialize(self):
        self._L.om_initialize(self._s)

    def set_state(self, U):
        self._L.om_set_state(self._s, np.ascontiguousarray(U, np.float64).ravel())

    def get_state(self):
        U = np.zeros(6 * self.n_cells)
        self._L.om_get_state(self._s, U)
        return U.reshape(-1, 6)

    def residual(self, U, update_limiters=True):
        R = np.zeros(6 * self.n_cells)
        self._L.om_residual(self._s, np.ascontiguousarray(U, np.float64).ravel(), R, int(update_limiters))
        return R.reshape(-1, 6)

    def gradients(self, U):
        self._L.om_gradients(self._s, np.ascontiguousarray(U, np.float64).ravel())
        g = np.zeros(10 * self.n_cells)
        self._L.om_get_gradients(self._s, g)
        return g.reshape(-1, 10)

    def limiters(self, U):
        u = np.ascontiguousarray(U, np.float64).ravel()
        self._L.om_gradients(self._s, u)
        self._L.om_limiters(self._s, u)
        return self.get_limiters()

    def get_limiters(self):
        p = np.zeros(self.n_cells)
        self._L.om_get_limiters(self._s, p)
        return p

    def set_limiters(self, phi):
        self._L.om_set_limiters(self._s, np.ascontiguousarray(phi, np.float64))

    def local_timestep(self, cfl):
        self._L.om_local_timestep(self._s, float(cfl))
        dt = np.zeros(self.n_cells)
        self._L.om_get_dt(self._s, dt)
        return dt

    def set_dt(self, dt):
        self._L.om_set_dt(self._s, np.ascontiguousarray(dt, np.float64))

    def preconditioner(self):
        D = np.zeros(self.n_cells)
        self._L.om_preconditioner(self._s, D)
        return D

    def apply_jacobian(self, Ub, Rb, v):
        J = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        self._L.om_apply_jacobian(self._s, c(Ub), c(Rb), c(v), J)
        return J.reshape(-1, 6)

    def gmres(self, Ub, Rb, rhs):
        x = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        it = self._L.om_gmres(self._s, c(Ub), c(Rb), c(rhs), x)
        return it, x.reshape(-1, 6)

    def norm_vm(self, R):
        return self._L.om_norm_vm(self._s, np.ascontiguousarray(R, np.float64).ravel())

    def solveImplicit(self, tol, max_steps):
        a, b, c, d = np.zeros(max_steps), np.zeros(max_steps), np.zeros(max_steps), np.zeros(max_steps)
        it = np.zeros(max_steps, np.int32)
        n = self._L.om_solve_implicit(self._s, float(tol), int(max_steps), a, b, c, it, d)
        return {"res_vm": a[:n], "res_abs": b[:n], "cfl": c[:n], "gmres_iters": it[:n], "res_rho": d[:n]}

    def setLimiterFreeze(self, step, cfl=10.0):
        """The limiter-freeze rule (reference: step > 150 or CFL > 10); step = -1 keeps the
        current limiter for the whole solve."""
        self._L.om_set_freeze(self._s, int(step), float(cfl))

    def setStopRho(self, tol):
        """Also stop solveImplicit once the density residual is at or below tol (0 = off)."""
        self._L.om_set_stop_rho(self._s, float(tol))

    def norm_vm_rho(self, R):
        return self._L.om_norm_vm_rho(self._s, np.ascontiguousarray(R, np.float64).ravel())

    def drag(self):
        return self._L.om_drag(self._s)

    def entropy_error(self):
        return self._L.om_entropy_error(self._s)

    def wall_coefficients(self, tag=4):
        """x_mid, Cp, Cf of the boundary faces with ``tag`` in face order (current state)."""
        n = self._L.om_wall_coefficients(self._s, int(tag), None, None, None)
        x, cp, cf = np.zeros(n), np.zeros(n), np.zeros(n)
        if n:
            self._L.om_wall_coefficients(self._s, int(tag), x.ctypes.data, cp.ctypes.data, cf.ctypes.data)
        return x, cp, cf

    def wall_distance(self):
        d = np.zeros(self.n_cells)
        self._L.om_wall_distance(self._s, d)
        return d

    OBJECTIVES = {"pressure_drag": 0, "skin_friction_drag": 1, "wall_pressure": 2}

    def objective(self, kind, x0=-1e300, x1=1e300, gradient=True):
        k = self.OBJECTIVES[kind] if isinstance(kind, str) else int(kind)
        g = np.zeros(6 * self.n_cells) if gradient else None
        J = self._L.om_objective(self._s, k, float(x0), float(x1), g.ctypes.data if gradient else None)
        return (J, g.reshape(-1, 6)) if gradient else J

    def residual_sst(self, U, turb_intensity=0.001, mut_ratio=0.01):
        """Residual of the mean flow plus the SST k and w equations (nv = 6, AoS)."""
        R = np.zeros(6 * self.n_cells)
        self._L.om_residual_sst(self._s, np.ascontiguousarray(U, np.float64).ravel(), R, float(turb_intensity),
                                float(mut_ratio))
        return R.reshape(-1, 6)

    def sst_freestream(self, turb_intensity=0.001, mut_ratio=0.01):
        kw = np.zeros(2)
        self._L.om_sst_freestream(self._s, float(turb_intensity), float(mut_ratio), kw)
        return float(kw[0]), float(kw[1])


def ref_available(variant: str = "bump") -> bool:
    return os.path.exists(os.path.join(REF, f"libref_{variant}.so"))


def ref_variant(bcset: str, viscous: bool) -> str:
    if bcset == "supersonic":
        if viscous:
            raise ValueError("no reference build of the supersonic set with the viscous term")
        return "supersonic"
    return bcset + ("_visc" if viscous else "")


class RefSolver(_Base):
    """The reference's own Solver, compiled from its sources (oracle/_ref)."""

    _libs: dict = {}

    def __init__(self, spec, variant="bump"):
        path = os.path.join(REF, f"libref_{variant}.so")
        if variant not in RefSolver._libs:
            lib = C.CDLL(path)
            vp = C.c_void_p
            sig = {
                "ref_create": (vp, [C.c_int, _dp, C.c_int, _ip, C.c_int, _ip]),
                "ref_destroy": (None, [vp]),
                "ref_sizes": (None, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
                "ref_faces": (None, [vp, _ip, _dp]),
                "ref_cells": (None, [vp, _dp]),
                "ref_set_method": (None, [vp, C.c_int, C.c_int]),
                "ref_set_flow_conditions": (None, [vp, C.c_double, C.c_double, C.c_double]),
                "ref_set_freestream_static": (None, [vp, C.c_double, C.c_double, C.c_double]),
                "ref_set_kinematic_viscosity": (None, [vp, C.c_double, C.c_double]),
                "ref_get_params": (None, [vp, _dp]),
                "ref_initialize": (None, [vp]),
                "ref_set_state": (None, [vp, _dp]),
                "ref_get_state": (None, [vp, _dp]),
                "ref_residual": (None, [vp, _dp, _dp, C.c_int]),
                "ref_gradients": (None, [vp, _dp, _dp]),
                "ref_limiters": (None, [vp, _dp, _dp]),
                "ref_get_limiters": (None, [vp, _dp]),
                "ref_set_limiters": (None, [vp, _dp]),
                "ref_local_timestep": (None, [vp, C.c_double, _dp]),
                "ref_preconditioner": (None, [vp, _dp]),
                "ref_apply_jacobian": (None, [vp, _dp, _dp, _dp, _dp]),
                "ref_gmres": (C.c_int, [vp, _dp, _dp, _dp, _dp]),
                "ref_norm_vm": (C.c_double, [vp, _dp]),
                "ref_solve_implicit": (C.c_int, [vp, C.c_double, C.c_int, _dp, _dp, _dp, _ip]),
                "ref_wall_distance": (None, [vp, _dp]),
                "ref_drag": (C.c_double, [vp]),
                "ref_entropy_error": (C.c_double, [vp]),
                "ref_skin_friction": (C.c_int, [vp, C.c_char_p, _dp, _dp, C.c_int]),
                "ref_time_step_explicit": (None, [vp, C.c_double]),
                "ref_solve_unsteady": (None, [vp, C.c_double, C.c_int]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            RefSolver._libs[variant] = lib
        L = RefSolver._libs[variant]
        self._L = L
        self._arrays = _mesh_arrays(spec)
        xy, cells, bed = self._arrays
        self._h = L.ref_create(spec.n_nodes, xy, spec.n_cells, cells, spec.bedges.shape[0], bed)
        nc, nf = C.c_int(), C.c_int()
        L.ref_sizes(self._h, C.byref(nc), C.byref(nf))
        self.n_cells, self.n_faces = nc.value, nf.value

    def __del__(self):
        try:
            self._L.ref_destroy(self._h)
        except Exception:
            pass

    def faces(self):
        i5 = np.zeros(5 * self.n_faces, np.int32)
        d5 = np.zeros(5 * self.n_faces)
        self._L.ref_faces(self._h, i5, d5)
        return i5.reshape(-1, 5), d5.reshape(-1, 5)

    def cells(self):
        d = np.zeros(3 * self.n_cells)
        self._L.ref_cells(self._h, d)
        return d.reshape(-1, 3)

    def setNumericalMethod(self, flux, spatial):
        self._L.ref_set_method(self._h, FLUX[flux], SPATIAL[spatial])

    def setFlowConditions(self, M, P, T):
        self._L.ref_set_flow_conditions(self._h, M, P, T)

    def setFreestreamStatic(self, M, P, T):
        self._L.ref_set_freestream_static(self._h, M, P, T)

    def setKinematicViscosity(self, Re, L):
        self._L.ref_set_kinematic_viscosity(self._h, Re, L)

    def params(self):
        o = np.zeros(6)
        self._L.ref_get_params(self._h, o)
        return dict(zip(["M_inf", "P0", "T0", "Pexit", "nu", "R_gas"], o))

    def initialize(self):
        self._L.ref_initialize(self._h)

    def set_state(self, U):
        self._L.ref_set_state(self._h, np.ascontiguousarray(U, np.float64).ravel())

    def get_state(self):
        U = np.zeros(6 * self.n_cells)
        self._L.ref_get_state(self._h, U)
        return U.reshape(-1, 6)

    def residual(self, U, update_limiters=True):
        R = np.zeros(6 * self.n_cells)
        self._L.ref_residual(self._h, np.ascontiguousarray(U, np.float64).ravel(), R, int(update_limiters))
        return R.reshape(-1, 6)

    def gradients(self, U):
        g = np.zeros(10 * self.n_cells)
        self._L.ref_gradients(self._h, np.ascontiguousarray(U, np.float64).ravel(), g)
        return g.reshape(-1, 10)

    def limiters(self, U):
        p = np.zeros(self.n_cells)
        self._L.ref_limiters(self._h, np.ascontiguousarray(U, np.float64).ravel(), p)
        return p

    def get_limiters(self):
        p = np.zeros(self.n_cells)
        self._L.ref_get_limiters(self._h, p)
        return p

    def set_limiters(self, phi):
        self._L.ref_set_limiters(self._h, np.ascontiguousarray(phi, np.float64))

    def local_timestep(self, cfl):
        dt = np.zeros(self.n_cells)
        self._L.ref_local_timestep(self._h, float(cfl), dt)
        return dt

    def preconditioner(self):
        D = np.zeros(self.n_cells)
        self._L.ref_preconditioner(self._h, D)
        return D

    def apply_jacobian(self, Ub, Rb, v):
        J = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        self._L.ref_apply_jacobian(self._h, c(Ub), c(Rb), c(v), J)
        return J.reshape(-1, 6)

    def gmres(self, Ub, Rb, rhs):
        x = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        it = self._L.ref_gmres(self._h, c(Ub), c(Rb), c(rhs), x)
        return it, x.reshape(-1, 6)

    def norm_vm(self, R):
        return self._L.ref_norm_vm(self._h, np.ascontiguousarray(R, np.float64).ravel())

    def solveImplicit(self, tol, max_steps):
        a, b, c = np.zeros(max_steps), np.zeros(max_steps), np.zeros(max_steps)
        it = np.zeros(max_steps, np.int32)
        n = self._L.ref_solve_implicit(self._h, float(tol), int(max_steps), a, b, c, it)
        return {"res_vm": a[:n], "res_abs": b[:n], "cfl": c[:n], "gmres_iters": it[:n]}

    def wall_distance(self):
        d = np.zeros(self.n_cells)
        self._L.ref_wall_distance(self._h, d)
        return d

    def drag(self):
        return self._L.ref_drag(self._h)

    def entropy_error(self):
        return self._L.ref_entropy_error(self._h)

    def skin_friction(self, path):
        """(x, Cf) rows of the reference's skin-friction CSV (sorted by x, 6 digits)."""
        cap = self.n_faces
        x, cf = np.zeros(cap), np.zeros(cap)
        n = self._L.ref_skin_friction(self._h, str(path).encode(), x, cf, cap)
        return x[:n], cf[:n]

    def timeStepExplicit(self, dt):
        self._L.ref_time_step_explicit(self._h, float(dt))

    def solveUnsteady(self, dt_phy, max_time_steps):
        self._L.ref_solve_unsteady(self._h, float(dt_phy), int(max_time_steps))
