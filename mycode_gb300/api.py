"""Python front-end of libcfdgpu (ctypes over the C ABI in include/cfdg.h).

Mirrors the reference's class surface so drivers and tests read like the
reference's own code: ``Mesh.load`` / faces / cells (include/Mesh.hpp) and
``Solver`` with setNumericalMethod, setFlowConditions, setFreestreamStatic,
setKinematicViscosity, initialize, computeResiduals, solveImplicit, getSolution
(include/Solver.hpp).  States and residuals are numpy arrays in the reference's
AoS layout: shape (n_cells, 6), columns rho, rhou, rhov, rhoE, rhok, rhow, cells in
the order the mesh was given.

There is no CPU path: every compute call runs the CUDA kernels and raises
:class:`CfdgError` when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcfdgpu.so")

FLUX = {"LLF": 0, "ROE": 1, "HLLC": 2, "AUSM": 3}
SPATIAL = {"FIRST_ORDER": 0, "SECOND_ORDER_CENTRAL": 1, "SECOND_ORDER_LIMITED": 2}
BCSET = {"bump": 0, "supersonic": 1, "plate": 2}
INIT = {"bump": 0, "freestream": 1}
PRECISION = {"fp64": 0, "mixed": 1}
JV = {"fd": 0, "exact": 1}
RENUMBER = {"none": 0, "hilbert": 1, "rcm": 2}
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_NAN", 4: "ERR_NOT_CONVERGED", 5: "ERR_TIMEOUT",
          6: "ERR_MESH", 7: "ERR_UNSUPPORTED"}


class CfdgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [
        ("flux", C.c_int), ("spatial", C.c_int), ("bcset", C.c_int), ("init", C.c_int),
        ("viscous", C.c_int), ("turbulence", C.c_int), ("precision", C.c_int), ("jv", C.c_int),
        ("gmres_m", C.c_int), ("gmres_tol", C.c_double), ("gamma", C.c_double), ("R_gas", C.c_double),
        ("Pr", C.c_double), ("nu", C.c_double), ("cfl0", C.c_double), ("cfl_max", C.c_double),
        ("limiter_freeze_step", C.c_int), ("limiter_freeze_cfl", C.c_double),
        ("turb_intensity", C.c_double), ("mut_ratio", C.c_double), ("shock_deflection_deg", C.c_double),
        ("renumber", C.c_int), ("device", C.c_int), ("krylov", C.c_int), ("persistent", C.c_int), ("pdl", C.c_int),
        ("barrier_poll_limit", C.c_int), ("newton_chain", C.c_int), ("startup_first_order", C.c_int),
        ("update_limit", C.c_double), ("gather_split_cells", C.c_int),
    ]


class Step(C.Structure):
    _fields_ = [("res_vm", C.c_double), ("res_abs", C.c_double), ("res_rho", C.c_double),
                ("cfl", C.c_double), ("gmres_iters", C.c_int), ("limiter_updated", C.c_int),
                ("seconds", C.c_double), ("device_ms", C.c_double), ("krylov_ms", C.c_double)]


_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def _opt_dp(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))


SIGNATURES = {
    "cfdg_version": (C.c_char_p, []),
    "cfdg_last_error": (C.c_char_p, []),
    "cfdg_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "cfdg_config_default": (None, [C.POINTER(Config)]),
    "cfdg_mesh_create": (C.c_int, [C.c_int, _dp, C.c_int, _ip, C.c_int, _vp, C.c_int, C.POINTER(_vp)]),
    "cfdg_mesh_load_gmsh": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(_vp)]),
    "cfdg_mesh_create_gpu": (C.c_int, [C.c_int, _dp, C.c_int, _ip, C.c_int, _vp, C.c_int, C.c_int, C.POINTER(_vp)]),
    "cfdg_mesh_sizes": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cfdg_mesh_faces": (C.c_int, [_vp, _ip, _dp]),
    "cfdg_mesh_cells": (C.c_int, [_vp, _dp]),
    "cfdg_mesh_permutation": (C.c_int, [_vp, _ip, _ip]),
    "cfdg_mesh_destroy": (None, [_vp]),
    "cfdg_solver_create": (C.c_int, [_vp, C.POINTER(Config), C.POINTER(_vp)]),
    "cfdg_solver_destroy": (None, [_vp]),
    "cfdg_set_numerical_method": (C.c_int, [_vp, C.c_int, C.c_int]),
    "cfdg_set_flow_conditions": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double]),
    "cfdg_set_freestream_static": (C.c_int, [_vp, C.c_double, C.c_double, C.c_double]),
    "cfdg_set_kinematic_viscosity": (C.c_int, [_vp, C.c_double, C.c_double]),
    "cfdg_initialize": (C.c_int, [_vp]),
    "cfdg_get_params": (C.c_int, [_vp, _dp]),
    "cfdg_set_state": (C.c_int, [_vp, _dp]),
    "cfdg_get_state": (C.c_int, [_vp, _dp]),
    "cfdg_residual": (C.c_int, [_vp, C.c_void_p, _dp, C.c_int]),
    "cfdg_gradients": (C.c_int, [_vp, C.c_void_p, _dp]),
    "cfdg_limiters": (C.c_int, [_vp, C.c_void_p, _dp]),
    "cfdg_get_limiters": (C.c_int, [_vp, _dp]),
    "cfdg_set_limiters": (C.c_int, [_vp, _dp]),
    "cfdg_local_timestep": (C.c_int, [_vp, C.c_double, C.c_void_p]),
    "cfdg_set_timestep": (C.c_int, [_vp, _dp]),
    "cfdg_preconditioner": (C.c_int, [_vp, _dp]),
    "cfdg_jv": (C.c_int, [_vp, _dp, C.c_void_p, _dp, _dp, C.c_int]),
    "cfdg_gmres": (C.c_int, [_vp, C.c_void_p, C.c_void_p, _dp, _dp, C.POINTER(C.c_int)]),
    "cfdg_norm_vm": (C.c_int, [_vp, _dp, C.POINTER(C.c_double)]),
    "cfdg_solve_implicit": (C.c_int, [_vp, C.c_double, C.c_int, C.POINTER(Step), C.POINTER(C.c_int)]),
    "cfdg_newton_step": (C.c_int, [_vp, C.c_double, C.POINTER(Step), C.POINTER(C.c_int)]),
    "cfdg_newton_steps": (C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.c_void_p, C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    "cfdg_reset_newton": (C.c_int, [_vp]),
    "cfdg_get_newton_state": (C.c_int, [_vp, C.POINTER(C.c_double), C.POINTER(C.c_int)]),
    "cfdg_set_newton_state": (C.c_int, [_vp, C.c_double, C.c_int]),
    "cfdg_set_cfl_max": (C.c_int, [_vp, C.c_double]),
    "cfdg_fp64_pipe_rate": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "cfdg_set_krylov": (C.c_int, [_vp, C.c_int]),
    "cfdg_vjp": (C.c_int, [_vp, C.c_void_p, _dp, _dp]),
    "cfdg_wall_coefficients": (C.c_int, [_vp, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int)]),
    "cfdg_wall_distance": (C.c_int, [_vp, C.c_void_p]),
    "cfdg_residual32": (C.c_int, [_vp, C.c_void_p, _dp]),
    "cfdg_time_step_explicit": (C.c_int, [_vp, C.c_double, C.POINTER(C.c_double)]),
    "cfdg_solve_unsteady": (C.c_int, [_vp, C.c_double, C.c_int, C.c_void_p, C.c_void_p]),
    "cfdg_jv32": (C.c_int, [_vp, _dp, _dp, _dp]),
    "cfdg_objective": (C.c_int, [_vp, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.c_void_p]),
    "cfdg_drag": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "cfdg_entropy_error": (C.c_int, [_vp, C.POINTER(C.c_double)]),
    "cfdg_residual_device": (C.c_int, [_vp, C.c_int]),
    "cfdg_vjp_device": (C.c_int, [_vp]),
    "cfdg_synchronize": (C.c_int, [_vp]),
    "cfdg_set_timing": (C.c_int, [_vp, C.c_int]),
    "cfdg_kernel_times": (C.c_int, [_vp] + [C.POINTER(C.c_double)] * 4),
    "cfdg_kernel_stats": (C.c_int, [_vp, _dp, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS"), C.c_int]),
    "cfdg_flush_l2": (C.c_int, [_vp, C.c_size_t]),
    "cfdg_launch_count": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "cfdg_krylov_info": (C.c_int, [_vp, np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]),
    "cfdg_norm_vm_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_void_p, C.c_void_p]),
}


def lib():
    """The loaded libcfdgpu.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CfdgError(2, f"{LIB_PATH} is missing: build it with mycode_gb300.build.build() "
                               "(this package has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(st: int):
    if st != 0:
        raise CfdgError(st, lib().cfdg_last_error().decode())


def device_count() -> int:
    n = C.c_int(0)
    _check(lib().cfdg_device_count(C.byref(n)))
    return n.value


def fp64_pipe_rate(device: int = 0) -> float:
    """Thread-level FP64 FMAs per second of the device's FP64 pipe (a live measurement)."""
    r = C.c_double(0.0)
    _check(lib().cfdg_fp64_pipe_rate(int(device), C.byref(r)))
    return r.value


def default_config(**overrides) -> Config:
    c = Config()
    lib().cfdg_config_default(C.byref(c))
    for k, v in overrides.items():
        if k == "flux" and isinstance(v, str):
            v = FLUX[v]
        elif k == "spatial" and isinstance(v, str):
            v = SPATIAL[v]
        elif k == "bcset" and isinstance(v, str):
            v = BCSET[v]
        elif k == "init" and isinstance(v, str):
            v = INIT[v]
        elif k == "precision" and isinstance(v, str):
            v = PRECISION[v]
        elif k == "jv" and isinstance(v, str):
            v = JV[v]
        elif k == "renumber" and isinstance(v, str):
            v = RENUMBER[v]
        elif k == "turbulence" and isinstance(v, str):
            v = {"none": 0, "sst": 1}[v]
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


class Mesh:
    """Mesh::load / buildConnectivity / computeGeometry (src/Mesh.cpp:10-201), renumbered for the GPU."""

    def __init__(self, handle):
        self._h = handle
        nc, nf, nb = C.c_int(), C.c_int(), C.c_int()
        _check(lib().cfdg_mesh_sizes(self._h, C.byref(nc), C.byref(nf), C.byref(nb)))
        self.n_cells, self.n_faces, self.n_boundary_faces = nc.value, nf.value, nb.value

    @classmethod
    def from_spec(cls, spec, renumber="hilbert", gpu=None) -> "Mesh":
        """The mesh of a spec; gpu = a device ordinal builds it with kernels on that GPU
        (cfdg_mesh_create_gpu, the same mesh bit for bit), None on the host."""
        xy = np.ascontiguousarray(spec.nodes, dtype=np.float64).ravel()
        cells = np.ascontiguousarray(spec.cells, dtype=np.int32).ravel()
        bed = np.ascontiguousarray(spec.bedges, dtype=np.int32).ravel()
        h = _vp()
        ren = RENUMBER[renumber] if isinstance(renumber, str) else int(renumber)
        bptr = bed.ctypes.data_as(_vp) if bed.size else None
        if gpu is None:
            _check(lib().cfdg_mesh_create(spec.n_nodes, xy, spec.n_cells, cells, spec.bedges.shape[0], bptr, ren,
                                          C.byref(h)))
        else:
            _check(lib().cfdg_mesh_create_gpu(spec.n_nodes, xy, spec.n_cells, cells, spec.bedges.shape[0], bptr, ren,
                                              int(gpu), C.byref(h)))
        m = cls(h)
        m._keep = (xy, cells, bed)
        return m

    @classmethod
    def load(cls, path: str, renumber="hilbert") -> "Mesh":
        h = _vp()
        _check(lib().cfdg_mesh_load_gmsh(path.encode(), RENUMBER[renumber] if isinstance(renumber, str)
                                         else int(renumber), C.byref(h)))
        return cls(h)

    def faces(self):
        i5 = np.zeros(5 * self.n_faces, np.int32)
        d5 = np.zeros(5 * self.n_faces)
        _check(lib().cfdg_mesh_faces(self._h, i5, d5))
        return i5.reshape(-1, 5), d5.reshape(-1, 5)

    def cells(self):
        d = np.zeros(3 * self.n_cells)
        _check(lib().cfdg_mesh_cells(self._h, d))
        return d.reshape(-1, 3)

    def permutation(self):
        cp = np.zeros(self.n_cells, np.int32)
        fp = np.zeros(self.n_faces, np.int32)
        _check(lib().cfdg_mesh_permutation(self._h, cp, fp))
        return cp, fp

    def __del__(self):
        try:
            lib().cfdg_mesh_destroy(self._h)
        except Exception:
            pass


class Solver:
    """The GPU solver with the reference Solver's method names (include/Solver.hpp:26-66)."""

    def __init__(self, mesh: Mesh, config: Config | None = None, **overrides):
        self.mesh = mesh
        cfg = config if config is not None else default_config(**overrides)
        if config is not None:
            for k, v in overrides.items():
                setattr(cfg, k, v)
        self.config = cfg
        h = _vp()
        _check(lib().cfdg_solver_create(mesh._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self.n_cells = mesh.n_cells

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().cfdg_solver_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def close(self):
        self.__del__()

    # ---- configuration (Solver setters)
    def setNumericalMethod(self, flux, spatial):
        _check(lib().cfdg_set_numerical_method(self._h, FLUX[flux] if isinstance(flux, str) else flux,
                                               SPATIAL[spatial] if isinstance(spatial, str) else spatial))

    def setFlowConditions(self, M, P, T):
        _check(lib().cfdg_set_flow_conditions(self._h, M, P, T))

    def setFreestreamStatic(self, M, P, T):
        _check(lib().cfdg_set_freestream_static(self._h, M, P, T))

    def setKinematicViscosity(self, Re, L):
        _check(lib().cfdg_set_kinematic_viscosity(self._h, Re, L))

    def initialize(self):
        _check(lib().cfdg_initialize(self._h))

    def params(self):
        o = np.zeros(6)
        _check(lib().cfdg_get_params(self._h, o))
        return dict(zip(["M_inf", "P0", "T0", "Pexit", "nu", "R_gas"], o))

    # ---- state
    def set_state(self, U):
        _check(lib().cfdg_set_state(self._h, np.ascontiguousarray(U, np.float64).ravel()))

    def getSolution(self, out=None):
        """The state in the reference's AoS layout (n_cells x 6); into ``out`` (a C-contiguous
        float64 array of that size, e.g. pinned host memory) when given."""
        if out is None:
            U = np.zeros(6 * self.n_cells)
            _check(lib().cfdg_get_state(self._h, U))
            return U.reshape(-1, 6)
        if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != 6 * self.n_cells:
            raise ValueError("getSolution: out must be a C-contiguous float64 array of n_cells x 6")
        _check(lib().cfdg_get_state(self._h, out.reshape(-1)))
        return out

    get_state = getSolution

    # ---- residual path
    def computeResiduals(self, U=None, update_limiters=True, out=None):
        """R(U) in the reference's AoS layout; into ``out`` (a C-contiguous float64 array of
        n_cells x 6, e.g. pinned host memory) when given."""
        if out is None:
            R = np.zeros(6 * self.n_cells)
        else:
            if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != 6 * self.n_cells:
                raise ValueError("computeResiduals: out must be a C-contiguous float64 array of n_cells x 6")
            R = out.reshape(-1)
        u = None if U is None else np.ascontiguousarray(U, np.float64).ravel()
        _check(lib().cfdg_residual(self._h, None if u is None else u.ctypes.data_as(_vp), R, int(update_limiters)))
        return R.reshape(-1, 6)

    residual = computeResiduals

    def gradients(self, U=None):
        g = np.zeros(10 * self.n_cells)
        u = None if U is None else np.ascontiguousarray(U, np.float64).ravel()
        _check(lib().cfdg_gradients(self._h, None if u is None else u.ctypes.data_as(_vp), g))
        return g.reshape(-1, 10)

    def limiters(self, U=None):
        p = np.zeros(self.n_cells)
        u = None if U is None else np.ascontiguousarray(U, np.float64).ravel()
        _check(lib().cfdg_limiters(self._h, None if u is None else u.ctypes.data_as(_vp), p))
        return p

    def get_limiters(self):
        p = np.zeros(self.n_cells)
        _check(lib().cfdg_get_limiters(self._h, p))
        return p

    def set_limiters(self, phi):
        _check(lib().cfdg_set_limiters(self._h, np.ascontiguousarray(phi, np.float64)))

    def local_timestep(self, cfl):
        dt = np.zeros(self.n_cells)
        _check(lib().cfdg_local_timestep(self._h, float(cfl), dt.ctypes.data_as(_vp)))
        return dt

    def set_dt(self, dt):
        _check(lib().cfdg_set_timestep(self._h, np.ascontiguousarray(dt, np.float64)))

    def preconditioner(self):
        D = np.zeros(self.n_cells)
        _check(lib().cfdg_preconditioner(self._h, D))
        return D

    def apply_jacobian(self, Ub, Rb, v, mode="fd"):
        J = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        rb = None if Rb is None else c(Rb)
        _check(lib().cfdg_jv(self._h, c(Ub), None if rb is None else rb.ctypes.data_as(_vp), c(v), J,
                             JV[mode] if isinstance(mode, str) else mode))
        return J.reshape(-1, 6)

    def residual32(self, U=None):
        """FP32 residual (mixed-precision solvers), widened to FP64 AoS."""
        R = np.zeros(6 * self.n_cells)
        u = None if U is None else np.ascontiguousarray(U, np.float64).ravel()
        _check(lib().cfdg_residual32(self._h, None if u is None else u.ctypes.data_as(_vp), R))
        return R.reshape(-1, 6)

    def apply_jacobian32(self, Ub, v):
        """FP32 exact J v (mixed-precision solvers), widened to FP64 AoS."""
        J = np.zeros(6 * self.n_cells)
        c = lambda a: np.ascontiguousarray(a, np.float64).ravel()
        _check(lib().cfdg_jv32(self._h, c(Ub), c(v), J))
        return J.reshape(-1, 6)

    def gmres(self, Ub, Rb, rhs):
        x = np.zeros(6 * self.n_cells)
        c = lambda a: None if a is None else np.ascontiguousarray(a, np.float64).ravel()
        ub, rb = c(Ub), c(Rb)
        it = C.c_int(0)
        _check(lib().cfdg_gmres(self._h, None if ub is None else ub.ctypes.data_as(_vp),
                                None if rb is None else rb.ctypes.data_as(_vp), c(rhs), x, C.byref(it)))
        return it.value, x.reshape(-1, 6)

    def norm_vm(self, R):
        o = C.c_double()
        _check(lib().cfdg_norm_vm(self._h, np.ascontiguousarray(R, np.float64).ravel(), C.byref(o)))
        return o.value

    def solveImplicit(self, tol=1e-6, max_steps=50, raise_on_nonconvergence=False):
        tr = (Step * max(max_steps, 1))()
        n = C.c_int(0)
        st = lib().cfdg_solve_implicit(self._h, float(tol), int(max_steps), tr, C.byref(n))
        if st != 0 and not (st == 4 and not raise_on_nonconvergence):
            _check(st)
        recs = tr[: n.value]
        return {
            "res_vm": np.array([r.res_vm for r in recs]),
            "res_abs": np.array([r.res_abs for r in recs]),
            "res_rho": np.array([r.res_rho for r in recs]),
            "cfl": np.array([r.cfl for r in recs]),
            "gmres_iters": np.array([r.gmres_iters for r in recs], dtype=np.int32),
            "seconds": np.array([r.seconds for r in recs]),
            "device_ms": np.array([r.device_ms for r in recs]),
            "krylov_ms": np.array([r.krylov_ms for r in recs]),
            "converged": st == 0,
        }

    def timeStepExplicit(self, dt):
        """Solver::timeStepExplicit: returns norm_L2 of the residual the step used."""
        r = C.c_double()
        _check(lib().cfdg_time_step_explicit(self._h, float(dt), C.byref(r)))
        return r.value

    def solveUnsteady(self, dt_phy, max_time_steps):
        """Solver::solveUnsteady: per physical step the Newton steps taken and the last
        residual."""
        n = int(max_time_steps)
        it = np.zeros(max(n, 1), np.int32)
        res = np.zeros(max(n, 1))
        _check(lib().cfdg_solve_unsteady(self._h, float(dt_phy), n, it.ctypes.data_as(_vp), res.ctypes.data_as(_vp)))
        return {"newton_steps": it[:n], "res_vm": res[:n]}

    def newton_step(self, tol=0.0):
        s = Step()
        cv = C.c_int(0)
        _check(lib().cfdg_newton_step(self._h, float(tol), C.byref(s), C.byref(cv)))
        return s, bool(cv.value)

    def newton_steps(self, k, tol=0.0, tol_rho=0.0):
        """k Newton steps enqueued back to back (graph driver: one host synchronisation),
        stopping at res_vm < tol or (tol_rho > 0) a density residual <= tol_rho after step 5;
        returns (records of the steps taken, converged)."""
        tr = (Step * max(int(k), 1))()
        n, cv = C.c_int(0), C.c_int(0)
        _check(lib().cfdg_newton_steps(self._h, float(tol), float(tol_rho), int(k), C.cast(tr, C.c_void_p), C.byref(n),
                                       C.byref(cv)))
        return list(tr[: n.value]), bool(cv.value)

    def set_krylov(self, mode):
        _check(lib().cfdg_set_krylov(self._h, {"host": 0, "graph": 1, "stream": 2}.get(mode, mode)))

    def reset_newton(self):
        _check(lib().cfdg_reset_newton(self._h))

    def newton_state(self):
        """(CFL, step) of the pseudo-transient driver."""
        c, n = C.c_double(), C.c_int()
        _check(lib().cfdg_get_newton_state(self._h, C.byref(c), C.byref(n)))
        return c.value, n.value

    def set_newton_state(self, cfl, step):
        _check(lib().cfdg_set_newton_state(self._h, float(cfl), int(step)))

    def set_cfl_max(self, cfl_max):
        """The pseudo-transient control's CFL cap, from the next Newton step on."""
        _check(lib().cfdg_set_cfl_max(self._h, float(cfl_max)))

    def vjp(self, lam, U=None):
        g = np.zeros(6 * self.n_cells)
        u = None if U is None else np.ascontiguousarray(U, np.float64).ravel()
        _check(lib().cfdg_vjp(self._h, None if u is None else u.ctypes.data_as(_vp),
                              np.ascontiguousarray(lam, np.float64).ravel(), g))
        return g.reshape(-1, 6)

    # ---- device-resident path and instrumentation
    def residual_device(self, update_limiters=True):
        _check(lib().cfdg_residual_device(self._h, int(update_limiters)))

    def vjp_device(self):
        _check(lib().cfdg_vjp_device(self._h))

    def synchronize(self):
        _check(lib().cfdg_synchronize(self._h))

    def set_timing(self, on=True):
        """True: events around every kernel and every Newton step; "steps": around each
        Newton step only; False: off."""
        _check(lib().cfdg_set_timing(self._h, 2 if on == "steps" else int(bool(on))))

    def kernel_times(self):
        v = [C.c_double() for _ in range(4)]
        _check(lib().cfdg_kernel_times(self._h, *[C.byref(x) for x in v]))
        return dict(zip(["prim", "grad", "flux", "gather"], [x.value for x in v]))

    KERNEL_CLASSES = ["residual.prim", "residual.grad", "residual.flux", "residual.gather",
                      "jv.prim", "jv.grad", "jv.flux", "jv.gather",
                      "vjp.forward", "vjp.flux_adj", "vjp.cell1", "vjp.cell2",
                      "krylov.prim_z", "krylov.grad", "krylov.flux", "krylov.gather_dot", "krylov.update_dot",
                      "krylov.update_final"]

    def kernel_stats(self, reset=False):
        ms = np.zeros(len(self.KERNEL_CLASSES))
        n = np.zeros(len(self.KERNEL_CLASSES), np.int64)
        _check(lib().cfdg_kernel_stats(self._h, ms, n, int(reset)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.KERNEL_CLASSES)}

    def flush_l2(self, nbytes=256 << 20):
        _check(lib().cfdg_flush_l2(self._h, int(nbytes)))

    # ---- wall quantities (calculateDrag, extractSkinFriction, calculateEntropyError)
    def wall_coefficients(self, tag=4):
        """x_mid, Cp and Cf of the boundary faces with ``tag``, in reference face order."""
        n = C.c_int(0)
        _check(lib().cfdg_wall_coefficients(self._h, int(tag), None, None, None, C.byref(n)))
        x, cp, cf = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        if n.value:
            _check(lib().cfdg_wall_coefficients(self._h, int(tag), x.ctypes.data_as(_vp), cp.ctypes.data_as(_vp),
                                                cf.ctypes.data_as(_vp), C.byref(n)))
        return x, cp, cf

    def wall_distance(self):
        d = np.zeros(self.n_cells)
        _check(lib().cfdg_wall_distance(self._h, d.ctypes.data_as(_vp)))
        return d

    OBJECTIVES = {"pressure_drag": 0, "skin_friction_drag": 1, "wall_pressure": 2}

    def objective(self, kind, x0=-1e300, x1=1e300, gradient=True):
        """J (and dJ/dU, AoS) of a wall objective: pressure_drag, skin_friction_drag or
        wall_pressure (over tag-4 faces with x0 <= x_mid <= x1)."""
        k = self.OBJECTIVES[kind] if isinstance(kind, str) else int(kind)
        J = C.c_double()
        g = np.zeros(6 * self.n_cells) if gradient else None
        _check(lib().cfdg_objective(self._h, k, float(x0), float(x1), C.byref(J),
                                    g.ctypes.data_as(_vp) if gradient else None))
        return (J.value, g.reshape(-1, 6)) if gradient else J.value

    def drag(self):
        d = C.c_double()
        _check(lib().cfdg_drag(self._h, C.byref(d)))
        return d.value

    def entropy_error(self):
        e = C.c_double()
        _check(lib().cfdg_entropy_error(self._h, C.byref(e)))
        return e.value

    def launch_count(self):
        n = C.c_longlong()
        _check(lib().cfdg_launch_count(self._h, C.byref(n)))
        return n.value

    def krylov_info(self):
        """The Krylov driver in effect: mode, kernels per Arnoldi iteration of the last
        built graph body, programmatic dependent launch in the body, persistent kernel."""
        v = np.zeros(4, np.int32)
        _check(lib().cfdg_krylov_info(self._h, v))
        return {"mode": int(v[0]), "body_kernels": int(v[1]), "pdl": bool(v[2]), "persistent": bool(v[3])}
