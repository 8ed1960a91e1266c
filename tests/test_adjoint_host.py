"""The hand-written adjoint of the face function (mycode_gb300/csrc/adjoint.cuh) against
central differences of the forward face function (face.cuh), both built for the host
from the library's own headers by a test-only harness: every flux scheme, spatial order,
boundary-condition set and tag, with and without the viscous term."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "adjoint_harness", "face_harness.cpp")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("adj") / "face_harness.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", so])
    lib = C.CDLL(so)
    lib.face_eval.argtypes = [_dp, _ip, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, _dp]
    lib.face_adj.argtypes = [_dp, _ip, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
    return lib


def flow_params(M=0.5, P=101325.0, T=300.0, nu=1.5e-3):
    g, Rg = 1.4, 287.0
    fT = 1 + 0.5 * (g - 1) * M * M
    T0, P0 = T * fT, P * fT ** (g / (g - 1))
    rho = P / (Rg * T)
    u = M * np.sqrt(g * Rg * T)
    fs = [rho, rho * u, 0.0, P / (g - 1) + 0.5 * rho * u * u]
    return np.array([g, Rg, 0.72, nu, M, P0, T0, P] + fs + fs, dtype=np.float64)


def state(rng, rho=1.2, u=170.0, v=20.0, p=101325.0, amp=0.1):
    r = rho * (1 + amp * rng.uniform(-1, 1))
    uu = u * (1 + amp * rng.uniform(-1, 1))
    vv = v + amp * u * rng.uniform(-1, 1)
    pp = p * (1 + amp * rng.uniform(-1, 1))
    return np.array([r, r * uu, r * vv, pp / 0.4 + 0.5 * r * (uu * uu + vv * vv), 0.0, 0.0])


def check(lib, p, fl, seed, u=170.0, v=20.0):
    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi)
    g = np.array([np.cos(th), np.sin(th), 0.013, 0.004, -0.003, -0.005, 0.002, -0.009, 0.005])
    UL, UR = state(rng, u=u, v=v), state(rng, u=u, v=v)
    scale = np.array([1.0, 100.0, 100.0, 1e5, 1, 1, 1e3, 1e3, 1e3, 1e3])
    gL = rng.standard_normal(10) * np.array([1, 1, 100, 100, 100, 100, 1e4, 1e4, 10, 10])
    gR = rng.standard_normal(10) * np.array([1, 1, 100, 100, 100, 100, 1e4, 1e4, 10, 10])
    phL, phR = rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9)
    fl = np.asarray(fl, dtype=np.int32)
    lam = rng.standard_normal(6)
    lam[4:] = 0
    out = np.zeros(6)

    def f(UL_, UR_, gL_, gR_, a, b):
        lib.face_eval(p, fl, g, UL_, UR_, gL_, gR_, a, b, out)
        return float(lam @ out)

    ULb, URb, gLb, gRb, phb = np.zeros(6), np.zeros(6), np.zeros(10), np.zeros(10), np.zeros(2)
    lib.face_adj(p, fl, g, UL, UR, gL, gR, phL, phR, lam.copy(), ULb, URb, gLb, gRb, phb)
    base = abs(f(UL, UR, gL, gR, phL, phR)) + 1.0
    gscale = np.array([1, 1, 100, 100, 100, 100, 1e4, 1e4, 10, 10], dtype=float)

    def deriv(fun, x0, h):
        # central differences at h and h/2 combined by Richardson extrapolation
        d1 = (fun(x0 + h) - fun(x0 - h)) / (2 * h)
        d2 = (fun(x0 + h / 2) - fun(x0 - h / 2)) / h
        return (4 * d2 - d1) / 3

    checks = []
    for name, vec, adj, n in (("UL", UL, ULb, 4), ("UR", UR, URb, 4), ("gL", gL, gLb, 10), ("gR", gR, gRb, 10)):
        for k in range(n):
            h = 1e-4 * (abs(vec[k]) + 1e-3) if name.startswith("U") else 1e-3 * gscale[k]

            def fun(x, name=name, k=k):
                v = {"UL": UL, "UR": UR, "gL": gL, "gR": gR}
                w = v[name].copy()
                w[k] = x
                v[name] = w
                return f(v["UL"], v["UR"], v["gL"], v["gR"], phL, phR)

            checks.append((name, k, deriv(fun, vec[k], h), adj[k]))
    checks.append(("phL", 0, deriv(lambda x: f(UL, UR, gL, gR, x, phR), phL, 1e-3), phb[0]))
    checks.append(("phR", 0, deriv(lambda x: f(UL, UR, gL, gR, phL, x), phR, 1e-3), phb[1]))
    for name, k, d, a in checks:
        tol = 1e-6 * (abs(d) + abs(a)) + 1e-10 * base
        assert abs(d - a) <= tol, f"{name}[{k}]: fd {d:.10e} adjoint {a:.10e}"


FLUXES = [0, 1, 2]


@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("spatial", [0, 1, 2])
@pytest.mark.parametrize("viscous", [0, 1])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_interior_face_adjoint(harness, flux, spatial, viscous, seed):
    check(harness, flow_params(), [0, flux, spatial, viscous, 1, 0], seed)


@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("seed", [4, 5])
def test_supersonic_and_reversed_flow(harness, flux, seed):
    # wave-speed branches of HLLC / Roe: supersonic both ways and subsonic reversed
    for u, v in ((600.0, 10.0), (-600.0, 30.0), (-150.0, 60.0), (5.0, 3.0)):
        check(harness, flow_params(M=2.0), [1, flux, 2, 1, 1, 0], seed, u=u, v=v)


@pytest.mark.parametrize("bcset,tags", [(0, [1, 2, 3, 7]), (1, [1, 2, 3, 6, 7]), (2, [1, 2, 3, 4, 5, 7])])
@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("viscous", [0, 1])
def test_boundary_face_adjoint(harness, bcset, tags, flux, viscous):
    for tag in tags:
        for seed in (7, 8):
            check(harness, flow_params(), [bcset, flux, 2, viscous, 0, tag], seed)


# ---------------------------------------------------------------- SST (nv = 6)
def _sst_lib(lib):
    if not getattr(lib, "_sst_ready", False):
        lib.sst_face_eval.argtypes = [_dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, _dp, _dp]
        lib.sst_face_adj.argtypes = [_dp, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, _dp, _dp,
                                     _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        lib.sst_cell_eval.argtypes = [_dp, _dp, _dp]
        lib.sst_cell_adj.argtypes = [_dp, _dp, _dp, _dp]
        lib._sst_ready = True
    return lib


def sst_params(M=0.5, nu=1.5e-3, k_inf=0.2, w_inf=300.0):
    return np.concatenate([flow_params(M=M, nu=nu), [k_inf, w_inf]])


def _deriv(fun, x0, h):
    d1 = (fun(x0 + h) - fun(x0 - h)) / (2 * h)
    d2 = (fun(x0 + h / 2) - fun(x0 - h / 2)) / h
    return (4 * d2 - d1) / 3


def check_sst_cell(lib, seed):
    lib = _sst_lib(lib)
    rng = np.random.default_rng(seed)
    p = sst_params()
    r = 1.2 * (1 + 0.1 * rng.uniform(-1, 1))
    k = 4.0 * (1 + 0.5 * rng.uniform(-1, 1))
    w = 300.0 * (1 + 0.5 * rng.uniform(-1, 1))
    grads = rng.standard_normal(8) * np.array([3e3, 3e3, 3e3, 3e3, 400, 400, 3e4, 3e4])
    d = rng.uniform(0.03, 0.3)
    x = np.concatenate([[r, k, w], grads, [d]])
    lam = rng.standard_normal(4) * np.array([1e3, 1.0, 1e-3, 1e-5])
    out = np.zeros(4)

    def f(xx):
        lib.sst_cell_eval(p, xx, out)
        return float(lam @ out)

    xb = np.zeros(11)
    lib.sst_cell_adj(p, x, lam.copy(), xb)
    base = abs(f(x)) + 1e-300
    for q in range(11):
        h = 1e-4 * (abs(x[q]) + 1e-3)

        def fun(v, q=q):
            y = x.copy()
            y[q] = v
            return f(y)

        dfd = _deriv(fun, x[q], h)
        tol = 1e-6 * (abs(dfd) + abs(xb[q])) + 1e-10 * base / (abs(x[q]) + 1e-3)
        assert abs(dfd - xb[q]) <= tol, f"input {q}: fd {dfd:.10e} adjoint {xb[q]:.10e}"


@pytest.mark.parametrize("seed", range(12))
def test_sst_cell_adjoint(harness, seed):
    check_sst_cell(harness, seed)


def check_sst_face(lib, fl, seed, M=0.5, u=170.0, v=20.0):
    lib = _sst_lib(lib)
    rng = np.random.default_rng(seed)
    p = sst_params(M=M)
    th = rng.uniform(0, 2 * np.pi)
    g = np.array([np.cos(th), np.sin(th), 0.013, 0.004, -0.003, -0.005, 0.002, -0.009, 0.005])
    if not fl[4]:
        g[5:] = 0.0

    def turb(U):
        U = U.copy()
        U[4] = U[0] * 4.0 * (1 + 0.5 * rng.uniform(-1, 1))
        U[5] = U[0] * 300.0 * (1 + 0.5 * rng.uniform(-1, 1))
        return U

    UL, UR = turb(state(rng, u=u, v=v)), turb(state(rng, u=u, v=v))
    gsc = np.array([1, 1, 100, 100, 100, 100, 1e4, 1e4, 10, 10], dtype=float)
    gksc = np.array([400, 400, 3e4, 3e4], dtype=float)
    gL, gR = rng.standard_normal(10) * gsc, rng.standard_normal(10) * gsc
    gkL, gkR = rng.standard_normal(4) * gksc, rng.standard_normal(4) * gksc
    phL, phR = rng.uniform(0.2, 0.9), rng.uniform(0.2, 0.9)
    t = np.array([0.02 * rng.uniform(0.5, 1.5), 0.02 * rng.uniform(0.5, 1.5), rng.uniform(0.2, 0.8),
                  rng.uniform(0.2, 0.8)])
    fl = np.asarray(fl, dtype=np.int32)
    lam = rng.standard_normal(6)
    out = np.zeros(6)
    names = ["UL", "UR", "gL", "gR", "gkL", "gkR", "t"]
    vals = dict(UL=UL, UR=UR, gL=gL, gR=gR, gkL=gkL, gkR=gkR, t=t)

    def f(vv, a=phL, b=phR):
        lib.sst_face_eval(p, fl, g, vv["UL"], vv["UR"], vv["gL"], vv["gR"], vv["gkL"], vv["gkR"], a, b, vv["t"], out)
        return float(lam @ out)

    adj = {k: np.zeros(len(vals[k])) for k in names}
    phb = np.zeros(2)
    lib.sst_face_adj(p, fl, g, UL, UR, gL, gR, gkL, gkR, phL, phR, t, lam.copy(), adj["UL"], adj["UR"], adj["gL"],
                     adj["gR"], adj["gkL"], adj["gkR"], phb, adj["t"])
    base = abs(f(vals)) + 1.0
    scales = dict(gL=gsc, gR=gsc, gkL=gksc, gkR=gksc)
    for name in names:
        for q in range(len(vals[name])):
            x0 = vals[name][q]
            if name in scales:
                h = 1e-3 * scales[name][q]
            elif name == "t":  # the flux is linear in mu_t and F1: a wide step keeps round-off out
                h = 1e-2 * (abs(x0) + 1e-3)
            else:
                h = 1e-4 * (abs(x0) + 1e-3)

            def fun(x, name=name, q=q):
                vv = {k: a.copy() for k, a in vals.items()}
                vv[name][q] = x
                return f(vv)

            dfd = _deriv(fun, x0, h)
            a = adj[name][q]
            tol = 1e-6 * (abs(dfd) + abs(a)) + 1e-10 * base
            assert abs(dfd - a) <= tol, f"{name}[{q}]: fd {dfd:.10e} adjoint {a:.10e}"
    for s_, (dfd, a) in enumerate(((_deriv(lambda x: f(vals, x, phR), phL, 1e-3), phb[0]),
                                   (_deriv(lambda x: f(vals, phL, x), phR, 1e-3), phb[1]))):
        assert abs(dfd - a) <= 1e-6 * (abs(dfd) + abs(a)) + 1e-10 * base, f"phi[{s_}]"


@pytest.mark.parametrize("flux", FLUXES)
@pytest.mark.parametrize("spatial", [0, 1, 2])
@pytest.mark.parametrize("seed", [1, 2])
def test_sst_interior_face_adjoint(harness, flux, spatial, seed):
    check_sst_face(harness, [2, flux, spatial, 1, 1, 0], seed)


@pytest.mark.parametrize("bcset,tags", [(0, [1, 2, 3]), (1, [1, 2, 3, 6]), (2, [1, 2, 3, 4, 5])])
@pytest.mark.parametrize("flux", FLUXES)
def test_sst_boundary_face_adjoint(harness, bcset, tags, flux):
    for tag in tags:
        for seed in (7, 8):
            check_sst_face(harness, [bcset, flux, 2, 1, 0, tag], seed)


def test_shared_reciprocal_quotient_is_the_division(harness):
    """quot_by_recip (Markstein's correction of a * (1/b)), which the FP64 residual uses
    for quotients that share a divisor, gives the bits of a / b: random operands over a wide
    exponent range, divisors with all-ones and near-power-of-two significands, and the
    magnitudes the residual divides (volumes, densities, squared distances)."""
    rng = np.random.default_rng(7)
    n = 400_000
    a = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-300, 300, n)) * rng.choice([-1.0, 1.0], n)
    b = rng.uniform(1.0, 2.0, n) * np.exp2(rng.integers(-60, 60, n))
    b[: n // 8] = np.exp2(rng.integers(-40, 40, n // 8)) * (2.0 - 2.0 ** -52)      # all-ones significands
    b[n // 8: n // 4] = np.exp2(rng.integers(-40, 40, n // 8)) * (1.0 + rng.integers(0, 16, n // 8) * 2.0 ** -52)
    vol = rng.uniform(1e-9, 1e-2, n)
    a2 = rng.standard_normal(n) * 10.0 ** rng.integers(-8, 6, n)
    f = harness.quot_mismatches
    f.restype = C.c_long
    f.argtypes = [C.c_long, C.c_void_p, C.c_void_p]
    for x, y in ((a, b), (a2, vol)):
        x = np.ascontiguousarray(x)
        y = np.ascontiguousarray(y)
        assert f(n, x.ctypes.data, y.ctypes.data) == 0

