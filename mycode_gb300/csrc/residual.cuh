// Residual kernels R(U) = sum_f (+-) F_f A_f on the renumbered SoA mesh.
//
// One evaluation is four launches:
//   k_prim    per cell   W = (rho, u, v, p, T [, k, w])           reads U
//   k_grad    per cell   Green-Gauss gradients + Barth-Jespersen   gathers W over the
//                        limiter, no atomics                      cell's faces
//   k_flux    per face   reconstruction, Riemann flux, viscous    writes F*A per face
//                        flux
//   k_gather  per cell   R_i = sum of +-F*A over the cell's faces in the reference's
//                        face order (deterministic, bit-reproducible)
//
// The kernels are templated on the scalar S: double / float for the residual, and
// Dual<double> / Dual<float> for the exact forward linearisation (J v with the limiter
// frozen), where every array has a value plane and a derivative plane.
#pragma once
#include <cuda_runtime.h>
#include "physics.cuh"

namespace cfdg {

// SoA mesh view; faces [0, nfi) are interior, [nfi, nf) boundary.
template <class R>
struct MeshView {
    int nc, nf, nfi;
    const int* cf;     // [4][nc] per cell: (face << 1) | side, side 1 = cell is the neighbour; -1 pads
    const int* fo;     // [nf] owner cell
    const int* fn;     // [nf] neighbour cell, -1 on the boundary
    const int* ftag;   // [nf] physical tag (0 interior)
    const R* nx;       // [nf] unit normal, owner -> neighbour
    const R* ny;
    const R* area;
    const R* dxo;      // [nf] face midpoint minus owner centroid
    const R* dyo;
    const R* dxn;      // [nf] face midpoint minus neighbour centroid (0 on the boundary)
    const R* dyn;
    const R* dxlr;     // [nf] neighbour centroid minus owner centroid (0 on the boundary)
    const R* dylr;
    const R* vol;      // [nc]
};

// A field of `planes` SoA planes of length n: value planes v and, for Dual kernels,
// derivative planes d (nullptr for real-valued kernels).
template <class R>
struct Field {
    R* v;
    R* d;
    long n;
};

template <class S> struct Acc;
template <> struct Acc<double> {
    template <class R> static CFD_HD double ld(const Field<R>& f, int p, long i) { return f.v[p * f.n + i]; }
    template <class R> static CFD_HD void st(const Field<R>& f, int p, long i, double x) { f.v[p * f.n + i] = x; }
};
template <> struct Acc<float> {
    template <class R> static CFD_HD float ld(const Field<R>& f, int p, long i) { return f.v[p * f.n + i]; }
    template <class R> static CFD_HD void st(const Field<R>& f, int p, long i, float x) { f.v[p * f.n + i] = x; }
};
template <class R> struct Acc<Dual<R>> {
    static CFD_HD Dual<R> ld(const Field<R>& f, int p, long i) {
        return Dual<R>(f.v[p * f.n + i], f.d ? f.d[p * f.n + i] : R(0));
    }
    static CFD_HD void st(const Field<R>& f, int p, long i, Dual<R> x) {
        if (f.v) f.v[p * f.n + i] = x.v;
        f.d[p * f.n + i] = x.d;
    }
};

// primitive planes
enum { W_R = 0, W_U = 1, W_V = 2, W_P = 3, W_T = 4, W_K = 5, W_W = 6 };
// gradient planes, (x, y) pairs in CellGradient member order (include/Solver.hpp:13-24)
enum { G_R = 0, G_U = 2, G_V = 4, G_P = 6, G_T = 8, G_K = 10, G_W = 12 };

template <int NV> struct Planes {
    static constexpr int W = NV == 6 ? 7 : 5;
    static constexpr int G = NV == 6 ? 14 : 10;
};

template <class S, int NV, class R>
__device__ __forceinline__ CS<S> load_cs(const Field<R>& U, const Field<R>& W, long i) {
    CS<S> c;
    c.r = Acc<S>::ld(U, 0, i);
    c.ru = Acc<S>::ld(U, 1, i);
    c.rv = Acc<S>::ld(U, 2, i);
    c.rE = Acc<S>::ld(U, 3, i);
    if (NV == 6) {
        c.rk = Acc<S>::ld(U, 4, i);
        c.rw = Acc<S>::ld(U, 5, i);
    } else {
        c.rk = S(R(0));
        c.rw = S(R(0));
    }
    c.u = Acc<S>::ld(W, W_U, i);
    c.v = Acc<S>::ld(W, W_V, i);
    c.p = Acc<S>::ld(W, W_P, i);
    return c;
}

// ---------------------------------------------------------------- k_prim
// u, v, p, T as the reference computes them per face (src/Solver.cpp:93-102).
template <class S, int NV, class R>
__global__ void __launch_bounds__(256) k_prim(int nc, Flow<R> F, Field<R> U, Field<R> W) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    S r = Acc<S>::ld(U, 0, i), ru = Acc<S>::ld(U, 1, i), rv = Acc<S>::ld(U, 2, i), rE = Acc<S>::ld(U, 3, i);
    S u = ru / r, v = rv / r;
    S p = pressure(F, r, ru, rv, rE);
    S T = p / (r * F.Rgas);
    Acc<S>::st(W, W_R, i, r);
    Acc<S>::st(W, W_U, i, u);
    Acc<S>::st(W, W_V, i, v);
    Acc<S>::st(W, W_P, i, p);
    Acc<S>::st(W, W_T, i, T);
    if (NV == 6) {
        Acc<S>::st(W, W_K, i, Acc<S>::ld(U, 4, i) / r);
        Acc<S>::st(W, W_W, i, Acc<S>::ld(U, 5, i) / r);
    }
}

// ---------------------------------------------------------------- k_grad
// computeGradients (src/Solver.cpp:81-149) as a per-cell gather over the cell's faces
// in reference face order, then (limited scheme, limiter not frozen) computeLimiters
// (src/Solver.cpp:152-253) for the same cell from its own fresh gradient.
template <class S, int NV, class R>
__global__ void __launch_bounds__(256) k_grad(MeshView<R> m, Flow<R> F, Field<R> U, Field<R> W, Field<R> G,
                                              R* phi, int do_limiter) {
    constexpr int NQ = NV == 6 ? 7 : 5;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    S wi[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) wi[q] = Acc<S>::ld(W, q, i);
    S acc[2 * NQ];
#pragma unroll
    for (int q = 0; q < 2 * NQ; ++q) acc[q] = S(R(0));
    R pmax = val(wi[W_P]), pmin = val(wi[W_P]);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * m.nc + i];
        if (e < 0) break;
        int f = e >> 1, side = e & 1;
        R nx = m.nx[f], ny = m.ny[f], A = m.area[f];
        S wj[NQ];
        int j = side ? m.fo[f] : m.fn[f];
        if (j >= 0) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) wj[q] = Acc<S>::ld(W, q, j);
        } else {
            CS<S> Ui = load_cs<S, NV>(U, W, i);
            CS<S> g = ghost_state(F, Ui, m.ftag[f], nx, ny);
            wj[W_R] = g.r;
            wj[W_U] = g.u;
            wj[W_V] = g.v;
            wj[W_P] = g.p;
            wj[W_T] = g.p / (g.r * F.Rgas);
            if (NV == 6) {
                wj[W_K] = g.rk / g.r;
                wj[W_W] = g.rw / g.r;
            }
        }
        pmax = smax(pmax, val(wj[W_P]));
        pmin = smin(pmin, val(wj[W_P]));
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            S ph = R(0.5) * (wi[q] + wj[q]);
            S tx = ph * nx * A, ty = ph * ny * A;
            if (side) {
                acc[2 * q] = acc[2 * q] - tx;
                acc[2 * q + 1] = acc[2 * q + 1] - ty;
            } else {
                acc[2 * q] = acc[2 * q] + tx;
                acc[2 * q + 1] = acc[2 * q + 1] + ty;
            }
        }
    }
    R vol = m.vol[i];
    // gradient planes are in CellGradient order rho, u, v, p, T (= primitive order)
#pragma unroll
    for (int q = 0; q < 2 * NQ; ++q) {
        acc[q] = acc[q] / vol;
        Acc<S>::st(G, q, i, acc[q]);
    }
    if (!do_limiter) return;
    // Barth-Jespersen on pressure reconstructed through T; one phi per cell
    const R eps = R(1e-12);
    R pc = val(wi[W_P]);
    R rho = val(wi[W_R]);
    R Tc = val(wi[W_T]);
    R gTx = val(acc[G_T]), gTy = val(acc[G_T + 1]);
    R lim = R(1.0);
#pragma unroll 1
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * m.nc + i];
        if (e < 0) break;
        int f = e >> 1, side = e & 1;
        R dx = side ? m.dxn[f] : m.dxo[f];
        R dy = side ? m.dyn[f] : m.dyo[f];
        R Tf = Tc + R(1.0) * (gTx * dx + gTy * dy);
        R Pf = rho * F.Rgas * Tf;
        R d2 = Pf - pc;
        R a = R(1.0);
        if (d2 > R(0.0)) {
            a = (pmax - pc) / (d2 + eps);
            a = smin(R(1.0), a);
        } else if (d2 < R(0.0)) {
            a = (pmin - pc) / (d2 - eps);
            a = smin(R(1.0), a);
        }
        lim = smin(lim, a);
    }
    phi[i] = lim;
}

// ---------------------------------------------------------------- k_flux
// The face loop of computeResiduals (src/Solver.cpp:543-800): reconstruction, the
// wall pressure flux or the Riemann flux, and (viscous) the Navier-Stokes flux from
// averaged and corrected cell gradients.  Writes F*A per face.
template <class S, int NV, class R>
__global__ void __launch_bounds__(256) k_flux(MeshView<R> m, Flow<R> F, Field<R> U, Field<R> W, Field<R> G,
                                              const R* __restrict__ phi, Field<R> FA) {
    long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    int o = m.fo[f], n = m.fn[f];
    R nx = m.nx[f], ny = m.ny[f], A = m.area[f];
    int tag = n >= 0 ? 0 : m.ftag[f];
    CS<S> L = load_cs<S, NV>(U, W, o);
    CS<S> Rt = n >= 0 ? load_cs<S, NV>(U, W, n) : ghost_state(F, L, tag, nx, ny);
    CS<S> Lr = L, Rr = Rt;
    if (F.spatial != SP_FIRST && n >= 0) {
        R dxL = m.dxo[f], dyL = m.dyo[f], dxR = m.dxn[f], dyR = m.dyn[f];
        S phL = F.spatial == SP_LIMITED ? S(phi[o]) : S(R(0.5));
        S phR = F.spatial == SP_LIMITED ? S(phi[n]) : S(R(0.5));
        S rLf = L.r + phL * (Acc<S>::ld(G, G_R, o) * dxL + Acc<S>::ld(G, G_R + 1, o) * dyL);
        S pLf = L.p + phL * (Acc<S>::ld(G, G_P, o) * dxL + Acc<S>::ld(G, G_P + 1, o) * dyL);
        S uLf = L.u + phL * (Acc<S>::ld(G, G_U, o) * dxL + Acc<S>::ld(G, G_U + 1, o) * dyL);
        S vLf = L.v + phL * (Acc<S>::ld(G, G_V, o) * dxL + Acc<S>::ld(G, G_V + 1, o) * dyL);
        if (val(rLf) < R(1e-4)) rLf = L.r;
        if (val(pLf) < R(1e-4)) pLf = L.p;
        Lr = p2c(F, rLf, uLf, vLf, pLf, S(R(0)), S(R(0)));
        S rRf = Rt.r + phR * (Acc<S>::ld(G, G_R, n) * dxR + Acc<S>::ld(G, G_R + 1, n) * dyR);
        S pRf = Rt.p + phR * (Acc<S>::ld(G, G_P, n) * dxR + Acc<S>::ld(G, G_P + 1, n) * dyR);
        S uRf = Rt.u + phR * (Acc<S>::ld(G, G_U, n) * dxR + Acc<S>::ld(G, G_U + 1, n) * dyR);
        S vRf = Rt.v + phR * (Acc<S>::ld(G, G_V, n) * dxR + Acc<S>::ld(G, G_V + 1, n) * dyR);
        if (val(rRf) < R(1e-4)) rRf = Rt.r;
        if (val(pRf) < R(1e-4)) pRf = Rt.p;
        Rr = p2c(F, rRf, uRf, vRf, pRf, S(R(0)), S(R(0)));
    }
    Flux6<S> TF;
    if (n < 0 && (tag == 3 || tag == 4)) {
        S pw = Lr.p;
        TF.f[0] = S(R(0.0));
        TF.f[1] = pw * nx;
        TF.f[2] = pw * ny;
        TF.f[3] = S(R(0.0));
        TF.f[4] = S(R(0.0));
        TF.f[5] = S(R(0.0));
    } else {
        TF = inviscid_flux(F, Lr, Rr, nx, ny);
    }
    if (F.viscous) {
        S rf = R(0.5) * (L.r + Rt.r);
        S uf = R(0.5) * (L.u + Rt.u);
        S vf = R(0.5) * (L.v + Rt.v);
        S dudx, dudy, dvdx, dvdy, dTdx, dTdy;
        if (n < 0 && tag == 4) {
            R dx = m.dxo[f], dy = m.dyo[f];
            R d2 = dx * dx + dy * dy;
            S uc = L.u, vc = L.v;
            dudx = -uc * dx / d2;
            dudy = -uc * dy / d2;
            dvdx = -vc * dx / d2;
            dvdy = -vc * dy / d2;
            dTdx = S(R(0.0));
            dTdy = S(R(0.0));
        } else {
            int nn = n >= 0 ? n : o;
            dudx = R(0.5) * (Acc<S>::ld(G, G_U, o) + Acc<S>::ld(G, G_U, nn));
            dudy = R(0.5) * (Acc<S>::ld(G, G_U + 1, o) + Acc<S>::ld(G, G_U + 1, nn));
            dvdx = R(0.5) * (Acc<S>::ld(G, G_V, o) + Acc<S>::ld(G, G_V, nn));
            dvdy = R(0.5) * (Acc<S>::ld(G, G_V + 1, o) + Acc<S>::ld(G, G_V + 1, nn));
            dTdx = R(0.5) * (Acc<S>::ld(G, G_T, o) + Acc<S>::ld(G, G_T, nn));
            dTdy = R(0.5) * (Acc<S>::ld(G, G_T + 1, o) + Acc<S>::ld(G, G_T + 1, nn));
            R dxLR = m.dxlr[f], dyLR = m.dylr[f];
            R d2 = dxLR * dxLR + dyLR * dyLR;
            if (d2 > R(1e-14)) {
                S du = Rt.u - L.u;
                S dv = Rt.v - L.v;
                S a0 = dudx, b0 = dudy, c0 = dvdx, e0 = dvdy;
                dudx = a0 - (a0 * dxLR + b0 * dyLR - du) * dxLR / d2;
                dudy = b0 - (a0 * dxLR + b0 * dyLR - du) * dyLR / d2;
                dvdx = c0 - (c0 * dxLR + e0 * dyLR - dv) * dxLR / d2;
                dvdy = e0 - (c0 * dxLR + e0 * dyLR - dv) * dyLR / d2;
            }
        }
        R Cp = F.gam * F.Rgas / (F.gam - R(1.0));
        S mu = rf * F.nu;
        S kc = mu * Cp / F.Pr;
        S div = dudx + dvdy;
        S txx = mu * (R(2.0) * dudx - (R(2.0) / R(3.0)) * div);
        S tyy = mu * (R(2.0) * dvdy - (R(2.0) / R(3.0)) * div);
        S txy = mu * (dudy + dvdx);
        S qx = -kc * dTdx, qy = -kc * dTdy;
        S wx = uf * txx + vf * txy - qx;
        S wy = uf * txy + vf * tyy - qy;
        TF.f[0] = TF.f[0] - S(R(0.0));
        TF.f[1] = TF.f[1] - (txx * nx + txy * ny);
        TF.f[2] = TF.f[2] - (txy * nx + tyy * ny);
        TF.f[3] = TF.f[3] - (wx * nx + wy * ny);
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) Acc<S>::st(FA, c, f, TF.f[c] * A);
}

// ---------------------------------------------------------------- k_gather
// R_i = sum over the cell's faces, in reference face order, of +F*A (owner) or -F*A
// (neighbour) (src/Solver.cpp:795-799).  Optionally adds diag_v * vol/(dt + 1e-30)
// (the time term of applyJacobian, src/Solver.cpp:1381-1384).
template <class R, int NV>
__global__ void __launch_bounds__(256) k_gather(MeshView<R> m, const R* __restrict__ FA, long fa_stride,
                                                R* __restrict__ Rout, long r_stride,
                                                const R* __restrict__ diag_v, const R* __restrict__ dt) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    R acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = R(0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * m.nc + i];
        if (e < 0) break;
        long f = e >> 1;
        if (e & 1) {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] - FA[c * fa_stride + f];
        } else {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] + FA[c * fa_stride + f];
        }
    }
    if (diag_v) {
        R tc = m.vol[i] / (dt[i] + R(1e-30));
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = acc[c] + diag_v[c * r_stride + i] * tc;
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) Rout[c * r_stride + i] = acc[c];
}

}  // namespace cfdg
