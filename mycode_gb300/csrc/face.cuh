// The residual's face function: F*A for one face from the two cell states, their
// gradients and limiters (the body of the face loop of computeResiduals,
// src/Solver.cpp:543-800).  Shared by the residual kernel (any scalar type) and by the
// adjoint, which differentiates exactly this sequence of operations.
#pragma once
#include <type_traits>
#include "physics.cuh"
#include "sst.cuh"

namespace cfdg {

template <class R>
struct FaceGeo {
    R nx, ny, A;
    R dxL, dyL, dxR, dyR;  // face midpoint minus owner / neighbour centroid
    R dxlr, dylr;          // neighbour minus owner centroid (0 on the boundary)
    R d2lr, id2lr;         // dxlr^2 + dylr^2 and its reciprocal (0 on the boundary), formed
                           // once per mesh with the expressions the viscous flux would use
};

// d2lr and id2lr of g from its dxlr, dylr (the mesh upload and host harnesses)
template <class R>
CFD_HD void geo_derived(FaceGeo<R>& g) {
    g.d2lr = g.dxlr * g.dxlr + g.dylr * g.dylr;
    g.id2lr = g.d2lr > R(0) ? R(1) / g.d2lr : R(0);
}

// gradient layout per cell: (x, y) pairs of rho, u, v, p, T
enum { FG_R = 0, FG_U = 2, FG_V = 4, FG_P = 6, FG_T = 8 };

// Ghost or neighbour state of the face: the neighbour when interior, else the ghost of L.
template <class S, class R>
CFD_HD CS<S> face_right(const Flow<R>& F, const CS<S>& L, const CS<S>& Rn, bool interior, int tag, R nx, R ny,
                        R dwall = R(0)) {
    return interior ? Rn : ghost_state(F, L, tag, nx, ny, dwall);
}

// normal distance from the owner's centroid to a boundary face (SST wall value of w)
template <class R>
CFD_HD R wall_normal_distance(const FaceGeo<R>& g) {
    R d = g.dxL * g.nx + g.dyL * g.ny;
    return lt0(d) ? -d : d;
}

// Second-order reconstruction of one side (src/Solver.cpp:596-623)
template <class S, class R>
CFD_HD CS<S> reconstruct(const Flow<R>& F, const CS<S>& C, const S* g, S ph, R dx, R dy) {
    S rf = C.r + ph * (g[FG_R] * dx + g[FG_R + 1] * dy);
    S pf = C.p + ph * (g[FG_P] * dx + g[FG_P + 1] * dy);
    S uf = C.u + ph * (g[FG_U] * dx + g[FG_U + 1] * dy);
    S vf = C.v + ph * (g[FG_V] * dx + g[FG_V + 1] * dy);
    if (lt(rf, R(1e-4))) rf = C.r;
    if (lt(pf, R(1e-4))) pf = C.p;
    return p2c(F, rf, uf, vf, pf, S(R(0)), S(R(0)));
}

// F*A of one face.  L: owner state; Rn: neighbour state (ignored on the boundary);
// gL/gR: the owner's / neighbour's 10 gradient values (gR ignored on the boundary);
// phL/phR: limiter values (used by the limited scheme); mutf: face eddy viscosity
// (SST only; it adds to mu in the stresses and as mu_t Cp / Pr_t to the conductivity).
template <class S, class R>
CFD_HD Flux6<S> face_flux(const Flow<R>& F, const CS<S>& L, const CS<S>& Rn, bool interior, int tag,
                          const FaceGeo<R>& g, const S* gL, const S* gR, S phL, S phR, S mutf = S(R(0))) {
    const R nx = g.nx, ny = g.ny;
    CS<S> Rt = face_right(F, L, Rn, interior, tag, nx, ny, wall_normal_distance(g));
    CS<S> Lr = L, Rr = Rt;
    if (F.spatial != SP_FIRST && interior) {
        S pl = F.spatial == SP_LIMITED ? phL : S(R(0.5));
        S pr = F.spatial == SP_LIMITED ? phR : S(R(0.5));
        Lr = reconstruct(F, L, gL, pl, g.dxL, g.dyL);
        Rr = reconstruct(F, Rt, gR, pr, g.dxR, g.dyR);
    }
    Flux6<S> TF;
    if (!interior && (tag == 3 || tag == 4)) {
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
        const S* gRv = interior ? gR : gL;
        S rf = half(L.r + Rt.r);
        S uf = half(L.u + Rt.u);
        S vf = half(L.v + Rt.v);
        S dudx, dudy, dvdx, dvdy, dTdx, dTdy;
        if (!interior && tag == 4) {
            R dx = g.dxL, dy = g.dyL;
            R d2 = dx * dx + dy * dy;
            const R id2 = R(1.0) / d2;  // FP64: four quotients by one reciprocal (div_shared)
            S uc = L.u, vc = L.v;
            dudx = div_shared(-uc * dx, d2, id2);
            dudy = div_shared(-uc * dy, d2, id2);
            dvdx = div_shared(-vc * dx, d2, id2);
            dvdy = div_shared(-vc * dy, d2, id2);
            dTdx = S(R(0.0));
            dTdy = S(R(0.0));
        } else {
            dudx = half(gL[FG_U] + gRv[FG_U]);
            dudy = half(gL[FG_U + 1] + gRv[FG_U + 1]);
            dvdx = half(gL[FG_V] + gRv[FG_V]);
            dvdy = half(gL[FG_V + 1] + gRv[FG_V + 1]);
            dTdx = half(gL[FG_T] + gRv[FG_T]);
            dTdy = half(gL[FG_T + 1] + gRv[FG_T + 1]);
            // FP64: precomputed per mesh, the same bits as formed here; the FP32 views form
            // them in the kernel (their FMA contraction and approximate divide)
            constexpr bool pre = std::is_same<R, double>::value;
            const R d2 = pre ? g.d2lr : g.dxlr * g.dxlr + g.dylr * g.dylr;
            if (lt(R(1e-14), d2)) {
                const R id2 = pre ? g.id2lr : R(1.0) / d2;  // FP64: four quotients by one reciprocal
                S du = Rt.u - L.u;
                S dv = Rt.v - L.v;
                S a0 = dudx, b0 = dudy, c0 = dvdx, e0 = dvdy;
                dudx = a0 - div_shared((a0 * g.dxlr + b0 * g.dylr - du) * g.dxlr, d2, id2);
                dudy = b0 - div_shared((a0 * g.dxlr + b0 * g.dylr - du) * g.dylr, d2, id2);
                dvdx = c0 - div_shared((c0 * g.dxlr + e0 * g.dylr - dv) * g.dxlr, d2, id2);
                dvdy = e0 - div_shared((c0 * g.dxlr + e0 * g.dylr - dv) * g.dylr, d2, id2);
            }
        }
        const R Cp = F.Cp;
        S mu = rf * F.nu;
        S kc = div_shared(mu * Cp, F.Pr, F.inv_Pr);  // FP64: by the reciprocal of Pr, the same bits
        if (F.sst) {
            kc = kc + div_shared(mutf * Cp, F.Pr_t, F.inv_Prt);
            mu = mu + mutf;
        }
        S div = dudx + dvdy;
        S txx = mu * (twice(dudx) - (R(2.0) / R(3.0)) * div);
        S tyy = mu * (twice(dvdy) - (R(2.0) / R(3.0)) * div);
        S txy = mu * (dudy + dvdx);
        S qx = -kc * dTdx, qy = -kc * dTdy;
        S wx = uf * txx + vf * txy - qx;
        S wy = uf * txy + vf * tyy - qy;
        TF.f[0] = TF.f[0] - S(R(0.0));
        TF.f[1] = TF.f[1] - (txx * nx + txy * ny);
        TF.f[2] = TF.f[2] - (txy * nx + tyy * ny);
        TF.f[3] = TF.f[3] - (wx * nx + wy * ny);
    }
    Flux6<S> out;
#pragma unroll
    for (int c = 0; c < 6; ++c) out.f[c] = TF.f[c] * g.A;
    return out;
}

// F*A of one face with the SST model: the mean-flow rows with the face eddy viscosity
// mu_t,f = (mu_t,L + mu_t,R) / 2 (zero at a no-slip wall), then the k and w rows
// (sst_face_flux) from the mean flow's mass flux.  gkL/gkR: k_x, k_y, w_x, w_y of each
// side.  On the boundary the right-hand mu_t, F1 and k, w gradients are the owner's.
// kwL/kwR: the specific k, w (rho k / rho, rho w / rho) of the owner and the neighbour, the
// primitives the cells already hold (the same quotients); on the boundary the ghost's are
// formed here.
template <class S, class R>
CFD_HD Flux6<S> face_flux_sst(const Flow<R>& F, const CS<S>& L, const CS<S>& Rn, bool interior, int tag,
                              const FaceGeo<R>& g, const S* gL, const S* gR, const S* gkL, const S* gkR, S phL,
                              S phR, S mutL, S mutR, S F1L, S F1R, const S* kwL, const S* kwR) {
    bool wall = !interior && tag == 4;
    if (!interior) {
        mutR = mutL;
        F1R = F1L;
    }
    S mutf = wall ? S(R(0)) : half(mutL + mutR);
    S F1f = half(F1L + F1R);
    Flux6<S> out = face_flux(F, L, Rn, interior, tag, g, gL, gR, phL, phR, mutf);
    CS<S> Rt = face_right(F, L, Rn, interior, tag, g.nx, g.ny, wall_normal_distance(g));
    const S* gkRv = interior ? gkR : gkL;
    S Fk, Fw;
    S kR, wR;
    if (interior) {
        kR = kwR[0];
        wR = kwR[1];
    } else {
        const S ig = recip_for(Rt.r);
        kR = quot_shared(Rt.rk, Rt.r, ig);
        wR = quot_shared(Rt.rw, Rt.r, ig);
    }
    sst_face_flux(F, out.f[0], kwL[0], kwL[1], kR, wR, half(L.r + Rt.r), mutf, F1f, gkL, gkRv, wall, g.nx, g.ny,
                  g.A, g.dxL, g.dyL, g.dxlr, g.dylr, g.d2lr, g.id2lr, Fk, Fw);
    out.f[4] = Fk;
    out.f[5] = Fw;
    return out;
}

}  // namespace cfdg
