// Menter SST turbulence model, 2003 variant (Menter, Kuntz & Langtry 2003, "Ten years of
// industrial experience with the SST turbulence model"; the "SST-2003" form of the NASA
// Turbulence Modeling Resource).  The reference solver carries only scaffolding for it
// (State::rhok/rhow, include/Types.hpp:63-68; the k/w gradient slots,
// include/Solver.hpp:22-23; computeWallDistances, src/Solver.cpp:1981-2015), so these
// terms have no reference counterpart.
//
//   mu_t   = rho a1 k / max(a1 w, S F2)
//   P      = min(mu_t S^2, 10 beta* rho k w)                    (k production)
//   S_k    = P - beta* rho w k
//   S_w    = (gamma rho / mu_t) P - beta rho w^2 + 2 (1 - F1) rho sigma_w2 grad k . grad w / w
//            (mu_t + 1e-30 in the first term: P = mu_t = 0 where k = 0)
//   F1     = tanh(arg1^4), arg1 = min(max(sqrt k / (beta* w d), 500 nu / (d^2 w)),
//                                     4 rho sigma_w2 k / (CD_kw d^2))
//   CD_kw  = max(2 rho sigma_w2 grad k . grad w / w, 1e-10)
//   F2     = tanh(arg2^2), arg2 = max(2 sqrt k / (beta* w d), 500 nu / (d^2 w))
//   S      = sqrt(2 S_ij S_ij) from the Green-Gauss velocity gradients
// Coefficients are blended phi = F1 phi1 + (1 - F1) phi2.  Laminar viscosity is the
// reference's constant-nu model, mu = rho nu.  The -2/3 rho k delta_ij part of the
// Reynolds stress is neglected.
#pragma once
#include "physics.cuh"

namespace cfdg {

struct SstConst {
    static constexpr double beta_s = 0.09, a1 = 0.31;
    static constexpr double sk1 = 0.85, sw1 = 0.5, b1 = 0.075, g1 = 5.0 / 9.0;
    static constexpr double sk2 = 1.0, sw2 = 0.856, b2 = 0.0828, g2 = 0.44;
    static constexpr double w_min_frac = 1e-6;  // floor of w relative to the free-stream w
};

// cell quantities of the model
template <class S>
struct SstCell {
    S mut, F1, Sk, Sw;  // eddy viscosity, blending, sources per unit volume
};

template <class S> CFD_HD S tanh_(S x) { return tanh(x); }

// One cell.  r, k, w: density and specific k, w; ux..vy: velocity gradient; kx..wy: k
// and w gradients; d: wall distance.
template <class S, class R>
CFD_HD SstCell<S> sst_cell(const Flow<R>& F, S r, S k, S w, S ux, S uy, S vx, S vy, S kx, S ky, S wx, S wy, R d) {
    typedef SstConst C;
    const R bs = R(C::beta_s), a1 = R(C::a1);
    S kp = smax(k, S(R(0)));
    S wp = smax(w, S(F.w_inf * R(C::w_min_frac)));
    S Sxy = R(0.5) * (uy + vx);
    S S2 = R(2) * (ux * ux + vy * vy + R(2) * Sxy * Sxy);
    S Smag = sqrt(S2 + S(R(1e-30)));
    S nu = S(F.nu);
    R dd = d > R(1e-30) ? d : R(1e-30);
    S gkgw = kx * wx + ky * wy;
    S CDkw = smax(R(2) * r * R(C::sw2) * gkgw / wp, S(R(1e-10)));
    S sk = sqrt(kp + S(R(1e-30)));
    S t1 = sk / (bs * wp * dd);
    S t2 = R(500) * nu / (dd * dd * wp);
    S arg1 = smin(smax(t1, t2), R(4) * r * R(C::sw2) * kp / (CDkw * dd * dd));
    S a14 = arg1 * arg1 * arg1 * arg1;
    S F1 = tanh_(a14);
    S arg2 = smax(R(2) * t1, t2);
    S F2 = tanh_(arg2 * arg2);
    S mut = r * a1 * kp / smax(a1 * wp, Smag * F2);
    S beta = F1 * R(C::b1) + (R(1) - F1) * R(C::b2);
    S gam = F1 * R(C::g1) + (R(1) - F1) * R(C::g2);
    S P = smin(mut * S2, R(10) * bs * r * kp * wp);
    SstCell<S> o;
    o.mut = mut;
    o.F1 = F1;
    o.Sk = P - bs * r * wp * kp;
    o.Sw = gam * r / (mut + S(R(1e-30))) * P - beta * r * wp * wp + R(2) * (R(1) - F1) * r * R(C::sw2) * gkgw / wp;
    return o;
}

// k and w face fluxes times the face area: first-order upwind advection with the Riemann
// mass flux (mdotA = mass flux times area), and diffusion (mu + sigma mu_t) grad(phi).n A
// with averaged, corrected face gradients (one-sided at a no-slip wall).
template <class S, class R>
CFD_HD void sst_face_flux(const Flow<R>& F, S mdotA, S kL, S wL, S kR, S wR, S rf, S mutf, S F1f, const S* gkL,
                          const S* gkR, bool wall, R nx, R ny, R A, R dxL, R dyL, R dxlr, R dylr, S& Fk, S& Fw) {
    typedef SstConst C;
    S mp = smax(mdotA, S(R(0))), mm = smin(mdotA, S(R(0)));
    Fk = mp * kL + mm * kR;
    Fw = mp * wL + mm * wR;
    S mu = rf * F.nu;
    S sk = F1f * R(C::sk1) + (R(1) - F1f) * R(C::sk2);
    S sw = F1f * R(C::sw1) + (R(1) - F1f) * R(C::sw2);
    S dkn, dwn;
    if (wall) {
        R d2 = dxL * dxL + dyL * dyL;
        R dn = dxL * nx + dyL * ny;
        // (phi_face - phi_c) (d . n) / |d|^2, phi_face = 0 for k and w_face for w
        dkn = (S(R(0)) - kL) * dn / d2;
        dwn = (R(0.5) * (wL + wR) - wL) * dn / d2;
    } else {
        S kx = R(0.5) * (gkL[0] + gkR[0]), ky = R(0.5) * (gkL[1] + gkR[1]);
        S wx = R(0.5) * (gkL[2] + gkR[2]), wy = R(0.5) * (gkL[3] + gkR[3]);
        R d2 = dxlr * dxlr + dylr * dylr;
        if (d2 > R(1e-14)) {
            S ck = (kx * dxlr + ky * dylr - (kR - kL)) / d2;
            S cw = (wx * dxlr + wy * dylr - (wR - wL)) / d2;
            kx = kx - ck * dxlr;
            ky = ky - ck * dylr;
            wx = wx - cw * dxlr;
            wy = wy - cw * dylr;
        }
        dkn = kx * nx + ky * ny;
        dwn = wx * nx + wy * ny;
    }
    Fk = Fk - (mu + sk * mutf) * dkn * A;
    Fw = Fw - (mu + sw * mutf) * dwn * A;
}

// free-stream k and w from turbulence intensity and eddy-viscosity ratio
inline void sst_freestream(double Tu, double ratio, double U, double nu, double& k, double& w) {
    k = 1.5 * (Tu * U) * (Tu * U);
    w = k / (ratio * nu);
}

}  // namespace cfdg
