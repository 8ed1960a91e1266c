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
#include <type_traits>
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

// tanh where its rounded value is settled without evaluating it.  1 - tanh x = 2 / (e^{2x}
// + 1) is below half an ulp of 1 (2^-54 in FP64, 2^-25 in FP32) from x = 19.06 (8.66), so
// from TANH_ONE on the rounded tanh is 1; tanh x = x (1 - x^2 / 3 + ...) rounds to x below
// TANH_ID (x^2 / 3 under half an ulp).  In the SST model F1 = tanh(arg1^4) and F2 =
// tanh(arg2^2) sit in those two ranges in most cells (near a wall and in the free stream), so
// most calls cost a comparison.  Checked bit for bit against CUDA's tanh on both sides of
// both thresholds (tests/test_gpu_exact64.py).
template <class R> struct TanhSat;
template <> struct TanhSat<double> { static constexpr double one = 19.5, id = 7.450580596923828e-09; };  // 2^-27
template <> struct TanhSat<float> { static constexpr float one = 9.5f, id = 1.220703125e-04f; };        // 2^-13
template <class R>
CFD_HD R tanh_sat(R x) {
    const R ax = x < R(0) ? -x : x;
    if (ax < TanhSat<R>::id) return x;
    if (x >= TanhSat<R>::one) return R(1);
    return tanh(x);
}
template <class S> CFD_HD S tanh_(S x) { return tanh(x); }
CFD_HD double tanh_(double x) { return tanh_sat(x); }
CFD_HD float tanh_(float x) { return tanh_sat(x); }
// the dual number's: the value as above, the derivative (1 - t^2) x' (0 where t is 1)
template <class R> CFD_HD Dual<R> tanh_(Dual<R> a) {
    const R t = tanh_sat(a.v);
    return Dual<R>(t, (R(1) - t * t) * a.d);
}

// One cell.  r, k, w: density and specific k, w; ux..vy: velocity gradient; kx..wy: k
// and w gradients; idd: 1 / max(d, 1e-30) of the wall distance d (a mesh invariant, formed
// once with the wall distances).
template <class S, class R>
CFD_HD SstCell<S> sst_cell_id(const Flow<R>& F, S r, S k, S w, S ux, S uy, S vx, S vy, S kx, S ky, S wx, S wy,
                              R idd) {
    typedef SstConst C;
    const R bs = R(C::beta_s), a1 = R(C::a1);
    S kp = smax(k, S(R(0)));
    S wp = smax(w, S(F.w_inf * R(C::w_min_frac)));
    S Sxy = half(uy + vx);
    S S2 = twice(ux * ux + vy * vy + twice(Sxy) * Sxy);
    S Smag = sqrt(S2 + S(R(1e-30)));
    S nu = S(F.nu);
    // one reciprocal per divisor (w, d, CD_kw, the eddy viscosity's denominator)
    const S iwp = R(1) / wp;
    S gkgw = kx * wx + ky * wy;
    S CDkw = smax(twice(r) * R(C::sw2) * gkgw * iwp, S(R(1e-10)));
    S sk = sqrt(kp + S(R(1e-30)));
    S t1 = sk * iwp * (idd / bs);
    S t2 = R(500) * nu * iwp * (idd * idd);
    S arg1 = smin(smax(t1, t2), R(4) * r * R(C::sw2) * kp / CDkw * (idd * idd));
    // tanh(x) is 1 to double precision for x > 20: capping the arguments there changes no
    // value and keeps arg^4 (up to 1e45 next to a wall) inside FP32 range
    arg1 = smin(arg1, S(R(10)));
    S a14 = arg1 * arg1 * arg1 * arg1;
    S F1 = tanh_(a14);
    S arg2 = smin(smax(twice(t1), t2), S(R(100)));
    S F2 = tanh_(arg2 * arg2);
    S mut = r * a1 * kp / smax(a1 * wp, Smag * F2);
    S beta = F1 * R(C::b1) + (R(1) - F1) * R(C::b2);
    S gam = F1 * R(C::g1) + (R(1) - F1) * R(C::g2);
    S P = smin(mut * S2, R(10) * bs * r * kp * wp);
    SstCell<S> o;
    o.mut = mut;
    o.F1 = F1;
    o.Sk = P - bs * r * wp * kp;
    o.Sw = gam * r / (mut + S(R(1e-30))) * P - beta * r * wp * wp + R(2) * (R(1) - F1) * r * R(C::sw2) * gkgw * iwp;
    return o;
}

// the same from the wall distance d itself
template <class S, class R>
CFD_HD SstCell<S> sst_cell(const Flow<R>& F, S r, S k, S w, S ux, S uy, S vx, S vy, S kx, S ky, S wx, S wy, R d) {
    const R dd = lt(R(1e-30), d) ? d : R(1e-30);
    return sst_cell_id(F, r, k, w, ux, uy, vx, vy, kx, ky, wx, wy, R(1) / dd);
}

// k and w face fluxes times the face area: first-order upwind advection with the Riemann
// mass flux (mdotA = mass flux times area), and diffusion (mu + sigma mu_t) grad(phi).n A
// with averaged, corrected face gradients (one-sided at a no-slip wall).
template <class S, class R>
CFD_HD void sst_face_flux(const Flow<R>& F, S mdotA, S kL, S wL, S kR, S wR, S rf, S mutf, S F1f, const S* gkL,
                          const S* gkR, bool wall, R nx, R ny, R A, R dxL, R dyL, R dxlr, R dylr, R d2lr,
                          R id2lr, S& Fk, S& Fw) {
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
        const R id2 = R(1) / d2;  // FP64: the two quotients through one reciprocal (div_shared)
        // (phi_face - phi_c) (d . n) / |d|^2, phi_face = 0 for k and w_face for w
        dkn = div_shared((S(R(0)) - kL) * dn, d2, id2);
        dwn = div_shared((half(wL + wR) - wL) * dn, d2, id2);
    } else {
        S kx = half(gkL[0] + gkR[0]), ky = half(gkL[1] + gkR[1]);
        S wx = half(gkL[2] + gkR[2]), wy = half(gkL[3] + gkR[3]);
        // dxlr^2 + dylr^2 and its reciprocal: precomputed per mesh for FP64 (the viscous
        // flux's too), formed here for the FP32 views
        constexpr bool pre = std::is_same<R, double>::value;
        const R d2 = pre ? d2lr : dxlr * dxlr + dylr * dylr;
        if (lt(R(1e-14), d2)) {
            const R id2 = pre ? id2lr : R(1) / d2;
            S ck = div_shared(kx * dxlr + ky * dylr - (kR - kL), d2, id2);
            S cw = div_shared(wx * dxlr + wy * dylr - (wR - wL), d2, id2);
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

// ---------------------------------------------------------------- reverse mode
// Adjoints of sst_cell's inputs from the adjoints of (mu_t, F1, S_k, S_w), along the
// branches the forward takes at the same point (the same selections as the Dual forward,
// so the VJP is the exact transpose of the J v).  Accumulates into the *b outputs.
template <class R>
CFD_HD void sst_cell_b(const Flow<R>& F, R r, R k, R w, R ux, R uy, R vx, R vy, R kx, R ky, R wx, R wy, R idd,
                       R mutb, R F1b, R Skb, R Swb, R& rb, R& kb, R& wb, R& uxb, R& uyb, R& vxb, R& vyb, R& kxb,
                       R& kyb, R& wxb, R& wyb) {
    typedef SstConst C;
    const R bs = R(C::beta_s), a1 = R(C::a1), sw2 = R(C::sw2);
    // forward
    const R wmin = F.w_inf * R(C::w_min_frac);
    bool kneg = k < R(0), wlow = w < wmin;
    R kp = kneg ? R(0) : k;
    R wp = wlow ? wmin : w;
    R Sxy = R(0.5) * (uy + vx);
    R S2 = R(2) * (ux * ux + vy * vy + R(2) * Sxy * Sxy);
    R Smag = sqrt(S2 + R(1e-30));
    R nu = F.nu;
    R gkgw = kx * wx + ky * wy;
    const R iwp = R(1) / wp;  // the forward's reciprocal (sst_cell_id); idd = 1 / max(d, 1e-30)
    R CDa = R(2) * r * sw2 * gkgw * iwp;
    bool cdclip = CDa < R(1e-10);
    R CDkw = cdclip ? R(1e-10) : CDa;
    const R iCD = R(1) / CDkw;
    R sk = sqrt(kp + R(1e-30));
    R t1 = sk * iwp * (idd / bs);
    R t2 = R(500) * nu * iwp * (idd * idd);
    bool m1t2 = t1 < t2;
    R m1 = m1t2 ? t2 : t1;
    R t3 = R(4) * r * sw2 * kp * iCD * (idd * idd);
    bool a1t3 = t3 < m1;
    R arg1u = a1t3 ? t3 : m1;
    bool a1cap = R(10) < arg1u;
    R arg1 = a1cap ? R(10) : arg1u;
    R a14 = arg1 * arg1 * arg1 * arg1;
    R F1 = tanh_sat(a14);
    bool a2t2 = R(2) * t1 < t2;
    R arg2u = a2t2 ? t2 : R(2) * t1;
    bool a2cap = R(100) < arg2u;
    R arg2 = a2cap ? R(100) : arg2u;
    R F2 = tanh_sat(arg2 * arg2);
    R da = a1 * wp, ds = Smag * F2;
    bool dens = da < ds;
    R den = dens ? ds : da;
    const R iden = R(1) / den;
    R mut = r * a1 * kp * iden;
    R beta = F1 * R(C::b1) + (R(1) - F1) * R(C::b2);
    R gam = F1 * R(C::g1) + (R(1) - F1) * R(C::g2);
    R Pu = mut * S2, Pl = R(10) * bs * r * kp * wp;
    bool plim = Pl < Pu;
    R P = plim ? Pl : Pu;
    R me = mut + R(1e-30);
    const R ime = R(1) / me;
    // reverse
    R rb_ = 0, kpb = 0, wpb = 0, Pb = 0, gamb = 0, betab = 0, gkgwb = 0;
    R mutb_ = mutb, F1b_ = F1b;
    gamb += Swb * r * ime * P;
    rb_ += Swb * gam * ime * P;
    mutb_ -= Swb * gam * r * P * ime * ime;
    Pb += Swb * gam * r * ime;
    betab -= Swb * r * wp * wp;
    rb_ -= Swb * beta * wp * wp;
    wpb -= Swb * R(2) * beta * r * wp;
    F1b_ -= Swb * R(2) * r * sw2 * gkgw * iwp;
    rb_ += Swb * R(2) * (R(1) - F1) * sw2 * gkgw * iwp;
    gkgwb += Swb * R(2) * (R(1) - F1) * r * sw2 * iwp;
    wpb -= Swb * R(2) * (R(1) - F1) * r * sw2 * gkgw * iwp * iwp;
    Pb += Skb;
    rb_ -= Skb * bs * wp * kp;
    wpb -= Skb * bs * r * kp;
    kpb -= Skb * bs * r * wp;
    R S2b = 0;
    if (plim) {
        rb_ += Pb * R(10) * bs * kp * wp;
        kpb += Pb * R(10) * bs * r * wp;
        wpb += Pb * R(10) * bs * r * kp;
    } else {
        mutb_ += Pb * S2;
        S2b += Pb * mut;
    }
    F1b_ += betab * (R(C::b1) - R(C::b2)) + gamb * (R(C::g1) - R(C::g2));
    rb_ += mutb_ * a1 * kp * iden;
    kpb += mutb_ * r * a1 * iden;
    R denb = -mutb_ * mut * iden;
    R Smagb = 0, F2b = 0;
    if (dens) {
        Smagb += denb * F2;
        F2b += denb * Smag;
    } else {
        wpb += denb * a1;
    }
    R arg2b = a2cap ? R(0) : F2b * (R(1) - F2 * F2) * R(2) * arg2;
    R t1b = 0, t2b = 0;
    if (a2t2) t2b += arg2b;
    else t1b += R(2) * arg2b;
    R a14b = F1b_ * (R(1) - F1 * F1);
    R arg1b = a1cap ? R(0) : a14b * R(4) * arg1 * arg1 * arg1;
    R t3b = 0, m1b = 0;
    if (a1t3) t3b += arg1b;
    else m1b += arg1b;
    R CDkwb = 0;
    rb_ += t3b * R(4) * sw2 * kp * iCD * (idd * idd);
    kpb += t3b * R(4) * r * sw2 * iCD * (idd * idd);
    CDkwb -= t3b * t3 * iCD;
    if (m1t2) t2b += m1b;
    else t1b += m1b;
    wpb -= t2b * t2 * iwp;
    R skb = t1b * iwp * (idd / bs);
    wpb -= t1b * t1 * iwp;
    kpb += skb / (sk + sk);
    if (!cdclip) {
        rb_ += CDkwb * R(2) * sw2 * gkgw * iwp;
        gkgwb += CDkwb * R(2) * r * sw2 * iwp;
        wpb -= CDkwb * CDa * iwp;
    }
    kxb += gkgwb * wx;
    wxb += gkgwb * kx;
    kyb += gkgwb * wy;
    wyb += gkgwb * ky;
    S2b += Smagb / (Smag + Smag);
    uxb += S2b * R(4) * ux;
    vyb += S2b * R(4) * vy;
    R Sxyb = S2b * R(8) * Sxy;
    uyb += R(0.5) * Sxyb;
    vxb += R(0.5) * Sxyb;
    if (!wlow) wb += wpb;
    if (!kneg) kb += kpb;
    rb += rb_;
}

// Adjoints of sst_face_flux's inputs from (Fkb, Fwb).  gkLb / gkRb: k_x, k_y, w_x, w_y.
template <class R>
CFD_HD void sst_face_flux_b(const Flow<R>& F, R mdotA, R kL, R wL, R kR, R wR, R rf, R mutf, R F1f, const R* gkL,
                            const R* gkR, bool wall, R nx, R ny, R A, R dxL, R dyL, R dxlr, R dylr, R d2lr,
                            R id2lr, R Fkb, R Fwb,
                            R& mdotAb, R& kLb, R& wLb, R& kRb, R& wRb, R& rfb, R& mutfb, R& F1fb, R* gkLb,
                            R* gkRb) {
    typedef SstConst C;
    // forward
    bool mneg = mdotA < R(0), mpos = R(0) < mdotA;
    R mp = mneg ? R(0) : mdotA, mm = mpos ? R(0) : mdotA;
    R mu = rf * F.nu;
    R sk = F1f * R(C::sk1) + (R(1) - F1f) * R(C::sk2);
    R sw = F1f * R(C::sw1) + (R(1) - F1f) * R(C::sw2);
    R Dk = mu + sk * mutf, Dw = mu + sw * mutf;
    R dkn, dwn;
    R d2w = dxL * dxL + dyL * dyL, dnw = dxL * nx + dyL * ny;
    R kx = 0, ky = 0, wx = 0, wy = 0;
    bool corr = !wall && d2lr > R(1e-14);  // d2lr, id2lr: |x_R - x_L|^2 and its reciprocal
    const R id2w = wall ? R(1) / d2w : R(0), id2 = corr ? id2lr : R(0);
    if (wall) {
        dkn = (R(0) - kL) * dnw * id2w;
        dwn = (R(0.5) * (wL + wR) - wL) * dnw * id2w;
    } else {
        kx = R(0.5) * (gkL[0] + gkR[0]);
        ky = R(0.5) * (gkL[1] + gkR[1]);
        wx = R(0.5) * (gkL[2] + gkR[2]);
        wy = R(0.5) * (gkL[3] + gkR[3]);
        R kxc = kx, kyc = ky, wxc = wx, wyc = wy;
        if (corr) {
            R ck = (kx * dxlr + ky * dylr - (kR - kL)) * id2;
            R cw = (wx * dxlr + wy * dylr - (wR - wL)) * id2;
            kxc = kx - ck * dxlr;
            kyc = ky - ck * dylr;
            wxc = wx - cw * dxlr;
            wyc = wy - cw * dylr;
        }
        dkn = kxc * nx + kyc * ny;
        dwn = wxc * nx + wyc * ny;
    }
    // reverse of Fk = mp kL + mm kR - Dk dkn A (and w)
    R mpb = Fkb * kL + Fwb * wL, mmb = Fkb * kR + Fwb * wR;
    kLb += Fkb * mp;
    kRb += Fkb * mm;
    wLb += Fwb * mp;
    wRb += Fwb * mm;
    R Dkb = -Fkb * dkn * A, Dwb = -Fwb * dwn * A;
    R dknb = -Fkb * Dk * A, dwnb = -Fwb * Dw * A;
    R mub = Dkb + Dwb;
    R skb = Dkb * mutf, swb = Dwb * mutf;
    mutfb += Dkb * sk + Dwb * sw;
    F1fb += skb * (R(C::sk1) - R(C::sk2)) + swb * (R(C::sw1) - R(C::sw2));
    rfb += mub * F.nu;
    if (!mneg) mdotAb += mpb;
    if (!mpos) mdotAb += mmb;
    if (wall) {
        kLb -= dknb * dnw * id2w;
        R t = dwnb * dnw * id2w;
        wLb += t * (R(0.5) - R(1));
        wRb += t * R(0.5);
    } else {
        R kxb = dknb * nx, kyb = dknb * ny, wxb = dwnb * nx, wyb = dwnb * ny;
        if (corr) {
            R ckb = -(kxb * dxlr + kyb * dylr), cwb = -(wxb * dxlr + wyb * dylr);
            const R ckd = ckb * id2, cwd = cwb * id2;
            kxb += ckd * dxlr;
            kyb += ckd * dylr;
            kRb -= ckd;
            kLb += ckd;
            wxb += cwd * dxlr;
            wyb += cwd * dylr;
            wRb -= cwd;
            wLb += cwd;
        }
        gkLb[0] += R(0.5) * kxb;
        gkRb[0] += R(0.5) * kxb;
        gkLb[1] += R(0.5) * kyb;
        gkRb[1] += R(0.5) * kyb;
        gkLb[2] += R(0.5) * wxb;
        gkRb[2] += R(0.5) * wxb;
        gkLb[3] += R(0.5) * wyb;
        gkRb[3] += R(0.5) * wyb;
    }
}

// free-stream k and w from turbulence intensity and eddy-viscosity ratio
inline void sst_freestream(double Tu, double ratio, double U, double nu, double& k, double& w) {
    k = 1.5 * (Tu * U) * (Tu * U);
    w = k / (ratio * nu);
}

}  // namespace cfdg
