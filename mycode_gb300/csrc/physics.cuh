// Point-wise physics of the residual: pressure, normal flux, the LLF / Roe / HLLC
// Riemann fluxes, ghost states, prim->cons and the viscous face flux.
//
// Every function is templated on the scalar S (double, float, or Dual<double|float>
// for the exact linearisation) and keeps the reference's floating-point operation
// order, so the double instantiation compiled without FMA contraction reproduces the
// reference's CPU arithmetic bit for bit.  Citations are to AmberMond/mycode.
#pragma once
#include "dual.cuh"
#include "exact64.cuh"

namespace cfdg {

using ::sqrt;
using ::fabs;
using ::pow;
using ::tanh;

enum FluxScheme { FLUX_LLF = 0, FLUX_ROE = 1, FLUX_HLLC = 2, FLUX_AUSM = 3 };
enum SpatialScheme { SP_FIRST = 0, SP_CENTRAL = 1, SP_LIMITED = 2 };
enum BcSet { BC_BUMP = 0, BC_SUPERSONIC = 1, BC_PLATE = 2 };

// a / b correctly rounded, from y = RN(1/b): q = RN(a y) is within an ulp of a / b, the
// remainder a - b q is exact under an FMA, and RN(q + (a - b q) y) = RN(a / b) (Markstein's
// theorem: P. Markstein, IBM J. Res. Dev. 34(1), 1990).  Finite operands without
// underflow; a = -0 would give +0 (sums that start from +0 never are -0).  Several
// quotients by one b then cost one divide and three FP64 operations each, where a GB300
// FP64 divide costs about seven.
CFD_HD double quot_by_recip(double a, double b, double y) {
    const double q = a * y;
    return fma(fma(-q, b, a), y, q);
}
// a / b by the reciprocal y = 1 / b for FP64 (the same bits as the division), plain
// division for the other scalar types
template <class S, class R> CFD_HD S div_shared(S a, R b, R) { return a / b; }
CFD_HD double div_shared(double a, double b, double y) { return quot_by_recip(a, b, y); }
// the same with a divisor of the scalar type: recip_for(b) is 1 / b for FP64 (unused
// otherwise), quot_shared(a, b, y) the quotient.  The flux functions take every quotient
// by a state's density this way, so after inlining all of them share the one reciprocal
// that make_cs takes for u and v.
template <class S> CFD_HD S recip_for(S) { return S(1.0f); }
CFD_HD double recip_for(double b) { return 1.0 / b; }
template <class S> CFD_HD S quot_shared(S a, S b, S) { return a / b; }
CFD_HD double quot_shared(double a, double b, double y) { return quot_by_recip(a, b, y); }

// libstdc++'s std::max / std::min selection rule (NaN behaviour included; FP64: the
// comparison on the integer pipes, exact64.cuh, the same selection for non-NaN operands)
template <class S> CFD_HD S smax(S a, S b) { return (val(a) < val(b)) ? b : a; }
template <class S> CFD_HD S smin(S a, S b) { return (val(b) < val(a)) ? b : a; }
CFD_HD double smax(double a, double b) { return lt_exact(a, b) ? b : a; }
CFD_HD double smin(double a, double b) { return lt_exact(b, a) ? b : a; }

// Flow constants seen by the kernels (set on the host from the Solver setters).
template <class R>
struct Flow {
    R gam;      // ratio of specific heats (include/Flux.hpp:9, include/Solver.hpp:91)
    R Rgas;     // gas constant (include/Solver.hpp:92)
    R Pr;       // Prandtl number (src/Solver.cpp:541)
    R nu;       // kinematic viscosity (include/Solver.hpp:42)
    R Minf, P0, T0, Pexit;   // setFlowConditions (src/Solver.cpp:12-32)
    R fs[4];    // frozen free-stream state (src/Solver.cpp:979-985); exact host copy
    R shock[4]; // post-shock inflow state for tag 6 (no reference counterpart)
    // SST (no reference counterpart; parity unpinned)
    R k_inf, w_inf, Pr_t;
    R inv_Pr, inv_Prt;  // RN(1 / Pr), RN(1 / Pr_t): quotients by them through quot_by_recip
    // per-flow constants the face and cell functions would otherwise form per call (FP64:
    // each the same bits as the expression it replaces): gamma - 1, RN(1 / (gamma - 1)),
    // Cp = RN(gamma Rgas / (gamma - 1))
    R gm1, igm1, Cp;
    int bcset, flux, spatial, viscous;
    int sst;    // 1: the state carries rhok, rhow (SST)
};

// The derived constants of F from gam, Rgas, Pr and Pr_t (correctly rounded divisions).
template <class R>
inline void flow_derived(Flow<R>& F) {
    F.inv_Pr = R(1) / F.Pr;
    F.inv_Prt = R(1) / F.Pr_t;
    F.gm1 = F.gam - R(1);
    F.igm1 = R(1) / F.gm1;
    F.Cp = F.gam * F.Rgas / F.gm1;
}

// Conservative state with its derived primitives u, v, p (reference formulas).
template <class S>
struct CS {
    S r, ru, rv, rE, rk, rw;
    S u, v, p;
};

// getPressure (include/Flux.hpp:12-15)
template <class S, class R>
CFD_HD S pressure(const Flow<R>& F, S r, S ru, S rv, S rE) {
    S V2 = (ru * ru + rv * rv) / (r * r);
    return F.gm1 * (rE - half(r) * V2);
}

template <class S, class R>
CFD_HD CS<S> make_cs(const Flow<R>& F, S r, S ru, S rv, S rE, S rk, S rw) {
    CS<S> c;
    c.r = r; c.ru = ru; c.rv = rv; c.rE = rE; c.rk = rk; c.rw = rw;
    const S ir = recip_for(r);  // FP64: u and v by one reciprocal (quot_shared)
    c.u = quot_shared(ru, r, ir);
    c.v = quot_shared(rv, r, ir);
    c.p = pressure(F, r, ru, rv, rE);
    return c;
}

// primitiveToConservative (src/Solver.cpp:498-501)
template <class S, class R>
CFD_HD CS<S> p2c(const Flow<R>& F, S r, S u, S v, S p, S k, S w) {
    S rE = div_shared(p, F.gm1, F.igm1) + half(r) * (u * u + v * v);
    return make_cs(F, r, r * u, r * v, rE, r * k, r * w);
}

template <class S>
struct Flux6 { S f[6]; };

// computeNormalFlux (include/Flux.hpp:23-34); k and w components are zero
template <class S, class R>
CFD_HD Flux6<S> normal_flux(const CS<S>& U, R nx, R ny) {
    S un = U.u * nx + U.v * ny;
    Flux6<S> o;
    o.f[0] = U.r * un;
    o.f[1] = U.ru * un + U.p * nx;
    o.f[2] = U.rv * un + U.p * ny;
    o.f[3] = (U.rE + U.p) * un;
    o.f[4] = S(R(0));
    o.f[5] = S(R(0));
    return o;
}

// computeFluxLLF (include/Flux.hpp:81-108)
template <class S, class R>
CFD_HD Flux6<S> flux_llf(const Flow<R>& F, const CS<S>& L, const CS<S>& Rt, R nx, R ny) {
    Flux6<S> FL = normal_flux(L, nx, ny), FR = normal_flux(Rt, nx, ny);
    S unL = L.u * nx + L.v * ny;
    S cL = sqrt(quot_shared(F.gam * L.p, L.r, recip_for(L.r)));
    S unR = Rt.u * nx + Rt.v * ny;
    S cR = sqrt(quot_shared(F.gam * Rt.p, Rt.r, recip_for(Rt.r)));
    S a = smax(fabs(unL) + cL, fabs(unR) + cR);
    S ha = half(a);
    S UL[6] = {L.r, L.ru, L.rv, L.rE, L.rk, L.rw};
    S UR[6] = {Rt.r, Rt.ru, Rt.rv, Rt.rE, Rt.rk, Rt.rw};
    Flux6<S> o;
#pragma unroll
    for (int c = 0; c < 6; ++c) o.f[c] = half(FL.f[c] + FR.f[c]) - (UR[c] - UL[c]) * ha;
    return o;
}

// computeFluxROE with Harten's entropy fix (include/Flux.hpp:112-213)
template <class S, class R>
CFD_HD Flux6<S> flux_roe(const Flow<R>& F, const CS<S>& L, const CS<S>& Rt, R nx, R ny) {
    S hL = quot_shared(L.rE + L.p, L.r, recip_for(L.r));
    S hR = quot_shared(Rt.rE + Rt.p, Rt.r, recip_for(Rt.r));
    S sL = sqrt(L.r), sR = sqrt(Rt.r);
    S inv = R(1.0) / (sL + sR);
    S ut = (sL * L.u + sR * Rt.u) * inv;
    S vt = (sL * L.v + sR * Rt.v) * inv;
    S ht = (sL * hL + sR * hR) * inv;
    S V2 = ut * ut + vt * vt;
    S c2 = F.gm1 * (ht - half(V2));
    S ct = sqrt(smax(c2, S(R(1e-8))));
    S unt = ut * nx + vt * ny;
    S utt = -ut * ny + vt * nx;
    S lam[4] = {unt - ct, unt, unt, unt + ct};
    S eps = R(0.1) * ct;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (lt(fabs(lam[i]), eps)) lam[i] = half(lam[i] * lam[i] / eps + eps);
        lam[i] = fabs(lam[i]);
    }
    S dr = Rt.r - L.r, du = Rt.u - L.u, dv = Rt.v - L.v, dp = Rt.p - L.p;
    S dun = du * nx + dv * ny;
    S dut = -du * ny + dv * nx;
    S rt = sL * sR;
    S al0 = R(0.5) / c2 * (dp - rt * ct * dun);
    S al1 = dr - dp / c2;
    S al2 = rt * dut;
    S al3 = R(0.5) / c2 * (dp + rt * ct * dun);
    S w1 = lam[0] * al0, w2 = lam[1] * al1, w3 = lam[2] * al2, w4 = lam[3] * al3;
    S D[6];
    D[0] = w1 * R(1.0) + w2 * R(1.0) + w3 * R(0.0) + w4 * R(1.0);
    D[1] = w1 * (ut - ct * nx) + w2 * ut + w3 * (-ny) + w4 * (ut + ct * nx);
    D[2] = w1 * (vt - ct * ny) + w2 * vt + w3 * nx + w4 * (vt + ct * ny);
    D[3] = w1 * (ht - unt * ct) + w2 * half(V2) + w3 * utt + w4 * (ht + unt * ct);
    D[4] = fabs(unt) * (quot_shared(Rt.rk, Rt.r, recip_for(Rt.r)) - quot_shared(L.rk, L.r, recip_for(L.r))) * rt;
    D[5] = fabs(unt) * (quot_shared(Rt.rw, Rt.r, recip_for(Rt.r)) - quot_shared(L.rw, L.r, recip_for(L.r))) * rt;
    Flux6<S> FL = normal_flux(L, nx, ny), FR = normal_flux(Rt, nx, ny);
    Flux6<S> o;
#pragma unroll
    for (int c = 0; c < 6; ++c) o.f[c] = half(FL.f[c] + FR.f[c]) - half(D[c]);
    return o;
}

// computeFluxHLLC with Roe-averaged (Einfeldt) wave speeds (include/Flux.hpp:36-76).
// The star state is built with the 4-argument State constructor, so its k and w are 0.
template <class S, class R>
CFD_HD Flux6<S> flux_hllc(const Flow<R>& F, const CS<S>& L, const CS<S>& Rt, R nx, R ny) {
    S unL = L.u * nx + L.v * ny, unR = Rt.u * nx + Rt.v * ny;
    S cL = sqrt(quot_shared(F.gam * L.p, L.r, recip_for(L.r))), cR = sqrt(quot_shared(F.gam * Rt.p, Rt.r, recip_for(Rt.r)));
    S hL = quot_shared(L.rE + L.p, L.r, recip_for(L.r)), hR = quot_shared(Rt.rE + Rt.p, Rt.r, recip_for(Rt.r));
    S sL = sqrt(L.r), sR = sqrt(Rt.r);
    const S iLR = recip_for(sL + sR);  // FP64: the three quotients by sL + sR through one reciprocal
    S ut = quot_shared(sL * L.u + sR * Rt.u, sL + sR, iLR);
    S vt = quot_shared(sL * L.v + sR * Rt.v, sL + sR, iLR);
    S ht = quot_shared(sL * hL + sR * hR, sL + sR, iLR);
    S unt = ut * nx + vt * ny;
    S ct = sqrt(F.gm1 * (ht - half(ut * ut + vt * vt)));
    S SL = smin(unL - cL, unt - ct);
    S SR = smax(unR + cR, unt + ct);
    S Ss = (Rt.p - L.p + L.r * unL * (SL - unL) - Rt.r * unR * (SR - unR)) /
           (L.r * (SL - unL) - Rt.r * (SR - unR));
    if (ge0(SL)) return normal_flux(L, nx, ny);
    if (le0(SR)) return normal_flux(Rt, nx, ny);
    const bool left = ge0(Ss);
    const CS<S>& K = left ? L : Rt;
    S SK = left ? SL : SR;
    S unK = left ? unL : unR;
    const S iK = left ? recip_for(L.r) : recip_for(Rt.r);  // the sound speeds' reciprocals
    S coef = K.r * (SK - unK) / (SK - Ss);
    S Us[6];
    Us[0] = coef;
    Us[1] = coef * (K.u + (Ss - unK) * nx);
    Us[2] = coef * (K.v + (Ss - unK) * ny);
    Us[3] = coef * (quot_shared(K.rE, K.r, iK) + (Ss - unK) * (Ss + K.p / (K.r * (SK - unK))));
    Us[4] = S(R(0));
    Us[5] = S(R(0));
    S UK[6] = {K.r, K.ru, K.rv, K.rE, K.rk, K.rw};
    Flux6<S> FK = normal_flux(K, nx, ny);
    Flux6<S> o;
#pragma unroll
    for (int c = 0; c < 6; ++c) o.f[c] = FK.f[c] + (Us[c] - UK[c]) * SK;
    return o;
}

// computeInviscidFlux (include/Flux.hpp:216-227): AUSM falls through to LLF
template <class S, class R>
CFD_HD Flux6<S> inviscid_flux(const Flow<R>& F, const CS<S>& L, const CS<S>& Rt, R nx, R ny) {
    if (F.flux == FLUX_ROE) return flux_roe(F, L, Rt, nx, ny);
    if (F.flux == FLUX_HLLC) return flux_hllc(F, L, Rt, nx, ny);
    return flux_llf(F, L, Rt, nx, ny);
}

// slip-wall reflection (src/Solver.cpp:845-860): k and w copied from the interior
template <class S, class R>
CFD_HD CS<S> slip_ghost(const Flow<R>& F, const CS<S>& U, R nx, R ny) {
    S vn = U.u * nx + U.v * ny;
    S ug = U.u - R(2.0) * vn * nx;
    S vg = U.v - R(2.0) * vn * ny;
    return make_cs(F, U.r, U.r * ug, U.r * vg, U.rE, U.rk, U.rw);
}

template <class S, class R>
CFD_HD CS<S> const_state(const Flow<R>& F, const R* s4) {
    return make_cs(F, S(s4[0]), S(s4[1]), S(s4[2]), S(s4[3]), S(R(0)), S(R(0)));
}

// getBoundaryGhostState: bump set (src/Solver.cpp:806-863), supersonic set
// (:973-1011), laminar-plate / SWBLI set (:1088-1139).  Tag 6 (post-shock inflow)
// has no reference counterpart.  For the SST variables the turbulent far field and
// wall values follow the SST model's boundary rules (parity unpinned).
// With SST (F.sst) the turbulence variables of the ghost are set by the model's rules
// instead of the reference's zeros: free stream at inflow and far-field tags,
// extrapolation at the pressure outlet, and at a no-slip wall k_face = 0 and
// w_face = 60 nu / (beta1 d^2) with d = dwall, the normal distance of the wall face.
template <class S, class R>
CFD_HD CS<S> sst_ghost(const Flow<R>& F, CS<S> g, const CS<S>& U, int kind, R dwall) {
    if (!F.sst) return g;
    if (kind == 0) {          // free stream
        g.rk = g.r * F.k_inf;
        g.rw = g.r * F.w_inf;
    } else if (kind == 1) {   // extrapolate the specific values
        g.rk = g.r * (U.rk / U.r);
        g.rw = g.r * (U.rw / U.r);
    } else {                  // no-slip wall
        R d = dwall > R(1e-30) ? dwall : R(1e-30);
        R ww = R(60.0) * F.nu / (R(0.075) * d * d);
        g.rk = -g.r * (U.rk / U.r);
        g.rw = g.r * (R(2.0) * ww - U.rw / U.r);
    }
    return g;
}

template <class S, class R>
CFD_HD CS<S> ghost_state(const Flow<R>& F, const CS<S>& U, int tag, R nx, R ny, R dwall = R(0)) {
    const R g = F.gam;
    if (F.bcset == BC_BUMP) {
        if (tag == 1) {
            S pu = smin(U.p, S(F.P0 - R(1e-4)));
            S Tg = F.T0 * pow(pu / F.P0, (g - R(1.0)) / g);
            S rg = pu / (F.Rgas * Tg);
            R Cp = g * F.Rgas / (g - R(1.0));
            S V2 = R(2.0) * Cp * (F.T0 - Tg);
            S V = gt0(V2) ? sqrt(V2) : S(R(0.0));
            return sst_ghost(F, p2c(F, rg, V, S(R(0.0)), pu, S(R(0)), S(R(0))), U, 0, dwall);
        } else if (tag == 2) {
            return sst_ghost(F, p2c(F, U.r, U.u, U.v, S(F.Pexit), S(R(0)), S(R(0))), U, 1, dwall);
        } else if (tag == 3) {
            return slip_ghost(F, U, nx, ny);
        }
        return U;
    } else if (F.bcset == BC_SUPERSONIC) {
        if (tag == 1) return sst_ghost(F, const_state<S>(F, F.fs), U, 0, dwall);
        if (tag == 2) return U;
        if (tag == 3) return slip_ghost(F, U, nx, ny);
        if (tag == 6) return sst_ghost(F, const_state<S>(F, F.shock), U, 0, dwall);
        return U;
    } else {
        if (tag == 1 || tag == 5) {
            CS<S> c = const_state<S>(F, F.fs);
            c.rk = S(c.r * F.k_inf);
            c.rw = S(c.r * F.w_inf);
            return c;
        }
        if (tag == 6) {
            CS<S> c = const_state<S>(F, F.shock);
            c.rk = S(c.r * F.k_inf);
            c.rw = S(c.r * F.w_inf);
            return c;
        }
        if (tag == 2) return U;
        if (tag == 3) return slip_ghost(F, U, nx, ny);
        if (tag == 4) {
            S ug = -(U.ru / U.r), vg = -(U.rv / U.r);
            S ek = half(U.ru * U.ru + U.rv * U.rv) / U.r;
            S pin = (g - R(1.0)) * (U.rE - ek);
            S Tin = pin / (U.r * F.Rgas);
            S rg = pin / (F.Rgas * Tin);
            return sst_ghost(F, p2c(F, rg, ug, vg, pin, S(R(0)), S(R(0))), U, 2, dwall);
        }
        return U;
    }
}

}  // namespace cfdg
