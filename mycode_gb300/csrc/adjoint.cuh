// Reverse-mode (adjoint) derivatives of the face function, written by hand.
//
// Each *_b function recomputes its forward intermediates and accumulates adjoints of its
// inputs from the adjoint of its output ("b" = bar).  Branches (min/max selections,
// HLLC wave regions, the Harten fix, reconstruction clips, boundary tags) follow the
// forward evaluation at the same point.  A state's adjoint is carried as CSb: one entry
// per CS field (r, ru, rv, rE, rk, rw and the derived u, v, p); cs_back() folds the
// derived fields into the conservative ones through u = ru/r, v = rv/r, p = pressure.
#pragma once
#include "face.cuh"

namespace cfdg {

template <class R>
struct CSb {
    R r, ru, rv, rE, rk, rw, u, v, p;
    CFD_HD void zero() { r = ru = rv = rE = rk = rw = u = v = p = R(0); }
};

template <class R>
CFD_HD CSb<R> csb_zero() {
    CSb<R> b;
    b.zero();
    return b;
}

// getPressure (include/Flux.hpp:12-15)
// (The reverse code multiplies by reciprocals instead of dividing where a value is
// divided more than once: GB300's FP64 divide costs about ten FP64 operations, and the
// adjoint, unlike the residual, has no bit-for-bit reference to follow.)
//
// p = (g-1)(rE - (ru^2 + rv^2) / (2 r)): dp/drE = g-1, dp/dru = -(g-1) u, dp/drv = -(g-1) v,
// dp/dr = (g-1)(u^2 + v^2)/2 with u = ru/r, v = rv/r
template <class R>
CFD_HD void pressure_b_uv(const Flow<R>& F, R u, R v, R pb, R& rb, R& rub, R& rvb, R& rEb) {
    R t = (F.gam - R(1.0)) * pb;
    rEb += t;
    rub -= t * u;
    rvb -= t * v;
    rb += R(0.5) * t * (u * u + v * v);
}

template <class R>
CFD_HD void pressure_b(const Flow<R>& F, R r, R ru, R rv, R rE, R pb, R& rb, R& rub, R& rvb, R& rEb) {
    R ir = R(1) / r;
    pressure_b_uv(F, ru * ir, rv * ir, pb, rb, rub, rvb, rEb);
}

// make_cs: conservative adjoints of a state from the adjoints of all its fields
template <class R>
CFD_HD void cs_back(const Flow<R>& F, const CS<R>& c, const CSb<R>& b, R* ub) {
    R ir = R(1) / c.r;
    R bu = b.u * ir, bv = b.v * ir;
    ub[0] += b.r - bu * c.u - bv * c.v;
    ub[1] += b.ru + bu;
    ub[2] += b.rv + bv;
    ub[3] += b.rE;
    ub[4] += b.rk;
    ub[5] += b.rw;
    pressure_b_uv(F, c.u, c.v, b.p, ub[0], ub[1], ub[2], ub[3]);
}

// Same folding into a CSb (conservative entries only) of the state c itself
template <class R>
CFD_HD void cs_fold(const Flow<R>& F, const CS<R>& c, CSb<R>& b) {
    R ub[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    cs_back(F, c, b, ub);
    b.r = ub[0]; b.ru = ub[1]; b.rv = ub[2]; b.rE = ub[3]; b.rk = ub[4]; b.rw = ub[5];
    b.u = b.v = b.p = R(0);
}

// primitiveToConservative followed by make_cs (src/Solver.cpp:498-501): adjoints of
// (r, u, v, p) from the adjoint of the resulting state (k = w = 0 inputs)
template <class R>
CFD_HD void p2c_b(const Flow<R>& F, R r, R u, R v, R p, const CSb<R>& ob, R& rb, R& ub, R& vb, R& pb) {
    CS<R> o;  // the fields cs_back reads of p2c(r, u, v, p)
    o.r = r;
    o.u = u;
    o.v = v;
    R cb[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    cs_back(F, o, ob, cb);
    // rE = p/(g-1) + 0.5 r (u^2 + v^2); ru = r u; rv = r v
    R q2 = u * u + v * v;
    rb += cb[0] + cb[1] * u + cb[2] * v + cb[3] * R(0.5) * q2;
    ub += cb[1] * r + cb[3] * r * u;
    vb += cb[2] * r + cb[3] * r * v;
    pb += cb[3] / (F.gam - R(1.0));
}

// computeNormalFlux (include/Flux.hpp:23-34)
template <class R>
CFD_HD void normal_flux_b(const CS<R>& U, R nx, R ny, const R* Fb, CSb<R>& Ub) {
    R un = U.u * nx + U.v * ny;
    R unb = Fb[0] * U.r + Fb[1] * U.ru + Fb[2] * U.rv + Fb[3] * (U.rE + U.p);
    Ub.r += Fb[0] * un;
    Ub.ru += Fb[1] * un;
    Ub.rv += Fb[2] * un;
    Ub.rE += Fb[3] * un;
    Ub.p += Fb[1] * nx + Fb[2] * ny + Fb[3] * un;
    Ub.u += unb * nx;
    Ub.v += unb * ny;
}

template <class R>
CFD_HD R sgn(R x) { return x < R(0) ? R(-1) : R(1); }

// c = sqrt(g p / r)
// (dc/dp = g / (2 c r), dc/dr = -c / (2 r) since c^2 = g p / r)
template <class R>
CFD_HD void sound_b(const Flow<R>& F, const CS<R>& U, R c, R cb, CSb<R>& Ub) {
    R t = cb / ((c + c) * U.r);
    Ub.p += t * F.gam;
    Ub.r -= t * c * c;
}

// computeFluxLLF (include/Flux.hpp:81-108)
template <class R>
CFD_HD void flux_llf_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rt, R nx, R ny, const R* Fb, CSb<R>& Lb,
                       CSb<R>& Rb) {
    R unL = L.u * nx + L.v * ny, unR = Rt.u * nx + Rt.v * ny;
    R cL = sqrt(F.gam * L.p / L.r), cR = sqrt(F.gam * Rt.p / Rt.r);
    R aL = fabs(unL) + cL, aR = fabs(unR) + cR;
    R a = smax(aL, aR);
    R ha = R(0.5) * a;
    R UL[6] = {L.r, L.ru, L.rv, L.rE, L.rk, L.rw};
    R UR[6] = {Rt.r, Rt.ru, Rt.rv, Rt.rE, Rt.rk, Rt.rw};
    R hab = R(0);
    R ULb[6], URb[6], FLb[6];
    for (int c = 0; c < 6; ++c) {
        FLb[c] = Fb[c] * R(0.5);
        hab -= Fb[c] * (UR[c] - UL[c]);
        URb[c] = -Fb[c] * ha;
        ULb[c] = Fb[c] * ha;
    }
    Lb.r += ULb[0]; Lb.ru += ULb[1]; Lb.rv += ULb[2]; Lb.rE += ULb[3]; Lb.rk += ULb[4]; Lb.rw += ULb[5];
    Rb.r += URb[0]; Rb.ru += URb[1]; Rb.rv += URb[2]; Rb.rE += URb[3]; Rb.rk += URb[4]; Rb.rw += URb[5];
    R ab = R(0.5) * hab;
    R aLb = (aL < aR) ? R(0) : ab;
    R aRb = (aL < aR) ? ab : R(0);
    R unLb = aLb * sgn(unL), unRb = aRb * sgn(unR);
    sound_b(F, L, cL, aLb, Lb);
    sound_b(F, Rt, cR, aRb, Rb);
    Lb.u += unLb * nx; Lb.v += unLb * ny;
    Rb.u += unRb * nx; Rb.v += unRb * ny;
    normal_flux_b(L, nx, ny, FLb, Lb);
    normal_flux_b(Rt, nx, ny, FLb, Rb);
}

// computeFluxROE with Harten's entropy fix (include/Flux.hpp:112-213)
template <class R>
CFD_HD void flux_roe_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rt, R nx, R ny, const R* Fb, CSb<R>& Lb,
                       CSb<R>& Rb) {
    const R gm = F.gam - R(1.0);
    // forward
    const R irL = R(1) / L.r, irR = R(1) / Rt.r;
    R hL = (L.rE + L.p) * irL, hR = (Rt.rE + Rt.p) * irR;
    R sL = sqrt(L.r), sR = sqrt(Rt.r);
    R S = sL + sR;
    R inv = R(1.0) / S;
    R nu_ = sL * L.u + sR * Rt.u, nv_ = sL * L.v + sR * Rt.v, nh_ = sL * hL + sR * hR;
    R ut = nu_ * inv, vt = nv_ * inv, ht = nh_ * inv;
    R V2 = ut * ut + vt * vt;
    R c2 = gm * (ht - R(0.5) * V2);
    R c2c = smax(c2, R(1e-8));
    R ct = sqrt(c2c);
    R unt = ut * nx + vt * ny;
    R utt = -ut * ny + vt * nx;
    R raw[4] = {unt - ct, unt, unt, unt + ct};
    R eps = R(0.1) * ct;
    const R ieps = R(1) / eps;
    R fix[4], lam[4];
    bool fixed[4];
    for (int i = 0; i < 4; ++i) {
        fixed[i] = fabs(raw[i]) < eps;
        fix[i] = fixed[i] ? R(0.5) * (raw[i] * raw[i] * ieps + eps) : raw[i];
        lam[i] = fabs(fix[i]);
    }
    R dr = Rt.r - L.r, du = Rt.u - L.u, dv = Rt.v - L.v, dp = Rt.p - L.p;
    R dun = du * nx + dv * ny;
    R dut = -du * ny + dv * nx;
    R rt = sL * sR;
    const R ic2 = R(1) / c2;
    R k0 = R(0.5) * ic2;
    R in0 = dp - rt * ct * dun, in3 = dp + rt * ct * dun;
    R al0 = k0 * in0, al1 = dr - dp * ic2, al2 = rt * dut, al3 = k0 * in3;
    R w1 = lam[0] * al0, w2 = lam[1] * al1, w3 = lam[2] * al2, w4 = lam[3] * al3;
    R aunt = fabs(unt);
    R kd = Rt.rk * irR - L.rk * irL;
    R wd = Rt.rw * irR - L.rw * irL;
    // reverse: F = 0.5 (FL + FR) - 0.5 D
    R FLb[6], Db[6];
    for (int c = 0; c < 6; ++c) {
        FLb[c] = R(0.5) * Fb[c];
        Db[c] = -R(0.5) * Fb[c];
    }
    normal_flux_b(L, nx, ny, FLb, Lb);
    normal_flux_b(Rt, nx, ny, FLb, Rb);
    R w1b = 0, w2b = 0, w3b = 0, w4b = 0, utb = 0, vtb = 0, htb = 0, ctb = 0, untb = 0, uttb = 0, V2b = 0, rtb = 0;
    R auntb = 0;
    // D4, D5
    auntb += Db[4] * kd * rt + Db[5] * wd * rt;
    R kdb = Db[4] * aunt * rt, wdb = Db[5] * aunt * rt;
    rtb += Db[4] * aunt * kd + Db[5] * aunt * wd;
    Rb.rk += kdb * irR;
    Rb.r -= (kdb * Rt.rk + wdb * Rt.rw) * irR * irR;
    Lb.rk -= kdb * irL;
    Lb.r += (kdb * L.rk + wdb * L.rw) * irL * irL;
    Rb.rw += wdb * irR;
    Lb.rw -= wdb * irL;
    untb += auntb * sgn(unt);
    // D3 = w1 (ht - unt ct) + w2 (0.5 V2) + w3 utt + w4 (ht + unt ct)
    w1b += Db[3] * (ht - unt * ct);
    htb += Db[3] * w1;
    untb -= Db[3] * w1 * ct;
    ctb -= Db[3] * w1 * unt;
    w2b += Db[3] * (R(0.5) * V2);
    V2b += Db[3] * w2 * R(0.5);
    w3b += Db[3] * utt;
    uttb += Db[3] * w3;
    w4b += Db[3] * (ht + unt * ct);
    htb += Db[3] * w4;
    untb += Db[3] * w4 * ct;
    ctb += Db[3] * w4 * unt;
    // D2 = w1 (vt - ct ny) + w2 vt + w3 nx + w4 (vt + ct ny)
    w1b += Db[2] * (vt - ct * ny);
    vtb += Db[2] * w1;
    ctb -= Db[2] * w1 * ny;
    w2b += Db[2] * vt;
    vtb += Db[2] * w2;
    w3b += Db[2] * nx;
    w4b += Db[2] * (vt + ct * ny);
    vtb += Db[2] * w4;
    ctb += Db[2] * w4 * ny;
    // D1 = w1 (ut - ct nx) + w2 ut + w3 (-ny) + w4 (ut + ct nx)
    w1b += Db[1] * (ut - ct * nx);
    utb += Db[1] * w1;
    ctb -= Db[1] * w1 * nx;
    w2b += Db[1] * ut;
    utb += Db[1] * w2;
    w3b += Db[1] * (-ny);
    w4b += Db[1] * (ut + ct * nx);
    utb += Db[1] * w4;
    ctb += Db[1] * w4 * nx;
    // D0 = w1 + w2 + w3 * 0 + w4
    w1b += Db[0];
    w2b += Db[0];
    w4b += Db[0];
    // w = lam * al
    R lamb[4] = {w1b * al0, w2b * al1, w3b * al2, w4b * al3};
    R al0b = w1b * lam[0], al1b = w2b * lam[1], al2b = w3b * lam[2], al3b = w4b * lam[3];
    // al0 = k0 in0, al3 = k0 in3, k0 = 0.5/c2
    R k0b = al0b * in0 + al3b * in3;
    R in0b = al0b * k0, in3b = al3b * k0;
    R dpb = in0b + in3b;
    rtb += (-in0b + in3b) * ct * dun;
    ctb += (-in0b + in3b) * rt * dun;
    R dunb = (-in0b + in3b) * rt * ct;
    R c2b = -k0b * R(0.5) * ic2 * ic2;
    // al1 = dr - dp / c2
    R drb = al1b;
    dpb -= al1b * ic2;
    c2b += al1b * dp * ic2 * ic2;
    // al2 = rt dut
    rtb += al2b * dut;
    R dutb = al2b * rt;
    // dun, dut
    R dub = dunb * nx - dutb * ny;
    R dvb = dunb * ny + dutb * nx;
    Rb.r += drb; Lb.r -= drb;
    Rb.u += dub; Lb.u -= dub;
    Rb.v += dvb; Lb.v -= dvb;
    Rb.p += dpb; Lb.p -= dpb;
    // Harten fix
    R epsb = 0;
    for (int i = 0; i < 4; ++i) {
        R fixb = lamb[i] * sgn(fix[i]);
        R rawb;
        if (fixed[i]) {
            rawb = fixb * raw[i] * ieps;
            epsb += fixb * R(0.5) * (R(1) - raw[i] * raw[i] * ieps * ieps);
        } else {
            rawb = fixb;
        }
        untb += rawb;
        if (i == 0) ctb -= rawb;
        if (i == 3) ctb += rawb;
    }
    ctb += R(0.1) * epsb;
    // unt, utt
    utb += untb * nx - uttb * ny;
    vtb += untb * ny + uttb * nx;
    // ct = sqrt(max(c2, 1e-8))
    R c2cb = ctb / (ct + ct);
    if (!(c2 < R(1e-8))) c2b += c2cb;
    // c2 = gm (ht - 0.5 V2)
    htb += c2b * gm;
    V2b -= R(0.5) * gm * c2b;
    utb += R(2) * ut * V2b;
    vtb += R(2) * vt * V2b;
    // ut = nu_ inv etc.
    R nub = utb * inv, nvb = vtb * inv, nhb = htb * inv;
    R invb = utb * nu_ + vtb * nv_ + htb * nh_;
    R sLb = nub * L.u + nvb * L.v + nhb * hL;
    R sRb = nub * Rt.u + nvb * Rt.v + nhb * hR;
    Lb.u += nub * sL; Rb.u += nub * sR;
    Lb.v += nvb * sL; Rb.v += nvb * sR;
    R hLb = nhb * sL, hRb = nhb * sR;
    R Sb = -invb * inv * inv;
    sLb += Sb + rtb * sR;
    sRb += Sb + rtb * sL;
    Lb.r += sLb / (sL + sL);
    Rb.r += sRb / (sR + sR);
    // h = (rE + p) / r
    R hLr = hLb * irL, hRr = hRb * irR;
    Lb.rE += hLr; Lb.p += hLr; Lb.r -= hLr * hL;
    Rb.rE += hRr; Rb.p += hRr; Rb.r -= hRr * hR;
}

// computeFluxHLLC (include/Flux.hpp:36-76)
template <class R>
CFD_HD void flux_hllc_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rt, R nx, R ny, const R* Fb, CSb<R>& Lb,
                        CSb<R>& Rb) {
    const R gm = F.gam - R(1.0);
    // one reciprocal per divisor (the forward's quotients by rho, by sL + sR and the star
    // state's, and every reverse quotient by the same values)
    const R irL = R(1) / L.r, irR = R(1) / Rt.r;
    R unL = L.u * nx + L.v * ny, unR = Rt.u * nx + Rt.v * ny;
    R cL = sqrt(F.gam * L.p * irL), cR = sqrt(F.gam * Rt.p * irR);
    R hL = (L.rE + L.p) * irL, hR = (Rt.rE + Rt.p) * irR;
    R sL = sqrt(L.r), sR = sqrt(Rt.r);
    R S = sL + sR;
    const R iS = R(1) / S;
    R nu_ = sL * L.u + sR * Rt.u, nv_ = sL * L.v + sR * Rt.v, nh_ = sL * hL + sR * hR;
    R ut = nu_ * iS, vt = nv_ * iS, ht = nh_ * iS;
    R unt = ut * nx + vt * ny;
    R c2t = gm * (ht - R(0.5) * (ut * ut + vt * vt));
    R ct = sqrt(c2t);
    R aSL = unL - cL, bSL = unt - ct;
    R SL = smin(aSL, bSL);
    R aSR = unR + cR, bSR = unt + ct;
    R SR = smax(aSR, bSR);
    R num = Rt.p - L.p + L.r * unL * (SL - unL) - Rt.r * unR * (SR - unR);
    R den = L.r * (SL - unL) - Rt.r * (SR - unR);
    R Ss = num / den;
    if (SL >= R(0.0)) {
        normal_flux_b(L, nx, ny, Fb, Lb);
        return;
    }
    if (SR <= R(0.0)) {
        normal_flux_b(Rt, nx, ny, Fb, Rb);
        return;
    }
    const bool left = Ss >= R(0.0);
    const CS<R>& K = left ? L : Rt;
    CSb<R>& Kb = left ? Lb : Rb;
    const R iK = left ? irL : irR;
    const R iden = R(1) / den;
    R SK = left ? SL : SR;
    R unK = left ? unL : unR;
    R A = K.r * (SK - unK);
    R B = SK - Ss;
    const R iA = R(1) / A, iB = R(1) / B;
    R coef = A * iB;
    R t = Ss - unK;
    R q = K.p * iA;
    const R eK = K.rE * iK;
    R e = eK + t * (Ss + q);
    R Us[6] = {coef, coef * (K.u + t * nx), coef * (K.v + t * ny), coef * e, R(0), R(0)};
    R UK[6] = {K.r, K.ru, K.rv, K.rE, K.rk, K.rw};
    normal_flux_b(K, nx, ny, Fb, Kb);
    R SKb = 0, Usb[4];
    for (int c = 0; c < 6; ++c) SKb += Fb[c] * (Us[c] - UK[c]);
    for (int c = 0; c < 4; ++c) Usb[c] = Fb[c] * SK;
    Kb.r -= Fb[0] * SK; Kb.ru -= Fb[1] * SK; Kb.rv -= Fb[2] * SK; Kb.rE -= Fb[3] * SK;
    Kb.rk -= Fb[4] * SK; Kb.rw -= Fb[5] * SK;
    R coefb = Usb[0], tb = 0, Ssb = 0, unKb = 0, Ab = 0;
    // Us3 = coef e
    coefb += Usb[3] * e;
    R eb = Usb[3] * coef;
    Kb.rE += eb * iK;
    Kb.r -= eb * eK * iK;
    tb += eb * (Ss + q);
    Ssb += eb * t;
    R qb = eb * t;
    Kb.p += qb * iA;
    Ab -= qb * q * iA;
    // Us2, Us1
    coefb += Usb[2] * (K.v + t * ny) + Usb[1] * (K.u + t * nx);
    Kb.v += Usb[2] * coef;
    Kb.u += Usb[1] * coef;
    tb += Usb[2] * coef * ny + Usb[1] * coef * nx;
    // t = Ss - unK
    Ssb += tb;
    unKb -= tb;
    // coef = A / B, B = SK - Ss
    Ab += coefb * iB;
    R Bb = -coefb * coef * iB;
    SKb += Bb;
    Ssb -= Bb;
    // A = K.r (SK - unK)
    Kb.r += Ab * (SK - unK);
    SKb += Ab * K.r;
    unKb -= Ab * K.r;
    R SLb = left ? SKb : R(0), SRb = left ? R(0) : SKb;
    R unLb = left ? unKb : R(0), unRb = left ? R(0) : unKb;
    // Ss = num / den
    R numb = Ssb * iden, denb = -Ssb * Ss * iden;
    Rb.p += numb;
    Lb.p -= numb;
    Lb.r += numb * unL * (SL - unL) + denb * (SL - unL);
    unLb += numb * (L.r * (SL - unL) - L.r * unL) - denb * L.r;
    SLb += numb * L.r * unL + denb * L.r;
    Rb.r -= numb * unR * (SR - unR) + denb * (SR - unR);
    unRb -= numb * (Rt.r * (SR - unR) - Rt.r * unR) - denb * Rt.r;
    SRb -= numb * Rt.r * unR + denb * Rt.r;
    // SL = min(aSL, bSL), SR = max(aSR, bSR)
    R aSLb = (bSL < aSL) ? R(0) : SLb, bSLb = (bSL < aSL) ? SLb : R(0);
    R aSRb = (aSR < bSR) ? R(0) : SRb, bSRb = (aSR < bSR) ? SRb : R(0);
    unLb += aSLb;
    R cLb = -aSLb;
    unRb += aSRb;
    R cRb = aSRb;
    R untb = bSLb + bSRb;
    R ctb = -bSLb + bSRb;
    // ct = sqrt(c2t), c2t = gm (ht - 0.5 (ut^2 + vt^2))
    R c2tb = ctb / (ct + ct);
    R htb = gm * c2tb;
    R utb = -gm * c2tb * ut + untb * nx;
    R vtb = -gm * c2tb * vt + untb * ny;
    // ut = nu_ / S
    R nub = utb * iS, nvb = vtb * iS, nhb = htb * iS;
    R Sb = -(utb * ut + vtb * vt + htb * ht) * iS;
    R sLb = Sb + nub * L.u + nvb * L.v + nhb * hL;
    R sRb = Sb + nub * Rt.u + nvb * Rt.v + nhb * hR;
    Lb.u += nub * sL; Rb.u += nub * sR;
    Lb.v += nvb * sL; Rb.v += nvb * sR;
    R hLb = nhb * sL, hRb = nhb * sR;
    Lb.r += sLb / (sL + sL);
    Rb.r += sRb / (sR + sR);
    Lb.rE += hLb * irL; Lb.p += hLb * irL; Lb.r -= hLb * hL * irL;
    Rb.rE += hRb * irR; Rb.p += hRb * irR; Rb.r -= hRb * hR * irR;
    sound_b(F, L, cL, cLb, Lb);
    sound_b(F, Rt, cR, cRb, Rb);
    Lb.u += unLb * nx; Lb.v += unLb * ny;
    Rb.u += unRb * nx; Rb.v += unRb * ny;
}

template <class R>
CFD_HD void inviscid_flux_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rt, R nx, R ny, const R* Fb, CSb<R>& Lb,
                            CSb<R>& Rb) {
    if (F.flux == FLUX_ROE) flux_roe_b(F, L, Rt, nx, ny, Fb, Lb, Rb);
    else if (F.flux == FLUX_HLLC) flux_hllc_b(F, L, Rt, nx, ny, Fb, Lb, Rb);
    else flux_llf_b(F, L, Rt, nx, ny, Fb, Lb, Rb);
}

// Adjoint of ghost_state: accumulates into the interior state's field adjoints.  With
// SST the ghost's rho k and rho w follow sst_ghost (free stream, extrapolated, or the
// no-slip wall values at the normal distance dwall).
template <class R>
CFD_HD void ghost_state_b(const Flow<R>& F, const CS<R>& U, int tag, R nx, R ny, const CSb<R>& gb_in, CSb<R>& Ub,
                          R dwall = R(0)) {
    const R g = F.gam;
    CS<R> gs = ghost_state(F, U, tag, nx, ny, dwall);
    // adjoints of the ghost's conservative variables
    R cb[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
    cs_back(F, gs, gb_in, cb);
    if (F.sst) {
        // 0 free stream, 1 extrapolated, 2 no-slip wall, -1 copied with the state
        int kind = -1;
        if (F.bcset == BC_BUMP) kind = tag == 1 ? 0 : tag == 2 ? 1 : -1;
        else if (F.bcset == BC_SUPERSONIC) kind = (tag == 1 || tag == 6) ? 0 : -1;
        else kind = tag == 4 ? 2 : -1;
        if (kind >= 0) {
            R kb = cb[4], wb = cb[5];
            cb[4] = cb[5] = R(0);
            if (kind == 0) {
                cb[0] += kb * F.k_inf + wb * F.w_inf;
            } else {
                R ku = U.rk / U.r, wu = U.rw / U.r;
                R kub, wub;
                if (kind == 1) {
                    cb[0] += kb * ku + wb * wu;
                    kub = kb * gs.r;
                    wub = wb * gs.r;
                } else {
                    R d = dwall > R(1e-30) ? dwall : R(1e-30);
                    R ww = R(60.0) * F.nu / (R(0.075) * d * d);
                    cb[0] += -kb * ku + wb * (R(2.0) * ww - wu);
                    kub = -kb * gs.r;
                    wub = -wb * gs.r;
                }
                Ub.rk += kub / U.r;
                Ub.rw += wub / U.r;
                Ub.r -= (kub * ku + wub * wu) / U.r;
            }
        }
    }
    auto slip = [&]() {
        R vn = U.u * nx + U.v * ny;
        R ug = U.u - R(2.0) * vn * nx, vg = U.v - R(2.0) * vn * ny;
        Ub.r += cb[0] + cb[1] * ug + cb[2] * vg;
        R ugb = cb[1] * U.r, vgb = cb[2] * U.r;
        Ub.rE += cb[3];
        Ub.rk += cb[4];
        Ub.rw += cb[5];
        R vnb = -R(2.0) * (ugb * nx + vgb * ny);
        Ub.u += ugb + vnb * nx;
        Ub.v += vgb + vnb * ny;
    };
    auto copy = [&]() {
        Ub.r += cb[0]; Ub.ru += cb[1]; Ub.rv += cb[2]; Ub.rE += cb[3]; Ub.rk += cb[4]; Ub.rw += cb[5];
    };
    if (F.bcset == BC_BUMP) {
        if (tag == 1) {
            R pu = smin(U.p, F.P0 - R(1e-4));
            R e = (g - R(1.0)) / g;
            R Tg = F.T0 * pow(pu / F.P0, e);
            R rg = pu / (F.Rgas * Tg);
            R Cp = g * F.Rgas / (g - R(1.0));
            R V2 = R(2.0) * Cp * (F.T0 - Tg);
            R V = V2 > R(0) ? sqrt(V2) : R(0.0);
            // the ghost's conservative state from p2c(rg, V, 0, pu)
            R rgb = cb[0] + cb[1] * V + cb[3] * R(0.5) * V * V;
            R Vb = cb[1] * rg + cb[3] * rg * V;
            R pub = cb[3] / (g - R(1.0));
            R V2b = V2 > R(0) ? Vb / (V + V) : R(0);
            R Tgb = -R(2.0) * Cp * V2b;
            pub += rgb / (F.Rgas * Tg);
            Tgb -= rgb * rg / Tg;
            pub += Tgb * e * Tg / pu;
            if (!(F.P0 - R(1e-4) < U.p)) Ub.p += pub;
        } else if (tag == 2) {
            // p2c(U.r, U.u, U.v, Pexit)
            Ub.r += cb[0] + cb[1] * U.u + cb[2] * U.v + cb[3] * R(0.5) * (U.u * U.u + U.v * U.v);
            Ub.u += cb[1] * U.r + cb[3] * U.r * U.u;
            Ub.v += cb[2] * U.r + cb[3] * U.r * U.v;
        } else if (tag == 3) {
            slip();
        } else {
            copy();
        }
    } else if (F.bcset == BC_SUPERSONIC) {
        if (tag == 2) copy();
        else if (tag == 3) slip();
        else if (tag != 1 && tag != 6) copy();
    } else {
        if (tag == 1 || tag == 5 || tag == 6) return;
        if (tag == 2) copy();
        else if (tag == 3) slip();
        else if (tag == 4) {
            R ug = -(U.ru / U.r), vg = -(U.rv / U.r);
            R ek = R(0.5) * (U.ru * U.ru + U.rv * U.rv) / U.r;
            R pin = (g - R(1.0)) * (U.rE - ek);
            R Tin = pin / (U.r * F.Rgas);
            R rg = pin / (F.Rgas * Tin);
            // ghost = p2c(rg, ug, vg, pin, 0, 0)
            R rgb = cb[0] + cb[1] * ug + cb[2] * vg + cb[3] * R(0.5) * (ug * ug + vg * vg);
            R ugb = cb[1] * rg + cb[3] * rg * ug;
            R vgb = cb[2] * rg + cb[3] * rg * vg;
            R pinb = cb[3] / (g - R(1.0));
            // rg = pin / (R Tin), Tin = pin / (U.r R)
            pinb += rgb / (F.Rgas * Tin);
            R Tinb = -rgb * rg / Tin;
            pinb += Tinb / (U.r * F.Rgas);
            Ub.r -= Tinb * Tin / U.r;
            // pin = (g-1)(rE - ek), ek = 0.5 (ru^2 + rv^2) / r
            Ub.rE += pinb * (g - R(1.0));
            R ekb = -pinb * (g - R(1.0));
            Ub.ru += ekb * U.ru / U.r;
            Ub.rv += ekb * U.rv / U.r;
            Ub.r -= ekb * ek / U.r;
            // ug = -(ru / r)
            Ub.ru -= ugb / U.r;
            Ub.r += ugb * U.ru / (U.r * U.r);
            Ub.rv -= vgb / U.r;
            Ub.r += vgb * U.rv / (U.r * U.r);
        } else {
            copy();
        }
    }
}

// Adjoint of reconstruct(): into the side's state field adjoints, its gradient adjoints
// and its limiter adjoint
template <class R>
CFD_HD void reconstruct_b(const Flow<R>& F, const CS<R>& C, const R* g, R ph, R dx, R dy, const CSb<R>& ob,
                          CSb<R>& Cb, R* gb, R& phb) {
    R sr = g[FG_R] * dx + g[FG_R + 1] * dy;
    R sp = g[FG_P] * dx + g[FG_P + 1] * dy;
    R su = g[FG_U] * dx + g[FG_U + 1] * dy;
    R sv = g[FG_V] * dx + g[FG_V + 1] * dy;
    R rf = C.r + ph * sr, pf = C.p + ph * sp, uf = C.u + ph * su, vf = C.v + ph * sv;
    bool cr = rf < R(1e-4), cp = pf < R(1e-4);
    if (cr) rf = C.r;
    if (cp) pf = C.p;
    R rfb = 0, ufb = 0, vfb = 0, pfb = 0;
    p2c_b(F, rf, uf, vf, pf, ob, rfb, ufb, vfb, pfb);
    Cb.r += rfb;
    Cb.p += pfb;
    Cb.u += ufb;
    Cb.v += vfb;
    if (!cr) {
        phb += rfb * sr;
        gb[FG_R] += rfb * ph * dx;
        gb[FG_R + 1] += rfb * ph * dy;
    }
    if (!cp) {
        phb += pfb * sp;
        gb[FG_P] += pfb * ph * dx;
        gb[FG_P + 1] += pfb * ph * dy;
    }
    phb += ufb * su + vfb * sv;
    gb[FG_U] += ufb * ph * dx;
    gb[FG_U + 1] += ufb * ph * dy;
    gb[FG_V] += vfb * ph * dx;
    gb[FG_V + 1] += vfb * ph * dy;
}

// Adjoint of face_flux.  FAb: adjoint of the face's F*A (6 entries, unused ones zero).
// Accumulates into the owner's field adjoints Lb, the neighbour's Rnb (interior only),
// the 10 gradient adjoints of each side and the limiter adjoints.
template <class R>
CFD_HD void face_flux_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rn, bool interior, int tag,
                        const FaceGeo<R>& g, const R* gL, const R* gR, R phL, R phR, const R* FAb, CSb<R>& Lb,
                        CSb<R>& Rnb, R* gLb, R* gRb, R& phLb, R& phRb, R mutf = R(0), R* mutfb = nullptr) {
    const R nx = g.nx, ny = g.ny;
    R TFb[6];
    for (int c = 0; c < 6; ++c) TFb[c] = FAb[c] * g.A;
    CS<R> Rt = face_right(F, L, Rn, interior, tag, nx, ny);
    CSb<R> Rtb = csb_zero<R>();
    // viscous part: TF = FE - FV
    if (F.viscous) {
        const R* gRv = interior ? gR : gL;
        R* gRvb = interior ? gRb : gLb;
        R rf = R(0.5) * (L.r + Rt.r);
        R uf = R(0.5) * (L.u + Rt.u);
        R vf = R(0.5) * (L.v + Rt.v);
        bool wall = !interior && tag == 4;
        R dx = g.dxL, dy = g.dyL, d2w = dx * dx + dy * dy;
        R a0, b0, c0, e0, dTdx, dTdy;
        // |x_R - x_L|^2 and its reciprocal: formed once per mesh (FaceGeo d2lr, id2lr)
        bool corr = !wall && g.d2lr > R(1e-14);
        const R id2w = wall ? R(1) / d2w : R(0), id2 = corr ? g.id2lr : R(0);
        R du = Rt.u - L.u, dv = Rt.v - L.v;
        R dudx, dudy, dvdx, dvdy;
        if (wall) {
            a0 = b0 = c0 = e0 = R(0);
            dudx = -L.u * dx * id2w;
            dudy = -L.u * dy * id2w;
            dvdx = -L.v * dx * id2w;
            dvdy = -L.v * dy * id2w;
            dTdx = dTdy = R(0);
        } else {
            a0 = R(0.5) * (gL[FG_U] + gRv[FG_U]);
            b0 = R(0.5) * (gL[FG_U + 1] + gRv[FG_U + 1]);
            c0 = R(0.5) * (gL[FG_V] + gRv[FG_V]);
            e0 = R(0.5) * (gL[FG_V + 1] + gRv[FG_V + 1]);
            dTdx = R(0.5) * (gL[FG_T] + gRv[FG_T]);
            dTdy = R(0.5) * (gL[FG_T + 1] + gRv[FG_T + 1]);
            dudx = a0; dudy = b0; dvdx = c0; dvdy = e0;
            if (corr) {
                R cu = (a0 * g.dxlr + b0 * g.dylr - du) * id2, cv = (c0 * g.dxlr + e0 * g.dylr - dv) * id2;
                dudx = a0 - cu * g.dxlr;
                dudy = b0 - cu * g.dylr;
                dvdx = c0 - cv * g.dxlr;
                dvdy = e0 - cv * g.dylr;
            }
        }
        R Cp = F.gam * F.Rgas / (F.gam - R(1.0));
        const R CpPr = Cp * F.inv_Pr, CpPrt = Cp * F.inv_Prt;
        R mu = rf * F.nu;
        R kc = mu * CpPr;
        if (F.sst) {
            kc = kc + mutf * CpPrt;
            mu = mu + mutf;
        }
        R div = dudx + dvdy;
        R txx = mu * (R(2.0) * dudx - (R(2.0) / R(3.0)) * div);
        R tyy = mu * (R(2.0) * dvdy - (R(2.0) / R(3.0)) * div);
        R txy = mu * (dudy + dvdx);
        // FV = (0, txx nx + txy ny, txy nx + tyy ny, wx nx + wy ny); TF -= FV
        R FVb1 = -TFb[1], FVb2 = -TFb[2], FVb3 = -TFb[3];
        R wxb = FVb3 * nx, wyb = FVb3 * ny;
        R txxb = FVb1 * nx + wxb * uf;
        R txyb = FVb1 * ny + FVb2 * nx + wxb * vf + wyb * uf;
        R tyyb = FVb2 * ny + wyb * vf;
        R ufb = wxb * txx + wyb * txy;
        R vfb = wxb * txy + wyb * tyy;
        R qxb = -wxb, qyb = -wyb;
        R kcb = -qxb * dTdx - qyb * dTdy;
        R dTdxb = -qxb * kc, dTdyb = -qyb * kc;
        // mu (and kc) of the stresses include mu_t with SST; the laminar part is rf nu
        R mufb = txxb * (R(2.0) * dudx - (R(2.0) / R(3.0)) * div) + tyyb * (R(2.0) * dvdy - (R(2.0) / R(3.0)) * div) +
                 txyb * (dudy + dvdx);
        R mub = kcb * CpPr + mufb;
        if (F.sst && mutfb) *mutfb += mufb + kcb * CpPrt;
        R divb = -(R(2.0) / R(3.0)) * mu * (txxb + tyyb);
        R dudxb = R(2.0) * mu * txxb + divb;
        R dvdyb = R(2.0) * mu * tyyb + divb;
        R dudyb = mu * txyb, dvdxb = mu * txyb;
        R rfb = mub * F.nu;
        Lb.r += R(0.5) * rfb;
        Rtb.r += R(0.5) * rfb;
        Lb.u += R(0.5) * ufb;
        Rtb.u += R(0.5) * ufb;
        Lb.v += R(0.5) * vfb;
        Rtb.v += R(0.5) * vfb;
        if (wall) {
            Lb.u -= (dudxb * dx + dudyb * dy) * id2w;
            Lb.v -= (dvdxb * dx + dvdyb * dy) * id2w;
        } else {
            R a0b = dudxb, b0b = dudyb, c0b = dvdxb, e0b = dvdyb;
            if (corr) {
                // dudx = a0 - cu dxlr, dudy = b0 - cu dylr with cu = (a0 dxlr + b0 dylr - du) / d2
                R cub = -(dudxb * g.dxlr + dudyb * g.dylr) * id2;
                R cvb = -(dvdxb * g.dxlr + dvdyb * g.dylr) * id2;
                a0b += cub * g.dxlr;
                b0b += cub * g.dylr;
                R dub_ = -cub;
                c0b += cvb * g.dxlr;
                e0b += cvb * g.dylr;
                R dvb_ = -cvb;
                Rtb.u += dub_;
                Lb.u -= dub_;
                Rtb.v += dvb_;
                Lb.v -= dvb_;
            }
            gLb[FG_U] += R(0.5) * a0b;
            gRvb[FG_U] += R(0.5) * a0b;
            gLb[FG_U + 1] += R(0.5) * b0b;
            gRvb[FG_U + 1] += R(0.5) * b0b;
            gLb[FG_V] += R(0.5) * c0b;
            gRvb[FG_V] += R(0.5) * c0b;
            gLb[FG_V + 1] += R(0.5) * e0b;
            gRvb[FG_V + 1] += R(0.5) * e0b;
            gLb[FG_T] += R(0.5) * dTdxb;
            gRvb[FG_T] += R(0.5) * dTdxb;
            gLb[FG_T + 1] += R(0.5) * dTdyb;
            gRvb[FG_T + 1] += R(0.5) * dTdyb;
        }
    }
    // inviscid part
    bool second = F.spatial != SP_FIRST && interior;
    R pl = F.spatial == SP_LIMITED ? phL : R(0.5);
    R pr = F.spatial == SP_LIMITED ? phR : R(0.5);
    CS<R> Lr = second ? reconstruct(F, L, gL, pl, g.dxL, g.dyL) : L;
    CS<R> Rr = second ? reconstruct(F, Rt, gR, pr, g.dxR, g.dyR) : Rt;
    CSb<R> Lrb = csb_zero<R>(), Rrb = csb_zero<R>();
    if (!interior && (tag == 3 || tag == 4)) {
        Lrb.p += TFb[1] * nx + TFb[2] * ny;
    } else {
        inviscid_flux_b(F, Lr, Rr, nx, ny, TFb, Lrb, Rrb);
    }
    if (second) {
        R plb = 0, prb = 0;
        reconstruct_b(F, L, gL, pl, g.dxL, g.dyL, Lrb, Lb, gLb, plb);
        reconstruct_b(F, Rt, gR, pr, g.dxR, g.dyR, Rrb, Rtb, gRb, prb);
        if (F.spatial == SP_LIMITED) {
            phLb += plb;
            phRb += prb;
        }
    } else {
        Lb.r += Lrb.r; Lb.ru += Lrb.ru; Lb.rv += Lrb.rv; Lb.rE += Lrb.rE; Lb.rk += Lrb.rk; Lb.rw += Lrb.rw;
        Lb.u += Lrb.u; Lb.v += Lrb.v; Lb.p += Lrb.p;
        Rtb.r += Rrb.r; Rtb.ru += Rrb.ru; Rtb.rv += Rrb.rv; Rtb.rE += Rrb.rE; Rtb.rk += Rrb.rk; Rtb.rw += Rrb.rw;
        Rtb.u += Rrb.u; Rtb.v += Rrb.v; Rtb.p += Rrb.p;
    }
    // the right state: neighbour or ghost of L
    if (interior) {
        Rnb.r += Rtb.r; Rnb.ru += Rtb.ru; Rnb.rv += Rtb.rv; Rnb.rE += Rtb.rE; Rnb.rk += Rtb.rk; Rnb.rw += Rtb.rw;
        Rnb.u += Rtb.u; Rnb.v += Rtb.v; Rnb.p += Rtb.p;
    } else {
        ghost_state_b(F, L, tag, nx, ny, Rtb, Lb);
    }
}

// Adjoint of face_flux_sst.  Besides face_flux_b's outputs: the adjoints of each side's
// k, w gradients (gkLb, gkRb: k_x, k_y, w_x, w_y), mu_t and F1.  On the boundary all of
// the right-hand ones are folded into the owner's.
template <class R>
CFD_HD void face_flux_sst_b(const Flow<R>& F, const CS<R>& L, const CS<R>& Rn, bool interior, int tag,
                            const FaceGeo<R>& g, const R* gL, const R* gR, const R* gkL, const R* gkR, R phL, R phR,
                            R mutL, R mutR, R F1L, R F1R, const R* FAb_in, CSb<R>& Lb, CSb<R>& Rnb, R* gLb, R* gRb,
                            R* gkLb, R* gkRb, R& phLb, R& phRb, R& mutLb, R& mutRb, R& F1Lb, R& F1Rb) {
    bool wall = !interior && tag == 4;
    if (!interior) {
        mutR = mutL;
        F1R = F1L;
    }
    R mutf = wall ? R(0) : R(0.5) * (mutL + mutR);
    R F1f = R(0.5) * (F1L + F1R);
    R dwl = wall_normal_distance(g);
    Flux6<R> out = face_flux(F, L, Rn, interior, tag, g, gL, gR, phL, phR, mutf);
    CS<R> Rt = face_right(F, L, Rn, interior, tag, g.nx, g.ny, dwl);
    const R* gkRv = interior ? gkR : gkL;
    R gkRvb[4] = {R(0), R(0), R(0), R(0)};
    R kL = L.rk / L.r, wL = L.rw / L.r, kR = Rt.rk / Rt.r, wR = Rt.rw / Rt.r;
    R mdotAb = 0, kLb = 0, wLb = 0, kRb = 0, wRb = 0, rfb = 0, mutfb = 0, F1fb = 0;
    sst_face_flux_b(F, out.f[0], kL, wL, kR, wR, R(0.5) * (L.r + Rt.r), mutf, F1f, gkL, gkRv, wall, g.nx, g.ny, g.A,
                    g.dxL, g.dyL, g.dxlr, g.dylr, g.d2lr, g.id2lr, FAb_in[4], FAb_in[5], mdotAb, kLb, wLb, kRb, wRb, rfb, mutfb, F1fb,
                    gkLb, gkRvb);
    // the mean flow, with the k and w rows' mass-flux adjoint added to row 0
    R FAb[6] = {FAb_in[0] + mdotAb, FAb_in[1], FAb_in[2], FAb_in[3], R(0), R(0)};
    face_flux_b(F, L, Rn, interior, tag, g, gL, gR, phL, phR, FAb, Lb, Rnb, gLb, gRb, phLb, phRb, mutf, &mutfb);
    // k = rho k / rho of both sides, and rf = (rho_L + rho_R) / 2
    Lb.rk += kLb / L.r;
    Lb.rw += wLb / L.r;
    Lb.r += R(0.5) * rfb - (kLb * kL + wLb * wL) / L.r;
    CSb<R> RtSb = csb_zero<R>();
    RtSb.rk = kRb / Rt.r;
    RtSb.rw = wRb / Rt.r;
    RtSb.r = R(0.5) * rfb - (kRb * kR + wRb * wR) / Rt.r;
    if (interior) {
        Rnb.r += RtSb.r;
        Rnb.rk += RtSb.rk;
        Rnb.rw += RtSb.rw;
    } else {
        ghost_state_b(F, L, tag, g.nx, g.ny, RtSb, Lb, dwl);
    }
    R mb = wall ? R(0) : R(0.5) * mutfb;
    R fb = R(0.5) * F1fb;
    if (interior) {
        mutLb += mb;
        mutRb += mb;
        F1Lb += fb;
        F1Rb += fb;
        for (int q = 0; q < 4; ++q) gkRb[q] += gkRvb[q];
    } else {
        mutLb += mb + mb;
        F1Lb += fb + fb;
        for (int q = 0; q < 4; ++q) gkLb[q] += gkRvb[q];
    }
}

}  // namespace cfdg
