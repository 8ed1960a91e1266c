// Test-only host build of the residual's face function (face.cuh) and its hand-written
// adjoint (adjoint.cuh), so the adjoint can be checked against finite differences of the
// same operation sequence on the CPU.  Not part of the library.
#include <cstring>

#include "../../mycode_gb300/csrc/adjoint.cuh"

using namespace cfdg;

namespace {
Flow<double> flow(const double* p, const int* fl) {
    Flow<double> F;
    F.gam = p[0]; F.Rgas = p[1]; F.Pr = p[2]; F.nu = p[3]; F.Minf = p[4]; F.P0 = p[5]; F.T0 = p[6]; F.Pexit = p[7];
    for (int k = 0; k < 4; ++k) { F.fs[k] = p[8 + k]; F.shock[k] = p[12 + k]; }
    F.k_inf = 0; F.w_inf = 0; F.Pr_t = 0.9;
    flow_derived(F);
    F.bcset = fl[0]; F.flux = fl[1]; F.spatial = fl[2]; F.viscous = fl[3];
    return F;
}
FaceGeo<double> geo(const double* g) {
    FaceGeo<double> G;
    G.nx = g[0]; G.ny = g[1]; G.A = g[2]; G.dxL = g[3]; G.dyL = g[4]; G.dxR = g[5]; G.dyR = g[6];
    G.dxlr = g[7]; G.dylr = g[8];
    geo_derived(G);
    return G;
}
CS<double> cs(const Flow<double>& F, const double* U) { return make_cs(F, U[0], U[1], U[2], U[3], U[4], U[5]); }
}  // namespace

extern "C" {

// quot_by_recip (physics.cuh) against IEEE division on n pairs: a = m_a 2^ea, b = m_b 2^eb
// from the given significand and exponent arrays; returns the number of pairs whose bits
// differ
long quot_mismatches(long n, const double* a, const double* b) {
    long bad = 0;
    for (long i = 0; i < n; ++i) {
        const double q = quot_by_recip(a[i], b[i], 1.0 / b[i]), ref = a[i] / b[i];
        if (std::memcmp(&q, &ref, sizeof(double)) != 0) ++bad;
    }
    return bad;
}

// fl: bcset, flux, spatial, viscous, interior, tag
void face_eval(const double* p, const int* fl, const double* g, const double* UL, const double* UR, const double* gL,
               const double* gR, double phL, double phR, double* out) {
    Flow<double> F = flow(p, fl);
    Flux6<double> o = face_flux(F, cs(F, UL), cs(F, UR), fl[4] != 0, fl[5], geo(g), gL, gR, phL, phR);
    for (int c = 0; c < 6; ++c) out[c] = o.f[c];
}

void face_adj(const double* p, const int* fl, const double* g, const double* UL, const double* UR, const double* gL,
              const double* gR, double phL, double phR, const double* FAb, double* ULb, double* URb, double* gLb,
              double* gRb, double* phb) {
    Flow<double> F = flow(p, fl);
    CS<double> L = cs(F, UL), Rn = cs(F, UR);
    CSb<double> Lb = csb_zero<double>(), Rb = csb_zero<double>();
    for (int q = 0; q < 10; ++q) { gLb[q] = 0; gRb[q] = 0; }
    phb[0] = phb[1] = 0;
    face_flux_b(F, L, Rn, fl[4] != 0, fl[5], geo(g), gL, gR, phL, phR, FAb, Lb, Rb, gLb, gRb, phb[0], phb[1]);
    for (int c = 0; c < 6; ++c) { ULb[c] = 0; URb[c] = 0; }
    cs_back(F, L, Lb, ULb);
    cs_back(F, Rn, Rb, URb);
}

// ---- SST (nv = 6): p[16], p[17] = k_inf, w_inf; t = mu_t,L, mu_t,R, F1_L, F1_R
void sst_face_eval(const double* p, const int* fl, const double* g, const double* UL, const double* UR,
                   const double* gL, const double* gR, const double* gkL, const double* gkR, double phL, double phR,
                   const double* t, double* out) {
    Flow<double> F = flow(p, fl);
    F.sst = 1; F.k_inf = p[16]; F.w_inf = p[17];
    const double kw[4] = {UL[4] / UL[0], UL[5] / UL[0], UR[4] / UR[0], UR[5] / UR[0]};
    Flux6<double> o = face_flux_sst(F, cs(F, UL), cs(F, UR), fl[4] != 0, fl[5], geo(g), gL, gR, gkL, gkR, phL, phR,
                                    t[0], t[1], t[2], t[3], kw, kw + 2);
    for (int c = 0; c < 6; ++c) out[c] = o.f[c];
}

void sst_face_adj(const double* p, const int* fl, const double* g, const double* UL, const double* UR,
                  const double* gL, const double* gR, const double* gkL, const double* gkR, double phL, double phR,
                  const double* t, const double* FAb, double* ULb, double* URb, double* gLb, double* gRb,
                  double* gkLb, double* gkRb, double* phb, double* tb) {
    Flow<double> F = flow(p, fl);
    F.sst = 1; F.k_inf = p[16]; F.w_inf = p[17];
    CS<double> L = cs(F, UL), Rn = cs(F, UR);
    CSb<double> Lb = csb_zero<double>(), Rb = csb_zero<double>();
    for (int q = 0; q < 10; ++q) { gLb[q] = 0; gRb[q] = 0; }
    for (int q = 0; q < 4; ++q) { gkLb[q] = 0; gkRb[q] = 0; tb[q] = 0; }
    phb[0] = phb[1] = 0;
    face_flux_sst_b(F, L, Rn, fl[4] != 0, fl[5], geo(g), gL, gR, gkL, gkR, phL, phR, t[0], t[1], t[2], t[3], FAb, Lb,
                    Rb, gLb, gRb, gkLb, gkRb, phb[0], phb[1], tb[0], tb[1], tb[2], tb[3]);
    for (int c = 0; c < 6; ++c) { ULb[c] = 0; URb[c] = 0; }
    cs_back(F, L, Lb, ULb);
    cs_back(F, Rn, Rb, URb);
}

// x = rho, k, w, u_x, u_y, v_x, v_y, k_x, k_y, w_x, w_y, d -> mu_t, F1, S_k, S_w
void sst_cell_eval(const double* p, const double* x, double* out) {
    int fl[4] = {2, 0, 1, 1};
    Flow<double> F = flow(p, fl);
    F.sst = 1; F.k_inf = p[16]; F.w_inf = p[17];
    SstCell<double> c = sst_cell(F, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9], x[10], x[11]);
    out[0] = c.mut; out[1] = c.F1; out[2] = c.Sk; out[3] = c.Sw;
}

void sst_cell_adj(const double* p, const double* x, const double* ob, double* xb) {
    int fl[4] = {2, 0, 1, 1};
    Flow<double> F = flow(p, fl);
    F.sst = 1; F.k_inf = p[16]; F.w_inf = p[17];
    for (int q = 0; q < 11; ++q) xb[q] = 0;
    const double idd = 1.0 / (x[11] > 1e-30 ? x[11] : 1e-30);
    sst_cell_b(F, x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7], x[8], x[9], x[10], idd, ob[0], ob[1], ob[2],
               ob[3], xb[0], xb[1], xb[2], xb[3], xb[4], xb[5], xb[6], xb[7], xb[8], xb[9], xb[10]);
}

}  // extern "C"
