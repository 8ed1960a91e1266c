// Adjoint (VJP) of the full residual: gU = (dR/dU)^T lambda, FP64.
//
// After a forward recomputation of W, G and phi (k_prim, k_grad with the limiter), three
// kernels, all deterministic (no atomics, every sum in a fixed order):
//   k_flux_adj   per face: reverse of face_flux; writes the owner's and the neighbour's
//                contributions (conservative adjoints, 10 gradient adjoints, limiter
//                adjoint) into two face-side slots
//   k_adj_cell1  per cell: gathers its face-side slots; reverse of the Barth-Jespersen
//                limiter along the forward's argmin/argmax (src/Solver.cpp:152-253);
//                reverse of the Green-Gauss gradient for the cell's own half of every face
//                (ghost halves go back through the ghost state); stores the gradient
//                accumulator adjoint for the neighbours
//   k_adj_cell2  per cell: the neighbours' halves of the Green-Gauss reverse and the
//                limiter pressure adjoints that chose this cell, folded into gU
// With SST (NV = 6) the face kernel also reverses the k and w fluxes (sst_face_flux_b)
// and the face eddy viscosity, the face slots carry the adjoints of the cell's mu_t and
// F1, the first cell kernel reverses the cell's model terms (sst_cell_b) and the Green-
// Gauss reverse runs over seven quantities (rho, u, v, p, T, k, w).
#pragma once
#include "adjoint.cuh"
#include "residual.cuh"

namespace cfdg {

// face-side slots: cons (NV), gradients (10, or 14 with SST), phi, and with SST mu_t, F1
template <int NV> struct AdjSlot {
    static constexpr int G = Planes<NV>::G;
    static constexpr int PHI = NV + G;
    static constexpr int MUT = PHI + 1, F1 = PHI + 2;
    static constexpr int N = NV == 6 ? PHI + 3 : PHI + 1;
};

struct AdjBufs {
    double* fb0;       // [N][nf] owner-side slots
    double* fb1;       // [N][nf] neighbour-side slots
    double* gpart;     // [NV][nc] gU without the neighbours' contributions
    double* accb;      // [G][nc] adjoint of the gradient accumulators (G = acc / vol)
    double* pmaxb;     // [nc] adjoint of the cell's pmax
    double* pminb;     // [nc]
    int* pmax_face;    // [nc] face whose neighbour pressure set pmax (-1: own or ghost)
    int* pmin_face;    // [nc]
};

template <int NV>
__global__ void __launch_bounds__(128) k_flux_adj(MeshView<double> m, Flow<double> F, Field<double> U,
                                                  Field<double> W, Field<double> G, const double* __restrict__ phi,
                                                  const double* __restrict__ lam, AdjBufs b, Field<double> T) {
    typedef AdjSlot<NV> SL;
    long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    long nc = m.nc, nf = m.nf;
    int o = m.fo[f], n = m.fn[f];
    bool interior = n >= 0;
    int tag = interior ? 0 : m.ftag[f];
    FaceGeo<double> g = load_geo(m, f);
    CS<double> L = load_cs<double, NV>(U, W, o);
    CS<double> Rn = interior ? load_cs<double, NV>(U, W, n) : L;
    double gL[10], gR[10];
    for (int q = 0; q < 10; ++q) { gL[q] = 0.0; gR[q] = 0.0; }
    if ((F.spatial != SP_FIRST && interior) || F.viscous) {
        load_grad<double, NV>(G, o, gL);
        if (interior) load_grad<double, NV>(G, n, gR);
    }
    double phL = 1.0, phR = 1.0;
    if (F.spatial == SP_LIMITED && interior) {
        phL = phi[o];
        phR = phi[n];
    }
    double FAb[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < NV; ++c) FAb[c] = lam[c * nc + o] - (interior ? lam[c * nc + n] : 0.0);
    CSb<double> Lb = csb_zero<double>(), Rnb = csb_zero<double>();
    double gLb[10], gRb[10], phLb = 0.0, phRb = 0.0;
    for (int q = 0; q < 10; ++q) { gLb[q] = 0.0; gRb[q] = 0.0; }
    double gkLb[4] = {0, 0, 0, 0}, gkRb[4] = {0, 0, 0, 0};
    double mutLb = 0.0, mutRb = 0.0, F1Lb = 0.0, F1Rb = 0.0;
    if constexpr (NV == 6) {
        double gk[8] = {G.v[G_K * nc + o], G.v[(G_K + 1) * nc + o], G.v[G_W * nc + o], G.v[(G_W + 1) * nc + o],
                        0.0, 0.0, 0.0, 0.0};
        double mutR = 0.0, F1R = 0.0;
        if (interior) {
            gk[4] = G.v[G_K * nc + n];
            gk[5] = G.v[(G_K + 1) * nc + n];
            gk[6] = G.v[G_W * nc + n];
            gk[7] = G.v[(G_W + 1) * nc + n];
            mutR = T.v[n];
            F1R = T.v[nc + n];
        }
        face_flux_sst_b(F, L, Rn, interior, tag, g, gL, gR, gk, gk + 4, phL, phR, T.v[o], mutR, T.v[nc + o], F1R, FAb,
                        Lb, Rnb, gLb, gRb, gkLb, gkRb, phLb, phRb, mutLb, mutRb, F1Lb, F1Rb);
    } else {
        face_flux_b(F, L, Rn, interior, tag, g, gL, gR, phL, phR, FAb, Lb, Rnb, gLb, gRb, phLb, phRb);
    }
    double uL[6] = {0, 0, 0, 0, 0, 0}, uR[6] = {0, 0, 0, 0, 0, 0};
    cs_back(F, L, Lb, uL);
    if (interior) cs_back(F, Rn, Rnb, uR);
    for (int c = 0; c < NV; ++c) {
        b.fb0[c * nf + f] = uL[c];
        b.fb1[c * nf + f] = uR[c];
    }
    for (int q = 0; q < 10; ++q) {
        b.fb0[(NV + q) * nf + f] = gLb[q];
        b.fb1[(NV + q) * nf + f] = gRb[q];
    }
    b.fb0[SL::PHI * nf + f] = phLb;
    b.fb1[SL::PHI * nf + f] = phRb;
    if constexpr (NV == 6) {
        for (int q = 0; q < 4; ++q) {
            b.fb0[(NV + 10 + q) * nf + f] = gkLb[q];
            b.fb1[(NV + 10 + q) * nf + f] = gkRb[q];
        }
        b.fb0[SL::MUT * nf + f] = mutLb;
        b.fb1[SL::MUT * nf + f] = mutRb;
        b.fb0[SL::F1 * nf + f] = F1Lb;
        b.fb1[SL::F1 * nf + f] = F1Rb;
    }
}

// (rho, u, v, p, T[, k, w]) adjoints of a state -> its CS field adjoints
// (T = p / (rho R), k = rho k / rho, w = rho w / rho)
template <int NQ>
__device__ __forceinline__ void w_to_csb(const Flow<double>& F, double r, double p, double rk, double rw,
                                         const double* wb, CSb<double>& cb) {
    const double ir = 1.0 / r, irR = ir / F.Rgas;
    double T = p * irR;
    cb.r += wb[W_R] - wb[W_T] * T * ir;
    cb.u += wb[W_U];
    cb.v += wb[W_V];
    cb.p += wb[W_P] + wb[W_T] * irR;
    if constexpr (NQ == 7) {
        cb.rk += wb[W_K] * ir;
        cb.rw += wb[W_W] * ir;
        cb.r -= (wb[W_K] * rk + wb[W_W] * rw) * ir * ir;
    }
}

template <int NV>
__global__ void __launch_bounds__(128) k_adj_cell1(MeshView<double> m, Flow<double> F, Field<double> U,
                                                   Field<double> W, Field<double> G, const double* __restrict__ phi,
                                                   int limited, AdjBufs b, const double* __restrict__ lam,
                                                   const double* __restrict__ dwall) {
    typedef AdjSlot<NV> SL;
    constexpr int NG = SL::G, NQ = NG / 2;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    long nc = m.nc, nf = m.nf;
    double ub[6] = {0, 0, 0, 0, 0, 0}, gb[NG], phb = 0.0, mutb = 0.0, F1b = 0.0;
    for (int q = 0; q < NG; ++q) gb[q] = 0.0;
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        long f = e >> 1;
        const double* s = (e & 1) ? b.fb1 : b.fb0;
        for (int c = 0; c < NV; ++c) ub[c] += s[c * nf + f];
        for (int q = 0; q < NG; ++q) gb[q] += s[(NV + q) * nf + f];
        phb += s[SL::PHI * nf + f];
        if constexpr (NV == 6) {
            mutb += s[SL::MUT * nf + f];
            F1b += s[SL::F1 * nf + f];
        }
    }
    CS<double> Ui = load_cs<double, NV>(U, W, i);
    CSb<double> cb = csb_zero<double>();
    double wi[NQ];
    for (int q = 0; q < NQ; ++q) wi[q] = W.v[q * nc + i];
    double wb[NQ];
    for (int q = 0; q < NQ; ++q) wb[q] = 0.0;
    if constexpr (NV == 6) {
        // the cell's model terms: R_k -= S_k vol, R_w -= S_w vol
        double vol = m.vol[i];
        double Skb = -lam[4 * nc + i] * vol, Swb = -lam[5 * nc + i] * vol;
        const double* Gi = G.v;
        sst_cell_b(F, wi[W_R], wi[W_K], wi[W_W], Gi[G_U * nc + i], Gi[(G_U + 1) * nc + i], Gi[G_V * nc + i],
                   Gi[(G_V + 1) * nc + i], Gi[G_K * nc + i], Gi[(G_K + 1) * nc + i], Gi[G_W * nc + i],
                   Gi[(G_W + 1) * nc + i], dwall[nc + i], mutb, F1b, Skb, Swb, wb[W_R], wb[W_K], wb[W_W], gb[G_U],
                   gb[G_U + 1], gb[G_V], gb[G_V + 1], gb[G_K], gb[G_K + 1], gb[G_W], gb[G_W + 1]);
    }
    double pmaxb = 0.0, pminb = 0.0;
    int pmax_face = -1, pmin_face = -1;
    if (limited && phb != 0.0) {
        // forward Barth-Jespersen with the selections recorded
        const double eps = 1e-12;
        double pc = wi[W_P], rho = wi[W_R], Tc = wi[W_T];
        double gTx = G.v[G_T * nc + i], gTy = G.v[(G_T + 1) * nc + i];
        double pmax = pc, pmin = pc;
        int amax = -1, amin = -1;  // k of the face, -1 = the cell itself
        for (int k = 0; k < 4; ++k) {
            int e = m.cf[(long)k * nc + i];
            if (e < 0) break;
            int f = e >> 1, side = e & 1;
            int j = side ? m.fo[f] : m.fn[f];
            double pj;
            if (j >= 0) pj = W.v[W_P * nc + j];
            else pj = ghost_state(F, Ui, m.ftag[f], m.nx[f], m.ny[f]).p;
            if (pmax < pj) { pmax = pj; amax = k; }
            if (pj < pmin) { pmin = pj; amin = k; }
        }
        double lim = 1.0;
        int win = -1;
        bool win_ratio = false;
        double win_d2 = 0.0, win_a = 0.0, win_dx = 0.0, win_dy = 0.0;
        for (int k = 0; k < 4; ++k) {
            int e = m.cf[(long)k * nc + i];
            if (e < 0) break;
            int f = e >> 1, side = e & 1;
            double dx = side ? m.dxn[f] : m.dxo[f];
            double dy = side ? m.dyn[f] : m.dyo[f];
            double Tf = Tc + 1.0 * (gTx * dx + gTy * dy);
            double Pf = rho * F.Rgas * Tf;
            double d2 = Pf - pc;
            double a = 1.0;
            bool ratio = false;
            // as the forward: the divide only where the ratio can be below one
            if (d2 > 0.0) {
                if (!(pmax - pc >= d2 + eps)) {
                    double r = (pmax - pc) / (d2 + eps);
                    ratio = r < 1.0;
                    a = ratio ? r : 1.0;
                }
            } else if (d2 < 0.0) {
                if (!(pmin - pc <= d2 - eps)) {
                    double r = (pmin - pc) / (d2 - eps);
                    ratio = r < 1.0;
                    a = ratio ? r : 1.0;
                }
            }
            if (a < lim) {
                lim = a;
                win = k;
                win_ratio = ratio;
                win_d2 = d2;
                win_a = a;
                win_dx = dx;
                win_dy = dy;
            }
        }
        if (win >= 0 && win_ratio) {
            double ab = phb;
            double den = win_d2 > 0.0 ? win_d2 + eps : win_d2 - eps;
            const double iden = 1.0 / den;
            double extb = ab * iden;  // adjoint of pmax (or pmin)
            double pcb = -ab * iden;
            double d2b = -ab * win_a * iden;
            double Pfb = d2b;
            pcb -= d2b;
            wb[W_R] += Pfb * F.Rgas * (Tc + 1.0 * (gTx * win_dx + gTy * win_dy));
            double Tfb = Pfb * rho * F.Rgas;
            wb[W_T] += Tfb;
            gb[G_T] += Tfb * win_dx;
            gb[G_T + 1] += Tfb * win_dy;
            wb[W_P] += pcb;
            int a_k = win_d2 > 0.0 ? amax : amin;
            if (a_k < 0) {
                wb[W_P] += extb;
            } else {
                int e = m.cf[(long)a_k * nc + i];
                int f = e >> 1, side = e & 1;
                int j = side ? m.fo[f] : m.fn[f];
                if (j >= 0) {
                    if (win_d2 > 0.0) { pmaxb = extb; pmax_face = f; }
                    else { pminb = extb; pmin_face = f; }
                } else {
                    CSb<double> gsb = csb_zero<double>();
                    gsb.p = extb;
                    ghost_state_b(F, Ui, m.ftag[f], m.nx[f], m.ny[f], gsb, cb);
                }
            }
        }
    }
    // Green-Gauss reverse, own half of every face (G = acc / vol)
    const double ivol = m.ivol[i];  // 1 / vol, formed once per mesh
    double accb[NG];
    for (int q = 0; q < NG; ++q) {
        accb[q] = gb[q] * ivol;
        b.accb[q * nc + i] = accb[q];
    }
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        int f = e >> 1, side = e & 1;
        double nx = m.nx[f], ny = m.ny[f], A = m.area[f];
        double sgn_ = side ? -1.0 : 1.0;
        double phbq[NQ];
        for (int q = 0; q < NQ; ++q) phbq[q] = sgn_ * (accb[2 * q] * nx * A + accb[2 * q + 1] * ny * A);
        for (int q = 0; q < NQ; ++q) wb[q] += 0.5 * phbq[q];
        int j = side ? m.fo[f] : m.fn[f];
        if (j < 0) {
            // ghost half: back through the ghost's primitives and the ghost state
            double dn = m.dxo[f] * nx + m.dyo[f] * ny;
            dn = dn < 0.0 ? -dn : dn;
            CS<double> gs = ghost_state(F, Ui, m.ftag[f], nx, ny, dn);
            double gwb[NQ];
            for (int q = 0; q < NQ; ++q) gwb[q] = 0.5 * phbq[q];
            CSb<double> gsb = csb_zero<double>();
            w_to_csb<NQ>(F, gs.r, gs.p, gs.rk, gs.rw, gwb, gsb);
            ghost_state_b(F, Ui, m.ftag[f], nx, ny, gsb, cb, dn);
        }
    }
    w_to_csb<NQ>(F, wi[W_R], wi[W_P], Ui.rk, Ui.rw, wb, cb);
    cs_back(F, Ui, cb, ub);
    for (int c = 0; c < NV; ++c) b.gpart[c * nc + i] = ub[c];
    b.pmaxb[i] = pmaxb;
    b.pminb[i] = pminb;
    b.pmax_face[i] = pmax_face;
    b.pmin_face[i] = pmin_face;
}

template <int NV>
__global__ void __launch_bounds__(128) k_adj_cell2(MeshView<double> m, Flow<double> F, Field<double> U,
                                                   Field<double> W, AdjBufs b, double* __restrict__ gU) {
    constexpr int NQ = Planes<NV>::G / 2;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    long nc = m.nc;
    double wb[NQ];
    for (int q = 0; q < NQ; ++q) wb[q] = 0.0;
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        int f = e >> 1, side = e & 1;
        int j = side ? m.fo[f] : m.fn[f];
        if (j < 0) continue;
        // neighbour j's half of this face: j is owner when this cell is the neighbour
        double sj = side ? 1.0 : -1.0;
        double nx = m.nx[f], ny = m.ny[f], A = m.area[f];
        for (int q = 0; q < NQ; ++q)
            wb[q] += 0.5 * sj * (b.accb[(2 * q) * nc + j] * nx * A + b.accb[(2 * q + 1) * nc + j] * ny * A);
        if (b.pmax_face[j] == f) wb[W_P] += b.pmaxb[j];
        if (b.pmin_face[j] == f) wb[W_P] += b.pminb[j];
    }
    CS<double> Ui = load_cs<double, NV>(U, W, i);
    CSb<double> cb = csb_zero<double>();
    w_to_csb<NQ>(F, W.v[W_R * nc + i], W.v[W_P * nc + i], Ui.rk, Ui.rw, wb, cb);
    double ub[6] = {0, 0, 0, 0, 0, 0};
    cs_back(F, Ui, cb, ub);
    for (int c = 0; c < NV; ++c) gU[c * nc + i] = b.gpart[c * nc + i] + ub[c];
}

}  // namespace cfdg
