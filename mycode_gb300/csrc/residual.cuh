// Residual kernels R(U) = sum_f (+-) F_f A_f on the renumbered SoA mesh.
//
// One evaluation is four launches (five with the SST cell terms, k_sst_cell):
//   k_prim    per cell   W = (rho, u, v, p, T [, k, w])           reads U
//   k_grad    per cell   Green-Gauss gradients + Barth-Jespersen   gathers W over the
//                        limiter, no atomics                      cell's faces
//   k_flux    per face   reconstruction, Riemann flux, viscous    writes F*A per face
//                        flux
//   k_gather  per cell   R_i = sum of +-F*A over the cell's faces in the reference's
//                        face order (deterministic, bit-reproducible)
// The FP64 residual on a mesh of 100,000 or more interior faces splits the gradient in
// two (k_grad_faces64: each interior face's Green-Gauss terms once; k_grad64<NV, true>:
// the per-cell sums in face order and the limiter), the same bits with fewer FP64
// instructions; the FP32 views' gradients read the neighbours and face geometry from
// per-cell copies (CellFaces, k_grad_cf).  Through cfdg_residual with pinned host buffers
// the first and last launch are k_rows_prim and k_gather_rows (the caller's rows in place).
//
// The kernels are templated on the scalar S: double / float for the residual, and
// Dual<double> / Dual<float> for the exact forward linearisation (J v with the limiter
// frozen), where every array has a value plane and a derivative plane.
#pragma once
#include <cuda_runtime.h>
#include <type_traits>
#include "face.cuh"
#include "pdl.cuh"
#include "sst.cuh"

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
    const R* d2lr;     // [nf] dxlr^2 + dylr^2 (0 on the boundary), formed once per mesh
    const R* id2lr;    // [nf] its reciprocal (0 on the boundary)
    const R* ivol;     // [nc] 1 / vol
};

// Per-cell copies of each face entry's neighbour cell and face geometry, [4][nc] planes
// beside cf (the neighbour -1 for boundary entries and pads, the geometry 0 for pads): a
// gradient kernel given them reads them with the cell's own coalesced loads, so its only
// dependent loads are the neighbours' primitives (through the face index, the neighbour
// and the geometry are a second dependent level).  The values are the face arrays' own.
template <class R>
struct CellFaces {
    const int* nbr;
    const R* nx;
    const R* ny;
    const R* A;
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
    template <class R> static CFD_HD double ld_tangent(const Field<R>& f, int p, long i) { return f.v[p * f.n + i]; }
    template <class R> static CFD_HD void st(const Field<R>& f, int p, long i, double x) { f.v[p * f.n + i] = x; }
};
template <> struct Acc<float> {
    template <class R> static CFD_HD float ld(const Field<R>& f, int p, long i) { return f.v[p * f.n + i]; }
    template <class R> static CFD_HD float ld_tangent(const Field<R>& f, int p, long i) { return f.v[p * f.n + i]; }
    template <class R> static CFD_HD void st(const Field<R>& f, int p, long i, float x) { f.v[p * f.n + i] = x; }
};
template <class R> struct Acc<Dual<R>> {
    static CFD_HD Dual<R> ld(const Field<R>& f, int p, long i) {
        return Dual<R>(f.v[p * f.n + i], f.d ? f.d[p * f.n + i] : R(0));
    }
    // the derivative plane alone (value 0): for sums whose derivative does not depend on
    // the values
    static CFD_HD Dual<R> ld_tangent(const Field<R>& f, int p, long i) { return Dual<R>(R(0), f.d[p * f.n + i]); }
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
__device__ __forceinline__ void prim_cell(const Flow<R>& F, S r, S ru, S rv, S rE, S rk, S rw, Field<R> W, long i) {
    const S ir = recip_for(r);  // FP64: u and v by one reciprocal (quot_shared)
    S u = quot_shared(ru, r, ir), v = quot_shared(rv, r, ir);
    S p = pressure(F, r, ru, rv, rE);
    S T = p / (r * F.Rgas);
    Acc<S>::st(W, W_R, i, r);
    Acc<S>::st(W, W_U, i, u);
    Acc<S>::st(W, W_V, i, v);
    Acc<S>::st(W, W_P, i, p);
    Acc<S>::st(W, W_T, i, T);
    if (NV == 6) {
        // the specific k and w through the same reciprocal of rho (FP64: RN(rk / r) for
        // finite nonzero quotients; a zero rk gives +0)
        Acc<S>::st(W, W_K, i, quot_shared(rk, r, ir));
        Acc<S>::st(W, W_W, i, quot_shared(rw, r, ir));
    }
}

template <class S, int NV, class R>
__global__ void __launch_bounds__(256) k_prim(int nc, Flow<R> F, Field<R> U, Field<R> W) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    S r = Acc<S>::ld(U, 0, i), ru = Acc<S>::ld(U, 1, i), rv = Acc<S>::ld(U, 2, i), rE = Acc<S>::ld(U, 3, i);
    S rk = S(R(0)), rw = S(R(0));
    if (NV == 6) {
        rk = Acc<S>::ld(U, 4, i);
        rw = Acc<S>::ld(U, 5, i);
    }
    prim_cell<S, NV>(F, r, ru, rv, rE, rk, rw, W, i);
}

// ---------------------------------------------------------------- k_grad
// computeGradients (src/Solver.cpp:81-149) as a per-cell gather over the cell's faces
// in reference face order, then (limited scheme, limiter not frozen) computeLimiters
// (src/Solver.cpp:152-253) for the same cell from its own fresh gradient.
// CF: the neighbours and face geometry from cx (CellFaces) instead of through the faces.
// TAN: the tangent-only gradient of a Krylov body (S a dual number, derivative planes
// written, no limiter).  Everything else as the generic kernel computes it.
// FT (FP64 residual): each interior face's Green-Gauss terms (ph n_x A, ph n_y A per
// primitive) read from ft, where k_grad_faces64 formed them once per face (planes of
// ftn = nfi entries), instead of formed again by each of the face's two cells; the
// neighbour's pressure is still read for the limiter's bounds.
template <class S, int NV, class R, bool CF = false, bool FT = false, bool TAN = false>
__device__ __forceinline__ void grad_item(const MeshView<R>& m, const Flow<R>& F, const Field<R>& U,
                                          const Field<R>& W, const Field<R>& G, R* phi, int do_limiter, long i,
                                          const int* done = nullptr, CellFaces<R> cx = {}, const R* ft = nullptr,
                                          long ftn = 0) {
    // done: a finished Krylov solve (krylov.cuh); read with the mesh loads, tested after
    const int skip = done ? *done : 0;
    constexpr int NQ = NV == 6 ? 7 : 5;
    // a dual gradient with no value planes to write (J v about a fixed point whose value
    // planes are current): the face sums' derivatives need only the neighbours' derivative
    // planes (the ghost states read the cell's own values)
    const bool tangent = TAN || (!std::is_same<S, R>::value && G.v == nullptr && !do_limiter);
    // Mesh data first (face entries, then each face's normal, area and neighbour, and for
    // a boundary face its distance and tag): no kernel writes it, so it is loaded before
    // the wait for the predecessor's primitives (pdl.cuh) and only the primitive loads
    // follow the wait.  The -1 pads are trailing, so skipping them is stopping at them.
    int ek[4], nbr[4], ftg[4];
    R fnx[4], fny[4], fA[4], fdn[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ek[k] = m.cf[(long)k * m.nc + i];
    if constexpr (CF) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long q = (long)k * m.nc + i;
            nbr[k] = cx.nbr[q];
            fnx[k] = cx.nx[q];
            fny[k] = cx.ny[q];
            fA[k] = cx.A[q];
        }
    }
    if (skip) return;  // tested with the first loads in flight, before the dependent ones
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int e = ek[k];
        if constexpr (!CF) {
            nbr[k] = -1;
            fnx[k] = fny[k] = fA[k] = R(0);
        }
        ftg[k] = 0;
        fdn[k] = R(0);
        if (e < 0) continue;
        const int f = e >> 1;
        if constexpr (!CF) {
            fnx[k] = m.nx[f];
            fny[k] = m.ny[f];
            fA[k] = m.area[f];
            nbr[k] = (e & 1) ? m.fo[f] : m.fn[f];
        }
        if (nbr[k] < 0) {
            fdn[k] = m.dxo[f] * fnx[k] + m.dyo[f] * fny[k];
            ftg[k] = m.ftag[f];
        }
    }
    pdl_wait();
    pdl_trigger();
    S wi[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) wi[q] = Acc<S>::ld(W, q, i);
    S acc[2 * NQ];
#pragma unroll
    for (int q = 0; q < 2 * NQ; ++q) acc[q] = S(R(0));
    R pmax = val(wi[W_P]), pmin = val(wi[W_P]);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int e = ek[k];
        if (e < 0) continue;
        int side = e & 1;
        R nx = fnx[k], ny = fny[k], A = fA[k];
        S wj[NQ];
        int j = nbr[k];
        if constexpr (FT) {
            if (j >= 0) {
                // the face's terms, formed once for its two cells (the same bits: the half
                // sum is commutative, the products the same expressions)
                const long f = e >> 1;
                const R pj = W.v[W_P * W.n + j];
                pmax = smax(pmax, pj);
                pmin = smin(pmin, pj);
#pragma unroll
                for (int q = 0; q < NQ; ++q) {
                    const R tx = ft[(2 * q) * ftn + f], ty = ft[(2 * q + 1) * ftn + f];
                    if (side) {
                        acc[2 * q] = acc[2 * q] - tx;
                        acc[2 * q + 1] = acc[2 * q + 1] - ty;
                    } else {
                        acc[2 * q] = acc[2 * q] + tx;
                        acc[2 * q + 1] = acc[2 * q + 1] + ty;
                    }
                }
                continue;
            }
        }
        if (j >= 0) {
            if (tangent) {
#pragma unroll
                for (int q = 0; q < NQ; ++q) wj[q] = Acc<S>::ld_tangent(W, q, j);
            } else {
#pragma unroll
                for (int q = 0; q < NQ; ++q) wj[q] = Acc<S>::ld(W, q, j);
            }
        } else {
            CS<S> Ui = load_cs<S, NV>(U, W, i);
            R dn = fdn[k];
            CS<S> g = ghost_state(F, Ui, ftg[k], nx, ny, dn < R(0) ? -dn : dn);
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
            S ph = half(wi[q] + wj[q]);
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
    // 1 / vol: FP64 once per mesh (the same bits), the FP32 views in the kernel; FP64: the
    // quotients by it (div_shared)
    const R ivol = std::is_same<R, double>::value ? m.ivol[i] : R(1.0) / vol;
    // gradient planes are in CellGradient order rho, u, v, p, T (= primitive order)
#pragma unroll
    for (int q = 0; q < 2 * NQ; ++q) {
        acc[q] = div_shared(acc[q], vol, ivol);
        if constexpr (TAN) G.d[q * G.n + i] = acc[q].d;
        else Acc<S>::st(G, q, i, acc[q]);
    }
    if (TAN || !do_limiter) return;
    // Barth-Jespersen on pressure reconstructed through T; one phi per cell
    const R eps = R(1e-12);
    R pc = val(wi[W_P]);
    R rho = val(wi[W_R]);
    R Tc = val(wi[W_T]);
    R gTx = val(acc[G_T]), gTy = val(acc[G_T + 1]);
    R lim = R(1.0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int e = ek[k];
        if (e < 0) continue;
        int f = e >> 1, side = e & 1;
        R dx = side ? m.dxn[f] : m.dxo[f];
        R dy = side ? m.dyn[f] : m.dyo[f];
        R Tf = Tc + R(1.0) * (gTx * dx + gTy * dy);
        R Pf = rho * F.Rgas * Tf;
        R d2 = Pf - pc;
        R a = R(1.0);
        // a = min(1, x / y): when x / y >= 1 exactly (x >= y > 0, or x <= y < 0) the rounded
        // quotient is >= 1 too and a is 1: the divide runs only for the faces that limit
        if (gt0(d2)) {
            const R x = pmax - pc, y = d2 + eps;
            if (lt(x, y)) a = smin(R(1.0), x / y);
        } else if (lt0(d2)) {
            const R x = pmin - pc, y = d2 - eps;
            if (lt(y, x)) a = smin(R(1.0), x / y);
        }
        lim = smin(lim, a);
    }
    phi[i] = lim;
}

// Resident 256-thread blocks per SM asked of the compiler for the shared gradient and
// face-flux templates (the register cap is 65536 / (256 x blocks)).
#ifndef GRAD_DUAL_MINB
#define GRAD_DUAL_MINB 2
#endif
#ifndef FLUX_DUAL_MINB
#define FLUX_DUAL_MINB 2
#endif
template <class S> struct MinBlocks { static constexpr int grad = 1, flux = 1; };
template <> struct MinBlocks<Dual<float>> { static constexpr int grad = GRAD_DUAL_MINB, flux = FLUX_DUAL_MINB; };

// lim_dev (optional): the limiter is recomputed only when *lim_dev is also set (a Newton
// step whose limiter-freeze decision was taken on the device)
template <class S, int NV, class R>
__global__ void __launch_bounds__(256, MinBlocks<S>::grad) k_grad(MeshView<R> m, Flow<R> F, Field<R> U, Field<R> W, Field<R> G,
                                              R* phi, int do_limiter, const int* done, const int* lim_dev) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    if (lim_dev && !*lim_dev) do_limiter = 0;
    grad_item<S, NV>(m, F, U, W, G, phi, do_limiter, i, done);  // waits for its predecessor (pdl.cuh)
}

// k_grad with the neighbours and face geometry from per-cell copies (CellFaces).  The
// tangent-only dual gradient of a Krylov body (TAN) runs four resident 256-thread blocks per
// SM (three with SST: 64 / 80 registers, no spills), where the generic template's 128
// registers keep two: the neighbour loads are its latency, and more warps keep more of them
// in flight.  The FP32 value gradient (with its limiter) and the full dual gradient run two.
template <class S, int NV, bool TAN> struct GradCfBlocks { static constexpr int value = 2; };
template <class S, int NV> struct GradCfBlocks<S, NV, true> { static constexpr int value = NV == 6 ? 3 : 4; };

template <class S, int NV, class R, bool TAN>
__global__ void __launch_bounds__(256, (GradCfBlocks<S, NV, TAN>::value)) k_grad_cf(MeshView<R> m, CellFaces<R> cx,
                                                                                  Flow<R> F, Field<R> U, Field<R> W,
                                                                                  Field<R> G, R* phi, int do_limiter,
                                                                                  const int* done) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    grad_item<S, NV, R, true, false, TAN>(m, F, U, W, G, phi, do_limiter, i, done, cx);  // waits for its predecessor
}

// ---------------------------------------------------------------- k_flux
// The face loop of computeResiduals (src/Solver.cpp:543-800) through face_flux:
// reconstruction, the wall pressure flux or the Riemann flux, and (viscous) the
// Navier-Stokes flux from averaged and corrected cell gradients.  Writes F*A per face.
template <class S, int NV, class R>
__device__ __forceinline__ void load_grad(const Field<R>& G, long i, S* g) {
#pragma unroll
    for (int q = 0; q < 10; ++q) g[q] = Acc<S>::ld(G, q, i);
}

template <class R>
__device__ __forceinline__ FaceGeo<R> load_geo(const MeshView<R>& m, long f) {
    FaceGeo<R> g;
    g.nx = m.nx[f];
    g.ny = m.ny[f];
    g.A = m.area[f];
    g.dxL = m.dxo[f];
    g.dyL = m.dyo[f];
    g.dxR = m.dxn[f];
    g.dyR = m.dyn[f];
    g.dxlr = m.dxlr[f];
    g.dylr = m.dylr[f];
    g.d2lr = m.d2lr[f];
    g.id2lr = m.id2lr[f];
    return g;
}

// SST cell terms (sst.cuh): T planes 0 mu_t, 1 F1, 2 S_k vol, 3 S_w vol; dwall holds the
// wall distances and, from nc on, 1 / max(d, 1e-30) (k_wall_distance)
template <class S, int NV, class R>
__device__ __forceinline__ void sst_item(const MeshView<R>& m, const Flow<R>& F, const Field<R>& W,
                                         const Field<R>& G, const R* __restrict__ dwall, const Field<R>& T, long i) {
    // 1 / max(d, 1e-30): FP64 from k_wall_distance (the same bits), the FP32 views in the kernel
    const R dwi = dwall[i];
    const R idd = std::is_same<R, double>::value ? dwall[(long)m.nc + i] : R(1) / (lt(R(1e-30), dwi) ? dwi : R(1e-30));
    SstCell<S> c = sst_cell_id(F, Acc<S>::ld(W, W_R, i), Acc<S>::ld(W, W_K, i), Acc<S>::ld(W, W_W, i),
                            Acc<S>::ld(G, G_U, i), Acc<S>::ld(G, G_U + 1, i), Acc<S>::ld(G, G_V, i),
                            Acc<S>::ld(G, G_V + 1, i), Acc<S>::ld(G, G_K, i), Acc<S>::ld(G, G_K + 1, i),
                            Acc<S>::ld(G, G_W, i), Acc<S>::ld(G, G_W + 1, i), idd);
    R vol = m.vol[i];
    Acc<S>::st(T, 0, i, c.mut);
    Acc<S>::st(T, 1, i, c.F1);
    Acc<S>::st(T, 2, i, c.Sk * vol);
    Acc<S>::st(T, 3, i, c.Sw * vol);
}

template <class S, int NV, class R>
__global__ void __launch_bounds__(256) k_sst_cell(MeshView<R> m, Flow<R> F, Field<R> W, Field<R> G,
                                                  const R* __restrict__ dwall, Field<R> T, const int* done) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc || (done && *done)) return;
    pdl_wait();
    pdl_trigger();
    sst_item<S, NV>(m, F, W, G, dwall, T, i);
}

template <class S, int NV, class R>
__device__ __forceinline__ void flux_item(const MeshView<R>& m, const Flow<R>& F, const Field<R>& U,
                                          const Field<R>& W, const Field<R>& G, const R* __restrict__ phi,
                                          const Field<R>& FA, const Field<R>& T, long f, const int* done = nullptr) {
    const int skip = done ? *done : 0;  // a finished Krylov solve: tested after the first loads
    int o = m.fo[f], n = m.fn[f];
    bool interior = n >= 0;
    int tag = interior ? 0 : m.ftag[f];
    FaceGeo<R> g = load_geo(m, f);
    if (skip) return;
    CS<S> L = load_cs<S, NV>(U, W, o);
    CS<S> Rn = interior ? load_cs<S, NV>(U, W, n) : L;
    // the state and primitives come from two or more kernels back in the Arnoldi body,
    // the gradients, limiter and SST terms from the predecessor (pdl.cuh)
    pdl_wait();
    pdl_trigger();
    S gL[10], gR[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) { gL[q] = S(R(0)); gR[q] = S(R(0)); }
    const bool second = F.spatial != SP_FIRST;
    if ((second && interior) || F.viscous) {
        load_grad<S, NV>(G, o, gL);
        if (interior) load_grad<S, NV>(G, n, gR);
    }
    S phL = S(R(1)), phR = S(R(1));
    if (F.spatial == SP_LIMITED && interior) {
        phL = S(phi[o]);
        phR = S(phi[n]);
    }
    if constexpr (NV == 6) {
        S gk[8];
        gk[0] = Acc<S>::ld(G, G_K, o);
        gk[1] = Acc<S>::ld(G, G_K + 1, o);
        gk[2] = Acc<S>::ld(G, G_W, o);
        gk[3] = Acc<S>::ld(G, G_W + 1, o);
        gk[4] = gk[0], gk[5] = gk[1], gk[6] = gk[2], gk[7] = gk[3];
        S mutR = S(R(0)), F1R = S(R(0));
        // specific k, w of the two cells: the primitives k_prim formed (rho k / rho, rho w / rho)
        S kw[4] = {Acc<S>::ld(W, W_K, o), Acc<S>::ld(W, W_W, o), S(R(0)), S(R(0))};
        if (interior) {
            gk[4] = Acc<S>::ld(G, G_K, n);
            gk[5] = Acc<S>::ld(G, G_K + 1, n);
            gk[6] = Acc<S>::ld(G, G_W, n);
            gk[7] = Acc<S>::ld(G, G_W + 1, n);
            mutR = Acc<S>::ld(T, 0, n);
            F1R = Acc<S>::ld(T, 1, n);
            kw[2] = Acc<S>::ld(W, W_K, n);
            kw[3] = Acc<S>::ld(W, W_W, n);
        }
        Flux6<S> out = face_flux_sst(F, L, Rn, interior, tag, g, gL, gR, gk, gk + 4, phL, phR, Acc<S>::ld(T, 0, o),
                                     mutR, Acc<S>::ld(T, 1, o), F1R, kw, kw + 2);
#pragma unroll
        for (int c = 0; c < 6; ++c) Acc<S>::st(FA, c, f, out.f[c]);
        return;
    }
    Flux6<S> out = face_flux(F, L, Rn, interior, tag, g, gL, gR, phL, phR);
#pragma unroll
    for (int c = 0; c < NV; ++c) Acc<S>::st(FA, c, f, out.f[c]);
}

template <class S, int NV, class R>
__global__ void __launch_bounds__(256, MinBlocks<S>::flux) k_flux(MeshView<R> m, Flow<R> F, Field<R> U, Field<R> W, Field<R> G,
                                              const R* __restrict__ phi, Field<R> FA, Field<R> T, const int* done) {
    long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    flux_item<S, NV>(m, F, U, W, G, phi, FA, T, f, done);
}

// The FP64 residual's gradient and face-flux kernels: grad_item / flux_item under launch
// bounds that keep more warps resident than the shared templates' 256-thread bound (which
// lets the compiler take 149 / 181 registers: one block, eight warps per SM).  Both kernels
// are bound by GB300's FP64 pipe, whose long instruction latencies need more warps per
// sub-partition.  Measured on the 4M-cell SST bump: gradients 4.81 -> 4.51 ms with at
// least two 256-thread blocks per SM (128 registers), face fluxes 6.32 -> 5.86 ms with at
// least three 128-thread blocks (170 registers); 128-thread blocks x 3 for the gradients
// 4.55 ms, 64-thread blocks x 5-6 the same as x 3.
constexpr unsigned GRAD64_THREADS = 256;

// FT: the interior faces' Green-Gauss terms from ft (k_grad_faces64), planes of m.nfi
template <int NV, bool FT>
__global__ void __launch_bounds__(GRAD64_THREADS, 2) k_grad64(MeshView<double> m, Flow<double> F, Field<double> U,
                                                   Field<double> W, Field<double> G, double* phi, int do_limiter,
                                                   const int* lim_dev, const double* __restrict__ ft) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    if (lim_dev && !*lim_dev) do_limiter = 0;
    grad_item<double, NV, double, false, FT>(m, F, U, W, G, phi, do_limiter, i, nullptr, {}, ft, m.nfi);
}

// The Green-Gauss terms of each interior face, once: ph = (w_owner + w_neighbour) / 2 and
// ph n_x A, ph n_y A for every primitive, the expressions the per-cell gather forms on each
// side of the face (src/Solver.cpp:104-147), into planes 2q (x) and 2q + 1 (y) of nfi
// entries.  Half of the gradient's FP64 work on the faces is forming these terms; the
// gradient kernel adds them in each cell's face order.
template <int NV>
__global__ void __launch_bounds__(256) k_grad_faces64(MeshView<double> m, Field<double> W, double* __restrict__ ft) {
    const long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nfi) return;
    constexpr int NQ = NV == 6 ? 7 : 5;
    const long o = m.fo[f], n = m.fn[f];
    const double nx = m.nx[f], ny = m.ny[f], A = m.area[f];
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
        const double ph = half(W.v[q * W.n + o] + W.v[q * W.n + n]);
        ft[(2 * q) * (long)m.nfi + f] = ph * nx * A;
        ft[(2 * q + 1) * (long)m.nfi + f] = ph * ny * A;
    }
}

constexpr unsigned FLUX64_THREADS = 128;

template <int NV>
__global__ void __launch_bounds__(FLUX64_THREADS, 3) k_flux64(MeshView<double> m, Flow<double> F, Field<double> U,
                                                              Field<double> W, Field<double> G,
                                                              const double* __restrict__ phi, Field<double> FA,
                                                              Field<double> T) {
    long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= m.nf) return;
    flux_item<double, NV>(m, F, U, W, G, phi, FA, T, f, nullptr);
}

// ---------------------------------------------------------------- k_gather
// R_i = sum over the cell's faces, in reference face order, of +F*A (owner) or -F*A
// (neighbour) (src/Solver.cpp:795-799).  Optionally adds diag_v * vol/(dt + 1e-30)
// (the time term of applyJacobian, src/Solver.cpp:1381-1384).
// The faces' F*A of cell i in reference face order (+ owner, - neighbour), minus the SST
// sources (times the cell volume) when given
template <class R, int NV>
__device__ __forceinline__ void gather_cell(const MeshView<R>& m, const R* __restrict__ FA, long fa_stride,
                                            const R* __restrict__ src, long r_stride, long i, R (&acc)[NV]) {
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = R(0);
    int ek[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ek[k] = m.cf[(long)k * m.nc + i];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        int e = ek[k];
        if (e < 0) continue;
        long f = e >> 1;
        if (e & 1) {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] - FA[c * fa_stride + f];
        } else {
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] = acc[c] + FA[c * fa_stride + f];
        }
    }
    if constexpr (NV == 6) {
        // SST sources (times the cell volume): R = sum of fluxes - S vol
        if (src) {
            acc[4] = acc[4] - src[i];
            acc[5] = acc[5] - src[r_stride + i];
        }
    }
}

template <class R, int NV>
__global__ void __launch_bounds__(256) k_gather(MeshView<R> m, const R* __restrict__ FA, long fa_stride,
                                                R* __restrict__ Rout, long r_stride,
                                                const R* __restrict__ diag_v, const R* __restrict__ dt,
                                                const R* __restrict__ src) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    R acc[NV];
    gather_cell<R, NV>(m, FA, fa_stride, src, r_stride, i, acc);
    if (diag_v) {
        R tc = m.vol[i] / (dt[i] + R(1e-30));
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = acc[c] + diag_v[c * r_stride + i] * tc;
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) Rout[c * r_stride + i] = acc[c];
}

// ---------------------------------------------------------------- caller rows in place
// Caller rows (stride doubles each, the caller's numbering) are moved by the kernels
// themselves, with no staging buffer or copy engine.  A block owns ROW_BLOCK consecutive
// rows: it moves them as one contiguous span (consecutive threads, consecutive addresses:
// every link transaction carries whole lines) through shared memory, and each thread
// exchanges its row with the SoA planes at the row's internal index iperm[row].  (One
// thread per row, reading its row's doubles one by one, moved every line of the span
// `stride` times: a quarter of the copy engines' rate.)  Launched with ROW_BLOCK threads.
constexpr int ROW_BLOCK = 256;
constexpr int ROW_MAX_STRIDE = 14;

// rows [r0, r0 + rows) of aos into sm (rows * stride doubles); returns rows
__device__ __forceinline__ int rows_load(const double* __restrict__ aos, long nrows, int stride, double* sm, long& r0) {
    r0 = (long)blockIdx.x * ROW_BLOCK;
    const long left = nrows - r0;
    const int rows = left < ROW_BLOCK ? (int)left : ROW_BLOCK;
    const long n = (long)rows * stride;
    const double* src = aos + r0 * stride;
    if ((stride & 1) == 0 && (reinterpret_cast<size_t>(src) & 15) == 0) {
        const double2* s2 = reinterpret_cast<const double2*>(src);
        double2* d2 = reinterpret_cast<double2*>(sm);
        for (long q = threadIdx.x; q < n / 2; q += ROW_BLOCK) d2[q] = s2[q];
    } else {
        for (long q = threadIdx.x; q < n; q += ROW_BLOCK) sm[q] = src[q];
    }
    __syncthreads();
    return rows;
}

__device__ __forceinline__ void rows_store(double* __restrict__ aos, long r0, int rows, int stride, const double* sm) {
    __syncthreads();
    const long n = (long)rows * stride;
    double* dst = aos + r0 * stride;
    if ((stride & 1) == 0 && (reinterpret_cast<size_t>(dst) & 15) == 0) {
        const double2* s2 = reinterpret_cast<const double2*>(sm);
        double2* d2 = reinterpret_cast<double2*>(dst);
        for (long q = threadIdx.x; q < n / 2; q += ROW_BLOCK) d2[q] = s2[q];
    } else {
        for (long q = threadIdx.x; q < n; q += ROW_BLOCK) dst[q] = sm[q];
    }
}

// The first and last stage of a residual evaluation whose state and residual live in a
// caller's pinned AoS arrays (6 doubles per cell, the caller's numbering): the rows cross
// the CPU-GPU link inside these kernels (staged in shared memory by rows_load /
// rows_store), so the link transfer overlaps the primitives' and the gather's arithmetic
// instead of preceding and following it.  Same arithmetic as k_prim and k_gather.

// k_prim of the caller's rows: U planes and W planes at each row's internal index
template <int NV>
__global__ void __launch_bounds__(ROW_BLOCK) k_rows_prim(int nc, Flow<double> F, const double* __restrict__ aos,
                                                       const int* __restrict__ iperm, Field<double> U, Field<double> W) {
    __shared__ __align__(16) double sm[ROW_BLOCK * 6];
    long r0;
    const int rows = rows_load(aos, nc, 6, sm, r0);
    if ((int)threadIdx.x >= rows) return;
    const double* row = sm + threadIdx.x * 6;
    const long c = iperm[r0 + threadIdx.x];
    const double r = row[0], ru = row[1], rv = row[2], rE = row[3];
    const double rk = NV == 6 ? row[4] : 0.0, rw = NV == 6 ? row[5] : 0.0;
    U.v[c] = r;
    U.v[U.n + c] = ru;
    U.v[2 * U.n + c] = rv;
    U.v[3 * U.n + c] = rE;
    if (NV == 6) {
        U.v[4 * U.n + c] = rk;
        U.v[5 * U.n + c] = rw;
    }
    prim_cell<double, NV>(F, r, ru, rv, rE, rk, rw, W, c);
}

// k_gather into the caller's rows (slots NV..5 zero)
template <int NV>
__global__ void __launch_bounds__(ROW_BLOCK) k_gather_rows(MeshView<double> m, const double* __restrict__ FA,
                                                         long fa_stride, const double* __restrict__ src,
                                                         const int* __restrict__ iperm, double* __restrict__ aos) {
    __shared__ __align__(16) double sm[ROW_BLOCK * 6];
    const long r0 = (long)blockIdx.x * ROW_BLOCK;
    const long left = (long)m.nc - r0;
    const int rows = left < ROW_BLOCK ? (int)left : ROW_BLOCK;
    if ((int)threadIdx.x < rows) {
        const long c = iperm[r0 + threadIdx.x];
        double acc[NV];
        gather_cell<double, NV>(m, FA, fa_stride, src, m.nc, c, acc);
#pragma unroll
        for (int k = 0; k < 6; ++k) sm[threadIdx.x * 6 + k] = k < NV ? acc[k] : 0.0;
    }
    rows_store(aos, r0, rows, 6, sm);
}

}  // namespace cfdg
