// Wall quantities and the wall distance, built with --fmad=false so each value is the
// reference's own expression evaluated in the same IEEE order:
//   wall distance   computeWallDistances (src/Solver.cpp:1981-2015)
//   Cp, Cf          extractSkinFriction (src/Solver.cpp:1899-1979); Cp = (p - p_inf) / q_inf
//   drag            calculateDrag (src/Solver.cpp:1307-1325), summed in reference face order
//   entropy error   calculateEntropyError (src/Solver.cpp:1620-1646)
//   objectives      the pressure drag, the skin-friction drag and a wall-pressure
//                   integral, with their gradients dJ/dU (the adjoint's right-hand side)
#include "launch.hpp"

namespace cfdg {

constexpr int WD_TILE = 512;

// d_i = min over wall faces of |x_c,i - x_mid,w| (the squared minimum, then one sqrt),
// 1e10 when there is no wall.  Wall midpoints are staged through shared memory in tiles.
__global__ void __launch_bounds__(256) k_wall_distance(long nc, const double* __restrict__ xc,
                                                       const double* __restrict__ yc, int nw,
                                                       const double* __restrict__ wx, const double* __restrict__ wy,
                                                       double* __restrict__ d, float* __restrict__ d32) {
    __shared__ double sx[WD_TILE], sy[WD_TILE];
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double x = i < nc ? xc[i] : 0.0, y = i < nc ? yc[i] : 0.0;
    double best = 1e20;
    for (int t0 = 0; t0 < nw; t0 += WD_TILE) {
        int nt = nw - t0 < WD_TILE ? nw - t0 : WD_TILE;
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += blockDim.x) {
            sx[k] = wx[t0 + k];
            sy[k] = wy[t0 + k];
        }
        __syncthreads();
        for (int k = 0; k < nt; ++k) {
            double dx = x - sx[k], dy = y - sy[k];
            double d2 = dx * dx + dy * dy;
            if (d2 < best) best = d2;
        }
    }
    if (i < nc) {
        double r = nw > 0 ? sqrt(best) : 1e10;
        d[i] = r;
        // planes 2: the reciprocal of max(d, 1e-30) that the SST cell terms use (sst_cell_id)
        const double dd = 1e-30 < r ? r : 1e-30;
        d[nc + i] = 1.0 / dd;
        if (d32) {
            const float rf = (float)r, ddf = 1e-30f < rf ? rf : 1e-30f;
            d32[i] = rf;
            d32[nc + i] = 1.0f / ddf;
        }
    }
}

// Per listed boundary face (device slots): Cp and Cf from the owner cell, and the
// pressure-drag term -p A n_x.
template <int NV>
__global__ void k_wall_coeff(int n, const int* __restrict__ slots, MeshView<double> m, Flow<double> F,
                             const double* __restrict__ U, double q_inf, double p_inf, double* __restrict__ cp,
                             double* __restrict__ cf, double* __restrict__ drag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    long f = slots[k];
    long o = m.fo[f], nc = m.nc;
    double r = U[o], ru = U[nc + o], rv = U[2 * nc + o], rE = U[3 * nc + o];
    double p = pressure(F, r, ru, rv, rE);
    double nx = m.nx[f], ny = m.ny[f];
    double uc = ru / r, vc = rv / r;
    double tx = -ny, ty = nx;
    if (tx < 0) {
        tx = -tx;
        ty = -ty;
    }
    double ut = uc * tx + vc * ty;
    double dn = fabs(m.dxo[f] * nx + m.dyo[f] * ny);
    if (dn < 1e-12) dn = 1e-12;
    double dudn = ut / dn;
    double mu = r * F.nu;
    double tau = mu * dudn;
    cf[k] = tau / q_inf;
    cp[k] = (p - p_inf) / q_inf;
    drag[k] = -p * m.area[f] * nx;
}

// sum of terms[0..n) in order, one thread: the reference's sequential accumulation
__global__ void k_sum_in_order(int n, const double* __restrict__ terms, double* out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += terms[k];
    *out = s;
}

template <int NV>
__global__ void __launch_bounds__(RED_THREADS) k_entropy(long nc, Flow<double> F, const double* __restrict__ U,
                                                         const double* __restrict__ vol, double s_ref, RedScratch rs,
                                                         double* out2) {
    double v[2] = {0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double r = U[i];
        double p = pressure(F, r, U[nc + i], U[2 * nc + i], U[3 * nc + i]);
        if (p <= 0 || r <= 0) continue;
        double sl = p / pow(r, F.gam);
        double e = (sl - s_ref) / s_ref;
        v[0] += (e * e) * vol[i];
        v[1] += vol[i];
    }
    grid_finish<2>(v, rs, out2);
}

// Wall objectives, per listed boundary face of the owner state (the adjoint's right-hand
// sides): 0 pressure drag -p A n_x (calculateDrag), 1 skin-friction drag tau_w A t_x with
// tau_w = rho nu u_t / dn (extractSkinFriction's shear), 2 wall-pressure integral p A.
// Face weights scale each face's term (0 drops it).
template <int NV>
__device__ __forceinline__ double objective_term(int kind, long f, const MeshView<double>& m,
                                                 const Flow<double>& F, const double* __restrict__ U, double* gb) {
    long o = m.fo[f], nc = m.nc;
    double r = U[o], ru = U[nc + o], rv = U[2 * nc + o], rE = U[3 * nc + o];
    double nx = m.nx[f], ny = m.ny[f], A = m.area[f];
    if (kind == 1) {
        double tx = -ny, ty = nx;
        if (tx < 0) {
            tx = -tx;
            ty = -ty;
        }
        double dn = fabs(m.dxo[f] * nx + m.dyo[f] * ny);
        if (dn < 1e-12) dn = 1e-12;
        double uc = ru / r, vc = rv / r;
        double ut = uc * tx + vc * ty;
        double tau = (r * F.nu) * (ut / dn);
        if (gb) {
            // tau = nu (ru t_x + rv t_y) / dn exactly: no dependence on rho
            double c = F.nu / dn * A * tx;
            gb[0] = 0.0;
            gb[1] = c * tx;
            gb[2] = c * ty;
            gb[3] = 0.0;
        }
        return tau * A * tx;
    }
    double p = pressure(F, r, ru, rv, rE);
    double s = kind == 0 ? -A * nx : A;
    if (gb) {
        double gm = F.gam - 1.0, u = ru / r, v = rv / r;
        gb[0] = s * gm * 0.5 * (u * u + v * v);
        gb[1] = -s * gm * u;
        gb[2] = -s * gm * v;
        gb[3] = s * gm;
    }
    return kind == 0 ? -p * A * nx : p * A;
}

template <int NV>
__global__ void k_objective_terms(int n, const int* __restrict__ slots, const double* __restrict__ w, int kind,
                                  MeshView<double> m, Flow<double> F, const double* __restrict__ U,
                                  double* __restrict__ terms) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    terms[k] = w[k] * objective_term<NV>(kind, slots[k], m, F, U, nullptr);
}

// dJ/dU per cell (SoA planes), gathered over the cell's boundary faces with their weights
// (wslot: weight per boundary slot, slots [nfi, nf))
template <int NV>
__global__ void k_objective_grad(int kind, MeshView<double> m, Flow<double> F, const double* __restrict__ U,
                                 const double* __restrict__ wslot, double* __restrict__ g) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    long nc = m.nc;
    double acc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) acc[c] = 0.0;
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        long f = e >> 1;
        if (f < m.nfi) continue;
        double wf = wslot[f - m.nfi];
        if (wf == 0.0) continue;
        double gb[4];
        objective_term<NV>(kind, f, m, F, U, gb);
        for (int c = 0; c < 4; ++c) acc[c] += wf * gb[c];
    }
#pragma unroll
    for (int c = 0; c < NV; ++c) g[c * nc + i] = acc[c];
}

void launch_objective(int nv, int kind, int n, const int* slots, const double* w, const double* wslot,
                      const MeshView<double>& m, const Flow<double>& F, const double* U, double* terms, double* J,
                      double* grad, cudaStream_t s) {
    if (n > 0)
        NV_SWITCH(nv, (k_objective_terms<NVC><<<grid_for(n, 128), 128, 0, s>>>(n, slots, w, kind, m, F, U, terms)));
    k_sum_in_order<<<1, 32, 0, s>>>(n, terms, J);
    if (grad) NV_SWITCH(nv, (k_objective_grad<NVC><<<grid_for(m.nc), 256, 0, s>>>(kind, m, F, U, wslot, grad)));
}

void launch_wall_distance(long nc, const double* xc, const double* yc, int nw, const double* wx, const double* wy,
                          double* d, float* d32, cudaStream_t s) {
    k_wall_distance<<<grid_for(nc), 256, 0, s>>>(nc, xc, yc, nw, wx, wy, d, d32);
}

void launch_wall_coeff(int nv, int n, const int* slots, const MeshView<double>& m, const Flow<double>& F,
                       const double* U, double q_inf, double p_inf, double* cp, double* cf, double* drag,
                       cudaStream_t s) {
    if (n <= 0) return;
    NV_SWITCH(nv, (k_wall_coeff<NVC><<<grid_for(n, 128), 128, 0, s>>>(n, slots, m, F, U, q_inf, p_inf, cp, cf, drag)));
}

void launch_sum_in_order(int n, const double* terms, double* out, cudaStream_t s) {
    k_sum_in_order<<<1, 32, 0, s>>>(n, terms, out);
}

void launch_entropy(int nv, long nc, const Flow<double>& F, const double* U, const double* vol, double s_ref,
                    RedScratch rs, double* out2, cudaStream_t s) {
    NV_SWITCH(nv, (k_entropy<NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, F, U, vol, s_ref, rs, out2)));
}

}  // namespace cfdg
