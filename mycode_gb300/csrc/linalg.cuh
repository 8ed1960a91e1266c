// Vector kernels of the Newton-Krylov loop and the per-cell pseudo-time kernels.
//
// Reductions accumulate in FP64 whatever the vector type, with a fixed grid and a
// fixed combination order (per-block partials, then the last block to finish sums
// the partials in index order), so every result is run-to-run deterministic.
// Vectors are flat arrays of nv*nc entries (SoA planes of the state).
#pragma once
#include <cuda_runtime.h>
#include "residual.cuh"

namespace cfdg {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 608;  // 4 blocks per SM on a 152-SM part

struct RedScratch {
    double* partial;     // [RED_BLOCKS * 2]
    unsigned* counter;   // one ticket counter, left at 0 after each reduction
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of up to two values; result valid in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K]) {
    __shared__ double sm[K][RED_THREADS / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = warp_sum(v[k]);
        if (lane == 0) sm[k][w] = s;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double s = lane < (int)(blockDim.x >> 5) ? sm[k][lane] : 0.0;
            v[k] = warp_sum(s);
        }
    }
}

// Finishes a grid reduction of K values: block partials, then the last block sums
// them in a fixed order and writes out[0..K).  Returns true in the thread that wrote.
template <int K>
__device__ __forceinline__ bool grid_finish(double (&v)[K], RedScratch rs, double* out) {
    __shared__ bool last;
    block_sum<K>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) rs.partial[k * RED_BLOCKS + blockIdx.x] = v[k];
        __threadfence();
        unsigned t = atomicAdd(rs.counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double s[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        s[k] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            s[k] += ((volatile double*)rs.partial)[k * RED_BLOCKS + b];
    }
    block_sum<K>(s);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = s[k];
        *rs.counter = 0u;
    }
    return threadIdx.x == 0;
}

// sum over cells of sum_c a_c b_c (planes in component order, as Solver::dot_product
// src/Solver.cpp:1258-1264); a == b gives the squared norm (norm_L2, :1250-1256)
template <class TA, class TB, int NV>
__global__ void __launch_bounds__(RED_THREADS) k_dot(long nc, const TA* __restrict__ a, const TB* __restrict__ b,
                                                     RedScratch rs, double* out) {
    double v[1] = {0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double s = (double)a[i] * (double)b[i];
#pragma unroll
        for (int c = 1; c < NV; ++c) s = s + (double)a[c * nc + i] * (double)b[c * nc + i];
        v[0] += s;
    }
    grid_finish<1>(v, rs, out);
}

// Fused modified Gram-Schmidt step: w -= h_prev * v_prev (when v_prev != null), then
// out = <w, v_next> (when v_next != null) else out = <w, w>.  The update keeps the
// reference's expression V[j+1] - V[i] * H[i][j] (src/Solver.cpp:1546).
template <class T, int NV>
__global__ void __launch_bounds__(RED_THREADS) k_mgs(long nc, T* __restrict__ w, const T* __restrict__ v_prev,
                                                     const double* h_prev, const T* __restrict__ v_next,
                                                     RedScratch rs, double* out) {
    double v[1] = {0.0};
    T h = v_prev ? (T)(*h_prev) : T(0);
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            T x = w[q];
            if (v_prev) {
                x = x - v_prev[q] * h;
                w[q] = x;
            }
            T y = v_next ? v_next[q] : x;
            s = (c == 0) ? (double)x * (double)y : s + (double)x * (double)y;
        }
        v[0] += s;
    }
    grid_finish<1>(v, rs, out);
}

// x *= 1/h with h = sqrt(*h_sq) when h > thresh (the breakdown guard of
// src/Solver.cpp:1550-1558)
template <class T>
__global__ void k_scale_guard(long n, T* x, const double* h_sq, double thresh) {
    double hv = sqrt(*h_sq);
    if (!(hv > thresh)) return;
    T ih = (T)(1.0 / hv);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) x[q] = x[q] * ih;
}

// x = a * s (s a device scalar, inverted when invert != 0)
template <class TO, class TI>
__global__ void k_scale_from(long n, TO* x, const TI* a, const double* s, int invert) {
    double sv = invert ? 1.0 / *s : *s;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        x[q] = (TO)(a[q] * (TI)sv);
}

// The preconditioner holds one value per cell for the mean flow (plane 0 of D); with SST
// (NV = 6) planes 1 and 2 hold the k and w values, which add the destruction terms.
template <int NV>
__device__ __forceinline__ void d_inv(const double* __restrict__ D, long nc, long i, double* id) {
    id[0] = 1.0 / D[i];
#pragma unroll
    for (int c = 1; c < NV; ++c) id[c] = id[0];
    if (NV == 6) {
        id[4] = 1.0 / D[nc + i];
        id[5] = 1.0 / D[2 * nc + i];
    }
}

// z = V * (1 / D) per cell (src/Solver.cpp:1536-1538), with sum of squares of z
template <class TV, class TZ, int NV>
__global__ void __launch_bounds__(RED_THREADS) k_precond_apply(long nc, const TV* __restrict__ V,
                                                               const double* __restrict__ D, TZ* __restrict__ z,
                                                               RedScratch rs, double* out_sq) {
    double v[1] = {0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double idd[NV];
        d_inv<NV>(D, nc, i, idd);
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            TZ zz = (TZ)(V[c * nc + i] * (TV)idd[c]);
            z[c * nc + i] = zz;
            s = (c == 0) ? (double)zz * (double)zz : s + (double)zz * (double)zz;
        }
        v[0] += s;
    }
    if (out_sq) grid_finish<1>(v, rs, out_sq);
}

// FD perturbation: Up = U + v * eps with eps = 1e-7 (1 + |U|) / (|v| + 1e-30)
// (src/Solver.cpp:1342-1362); norms given as squared sums
static __global__ void k_fd_perturb(long n, const double* __restrict__ U, const double* __restrict__ v,
                             const double* u_sq, const double* v_sq, double* __restrict__ Up, double* eps_out) {
    double eps = 1e-7 * (1.0 + sqrt(*u_sq)) / (sqrt(*v_sq) + 1e-30);
    if (blockIdx.x == 0 && threadIdx.x == 0) *eps_out = eps;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) Up[q] = U[q] + v[q] * eps;
}

// Jv = (Rp - Rb) * (1/eps) + v * (vol / (dt + 1e-30)) (src/Solver.cpp:1378-1385)
template <int NV>
__global__ void k_fd_combine(long nc, const double* __restrict__ Rp, const double* __restrict__ Rb,
                             const double* __restrict__ v, const double* eps, const double* __restrict__ vol,
                             const double* __restrict__ dt, double* __restrict__ Jv) {
    double ie = 1.0 / *eps;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double tc = vol[i] / (dt[i] + 1e-30);
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            Jv[q] = (Rp[q] - Rb[q]) * ie + v[q] * tc;
        }
    }
}

// x = sum_i (V_i * y_i) * (1/D) accumulated in i order (src/Solver.cpp:1610-1615)
template <class TV, int NV>
__global__ void k_gmres_solution(long nc, const TV* __restrict__ V, long vstride, const double* y, int k,
                                 const double* __restrict__ D, double* __restrict__ x) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double id[NV];
        d_inv<NV>(D, nc, i, id);
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            double acc = 0.0;
            for (int j = 0; j <= k; ++j) acc = acc + (double)V[j * vstride + q] * y[j] * id[c];
            x[q] = acc;
        }
    }
}

// Volume-weighted residual norm pieces (src/Solver.cpp:1280-1303): sum of
// (sum_c (R_c/vol)^2) * vol, sum of vol, and the density-only sum
template <int NV>
__global__ void __launch_bounds__(RED_THREADS) k_norm_vm(long nc, const double* __restrict__ R,
                                                         const double* __restrict__ vol, RedScratch rs, double* out3) {
    double v[3] = {0.0, 0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double vv = vol[i], iv = 1.0 / vv;  // the quotients by one reciprocal (quot_by_recip)
        double s = 0.0;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            double r = quot_by_recip(R[c * nc + i], vv, iv);
            s = (c == 0) ? r * r : s + r * r;
        }
        double r0 = quot_by_recip(R[i], vv, iv);
        v[0] += s * vv;
        v[1] += vv;
        v[2] += r0 * r0 * vv;
    }
    grid_finish<3>(v, rs, out3);
}

// The residual reductions of a Newton step in one pass over R: the volume-weighted norm
// pieces of k_norm_vm (same arithmetic), sum R^2 (as k_dot, summed in this kernel's own
// order) into out4[0..3], and rhs = -R.  Clears *flag (the update's non-finite flag).
template <int NV>
__global__ void __launch_bounds__(RED_THREADS) k_step_norms(long nc, const double* __restrict__ R,
                                                            const double* __restrict__ vol, double* __restrict__ rhs,
                                                            RedScratch rs, double* out4, int* flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *flag = 0;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double vv = vol[i], iv = 1.0 / vv;  // the quotients by one reciprocal (quot_by_recip)
        double s = 0.0, q = 0.0;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const double Rc = R[c * nc + i];
            rhs[c * nc + i] = -Rc;
            double r = quot_by_recip(Rc, vv, iv);
            s = (c == 0) ? r * r : s + r * r;
            q += Rc * Rc;
        }
        double r0 = quot_by_recip(R[i], vv, iv);
        v[0] += s * vv;
        v[1] += vv;
        v[2] += r0 * r0 * vv;
        v[3] += q;
    }
    grid_finish<4>(v, rs, out4);
}

// k_gather (FP64) of a Newton step fused with k_step_norms: R (the same bits), rhs = -R,
// the norm pieces and sum R^2 into out4, *flag cleared.  Grid-stride over the cells with
// at most RED_BLOCKS blocks (the partials of grid_finish).
template <int NV>
__global__ void __launch_bounds__(RED_THREADS) k_gather_norms(MeshView<double> m, const double* __restrict__ FA,
                                                              long fa_stride, double* __restrict__ Rout,
                                                              const double* __restrict__ src,
                                                              double* __restrict__ rhs, RedScratch rs, double* out4,
                                                              int* flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *flag = 0;
    const long nc = m.nc;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double acc[NV];
        gather_cell<double, NV>(m, FA, fa_stride, src, nc, i, acc);
        const double vv = m.vol[i], iv = m.ivol[i];  // the quotients by 1 / vol (quot_by_recip)
        double s = 0.0, q = 0.0;
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            Rout[c * nc + i] = acc[c];
            rhs[c * nc + i] = -acc[c];
            double r = quot_by_recip(acc[c], vv, iv);
            s = (c == 0) ? r * r : s + r * r;
            q += acc[c] * acc[c];
        }
        double r0 = quot_by_recip(acc[0], vv, iv);
        v[0] += s * vv;
        v[1] += vv;
        v[2] += r0 * r0 * vv;
        v[3] += q;
    }
    grid_finish<4>(v, rs, out4);
}

// The mixed-precision prologue of a Krylov solve in one pass per cell, FP32 arithmetic on
// the FP64 state: U32 = Ub (the linearisation state), phi32 = phi; at the current state
// U, W the local time step (k_local_dt's expression; from *cfl, or the given dt when
// cfl is null) into dt32 and the diagonal preconditioner (k_precond's expression) into D
// (FP64 storage) and its reciprocals into Dinv32.  The preconditioner and the
// pseudo-time term only shape the FP32 linear system, whose J v is FP32 already.
template <int NV>
__global__ void __launch_bounds__(256) k_mixed_pre(MeshView<float> m, Flow<float> F, const double* __restrict__ U,
                                                   const double* __restrict__ Ub,
                                                   const double* __restrict__ W, const double* __restrict__ phi,
                                                   const double* __restrict__ mut, const double* cfl,
                                                   const double* __restrict__ dt_in, float* __restrict__ U32,
                                                   float* __restrict__ phi32, float* __restrict__ dt32,
                                                   double* __restrict__ D, float* __restrict__ Dinv32) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    const long nc = m.nc;
#pragma unroll
    for (int c = 0; c < NV; ++c) U32[c * nc + i] = (float)Ub[c * nc + i];
    phi32[i] = (float)phi[i];
    int ek[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) ek[k] = m.cf[(long)k * nc + i];
    const float vol = m.vol[i];
    float dt;
    if (cfl) {
        const float r = (float)U[i], ru = (float)U[nc + i], rv = (float)U[2 * nc + i];
        const float c = sqrtf(F.gam * (float)W[3 * nc + i] / r);
        float lam = 1e-12f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int e = ek[k];
            if (e < 0) continue;
            const int f = e >> 1;
            const float un = (e & 1) ? (ru * (-m.nx[f]) + rv * (-m.ny[f])) / r : (ru * m.nx[f] + rv * m.ny[f]) / r;
            lam += (fabsf(un) + c) * m.area[f];
        }
        dt = (float)*cfl * vol / lam;
    } else {
        dt = (float)dt_in[i];
    }
    dt32[i] = dt;
    auto state = [&](long j) {
        CS<float> q;
        q.r = (float)U[j];
        q.ru = (float)U[nc + j];
        q.rv = (float)U[2 * nc + j];
        q.rE = (float)U[3 * nc + j];
        q.rk = NV == 6 ? (float)U[4 * nc + j] : 0.f;
        q.rw = NV == 6 ? (float)U[5 * nc + j] : 0.f;
        q.u = (float)W[W_U * nc + j];
        q.v = (float)W[W_V * nc + j];
        q.p = (float)W[W_P * nc + j];
        return q;
    };
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int e = ek[k];
        if (e < 0) continue;
        const int f = e >> 1;
        const int o = m.fo[f], n = m.fn[f];
        const float nx = m.nx[f], ny = m.ny[f];
        const CS<float> L = state(o);
        const CS<float> Rr = n >= 0 ? state(n) : ghost_state(F, L, m.ftag[f], nx, ny);
        const float g = F.gam;
        const float cL = sqrtf(g * L.p / L.r);
        const float cR = sqrtf(g * (Rr.p > 0 ? Rr.p : 1e-3f) / (Rr.r > 0 ? Rr.r : 1e-3f));
        const float cf = 0.5f * (cL + cR);
        const float vn = fabsf(0.5f * (L.u + Rr.u) * nx + 0.5f * (L.v + Rr.v) * ny);
        const float li = vn + cf;
        const float dx = sqrtf(m.vol[o]);
        float mu = 0.5f * (L.r + Rr.r) * F.nu;
        if (NV == 6 && mut) mu = mu + 0.5f * ((float)mut[o] + (float)mut[n >= 0 ? n : o]);
        const float lv = 2.f * mu / (0.5f * (L.r + Rr.r) * dx + 1e-12f);
        acc += (li + lv) * m.area[f] * 0.5f;
    }
    float d = vol / (dt + 1e-30f) + acc;
    if (d < 1e-12f) d = 1e-12f;
    D[i] = d;
    Dinv32[i] = 1.f / d;
    if (NV == 6) {
        const float w = (float)W[W_W * nc + i];
        const float dk = d + (float)SstConst::beta_s * w * vol, dw = d + 2.f * (float)SstConst::b1 * w * vol;
        D[nc + i] = dk;
        D[2 * nc + i] = dw;
        Dinv32[nc + i] = 1.f / dk;
        Dinv32[2 * nc + i] = 1.f / dw;
    }
}

// computeLocalTimeStep (src/Solver.cpp:1388-1422) as a per-cell gather: each face
// adds (|u_n| + c) A from the cell's own state, owner and neighbour with their own
// expressions, summed in reference face order from 1e-12.  cfl_dev (optional): the CFL
// number from device memory (a Newton step whose CFL control ran on the device).
template <int NV>
__global__ void k_local_dt(MeshView<double> m, Flow<double> F, const double* __restrict__ U,
                           const double* __restrict__ W, double cfl, double* __restrict__ dt,
                           const double* __restrict__ cfl_dev) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    if (cfl_dev) cfl = *cfl_dev;
    long nc = m.nc;
    double r = U[i], ru = U[nc + i], rv = U[2 * nc + i];
    double p = W[3 * nc + i];
    double c = sqrt(F.gam * p / r);
    double lam = 1e-12;
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        int f = e >> 1;
        double un = (e & 1) ? (ru * (-m.nx[f]) + rv * (-m.ny[f])) / r : (ru * m.nx[f] + rv * m.ny[f]) / r;
        lam += (fabs(un) + c) * m.area[f];
    }
    dt[i] = cfl * m.vol[i] / lam;
}

// computeDiagonalPreconditioner (src/Solver.cpp:1424-1465) as a per-cell gather; each
// face term is evaluated with the owner as L exactly as the reference's face loop.
// With SST (NV = 6, mut = the cell eddy viscosity) the viscous eigenvalue uses mu + mu_t,
// and planes 1 and 2 of D add the linearised destruction of k (beta* w vol) and of w
// (2 beta1 w vol) to the k and w diagonals.
template <int NV>
__global__ void k_precond(MeshView<double> m, Flow<double> F, const double* __restrict__ U,
                          const double* __restrict__ W, const double* __restrict__ dt, double* __restrict__ D,
                          const double* __restrict__ mut) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.nc) return;
    long nc = m.nc;
    double acc = 0.0;
    for (int k = 0; k < 4; ++k) {
        int e = m.cf[(long)k * nc + i];
        if (e < 0) break;
        int f = e >> 1;
        int o = m.fo[f], n = m.fn[f];
        CS<double> L = load_cs<double, NV>(Field<double>{(double*)U, nullptr, nc}, Field<double>{(double*)W, nullptr, nc}, o);
        CS<double> Rr = n >= 0 ? load_cs<double, NV>(Field<double>{(double*)U, nullptr, nc}, Field<double>{(double*)W, nullptr, nc}, n)
                               : ghost_state(F, L, m.ftag[f], m.nx[f], m.ny[f]);
        double g = F.gam;
        double cL = sqrt(g * L.p / L.r);
        double cR = sqrt(g * (Rr.p > 0 ? Rr.p : 1e-3) / (Rr.r > 0 ? Rr.r : 1e-3));
        double cf = 0.5 * (cL + cR);
        double uf = 0.5 * (L.u + Rr.u);
        double vf = 0.5 * (L.v + Rr.v);
        double vn = fabs(uf * m.nx[f] + vf * m.ny[f]);
        double li = vn + cf;
        double dx = sqrt(m.vol[o]);
        double mu = 0.5 * (L.r + Rr.r) * F.nu;
        if (NV == 6 && mut) mu = mu + 0.5 * (mut[o] + mut[n >= 0 ? n : o]);
        double lv = 2.0 * mu / (0.5 * (L.r + Rr.r) * dx + 1e-12);
        double lt = (li + lv) * m.area[f];
        acc += lt * 0.5;
    }
    double v = m.vol[i];
    double d = (v / (dt[i] + 1e-30)) + acc;
    if (d < 1e-12) d = 1e-12;
    D[i] = d;
    if (NV == 6) {
        double w = W[W_W * nc + i];
        D[nc + i] = d + SstConst::beta_s * w * v;
        D[2 * nc + i] = d + 2.0 * SstConst::b1 * w * v;
    }
}

// Newton update with the positivity clamps of src/Solver.cpp:1760-1778 (and, for SST,
// k >= 0 and w >= wmin); flags a non-finite state in *bad (bit 0) without stopping.
template <int NV>
__global__ void k_newton_update(long nc, double* __restrict__ U, const double* __restrict__ dU, double relax,
                                double gam, double wmin, int* bad) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double u[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) u[c] = U[c * nc + i] + dU[c * nc + i] * relax;
    double ke = 0.5 * (u[1] * u[1] + u[2] * u[2]) / (u[0] + 1e-12);
    double pn = (gam - 1.0) * (u[3] - ke);
    if (u[0] < 1e-5) u[0] = 1e-5;
    if (pn < 1e-5) {
        pn = 1e-5;
        u[3] = pn / (gam - 1.0) + ke;
    }
    if constexpr (NV == 6) {
        if (u[4] < 0.0) u[4] = 0.0;
        if (u[5] < u[0] * wmin) u[5] = u[0] * wmin;
    }
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        ok = ok && isfinite(u[c]);
        U[c * nc + i] = u[c];
    }
    if (!ok) atomicOr(bad, 1);
}

// The same update with the step's decisions taken on the device from the residual norm
// pieces norms[0..1] (sum of R^2 vol, sum of vol): no update when the volume-weighted
// norm is below tol (converged) or not finite, relaxation 0.5 above 1e6 (as the host
// driver, src/Solver.cpp:1753-1758).  Lets the whole Newton step run without a host
// round trip before the update.
template <int NV>
__global__ void k_newton_update_dev(long nc, double* __restrict__ U, const double* __restrict__ dU,
                                    const double* __restrict__ norms, double tol, double gam, double wmin, int* bad) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double s0 = norms[0], s1 = norms[1];
    const double resVM = s1 == 0 ? 0.0 : sqrt(s0 / s1);
    if (!(resVM >= tol) || !isfinite(resVM)) return;
    double relax = 1.0;
    if (resVM > 1e6) relax = 0.5;
    else if (resVM > 2e3 && resVM < 1e2) relax = 0.9;
    double u[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) u[c] = U[c * nc + i] + dU[c * nc + i] * relax;
    double ke = 0.5 * (u[1] * u[1] + u[2] * u[2]) / (u[0] + 1e-12);
    double pn = (gam - 1.0) * (u[3] - ke);
    if (u[0] < 1e-5) u[0] = 1e-5;
    if (pn < 1e-5) {
        pn = 1e-5;
        u[3] = pn / (gam - 1.0) + ke;
    }
    if constexpr (NV == 6) {
        if (u[4] < 0.0) u[4] = 0.0;
        if (u[5] < u[0] * wmin) u[5] = u[0] * wmin;
    }
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        ok = ok && isfinite(u[c]);
        U[c * nc + i] = u[c];
    }
    if (!ok) atomicOr(bad, 1);
}

// The scalar control of a Newton step on the device, so that steps can follow one
// another without the host: the step's record, then (not converged, residual finite) the
// reference's CFL control (src/Solver.cpp:1747-1750, :1780-1796), the step counter and the
// next step's limiter-freeze decision (src/Solver.cpp:1714).  The same expressions in the
// same order as the host driver, so the trace is the same bit for bit.
struct NewtonCtl {
    int* ctl;        // [0] step, [1] stop (0 running, 1 converged, 2 non-finite residual),
                     // [2] the current step recomputes the limiter
    double* cfl;     // the CFL number (the next step's local time step reads it)
    double* rec;     // NEWTON_REC doubles per step of the chain
    const int* gi;   // the GMRES solve's ints: gi[1] = its last iteration
    int freeze_step;
    double freeze_cfl, cfl_max;
    int limited;     // second-order limited scheme
    double tol_rho;  // also stop at a density residual at or below this after step 5 (0 = off)
};
// record: res_vm, res_abs, res_rho, CFL used, GMRES iterations of the step's solve,
// limiter recomputed, outcome (0 updated, 1 converged, 2 non-finite residual, 3 not taken:
// an earlier step of the chain stopped), step index
constexpr int NEWTON_REC = 8;

// the step is converged: the reference's test on the all-component norm, or the optional
// density test (step is the step's index; every thread evaluates this from the same norms)
__device__ __forceinline__ bool newton_converged(const NewtonCtl& c, const double* norms, double resVM, double tol,
                                                 int step) {
    if (resVM < tol) return true;
    if (c.tol_rho > 0.0 && step > 5) {
        const double s1 = norms[1];
        const double rho = s1 == 0 ? 0.0 : sqrt(norms[2] / s1);
        return rho <= c.tol_rho;
    }
    return false;
}

__device__ __forceinline__ void newton_control(const NewtonCtl& c, const double* norms, double tol, int k) {
    const double s0 = norms[0], s1 = norms[1];
    const double resVM = s1 == 0 ? 0.0 : sqrt(s0 / s1);
    double* r = c.rec + (long)NEWTON_REC * k;
    const double cfl = *c.cfl;
    const int step = c.ctl[0];
    const int it = c.gi[1] + 1;
    r[0] = resVM;
    r[1] = sqrt(norms[3]);
    r[2] = s1 == 0 ? 0.0 : sqrt(norms[2] / s1);
    r[3] = cfl;
    r[4] = it;
    r[5] = c.ctl[2];
    r[7] = step;
    if (c.ctl[1]) {
        r[6] = 3.0;
        return;
    }
    if (!isfinite(resVM)) {
        c.ctl[1] = 2;
        r[6] = 2.0;
        return;
    }
    if (newton_converged(c, norms, resVM, tol, step)) {
        c.ctl[1] = 1;
        r[6] = 1.0;
        return;
    }
    r[6] = 0.0;
    double cf = cfl;
    if (it >= 29) {
        cf *= 0.5;
        if (cf < 0.05) cf = 0.05;
    }
    if (step > 5) {
        if (resVM > 1e6) cf *= 1.2;
        else cf *= 1.5;
        if (it >= 25) cf *= 0.5;
        if (cf > c.cfl_max) cf = c.cfl_max;
        if (cf < 0.1) cf = 0.1;
    }
    *c.cfl = cf;
    c.ctl[0] = step + 1;
    c.ctl[2] = (c.limited && !((step + 1) > c.freeze_step || cf > c.freeze_cfl)) ? 1 : 0;
}

// Optional local limit of a Newton update (no reference counterpart; off unless the
// caller asks, cfdg_config.update_limit): the cell's update du is scaled by the largest
// a <= 1 with |a d rho| <= lim rho, |a dp| <= lim p (dp the update's pressure change to
// first order) and, with SST, neither rho k nor rho w falling by more than lim of itself.
template <int NV>
__device__ __forceinline__ double update_scale(const double* u0, const double* du, double gam, double lim) {
    if (!(lim > 0.0)) return 1.0;
    double a = 1.0;
    const double r = u0[0];
    if (!(r > 0.0)) return 1.0;
    const double ir = 1.0 / r, uu = u0[1] * ir, vv = u0[2] * ir;
    const double p = (gam - 1.0) * (u0[3] - 0.5 * (u0[1] * uu + u0[2] * vv));
    const double dp = (gam - 1.0) * (du[3] - uu * du[1] - vv * du[2] + 0.5 * (uu * uu + vv * vv) * du[0]);
    if (fabs(du[0]) * a > lim * r) a = lim * r / fabs(du[0]);
    if (p > 0.0 && fabs(dp) * a > lim * p) a = lim * p / fabs(dp);
    if constexpr (NV == 6) {
        for (int c = 4; c < 6; ++c)
            if (u0[c] > 0.0 && du[c] < 0.0 && -du[c] * a > lim * u0[c]) a = lim * u0[c] / (-du[c]);
    }
    return a;
}

// k_newton_update_dev's update plus the scalar control in thread 0 of block 0 (chain
// step k, the solve's step `step` when no earlier step of the chain stopped).  The other
// threads take their converged / non-finite / relaxation decisions from the same norms,
// so a step after a stop changes nothing.
template <int NV>
__global__ void k_newton_update_chain(long nc, double* __restrict__ U, const double* __restrict__ dU,
                                      const double* __restrict__ norms, double tol, double gam, double wmin, int* bad,
                                      NewtonCtl c, int k, int step, double ulim) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) newton_control(c, norms, tol, k);
    if (i >= nc) return;
    const double s0 = norms[0], s1 = norms[1];
    const double resVM = s1 == 0 ? 0.0 : sqrt(s0 / s1);
    if (!isfinite(resVM) || newton_converged(c, norms, resVM, tol, step)) return;
    double relax = 1.0;
    if (resVM > 1e6) relax = 0.5;
    else if (resVM > 2e3 && resVM < 1e2) relax = 0.9;
    double u[NV], u0[NV], du[NV];
#pragma unroll
    for (int cc = 0; cc < NV; ++cc) {
        u0[cc] = U[cc * nc + i];
        du[cc] = dU[cc * nc + i] * relax;
    }
    const double a = update_scale<NV>(u0, du, gam, ulim);
#pragma unroll
    for (int cc = 0; cc < NV; ++cc) u[cc] = ulim > 0.0 ? u0[cc] + du[cc] * a : u0[cc] + du[cc];
    double ke = 0.5 * (u[1] * u[1] + u[2] * u[2]) / (u[0] + 1e-12);
    double pn = (gam - 1.0) * (u[3] - ke);
    if (u[0] < 1e-5) u[0] = 1e-5;
    if (pn < 1e-5) {
        pn = 1e-5;
        u[3] = pn / (gam - 1.0) + ke;
    }
    if constexpr (NV == 6) {
        if (u[4] < 0.0) u[4] = 0.0;
        if (u[5] < u[0] * wmin) u[5] = u[0] * wmin;
    }
    bool ok = true;
#pragma unroll
    for (int cc = 0; cc < NV; ++cc) {
        ok = ok && isfinite(u[cc]);
        U[cc * nc + i] = u[cc];
    }
    if (!ok) atomicOr(bad, 1);
}

// timeStepExplicit (src/Solver.cpp:1219-1243): U -= R (dt / vol), then rho >= 1e-3 and
// rhoE - kinetic energy >= 1e-3, in the reference's operation order; flags non-finite
template <int NV>
__global__ void k_explicit_update(long nc, double* __restrict__ U, const double* __restrict__ R,
                                  const double* __restrict__ vol, double dt, int* bad) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const double s = dt / vol[i];
    double u[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) u[c] = U[c * nc + i] - R[c * nc + i] * s;
    if (u[0] < 1e-3) u[0] = 1e-3;
    double ke = 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0];
    double ie = u[3] - ke;
    if (ie < 1e-3) u[3] = ke + 1e-3;
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        ok = ok && isfinite(u[c]);
        U[c * nc + i] = u[c];
    }
    if (!ok) atomicOr(bad, 1);
}

// solveUnsteady's Newton right-hand side (src/Solver.cpp:1822-1838):
// F = (U - U_old) vol / dt + R, rhs = -F, with the pieces of the volume-weighted norm of
// F / vol over rho, rhou, rhov, rhoE: out2 = (sum of |F/vol|^2 vol, sum of vol)
template <int NV>
__global__ void __launch_bounds__(RED_THREADS) k_unsteady_rhs(long nc, const double* __restrict__ U,
                                                              const double* __restrict__ Uold,
                                                              const double* __restrict__ R,
                                                              const double* __restrict__ vol, double dt,
                                                              double* __restrict__ rhs, RedScratch rs, double* out2) {
    double v[2] = {0.0, 0.0};
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        const double vl = vol[i];
        const double s = vl / dt;
        double f[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            f[c] = (U[q] - Uold[q]) * s + R[q];
            rhs[q] = f[c] * (-1.0);
        }
        double a = f[0] / vl, b = f[1] / vl, c2 = f[2] / vl, e = f[3] / vl;
        v[0] += (a * a + b * b + c2 * c2 + e * e) * vl;
        v[1] += vl;
    }
    grid_finish<2>(v, rs, out2);
}

// U += relax * dU (the dual-time Newton update of src/Solver.cpp:1853-1856, no clamps)
template <int NV>
__global__ void k_relaxed_add(long nc, double* __restrict__ U, const double* __restrict__ dU, double relax, int* bad) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        long q = c * nc + i;
        double u = U[q] + dU[q] * relax;
        ok = ok && isfinite(u);
        U[q] = u;
    }
    if (!ok) atomicOr(bad, 1);
}

static __global__ void k_fill(long n, double* __restrict__ x, double v) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) x[q] = v;
}

// AoS (stride doubles per cell, reference numbering) <-> SoA (np planes, internal
// numbering); AoS slots np..stride-1 are written as zero
template <class T>
__global__ void k_aos_to_soa(long nc, int np, int stride, const double* __restrict__ aos, const int* __restrict__ perm,
                             T* __restrict__ soa) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    long src = (long)perm[i] * stride;
    for (int c = 0; c < np; ++c) soa[c * nc + i] = (T)aos[src + c];
}
template <class T>
__global__ void k_soa_to_aos(long nc, int np, int stride, const T* __restrict__ soa, const int* __restrict__ perm,
                             double* __restrict__ aos) {
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    long dst = (long)perm[i] * stride;
    for (int c = 0; c < stride; ++c) aos[dst + c] = c < np ? (double)soa[c * nc + i] : 0.0;
}

// ---- a caller's pinned AoS array read or written in place over the CPU-GPU link
// (row staging: residual.cuh rows_load / rows_store)
// np planes of soa (internal numbering) from a caller's rows of `stride` doubles
static __global__ void __launch_bounds__(ROW_BLOCK) k_rows_to_soa(long nc, int np, int stride, const double* __restrict__ aos,
                                                         const int* __restrict__ iperm, double* __restrict__ soa) {
    __shared__ __align__(16) double sm[ROW_BLOCK * ROW_MAX_STRIDE];
    long r0;
    const int rows = rows_load(aos, nc, stride, sm, r0);
    if ((int)threadIdx.x >= rows) return;
    const long c = iperm[r0 + threadIdx.x];
    for (int k = 0; k < np; ++k) soa[k * nc + c] = sm[threadIdx.x * stride + k];
}

// a caller's rows of `stride` doubles from np planes of soa (slots np..stride-1 zero)
template <class T>
__global__ void __launch_bounds__(ROW_BLOCK) k_soa_to_rows(long nc, int np, int stride, const T* __restrict__ soa,
                                                         const int* __restrict__ iperm, double* __restrict__ aos) {
    __shared__ __align__(16) double sm[ROW_BLOCK * ROW_MAX_STRIDE];
    const long r0 = (long)blockIdx.x * ROW_BLOCK;
    const long left = nc - r0;
    const int rows = left < ROW_BLOCK ? (int)left : ROW_BLOCK;
    if ((int)threadIdx.x < rows) {
        const long c = iperm[r0 + threadIdx.x];
        for (int k = 0; k < stride; ++k) sm[threadIdx.x * stride + k] = k < np ? (double)soa[k * nc + c] : 0.0;
    }
    rows_store(aos, r0, rows, stride, sm);
}

}  // namespace cfdg
