// Device-resident GMRES: the Arnoldi iteration runs as the body of a CUDA-graph WHILE
// node, with the Hessenberg column, the Givens rotations and the convergence test on the
// device, so a whole Krylov solve is one graph launch with no host round trip.
//
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2).  Each pass's dot
// products are fused into the kernel that produces the vector they read.  With the exact
// (dual-number) J v an iteration is five kernels and two grid reductions:
//   V_j = w - V h2 (deferred), z = V_j / D, dual primitives    (k_gmres_prim_z)
//   dual gradients, dual face fluxes                           (k_grad, k_flux)
//   J v gather   -> w and h1 = V^T w                           (k_gmres_gather_dot)
//   w -= V h1    -> w, h2 = V^T w and |w|^2; Givens step        (k_gmres_update_dot<T, true>)
// The norm of V_{j+1} = w - V h2 is taken as |w|^2 - |h2|^2 (Pythagoras over the
// orthonormal basis, as in the one-reduction CGS2 variants of Swirydowicz, Langou,
// Ananthan, Yang and Thomas, "Low synchronization Gram-Schmidt and GMRES algorithms",
// Numer. Linear Algebra Appl. 2021), so V_{j+1} itself is formed by the next iteration's
// first kernel and never needs a reduction of its own.  The FD J v path keeps the
// explicit final pass:
//   w -= V h2    -> V_{j+1}, |V_{j+1}|, and the Givens step  (k_gmres_update_final)
// Every thread reads back only the elements it wrote itself, so no grid barrier is
// needed inside a kernel; the last block to finish each kernel sums the block partials
// in block order (deterministic).  Basis vectors are stored unnormalised with a scale
// factor sc[i] = 1/|V_i| (FP64) applied wherever they are read.  The Givens and
// least-squares arithmetic is the reference's (src/Solver.cpp:1562-1599) in FP64.
//
// Termination: the last block of k_gmres_update_final is the only place that advances j;
// it runs once per body execution and clears the loop condition when j + 1 reaches m (or
// on convergence), so the loop runs at most m times.  The same kernels also run outside a
// graph (in_graph = 0), launched one iteration at a time by a host loop that reads the
// done flag: the stream driver, which times every kernel with events.
#pragma once
#include <cuda_runtime.h>
#include "linalg.cuh"

namespace cfdg {

constexpr int KRY_MAXM = 128;  // largest Krylov dimension of the device solver

struct GmresDev {
    int* gi;          // [0] j, [1] k (last iteration), [2] done, [3] m
    double* beta;     // [0] beta, [1] tol, [2] beta^2
    double* g;        // [m+1]
    double* cs;       // [m]
    double* sn;       // [m]
    double* H;        // [(m+1) * m], column j at H + j*(m+1)
    double* y;        // [m]
    double* h1;       // [m+1] first CGS pass
    double* h2;       // [m+1] second CGS pass
    double* hsq;      // [2] squared norms ([1]: after the second pass)
    double* sc;       // [m+1] scale of each stored basis vector
    double* partial;  // [(KRY_MAXM+1) * RED_BLOCKS]
    unsigned* counter;
    int in_graph;     // 1: the kernels run inside the WHILE graph and set its condition
};

// beta = sqrt(|rhs|^2); empty solve when beta < 1e-12 (src/Solver.cpp:1514-1516)
static __global__ void k_gmres_init(GmresDev d, int m, double tol, cudaGraphConditionalHandle h) {
    double b = sqrt(d.beta[2]);
    d.beta[0] = b;
    d.beta[1] = tol;
    d.gi[0] = 0;
    d.gi[3] = m;
    for (int i = 0; i <= m; ++i) {
        d.g[i] = 0.0;
        d.sc[i] = 1.0;
    }
    for (int i = 0; i < m; ++i) { d.cs[i] = 0.0; d.sn[i] = 0.0; }
    d.g[0] = b;
    if (b < 1e-12) {
        d.gi[1] = -1;
        d.gi[2] = 1;
        if (d.in_graph) cudaGraphSetConditional(h, 0);
    } else {
        d.gi[1] = 0;
        d.gi[2] = 0;
    }
}

// Arithmetic of the vector kernels.  GB300 issues FP64 at 1/64 of its FP32 rate, so with
// an FP32 basis the per-element work (products, the update, per-thread and per-warp
// partial sums of at most a few hundred products) is FP32 and only the block and grid
// levels of each reduction are FP64; with an FP64 basis everything is FP64.
template <class T> struct KryAcc { typedef double type; };
template <> struct KryAcc<float> { typedef float type; };

template <class A>
__device__ __forceinline__ A warp_sum_t(A v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

constexpr int KRY_TILE = 16;  // basis vectors per pass over a thread's elements
constexpr int KRY_WARPS = RED_THREADS / 32;  // most warps of a block (blocks of 64-256 threads)

// per-warp sums of one tile of per-thread partial dots into wsum[vector][warp]
template <class A>
__device__ __forceinline__ void tile_to_smem(const A (&v)[KRY_TILE], int i0, int nt, double (*wsum)[KRY_WARPS]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < KRY_TILE; ++t)
        if (t < nt) {
            A s = warp_sum_t(v[t]);
            if (lane == 0) wsum[i0 + t][warp] = (double)s;
        }
}

// Block partials of h[0..j] from wsum, then in the last block to finish the sums over the
// blocks in block order: h[i] = sc[i] * sum (h[jraw] = sum, unscaled).  Returns true in
// the last block.
__device__ __forceinline__ bool dots_finish(const GmresDev& d, int j, double (*wsum)[KRY_WARPS], double* h,
                                            int jraw = -1) {
    __syncthreads();
    const int nwarp = blockDim.x >> 5;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double sb = 0.0;
        for (int w = 0; w < nwarp; ++w) sb += wsum[i][w];
        d.partial[(long)i * RED_BLOCKS + blockIdx.x] = sb;
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) last = atomicAdd(d.counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return false;
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = warp; i <= j; i += nwarp) {
        double sg = 0.0;
#pragma unroll 4
        for (int b = lane; b < (int)gridDim.x; b += 32) sg += __ldcg(d.partial + (long)i * RED_BLOCKS + b);
        sg = warp_sum(sg);
        if (lane == 0) h[i] = (i == jraw ? 1.0 : d.sc[i]) * sg;
    }
    __syncthreads();
    if (threadIdx.x == 0) *d.counter = 0u;
    return true;
}

// V0 = rhs * (1/beta)
template <class T>
__global__ void k_gmres_v0(long n, T* V0, const double* rhs, GmresDev d) {
    if (d.gi[2]) return;
    __shared__ double ib;
    if (threadIdx.x == 0) ib = 1.0 / d.beta[0];
    __syncthreads();
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        V0[q] = (T)(rhs[q] * ib);
}

// Dinv = 1 / D per plane (one plane, three with SST), once per solve
template <class T, int NV>
__global__ void k_gmres_dinv(long nc, const double* __restrict__ D, T* __restrict__ Dinv) {
    const long n = (NV == 6 ? 3 : 1) * nc;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
        Dinv[q] = (T)(1.0 / D[q]);
}

template <class T, int NV>
__device__ __forceinline__ T dinv_of(const T* __restrict__ Dinv, long nc, long i, int c, T d0) {
    return (NV == 6 && c >= 4) ? Dinv[(c - 3) * nc + i] : d0;
}

// z = V_j * (1/D) per cell (src/Solver.cpp:1536-1538)
template <class T, int NV>
__global__ void k_gmres_z(long nc, const T* V, long L, const T* __restrict__ Dinv, T* z, GmresDev d) {
    const int j = d.gi[0];
    const T* Vj = V + (long)j * L;
    const T sj = (T)d.sc[j];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        T a = Dinv[i];
#pragma unroll
        for (int c = 0; c < NV; ++c) z[c * nc + i] = Vj[c * nc + i] * sj * dinv_of<T, NV>(Dinv, nc, i, c, a);
    }
}

// For j > 0 first the deferred end of the previous iteration's orthogonalisation,
// V_j = w - sum_{i<j} h2[i] sc[i] V_i (stored unnormalised; sc[j] is already set), then
// z = V_j * (1/D) fused with the primitive stage of the dual J v: W.v, W.d of (U, z)
template <class T, int NV>
__global__ void __launch_bounds__(256) k_gmres_prim_z(int nc, Flow<T> F, const T* __restrict__ U, T* V, long L,
                                                      const T* __restrict__ Dinv, T* __restrict__ z, Field<T> W,
                                                      const T* __restrict__ w, GmresDev d) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ A hs[KRY_MAXM];
    if (j > 0) {
        for (int k = threadIdx.x; k < j; k += blockDim.x) hs[k] = (A)(d.h2[k] * d.sc[k]);
        __syncthreads();
    }
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    T* Vj = V + (long)j * L;
    const T sj = (T)d.sc[j];
    const T a = Dinv[i];
    T vj[NV];
    if (j > 0) {
        A acc[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = (A)w[c * nc + i];
#pragma unroll 2
        for (int k = 0; k < j; ++k) {
            const T* Vk = V + (long)k * L;
            const A hk = hs[k];
#pragma unroll
            for (int c = 0; c < NV; ++c) acc[c] -= hk * (A)Vk[c * nc + i];
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            vj[c] = (T)acc[c];
            Vj[c * nc + i] = vj[c];
        }
    } else {
#pragma unroll
        for (int c = 0; c < NV; ++c) vj[c] = Vj[c * nc + i];
    }
    Dual<T> u[6];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        T zc = vj[c] * sj * dinv_of<T, NV>(Dinv, nc, i, c, a);
        z[c * nc + i] = zc;
        u[c] = Dual<T>(U[c * nc + i], zc);
    }
    if (NV == 4) u[4] = u[5] = Dual<T>(T(0), T(0));
    prim_cell<Dual<T>, NV>(F, u[0], u[1], u[2], u[3], u[4], u[5], W, i);
}

// h[i] = sc[i] <w, V_i>, i = 0..j (the first pass of the FD J v path)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_multidot(long L, const T* __restrict__ w,
                                                                const T* __restrict__ V, GmresDev d, double* h) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ double wsum[KRY_MAXM + 1][KRY_WARPS];
    for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
        const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
        A v[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
        for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x) {
            A wq = (A)w[q];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t)
                if (t < nt) v[t] += wq * (A)V[(long)(i0 + t) * L + q];
        }
        tile_to_smem(v, i0, nt, wsum);
    }
    dots_finish(d, j, wsum, h);
}

// The gather of the dual J v (as k_gather: the faces' F*A derivatives in reference face
// order, minus the SST source derivatives, plus z vol / dt) into w, fused with the first
// CGS pass h1 = V^T w.  Grid-stride over cells (at most RED_BLOCKS blocks).
template <class T, int NV>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_gather_dot(MeshView<T> m, const T* __restrict__ FA,
                                                                  long fa_stride, T* __restrict__ w,
                                                                  const T* __restrict__ z, const T* __restrict__ dt,
                                                                  const T* __restrict__ src, const T* __restrict__ V,
                                                                  long L, GmresDev d) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    const long nc = m.nc;
    __shared__ double wsum[KRY_MAXM + 1][KRY_WARPS];
    for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
        const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
        A v[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
        for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
            T acc[NV];
            if (i0 == 0) {
#pragma unroll
                for (int c = 0; c < NV; ++c) acc[c] = T(0);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    int e = m.cf[(long)k * nc + i];
                    if (e < 0) break;
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
                    acc[4] = acc[4] - src[i];
                    acc[5] = acc[5] - src[nc + i];
                }
                T tc = m.vol[i] / (dt[i] + T(1e-30));
#pragma unroll
                for (int c = 0; c < NV; ++c) {
                    acc[c] = acc[c] + z[c * nc + i] * tc;
                    w[c * nc + i] = acc[c];
                }
            } else {
#pragma unroll
                for (int c = 0; c < NV; ++c) acc[c] = w[c * nc + i];
            }
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t)
                if (t < nt) {
                    const T* Vi = V + (long)(i0 + t) * L;
                    A s = A(0);
#pragma unroll
                    for (int c = 0; c < NV; ++c) s += (A)acc[c] * (A)Vi[c * nc + i];
                    v[t] += s;
                }
        }
        tile_to_smem(v, i0, nt, wsum);
    }
    dots_finish(d, j, wsum, d.h1);
}

__device__ __forceinline__ void givens_step(const GmresDev& d, cudaGraphConditionalHandle hnd, double hsq);

// w -= sum_{i<=j} h1[i] sc[i] V_i, fused with the second CGS pass h2 = V^T w.  With LAST
// (the exact J v body) also |w|^2, and the last block takes |V_{j+1}|^2 = |w|^2 - |h2|^2
// (clamped at 0), sets sc[j+1] = 1/|V_{j+1}| (1 under the breakdown guard |.| <= 1e-12 of
// src/Solver.cpp:1553-1558) and runs the Givens step; V_{j+1} = w - V h2 is formed by the
// next iteration's k_gmres_prim_z.
template <class T, bool LAST>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_update_dot(long L, T* __restrict__ w, const T* __restrict__ V,
                                                                  GmresDev d, cudaGraphConditionalHandle hnd) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ A hs[KRY_MAXM + 1];
    __shared__ double wsum[KRY_MAXM + 1][KRY_WARPS];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) hs[i] = (A)(d.h1[i] * d.sc[i]);
    __syncthreads();
    A nw = A(0);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x) {
        A a = (A)w[q];
        for (int i = 0; i <= j; ++i) a -= hs[i] * (A)V[(long)i * L + q];
        T t = (T)a;
        w[q] = t;
        if (LAST) nw += (A)t * (A)t;
    }
    if (LAST) {
        nw = warp_sum_t(nw);
        if ((threadIdx.x & 31) == 0) wsum[j + 1][threadIdx.x >> 5] = (double)nw;
    }
    for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
        const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
        A v[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
        for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x) {
            A wq = (A)w[q];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t)
                if (t < nt) v[t] += wq * (A)V[(long)(i0 + t) * L + q];
        }
        tile_to_smem(v, i0, nt, wsum);
    }
    if (!LAST) {
        dots_finish(d, j, wsum, d.h2);
        return;
    }
    if (!dots_finish(d, j + 1, wsum, d.h2, j + 1)) return;
    if (threadIdx.x >= 32) return;
    const int lane = threadIdx.x;
    double s2 = 0.0;
    for (int i = lane; i <= j; i += 32) {
        double h = d.h2[i];
        s2 += h * h;
    }
    s2 = __shfl_sync(0xffffffffu, warp_sum(s2), 0);
    const double hsq = fmax(d.h2[j + 1] - s2, 0.0);
    if (lane == 0) {
        d.hsq[1] = hsq;
        double hv = sqrt(hsq);
        d.sc[j + 1] = hv > 1e-12 ? 1.0 / hv : 1.0;
    }
    givens_step(d, hnd, hsq);
}

// Hessenberg column, Givens rotations and the convergence test (src/Solver.cpp:1550-1588);
// advances j or ends the loop.  Called by one full warp: the lanes stage the column and
// the previous rotations in shared memory, lane 0 runs the rotation chain there (the
// chain is serial; shared memory keeps its loads short), the lanes write back.
__device__ __forceinline__ void givens_step(const GmresDev& d, cudaGraphConditionalHandle hnd, double hsq) {
    __shared__ double col_s[KRY_MAXM + 2], cs_s[KRY_MAXM], sn_s[KRY_MAXM];
    const int lane = threadIdx.x & 31;
    const int j = d.gi[0], m = d.gi[3];
    double* col = d.H + (long)j * (m + 1);
    for (int i = lane; i <= j; i += 32) {
        col_s[i] = d.h1[i] + d.h2[i];
        if (i < j) {
            cs_s[i] = d.cs[i];
            sn_s[i] = d.sn[i];
        }
    }
    __syncwarp();
    if (lane == 0) {
        col_s[j + 1] = sqrt(hsq);
        for (int i = 0; i < j; ++i) {
            double t = cs_s[i] * col_s[i] + sn_s[i] * col_s[i + 1];
            col_s[i + 1] = -sn_s[i] * col_s[i] + cs_s[i] * col_s[i + 1];
            col_s[i] = t;
        }
        double a = col_s[j], b = col_s[j + 1], c, sn;
        if (fabs(b) < 1e-14) {
            c = 1.0;
            sn = 0.0;
        } else {
            double t = sqrt(a * a + b * b);
            c = a / t;
            sn = b / t;
        }
        d.cs[j] = c;
        d.sn[j] = sn;
        col_s[j] = c * a + sn * b;
        col_s[j + 1] = 0.0;
        double gj = d.g[j];
        d.g[j + 1] = -sn * gj;
        d.g[j] = c * gj;
        bool conv = fabs(-sn * gj) < d.beta[1] * d.beta[0];
        if (conv || j + 1 >= m) {
            d.gi[1] = j;
            d.gi[2] = 1;
            if (d.in_graph) cudaGraphSetConditional(hnd, 0);
        } else {
            d.gi[0] = j + 1;
        }
    }
    __syncwarp();
    for (int i = lane; i <= j + 1; i += 32) col[i] = col_s[i];
}

// V_{j+1} = w - sum_{i<=j} h2[i] sc[i] V_i, stored unnormalised, and |V_{j+1}|^2; the
// last block sets sc[j+1] = 1/|V_{j+1}| (1 under the breakdown guard |.| <= 1e-12 of
// src/Solver.cpp:1553-1558) and runs the Givens step.
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_update_final(long L, const T* __restrict__ w,
                                                                    T* __restrict__ V, GmresDev d,
                                                                    cudaGraphConditionalHandle hnd) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ A hs[KRY_MAXM + 1];
    __shared__ double wsum[KRY_WARPS];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) hs[i] = (A)(d.h2[i] * d.sc[i]);
    __syncthreads();
    T* Vn = V + (long)(j + 1) * L;
    A nrm = A(0);
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x) {
        A a = (A)w[q];
        for (int i = 0; i <= j; ++i) a -= hs[i] * (A)V[(long)i * L + q];
        T t = (T)a;
        Vn[q] = t;
        nrm += (A)t * (A)t;
    }
    nrm = warp_sum_t(nrm);
    if (lane == 0) wsum[warp] = (double)nrm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sb = 0.0;
        for (int w_ = 0; w_ < (int)(blockDim.x >> 5); ++w_) sb += wsum[w_];
        d.partial[blockIdx.x] = sb;
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) last = atomicAdd(d.counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    if (warp == 0) {
        double sg = 0.0;
#pragma unroll 4
        for (int b = lane; b < (int)gridDim.x; b += 32) sg += __ldcg(d.partial + b);
        sg = __shfl_sync(0xffffffffu, warp_sum(sg), 0);
        if (lane == 0) {
            d.hsq[1] = sg;
            double hv = sqrt(sg);
            d.sc[j + 1] = hv > 1e-12 ? 1.0 / hv : 1.0;
            *d.counter = 0u;
        }
        givens_step(d, hnd, sg);
    }
}

// back substitution H y = g over the k+1 leading columns (src/Solver.cpp:1592-1599)
static __global__ void k_gmres_backsub(GmresDev d) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int k = d.gi[1], m = d.gi[3];
    for (int i = k; i >= 0; --i) {
        double yi = d.g[i];
        for (int l = i + 1; l <= k; ++l) yi -= d.H[(long)l * (m + 1) + i] * d.y[l];
        d.y[i] = yi / d.H[(long)i * (m + 1) + i];
    }
}

// x = (sum_{i<=k} V_i sc_i y_i) / D (src/Solver.cpp:1610-1615, accumulated before the
// scaling); zero when the solve was empty
template <class T, int NV>
__global__ void k_gmres_solution_dev(long nc, const T* __restrict__ V, long L, GmresDev d,
                                     const double* __restrict__ D, double* __restrict__ x) {
    const int k = d.gi[1];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double id[NV];
        d_inv<NV>(D, nc, i, id);
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            double acc = 0.0;
            for (int j = 0; j <= k; ++j) acc += (double)V[j * L + q] * (d.y[j] * d.sc[j]);
            x[q] = acc * id[c];
        }
    }
}

}  // namespace cfdg
