// Device-resident GMRES: the Arnoldi iteration runs as the body of a CUDA-graph WHILE
// node, with the Hessenberg column, the Givens rotations and the convergence test on the
// device, so a whole Krylov solve is one graph launch with no host round trip.
//
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2): two multi-dot
// kernels and two update kernels per iteration whatever the iteration index, against
// j+2 launches for modified Gram-Schmidt.  The Givens/least-squares arithmetic is the
// reference's (src/Solver.cpp:1562-1599) in FP64.
//
// Termination: k_gmres_givens is the only kernel that advances j, it runs once per body
// execution, and it clears the loop condition when j + 1 reaches m (or on convergence),
// so the loop runs at most m times.
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
    double* hsq;      // [2] squared norms after each pass
    double* partial;  // [(KRY_MAXM+1) * RED_BLOCKS]
    unsigned* counter;
};

// beta = sqrt(|rhs|^2); empty solve when beta < 1e-12 (src/Solver.cpp:1514-1516)
static __global__ void k_gmres_init(GmresDev d, int m, double tol, cudaGraphConditionalHandle h) {
    double b = sqrt(d.beta[2]);
    d.beta[0] = b;
    d.beta[1] = tol;
    d.gi[0] = 0;
    d.gi[3] = m;
    for (int i = 0; i <= m; ++i) d.g[i] = 0.0;
    for (int i = 0; i < m; ++i) { d.cs[i] = 0.0; d.sn[i] = 0.0; }
    d.g[0] = b;
    if (b < 1e-12) {
        d.gi[1] = -1;
        d.gi[2] = 1;
        cudaGraphSetConditional(h, 0);
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

// block reduction of K per-thread values: warp sums in A, then FP64 across the warps;
// the FP64 block sums are valid in thread 0
template <class A, int K>
__device__ __forceinline__ void block_sum_mixed(const A (&v)[K], double (&out)[K]) {
    __shared__ double sm[K][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        A s = warp_sum_t(v[k]);
        if (lane == 0) sm[k][w] = (double)s;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double x = lane < (int)(blockDim.x >> 5) ? sm[k][lane] : 0.0;
            out[k] = warp_sum(x);
        }
    }
    __syncthreads();
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

// z = V_j * (1/D) per cell (src/Solver.cpp:1536-1538)
template <class T, int NV>
__global__ void k_gmres_z(long nc, const T* V, long L, const T* __restrict__ Dinv, T* z, GmresDev d) {
    const T* Vj = V + (long)d.gi[0] * L;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        T a = Dinv[i];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            T id = (NV == 6 && c >= 4) ? Dinv[(c - 3) * nc + i] : a;
            z[c * nc + i] = Vj[c * nc + i] * id;
        }
    }
}

// h[i] = <w, V_i>, i = 0..j.  Sixteen basis vectors per pass over w (each thread keeps
// sixteen partial products, independent loads in flight); warp sums per vector into
// shared memory with no block barrier between passes; one barrier, then the block's
// partials in FP64; the last block to finish sums them over the blocks in block order,
// one warp per basis vector.
constexpr int KRY_TILE = 16;

template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_multidot(long L, const T* __restrict__ w,
                                                                const T* __restrict__ V, GmresDev d, double* h) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    __shared__ double wsum[KRY_MAXM + 1][RED_THREADS / 32];
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
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t)
            if (t < nt) {
                A sv = warp_sum_t(v[t]);
                if (lane == 0) wsum[i0 + t][warp] = (double)sv;
            }
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double sb = 0.0;
        for (int ww = 0; ww < nwarp; ++ww) sb += wsum[i][ww];
        d.partial[(long)i * RED_BLOCKS + blockIdx.x] = sb;
    }
    __threadfence();
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) last = atomicAdd(d.counter, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int i = warp; i <= j; i += nwarp) {
        double sg = 0.0;
#pragma unroll 4
        for (int b = lane; b < (int)gridDim.x; b += 32) sg += __ldcg(d.partial + (long)i * RED_BLOCKS + b);
        sg = warp_sum(sg);
        if (lane == 0) h[i] = sg;
    }
    __syncthreads();
    if (threadIdx.x == 0) *d.counter = 0u;
}

// w -= sum_{i<=j} h[i] V_i, then |w|^2 into *hsq
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_update(long L, T* __restrict__ w, const T* __restrict__ V,
                                                              GmresDev d, const double* h, double* hsq) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ A hs[KRY_MAXM + 1];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) hs[i] = (A)h[i];
    __syncthreads();
    A v[1] = {A(0)};
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x) {
        A a = (A)w[q];
        for (int i = 0; i <= j; ++i) a -= hs[i] * (A)V[(long)i * L + q];
        T t = (T)a;
        w[q] = t;
        v[0] += (A)t * (A)t;
    }
    double bs[1];
    block_sum_mixed<A, 1>(v, bs);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        d.partial[blockIdx.x] = bs[0];
        __threadfence();
        last = atomicAdd(d.counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s[1] = {0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) s[0] += __ldcg(d.partial + b);
    block_sum_mixed<double, 1>(s, bs);
    if (threadIdx.x == 0) {
        *hsq = bs[0];
        *d.counter = 0u;
    }
}

// V_{j+1} = w / |w| when |w| > 1e-12 (the breakdown guard of src/Solver.cpp:1553-1558)
template <class T>
__global__ void k_gmres_store(long L, const T* w, T* V, GmresDev d) {
    const int j = d.gi[0];
    __shared__ T sc;
    if (threadIdx.x == 0) {
        double hv = sqrt(d.hsq[1]);
        sc = (T)(hv > 1e-12 ? 1.0 / hv : 1.0);
    }
    __syncthreads();
    T* Vn = V + (long)(j + 1) * L;
    const T s = sc;
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < L; q += (long)gridDim.x * blockDim.x)
        Vn[q] = w[q] * s;
}

// Hessenberg column, Givens rotations and the convergence test (src/Solver.cpp:1550-1588);
// advances j or ends the loop.  One thread.
static __global__ void k_gmres_givens(GmresDev d, cudaGraphConditionalHandle hnd) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int j = d.gi[0], m = d.gi[3];
    double* col = d.H + (long)j * (m + 1);
    for (int i = 0; i <= j; ++i) col[i] = d.h1[i] + d.h2[i];
    col[j + 1] = sqrt(d.hsq[1]);
    for (int i = 0; i < j; ++i) {
        double t = d.cs[i] * col[i] + d.sn[i] * col[i + 1];
        col[i + 1] = -d.sn[i] * col[i] + d.cs[i] * col[i + 1];
        col[i] = t;
    }
    double a = col[j], b = col[j + 1];
    if (fabs(b) < 1e-14) {
        d.cs[j] = 1.0;
        d.sn[j] = 0.0;
    } else {
        double t = sqrt(a * a + b * b);
        d.cs[j] = a / t;
        d.sn[j] = b / t;
    }
    col[j] = d.cs[j] * a + d.sn[j] * b;
    col[j + 1] = 0.0;
    d.g[j + 1] = -d.sn[j] * d.g[j];
    d.g[j] = d.cs[j] * d.g[j];
    bool conv = fabs(d.g[j + 1]) < d.beta[1] * d.beta[0];
    if (conv || j + 1 >= m) {
        d.gi[1] = j;
        d.gi[2] = 1;
        cudaGraphSetConditional(hnd, 0);
    } else {
        d.gi[0] = j + 1;
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

// x = (sum_{i<=k} V_i y_i) / D (src/Solver.cpp:1610-1615, accumulated before the
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
            for (int j = 0; j <= k; ++j) acc += (double)V[j * L + q] * d.y[j];
            x[q] = acc * id[c];
        }
    }
}

}  // namespace cfdg
