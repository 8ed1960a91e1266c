// Device-resident GMRES: the Arnoldi iteration runs as the body of a CUDA-graph WHILE
// node, with the Hessenberg column, the Givens rotations and the convergence test on the
// device, so a whole Krylov solve is one graph launch with no host round trip.
//
// Orthogonalisation is classical Gram-Schmidt applied twice (CGS2).  With the exact
// (dual-number) J v it runs in its delayed one-reduction form (DCGS2: Swirydowicz, Langou,
// Ananthan, Yang and Thomas, "Low synchronization Gram-Schmidt and GMRES algorithms",
// Numer. Linear Algebra Appl. 2021): J is applied to the pending vector P_j, the product
// of the first pass only, and the second pass of P_j happens one iteration later, from
// dots taken in the same reduction as the next first pass.  An iteration is four kernels
// and one grid reduction:
//   finish P_{j-1} (second pass, norm by Pythagoras) into V_{j-1}, first pass of the
//   last product into P_j, z = P_j / D, dual primitives   (k_gmres_prim_z; one extra
//   block: the Givens step of column j - 2, first-pass entries of column j - 1)
//   dual gradients, dual face fluxes                       (k_grad, k_flux)
//   J v gather -> w, block partials of the dots of
//   V_0..V_{j-1}, P_j with P_j and with w                  (k_gmres_gather_dot)
// The first-pass entries of the new Hessenberg column come from the Arnoldi relation
// J V s = V H s over the finished columns, so no reduction reads the corrected product.
// The FD J v path keeps the explicit three-kernel CGS2:
//   h1 = V^T w                                              (k_gmres_multidot)
//   w -= V h1, h2 = V^T w                                   (k_gmres_update_dot)
//   w -= V h2    -> V_{j+1}, |V_{j+1}|, and the Givens step  (k_gmres_update_final)
// Every thread reads back only the elements it wrote itself, so no grid barrier is
// needed inside a kernel.  A grid reduction is either finished by the last block to
// finish (a ticket counter, FD path) or, in the exact body, by every block of the next
// kernel from the block partials; both sum in a fixed order (deterministic).  Basis
// vectors are stored unnormalised with a scale factor sc[i] = 1/|V_i| (FP64) applied
// wherever they are read.  The Givens and least-squares arithmetic is the reference's
// (src/Solver.cpp:1562-1599) in FP64.
//
// Termination: the Givens step is the only place that ends the loop: it clears the loop
// condition and raises the done flag when j + 1 reaches m (or on convergence), so at most
// m columns are formed.  The exact J v graph body holds several iterations (a WHILE
// iteration costs ~3 us of its own on GB300); the kernels of the iterations after the
// finishing one see the done flag and return at once.  The same kernels also run outside
// a graph (in_graph = 0), launched one iteration at a time by a host loop that reads the
// done flag: the stream driver, which times every kernel with events.
#pragma once
#include <cuda_runtime.h>
#include "linalg.cuh"
#include "pdl.cuh"

namespace cfdg {

constexpr int KRY_MAXM = 128;  // largest Krylov dimension of the device solver
// Arnoldi iterations per WHILE-body execution with the exact J v; measured on the
// 28,800-cell plate with the four-kernel body: 3, 4, 5, 6 give 783.5, 783, 780, 780 M
// cell-residuals/s (the same GB300)
constexpr int KRY_BODY_ITERS = 4;
// Default cell count from which the gather and the dots of an Arnoldi iteration run as two
// kernels (k_gmres_gather_w, then k_gmres_gather_dot<..., true>; cfdg_config
// gather_split_cells): on large meshes the fused kernel's per-cell dependent face gathers
// hold back its streaming dots; on small ones the kernel boundary costs more than it saves
// (stream-driver stage times, laminar bump, FP32 basis: fused / split 10.1 / 12.4 us at 60k
// cells, 14.7 / 16.2 at 119k, 39.7 / 26.2 at 250k, 114 / 67 at 1M).
constexpr long KRY_SPLIT_GATHER_CELLS = 150000;

struct GmresDev {
    int* gi;          // [0] j (FD body), [1] k (last iteration), [2] done, [3] m, [4] this iteration
                      // (exact J v body), [5] products reduced (exact J v body); 16-byte aligned
    double* beta;     // [0] beta, [1] tol, [2] beta^2
    double* g;        // [m+1]
    double* cs;       // [m]
    double* sn;       // [m]
    double* H;        // [(m+1) * m], column j at H + j*(m+1) (rotated)
    double* Hu;       // [(m+1) * m], the same columns before the rotations (exact J v body)
    double* sig;      // [m+2] scale of each iteration's pending vector (exact J v body)
    double* ilam;     // [m+2] its first-pass vector over that vector (exact J v body)
    double* y;        // [m]
    double* h1;       // [m+1] first CGS pass (of the newest column)
    double* h2;       // [m+1] second CGS pass
    double* hsq;      // [2] squared norms ([1]: after the second pass)
    double* sc;       // [m+1] scale of each stored basis vector
    double* partial;  // [(2 KRY_MAXM + 3) * RED_BLOCKS] block partials (rows of RED_BLOCKS)
    int nb1;          // blocks of the gather kernel that writes them (exact J v body; set at launch)
    unsigned* counter;
    int in_graph;     // 1: the kernels run inside the WHILE graph and set its condition
    const int* skip;  // optional: when *skip is set the solve is empty (x = 0, no iteration):
                      // a chained Newton step after the chain stopped
};

// Arithmetic of the vector kernels.  On GB300 every FP64 warp instruction occupies its
// SM sub-partition for about 64 cycles (measured: a dependent FMA chain runs at 61
// cycles per FMA, a divide at 437, a square root at 684, whatever the number of active
// lanes), 64 times the cost of its FP32 counterpart.  With an FP32 basis all the vector
// arithmetic and the block and grid levels of the dot products are FP32 (the products
// are FP32 already; FP64 sums of them would halve a reduction error of ~1e-6 relative at
// 64 times the cost in the serial tails); the Hessenberg column, the rotations and the
// least squares stay FP64.  With an FP64 basis everything is FP64.
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

// per-warp sums of one tile of per-thread partial dots into wsum[vector][warp]: a
// butterfly reduce-scatter (each exchange step halves the values a lane holds: 8, 4, 2
// and 1 shuffles, then one more), 16 shuffles for the 16 dots instead of 5 per dot; lane
// l ends with dot 8 b4 + 4 b3 + 2 b2 + b1 (bk: bit k of l), summed over the warp
template <class A, class W>
__device__ __forceinline__ void tile_to_smem(const A (&v)[KRY_TILE], int i0, int nt, W (*wsum)[KRY_WARPS]) {
    static_assert(KRY_TILE == 16, "the butterfly is written for 16 values per lane");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    A x[8], y[4], z[2];
    bool hi = lane & 16;
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (hi ? v[k + 8] : v[k]) + __shfl_xor_sync(full, hi ? v[k] : v[k + 8], 16);
    hi = lane & 8;
#pragma unroll
    for (int k = 0; k < 4; ++k) y[k] = (hi ? x[k + 4] : x[k]) + __shfl_xor_sync(full, hi ? x[k] : x[k + 4], 8);
    hi = lane & 4;
#pragma unroll
    for (int k = 0; k < 2; ++k) z[k] = (hi ? y[k + 2] : y[k]) + __shfl_xor_sync(full, hi ? y[k] : y[k + 2], 4);
    hi = lane & 2;
    A u = (hi ? z[1] : z[0]) + __shfl_xor_sync(full, hi ? z[0] : z[1], 2);
    u += __shfl_xor_sync(full, u, 1);
    const int d = ((lane >> 4) & 1) * 8 + ((lane >> 3) & 1) * 4 + ((lane >> 2) & 1) * 2 + ((lane >> 1) & 1);
    if ((lane & 1) == 0 && d < nt) wsum[i0 + d][warp] = (W)u;
}

constexpr int KRY_RC = 2 * KRY_TILE;  // basis vectors held in registers by the one-pass kernels

// Sum of 8 values as a balanced tree (depth 3).
template <class A>
__device__ __forceinline__ A tree8(const A (&x)[8]) {
    return ((x[0] + x[1]) + (x[2] + x[3])) + ((x[4] + x[5]) + (x[6] + x[7]));
}

// This block's partials of the dots 0..j (sums of the per-warp sums in wsum) into
// partial[i * RED_BLOCKS + blockIdx.x]
template <class A>
__device__ __forceinline__ void block_partials(A* partial, int j, A (*wsum)[KRY_WARPS]) {
    __syncthreads();
    const int nwarp = blockDim.x >> 5;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        A x[8];
#pragma unroll
        for (int w = 0; w < 8; ++w) x[w] = w < nwarp ? wsum[i][w] : A(0);
        partial[(long)i * RED_BLOCKS + blockIdx.x] = tree8(x);
    }
}

// The sums over blocks b < nb of partial[i * RED_BLOCKS + b], i < nd, by the whole block:
// dot i = threadIdx.x / G gets an aligned group of G lanes (G the largest power of two up
// to 32 with G nd <= blockDim.x); each lane loads its strided share eight at a time and
// sums them as trees, the group reduces by shuffles.  Every lane of group i returns the
// sum (0 for i >= nd); the order is fixed, so every block that calls this gets the same
// bits.  *gsz returns G.  Needs nd <= blockDim.x, a multiple of 32.
template <class A>
__device__ __forceinline__ A partials_sum(const A* partial, int nd, int nb, int* gsz) {
    int G = 32;
    while (G > 1 && G * nd > (int)blockDim.x) G >>= 1;
    const int i = threadIdx.x / G, g = threadIdx.x % G;
    A sg = A(0);
    if (i < nd) {
        const A* p = partial + (long)i * RED_BLOCKS;
        for (int b0 = g; b0 < nb; b0 += 16 * G) {  // sixteen loads in flight per lane
            A x[8], y[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int b = b0 + k * G, c = b0 + (k + 8) * G;
                x[k] = b < nb ? __ldcg(p + b) : A(0);
                y[k] = c < nb ? __ldcg(p + c) : A(0);
            }
            sg += tree8(x) + tree8(y);
        }
    }
    for (int o = G >> 1; o > 0; o >>= 1) sg += __shfl_xor_sync(0xffffffffu, sg, o);
    *gsz = G;
    return sg;
}

// Block partials of h[0..j] from wsum, then in the last block to finish the sums over the
// blocks (partials_sum): h[i] = sc[i] * sum (h[jraw] = sum, unscaled), also into hsm when
// given.  One thread per block fences and takes the ticket after the block barrier (the
// fence is cumulative over the writes the barrier ordered before it).  scs: sc staged in
// shared memory (or null: read d.sc).  Returns true in the last block.  Needs j + 1 <=
// blockDim.x, a multiple of 32, and blockDim.x <= RED_THREADS.
template <class A>
__device__ __forceinline__ bool dots_finish(const GmresDev& d, int j, A (*wsum)[KRY_WARPS], double* h,
                                            int jraw = -1, const double* scs = nullptr, double* hsm = nullptr) {
    A* partial = reinterpret_cast<A*>(d.partial);
    block_partials(partial, j, wsum);
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(d.counter, 1u) == gridDim.x - 1;
        if (last) __threadfence();
    }
    __syncthreads();
    if (!last) return false;
    int G;
    const A sg = partials_sum(partial, j + 1, (int)gridDim.x, &G);
    const int i = threadIdx.x / G;
    if (i <= j && threadIdx.x % G == 0) {
        const double hv = (i == jraw ? 1.0 : (scs ? scs[i] : d.sc[i])) * (double)sg;
        h[i] = hv;
        if (hsm) hsm[i] = hv;
    }
    __syncthreads();
    if (threadIdx.x == 0) *d.counter = 0u;
    return true;
}

// Start of a solve: every block takes beta = sqrt(beta^2) (from
// *bsq when given, else d.beta[2]), block 0 initialises the solve state, and unless the
// solve is empty (beta < 1e-12, src/Solver.cpp:1514-1516) V0 = rhs * (1/beta).
template <class T>
__global__ void k_gmres_start(long n, T* V0, const double* rhs, GmresDev d, int m, double tol,
                              cudaGraphConditionalHandle h, const double* bsq) {
    __shared__ double ib;
    const double b2 = bsq ? *bsq : d.beta[2];
    const double b = sqrt(b2);
    const bool empty = b < 1e-12 || (d.skip && *d.skip);
    if (blockIdx.x == 0) {
        for (int i = threadIdx.x; i <= m; i += blockDim.x) {
            d.g[i] = i == 0 ? b : 0.0;
            d.sc[i] = 1.0;
            if (i < m) {
                d.cs[i] = 0.0;
                d.sn[i] = 0.0;
            }
        }
        if (threadIdx.x == 0) {
            d.beta[0] = b;
            d.beta[1] = tol;
            d.beta[2] = b2;
            d.gi[0] = 0;
            d.gi[3] = m;
            d.gi[4] = 0;
            d.gi[5] = 0;
            d.sig[0] = 1.0;
            d.ilam[0] = 1.0;
            if (empty) {
                d.gi[1] = -1;
                d.gi[2] = 1;
                if (d.in_graph) cudaGraphSetConditional(h, 0);
            } else {
                d.gi[1] = 0;
                d.gi[2] = 0;
            }
        }
    }
    if (empty) return;
    if (threadIdx.x == 0) ib = 1.0 / b;
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

// The Givens step for Hessenberg column j (src/Solver.cpp:1550-1588), run by one full
// warp.  Each FP64 warp instruction costs ~64 cycles on GB300 whatever the active lanes,
// so the work is spread over the lanes: the previous rotations applied to the new column
// are the affine recurrence carry_{i+1} = -s_i carry_i + c_i col[i+1] (carry_0 = col[0]),
// evaluated as a parallel prefix over 32 rotations at a time (compositions of affine
// maps, Kogge-Stone), and out[i] = c_i carry_i + s_i col[i+1] by every lane at once.  The
// new rotation takes c = a / sqrt(a^2 + b^2) as a * rsqrt(a^2 + b^2).  col[0..j] holds
// the column's entries above the subdiagonal hv, hsq = hv^2.  Ends the solve (done flag, loop condition) on
// convergence or when j + 1 reaches m.
// c0, s0: this lane's rotation of the first 32 (cs[lane], sn[lane]; 1, 0 past j), gj = g[j]
// and tolb = tol * beta, loaded by the caller ahead of time.
__device__ __forceinline__ void givens_column(const GmresDev& d, int j, int m, double* col, double hv, double hsq,
                                              cudaGraphConditionalHandle hnd, double c0, double s0, double gj,
                                              double tolb) {
    __shared__ double hout[KRY_MAXM + 2];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    double carry = col[0];
    for (int base = 0; base < j; base += 32) {
        const int i = base + lane;
        const bool act = i < j;
        const double ci = base == 0 ? c0 : (act ? d.cs[i] : 1.0), si = base == 0 ? s0 : (act ? d.sn[i] : 0.0);
        const double nx = act ? col[i + 1] : 0.0;
        const double snx = si * nx;
        double fa = act ? -si : 1.0, fb = act ? ci * nx : 0.0;  // f_i(x) = fa x + fb
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double ap = __shfl_up_sync(full, fa, o), bp = __shfl_up_sync(full, fb, o);
            if (lane >= o) {
                fb = fma(fa, bp, fb);
                fa = fa * ap;
            }
        }
        const double cnext = fma(fa, carry, fb);        // carry after rotation i
        double cprev = __shfl_up_sync(full, cnext, 1);  // carry before rotation i
        if (lane == 0) cprev = carry;
        if (act) hout[i] = fma(ci, cprev, snx);
        carry = __shfl_sync(full, cnext, 31);
    }
    if (lane == 0) {
        const double a = carry, b = hv;
        double c, sn;
        if (fabs(b) < 1e-14) {
            c = 1.0;
            sn = 0.0;
            hout[j] = a;
        } else {
            const double q = fma(a, a, hsq), rq = rsqrt(q);
            c = a * rq;
            sn = b * rq;
            hout[j] = q * rq;
        }
        hout[j + 1] = 0.0;
        d.cs[j] = c;
        d.sn[j] = sn;
        d.g[j + 1] = -sn * gj;
        d.g[j] = c * gj;
        const bool conv = fabs(-sn * gj) < tolb;
        if (conv || j + 1 >= m) {
            d.gi[1] = j;
            d.gi[2] = 1;
            if (d.in_graph) cudaGraphSetConditional(hnd, 0);
        }
    }
    __syncwarp();
    double* Hc = d.H + (long)j * (m + 1);
    for (int i = lane; i <= j + 1; i += 32) Hc[i] = hout[i];
}

// First kernel of iteration jn of the exact J v body (DCGS2).  Iteration j applied J to
// the pending vector P_j (slot j of V, scale sig[j]): w = J sig_j P_j.  With jn > 0 every
// block sums the gather kernel's block partials of <V_k, P_j> and <V_k, w> (k < j, V_k the
// stored basis vectors), |P_j|^2, <P_j, w> and |w|^2, then, with v_k = sc_k V_k:
//   s_k = sig_j <v_k, P_j>,  beta^2 = sig_j^2 |P_j|^2 - |s|^2         (Pythagoras)
//   V_j = P_j - sum_k sc_k^2 <V_k, P_j> V_k   (slot j; sc_j = sig_j / beta)
//   g_k = <v_k, w> (k < j),  g_j = (sig_j <P_j, w> - s.g) / beta = <v_j, w>
//   P_jn = w - sum_{k<=j} g_k v_k             (slot jn; sig_jn = 1 / |w|)
// J v_j = (w - J V s) / beta and J V s = V H s over the finished columns (the Arnoldi
// relation), so P_jn = beta (J v_j - V h_j) with the first-pass entries h_j = (g - H s) /
// beta: the pending vector sig_jn P_jn is lam_jn = sig_jn beta times the first-pass vector
// of J v_j.  Scaling by 1/|w| keeps every product's input at norm <= 1 (their dots stay
// in range in FP32 for stiff systems).  Column j - 1 is (h_{j-1} + s / lam_j, beta /
// lam_j); one extra block runs its Givens step (which can end the solve), then forms h_j
// and records sc_j, sig_jn, 1/lam_jn and this iteration's index for the gather kernel.
// Then z = sig_jn P_jn / D and the primitive stage of the dual J v: W.v, W.d of (U, z).
// j = 0 keeps P_0 = V_0 = rhs / |rhs| as it is (beta = 1).  The breakdown guard beta <=
// 1e-12 (src/Solver.cpp:1553-1558) keeps the scales finite; the Givens step then ends the
// solve.  Iteration m + 1 runs only the Givens step of column m - 1.
template <class T, int NV>
__global__ void __launch_bounds__(256, 4) k_gmres_prim_z(int nc, Flow<T> F, const T* __restrict__ U, T* V, long L,
                                                      const T* __restrict__ Dinv, T* __restrict__ z, Field<T> W,
                                                      const T* __restrict__ w, GmresDev d,
                                                      cudaGraphConditionalHandle hnd) {
    typedef typename KryAcc<T>::type A;
    const int4 ga = *reinterpret_cast<const int4*>(d.gi);
    const int4 gb = *reinterpret_cast<const int4*>(d.gi + 4);
    if (ga.z) return;  // the solve has ended
    pdl_trigger();     // the gradient kernel may launch now
    const int jn = gb.y, m = ga.w, j = jn - 1;
    const bool givens_block = blockIdx.x == gridDim.x - 1;
    // the Givens warp's inputs from earlier kernels (column j - 2's first-pass entries, the
    // rotations, g and tol beta) load with the partials below, not after them
    double pre_h1 = 0.0, pre_c = 1.0, pre_s = 0.0, pre_g = 0.0, pre_tolb = 0.0;
    if (givens_block && threadIdx.x < 32 && jn >= 2) {
        const int c = jn - 2, lane = threadIdx.x;
        if (lane <= c) pre_h1 = d.h1[lane];
        if (lane < c) {
            pre_c = d.cs[lane];
            pre_s = d.sn[lane];
        }
        pre_g = d.g[c];
        pre_tolb = d.beta[1] * d.beta[0];
    }
    __shared__ A cu[KRY_MAXM + 1], cp[KRY_MAXM + 1];  // coefficients of V_k in V_j and in P_jn
    __shared__ double dp[KRY_MAXM + 2], dw[KRY_MAXM + 2], sv[KRY_MAXM + 1];
    __shared__ double r_s, hv_s, hsq_s, scj_s, sgn_s, ilmn_s, ilam_s;
    if (jn > 0) {
        // the scales (lane k of warp 0: sc_k), sig_j and 1/lam_j load with the partials
        const double sigj = d.sig[j], ilamj = d.ilam[j];
        const double sclane = (int)threadIdx.x < j && threadIdx.x < 32 ? d.sc[threadIdx.x] : 0.0;
        // dots of slots 0..j with P_j (partial rows 0..j) and with w (rows j+1..2j+1), |w|^2
        // (row 2j+2), in windows of at most blockDim.x rows (partials_sum's limit)
        const int nrow = 2 * (j + 1) + 1;
        for (int base = 0; base < nrow; base += blockDim.x) {
            const int nd = nrow - base < (int)blockDim.x ? nrow - base : (int)blockDim.x;
            int G;
            const A sg = partials_sum(reinterpret_cast<const A*>(d.partial) + (long)base * RED_BLOCKS, nd, d.nb1, &G);
            const int r = base + (int)threadIdx.x / G;
            if ((int)threadIdx.x / G < nd && threadIdx.x % G == 0) {
                if (r <= j) dp[r] = (double)sg;
                else dw[r - j - 1] = (double)sg;
            }
        }
        __syncthreads();
        constexpr bool f32 = sizeof(A) == 4;
        if (threadIdx.x < 32 && f32 && !givens_block) {
            // cell blocks with an FP32 basis: the coefficients only feed FP32 arithmetic, so
            // warp 0 forms them in FP32 (a dependent FP64 operation costs as much as ~16 FP32
            // ones here); the Givens block forms the FP64 values of the Hessenberg column
            if constexpr (f32) {
                const float sigf = (float)sigj;
                float ss = 0.f, sg = 0.f;
                for (int k = threadIdx.x; k < j; k += 32) {
                    const float sck = (float)(k < 32 ? sclane : d.sc[k]);
                    const float pk = (float)dp[k], wk = (float)dw[k];
                    const float sk = sck * sigf * pk, gk = sck * wk;
                    cu[k] = sck * sck * pk;
                    cp[k] = gk * sck;
                    ss += sk * sk;
                    sg += sk * gk;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    ss += __shfl_xor_sync(0xffffffffu, ss, o);
                    sg += __shfl_xor_sync(0xffffffffu, sg, o);
                }
                if (threadIdx.x == 0) {
                    float r = 1.f;
                    if (j > 0) {
                        const float hsq = fmaxf(sigf * sigf * (float)dp[j] - ss, 0.f);
                        const float rq = hsq > 0.f ? rsqrtf(hsq) : 0.f;
                        r = hsq * rq * (float)ilamj > 1e-12f ? rq : 1.f;
                    }
                    const float gj = (sigf * (float)dw[j] - sg) * r;
                    cp[j] = gj * (sigf * r);
                    const float wsq = (float)dw[j + 1];
                    sgn_s = wsq > 0.f ? (double)rsqrtf(wsq) : 1.0;
                }
            }
        } else if (threadIdx.x < 32) {
            // warp 0: s_k, g_k and the coefficients, lane k; |s|^2 and s.g in the basis
            // precision (corrections of ~1e-7 relative with FP32)
            A ss = A(0), sg = A(0);
            for (int k = threadIdx.x; k < j; k += 32) {
                const double sck = k < 32 ? sclane : d.sc[k];
                const double sk = sck * sigj * dp[k], gk = sck * dw[k];
                sv[k] = sk;
                dw[k] = gk;
                cu[k] = (A)(sck * sck * dp[k]);
                cp[k] = (A)(gk * sck);
                ss += (A)sk * (A)sk;
                sg += (A)sk * (A)gk;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ss += __shfl_xor_sync(0xffffffffu, ss, o);
                sg += __shfl_xor_sync(0xffffffffu, sg, o);
            }
            if (threadIdx.x == 0) {
                double hsq = 1.0, hv = 1.0, r = 1.0;
                if (j > 0) {
                    hsq = fmax(sigj * sigj * dp[j] - (double)ss, 0.0);
                    const double rq = hsq > 0.0 ? rsqrt(hsq) : 0.0;
                    hv = hsq * rq;
                    r = hv * ilamj > 1e-12 ? rq : 1.0;  // the guard on the column's entry hv / lam_j
                }
                hsq_s = hsq;
                hv_s = hv;
                r_s = r;
                scj_s = sigj * r;
                const double gj = (sigj * dw[j] - (double)sg) * r;
                dw[j] = gj;
                cp[j] = (A)(gj * (sigj * r));
                // sig_jn = 1/|w|, 1/lam_jn = r/sig_jn = r |w| (multiplies: an FP64 divide costs
                // about seven dependent FMAs)
                const double wsq = dw[j + 1];
                // (with an FP32 basis the cell blocks' FP32 value, so both use the same scale)
                const double sgn = wsq > 0.0 ? (f32 ? (double)rsqrtf((float)wsq) : rsqrt(wsq)) : 1.0;
                sgn_s = sgn;
                ilmn_s = r * (wsq > 0.0 ? wsq * sgn : 1.0);
                ilam_s = ilamj;
            }
        }
        __syncthreads();
    }
    if (givens_block) {
        if (jn > 0) {
            __shared__ double col[KRY_MAXM + 2];
            const int c = j - 1;
            if (j > 0 && threadIdx.x < 32) {
                // column j - 1 is final: its first-pass entries plus s, subdiagonal beta
                // (P_j is lam_j times the first-pass vector of column j - 1)
                double* Hc = d.Hu + (long)c * (m + 1);
                const double il = ilam_s;
                for (int i = threadIdx.x; i <= c; i += 32) {
                    col[i] = (i < 32 ? pre_h1 : d.h1[i]) + sv[i] * il;
                    Hc[i] = col[i];
                }
                if (threadIdx.x == 0) {
                    col[c + 1] = hv_s * il;
                    Hc[c + 1] = col[c + 1];
                }
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                if (j > 0) {
                    const double hvc = col[c + 1];
                    givens_column(d, c, m, col, hvc, hvc * hvc, hnd, pre_c, pre_s, pre_g, pre_tolb);
                }
                if (threadIdx.x == 0) {
                    d.sc[j] = scj_s;
                    d.sig[jn] = sgn_s;
                    d.ilam[jn] = ilmn_s;
                    d.hsq[1] = hsq_s;
                }
            } else if (j < m) {
                // meanwhile warps 1.. form column j's first-pass entries h_j = (g - H s) / beta,
                // one row per thread; H s is a correction of the size of s, so it is summed in
                // the basis precision (columns before c from memory, column c from col)
                for (int i = (int)threadIdx.x - 32; i <= j; i += (int)blockDim.x - 32) {
                    A hs = A(0);
#pragma unroll 8
                    for (int k = i > 0 ? i - 1 : 0; k < c; ++k) hs += (A)d.Hu[(long)k * (m + 1) + i] * (A)sv[k];
                    if (j > 0 && i <= j) hs += (A)col[i] * (A)sv[c];
                    d.h1[i] = (dw[i] - (double)hs) * r_s;
                }
            }
        }
        if (threadIdx.x == 0) d.gi[4] = jn;
        return;
    }
    if (jn > m) return;  // the last column's Givens step only
    T* Vj = V + (long)(jn > 0 ? j : 0) * L;
    T* Vn = V + (long)jn * L;
    const T sn = jn > 0 ? (T)sgn_s : T(1);
    const A cpj = jn > 0 ? cp[j] : A(0);
    const long cstride = (long)(gridDim.x - 1) * blockDim.x;  // the cell blocks, grid-stride
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += cstride) {
    const T a = Dinv[i];
    T pn[NV];
    if (jn > 0) {
        A au[NV], ap[NV];
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            au[c] = (A)Vj[c * nc + i];
            ap[c] = (A)w[c * nc + i];
        }
#pragma unroll 2
        for (int k = 0; k < j; ++k) {
            const T* Vk = V + (long)k * L;
            const A uk = cu[k], pk = cp[k];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                const A vk = (A)Vk[c * nc + i];
                au[c] -= uk * vk;
                ap[c] -= pk * vk;
            }
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            const T uj = (T)au[c];
            if (j > 0) Vj[c * nc + i] = uj;
            pn[c] = (T)(ap[c] - cpj * (A)uj);
            Vn[c * nc + i] = pn[c];
        }
    } else {
#pragma unroll
        for (int c = 0; c < NV; ++c) pn[c] = Vn[c * nc + i];
    }
    Dual<T> u[6];
#pragma unroll
    for (int c = 0; c < NV; ++c) {
        T zc = pn[c] * sn * dinv_of<T, NV>(Dinv, nc, i, c, a);
        z[c * nc + i] = zc;
        u[c] = Dual<T>(U[c * nc + i], zc);
    }
    if (NV == 4) u[4] = u[5] = Dual<T>(T(0), T(0));
    prim_cell<Dual<T>, NV>(F, u[0], u[1], u[2], u[3], u[4], u[5], W, i);
    }
}

// h[i] = sc[i] <w, V_i>, i = 0..j (the first pass of the FD J v path)
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_multidot(long L, const T* __restrict__ w,
                                                                const T* __restrict__ V, GmresDev d, double* h) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ A wsum[KRY_MAXM + 1][KRY_WARPS];
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
// order, minus the SST source derivatives, plus z vol / dt) into w, fused with the one
// reduction of the iteration: the dots of slots 0..j of V (the basis vectors V_0..V_{j-1}
// and the pending vector P_j) with P_j and with w, and |w|^2, as block partials (rows
// 0..j, j+1..2j+1 and 2j+2 of partial) that every block of the next k_gmres_prim_z sums.
// Grid-stride over cells (gather_grid blocks).  With an FP32 basis the kernel fits 128
// registers without spills, so two blocks share an SM (a streaming pass over a
// million-cell basis needs the loads of more than one block in flight per SM).
// SPLIT (large meshes): w was gathered by k_gmres_gather_w (one thread per cell, the same
// arithmetic), and this kernel only streams w, P_j and the basis for the dots, with no
// dependent loads in its loop; the same grid and the same per-thread cells, so the block
// partials are the fused kernel's bit for bit.
template <class T, int NV, bool SPLIT = false>
__global__ void __launch_bounds__(RED_THREADS, sizeof(T) == 4 ? 2 : 1)
    k_gmres_gather_dot(MeshView<T> m, const T* __restrict__ FA,
                                                                  long fa_stride, T* __restrict__ w,
                                                                  const T* __restrict__ z, const T* __restrict__ dt,
                                                                  const T* __restrict__ src, const T* __restrict__ V,
                                                                  long L, GmresDev d) {
    typedef typename KryAcc<T>::type A;
    const int done = d.gi[2];
    const int j = d.gi[4];  // this iteration (set by k_gmres_prim_z)
    if (done) return;       // the solve has ended
    const long nc = m.nc;
    __shared__ A wsw[KRY_MAXM + 2][KRY_WARPS], wsp[KRY_MAXM + 1][KRY_WARPS];
    const T* Pj = V + (long)j * L;
    // w = the gathered J v of cell i (reference face order).  Everything but the face
    // fluxes comes from two or more kernels back (pdl.cuh), so a thread loads it for its
    // first cell before the wait for the fluxes.
    struct Pre {
        int ek[4];
        T tc, zc[NV], pj[NV], s4, s5;
    };
    auto pre = [&](long i, Pre& p) {
        if constexpr (SPLIT) {
#pragma unroll
            for (int c = 0; c < NV; ++c) p.pj[c] = Pj[c * nc + i];
            return;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) p.ek[k] = m.cf[(long)k * nc + i];
        p.tc = m.vol[i] / (dt[i] + T(1e-30));
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            p.zc[c] = z[c * nc + i];
            p.pj[c] = Pj[c * nc + i];
        }
        if constexpr (NV == 6) {
            p.s4 = src[i];
            p.s5 = src[nc + i];
        }
    };
    A nw = A(0);  // |w|^2
    auto gather = [&](long i, const Pre& p, T (&acc)[NV]) {
        if constexpr (SPLIT) {
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                acc[c] = w[c * nc + i];
                nw += (A)acc[c] * (A)acc[c];
            }
            return;
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) acc[c] = T(0);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int e = p.ek[k];
            if (e < 0) continue;  // pads only at the end of a cell's list
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
            acc[4] = acc[4] - p.s4;
            acc[5] = acc[5] - p.s5;
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            acc[c] = acc[c] + p.zc[c] * p.tc;
            w[c * nc + i] = acc[c];
            nw += (A)acc[c] * (A)acc[c];
        }
    };
    const long ifirst = (long)blockIdx.x * blockDim.x + threadIdx.x;
    Pre p0;
    if (ifirst < nc) pre(ifirst, p0);
    pdl_wait();  // the face fluxes are the predecessor's
    pdl_trigger();
    // one pass over the cells when the dots fit the register tiles (two tiles per product
    // with an FP32 basis, one with FP64), compiled for 8, 16 and RC basis vectors: the
    // early iterations' passes hold fewer accumulators, which leaves registers for loads in
    // flight (the same sums, in the same order, whichever form runs)
    constexpr int RC = sizeof(T) == 4 ? KRY_RC : KRY_TILE;
    auto one_pass = [&](auto ntv) {
        constexpr int NTV = decltype(ntv)::value;  // j < NTV
        A vw0[KRY_TILE], vw1[KRY_TILE], vp0[KRY_TILE], vp1[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) vw0[t] = vw1[t] = vp0[t] = vp1[t] = A(0);
        for (long i = ifirst; i < nc; i += (long)gridDim.x * blockDim.x) {
            T acc[NV];
            Pre p;
            if (i == ifirst) {
                p = p0;
            } else {
                pre(i, p);
            }
            gather(i, p, acc);
#pragma unroll
            for (int t = 0; t < NTV; ++t)
                if (t <= j) {
                    const T* Vi = V + (long)t * L;
                    A sw = A(0), sp = A(0);
#pragma unroll
                    for (int c = 0; c < NV; ++c) {
                        const A vt = (A)Vi[c * nc + i];
                        sw += (A)acc[c] * vt;
                        sp += (A)p.pj[c] * vt;
                    }
                    if (t < KRY_TILE) {
                        vw0[t] += sw;
                        vp0[t] += sp;
                    } else {
                        vw1[t - KRY_TILE] += sw;
                        vp1[t - KRY_TILE] += sp;
                    }
                }
        }
        const int n0 = j + 1 < KRY_TILE ? j + 1 : KRY_TILE;
        tile_to_smem(vw0, 0, n0, wsw);
        tile_to_smem(vp0, 0, n0, wsp);
        if (NTV > KRY_TILE && j >= KRY_TILE) {
            tile_to_smem(vw1, KRY_TILE, j + 1 - KRY_TILE, wsw);
            tile_to_smem(vp1, KRY_TILE, j + 1 - KRY_TILE, wsp);
        }
    };
    if (j < 8) {
        one_pass(std::integral_constant<int, 8>());
    } else if (j < KRY_TILE) {
        one_pass(std::integral_constant<int, KRY_TILE>());
    } else if (RC > KRY_TILE && j < RC) {
        one_pass(std::integral_constant<int, RC>());
    } else {
        for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
            const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
            A vw[KRY_TILE], vp[KRY_TILE];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t) vw[t] = vp[t] = A(0);
            for (long i = ifirst; i < nc; i += (long)gridDim.x * blockDim.x) {
                T acc[NV], pj[NV];
                if (i0 == 0) {
                    Pre p;
                    if (i == ifirst) {
                        p = p0;
                    } else {
                        pre(i, p);
                    }
                    gather(i, p, acc);
#pragma unroll
                    for (int c = 0; c < NV; ++c) pj[c] = p.pj[c];
                } else {
#pragma unroll
                    for (int c = 0; c < NV; ++c) {
                        acc[c] = w[c * nc + i];
                        pj[c] = Pj[c * nc + i];
                    }
                }
#pragma unroll
                for (int t = 0; t < KRY_TILE; ++t)
                    if (t < nt) {
                        const T* Vi = V + (long)(i0 + t) * L;
                        A sw = A(0), sp = A(0);
#pragma unroll
                        for (int c = 0; c < NV; ++c) {
                            const A vt = (A)Vi[c * nc + i];
                            sw += (A)acc[c] * vt;
                            sp += (A)pj[c] * vt;
                        }
                        vw[t] += sw;
                        vp[t] += sp;
                    }
            }
            tile_to_smem(vw, i0, nt, wsw);
            tile_to_smem(vp, i0, nt, wsp);
        }
    }
    // block partials only: every block of the next kernel sums them itself (partials_sum),
    // which costs less than a last-block reduction here and its fence and ticket
    nw = warp_sum_t(nw);
    if ((threadIdx.x & 31) == 0) wsw[j + 1][threadIdx.x >> 5] = nw;
    block_partials(reinterpret_cast<A*>(d.partial), j, wsp);
    block_partials(reinterpret_cast<A*>(d.partial) + (long)(j + 1) * RED_BLOCKS, j + 1, wsw);
    if (blockIdx.x == 0 && threadIdx.x == 0) d.gi[5] = j + 1;  // products reduced
}

// The gather of k_gmres_gather_dot alone (large meshes: its SPLIT form then takes the
// dots), one thread per cell: w = the faces' F*A derivatives in reference face order, minus
// the SST source derivatives, plus z vol / dt, with the fused kernel's arithmetic.
template <class T, int NV>
__global__ void __launch_bounds__(256) k_gmres_gather_w(MeshView<T> m, const T* __restrict__ FA, long fa_stride,
                                                        T* __restrict__ w, const T* __restrict__ z,
                                                        const T* __restrict__ dt, const T* __restrict__ src,
                                                        GmresDev d) {
    const long nc = m.nc;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (d.gi[2] || i >= nc) return;  // the solve has ended
    const T tc = m.vol[i] / (dt[i] + T(1e-30));
    T zc[NV];
#pragma unroll
    for (int c = 0; c < NV; ++c) zc[c] = z[c * nc + i];
    pdl_wait();  // the face fluxes are the predecessor's
    pdl_trigger();
    T acc[NV];
    gather_cell<T, NV>(m, FA, fa_stride, src, nc, i, acc);
#pragma unroll
    for (int c = 0; c < NV; ++c) w[c * nc + i] = acc[c] + zc[c] * tc;
}

// w -= sum_{i<=j} h1[i] sc[i] V_i, fused with the second CGS pass h2 = V^T w (FD J v
// body); the last block to finish sums the h2 partials.
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_gmres_update_dot(long L, T* __restrict__ w, const T* __restrict__ V,
                                                                  GmresDev d) {
    typedef typename KryAcc<T>::type A;
    const int j = d.gi[0];
    __shared__ A hs[KRY_MAXM + 1];
    __shared__ A wsum[KRY_MAXM + 1][KRY_WARPS];
    __shared__ double scs[KRY_MAXM + 1];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        scs[i] = d.sc[i];
        hs[i] = (A)(d.h1[i] * scs[i]);
    }
    __syncthreads();
    // one pass (j < KRY_RC): each element's basis values stay in registers between the
    // update and the dots, and (FP32) a thread's three grid-stride elements are loaded
    // together, so their loads are in flight at once
    constexpr int EPT = sizeof(T) == 4 ? 3 : 1;
    const long stride = (long)gridDim.x * blockDim.x;
    const long qfirst = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j < KRY_RC) {
        T vv[EPT][KRY_RC];
        A a[EPT];
        A v0[KRY_TILE], v1[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) v0[t] = v1[t] = A(0);
        for (long q0 = qfirst; q0 < L; q0 += EPT * stride) {
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long q = q0 + e * stride;
                const bool ok = q < L;
                a[e] = ok ? (A)w[q] : A(0);
#pragma unroll
                for (int t = 0; t < KRY_RC; ++t) vv[e][t] = ok && t <= j ? V[(long)t * L + q] : T(0);
            }
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                const long q = q0 + e * stride;
                if (q >= L) continue;
                A ae = a[e];
#pragma unroll
                for (int t = 0; t < KRY_RC; ++t)
                    if (t <= j) ae -= hs[t] * (A)vv[e][t];
                const T tq = (T)ae;
                w[q] = tq;
#pragma unroll
                for (int t = 0; t < KRY_TILE; ++t) {
                    v0[t] += (A)tq * (A)vv[e][t];
                    v1[t] += (A)tq * (A)vv[e][KRY_TILE + t];
                }
            }
        }
        tile_to_smem(v0, 0, j + 1 < KRY_TILE ? j + 1 : KRY_TILE, wsum);
        if (j >= KRY_TILE) tile_to_smem(v1, KRY_TILE, j + 1 - KRY_TILE, wsum);
    } else {
        for (long q = qfirst; q < L; q += stride) {
            A a = (A)w[q];
            for (int i = 0; i <= j; ++i) a -= hs[i] * (A)V[(long)i * L + q];
            w[q] = (T)a;
        }
        for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
            const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
            A v[KRY_TILE];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
            for (long q = qfirst; q < L; q += stride) {
                A wq = (A)w[q];
#pragma unroll
                for (int t = 0; t < KRY_TILE; ++t)
                    if (t < nt) v[t] += wq * (A)V[(long)(i0 + t) * L + q];
            }
            tile_to_smem(v, i0, nt, wsum);
        }
    }
    dots_finish(d, j, wsum, d.h2, -1, scs);
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

// back substitution H y = g over the k+1 leading columns (src/Solver.cpp:1592-1599), by
// one warp: the triangle is staged in shared memory, the reciprocals of the diagonal are
// taken by all lanes at once, then column by column (l = k .. 0) y_l = g_l / H_ll and every
// lane i < l takes g_i -= H_il y_l, so the serial chain is one multiply and one FMA per
// column (an FP64 warp instruction costs ~64 cycles on GB300, a divide about seven of them).
constexpr int KRY_BS = 64;  // columns of the triangle staged in shared memory (33 KB)

static __global__ void k_gmres_backsub(GmresDev d) {
    __shared__ double R[KRY_BS][KRY_BS + 1], gs[KRY_MAXM + 1], rd[KRY_MAXM + 1], ys[KRY_MAXM + 1];
    if (blockIdx.x != 0 || threadIdx.x >= 32) return;
    const int k = d.gi[1], m = d.gi[3], lane = threadIdx.x;
    if (k < 0) return;
    const bool staged = k < KRY_BS;
    // H_il = column l, row i (i <= l)
    auto Hil = [&](int i, int l) { return staged ? R[l][i] : d.H[(long)l * (m + 1) + i]; };
    if (staged)
        for (int l = 0; l <= k; ++l)
            for (int i = lane; i <= l; i += 32) R[l][i] = d.H[(long)l * (m + 1) + i];
    for (int i = lane; i <= k; i += 32) gs[i] = d.g[i];
    __syncwarp();
    for (int i = lane; i <= k; i += 32) rd[i] = 1.0 / Hil(i, i);
    __syncwarp();
    for (int l = k; l >= 0; --l) {
        const double yl = gs[l] * rd[l];
        if (lane == 0) ys[l] = yl;
        for (int i = lane; i < l; i += 32) gs[i] = fma(-Hil(i, l), yl, gs[i]);
        __syncwarp();
    }
    for (int i = lane; i <= k; i += 32) d.y[i] = ys[i];
}

// x = (sum_{i<=k} V_i sc_i y_i) / D (src/Solver.cpp:1610-1615, accumulated before the
// scaling); zero when the solve was empty
// With an FP32 basis the sum is FP32 (the update only has to solve the Newton system to
// the GMRES tolerance) and 1/D the FP32 reciprocal the solve used (Dinv32).
template <class T, int NV>
__global__ void k_gmres_solution_dev(long nc, const T* __restrict__ V, long L, GmresDev d,
                                     const double* __restrict__ D, const T* __restrict__ Dinv32,
                                     double* __restrict__ x) {
    typedef typename KryAcc<T>::type A;
    __shared__ A ys[KRY_MAXM];
    const int k = d.gi[1];
    for (int j = threadIdx.x; j <= k; j += blockDim.x) ys[j] = (A)(d.y[j] * d.sc[j]);
    __syncthreads();
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += (long)gridDim.x * blockDim.x) {
        double id[NV];
        if (sizeof(T) == 4) {
#pragma unroll
            for (int c = 0; c < NV; ++c) id[c] = (double)dinv_of<T, NV>(Dinv32, nc, i, c, Dinv32[i]);
        } else {
            d_inv<NV>(D, nc, i, id);
        }
#pragma unroll
        for (int c = 0; c < NV; ++c) {
            long q = c * nc + i;
            A acc = A(0);
            for (int j = 0; j <= k; ++j) acc += (A)V[j * L + q] * ys[j];
            x[q] = (double)acc * id[c];
        }
    }
}

}  // namespace cfdg
