// One Arnoldi iteration of the exact-J v GMRES as a single persistent kernel: the phases
// of the fused body (z with the dual primitives, dual gradients [+ SST terms], dual face
// fluxes, the gather with the first CGS pass, the first update with the second pass, the
// final update with the norm and the Givens step) separated by grid barriers instead of
// kernel boundaries.  At small meshes every phase is latency-bound and the kernel
// boundaries (launch, ramp, the last block's serial tail) were most of the iteration.
//
// Each phase works grid-stride on its items with exactly the arithmetic of the separate
// kernels (the same device functions).  Reductions: every block writes its partials, and
// after the barrier EVERY block sums all partials itself in the same fixed order (so all
// blocks hold bit-identical h), one warp per basis vector; only block 0 writes the results
// and runs the Givens step.
//
// The grid barrier waits with an iteration limit: a barrier that is not completed in time
// (the blocks were not all resident) sets bar[2] and returns, the kernel then finishes
// with wrong numbers but finishes; the host reports the flag as an error.  The kernel is
// launched with at most the blocks that fit on the GPU at once (occupancy query).
//
// Measured on the 28,800-cell laminar plate it did not beat the multi-kernel body of the
// time for the FP32 basis (63-72 vs 54-64 us per iteration; the four-kernel delayed-CGS2
// body since runs an iteration in about 30 us) and matched it in FP64 (186-200 vs 186-211
// us), so the multi-kernel body is the default; the switch is cfdg_config.persistent.
// This kernel keeps the two-reduction CGS2 (its own phases; the same GMRES state).
#pragma once
#include "krylov.cuh"

namespace cfdg {

struct GridBar {
    unsigned* count;  // arrivals of the current barrier
    unsigned* gen;    // barrier generation
    int* err;         // set when a wait ran out
    unsigned limit;   // polls before a wait gives up (2^24 by default)
};

// all blocks of the grid wait here; bounded wait (at most b.limit polls)
__device__ __forceinline__ void grid_barrier(const GridBar& b) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = b.gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(b.count, 1u);
        if (arrived == gridDim.x - 1) {
            *b.count = 0u;
            __threadfence();
            atomicAdd(b.gen, 1u);
        } else {
            unsigned polls = 0;
            while (*vgen == g) {
                if (++polls > b.limit) {  // each poll is an L2 round trip: 2^24 are seconds
                    atomicExch(b.err, 1);
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
}

template <class T>
struct ArnoldiArgs {
    MeshView<T> m;
    Flow<T> F;
    const T* U;        // linearisation point (value planes)
    T* z;              // V_j / D
    Field<T> W, G;     // primitives and gradients (value and derivative planes)
    Field<T> FA;       // face flux derivatives
    Field<T> Tsst;     // SST cell terms (value and derivative planes), nv = 6
    const T* dwall;
    const T* phi;      // frozen limiter
    const T* dt;
    const T* Dinv;
    T* w;
    T* V;
    long L;
    GmresDev d;
    double* part;      // 2 (KRY_MAXM + 1) RED_BLOCKS + RED_BLOCKS partials
    GridBar bar;
};

// every block: h[i] = sc[i] * sum over blocks of part[i][b], i = 0..j, into hs (shared)
template <class A>
__device__ __forceinline__ void reduce_all_blocks(const GmresDev& d, const double* part, int j, A* hs, double* hd) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int i = warp; i <= j; i += nwarp) {
        double s = 0.0;
#pragma unroll 4
        for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(part + (long)i * RED_BLOCKS + b);
        s = warp_sum(s);
        if (lane == 0) {
            double h = d.sc[i] * s;
            hd[i] = h;
            hs[i] = (A)(h * d.sc[i]);  // the update's coefficient: h_i times V_i's scale
        }
    }
    __syncthreads();
}

// the block's per-vector partials from wsum into part[i][blockIdx], then the barrier
template <int NW>
__device__ __forceinline__ void block_partials(const double (*wsum)[NW], int j, double* part) {
    __syncthreads();
    const int nwarp = blockDim.x >> 5;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double sb = 0.0;
        for (int w = 0; w < nwarp; ++w) sb += wsum[i][w];
        part[(long)i * RED_BLOCKS + blockIdx.x] = sb;
    }
}

template <class T, int NV>
__global__ void __launch_bounds__(RED_THREADS, sizeof(T) == 4 ? 2 : 1) k_arnoldi(ArnoldiArgs<T> a,
                                                                          cudaGraphConditionalHandle hnd) {
    typedef typename KryAcc<T>::type A;
    typedef Dual<T> S;
    const GmresDev& d = a.d;
    const MeshView<T>& m = a.m;
    const long nc = m.nc, nf = m.nf, L = a.L;
    const int j = d.gi[0];
    // items are dealt to the grid warp by warp, round-robin over the blocks (warp w of
    // block b is global warp w * gridDim + b), so that a phase with fewer items than
    // threads still spreads over every SM while each warp reads consecutive items
    const long gstride = (long)gridDim.x * blockDim.x;
    const long gtid = ((long)(threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32 + (threadIdx.x & 31);
    __shared__ double wsum[KRY_MAXM + 1][KRY_WARPS];
    __shared__ A hs[KRY_MAXM + 1];
    __shared__ double hd[KRY_MAXM + 1];
    double* part1 = a.part;
    double* part2 = a.part + (long)(KRY_MAXM + 1) * RED_BLOCKS;
    double* part3 = a.part + 2L * (KRY_MAXM + 1) * RED_BLOCKS;
    const Field<T> Ud{const_cast<T*>(a.U), a.z, nc};

    // 1. z = V_j sc_j / D and the dual primitives
    {
        const T* Vj = a.V + (long)j * L;
        const T sj = (T)d.sc[j];
        for (long i = gtid; i < nc; i += gstride) {
            const T d0 = a.Dinv[i];
            S u[6];
#pragma unroll
            for (int c = 0; c < NV; ++c) {
                T zc = Vj[c * nc + i] * sj * dinv_of<T, NV>(a.Dinv, nc, i, c, d0);
                a.z[c * nc + i] = zc;
                u[c] = S(a.U[c * nc + i], zc);
            }
            if (NV == 4) u[4] = u[5] = S(T(0), T(0));
            prim_cell<S, NV>(a.F, u[0], u[1], u[2], u[3], u[4], u[5], a.W, i);
        }
    }
    grid_barrier(a.bar);
    // 2. dual gradients (limiter frozen) [+ SST cell terms]
    for (long i = gtid; i < nc; i += gstride) grad_item<S, NV>(m, a.F, Ud, a.W, a.G, const_cast<T*>(a.phi), 0, i);
    grid_barrier(a.bar);
    if constexpr (NV == 6) {
        for (long i = gtid; i < nc; i += gstride) sst_item<S, NV>(m, a.F, a.W, a.G, a.dwall, a.Tsst, i);
        grid_barrier(a.bar);
    }
    // 3. dual face fluxes
    for (long f = gtid; f < nf; f += gstride) flux_item<S, NV>(m, a.F, Ud, a.W, a.G, a.phi, a.FA, a.Tsst, f);
    grid_barrier(a.bar);
    // 4. gather (+ time term, - SST sources) into w, first CGS pass partials
    {
        const T* FAd = a.FA.d;
        const T* src = NV == 6 ? a.Tsst.d + 2 * nc : nullptr;
        for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
            const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
            A v[KRY_TILE];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
            for (long i = gtid; i < nc; i += gstride) {
                T acc[NV];
                if (i0 == 0) {
#pragma unroll
                    for (int c = 0; c < NV; ++c) acc[c] = T(0);
                    int ek[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) ek[k] = m.cf[(long)k * nc + i];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        int e = ek[k];
                        if (e < 0) continue;
                        long f = e >> 1;
                        if (e & 1) {
#pragma unroll
                            for (int c = 0; c < NV; ++c) acc[c] = acc[c] - FAd[c * nf + f];
                        } else {
#pragma unroll
                            for (int c = 0; c < NV; ++c) acc[c] = acc[c] + FAd[c * nf + f];
                        }
                    }
                    if constexpr (NV == 6) {
                        acc[4] = acc[4] - src[i];
                        acc[5] = acc[5] - src[nc + i];
                    }
                    T tc = m.vol[i] / (a.dt[i] + T(1e-30));
#pragma unroll
                    for (int c = 0; c < NV; ++c) {
                        acc[c] = acc[c] + a.z[c * nc + i] * tc;
                        a.w[c * nc + i] = acc[c];
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < NV; ++c) acc[c] = a.w[c * nc + i];
                }
#pragma unroll
                for (int t = 0; t < KRY_TILE; ++t)
                    if (t < nt) {
                        const T* Vi = a.V + (long)(i0 + t) * L;
                        A sacc = A(0);
#pragma unroll
                        for (int c = 0; c < NV; ++c) sacc += (A)acc[c] * (A)Vi[c * nc + i];
                        v[t] += sacc;
                    }
            }
            tile_to_smem(v, i0, nt, wsum);
        }
        block_partials<KRY_WARPS>(wsum, j, part1);
    }
    grid_barrier(a.bar);
    // 5. h1 (every block), w -= V h1, second pass partials
    reduce_all_blocks<A>(d, part1, j, hs, hd);
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i <= j; i += blockDim.x) d.h1[i] = hd[i];
    for (long q = gtid; q < L; q += gstride) {
        A x = (A)a.w[q];
        for (int i = 0; i <= j; ++i) x -= hs[i] * (A)a.V[(long)i * L + q];
        a.w[q] = (T)x;
    }
    for (int i0 = 0; i0 <= j; i0 += KRY_TILE) {
        const int nt = (j + 1 - i0) < KRY_TILE ? (j + 1 - i0) : KRY_TILE;
        A v[KRY_TILE];
#pragma unroll
        for (int t = 0; t < KRY_TILE; ++t) v[t] = A(0);
        for (long q = gtid; q < L; q += gstride) {
            A wq = (A)a.w[q];
#pragma unroll
            for (int t = 0; t < KRY_TILE; ++t)
                if (t < nt) v[t] += wq * (A)a.V[(long)(i0 + t) * L + q];
        }
        tile_to_smem(v, i0, nt, wsum);
    }
    block_partials<KRY_WARPS>(wsum, j, part2);
    grid_barrier(a.bar);
    // 6. h2 (every block), V_{j+1} = w - V h2 (unnormalised), norm partials
    reduce_all_blocks<A>(d, part2, j, hs, hd);
    if (blockIdx.x == 0)
        for (int i = threadIdx.x; i <= j; i += blockDim.x) d.h2[i] = hd[i];
    {
        T* Vn = a.V + (long)(j + 1) * L;
        A nrm = A(0);
        for (long q = gtid; q < L; q += gstride) {
            A x = (A)a.w[q];
            for (int i = 0; i <= j; ++i) x -= hs[i] * (A)a.V[(long)i * L + q];
            T t = (T)x;
            Vn[q] = t;
            nrm += (A)t * (A)t;
        }
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        nrm = warp_sum_t(nrm);
        __syncthreads();
        if (lane == 0) wsum[0][warp] = (double)nrm;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sb = 0.0;
            for (int w_ = 0; w_ < (int)(blockDim.x >> 5); ++w_) sb += wsum[0][w_];
            part3[blockIdx.x] = sb;
        }
    }
    grid_barrier(a.bar);
    // 7. block 0: the norm, the scale of V_{j+1}, the Givens step
    if (blockIdx.x != 0) return;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double sg = 0.0;
        for (int b = lane; b < (int)gridDim.x; b += 32) sg += __ldcg(part3 + b);
        sg = __shfl_sync(0xffffffffu, warp_sum(sg), 0);
        if (lane == 0) {
            d.hsq[1] = sg;
            double hv = sqrt(sg);
            d.sc[j + 1] = hv > 1e-12 ? 1.0 / hv : 1.0;
        }
        givens_step(d, hnd, sg);
    }
}

}  // namespace cfdg
