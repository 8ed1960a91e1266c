// Mesh ingest on the GPU: Mesh::buildConnectivity and Mesh::computeGeometry
// (AmberMond/mycode src/Mesh.cpp:102-201) and the renumbered device layout of
// build_mesh (mesh.cpp), computed by kernels instead of the host's hash map and sorts.
// The result is the same HostMesh bit for bit: the same face creation order (faces in
// order of their first half-edge, cell by cell), owner (the first cell), node order,
// geometry expressions (this translation unit is compiled without FMA contraction; the
// square roots and quotients are IEEE-rounded on both sides) and renumbering.
//
// Steps, over the half-edges q = 4 i + j (cell i, local edge j):
//   1. the edge key (lo, hi) of every half-edge; half-edges bucketed by lo (count, scan,
//      scatter) and each bucket sorted by (hi, q): equal keys are adjacent, in q order
//   2. the first half-edge of each edge opens a face; faces are numbered by a scan over
//      the first-occurrence flags in q order, which is the reference's creation order
//   3. boundary tags by looking the boundary edges up in the buckets (the last boundary
//      edge of a key wins, as the host map's assignment)
//   4. cell and face geometry, the zero-area check
//   5. Hilbert renumbering: keys from the centroids, a stable radix sort (ties in cell
//      order, as std::sort of (key, cell) pairs); reverse Cuthill-McKee stays on the host
//   6. face slots: interior faces bucketed by their lower new cell, boundary faces by
//      their owner after them, each bucket sorted by (higher cell or face, face)
//   7. the device layout: per-slot face data, per-cell face lists in reference face
//      order, the wall-face slots
// Everything is read back into the HostMesh the solver uploads from.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "mesh.hpp"

namespace cfdg {

void order_rcm_host(const HostMesh& m, std::vector<int>& perm);  // mesh.cpp

namespace {

constexpr int MT = 256;
inline unsigned mgrid(long n) { return (unsigned)((n + MT - 1) / MT); }

template <class T>
struct DBuf {
    T* p = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc((void**)&p, sizeof(T) * (n ? n : 1)); }
};

struct Err {
    std::string msg;
    bool set(cudaError_t e, const char* what) {
        if (e == cudaSuccess) return false;
        msg = std::string("GPU mesh build: ") + what + ": " + cudaGetErrorString(e);
        return true;
    }
};
#define MG_TRY(call) \
    if (E.set((call), #call)) return E.msg

// ---------------------------------------------------------------- exclusive scan (int)
constexpr int SCAN_B = 4 * MT;  // elements per block

__global__ void __launch_bounds__(MT) k_scan_blocks(const int* in, int* out, int* sums, long n) {
    __shared__ int wt[MT / 32];
    const long base = (long)blockIdx.x * SCAN_B + 4L * threadIdx.x;
    int v[4], loc[4], s = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        loc[k] = s;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wt[w] = x;
    __syncthreads();
    if (w == 0) {
        int z = lane < MT / 32 ? wt[lane] : 0;
#pragma unroll
        for (int o = 1; o < MT / 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, z, o);
            if (lane >= o) z += y;
        }
        if (lane < MT / 32) wt[lane] = z;
    }
    __syncthreads();
    const int excl = x - s + (w > 0 ? wt[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (base + k < n) out[base + k] = excl + loc[k];
    if (threadIdx.x == MT - 1) sums[blockIdx.x] = excl + s;
}

__global__ void k_scan_add(int* out, const int* offs, long n) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offs[i / SCAN_B];
}

// out = exclusive scan of in (out may be in); *total = the sum
std::string scan_excl(const int* in, int* out, long n, long* total, cudaStream_t st) {
    Err E;
    if (n <= 0) {
        *total = 0;
        return "";
    }
    const long nb = (n + SCAN_B - 1) / SCAN_B;
    DBuf<int> sums;
    MG_TRY(sums.alloc(nb));
    int last_in = 0;
    MG_TRY(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_TRY(cudaStreamSynchronize(st));
    k_scan_blocks<<<(unsigned)nb, MT, 0, st>>>(in, out, sums.p, n);
    MG_TRY(cudaGetLastError());
    if (nb > 1) {
        long t2 = 0;
        std::string e = scan_excl(sums.p, sums.p, nb, &t2, st);
        if (!e.empty()) return e;
        k_scan_add<<<mgrid(n), MT, 0, st>>>(out, sums.p, n);
        MG_TRY(cudaGetLastError());
    }
    int last_out = 0;
    MG_TRY(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    MG_TRY(cudaStreamSynchronize(st));
    *total = (long)last_out + last_in;
    return "";
}

// ---------------------------------------------------------------- stable LSD radix sort
// (uint64 key, int value) pairs on their low `bits` bits, 8 bits per pass.  A block ranks
// a tile of RS_TILE pairs in order: chunks of one pair per thread, ranks among equal
// digits within a warp (__match_any_sync), per-warp digit counts in shared memory, and a
// running per-digit offset from the scanned (digit-major, tile-minor) histogram.
constexpr int RS_CHUNKS = 8;
constexpr int RS_TILE = RS_CHUNKS * MT;

__global__ void __launch_bounds__(MT) k_radix_count(const uint64_t* key, long n, int shift, int ntiles, int* hist) {
    __shared__ int cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const long base = (long)blockIdx.x * RS_TILE;
    for (int c = 0; c < RS_CHUNKS; ++c) {
        const long i = base + (long)c * MT + threadIdx.x;
        if (i < n) atomicAdd(&cnt[(key[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(long)threadIdx.x * ntiles + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(MT) k_radix_scatter(const uint64_t* kin, const int* vin, uint64_t* kout, int* vout,
                                                      long n, int shift, int ntiles, const int* offs) {
    __shared__ int run[256];
    __shared__ int wcnt[MT / 32][256];
    run[threadIdx.x] = offs[(long)threadIdx.x * ntiles + blockIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const long base = (long)blockIdx.x * RS_TILE;
    for (int c = 0; c < RS_CHUNKS; ++c) {
#pragma unroll
        for (int k = 0; k < MT / 32; ++k) wcnt[k][threadIdx.x] = 0;
        __syncthreads();
        const long i = base + (long)c * MT + threadIdx.x;
        const bool valid = i < n;
        uint64_t kk = 0;
        int vv = 0;
        unsigned d = 256;
        if (valid) {
            kk = kin[i];
            vv = vin[i];
            d = (unsigned)((kk >> shift) & 255u);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int wrank = __popc(peers & lt);
        if (valid && wrank == 0) wcnt[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            int before = 0;
            for (int k = 0; k < w; ++k) before += wcnt[k][d];
            const int pos = run[d] + before + wrank;
            kout[pos] = kk;
            vout[pos] = vv;
        }
        __syncthreads();
        int tot = 0;
#pragma unroll
        for (int k = 0; k < MT / 32; ++k) tot += wcnt[k][threadIdx.x];
        run[threadIdx.x] += tot;
        __syncthreads();
    }
}

// sorts (key, val) in place by the low `bits` bits of key, stable
std::string radix_sort(uint64_t* key, int* val, long n, int bits, cudaStream_t st) {
    Err E;
    if (n <= 1) return "";
    const int ntiles = (int)((n + RS_TILE - 1) / RS_TILE);
    DBuf<uint64_t> k2;
    DBuf<int> v2, hist;
    MG_TRY(k2.alloc(n));
    MG_TRY(v2.alloc(n));
    MG_TRY(hist.alloc(256L * ntiles));
    uint64_t *ka = key, *kb = k2.p;
    int *va = val, *vb = v2.p;
    int passes = 0;
    for (int shift = 0; shift < bits; shift += 8, ++passes) {
        k_radix_count<<<ntiles, MT, 0, st>>>(ka, n, shift, ntiles, hist.p);
        MG_TRY(cudaGetLastError());
        long tot = 0;
        std::string e = scan_excl(hist.p, hist.p, 256L * ntiles, &tot, st);
        if (!e.empty()) return e;
        k_radix_scatter<<<ntiles, MT, 0, st>>>(ka, va, kb, vb, n, shift, ntiles, hist.p);
        MG_TRY(cudaGetLastError());
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (passes & 1) {
        MG_TRY(cudaMemcpyAsync(key, ka, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, st));
        MG_TRY(cudaMemcpyAsync(val, va, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    }
    MG_TRY(cudaStreamSynchronize(st));
    return "";
}

// ---------------------------------------------------------------- connectivity
__device__ __forceinline__ int cell_nv(const int* cells, long i) { return cells[4 * i + 3] >= 0 ? 4 : 3; }

// half-edge q = 4 i + j: lo, hi node (lo = -1 for the unused fourth slot of a triangle);
// counts per lo node
__global__ void k_half_edges(long nc, const int* cells, int* lo, int* hi, int* cnt) {
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 4 * nc) return;
    const long i = q >> 2;
    const int j = (int)(q & 3), nv = cell_nv(cells, i);
    if (j >= nv) {
        lo[q] = -1;
        return;
    }
    const int a = cells[4 * i + j], b = cells[4 * i + (j + 1) % nv];
    const int l = a < b ? a : b, h = a < b ? b : a;
    lo[q] = l;
    hi[q] = h;
    atomicAdd(&cnt[l], 1);
}

__global__ void k_bucket_scatter(long n, const int* bucket, const int* start, int* cur, int* out) {
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n || bucket[q] < 0) return;
    const int b = bucket[q];
    out[start[b] + atomicAdd(&cur[b], 1)] = (int)q;
}

// each bucket's items sorted by (k2[item], item): insertion sort (buckets hold a few items)
__global__ void k_bucket_sort(long nb, const int* start, const int* k2, int* items) {
    const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    const int s = start[b], e = start[b + 1];
    for (int x = s + 1; x < e; ++x) {
        const int it = items[x];
        const int kv = k2[it];
        int y = x - 1;
        while (y >= s && (k2[items[y]] > kv || (k2[items[y]] == kv && items[y] > it))) {
            items[y + 1] = items[y];
            --y;
        }
        items[y + 1] = it;
    }
}

// runs of equal hi within a node's bucket are the half-edges of one edge: the first
// opens the face (first[q] = 1, partner[q] = the second or -1); more than two is an error
__global__ void k_edges(long nn, const int* start, const int* items, const int* hi, int* first, int* partner,
                        int* bad_edge) {
    const long u = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    const int s = start[u], e = start[u + 1];
    int x = s;
    while (x < e) {
        int y = x + 1;
        while (y < e && hi[items[y]] == hi[items[x]]) ++y;
        const int q = items[x];
        first[q] = 1;
        partner[q] = y - x >= 2 ? items[x + 1] : -1;
        if (y - x > 2) atomicMin(bad_edge, items[x + 2]);  // the third cell to name the edge
        x = y;
    }
}

// faces in reference order: owner, neighbour, nodes; the face of every half-edge
__global__ void k_faces(long nq, const int* first, const int* fidx, const int* partner, const int* lo, const int* hi,
                        int* f_o, int* f_n, int* f_n1, int* f_n2, int* hface) {
    const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq || !first[q]) return;
    const int f = fidx[q], p = partner[q];
    f_o[f] = (int)(q >> 2);
    f_n[f] = p >= 0 ? (p >> 2) : -1;
    f_n1[f] = lo[q];
    f_n2[f] = hi[q];
    hface[q] = f;
    if (p >= 0) hface[p] = f;
}

// boundary edge e -> the face with its key; the last boundary edge of a key wins
__global__ void k_btags(int nbe, const int* bedges, const int* start, const int* items, const int* hi,
                        const int* hface, long nn, int nf, int* fbest) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbe) return;
    const int a = bedges[3 * e], b = bedges[3 * e + 1];
    const int l = a < b ? a : b, h = a < b ? b : a;
    if (l < 0 || l >= nn) return;
    for (int x = start[l]; x < start[l + 1]; ++x)
        if (hi[items[x]] == h) {
            const int f = hface[items[x]];  // the edge's first half-edge: its face is set
            if (f >= 0 && f < nf) atomicMax(&fbest[f], e);
            return;
        }
}

__global__ void k_ftag(int nf, const int* fbest, const int* bedges, int* f_tag) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    f_tag[f] = fbest[f] >= 0 ? bedges[3 * fbest[f] + 2] : 0;
}

// ---------------------------------------------------------------- geometry (src/Mesh.cpp:148-201)
__global__ void k_cell_geo(long nc, const double* xy, const int* cells, double* vol, double* xc, double* yc,
                           int* bad_cell) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const int* c = cells + 4 * i;
    double v;
    if (c[3] < 0) {
        const double x1 = xy[2 * c[0]], y1 = xy[2 * c[0] + 1], x2 = xy[2 * c[1]], y2 = xy[2 * c[1] + 1];
        const double x3 = xy[2 * c[2]], y3 = xy[2 * c[2] + 1];
        v = 0.5 * fabs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1));
        xc[i] = (x1 + x2 + x3) / 3.0;
        yc[i] = (y1 + y2 + y3) / 3.0;
    } else {
        double sx = 0, sy = 0, a = 0.0;
        for (int k = 0; k < 4; ++k) {
            sx += xy[2 * c[k]];
            sy += xy[2 * c[k] + 1];
        }
        xc[i] = sx / 4.0;
        yc[i] = sy / 4.0;
        for (int k = 0; k < 4; ++k) {
            const int n1 = c[k], n2 = c[(k + 1) % 4];
            a += (xy[2 * n1] * xy[2 * n2 + 1] - xy[2 * n2] * xy[2 * n1 + 1]);
        }
        v = 0.5 * fabs(a);
    }
    vol[i] = v;
    if (!(v > 0.0)) atomicMin(bad_cell, (int)i);
}

__global__ void k_face_geo(int nf, const double* xy, const int* f_n1, const int* f_n2, const int* f_o,
                           const double* xc, const double* yc, double* f_nx, double* f_ny, double* f_area,
                           double* f_xm, double* f_ym) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int a = f_n1[f], b = f_n2[f];
    const double dx = xy[2 * b] - xy[2 * a];
    const double dy = xy[2 * b + 1] - xy[2 * a + 1];
    const double A = sqrt(dx * dx + dy * dy);
    const double xm = 0.5 * (xy[2 * a] + xy[2 * b]);
    const double ym = 0.5 * (xy[2 * a + 1] + xy[2 * b + 1]);
    double nx = dy / A, ny = -dx / A;
    const double vx = xm - xc[f_o[f]];
    const double vy = ym - yc[f_o[f]];
    if (vx * nx + vy * ny < 0) {
        nx = -nx;
        ny = -ny;
    }
    f_area[f] = A;
    f_xm[f] = xm;
    f_ym[f] = ym;
    f_nx[f] = nx;
    f_ny[f] = ny;
}

// ---------------------------------------------------------------- renumbering
// Bounding box of the cell centroids in two passes: each of the first pass's blocks reduces
// a grid-stride share into part[4 * block + (x min, x max, y min, y max)], then one block
// reduces the parts (nb of them, x and y read through the same planes: stride 4) into out4.
// Selections only, so the result is exact in any order.
__global__ void k_minmax(long n, const double* x, const double* y, long stride, double* out4) {
    __shared__ double s[4][MT];
    double a = 1e300, b = -1e300, c = 1e300, d = -1e300;
    for (long i = (long)blockIdx.x * MT + threadIdx.x; i < n; i += (long)gridDim.x * MT) {
        const double xi = x[i * stride], yi = y[i * stride];
        a = fmin(a, xi);
        b = fmax(b, stride == 1 ? xi : x[i * stride + 1]);
        c = fmin(c, yi);
        d = fmax(d, stride == 1 ? yi : y[i * stride + 1]);
    }
    s[0][threadIdx.x] = a;
    s[1][threadIdx.x] = b;
    s[2][threadIdx.x] = c;
    s[3][threadIdx.x] = d;
    __syncthreads();
    for (int o = MT / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + o]);
            s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + o]);
            s[2][threadIdx.x] = fmin(s[2][threadIdx.x], s[2][threadIdx.x + o]);
            s[3][threadIdx.x] = fmax(s[3][threadIdx.x], s[3][threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x < 4) out4[4 * blockIdx.x + threadIdx.x] = s[threadIdx.x][0];
}

// Hilbert index of (x, y) on a 2^order grid (the quadrant walk of mesh.cpp's hilbert_index)
__device__ uint64_t hilbert_d(uint32_t x, uint32_t y, int order) {
    const uint32_t n = 1u << order;
    uint64_t d = 0;
    for (uint32_t s = n >> 1; s > 0; s >>= 1) {
        const uint32_t rx = (x & s) ? 1u : 0u;
        const uint32_t ry = (y & s) ? 1u : 0u;
        d += (uint64_t)s * s * ((3u * rx) ^ ry);
        if (ry == 0) {
            if (rx == 1) {
                x = n - 1 - x;
                y = n - 1 - y;
            }
            const uint32_t t = x;
            x = y;
            y = t;
        }
    }
    return d;
}

__global__ void k_hilbert_keys(long nc, const double* xc, const double* yc, double x0, double y0, double scale,
                               int order, uint64_t* key, int* val) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const uint32_t hx = (uint32_t)((xc[i] - x0) * scale);
    const uint32_t hy = (uint32_t)((yc[i] - y0) * scale);
    key[i] = hilbert_d(hx, hy, order);
    val[i] = (int)i;
}

__global__ void k_inverse(long n, const int* perm, int* inv) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) inv[perm[i]] = (int)i;
}

// face slot buckets: interior faces by their lower new cell, boundary faces by nc + owner;
// the secondary key is the higher new cell (interior) or the face itself (boundary)
__global__ void k_face_buckets(int nf, long nc, const int* f_o, const int* f_n, const int* inv, int* bucket, int* k2,
                               int* cnt) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const int o = inv[f_o[f]];
    int b, s;
    if (f_n[f] < 0) {
        b = (int)nc + o;
        s = f;
    } else {
        const int n = inv[f_n[f]];
        b = o < n ? o : n;
        s = o < n ? n : o;
    }
    bucket[f] = b;
    k2[f] = s;
    atomicAdd(&cnt[b], 1);
}

// per-slot face data (the same expressions as mesh.cpp / src/Solver.cpp:564-567, :729-730)
__global__ void k_slots(int nf, const int* face_perm, const int* inv, const int* f_o, const int* f_n, const int* f_tag,
                        const double* f_nx, const double* f_ny, const double* f_area, const double* f_xm,
                        const double* f_ym, const double* xc, const double* yc, int* fo, int* fn, int* ftag,
                        double* nx, double* ny, double* area, double* dxo, double* dyo, double* dxn, double* dyn,
                        double* dxlr, double* dylr, int* wall_flag) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nf) return;
    const int f = face_perm[s];
    const int o = f_o[f], n = f_n[f];
    fo[s] = inv[o];
    fn[s] = n >= 0 ? inv[n] : -1;
    ftag[s] = f_tag[f];
    nx[s] = f_nx[f];
    ny[s] = f_ny[f];
    area[s] = f_area[f];
    dxo[s] = f_xm[f] - xc[o];
    dyo[s] = f_ym[f] - yc[o];
    dxn[s] = n >= 0 ? f_xm[f] - xc[n] : 0.0;
    dyn[s] = n >= 0 ? f_ym[f] - yc[n] : 0.0;
    const int n2 = n >= 0 ? n : o;
    dxlr[s] = xc[n2] - xc[o];
    dylr[s] = yc[n2] - yc[o];
    wall_flag[s] = (n < 0 && f_tag[f] == 4) ? 1 : 0;
}

__global__ void k_compact(int n, const int* flag, const int* pos, int* out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n && flag[s]) out[pos[s]] = s;
}

// new cell i: its faces (reference face order) as (slot << 1) | side in cf[k][nc]; the
// cell data in the new order
__global__ void k_cells_new(long nc, const int* perm, const int* cells, const int* hface, const int* first,
                            const int* face_inv, const double* vol0, const double* xc0, const double* yc0, int* cf,
                            double* vol, double* xc, double* yc) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    const int c = perm[i];
    const int nv = cell_nv(cells, c);
    int fs[4], side[4];
    for (int j = 0; j < 4; ++j) {
        fs[j] = 0x7fffffff;
        side[j] = 0;
    }
    for (int j = 0; j < nv; ++j) {
        const long q = 4L * c + j;
        fs[j] = hface[q];
        side[j] = first[q] ? 0 : 1;
    }
    for (int a = 1; a < nv; ++a)  // by reference face index
        for (int b = a; b > 0 && fs[b - 1] > fs[b]; --b) {
            const int t = fs[b], u = side[b];
            fs[b] = fs[b - 1];
            side[b] = side[b - 1];
            fs[b - 1] = t;
            side[b - 1] = u;
        }
    for (int k = 0; k < 4; ++k) cf[(long)k * nc + i] = k < nv ? ((face_inv[fs[k]] << 1) | side[k]) : -1;
    vol[i] = vol0[c];
    xc[i] = xc0[c];
    yc[i] = yc0[c];
}

template <class T>
std::string down(std::vector<T>& v, const T* d, size_t n, cudaStream_t st) {
    Err E;
    v.resize(n);
    if (n) MG_TRY(cudaMemcpyAsync(v.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost, st));
    return "";
}

}  // namespace

std::string build_mesh_gpu(HostMesh& m, int n_nodes, const double* xy, int n_cells, const int* cells, int n_bedges,
                           const int* bedges, int renumber, int device, double* seconds) {
    Err E;
    if (n_nodes <= 0 || n_cells <= 0) return "mesh has no nodes or no cells";
    for (int i = 0; i < n_cells; ++i) {
        const int nv = cells[4 * i + 3] >= 0 ? 4 : 3;
        for (int k = 0; k < nv; ++k) {
            const int v = cells[4 * i + k];
            if (v < 0 || v >= n_nodes) {
                char b[128];
                std::snprintf(b, sizeof b, "cell %d refers to node %d outside [0, %d)", i, v, n_nodes);
                return b;
            }
        }
    }
    MG_TRY(cudaSetDevice(device));
    cudaStream_t st = nullptr;
    MG_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    cudaEvent_t ev0, ev1;
    MG_TRY(cudaEventCreate(&ev0));
    MG_TRY(cudaEventCreate(&ev1));
    struct EventGuard {
        cudaEvent_t a, b;
        ~EventGuard() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } eg{ev0, ev1};
    m = HostMesh();
    m.n_nodes = n_nodes;
    m.n_cells = n_cells;
    m.xy.assign(xy, xy + 2 * (size_t)n_nodes);
    m.cell_nodes.assign(cells, cells + 4 * (size_t)n_cells);
    const long nc = n_cells, nn = n_nodes, nq = 4 * nc;

    DBuf<double> dxy;
    DBuf<int> dcells, dbed, lo, hi, cnt, start, cur, items, first, partner, fidx, hface, bad;
    MG_TRY(dxy.alloc(2 * nn));
    MG_TRY(dcells.alloc(nq));
    MG_TRY(dbed.alloc(3 * (size_t)n_bedges));
    MG_TRY(lo.alloc(nq));
    MG_TRY(hi.alloc(nq));
    MG_TRY(cnt.alloc(nn + 1));
    MG_TRY(start.alloc(nn + 1));
    MG_TRY(cur.alloc(nn));
    MG_TRY(first.alloc(nq));
    MG_TRY(partner.alloc(nq));
    MG_TRY(fidx.alloc(nq));
    MG_TRY(hface.alloc(nq));
    MG_TRY(bad.alloc(2));
    MG_TRY(cudaEventRecord(ev0, st));
    MG_TRY(cudaMemcpyAsync(dxy.p, xy, sizeof(double) * 2 * nn, cudaMemcpyHostToDevice, st));
    MG_TRY(cudaMemcpyAsync(dcells.p, cells, sizeof(int) * nq, cudaMemcpyHostToDevice, st));
    if (n_bedges)
        MG_TRY(cudaMemcpyAsync(dbed.p, bedges, sizeof(int) * 3 * (size_t)n_bedges, cudaMemcpyHostToDevice, st));
    MG_TRY(cudaMemsetAsync(cnt.p, 0, sizeof(int) * (nn + 1), st));
    MG_TRY(cudaMemsetAsync(cur.p, 0, sizeof(int) * nn, st));
    MG_TRY(cudaMemsetAsync(first.p, 0, sizeof(int) * nq, st));
    MG_TRY(cudaMemsetAsync(hface.p, 0xff, sizeof(int) * nq, st));  // -1: no face (yet)
    const int big = 0x7fffffff;
    int hbad[2] = {big, big};
    MG_TRY(cudaMemcpyAsync(bad.p, hbad, sizeof(hbad), cudaMemcpyHostToDevice, st));

    // 1. half-edges bucketed by their lower node, each bucket in (hi, q) order
    k_half_edges<<<mgrid(nq), MT, 0, st>>>(nc, dcells.p, lo.p, hi.p, cnt.p);
    MG_TRY(cudaGetLastError());
    long nhe = 0;
    {
        std::string e = scan_excl(cnt.p, start.p, nn + 1, &nhe, st);
        if (!e.empty()) return e;
    }
    MG_TRY(items.alloc(nhe));
    k_bucket_scatter<<<mgrid(nq), MT, 0, st>>>(nq, lo.p, start.p, cur.p, items.p);
    k_bucket_sort<<<mgrid(nn), MT, 0, st>>>(nn, start.p, hi.p, items.p);
    // 2. edges, faces in creation order
    k_edges<<<mgrid(nn), MT, 0, st>>>(nn, start.p, items.p, hi.p, first.p, partner.p, bad.p);
    MG_TRY(cudaGetLastError());
    long nf = 0;
    {
        std::string e = scan_excl(first.p, fidx.p, nq, &nf, st);
        if (!e.empty()) return e;
    }
    m.n_faces = (int)nf;
    DBuf<int> f_o, f_n, f_n1, f_n2, f_tag, fbest;
    MG_TRY(f_o.alloc(nf));
    MG_TRY(f_n.alloc(nf));
    MG_TRY(f_n1.alloc(nf));
    MG_TRY(f_n2.alloc(nf));
    MG_TRY(f_tag.alloc(nf));
    MG_TRY(fbest.alloc(nf));
    k_faces<<<mgrid(nq), MT, 0, st>>>(nq, first.p, fidx.p, partner.p, lo.p, hi.p, f_o.p, f_n.p, f_n1.p, f_n2.p,
                                      hface.p);
    // 3. boundary tags
    MG_TRY(cudaMemsetAsync(fbest.p, 0xff, sizeof(int) * nf, st));
    if (n_bedges)
        k_btags<<<mgrid(n_bedges), MT, 0, st>>>(n_bedges, dbed.p, start.p, items.p, hi.p, hface.p, nn, (int)nf,
                                                fbest.p);
    k_ftag<<<mgrid(nf), MT, 0, st>>>((int)nf, fbest.p, dbed.p, f_tag.p);
    MG_TRY(cudaGetLastError());
    // 4. geometry
    DBuf<double> c_vol, c_xc, c_yc, f_nx, f_ny, f_area, f_xm, f_ym;
    MG_TRY(c_vol.alloc(nc));
    MG_TRY(c_xc.alloc(nc));
    MG_TRY(c_yc.alloc(nc));
    MG_TRY(f_nx.alloc(nf));
    MG_TRY(f_ny.alloc(nf));
    MG_TRY(f_area.alloc(nf));
    MG_TRY(f_xm.alloc(nf));
    MG_TRY(f_ym.alloc(nf));
    k_cell_geo<<<mgrid(nc), MT, 0, st>>>(nc, dxy.p, dcells.p, c_vol.p, c_xc.p, c_yc.p, bad.p + 1);
    k_face_geo<<<mgrid(nf), MT, 0, st>>>((int)nf, dxy.p, f_n1.p, f_n2.p, f_o.p, c_xc.p, c_yc.p, f_nx.p, f_ny.p,
                                         f_area.p, f_xm.p, f_ym.p);
    MG_TRY(cudaGetLastError());
    MG_TRY(cudaMemcpyAsync(hbad, bad.p, sizeof(hbad), cudaMemcpyDeviceToHost, st));
    MG_TRY(cudaStreamSynchronize(st));
    if (hbad[0] != big) {
        // the first half-edge, in cell order, that names an edge a third time (build_mesh's report)
        const int i = hbad[0] >> 2, j = hbad[0] & 3, nv = cells[4 * i + 3] >= 0 ? 4 : 3;
        char b[160];
        std::snprintf(b, sizeof b, "edge (%d,%d) is shared by more than two cells", cells[4 * i + j],
                      cells[4 * i + (j + 1) % nv]);
        return b;
    }
    if (hbad[1] != big) {
        char b[96];
        std::snprintf(b, sizeof b, "cell %d has zero or invalid area", hbad[1]);
        return b;
    }
    // 5. renumbering
    DBuf<int> perm, inv;
    MG_TRY(perm.alloc(nc));
    MG_TRY(inv.alloc(nc));
    if (renumber == RENUMBER_HILBERT) {
        DBuf<double> mm;
        DBuf<uint64_t> key;
        constexpr int MM_BLOCKS = 304;
        MG_TRY(mm.alloc(4 * (MM_BLOCKS + 1)));
        MG_TRY(key.alloc(nc));
        k_minmax<<<MM_BLOCKS, MT, 0, st>>>(nc, c_xc.p, c_yc.p, 1, mm.p + 4);
        // the parts: x min / x max at 4 b + 0 / 1, y min / y max at 4 b + 2 / 3
        k_minmax<<<1, MT, 0, st>>>(MM_BLOCKS, mm.p + 4, mm.p + 6, 4, mm.p);
        double h4[4];
        MG_TRY(cudaMemcpyAsync(h4, mm.p, sizeof(h4), cudaMemcpyDeviceToHost, st));
        MG_TRY(cudaStreamSynchronize(st));
        const int order = 16;
        const double span = std::max(h4[1] - h4[0], h4[3] - h4[2]) + 1e-300;
        const double scale = ((1u << order) - 1) / span;
        k_hilbert_keys<<<mgrid(nc), MT, 0, st>>>(nc, c_xc.p, c_yc.p, h4[0], h4[2], scale, order, key.p, perm.p);
        MG_TRY(cudaGetLastError());
        std::string e = radix_sort(key.p, perm.p, nc, 2 * order, st);
        if (!e.empty()) return e;
    } else if (renumber == RENUMBER_RCM) {
        // breadth-first and sequential: on the host, from the GPU's connectivity
        std::string e = down(m.f_o, f_o.p, nf, st);
        if (e.empty()) e = down(m.f_n, f_n.p, nf, st);
        if (!e.empty()) return e;
        MG_TRY(cudaStreamSynchronize(st));
        order_rcm_host(m, m.cell_perm);
        MG_TRY(cudaMemcpyAsync(perm.p, m.cell_perm.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, st));
    } else {
        m.cell_perm.resize(nc);
        for (long i = 0; i < nc; ++i) m.cell_perm[i] = (int)i;
        MG_TRY(cudaMemcpyAsync(perm.p, m.cell_perm.data(), sizeof(int) * nc, cudaMemcpyHostToDevice, st));
    }
    k_inverse<<<mgrid(nc), MT, 0, st>>>(nc, perm.p, inv.p);
    // 6. face slots
    DBuf<int> fbucket, fk2, fcnt, fstart, fcur, face_perm, face_inv;
    MG_TRY(fbucket.alloc(nf));
    MG_TRY(fk2.alloc(nf));
    MG_TRY(fcnt.alloc(2 * nc + 1));
    MG_TRY(fstart.alloc(2 * nc + 1));
    MG_TRY(fcur.alloc(2 * nc));
    MG_TRY(face_perm.alloc(nf));
    MG_TRY(face_inv.alloc(nf));
    MG_TRY(cudaMemsetAsync(fcnt.p, 0, sizeof(int) * (2 * nc + 1), st));
    MG_TRY(cudaMemsetAsync(fcur.p, 0, sizeof(int) * 2 * nc, st));
    k_face_buckets<<<mgrid(nf), MT, 0, st>>>((int)nf, nc, f_o.p, f_n.p, inv.p, fbucket.p, fk2.p, fcnt.p);
    MG_TRY(cudaGetLastError());
    long nslots = 0;
    {
        std::string e = scan_excl(fcnt.p, fstart.p, 2 * nc + 1, &nslots, st);
        if (!e.empty()) return e;
    }
    k_bucket_scatter<<<mgrid(nf), MT, 0, st>>>(nf, fbucket.p, fstart.p, fcur.p, face_perm.p);
    k_bucket_sort<<<mgrid(2 * nc), MT, 0, st>>>(2 * nc, fstart.p, fk2.p, face_perm.p);
    k_inverse<<<mgrid(nf), MT, 0, st>>>(nf, face_perm.p, face_inv.p);
    MG_TRY(cudaGetLastError());
    // 7. the device layout
    DBuf<int> fo, fn, ftag, wflag, wpos, wall;
    DBuf<double> nx, ny, area, dxo, dyo, dxn, dyn, dxlr, dylr, vol, xc, yc;
    DBuf<int> cf;
    MG_TRY(fo.alloc(nf));
    MG_TRY(fn.alloc(nf));
    MG_TRY(ftag.alloc(nf));
    MG_TRY(wflag.alloc(nf));
    MG_TRY(wpos.alloc(nf));
    for (DBuf<double>* b : {&nx, &ny, &area, &dxo, &dyo, &dxn, &dyn, &dxlr, &dylr}) MG_TRY(b->alloc(nf));
    for (DBuf<double>* b : {&vol, &xc, &yc}) MG_TRY(b->alloc(nc));
    MG_TRY(cf.alloc(4 * nc));
    k_slots<<<mgrid(nf), MT, 0, st>>>((int)nf, face_perm.p, inv.p, f_o.p, f_n.p, f_tag.p, f_nx.p, f_ny.p, f_area.p,
                                      f_xm.p, f_ym.p, c_xc.p, c_yc.p, fo.p, fn.p, ftag.p, nx.p, ny.p, area.p, dxo.p,
                                      dyo.p, dxn.p, dyn.p, dxlr.p, dylr.p, wflag.p);
    k_cells_new<<<mgrid(nc), MT, 0, st>>>(nc, perm.p, dcells.p, hface.p, first.p, face_inv.p, c_vol.p, c_xc.p, c_yc.p,
                                          cf.p, vol.p, xc.p, yc.p);
    MG_TRY(cudaGetLastError());
    long nwall = 0;
    {
        std::string e = scan_excl(wflag.p, wpos.p, nf, &nwall, st);
        if (!e.empty()) return e;
    }
    MG_TRY(wall.alloc(nwall));
    k_compact<<<mgrid(nf), MT, 0, st>>>((int)nf, wflag.p, wpos.p, wall.p);
    MG_TRY(cudaGetLastError());
    MG_TRY(cudaEventRecord(ev1, st));
    // read back into the HostMesh
    std::string e;
    auto dl = [&](auto& v, const auto* d, size_t n) {
        if (e.empty()) e = down(v, d, n, st);
    };
    dl(m.f_n1, f_n1.p, nf);
    dl(m.f_n2, f_n2.p, nf);
    dl(m.f_o, f_o.p, nf);
    dl(m.f_n, f_n.p, nf);
    dl(m.f_tag, f_tag.p, nf);
    dl(m.f_nx, f_nx.p, nf);
    dl(m.f_ny, f_ny.p, nf);
    dl(m.f_area, f_area.p, nf);
    dl(m.f_xm, f_xm.p, nf);
    dl(m.f_ym, f_ym.p, nf);
    dl(m.c_vol, c_vol.p, nc);
    dl(m.c_xc, c_xc.p, nc);
    dl(m.c_yc, c_yc.p, nc);
    dl(m.cell_perm, perm.p, nc);
    dl(m.cell_inv, inv.p, nc);
    dl(m.face_perm, face_perm.p, nf);
    dl(m.face_inv, face_inv.p, nf);
    dl(m.cf, cf.p, 4 * nc);
    dl(m.fo, fo.p, nf);
    dl(m.fn, fn.p, nf);
    dl(m.ftag, ftag.p, nf);
    dl(m.nx, nx.p, nf);
    dl(m.ny, ny.p, nf);
    dl(m.area, area.p, nf);
    dl(m.dxo, dxo.p, nf);
    dl(m.dyo, dyo.p, nf);
    dl(m.dxn, dxn.p, nf);
    dl(m.dyn, dyn.p, nf);
    dl(m.dxlr, dxlr.p, nf);
    dl(m.dylr, dylr.p, nf);
    dl(m.vol, vol.p, nc);
    dl(m.xc, xc.p, nc);
    dl(m.yc, yc.p, nc);
    dl(m.wall_faces, wall.p, nwall);
    if (!e.empty()) return e;
    MG_TRY(cudaStreamSynchronize(st));
    int nb = 0;
    for (long f = 0; f < nf; ++f) nb += m.f_n[f] < 0;
    m.n_interior = (int)nf - nb;
    if (seconds) {
        float ms = 0;
        MG_TRY(cudaEventElapsedTime(&ms, ev0, ev1));
        *seconds = ms * 1e-3;
    }
    return "";
}

}  // namespace cfdg
