// cfdg_norm_vm_noalloc: the volume-weighted residual norm for callers that cannot
// allocate device memory.
//
// Who needs it: an application whose device memory is owned by its own pool (it
// reserves the GPU up front and a cudaMalloc from a library would fail or fragment that
// pool), and a caller on a latency-bound path where cudaMalloc's implicit device
// synchronisation and unbounded latency are not acceptable.  Such a caller keeps its
// residual and cell volumes in its own device buffers and only needs the norm that
// drives the Newton convergence test.
//
// The reduction's scratch (one pair of partial sums per block and a ticket counter)
// is the file-scope array below, sized for NA_MAX_BLOCKS blocks of NA_CELLS_PER_BLOCK
// cells: at most 8,388,608 cells, 32 KiB plus the counter.  Every GPU that loads this
// library holds the array until the process exits.  All calls share it: the ticket
// counter is cleared before each launch, and two calls that overlap on the GPU (two
// streams, or two host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/cfdg.h"
#include "linalg.cuh"

namespace cfdg {
void set_error_message(const std::string& msg);  // solver.cu
}

namespace {

constexpr int NA_THREADS = 256;
constexpr int NA_CELLS_PER_THREAD = 16;
constexpr long NA_CELLS_PER_BLOCK = (long)NA_THREADS * NA_CELLS_PER_THREAD;   // 4096
constexpr int NA_MAX_BLOCKS = 2048;
constexpr long NA_MAX_CELLS = NA_CELLS_PER_BLOCK * NA_MAX_BLOCKS;             // 8,388,608
constexpr int NA_COUNTER_SLOT = 2 * NA_MAX_BLOCKS;                            // after the partials

// partial sums [0, NA_MAX_BLOCKS) sum of squares, [NA_MAX_BLOCKS, 2 NA_MAX_BLOCKS) volumes,
// then the ticket counter in the first 4 bytes of slot NA_COUNTER_SLOT
static __device__ __align__(256) double g_norm_scratch[2 * NA_MAX_BLOCKS + 32];

// The per-cell sum of norm_L2_VolumeWeighted (src/Solver.cpp:1280-1303) with the
// reference's own division R / vol per component; k_norm_vm takes the same quotients
// through a shared reciprocal with a correction step, which rounds to the same bits, so
// the per-cell terms agree exactly.  The sums over cells run in another order than
// k_norm_vm's (each block owns a fixed range of cells, the last block to finish combines
// the partials in index order and writes sqrt(sum_sq / total_vol)), so the two norms
// agree to rounding, not bit for bit.
__global__ void __launch_bounds__(NA_THREADS) k_norm_vm_static(long nc, int nv, const double* __restrict__ R,
                                                              const double* __restrict__ vol, double* scratch,
                                                              double* out) {
    double v[2] = {0.0, 0.0};
    long base = (long)blockIdx.x * NA_CELLS_PER_BLOCK;
    for (int k = 0; k < NA_CELLS_PER_THREAD; ++k) {
        long i = base + (long)k * NA_THREADS + threadIdx.x;
        if (i >= nc) break;
        double vv = vol[i];
        double s = 0.0;
        for (int c = 0; c < nv; ++c) {
            double r = R[c * nc + i] / vv;
            s = (c == 0) ? r * r : s + r * r;
        }
        v[0] += s * vv;
        v[1] += vv;
    }
    cfdg::block_sum<2>(v);
    unsigned* counter = reinterpret_cast<unsigned*>(scratch + NA_COUNTER_SLOT);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = v[0];
        scratch[NA_MAX_BLOCKS + blockIdx.x] = v[1];
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s[2] = {0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        s[0] += ((volatile double*)scratch)[b];
        s[1] += ((volatile double*)scratch)[NA_MAX_BLOCKS + b];
    }
    cfdg::block_sum<2>(s);
    if (threadIdx.x == 0) {
        out[0] = s[1] == 0.0 ? 0.0 : sqrt(s[0] / s[1]);
        *counter = 0u;
    }
}

std::mutex g_setup_mutex;
double* g_scratch_ptr[128] = {};

// Device address of the static scratch on the current device (the host-side name
// g_norm_scratch is only a stand-in, not a device address).  Looked up again on every
// call outside a stream capture, so a context torn down and made again (cudaDeviceReset)
// gets the address in its new module; inside a capture the address from the device's
// last uncaptured call is used, so a capture needs one uncaptured call on the device
// first (and a fresh one after a device reset).
cfdg_status scratch_address(cudaStream_t stream, double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cfdg::set_error_message(std::string("cfdg_norm_vm_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return CFDG_ERR_CUDA;
    }
    if (dev < 0 || dev >= 128) {
        cfdg::set_error_message("cfdg_norm_vm_noalloc: device ordinal above 127");
        return CFDG_ERR_ARG;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) {
        cfdg::set_error_message(std::string("cfdg_norm_vm_noalloc: cudaStreamIsCapturing: ") + cudaGetErrorString(e));
        return CFDG_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (cap != cudaStreamCaptureStatusNone) {
        if (!g_scratch_ptr[dev]) {
            cfdg::set_error_message("cfdg_norm_vm_noalloc: the first call on a device must come before any stream capture");
            return CFDG_ERR_ARG;
        }
    } else {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_norm_scratch);
        if (e != cudaSuccess || !p) {
            cfdg::set_error_message(std::string("cfdg_norm_vm_noalloc: cudaGetSymbolAddress: ") +
                                    cudaGetErrorString(e));
            return CFDG_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return CFDG_OK;
}

}  // namespace

extern "C" cfdg_status cfdg_norm_vm_noalloc(const double* R, const double* vol, long n_cells, int nv, double* out,
                                            void* stream) {
    if (!R || !vol || !out) {
        cfdg::set_error_message("cfdg_norm_vm_noalloc: null device pointer");
        return CFDG_ERR_ARG;
    }
    if (nv != 4 && nv != 6) {
        cfdg::set_error_message("cfdg_norm_vm_noalloc: nv must be 4 or 6");
        return CFDG_ERR_ARG;
    }
    if (n_cells < 1 || n_cells > NA_MAX_CELLS) {
        char b[160];
        std::snprintf(b, sizeof b,
                      "cfdg_norm_vm_noalloc: n_cells = %ld is outside [1, %ld], the capacity of its static scratch",
                      n_cells, NA_MAX_CELLS);
        cfdg::set_error_message(b);
        return CFDG_ERR_ARG;
    }
    double* scratch = nullptr;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cfdg_status st = scratch_address(s, &scratch);
    if (st != CFDG_OK) return st;
    cudaError_t e = cudaMemsetAsync(scratch + NA_COUNTER_SLOT, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) {
        cfdg::set_error_message(std::string("cfdg_norm_vm_noalloc: clearing the counter: ") + cudaGetErrorString(e));
        return CFDG_ERR_CUDA;
    }
    unsigned grid = (unsigned)((n_cells + NA_CELLS_PER_BLOCK - 1) / NA_CELLS_PER_BLOCK);
    k_norm_vm_static<<<grid, NA_THREADS, 0, s>>>(n_cells, nv, R, vol, scratch, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        cfdg::set_error_message(std::string("cfdg_norm_vm_noalloc: launch: ") + cudaGetErrorString(e));
        return CFDG_ERR_CUDA;
    }
    return CFDG_OK;
}
