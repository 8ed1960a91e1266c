// Host-side launchers.  The kernels live in three translation units so each gets its
// own floating-point contract:
//   kern_f64.cu  FP64 residual, pseudo-time and Krylov kernels, built with --fmad=false
//                so the arithmetic matches the reference's CPU code bit for bit
//   kern_f32.cu  FP32 residual and FP32-vector Krylov kernels (mixed precision), FMA on
//   kern_jv.cu   Dual-number (exact J v) kernels in FP64 and FP32, FMA on
#pragma once
#include <cuda_runtime.h>
#include "linalg.cuh"

namespace cfdg {

template <class R>
struct ResArgs {
    MeshView<R> m;
    Flow<R> F;
    int nv;
    Field<R> U, W, G, FA;   // for the Dual launch .d holds the derivative planes
    R* phi;
    R* out;                 // residual (or J v) planes, stride m.nc
    int do_limiter;
    const R* diag_v;        // optional: adds diag_v * vol / (dt + 1e-30)
    const R* dt;
    cudaStream_t stream;
    cudaEvent_t* ev;        // optional 5 events around the four kernels
    Field<R> T{nullptr, nullptr, 0};  // SST cell terms (mu_t, F1, S_k vol, S_w vol); nv = 6 only
    const R* dwall = nullptr;         // wall distance per cell; nv = 6 only
    bool pdl = false;                 // launch_jv_mid: programmatic dependent launch (pdl.cuh)
    const int* done = nullptr;        // launch_jv_mid: skip when *done (a finished Krylov solve)
    // launch_jv_mid: the value planes of W, G and T are current (launch_values at the start
    // of the solve: the linearisation point does not move within it), so the gradient and
    // SST kernels write derivative planes only and the gradient kernel reads only the
    // derivative planes of its neighbours
    bool tangent = false;
    const int* lim_dev = nullptr;     // launch_residual<double>: the limiter also needs *lim_dev
    // launch_residual<double> of a Newton step: the gather fused with the step's reductions
    // (k_gather_norms) when norms_out is set
    double* rhs_out = nullptr;
    double* norms_out = nullptr;
    int* flag = nullptr;
    RedScratch rs{nullptr, nullptr};
    // launch_residual<double> of a caller's pinned rows: the primitives are current
    // (launch_rows_prim formed them with U), and the gather writes the caller's rows of
    // 6 doubles in place (rows_out, device-visible address) through iperm instead of out
    bool prim_done = false;
    double* rows_out = nullptr;
    const int* iperm = nullptr;
    // launch_jv_mid: per-cell neighbours and face geometry for the gradient kernel
    // (k_grad_cf) when cfx.nbr is set
    CellFaces<R> cfx{nullptr, nullptr, nullptr, nullptr};
    // launch_residual<double>: the interior faces' Green-Gauss terms (2 x primitives planes of
    // m.nfi), formed once per face by k_grad_faces64 when set
    double* gft = nullptr;
};

// A kernel launch, with the programmatic stream-serialisation attribute when pdl: the
// kernel may then start before its predecessor in the stream (or graph) completes and
// must keep the rules of pdl.cuh.
template <typename... KArgs, typename... Args>
inline void launch_k(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    if (!pdl) {
        kern<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

// R(U) (kern_f64.cu for double, kern_f32.cu for float)
template <class R> void launch_residual(const ResArgs<R>& a);
// J v by forward linearisation with the limiter frozen (kern_jv.cu)
template <class R> void launch_jv(const ResArgs<R>& a);
// the middle of it (gradients, SST terms, face fluxes) for the fused Arnoldi body
template <class R> void launch_jv_mid(const ResArgs<R>& a);
// the value planes of the linearisation point: primitives, gradients (no limiter) and, with
// SST, the cell terms of a.U.v into a.W.v, a.G.v, a.T.v
template <class R> void launch_values(const ResArgs<R>& a);

// ---- vectors (T = double in kern_f64.cu, T = float in kern_f32.cu)
template <class T> void launch_dot(int nv, long nc, const T* a, const T* b, RedScratch rs, double* out, cudaStream_t s);
template <class T> void launch_mgs(int nv, long nc, T* w, const T* vprev, const double* hprev, const T* vnext,
                                   RedScratch rs, double* out, cudaStream_t s);
template <class T> void launch_scale_guard(long n, T* x, const double* h_sq, double thresh, cudaStream_t s);
template <class T> void launch_scale_from(long n, T* x, const double* a, const double* sc, int invert, cudaStream_t s);
template <class T> void launch_precond_apply(int nv, long nc, const T* V, const double* D, T* z, RedScratch rs,
                                             double* out_sq, cudaStream_t s);
template <class T> void launch_gmres_solution(int nv, long nc, const T* V, long vstride, const double* y, int k,
                                              const double* D, double* x, cudaStream_t s);
template <class T> void launch_aos_to_soa(long nc, int np, int stride, const double* aos, const int* perm, T* soa,
                                          cudaStream_t s);
template <class T> void launch_soa_to_aos(long nc, int np, int stride, const T* soa, const int* perm, double* aos,
                                          cudaStream_t s);
template <class T> void launch_convert(long n, const double* in, T* out, cudaStream_t s);
// a caller's pinned rows (stride doubles, caller numbering; device-visible address) in place:
// np planes of soa at the rows' internal indices iperm[row] (stride <= ROW_MAX_STRIDE)
template <class T> void launch_soa_to_rows(long nc, int np, int stride, const T* soa, const int* iperm, double* aos,
                                           cudaStream_t s);
void launch_rows_to_soa(long nc, int np, int stride, const double* aos, const int* iperm, double* soa, cudaStream_t s);

// ---- FP64 only (kern_f64.cu)
void launch_prim64(int nv, long nc, const Flow<double>& F, Field<double> U, Field<double> W, cudaStream_t s);
// k_prim of a caller's pinned rows (6 doubles each): U and W planes at iperm[row]
void launch_rows_prim(int nv, long nc, const Flow<double>& F, const double* aos, const int* iperm, Field<double> U,
                      Field<double> W, cudaStream_t s);
void launch_fd_perturb(long n, const double* U, const double* v, const double* u_sq, const double* v_sq, double* Up,
                       double* eps, cudaStream_t s);
void launch_fd_combine(int nv, long nc, const double* Rp, const double* Rb, const double* v, const double* eps,
                       const double* vol, const double* dt, double* Jv, cudaStream_t s);
void launch_norm_vm(int nv, long nc, const double* R, const double* vol, RedScratch rs, double* out3, cudaStream_t s);
// norm_vm pieces, sum R^2 (out4[3]) and rhs = -R in one pass; clears *flag
void launch_step_norms(int nv, long nc, const double* R, const double* vol, double* rhs, RedScratch rs, double* out4,
                       int* flag, cudaStream_t s);
// the mixed-precision prologue of a Krylov solve (linalg.cuh k_mixed_pre; kern_f32.cu)
void launch_mixed_pre(int nv, const MeshView<float>& m, const Flow<float>& F, const double* U, const double* Ub,
                      const double* W,
                      const double* phi, const double* mut, const double* cfl, const double* dt_in, float* U32,
                      float* phi32, float* dt32, double* D, float* Dinv32, cudaStream_t s);
// cfl_dev (optional): the CFL number from device memory instead of cfl
void launch_local_dt(int nv, const MeshView<double>& m, const Flow<double>& F, const double* U, const double* W,
                     double cfl, double* dt, cudaStream_t s, const double* cfl_dev = nullptr);
// D: one plane per cell, three with SST (mean flow, k, w); mut: SST eddy viscosity or null
void launch_precond(int nv, const MeshView<double>& m, const Flow<double>& F, const double* U, const double* W,
                    const double* dt, double* D, const double* mut, cudaStream_t s);
void launch_newton_update(int nv, long nc, double* U, const double* dU, double relax, double gam, double wmin, int* bad,
                          cudaStream_t s);
// the Newton update with its decisions (converged / non-finite / relaxation) on the device
void launch_newton_update_dev(int nv, long nc, double* U, const double* dU, const double* norms, double tol, double gam,
                              double wmin, int* bad, cudaStream_t s);
// the same update plus the step's scalar control on the device (step k of a chain)
void launch_newton_update_chain(int nv, long nc, double* U, const double* dU, const double* norms, double tol,
                                double gam, double wmin, int* bad, const NewtonCtl& c, int k, int step, double ulim,
                                cudaStream_t s);
// time stepping: timeStepExplicit's update, solveUnsteady's right-hand side and update
void launch_explicit_update(int nv, long nc, double* U, const double* R, const double* vol, double dt, int* bad,
                            cudaStream_t s);
void launch_unsteady_rhs(int nv, long nc, const double* U, const double* Uold, const double* R, const double* vol,
                         double dt, double* rhs, RedScratch rs, double* out2, cudaStream_t s);
void launch_relaxed_add(int nv, long nc, double* U, const double* dU, double relax, int* bad, cudaStream_t s);
void launch_fill(long n, double* x, double v, cudaStream_t s);
// FP64 pipe probe: each thread runs FP64_STREAM_CHAINS independent FMA chains of `iters`
// steps (kern_f64.cu)
constexpr int FP64_STREAM_CHAINS = 8;
void launch_fp64_fma_stream(int blocks, int threads, double* sink, int iters, cudaStream_t s);

inline unsigned grid_for(long n, int threads = 256) { return (unsigned)((n + threads - 1) / threads); }
// reduction / streaming grids: one entry per thread up to RED_BLOCKS blocks (enough warps
// in flight to hide latency), grid-stride beyond
inline unsigned red_grid(long n) {
    long b = (n + RED_THREADS - 1) / RED_THREADS;
    return (unsigned)(b < RED_BLOCKS ? (b < 1 ? 1 : b) : RED_BLOCKS);
}

// Per-cell and per-face kernels: blocks of 64-256 threads so that even small meshes
// spread over every SM (two blocks per SM at least where the mesh allows)
inline unsigned tpb_for(long n) { return n >= 2L * 152 * 256 ? 256u : (n >= 2L * 152 * 128 ? 128u : 64u); }
inline unsigned blocks_for(long n) { return grid_for(n, (int)tpb_for(n)); }

// Kernels that end in multi-dot reductions: blocks of RED_THREADS, one per SM at most, so
// the last block sums few partials with all its warps; grid-stride beyond
inline unsigned kry_grid(long n) {
    long b = (n + RED_THREADS - 1) / RED_THREADS;
    return (unsigned)(b < 152 ? (b < 1 ? 1 : b) : 152);
}
// blocks of the exact J v gather kernel (k_gmres_gather_dot): two per SM with an FP32
// basis (elem 4), one with FP64; its block partials are rows of RED_BLOCKS
inline unsigned gather_grid(long nc, int elem) {
    const long cap = elem == 4 ? 2 * 152 : 152;
    long b = (nc + RED_THREADS - 1) / RED_THREADS;
    return (unsigned)(b < cap ? (b < 1 ? 1 : b) : cap);
}

// instantiate a launch for nv = 4 or 6 (NVC is the compile-time count in __VA_ARGS__)
#define NV_SWITCH(nv, ...)                                      \
    do {                                                        \
        if ((nv) == 6) { constexpr int NVC = 6; __VA_ARGS__; } \
        else { constexpr int NVC = 4; __VA_ARGS__; }           \
    } while (0)

// ---- wall quantities and wall distance (kern_qoi.cu)
void launch_wall_distance(long nc, const double* xc, const double* yc, int nw, const double* wx, const double* wy,
                          double* d, float* d32, cudaStream_t s);
void launch_wall_coeff(int nv, int n, const int* slots, const MeshView<double>& m, const Flow<double>& F,
                       const double* U, double q_inf, double p_inf, double* cp, double* cf, double* drag,
                       cudaStream_t s);
void launch_sum_in_order(int n, const double* terms, double* out, cudaStream_t s);
void launch_entropy(int nv, long nc, const Flow<double>& F, const double* U, const double* vol, double s_ref,
                    RedScratch rs, double* out2, cudaStream_t s);
// J = sum in list order of w_k * term(face slots[k]); grad (SoA, may be null) = dJ/dU with
// the per-boundary-slot weights wslot
void launch_objective(int nv, int kind, int n, const int* slots, const double* w, const double* wslot,
                      const MeshView<double>& m, const Flow<double>& F, const double* U, double* terms, double* J,
                      double* grad, cudaStream_t s);

}  // namespace cfdg

// ---- device-resident GMRES (krylov.cuh); T = float in kern_f32.cu, double in kern_f64.cu
#include "krylov.cuh"
namespace cfdg {
// Blocks of k_gmres_prim_z: its cell blocks (grid-stride, elementwise: the count changes no
// result) and the Givens block, no more than are resident on the GPU at once at the
// kernel's register count.  A second, partial wave of cell blocks runs at a fraction of the
// SMs' memory parallelism and about doubles the kernel's time (the FP32 SST form: 77
// registers, three blocks per SM, 609 blocks at 4M cells).
template <class T, int NV>
unsigned prim_z_grid(long nc) {
    static int cap = 0;  // resident blocks on this GPU (0: not known yet)
    if (cap == 0) {
        int dev = 0, sms = 0, per = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_gmres_prim_z<T, NV>, RED_THREADS, 0) == cudaSuccess &&
            sms * per > 1)
            cap = sms * per;
        else
            cudaGetLastError();  // a failed query leaves no error behind; the grid is then
                                 // capped at RED_BLOCKS only, and the query runs again next time
    }
    long b = (nc + RED_THREADS - 1) / RED_THREADS;
    if (b > RED_BLOCKS) b = RED_BLOCKS;
    if (cap > 1 && b > cap - 1) b = cap - 1;
    if (b < 1) b = 1;
    return (unsigned)b + 1;
}

void launch_gmres_backsub(const GmresDev& d, cudaStream_t s);
// solve state and V0 = rhs / |rhs| (|rhs|^2 from *bsq, or d.beta[2] when bsq is null)
template <class T> void launch_gmres_start(long n, T* V0, const double* rhs, const GmresDev& d, int m, double tol,
                                           cudaGraphConditionalHandle h, const double* bsq, cudaStream_t s);
template <class T> void launch_gmres_dinv(int nv, long nc, const double* D, T* Dinv, cudaStream_t s);
template <class T> void launch_gmres_z(int nv, long nc, const T* V, long L, const T* Dinv, T* z, const GmresDev& d,
                                       cudaStream_t s);
template <class T> void launch_gmres_multidot(long L, const T* w, const T* V, const GmresDev& d, double* h, cudaStream_t s);
// the fused Arnoldi stages (krylov.cuh): the exact J v body's second pass of the pending
// vector + first pass of the last product + z + dual primitives (+ Givens), and its
// gather + the iteration's dots; the FD J v body's update + second pass and final
// update + norm + Givens
template <class T> void launch_gmres_prim_z(int nv, long nc, const Flow<T>& F, const T* U, T* V, long L,
                                            const T* Dinv, T* z, Field<T> W, const T* w, const GmresDev& d,
                                            cudaGraphConditionalHandle h, cudaStream_t s);
// split: the gather (k_gmres_gather_w) and the dots (k_gmres_gather_dot<..., true>) as two
// kernels, the same results bit for bit
template <class T> void launch_gmres_gather_dot(int nv, const MeshView<T>& m, const T* FA, T* w, const T* z,
                                                const T* dt, const T* src, const T* V, long L, const GmresDev& d,
                                                cudaStream_t s, bool pdl = false, bool split = false);
template <class T> void launch_gmres_update_dot(long L, T* w, const T* V, const GmresDev& d, cudaStream_t s);
template <class T> void launch_gmres_update_final(long L, const T* w, T* V, const GmresDev& d,
                                                  cudaGraphConditionalHandle h, cudaStream_t s);
template <class T> void launch_gmres_solution_dev(int nv, long nc, const T* V, long L, const GmresDev& d,
                                                  const double* D, const T* Dinv32, double* x, cudaStream_t s);
}  // namespace cfdg

// ---- one Arnoldi iteration as one persistent kernel (arnoldi.cuh, kern_jv.cu)
namespace cfdg {
template <class T> struct ArnoldiArgs;
// blocks that can be resident at once (at most RED_BLOCKS)
template <class T> int arnoldi_blocks(int nv);
// launch (cooperative when coop); returns the launch's error
template <class T> cudaError_t launch_arnoldi(int nv, const ArnoldiArgs<T>& a, cudaGraphConditionalHandle h,
                                              int blocks, bool coop, cudaStream_t s);
}  // namespace cfdg

// ---- adjoint of the FP64 residual (kern_adj.cu); a.phi receives the recomputed limiter
namespace cfdg {
struct AdjBufs;
void launch_vjp64(const ResArgs<double>& a, const double* lam, const AdjBufs& b, double* gU);
}  // namespace cfdg
