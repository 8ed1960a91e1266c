// Host side of libcfdgpu: the solver handle, device buffers, the GMRES and
// pseudo-transient Newton drivers, and the C ABI declared in include/cfdg.h.
//
// All arithmetic on vectors and states runs in the CUDA kernels (kern_*.cu).  The host
// keeps only what the reference keeps in scalars: the Hessenberg matrix, the Givens
// rotations and the CFL / relaxation logic of solveGMRES and solveImplicit
// (AmberMond/mycode src/Solver.cpp:1472-1618, :1696-1799), evaluated with the same
// expressions so the Newton trace follows the reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cfdg.h"
#include "adjoint_kernels.cuh"
#include "arnoldi.cuh"
#include "launch.hpp"
#include "mesh.hpp"

using namespace cfdg;

struct cfdg_mesh {
    HostMesh h;
};

namespace {

thread_local std::string g_err;

cfdg_status fail(cfdg_status st, const std::string& msg) {
    g_err = msg;
    return st;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define TRY(expr)                          \
    do {                                   \
        cfdg_status st_ = (expr);          \
        if (st_ != CFDG_OK) return st_;    \
    } while (0)

template <class T>
cfdg_status dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    CK(cudaMalloc((void**)p, n * sizeof(T)));
    CK(cudaMemset(*p, 0, n * sizeof(T)));
    return CFDG_OK;
}

template <class R>
struct GeoBuf {
    R *nx = nullptr, *ny = nullptr, *area = nullptr, *dxo = nullptr, *dyo = nullptr, *dxn = nullptr, *dyn = nullptr,
      *dxlr = nullptr, *dylr = nullptr, *vol = nullptr, *d2lr = nullptr, *id2lr = nullptr, *ivol = nullptr;
    void release() {
        R* a[] = {nx, ny, area, dxo, dyo, dxn, dyn, dxlr, dylr, vol, d2lr, id2lr, ivol};
        for (R* p : a) cudaFree(p);
    }
};

template <class R>
cfdg_status upload_geo(GeoBuf<R>& g, const HostMesh& h) {
    const std::vector<double>* src[] = {&h.nx, &h.ny, &h.area, &h.dxo, &h.dyo, &h.dxn, &h.dyn, &h.dxlr, &h.dylr, &h.vol};
    R** dst[] = {&g.nx, &g.ny, &g.area, &g.dxo, &g.dyo, &g.dxn, &g.dyn, &g.dxlr, &g.dylr, &g.vol};
    for (int k = 0; k < 10; ++k) {
        std::vector<R> tmp(src[k]->begin(), src[k]->end());
        TRY(dalloc(dst[k], tmp.size()));
        CK(cudaMemcpy(*dst[k], tmp.data(), tmp.size() * sizeof(R), cudaMemcpyHostToDevice));
    }
    // mesh invariants the kernels would otherwise form on every evaluation, with their
    // expressions in R (host code without contraction: the FP64 values have the bits of the
    // kernels' own FP64 arithmetic): |x_R - x_L|^2 and its reciprocal per face, 1 / vol per
    // cell
    const size_t nf = h.dxlr.size(), nc = h.vol.size();
    std::vector<R> d2(nf), id2(nf), iv(nc);
    for (size_t f = 0; f < nf; ++f) {
        FaceGeo<R> g;
        g.dxlr = (R)h.dxlr[f];
        g.dylr = (R)h.dylr[f];
        geo_derived(g);
        d2[f] = g.d2lr;
        id2[f] = g.id2lr;
    }
    for (size_t c = 0; c < nc; ++c) iv[c] = R(1) / (R)h.vol[c];
    TRY(dalloc(&g.d2lr, nf));
    TRY(dalloc(&g.id2lr, nf));
    TRY(dalloc(&g.ivol, nc));
    CK(cudaMemcpy(g.d2lr, d2.data(), nf * sizeof(R), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.id2lr, id2.data(), nf * sizeof(R), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g.ivol, iv.data(), nc * sizeof(R), cudaMemcpyHostToDevice));
    return CFDG_OK;
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

namespace cfdg {
// interior faces from which the FP64 residual forms the gradient's face terms once per face
// (k_grad_faces64); below, the per-cell gradient forms them on each side
constexpr int GRAD_FACE_TERMS_MIN_FACES = 100000;
// lets other translation units of the library report through cfdg_last_error()
void set_error_message(const std::string& msg) { g_err = msg; }
}  // namespace cfdg

struct cfdg_solver {
    const cfdg_mesh* mesh = nullptr;
    cfdg_config cfg;
    int nv = 4, nc = 0, nf = 0;
    long L = 0;  // nv * nc
    cudaStream_t st = nullptr;
    // flow parameters (Solver members, include/Solver.hpp:37-39, :93-95)
    double M_inf = 0, P0 = 0, T0 = 0, Pexit = 0, nu = 0.01;
    Flow<double> F;
    Flow<float> Ff;
    // device mesh
    int *cf = nullptr, *fo = nullptr, *fn = nullptr, *ftag = nullptr, *perm = nullptr;
    int* iperm = nullptr;  // [nc] caller cell -> internal cell (the inverse of perm)
    double* gft = nullptr; // [2 x primitives][nfi] the FP64 gradient's per-face terms (k_grad_faces64)
    GeoBuf<double> g64;
    GeoBuf<float> g32;
    // per-cell neighbours and FP32 face geometry for the mixed solve's dual gradient
    // (CellFaces, residual.cuh); mixed precision only
    int* cfx_nbr = nullptr;
    float* cfx_geo = nullptr;  // [3][4][nc]: nx, ny, area
    CellFaces<float> cfx32{nullptr, nullptr, nullptr, nullptr};
    MeshView<double> mv;
    MeshView<float> mvf;
    // FP64 state and work
    double *U = nullptr, *W = nullptr, *G = nullptr, *phi = nullptr, *FA = nullptr, *R = nullptr, *dt = nullptr,
           *D = nullptr;
    double *stage = nullptr;   // AoS staging, 14 doubles per cell
    double *Ub = nullptr, *Rb = nullptr, *Up = nullptr, *Rp = nullptr, *vtmp = nullptr, *x = nullptr, *rhs = nullptr;
    // dual (exact J v) work, FP64
    double *Wj = nullptr, *Wjd = nullptr, *Gj = nullptr, *Gjd = nullptr, *FAjd = nullptr;
    // SST (nv = 6): cell terms (mu_t, F1, S_k vol, S_w vol) and the wall distance
    double *Tt = nullptr, *Tj = nullptr, *Tjd = nullptr, *dwall = nullptr;
    float *T32 = nullptr, *T32d = nullptr, *dwall32 = nullptr;
    // FP32 (mixed precision) work
    float *U32 = nullptr, *W32 = nullptr, *W32d = nullptr, *G32 = nullptr, *G32d = nullptr, *FA32d = nullptr,
          *phi32 = nullptr, *dt32 = nullptr, *V32 = nullptr, *z32 = nullptr;
    // Krylov basis FP64, and 1/D of the solve in the basis precision
    double *V = nullptr, *z = nullptr, *dinv64 = nullptr;
    float* dinv32 = nullptr;
    int m_alloc = 0;
    // device-resident GMRES (graph with a WHILE node)
    GmresDev gd{};
    int* gdi = nullptr;
    double* gdd = nullptr;
    float* w32 = nullptr;
    double* w64 = nullptr;
    cudaGraphExec_t gexec = nullptr;
    const void* gkey[4] = {nullptr, nullptr, nullptr, nullptr};
    bool gnewton = false;  // the graph was built for a Newton step (newton_chain; enqueue_gmres_pre)
    int flow_version = 0, graph_version = -1;
    bool capturing = false;
    bool pdl_failed = false;  // the body would not build with programmatic dependent launch
    long long graph_pre = 0, graph_body = 0, graph_post = 0;
    // reductions
    RedScratch rs{nullptr, nullptr};
    double* scal = nullptr;  // [0] |U|^2 [1] |z|^2 [2] eps [3] beta^2 [4..6] vm [8..] H columns, y
    int* bad = nullptr;
    // Newton driver state
    double cfl = 0.1;
    int step = 0;
    bool limiter_valid = false;
    // instrumentation: CUDA events around the four stages of every residual (stat
    // classes 0-3: primitives, gradients with their face terms and SST cell terms, face
    // flux, gather) and exact J v (4-7) evaluation, resolved at the next stream sync
    int timing = 0;
    std::vector<cudaEvent_t> pool;
    size_t pool_used = 0;
    std::vector<std::pair<int, std::pair<size_t, int>>> pending;
    // classes 8-11: the VJP's forward recomputation, face adjoint, cell gathers 1 and 2
    // classes 12-17: the fused Krylov body (stream driver): second and first passes + z +
    // primitives, gradients (+ SST terms), face fluxes, gather + dots; 16-17 the FD body's
    // update + second pass and final update (not timed)
    static constexpr int NSTAT = 18;
    double kstat_ms[NSTAT] = {};
    long long kstat_n[NSTAT] = {};
    // adjoint work buffers (allocated on the first VJP)
    AdjBufs ab{};
    double* adj_mem = nullptr;
    int* adj_imem = nullptr;
    double* phi_adj = nullptr;
    float kms[4] = {0, 0, 0, 0};
    cudaEvent_t step_ev[4] = {nullptr, nullptr, nullptr, nullptr};  // step start/end, Krylov start/end
    long long launches = 0;
    unsigned char* l2buf = nullptr;
    size_t l2bytes = 0;
    int l2fill = 0;

    // nint + 1 events bracketing nint consecutive kernels of stat classes base..base+nint-1
    cudaEvent_t* take_events(int base, int nint = 4) {
        // per-kernel events at timing level 1 only; event nodes are not allowed in graph bodies
        if (timing != 1 || capturing) return nullptr;
        while (pool_used + nint + 1 > pool.size()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            pool.push_back(e);
        }
        pending.push_back({base, {pool_used, nint}});
        cudaEvent_t* e = &pool[pool_used];
        pool_used += nint + 1;
        return e;
    }

    // call only after the stream has been synchronised
    void collect() {
        for (auto& p : pending) {
            const size_t i0 = p.second.first;
            const int nint = p.second.second;
            for (int k = 0; k < nint; ++k) {
                float ms = 0;
                cudaEventElapsedTime(&ms, pool[i0 + k], pool[i0 + k + 1]);
                kstat_ms[p.first + k] += ms;
                ++kstat_n[p.first + k];
                if (p.first == 0 && k < 4) kms[k] = ms;
            }
        }
        pending.clear();
        pool_used = 0;
    }

    double* hcol(int j) { return scal + 16 + (size_t)j * (cfg.gmres_m + 2); }
    double* ydev() { return scal + 16 + (size_t)(cfg.gmres_m + 1) * (cfg.gmres_m + 2); }

    Field<double> f64(double* v, double* d = nullptr) { return Field<double>{v, d, nc}; }
    Field<double> ff64(double* v, double* d = nullptr) { return Field<double>{v, d, nf}; }
    Field<float> f32(float* v, float* d = nullptr) { return Field<float>{v, d, nc}; }
    Field<float> ff32(float* v, float* d = nullptr) { return Field<float>{v, d, nf}; }

    void set_flow() {
        F.gam = cfg.gamma;
        F.Rgas = cfg.R_gas;
        F.Pr = cfg.Pr;
        F.nu = nu;
        F.Minf = M_inf;
        F.P0 = P0;
        F.T0 = T0;
        F.Pexit = Pexit;
        F.bcset = cfg.bcset;
        F.flux = cfg.flux;
        F.spatial = cfg.spatial;
        F.viscous = cfg.viscous;
        ++flow_version;
        // frozen free stream, same expressions as src/Solver.cpp:979-985 (host IEEE
        // arithmetic without contraction gives the device's values)
        double g = cfg.gamma, M = M_inf;
        double fT = 1.0 + 0.5 * (g - 1.0) * M * M;
        double Ts = T0 / fT;
        double rho = Pexit / (cfg.R_gas * Ts);
        double c = std::sqrt(g * cfg.R_gas * Ts);
        double u = M * c;
        double rE = Pexit / (g - 1.0) + 0.5 * rho * (u * u + 0.0 * 0.0);
        F.fs[0] = rho;
        F.fs[1] = rho * u;
        F.fs[2] = rho * 0.0;
        F.fs[3] = rE;
        for (int k = 0; k < 4; ++k) F.shock[k] = F.fs[k];
        if (cfg.shock_deflection_deg > 0.0 && M > 1.0) post_shock(F.shock, rho, u, Pexit, g);
        F.sst = nv == 6 ? 1 : 0;
        F.k_inf = 0;
        F.w_inf = 0;
        if (F.sst) {
            // k = 1.5 (Tu U)^2, w = k / (nu mu_t/mu) from the configured intensity and ratio
            double kk, ww;
            sst_freestream(cfg.turb_intensity, cfg.mut_ratio, u, nu, kk, ww);
            F.k_inf = kk;
            F.w_inf = ww;
        }
        F.Pr_t = 0.9;
        // correctly rounded reciprocals and quotients (host IEEE division) for the kernels
        flow_derived(F);
        Ff.gam = (float)F.gam; Ff.Rgas = (float)F.Rgas; Ff.Pr = (float)F.Pr; Ff.nu = (float)F.nu;
        Ff.Minf = (float)F.Minf; Ff.P0 = (float)F.P0; Ff.T0 = (float)F.T0; Ff.Pexit = (float)F.Pexit;
        for (int k = 0; k < 4; ++k) { Ff.fs[k] = (float)F.fs[k]; Ff.shock[k] = (float)F.shock[k]; }
        Ff.k_inf = (float)F.k_inf; Ff.w_inf = (float)F.w_inf; Ff.Pr_t = (float)F.Pr_t;
        flow_derived(Ff);
        Ff.bcset = F.bcset; Ff.flux = F.flux; Ff.spatial = F.spatial; Ff.viscous = F.viscous; Ff.sst = F.sst;
    }

    // state behind an oblique shock of deflection theta (theta-beta-M relation, weak branch)
    void post_shock(double* out, double rho1, double u1, double p1, double g) {
        double M1 = M_inf, th = cfg.shock_deflection_deg * M_PI / 180.0;
        double beta = std::asin(1.0 / M1) + 1e-6, best = beta;
        for (int it = 0; it < 200000; ++it) {
            double b = std::asin(1.0 / M1) + it * (M_PI / 2 - std::asin(1.0 / M1)) / 200000.0;
            double t = std::atan(2.0 / std::tan(b) * (M1 * M1 * std::sin(b) * std::sin(b) - 1.0) /
                                 (M1 * M1 * (g + std::cos(2 * b)) + 2.0));
            if (t >= th) { best = b; break; }
        }
        beta = best;
        double Mn1 = M1 * std::sin(beta);
        double r2 = rho1 * (g + 1) * Mn1 * Mn1 / ((g - 1) * Mn1 * Mn1 + 2);
        double p2 = p1 * (1 + 2 * g / (g + 1) * (Mn1 * Mn1 - 1));
        double un1 = u1 * std::sin(beta), ut = u1 * std::cos(beta);
        double un2 = un1 * rho1 / r2;
        // flow turned by -theta (downwards) behind a shock from the upper boundary
        double V2 = std::sqrt(un2 * un2 + ut * ut);
        double ux = V2 * std::cos(th), uy = -V2 * std::sin(th);
        out[0] = r2;
        out[1] = r2 * ux;
        out[2] = r2 * uy;
        out[3] = p2 / (g - 1) + 0.5 * r2 * (ux * ux + uy * uy);
    }

    ResArgs<double> res64(double* Uin, double* out, int do_lim) {
        ResArgs<double> a;
        a.m = mv;
        a.F = F;
        a.nv = nv;
        a.U = f64(Uin);
        a.W = f64(W);
        a.G = f64(G);
        a.FA = ff64(FA);
        a.T = f64(Tt);
        a.dwall = dwall;
        a.phi = phi;
        a.out = out;
        a.do_limiter = do_lim;
        a.diag_v = nullptr;
        a.dt = nullptr;
        a.stream = st;
        a.ev = nullptr;
        a.gft = gft;
        return a;
    }

    // kernels of one FP64 residual (launch_residual<double>)
    int res64_kernels() const { return (nv == 6 ? 5 : 4) + (gft && mv.nfi > 0 ? 1 : 0); }

    // norms (a Newton step): the gather also writes rhs = -R, the norm pieces and |R|^2 into
    // scal[8..11] and clears the update's non-finite flag (k_gather_norms; `flag`, default
    // bad).  lim_dev: the limiter is recomputed only where *lim_dev is also set (a chained
    // Newton step, whose limiter-freeze decision is taken on the device).
    // prim_done: W already holds Uin's primitives (launch_rows_prim); rows_out: the gather
    // writes the residual into a caller's pinned rows in place (device-visible address)
    cfdg_status residual_dev(double* Uin, double* out, int update_limiters, bool norms = false, int* flag = nullptr,
                             const int* lim_dev = nullptr, bool prim_done = false, double* rows_out = nullptr) {
        int do_lim = (cfg.spatial == CFDG_SECOND_ORDER_LIMITED && update_limiters) ? 1 : 0;
        ResArgs<double> a = res64(Uin, out, do_lim);
        if (norms) {
            a.rhs_out = rhs;
            a.norms_out = scal + 8;
            a.flag = flag ? flag : bad;
            a.rs = rs;
        }
        a.lim_dev = lim_dev;
        a.prim_done = prim_done;
        a.rows_out = rows_out;
        a.iperm = iperm;
        a.ev = take_events(0);
        launch_residual<double>(a);
        launches += res64_kernels() - (prim_done ? 1 : 0);
        if (do_lim) limiter_valid = true;
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    // Device-visible address of a caller's page-locked host buffer, nullptr when it is
    // pageable.  Pinned buffers are read and written in place by the row kernels
    // (residual.cuh rows_load / rows_store) over the CPU-GPU link; pageable ones go through
    // the device staging buffer and a copy.
    static double* mapped(const void* host) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
        return static_cast<double*>(a.devicePointer);
    }

    // A caller's AoS array (reference numbering, 6 per cell) into np SoA planes (new
    // numbering); only enqueues (the entry point synchronises before it returns)
    cfdg_status upload_aos(const double* host, double* dev_soa, int np = -1) {
        if (np < 0) np = nv;
        if (double* hp = mapped(host)) {
            launch_rows_to_soa(nc, np, 6, hp, iperm, dev_soa, st);
        } else {
            CK(cudaMemcpyAsync(stage, host, sizeof(double) * 6 * (size_t)nc, cudaMemcpyHostToDevice, st));
            launch_aos_to_soa<double>(nc, np, 6, stage, perm, dev_soa, st);
        }
        ++launches;
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    // np SoA planes into a caller's AoS array (stride doubles per cell, zeros past np)
    cfdg_status download_aos(const double* dev_soa, double* host, int np, int stride) {
        double* hp = stride <= ROW_MAX_STRIDE ? mapped(host) : nullptr;
        if (hp) {
            launch_soa_to_rows<double>(nc, np, stride, dev_soa, iperm, hp, st);
        } else {
            launch_soa_to_aos<double>(nc, np, stride, dev_soa, perm, stage, st);
            CK(cudaMemcpyAsync(host, stage, sizeof(double) * stride * (size_t)nc, cudaMemcpyDeviceToHost, st));
        }
        ++launches;
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        collect();
        return CFDG_OK;
    }

    cfdg_status download_aos32(const float* dev_soa, double* host) {
        if (double* hp = mapped(host)) {
            launch_soa_to_rows<float>(nc, nv, 6, dev_soa, iperm, hp, st);
        } else {
            launch_soa_to_aos<float>(nc, nv, 6, dev_soa, perm, stage, st);
            CK(cudaMemcpyAsync(host, stage, sizeof(double) * 6 * (size_t)nc, cudaMemcpyDeviceToHost, st));
        }
        ++launches;
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        collect();
        return CFDG_OK;
    }

    // ---- FP32 entry points (the mixed-precision kernels on their own; mixed solvers only)
    // own FP32 direction and output vectors (the Krylov basis and its z are allocated
    // only with the first GMRES solve)
    float* f32out = nullptr;
    float* f32dir = nullptr;

    cfdg_status need_f32() {
        if (cfg.precision != CFDG_MIXED) return fail(CFDG_ERR_UNSUPPORTED, "FP32 entry points need precision = mixed");
        if (!f32out) TRY(dalloc(&f32out, (size_t)L));
        if (!f32dir) TRY(dalloc(&f32dir, (size_t)L));
        return CFDG_OK;
    }

    // FP32 residual of Ubase (limiter recomputed in FP32 for the limited scheme) into f32out
    cfdg_status residual32_dev(double* Ubase) {
        TRY(need_f32());
        launch_convert<float>(L, Ubase, U32, st);
        ResArgs<float> a;
        a.m = mvf;
        a.cfx = cfx32;
        a.F = Ff;
        a.nv = nv;
        a.U = f32(U32);
        a.W = f32(W32);
        a.G = f32(G32);
        a.FA = ff32(FA32d);
        a.T = f32(T32);
        a.dwall = dwall32;
        a.phi = phi32;
        a.out = f32out;
        a.do_limiter = cfg.spatial == CFDG_SECOND_ORDER_LIMITED ? 1 : 0;
        a.diag_v = nullptr;
        a.dt = nullptr;
        a.stream = st;
        a.ev = take_events(0);
        launch_residual<float>(a);
        launches += 1 + (nv == 6 ? 5 : 4);
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    // FP32 exact J v (dual numbers, limiter frozen at the FP64 phi, time term with dt) of
    // direction vdev about Ubase into f32out
    cfdg_status jv32_dev(double* Ubase, double* vdev) {
        TRY(need_f32());
        launch_convert<float>(L, Ubase, U32, st);
        launch_convert<float>(nc, phi, phi32, st);
        launch_convert<float>(nc, dt, dt32, st);
        launch_convert<float>(L, vdev, f32dir, st);
        ResArgs<float> a;
        a.m = mvf;
        a.cfx = cfx32;
        a.F = Ff;
        a.nv = nv;
        a.U = f32(U32, f32dir);
        a.W = f32(W32, W32d);
        a.G = f32(G32, G32d);
        a.FA = ff32(nullptr, FA32d);
        a.T = f32(T32, T32d);
        a.dwall = dwall32;
        a.phi = phi32;
        a.out = f32out;
        a.do_limiter = 0;
        a.diag_v = f32dir;
        a.dt = dt32;
        a.stream = st;
        a.ev = take_events(4);
        launch_jv<float>(a);
        launches += 4 + (nv == 6 ? 5 : 4);
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    cfdg_status read_scalars(int first, int n, double* out) {
        CK(cudaMemcpyAsync(out, scal + first, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        collect();
        return CFDG_OK;
    }

    // J v at Ub (FD about (Ub, Rb), or exact).  v, out FP64 device vectors.
    cfdg_status jv64(double* Ubase, double* Rbase, double* v, double* out, int mode, bool have_usq) {
        if (mode == CFDG_JV_FD) {
            if (!have_usq) { launch_dot<double>(nv, nc, Ubase, Ubase, rs, scal + 0, st); ++launches; }
            launch_dot<double>(nv, nc, v, v, rs, scal + 1, st);
            launch_fd_perturb(L, Ubase, v, scal + 0, scal + 1, Up, scal + 2, st);
            launches += 2;
            TRY(residual_dev(Up, Rp, 0));
            launch_fd_combine(nv, nc, Rp, Rbase, v, scal + 2, g64.vol, dt, out, st);
            ++launches;
        } else {
            ResArgs<double> a;
            a.m = mv;
            a.F = F;
            a.nv = nv;
            a.U = f64(Ubase, v);
            a.W = f64(Wj, Wjd);
            a.G = f64(Gj, Gjd);
            a.FA = ff64(nullptr, FAjd);
            a.T = f64(Tj, Tjd);
            a.dwall = dwall;
            a.phi = phi;
            a.out = out;
            a.do_limiter = 0;
            a.diag_v = v;
            a.dt = dt;
            a.stream = st;
            a.ev = take_events(4);
            launch_jv<double>(a);
            launches += nv == 6 ? 5 : 4;
        }
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    cfdg_status ensure_krylov() {
        int m = cfg.gmres_m;
        if (m_alloc >= m) return CFDG_OK;
        cudaFree(V); cudaFree(z); cudaFree(V32); cudaFree(z32); cudaFree(dinv32); cudaFree(dinv64);
        V = nullptr; z = nullptr; V32 = nullptr; z32 = nullptr; dinv32 = nullptr; dinv64 = nullptr;
        const size_t nd = (size_t)(nv == 6 ? 3 : 1) * nc;
        if (cfg.precision == CFDG_MIXED) {
            TRY(dalloc(&V32, (size_t)(m + 1) * L));
            TRY(dalloc(&z32, (size_t)L));
            TRY(dalloc(&dinv32, nd));
        } else {
            TRY(dalloc(&V, (size_t)(m + 1) * L));
            TRY(dalloc(&z, (size_t)L));
            TRY(dalloc(&dinv64, nd));
        }
        if (!bar) {
            // persistent Arnoldi kernel: barrier words and three sets of block partials
            TRY(dalloc(&bar, 4));
            TRY(dalloc(&apart, (2 * (size_t)(KRY_MAXM + 1) + 1) * RED_BLOCKS));
        }
        if (!chain_ctl) {
            TRY(dalloc(&chain_ctl, 4 + (size_t)CHAIN_MAX));
            TRY(dalloc(&chain_rec, (size_t)NEWTON_REC * CHAIN_MAX));
            CK(cudaMallocHost((void**)&chain_h, sizeof(double) * CHAIN_HOST_DOUBLES));
        }
        m_alloc = m;
        return CFDG_OK;
    }

    // a grid barrier of the persistent kernel gave up: reset its words, report
    cfdg_status barrier_timeout() {
        CK(cudaMemsetAsync(bar, 0, 4 * sizeof(unsigned), st));
        CK(cudaStreamSynchronize(st));
        return fail(CFDG_ERR_TIMEOUT, "a grid barrier of the persistent Arnoldi kernel timed out "
                                      "(its blocks were not all resident); set persistent = 0");
    }

    // the persistent Arnoldi kernel (arnoldi.cuh) replaces the fused four-kernel body in
    // the graph driver for the exact J v; grid = the blocks that fit at once
    unsigned* bar = nullptr;
    double* apart = nullptr;
    int ablocks = 0;
    bool use_persistent() const {
        return cfg.persistent && cfg.krylov == CFDG_KRYLOV_GRAPH &&
               (cfg.precision == CFDG_MIXED || cfg.jv == CFDG_JV_EXACT);
    }
    template <class T>
    ArnoldiArgs<T> arnoldi_args(const MeshView<T>& m, const Flow<T>& Fx, const T* Ub, T* zz, Field<T> Wf, Field<T> Gf,
                                Field<T> FAf, Field<T> Tf, const T* dw, const T* ph, const T* dtx, const T* di, T* ww,
                                T* VV) {
        ArnoldiArgs<T> a;
        a.m = m;
        a.F = Fx;
        a.U = Ub;
        a.z = zz;
        a.W = Wf;
        a.G = Gf;
        a.FA = FAf;
        a.Tsst = Tf;
        a.dwall = dw;
        a.phi = ph;
        a.dt = dtx;
        a.Dinv = di;
        a.w = ww;
        a.V = VV;
        a.L = L;
        a.d = gd;
        a.part = apart;
        a.bar = GridBar{bar, bar + 1, reinterpret_cast<int*>(bar + 2),
                        cfg.barrier_poll_limit > 0 ? (unsigned)cfg.barrier_poll_limit : (1u << 24)};
        return a;
    }

    // ---- adjoint: gU = (dR/dU)^T lam at Uin, limiter recomputed into a scratch buffer
    cfdg_status ensure_adj() {
        if (adj_mem) return CFDG_OK;
        const int N = nv == 6 ? AdjSlot<6>::N : AdjSlot<4>::N;
        const int NG = nv == 6 ? 14 : 10;
        size_t nd = 2 * (size_t)N * nf + (size_t)nv * nc + (size_t)NG * nc + 2 * (size_t)nc;
        TRY(dalloc(&adj_mem, nd));
        TRY(dalloc(&adj_imem, 2 * (size_t)nc));
        TRY(dalloc(&phi_adj, (size_t)nc));
        double* q = adj_mem;
        ab.fb0 = q; q += (size_t)N * nf;
        ab.fb1 = q; q += (size_t)N * nf;
        ab.gpart = q; q += (size_t)nv * nc;
        ab.accb = q; q += (size_t)NG * nc;
        ab.pmaxb = q; q += nc;
        ab.pminb = q;
        ab.pmax_face = adj_imem;
        ab.pmin_face = adj_imem + nc;
        return CFDG_OK;
    }

    cfdg_status vjp_dev(double* Uin, double* lam, double* gout) {
        TRY(ensure_adj());
        ResArgs<double> a = res64(Uin, nullptr, 0);
        a.phi = phi_adj;
        a.ev = take_events(8);
        launch_vjp64(a, lam, ab, gout);
        launches += (nv == 6 ? 6 : 5) + (gft && mv.nfi > 0 ? 1 : 0);
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    // ---- device-resident GMRES: one graph per (Ubase, Rbase, rhs, x, flow parameters)

    // preconditioner, FP32 copies, beta and V0 (graph prologue).  In a Newton step's graph
    // (newton) the primitives W of U are current (the step's residual computed them), the
    // step's reduction kernel has put |rhs|^2 in scal[11], and the mixed path takes its
    // local time step from the CFL number in scal[12]; otherwise dt is the caller's.
    void enqueue_gmres_pre(double* Ubase, double* rhsd, cudaGraphConditionalHandle h, bool newton) {
        const bool mixed = cfg.precision == CFDG_MIXED;
        if (!newton) {
            launch_prim64(nv, nc, F, f64(U), f64(W), st);
            ++launches;
        }
        if (mixed) {
            launch_mixed_pre(nv, mvf, Ff, U, Ubase, W, phi, nv == 6 ? Tt : nullptr, newton ? scal + 12 : nullptr, dt,
                             U32, phi32, dt32, D, dinv32, st);
            // the value planes of the FP32 linearisation point, once per solve: the Arnoldi
            // body's dual kernels then form and write derivative planes only
            ResArgs<float> a;
            a.m = mvf;
            a.cfx = cfx32;
            a.F = Ff;
            a.nv = nv;
            a.U = f32(U32);
            a.W = f32(W32);
            a.G = f32(G32);
            a.T = f32(T32);
            a.dwall = dwall32;
            a.phi = phi32;
            a.stream = st;
            launch_values<float>(a);
            launches += nv == 6 ? 3 : 2;
        } else {
            launch_precond(nv, mv, F, U, W, dt, D, Tt, st);
            launch_gmres_dinv<double>(nv, nc, D, dinv64, st);
            launches += 2;
            if (cfg.jv == CFDG_JV_FD) {
                launch_dot<double>(nv, nc, Ubase, Ubase, rs, scal + 0, st);
                ++launches;
            }
        }
        if (!newton) {
            launch_dot<double>(nv, nc, rhsd, rhsd, rs, gd.beta + 2, st);
            ++launches;
        }
        if (mixed) launch_gmres_start<float>(L, V32, rhsd, gd, cfg.gmres_m, cfg.gmres_tol, h, newton ? scal + 11 : nullptr, st);
        else launch_gmres_start<double>(L, V, rhsd, gd, cfg.gmres_m, cfg.gmres_tol, h, newton ? scal + 11 : nullptr, st);
        ++launches;
    }

    // one Arnoldi iteration (graph WHILE body)
    cfdg_status enqueue_gmres_body(double* Ubase, double* Rbase, cudaGraphConditionalHandle h) {
        const bool mixed = cfg.precision == CFDG_MIXED;
        // the exact (dual-number) J v runs fused with the Arnoldi kernels: z with the
        // primitives, the gather with the first CGS pass; the FD J v keeps its own kernels.
        if (use_persistent() && capturing) {
            if (!ablocks) ablocks = mixed ? arnoldi_blocks<float>(nv) : arnoldi_blocks<double>(nv);
            cudaError_t e;
            if (mixed)
                e = launch_arnoldi<float>(nv, arnoldi_args<float>(mvf, Ff, U32, z32, f32(W32, W32d), f32(G32, G32d),
                                                                   ff32(nullptr, FA32d), f32(T32, T32d), dwall32, phi32,
                                                                   dt32, dinv32, w32, V32),
                                          h, ablocks, false, st);
            else
                e = launch_arnoldi<double>(nv, arnoldi_args<double>(mv, F, Ubase, z, f64(Wj, Wjd), f64(Gj, Gjd),
                                                                     ff64(nullptr, FAjd), f64(Tj, Tjd), dwall, phi, dt,
                                                                     dinv64, w64, V),
                                           h, ablocks, false, st);
            if (e != cudaSuccess) return fail(CFDG_ERR_CUDA, std::string("Arnoldi kernel: ") + cudaGetErrorString(e));
            ++launches;
            return CFDG_OK;
        }
        // ev (stream driver with timing): 5 events around the 4 stages, stat classes 12-15
        cudaEvent_t* ev = (mixed || cfg.jv == CFDG_JV_EXACT) ? take_events(12, 4) : nullptr;
        // programmatic dependent launch for the kernels after the first (pdl.cuh); not
        // with per-kernel events, which time each kernel alone
        const bool pdl = cfg.pdl && !ev && !pdl_failed;
        // a graph body holds body_unroll() iterations (the kernels of the iterations after
        // the finishing one return at once)
        const int reps = capturing && (mixed || cfg.jv == CFDG_JV_EXACT) ? body_unroll() : 1;
        for (int rep = 0; rep < reps; ++rep) TRY(enqueue_arnoldi_iteration(Ubase, Rbase, h, ev, pdl));
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    int body_unroll() const { return KRY_BODY_ITERS; }
    // the exact J v body's gather and dots as two kernels (cfdg_config.gather_split_cells)
    bool gather_split() const {
        const long t = cfg.gather_split_cells == 0 ? KRY_SPLIT_GATHER_CELLS : (long)cfg.gather_split_cells;
        return t > 0 && (long)nc >= t;
    }
    // WHILE-body executions of a graph solve of `iters` iterations
    long long body_runs(int iters) const {
        if (use_persistent() || !(cfg.precision == CFDG_MIXED || cfg.jv == CFDG_JV_EXACT)) return iters;
        // the exact J v body runs twice more than the iterations: the column of iteration
        // j is final after the product of iteration j + 1, and its Givens step runs in the
        // first kernel of iteration j + 2
        const int u = body_unroll();
        return (iters + 2 + u - 1) / u;
    }

    cfdg_status enqueue_arnoldi_iteration(double* Ubase, double* Rbase, cudaGraphConditionalHandle h,
                                          cudaEvent_t* ev, bool pdl) {
        const bool mixed = cfg.precision == CFDG_MIXED;
        if (ev) CK(cudaEventRecord(ev[0], st));
        if (mixed) {
            launch_gmres_prim_z<float>(nv, nc, Ff, U32, V32, L, dinv32, z32, f32(nullptr, W32d), w32, gd, h, st);
            ResArgs<float> a;
            a.m = mvf;
            a.cfx = cfx32;
            a.F = Ff;
            a.nv = nv;
            a.U = f32(U32, z32);
            a.W = f32(W32, W32d);
            a.G = f32(G32, G32d);
            a.FA = ff32(nullptr, FA32d);
            a.T = f32(T32, T32d);
            a.dwall = dwall32;
            a.phi = phi32;
            a.stream = st;
            a.ev = ev ? ev + 1 : nullptr;
            a.pdl = pdl;
            a.done = gd.gi + 2;
            a.tangent = true;
            launch_jv_mid<float>(a);
            launch_gmres_gather_dot<float>(nv, mvf, FA32d, w32, z32, dt32, nv == 6 ? T32d + 2 * nc : nullptr, V32, L, gd,
                                           st, pdl, gather_split());
            if (ev) CK(cudaEventRecord(ev[4], st));
            launches += (nv == 6 ? 5 : 4) + (gather_split() ? 1 : 0);
        } else if (cfg.jv == CFDG_JV_EXACT) {
            launch_gmres_prim_z<double>(nv, nc, F, Ubase, V, L, dinv64, z, f64(Wj, Wjd), w64, gd, h, st);
            ResArgs<double> a;
            a.m = mv;
            a.F = F;
            a.nv = nv;
            a.U = f64(Ubase, z);
            a.W = f64(Wj, Wjd);
            a.G = f64(Gj, Gjd);
            a.FA = ff64(nullptr, FAjd);
            a.T = f64(Tj, Tjd);
            a.dwall = dwall;
            a.phi = phi;
            a.stream = st;
            a.ev = ev ? ev + 1 : nullptr;
            a.pdl = pdl;
            a.done = gd.gi + 2;
            launch_jv_mid<double>(a);
            launch_gmres_gather_dot<double>(nv, mv, FAjd, w64, z, dt, nv == 6 ? Tjd + 2 * nc : nullptr, V, L, gd, st,
                                            pdl, gather_split());
            if (ev) CK(cudaEventRecord(ev[4], st));
            launches += (nv == 6 ? 5 : 4) + (gather_split() ? 1 : 0);
        } else {
            launch_gmres_z<double>(nv, nc, V, L, dinv64, z, gd, st);
            ++launches;
            TRY(jv64(Ubase, Rbase, z, w64, cfg.jv, true));
            launch_gmres_multidot<double>(L, w64, V, gd, gd.h1, st);
            launch_gmres_update_dot<double>(L, w64, V, gd, st);
            launch_gmres_update_final<double>(L, w64, V, gd, h, st);
            launches += 3;
        }
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    void enqueue_gmres_post(double* xout) {
        launch_gmres_backsub(gd, st);
        if (cfg.precision == CFDG_MIXED) launch_gmres_solution_dev<float>(nv, nc, V32, L, gd, D, dinv32, xout, st);
        else launch_gmres_solution_dev<double>(nv, nc, V, L, gd, D, nullptr, xout, st);
        launches += 2;
    }

    cfdg_status build_gmres_graph(double* Ubase, double* Rbase, double* rhsd, double* xout, bool newton) {
        cfdg_status e = build_gmres_graph_once(Ubase, Rbase, rhsd, xout, newton);
        if (e != CFDG_OK && cfg.pdl && !pdl_failed) {
            // no programmatic dependent launch inside a conditional body on this driver:
            // build the body with plain launches
            pdl_failed = true;
            cudaGetLastError();
            e = build_gmres_graph_once(Ubase, Rbase, rhsd, xout, newton);
        }
        return e;
    }

    cfdg_status build_gmres_graph_once(double* Ubase, double* Rbase, double* rhsd, double* xout, bool newton) {
        // the captured kernels take GmresDev by value: they must be the graph's variant,
        // whose Givens step ends the WHILE loop; a Newton step's graph skips its solve once
        // a chain of steps has stopped (converged or non-finite)
        gd.in_graph = 1;
        gd.skip = newton ? chain_ctl + 1 : nullptr;
        if (gexec) {
            cudaGraphExecDestroy(gexec);
            gexec = nullptr;
        }
        cudaGraph_t G = nullptr;
        CK(cudaGraphCreate(&G, 0));
        cudaGraphConditionalHandle h;
        cfdg_status st_ = CFDG_OK;
        long long l0 = launches;
        std::vector<cudaGraphNode_t> leaf;
        cudaGraphNode_t cnode = nullptr;
        cudaGraph_t body = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaStreamCaptureStatus cs;
        cudaGraphNodeParams p = {};
        cudaError_t e = cudaGraphConditionalHandleCreate(&h, G, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) goto cuda_fail;
        capturing = true;
        e = cudaStreamBeginCaptureToGraph(st, G, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) goto cuda_fail;
        enqueue_gmres_pre(Ubase, rhsd, h, newton);
        e = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        if (e == cudaSuccess) leaf.assign(deps, deps + nd);
        {
            cudaError_t e2 = cudaStreamEndCapture(st, &G);
            if (e == cudaSuccess) e = e2;
        }
        if (e != cudaSuccess) goto cuda_fail;
        graph_pre = launches - l0;
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        e = cudaGraphAddNode(&cnode, G, leaf.data(), nullptr, leaf.size(), &p);
        if (e != cudaSuccess) goto cuda_fail;
        body = p.conditional.phGraph_out[0];
        l0 = launches;
        e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) goto cuda_fail;
        st_ = enqueue_gmres_body(Ubase, Rbase, h);
        {
            cudaError_t e2 = cudaStreamEndCapture(st, &body);
            if (st_ != CFDG_OK) {
                capturing = false;
                cudaGraphDestroy(G);
                return st_;
            }
            e = e2;
        }
        if (e != cudaSuccess) goto cuda_fail;
        graph_body = launches - l0;
        l0 = launches;
        e = cudaStreamBeginCaptureToGraph(st, G, &cnode, nullptr, 1, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) goto cuda_fail;
        enqueue_gmres_post(xout);
        e = cudaStreamEndCapture(st, &G);
        if (e != cudaSuccess) goto cuda_fail;
        graph_post = launches - l0;
        launches = l0 - graph_pre - graph_body;
        capturing = false;
        e = cudaGraphInstantiate(&gexec, G, 0);
        cudaGraphDestroy(G);
        if (e != cudaSuccess) {
            gexec = nullptr;
            return fail(CFDG_ERR_CUDA, std::string("GMRES graph instantiation: ") + cudaGetErrorString(e));
        }
        gkey[0] = Ubase; gkey[1] = Rbase; gkey[2] = rhsd; gkey[3] = xout;
        gnewton = newton;
        graph_version = flow_version;
        return CFDG_OK;
    cuda_fail:
        capturing = false;
        cudaGetLastError();
        if (G) cudaGraphDestroy(G);
        return fail(CFDG_ERR_CUDA, std::string("building the GMRES graph: ") + cudaGetErrorString(e));
    }

    // the graph's kernels launched one iteration at a time (no graph; the kernels see
    // in_graph = 0 and only raise the done flag), one host read of the flag per iteration
    cfdg_status gmres_stream(double* Ubase, double* Rbase, double* rhsd, double* xout, int* iters) {
        TRY(ensure_krylov());
        gd.in_graph = 0;
        gd.skip = nullptr;
        cudaGraphConditionalHandle none = 0;
        enqueue_gmres_pre(Ubase, rhsd, none, false);
        int done = 0;
        CK(cudaMemcpyAsync(&done, gd.gi + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        // the exact J v body finishes column j in the first kernel of iteration j + 2, so it
        // runs twice more than the iterations (the last run only ends the solve)
        const bool exact_body = cfg.precision == CFDG_MIXED || cfg.jv == CFDG_JV_EXACT;
        for (int it = 0; !done && it < cfg.gmres_m + (exact_body ? 2 : 0); ++it) {
            cfdg_status e = enqueue_gmres_body(Ubase, Rbase, none);
            if (e != CFDG_OK) {
                gd.in_graph = 1;
                return e;
            }
            CK(cudaMemcpyAsync(&done, gd.gi + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
        enqueue_gmres_post(xout);
        int k = -1;
        CK(cudaMemcpyAsync(&k, gd.gi + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        collect();
        gd.in_graph = 1;
        *iters = k + 1;
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    cfdg_status gmres_graph(double* Ubase, double* Rbase, double* rhsd, double* xout, int* iters) {
        TRY(ensure_krylov());
        if (!gexec || graph_version != flow_version || gkey[0] != Ubase || gkey[1] != Rbase || gkey[2] != rhsd ||
            gkey[3] != xout || gnewton)
            TRY(build_gmres_graph(Ubase, Rbase, rhsd, xout, false));
        CK(cudaGraphLaunch(gexec, st));
        int* hi = reinterpret_cast<int*>(hpin + 4);
        hi[2] = 0;
        CK(cudaMemcpyAsync(hi, gd.gi + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        if (bar) CK(cudaMemcpyAsync(hi + 2, bar + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        collect();
        if (hi[2]) return barrier_timeout();
        int k = hi[0];
        *iters = k + 1;
        launches += graph_pre + (long long)body_runs(k + 1) * graph_body + graph_post;
        return CFDG_OK;
    }

    // solveGMRES (src/Solver.cpp:1472-1618) about Ubase with the preconditioner of the
    // current state; rhs and xout are FP64 device vectors.
    cfdg_status gmres(double* Ubase, double* Rbase, double* rhsd, double* xout, int* iters) {
        if (cfg.krylov == CFDG_KRYLOV_GRAPH) return gmres_graph(Ubase, Rbase, rhsd, xout, iters);
        if (cfg.krylov == CFDG_KRYLOV_STREAM) return gmres_stream(Ubase, Rbase, rhsd, xout, iters);
        const int m = cfg.gmres_m;
        const bool mixed = cfg.precision == CFDG_MIXED;
        const int mode = mixed ? CFDG_JV_EXACT : cfg.jv;
        TRY(ensure_krylov());
        // preconditioner on the current state (computeDiagonalPreconditioner uses U_current)
        launch_prim64(nv, nc, F, f64(U), f64(W), st);
        launch_precond(nv, mv, F, U, W, dt, D, Tt, st);
        launches += 2;
        launch_dot<double>(nv, nc, rhsd, rhsd, rs, scal + 3, st);
        ++launches;
        double beta2;
        TRY(read_scalars(3, 1, &beta2));
        double beta = std::sqrt(beta2);
        *iters = 0;
        if (beta < 1e-12) {
            CK(cudaMemsetAsync(xout, 0, sizeof(double) * L, st));
            return CFDG_OK;
        }
        if (mixed) {
            // linearisation point and frozen limiter in FP32
            launch_convert<float>(L, Ubase, U32, st);
            launch_convert<float>(nc, phi, phi32, st);
            launch_convert<float>(nc, dt, dt32, st);
            launches += 3;
            // V0 = rhs * (1/beta) in FP32: scale by 1/beta computed on the device
            CK(cudaMemcpyAsync(scal + 5, &beta, sizeof(double), cudaMemcpyHostToDevice, st));
            launch_scale_from<float>(L, V32, rhsd, scal + 5, 1, st);
            ++launches;
        } else {
            CK(cudaMemcpyAsync(scal + 5, &beta, sizeof(double), cudaMemcpyHostToDevice, st));
            launch_scale_from<double>(L, V, rhsd, scal + 5, 1, st);
            ++launches;
            if (mode == CFDG_JV_FD) { launch_dot<double>(nv, nc, Ubase, Ubase, rs, scal + 0, st); ++launches; }
        }
        std::vector<double> H((size_t)(m + 1) * m, 0.0), sn(m, 0.0), cs(m, 0.0), g(m + 1, 0.0), col(m + 2);
        auto HH = [&](int i, int j) -> double& { return H[(size_t)i * m + j]; };
        g[0] = beta;
        int k = 0;
        for (int j = 0; j < m; ++j) {
            k = j;
            double* hc = hcol(j);
            if (mixed) {
                float* Vj = V32 + (size_t)j * L;
                float* Vj1 = V32 + (size_t)(j + 1) * L;
                launch_precond_apply<float>(nv, nc, Vj, D, z32, rs, nullptr, st);
                ResArgs<float> a;
                a.m = mvf;
                a.cfx = cfx32;
                a.F = Ff;
                a.nv = nv;
                a.U = f32(U32, z32);
                a.W = f32(W32, W32d);
                a.G = f32(G32, G32d);
                a.FA = ff32(nullptr, FA32d);
                a.T = f32(T32, T32d);
                a.dwall = dwall32;
                a.phi = phi32;
                a.out = Vj1;
                a.do_limiter = 0;
                a.diag_v = z32;
                a.dt = dt32;
                a.stream = st;
                a.ev = take_events(4);
                launch_jv<float>(a);
                launches += nv == 6 ? 6 : 5;
                for (int i = 0; i <= j; ++i) {
                    launch_mgs<float>(nv, nc, Vj1, i > 0 ? V32 + (size_t)(i - 1) * L : nullptr, hc + i - 1,
                                      V32 + (size_t)i * L, rs, hc + i, st);
                }
                launch_mgs<float>(nv, nc, Vj1, V32 + (size_t)j * L, hc + j, nullptr, rs, hc + j + 1, st);
                launch_scale_guard<float>(L, Vj1, hc + j + 1, 1e-12, st);
                launches += j + 3;
            } else {
                double* Vj = V + (size_t)j * L;
                double* Vj1 = V + (size_t)(j + 1) * L;
                launch_precond_apply<double>(nv, nc, Vj, D, z, rs, nullptr, st);
                ++launches;
                TRY(jv64(Ubase, Rbase, z, Vj1, mode, true));
                for (int i = 0; i <= j; ++i) {
                    launch_mgs<double>(nv, nc, Vj1, i > 0 ? V + (size_t)(i - 1) * L : nullptr, hc + i - 1,
                                       V + (size_t)i * L, rs, hc + i, st);
                }
                launch_mgs<double>(nv, nc, Vj1, V + (size_t)j * L, hc + j, nullptr, rs, hc + j + 1, st);
                launch_scale_guard<double>(L, Vj1, hc + j + 1, 1e-12, st);
                launches += j + 3;
            }
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(col.data(), hc, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            collect();
            for (int i = 0; i <= j; ++i) HH(i, j) = col[i];
            HH(j + 1, j) = std::sqrt(col[j + 1]);
            // Givens rotations (src/Solver.cpp:1562-1584)
            for (int i = 0; i < j; ++i) {
                double t = cs[i] * HH(i, j) + sn[i] * HH(i + 1, j);
                HH(i + 1, j) = -sn[i] * HH(i, j) + cs[i] * HH(i + 1, j);
                HH(i, j) = t;
            }
            double a = HH(j, j), b = HH(j + 1, j);
            if (std::fabs(b) < 1e-14) {
                cs[j] = 1.0;
                sn[j] = 0.0;
            } else {
                double t = std::sqrt(a * a + b * b);
                cs[j] = a / t;
                sn[j] = b / t;
            }
            HH(j, j) = cs[j] * a + sn[j] * b;
            HH(j + 1, j) = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (std::fabs(g[j + 1]) < cfg.gmres_tol * beta) break;
        }
        // back substitution (src/Solver.cpp:1592-1599)
        std::vector<double> y(k + 1);
        for (int i = k; i >= 0; --i) {
            y[i] = g[i];
            for (int l = i + 1; l <= k; ++l) y[i] -= HH(i, l) * y[l];
            y[i] /= HH(i, i);
        }
        CK(cudaMemcpyAsync(ydev(), y.data(), sizeof(double) * (k + 1), cudaMemcpyHostToDevice, st));
        if (mixed) launch_gmres_solution<float>(nv, nc, V32, L, ydev(), k, D, xout, st);
        else launch_gmres_solution<double>(nv, nc, V, L, ydev(), k, D, xout, st);
        ++launches;
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        collect();
        *iters = k + 1;
        return CFDG_OK;
    }

    cfdg_status step_time(cfdg_step& rec, double t0) {
        if (timing) CK(cudaEventRecord(step_ev[1], st));
        CK(cudaStreamSynchronize(st));
        collect();
        rec.seconds = now_s() - t0;
        if (timing) {
            float ms = 0;
            CK(cudaEventElapsedTime(&ms, step_ev[0], step_ev[1]));
            rec.device_ms = ms;
            if (rec.gmres_iters > 0) {
                CK(cudaEventElapsedTime(&ms, step_ev[2], step_ev[3]));
                rec.krylov_ms = ms;
            }
        }
        return CFDG_OK;
    }

    // ---- time stepping (src/Solver.cpp:1219-1243, :1801-1864)
    double* Uold = nullptr;  // solveUnsteady's U at the start of the physical step
    double physical_time = 0.0;
    long long exp_steps = 0;

    // timeStepExplicit: residual (limiter updated), U -= R dt / vol, positivity clamps;
    // res_l2 (optional) = norm_L2 of that residual
    cfdg_status time_step_explicit(double dtp, double* res_l2) {
        TRY(residual_dev(U, R, 1));
        if (res_l2) {
            launch_dot<double>(nv, nc, R, R, rs, scal + 11, st);
            ++launches;
        }
        CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
        launch_explicit_update(nv, nc, U, R, g64.vol, dtp, bad, st);
        ++launches;
        ++exp_steps;
        int hbad = 0;
        CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        if (res_l2) {
            double sq;
            TRY(read_scalars(11, 1, &sq));
            *res_l2 = std::sqrt(sq);
        } else {
            CK(cudaStreamSynchronize(st));
            collect();
        }
        if (hbad) return fail(CFDG_ERR_NAN, "non-finite state after explicit step " + std::to_string(exp_steps));
        return CFDG_OK;
    }

    // solveUnsteady: dual time stepping with BDF1, at most 15 Newton steps per physical
    // step to a residual of 1e-6 (after the first), GMRES with dt = dt_phy in the time
    // term and the preconditioner, update relaxed by 0.7.  Per physical step: Newton steps
    // taken and the last residual.
    cfdg_status solve_unsteady(double dt_phy, int n_steps, int* newton, double* res) {
        if (!Uold) TRY(dalloc(&Uold, (size_t)L));
        launch_fill(nc, dt, dt_phy, st);
        ++launches;
        for (int t = 1; t <= n_steps; ++t) {
            CK(cudaMemcpyAsync(Uold, U, sizeof(double) * L, cudaMemcpyDeviceToDevice, st));
            physical_time += dt_phy;
            int taken = 0;
            double resVM = 0.0;
            for (int step = 0; step < 15; ++step) {
                TRY(residual_dev(U, R, 1));
                launch_unsteady_rhs(nv, nc, U, Uold, R, g64.vol, dt_phy, rhs, rs, scal + 8, st);
                ++launches;
                double s2[2];
                TRY(read_scalars(8, 2, s2));
                resVM = std::sqrt(s2[0] / s2[1]);
                taken = step;
                if (!std::isfinite(resVM))
                    return fail(CFDG_ERR_NAN, "non-finite unsteady residual at time step " + std::to_string(t));
                if (resVM < 1e-6 && step > 0) break;
                int it = 0;
                TRY(gmres(U, R, rhs, x, &it));
                CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
                launch_relaxed_add(nv, nc, U, x, 0.7, bad, st);
                ++launches;
                taken = step + 1;
            }
            if (newton) newton[t - 1] = taken;
            if (res) res[t - 1] = resVM;
        }
        int hbad = 0;
        CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hbad) return fail(CFDG_ERR_NAN, "non-finite state in the unsteady solve");
        return CFDG_OK;
    }

    // pinned host words of the graph GMRES solve: [4] its last iteration, [6] the barrier flag
    double* hpin = nullptr;

    // ---- chained Newton steps (graph driver): the steps' scalar control on the device
    static constexpr int CHAIN_MAX = 64;
    // pinned host words: the records, the CFL, then the ints (ctl[0..3], per-step
    // non-finite flags, the persistent kernel's barrier flag)
    static constexpr int CHAIN_HOST_DOUBLES = NEWTON_REC * CHAIN_MAX + 1 + (4 + CHAIN_MAX + 2) / 2 + 1;
    int* chain_ctl = nullptr;     // device: NewtonCtl's ctl[0..3], then one non-finite flag per step
    double* chain_rec = nullptr;  // device: NEWTON_REC doubles per step
    double* chain_h = nullptr;
    std::vector<cudaEvent_t> chain_ev;

    // Up to k steps of solveImplicit (src/Solver.cpp:1705-1797) enqueued back to back with
    // one host synchronisation: per step the residual with its norms, |R|^2 and rhs = -R
    // (FP64: the local time step from the device CFL number), the GMRES graph and the
    // update, whose first thread records the step and runs the reference's CFL control,
    // step counter and limiter-freeze decision on the device (k_newton_update_chain).
    // Same arithmetic and decisions as one step at a time, so the trace is the same for
    // any k.  A step after convergence or a non-finite residual changes nothing (its solve
    // is empty, its update skipped) and is not reported.  recs gets the steps taken
    // (*n_done); *converged when the last of them found the residual below tol (or, with
    // tol_rho > 0, the density residual at or below tol_rho after step 5).
    cfdg_status newton_chain(double tol, int k, cfdg_step* recs, int* n_done, int* converged, double tol_rho = 0.0) {
        *converged = 0;
        *n_done = 0;
        if (k < 1) return CFDG_OK;
        if (k > CHAIN_MAX) k = CHAIN_MAX;
        // optional start-up (off by default): the first startup_first_order steps of a solve
        // run the first-order scheme, the chain stops where the configured scheme takes over
        const int want = step < cfg.startup_first_order ? CFDG_FIRST_ORDER : cfg.spatial;
        if (F.spatial != want) {
            F.spatial = want;
            Ff.spatial = want;
            ++flow_version;
        }
        if (step < cfg.startup_first_order) k = std::min(k, cfg.startup_first_order - step);
        double t0 = now_s();
        TRY(ensure_krylov());
        if (!gexec || graph_version != flow_version || gkey[0] != U || gkey[1] != R || gkey[2] != rhs || gkey[3] != x ||
            !gnewton) {
            CK(cudaStreamSynchronize(st));
            TRY(build_gmres_graph(U, R, rhs, x, true));
        }
        const bool mixed = cfg.precision == CFDG_MIXED;
        const bool limited = want == CFDG_SECOND_ORDER_LIMITED;
        double* hcfl = chain_h + NEWTON_REC * CHAIN_MAX;
        int* hc = reinterpret_cast<int*>(hcfl + 1);
        hc[0] = step;
        hc[1] = 0;
        hc[2] = !(step > cfg.limiter_freeze_step || cfl > cfg.limiter_freeze_cfl) ? 1 : 0;
        hc[3] = 0;
        *hcfl = cfl;
        CK(cudaMemcpyAsync(chain_ctl, hc, 4 * sizeof(int), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(scal + 12, hcfl, sizeof(double), cudaMemcpyHostToDevice, st));
        if (timing)
            while (chain_ev.size() < 4 * (size_t)k) {
                cudaEvent_t e;
                CK(cudaEventCreate(&e));
                chain_ev.push_back(e);
            }
        NewtonCtl c{chain_ctl, scal + 12, chain_rec, gd.gi, cfg.limiter_freeze_step, cfg.limiter_freeze_cfl,
                    cfg.cfl_max, limited ? 1 : 0, tol_rho};
        const double wmin = F.w_inf * SstConst::w_min_frac;
        for (int j = 0; j < k; ++j) {
            if (timing) CK(cudaEventRecord(chain_ev[4 * j], st));
            TRY(residual_dev(U, R, limited ? 1 : 0, true, chain_ctl + 4 + j, chain_ctl + 2));
            if (!mixed) {  // the mixed graph's prologue takes the local time step from scal[12]
                launch_local_dt(nv, mv, F, U, W, 0.0, dt, st, scal + 12);
                ++launches;
            }
            if (timing) CK(cudaEventRecord(chain_ev[4 * j + 1], st));
            CK(cudaGraphLaunch(gexec, st));
            if (timing) CK(cudaEventRecord(chain_ev[4 * j + 2], st));
            launch_newton_update_chain(nv, nc, U, x, scal + 8, tol, cfg.gamma, wmin, chain_ctl + 4 + j, c, j, step + j,
                                       cfg.update_limit, st);
            ++launches;
            if (timing) CK(cudaEventRecord(chain_ev[4 * j + 3], st));
        }
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(chain_h, chain_rec, sizeof(double) * NEWTON_REC * k, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hc, chain_ctl, sizeof(int) * (4 + k), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hcfl, scal + 12, sizeof(double), cudaMemcpyDeviceToHost, st));
        int* hbar = hc + 4 + CHAIN_MAX;
        *hbar = 0;
        if (bar) CK(cudaMemcpyAsync(hbar, bar + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        collect();
        const double wall = now_s() - t0;
        if (limited) limiter_valid = true;
        // every enqueued step ran its kernels; the WHILE body only in the steps that solved
        for (int j = 0; j < k; ++j) {
            const int its = (int)chain_h[NEWTON_REC * j + 4];
            launches += graph_pre + graph_post + (its > 0 ? body_runs(its) * graph_body : 0);
        }
        step = hc[0];
        cfl = *hcfl;
        if (*hbar) return barrier_timeout();
        cfdg_status result = CFDG_OK;
        int taken = 0;
        for (int j = 0; j < k; ++j) {
            const double* r = chain_h + NEWTON_REC * j;
            const int outcome = (int)r[6];
            if (outcome == 3) break;
            cfdg_step rec;
            rec.res_vm = r[0];
            rec.res_abs = r[1];
            rec.res_rho = r[2];
            rec.cfl = r[3];
            rec.gmres_iters = outcome == 0 ? (int)r[4] : 0;
            rec.limiter_updated = (int)r[5];
            rec.seconds = wall / k;
            rec.device_ms = 0;
            rec.krylov_ms = 0;
            if (timing) {
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, chain_ev[4 * j], chain_ev[4 * j + 3]));
                rec.device_ms = ms;
                if (outcome == 0) {
                    CK(cudaEventElapsedTime(&ms, chain_ev[4 * j + 1], chain_ev[4 * j + 2]));
                    rec.krylov_ms = ms;
                }
            }
            if (recs) recs[taken] = rec;
            ++taken;
            const int stepno = (int)r[7];
            if (outcome == 2) {
                result = fail(CFDG_ERR_NAN, "non-finite residual at Newton step " + std::to_string(stepno));
                break;
            }
            if (outcome == 1) {
                *converged = 1;
                break;
            }
            if (hc[4 + j]) {
                result = fail(CFDG_ERR_NAN, "non-finite state after the Newton update at step " + std::to_string(stepno));
                break;
            }
        }
        *n_done = taken;
        return result;
    }

    // one step of solveImplicit (src/Solver.cpp:1705-1797)
    cfdg_status newton_step(double tol, cfdg_step* info, int* converged) {
        if (cfg.krylov == CFDG_KRYLOV_GRAPH) {
            int n = 0;
            cfdg_step rec{};
            cfdg_status e = newton_chain(tol, 1, &rec, &n, converged);
            if (info && n) *info = rec;
            return e;
        }
        double t0 = now_s();
        *converged = 0;
        if (timing) CK(cudaEventRecord(step_ev[0], st));
        launch_prim64(nv, nc, F, f64(U), f64(W), st);
        launch_local_dt(nv, mv, F, U, W, cfl, dt, st);
        launches += 2;
        bool upd = !(step > cfg.limiter_freeze_step || cfl > cfg.limiter_freeze_cfl);
        TRY(residual_dev(U, R, upd ? 1 : 0));
        launch_norm_vm(nv, nc, R, g64.vol, rs, scal + 8, st);
        launch_dot<double>(nv, nc, R, R, rs, scal + 11, st);
        launches += 2;
        double s[4];
        TRY(read_scalars(8, 4, s));
        double resVM = s[1] == 0 ? 0.0 : std::sqrt(s[0] / s[1]);
        double resRho = s[1] == 0 ? 0.0 : std::sqrt(s[2] / s[1]);
        double resAbs = std::sqrt(s[3]);
        cfdg_step rec;
        rec.res_vm = resVM;
        rec.res_abs = resAbs;
        rec.res_rho = resRho;
        rec.cfl = cfl;
        rec.gmres_iters = 0;
        rec.limiter_updated = upd ? 1 : 0;
        rec.seconds = 0;
        rec.device_ms = 0;
        rec.krylov_ms = 0;
        if (!std::isfinite(resVM)) {
            if (info) *info = rec;
            return fail(CFDG_ERR_NAN, "non-finite residual at Newton step " + std::to_string(step));
        }
        if (resVM < tol) {
            *converged = 1;
            TRY(step_time(rec, t0));
            if (info) *info = rec;
            return CFDG_OK;
        }
        // RHS = -R
        double m1 = -1.0;
        CK(cudaMemcpyAsync(scal + 6, &m1, sizeof(double), cudaMemcpyHostToDevice, st));
        launch_scale_from<double>(L, rhs, R, scal + 6, 0, st);
        ++launches;
        int it = 0;
        if (timing) CK(cudaEventRecord(step_ev[2], st));
        TRY(gmres(U, R, rhs, x, &it));
        if (timing) CK(cudaEventRecord(step_ev[3], st));
        rec.gmres_iters = it;
        if (it >= 29) {
            cfl *= 0.5;
            if (cfl < 0.05) cfl = 0.05;
        }
        double relax = 1.0;
        if (resVM > 1e6) relax = 0.5;
        else if (resVM > 2e3 && resVM < 1e2) relax = 0.9;
        CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
        launch_newton_update(nv, nc, U, x, relax, cfg.gamma, F.w_inf * SstConst::w_min_frac, bad, st);
        ++launches;
        int hbad = 0;
        CK(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        TRY(step_time(rec, t0));
        if (step > 5) {
            if (resVM > 1e6) cfl *= 1.2;
            else cfl *= 1.5;
            if (it >= 25) cfl *= 0.5;
            if (cfl > cfg.cfl_max) cfl = cfg.cfl_max;
            if (cfl < 0.1) cfl = 0.1;
        }
        ++step;
        if (info) *info = rec;
        if (hbad) return fail(CFDG_ERR_NAN, "non-finite state after the Newton update at step " + std::to_string(step - 1));
        return CFDG_OK;
    }

    // distance from each cell centroid to the nearest no-slip wall face midpoint
    // (computeWallDistances, src/Solver.cpp:1981-2015), 1e10 without walls, into dwall
    // (and dwall32 when allocated), with 1 / max(d, 1e-30) in their second nc entries;
    // dwall is allocated here when the model has none
    cfdg_status wall_distance() {
        const HostMesh& h = mesh->h;
        if (!dwall) TRY(dalloc(&dwall, 2 * (size_t)nc));
        std::vector<double> wxy;
        for (int f = 0; f < h.n_faces; ++f)
            if (h.f_n[f] < 0 && h.f_tag[f] == 4) wxy.push_back(h.f_xm[f]);
        size_t nw = wxy.size();
        for (int f = 0; f < h.n_faces; ++f)
            if (h.f_n[f] < 0 && h.f_tag[f] == 4) wxy.push_back(h.f_ym[f]);
        double* tmp = nullptr;
        TRY(dalloc(&tmp, 2 * (size_t)nc + 2 * nw));
        bool ok = cudaMemcpy(tmp, h.xc.data(), sizeof(double) * nc, cudaMemcpyHostToDevice) == cudaSuccess &&
                  cudaMemcpy(tmp + nc, h.yc.data(), sizeof(double) * nc, cudaMemcpyHostToDevice) == cudaSuccess &&
                  (nw == 0 || cudaMemcpy(tmp + 2 * nc, wxy.data(), sizeof(double) * 2 * nw,
                                         cudaMemcpyHostToDevice) == cudaSuccess);
        if (ok) {
            launch_wall_distance(nc, tmp, tmp + nc, (int)nw, tmp + 2 * nc, tmp + 2 * nc + nw, dwall, dwall32, st);
            ++launches;
            ok = cudaStreamSynchronize(st) == cudaSuccess && cudaGetLastError() == cudaSuccess;
        }
        cudaFree(tmp);
        if (!ok) return fail(CFDG_ERR_CUDA, "wall distance failed");
        return CFDG_OK;
    }

    // wall quantities: boundary faces of one tag in reference face order, as device slots,
    // and the per-face outputs (cp, cf, drag terms) plus the drag sum
    int* qslots = nullptr;
    double* qbuf = nullptr;
    int qcap = 0;
    // objectives: listed faces, their weights, the per-boundary-slot weights, terms and J
    int* oslots = nullptr;
    double* obuf = nullptr;
    int ocap = 0;

    // J and (grad != null) dJ/dU into grad (device SoA) for objective kind; see cfdg.h
    cfdg_status objective(int kind, double x0, double x1, double* grad) {
        const HostMesh& h = mesh->h;
        int tag = kind == CFDG_OBJ_PRESSURE_DRAG ? 3 : 4;
        std::vector<int> faces = tagged_faces(tag);
        int n = (int)faces.size(), nb = nf - h.n_interior;
        std::vector<double> w(n, 1.0), wslot(nb, 0.0);
        for (int k = 0; k < n; ++k) {
            if (kind == CFDG_OBJ_WALL_PRESSURE) {
                double xm = h.f_xm[h.face_perm[faces[k]]];
                w[k] = (xm >= x0 && xm <= x1) ? 1.0 : 0.0;
            }
            wslot[faces[k] - h.n_interior] = w[k];
        }
        if (n + 1 > ocap || ocap == 0) {
            cudaFree(oslots);
            cudaFree(obuf);
            oslots = nullptr;
            obuf = nullptr;
            ocap = 0;
            TRY(dalloc(&oslots, (size_t)n + 1));
            TRY(dalloc(&obuf, 2 * ((size_t)n + 1) + (size_t)nb + 1));
            ocap = n + 1;
        }
        double* dw = obuf;
        double* dterms = obuf + ocap;
        double* dwslot = obuf + 2 * (size_t)ocap;
        double* dJ = dwslot + nb;
        if (n) {
            CK(cudaMemcpyAsync(oslots, faces.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(dw, w.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
        }
        if (nb) CK(cudaMemcpyAsync(dwslot, wslot.data(), sizeof(double) * nb, cudaMemcpyHostToDevice, st));
        launch_objective(nv, kind, n, oslots, dw, dwslot, mv, F, U, dterms, dJ, grad, st);
        launches += (n > 0) + 1 + (grad != nullptr);
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    // the device slots of the boundary faces with this tag, in reference face order
    std::vector<int> tagged_faces(int tag) const {
        const HostMesh& h = mesh->h;
        std::vector<int> out;
        for (int f = 0; f < h.n_faces; ++f)
            if (h.f_n[f] < 0 && h.f_tag[f] == tag) out.push_back(h.face_inv[f]);
        return out;
    }

    // free-stream q and p of extractSkinFriction (src/Solver.cpp:1904-1911)
    void freestream_q(double& q_inf, double& p_inf) const {
        double g = cfg.gamma;
        double factor_T = 1.0 + 0.5 * (g - 1.0) * M_inf * M_inf;
        double T_static = T0 / factor_T;
        double c_inf = std::sqrt(g * cfg.R_gas * T_static);
        double u_inf = M_inf * c_inf;
        double rho_inf = Pexit / (cfg.R_gas * T_static);
        q_inf = 0.5 * rho_inf * u_inf * u_inf;
        p_inf = Pexit;
    }

    // Cp, Cf and drag terms of the listed faces into qbuf (3 planes of qcap) and the
    // in-order drag sum into qbuf[3 * qcap]
    cfdg_status wall_terms(const std::vector<int>& faces) {
        int n = (int)faces.size();
        if (n > qcap) {
            cudaFree(qslots);
            cudaFree(qbuf);
            qslots = nullptr;
            qbuf = nullptr;
            qcap = 0;
            TRY(dalloc(&qslots, (size_t)n));
            TRY(dalloc(&qbuf, 3 * (size_t)n + 1));
            qcap = n;
        }
        if (n) CK(cudaMemcpyAsync(qslots, faces.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
        double q_inf, p_inf;
        freestream_q(q_inf, p_inf);
        launch_wall_coeff(nv, n, qslots, mv, F, U, q_inf, p_inf, qbuf, qbuf + qcap, qbuf + 2 * (size_t)qcap, st);
        launch_sum_in_order(n, qbuf + 2 * (size_t)qcap, qbuf + 3 * (size_t)qcap, st);
        launches += 2;
        CK(cudaGetLastError());
        return CFDG_OK;
    }

    void release() {
        cudaFree(qslots);
        cudaFree(qbuf);
        cudaFree(oslots);
        cudaFree(obuf);
        cudaFree(f32out);
        cudaFree(f32dir);
        cudaFree(Uold);
        cudaFree(bar);
        cudaFree(apart);
        if (hpin) cudaFreeHost(hpin);
        cudaFree(chain_ctl);
        cudaFree(chain_rec);
        if (chain_h) cudaFreeHost(chain_h);
        for (cudaEvent_t e : chain_ev) cudaEventDestroy(e);
        cudaFree(dinv32);
        cudaFree(dinv64);
        void* pt[] = {Tt, Tj, Tjd, dwall, T32, T32d, dwall32};
        for (void* p : pt) cudaFree(p);
        void* ps[] = {cf, fo, fn, ftag, perm, iperm, gft, U, W, G, phi, FA, R, dt, D, stage, Ub, Rb, Up, Rp, vtmp, x, rhs,
                      Wj, Wjd, Gj, Gjd, FAjd, U32, W32, W32d, G32, G32d, FA32d, phi32, dt32, V32, z32, V, z,
                      rs.partial, rs.counter, scal, bad};
        for (void* p : ps) cudaFree(p);
        g64.release();
        g32.release();
        cudaFree(cfx_nbr);
        cudaFree(cfx_geo);
        cudaFree(l2buf);
        cudaFree(gdi);
        cudaFree(gdd);
        cudaFree(w32);
        cudaFree(w64);
        cudaFree(adj_mem);
        cudaFree(adj_imem);
        cudaFree(phi_adj);
        if (gexec) cudaGraphExecDestroy(gexec);
        for (auto& e : pool) cudaEventDestroy(e);
        for (auto& e : step_ev) if (e) cudaEventDestroy(e);
        if (st) cudaStreamDestroy(st);
    }
};

// ------------------------------------------------------------------ C ABI

extern "C" {

const char* cfdg_version(void) { return "cfdg 0.1 (sm_103a)"; }

const char* cfdg_last_error(void) { return g_err.c_str(); }

cfdg_status cfdg_device_count(int* n) {
    if (!n) return fail(CFDG_ERR_ARG, "null pointer");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c = 0;
    }
    *n = c;
    return CFDG_OK;
}

void cfdg_config_default(cfdg_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->flux = CFDG_FLUX_HLLC;
    c->spatial = CFDG_SECOND_ORDER_LIMITED;
    c->bcset = CFDG_BC_BUMP;
    c->init = CFDG_INIT_BUMP;
    c->viscous = 0;
    c->turbulence = CFDG_TURB_NONE;
    c->precision = CFDG_FP64;
    c->jv = CFDG_JV_FD;
    c->gmres_m = 40;
    c->gmres_tol = 1e-2;
    c->gamma = 1.4;
    c->R_gas = 287.0;
    c->Pr = 0.72;
    c->nu = 0.01;
    c->cfl0 = 0.1;
    c->cfl_max = 10000.0;
    c->limiter_freeze_step = 150;
    c->limiter_freeze_cfl = 10.0;
    c->turb_intensity = 0.001;
    c->mut_ratio = 0.01;
    c->shock_deflection_deg = 0.0;
    c->renumber = CFDG_RENUMBER_HILBERT;
    c->device = 0;
    c->krylov = CFDG_KRYLOV_AUTO;
    c->persistent = 0;
    c->pdl = 1;
    c->barrier_poll_limit = 0;
    c->newton_chain = 8;
    c->startup_first_order = 0;
    c->update_limit = 0.0;
    c->gather_split_cells = 0;
}

cfdg_status cfdg_mesh_create(int n_nodes, const double* xy, int n_cells, const int* cells, int n_bedges,
                             const int* bedges, int renumber, cfdg_mesh** out) {
    if (!out || !xy || !cells || (n_bedges > 0 && !bedges) || n_nodes <= 0 || n_cells <= 0 || n_bedges < 0)
        return fail(CFDG_ERR_ARG, "cfdg_mesh_create: bad arguments");
    cfdg_mesh* m = new cfdg_mesh();
    std::string e = build_mesh(m->h, n_nodes, xy, n_cells, cells, n_bedges, bedges, renumber);
    if (!e.empty()) {
        delete m;
        return fail(CFDG_ERR_MESH, e);
    }
    *out = m;
    return CFDG_OK;
}

cfdg_status cfdg_mesh_create_gpu(int n_nodes, const double* xy, int n_cells, const int* cells, int n_bedges,
                                 const int* bedges, int renumber, int device, cfdg_mesh** out) {
    if (!out || !xy || !cells || (n_bedges > 0 && !bedges) || n_nodes <= 0 || n_cells <= 0 || n_bedges < 0)
        return fail(CFDG_ERR_ARG, "cfdg_mesh_create_gpu: bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return fail(CFDG_ERR_CUDA, "cfdg_mesh_create_gpu: no such CUDA device");
    }
    cfdg_mesh* m = new cfdg_mesh();
    std::string e = build_mesh_gpu(m->h, n_nodes, xy, n_cells, cells, n_bedges, bedges, renumber, device, nullptr);
    if (!e.empty()) {
        delete m;
        return fail(e.rfind("GPU mesh build:", 0) == 0 ? CFDG_ERR_CUDA : CFDG_ERR_MESH, e);
    }
    *out = m;
    return CFDG_OK;
}

cfdg_status cfdg_mesh_load_gmsh(const char* path, int renumber, cfdg_mesh** out) {
    if (!path || !out) return fail(CFDG_ERR_ARG, "cfdg_mesh_load_gmsh: null argument");
    std::vector<double> xy;
    std::vector<int> cells, bed;
    std::string e = read_gmsh(path, xy, cells, bed);
    if (!e.empty()) return fail(CFDG_ERR_MESH, e);
    if (cells.empty()) return fail(CFDG_ERR_MESH, std::string("no cells in ") + path);
    return cfdg_mesh_create((int)(xy.size() / 2), xy.data(), (int)(cells.size() / 4), cells.data(),
                            (int)(bed.size() / 3), bed.empty() ? nullptr : bed.data(), renumber, out);
}

cfdg_status cfdg_mesh_sizes(const cfdg_mesh* m, int* n_cells, int* n_faces, int* n_boundary_faces) {
    if (!m) return fail(CFDG_ERR_ARG, "null mesh");
    if (n_cells) *n_cells = m->h.n_cells;
    if (n_faces) *n_faces = m->h.n_faces;
    if (n_boundary_faces) *n_boundary_faces = m->h.n_faces - m->h.n_interior;
    return CFDG_OK;
}

cfdg_status cfdg_mesh_faces(const cfdg_mesh* m, int* i5, double* d5) {
    if (!m || !i5 || !d5) return fail(CFDG_ERR_ARG, "null argument");
    const HostMesh& h = m->h;
    for (int f = 0; f < h.n_faces; ++f) {
        i5[5 * f] = h.f_n1[f]; i5[5 * f + 1] = h.f_n2[f]; i5[5 * f + 2] = h.f_o[f];
        i5[5 * f + 3] = h.f_n[f]; i5[5 * f + 4] = h.f_tag[f];
        d5[5 * f] = h.f_nx[f]; d5[5 * f + 1] = h.f_ny[f]; d5[5 * f + 2] = h.f_area[f];
        d5[5 * f + 3] = h.f_xm[f]; d5[5 * f + 4] = h.f_ym[f];
    }
    return CFDG_OK;
}

cfdg_status cfdg_mesh_cells(const cfdg_mesh* m, double* d3) {
    if (!m || !d3) return fail(CFDG_ERR_ARG, "null argument");
    for (int c = 0; c < m->h.n_cells; ++c) {
        d3[3 * c] = m->h.c_vol[c]; d3[3 * c + 1] = m->h.c_xc[c]; d3[3 * c + 2] = m->h.c_yc[c];
    }
    return CFDG_OK;
}

cfdg_status cfdg_mesh_permutation(const cfdg_mesh* m, int* cell_perm, int* face_perm) {
    if (!m) return fail(CFDG_ERR_ARG, "null mesh");
    if (cell_perm) std::memcpy(cell_perm, m->h.cell_perm.data(), sizeof(int) * m->h.n_cells);
    if (face_perm) std::memcpy(face_perm, m->h.face_perm.data(), sizeof(int) * m->h.n_faces);
    return CFDG_OK;
}

void cfdg_mesh_destroy(cfdg_mesh* m) { delete m; }

cfdg_status cfdg_solver_create(const cfdg_mesh* m, const cfdg_config* cfg, cfdg_solver** out) {
    if (!m || !out) return fail(CFDG_ERR_ARG, "cfdg_solver_create: null argument");
    cfdg_config c;
    if (cfg) c = *cfg;
    else cfdg_config_default(&c);
    if (c.gmres_m < 1 || c.gmres_m > 400) return fail(CFDG_ERR_ARG, "gmres_m must be in [1, 400]");
    if (c.krylov < CFDG_KRYLOV_AUTO || c.krylov > CFDG_KRYLOV_STREAM) return fail(CFDG_ERR_ARG, "unknown krylov driver");
    if (c.krylov != CFDG_KRYLOV_HOST && c.gmres_m > KRY_MAXM)
        return fail(CFDG_ERR_ARG, "the graph Krylov driver supports gmres_m <= 128");
    if (c.flux < 0 || c.flux > 3 || c.spatial < 0 || c.spatial > 2 || c.bcset < 0 || c.bcset > 2)
        return fail(CFDG_ERR_ARG, "unknown flux, spatial scheme or boundary-condition set");
    if (c.turbulence != CFDG_TURB_NONE && c.turbulence != CFDG_TURB_SST) return fail(CFDG_ERR_ARG, "unknown turbulence model");
    if (c.turbulence == CFDG_TURB_SST && !c.viscous) return fail(CFDG_ERR_ARG, "SST needs the viscous term (viscous = 1)");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CFDG_ERR_CUDA, "no CUDA device available (this library has no CPU path)");
    }
    if (c.device < 0 || c.device >= ndev) return fail(CFDG_ERR_ARG, "device ordinal out of range");
    CK(cudaSetDevice(c.device));
    cfdg_solver* s = new cfdg_solver();
    s->mesh = m;
    s->cfg = c;
    s->nv = c.turbulence == CFDG_TURB_SST ? 6 : 4;
    s->nc = m->h.n_cells;
    s->nf = m->h.n_faces;
    s->L = (long)s->nv * s->nc;
    s->nu = c.nu;
    s->cfl = c.cfl0;
    if (s->cfg.krylov == CFDG_KRYLOV_AUTO)
        s->cfg.krylov = (c.precision == CFDG_MIXED || c.jv == CFDG_JV_EXACT) ? CFDG_KRYLOV_GRAPH : CFDG_KRYLOV_HOST;
    auto bail = [&](cfdg_status st) {
        s->release();
        delete s;
        return st;
    };
#define TRYS(expr)                       \
    do {                                 \
        cfdg_status st_ = (expr);        \
        if (st_ != CFDG_OK) return bail(st_); \
    } while (0)
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) return bail(fail(CFDG_ERR_CUDA, "stream"));
    for (auto& e : s->step_ev) cudaEventCreate(&e);
    const HostMesh& h = m->h;
    int nc = s->nc, nf = s->nf, nv = s->nv;
    long L = s->L;
    TRYS(dalloc(&s->cf, 4 * (size_t)nc));
    TRYS(dalloc(&s->fo, nf));
    TRYS(dalloc(&s->fn, nf));
    TRYS(dalloc(&s->ftag, nf));
    TRYS(dalloc(&s->perm, nc));
    if (cudaMemcpy(s->cf, h.cf.data(), sizeof(int) * 4 * (size_t)nc, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->fo, h.fo.data(), sizeof(int) * nf, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->fn, h.fn.data(), sizeof(int) * nf, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->ftag, h.ftag.data(), sizeof(int) * nf, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->perm, h.cell_perm.data(), sizeof(int) * nc, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(CFDG_ERR_CUDA, "mesh upload failed"));
    {
        std::vector<int> ip((size_t)nc);
        for (int i = 0; i < nc; ++i) ip[(size_t)h.cell_perm[i]] = i;
        TRYS(dalloc(&s->iperm, nc));
        if (cudaMemcpy(s->iperm, ip.data(), sizeof(int) * nc, cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(CFDG_ERR_CUDA, "mesh upload failed"));
    }
    TRYS(upload_geo(s->g64, h));
    TRYS(upload_geo(s->g32, h));
    auto view = [&](auto& g, auto& mvx) {
        mvx.nc = nc; mvx.nf = nf; mvx.nfi = h.n_interior;
        mvx.cf = s->cf; mvx.fo = s->fo; mvx.fn = s->fn; mvx.ftag = s->ftag;
        mvx.nx = g.nx; mvx.ny = g.ny; mvx.area = g.area; mvx.dxo = g.dxo; mvx.dyo = g.dyo;
        mvx.dxn = g.dxn; mvx.dyn = g.dyn; mvx.dxlr = g.dxlr; mvx.dylr = g.dylr; mvx.vol = g.vol;
        mvx.d2lr = g.d2lr; mvx.id2lr = g.id2lr; mvx.ivol = g.ivol;
    };
    view(s->g64, s->mv);
    view(s->g32, s->mvf);
    if (c.precision == CFDG_MIXED) {
        // CellFaces of the FP32 view: the same float values as g32's face arrays
        std::vector<int> nb(4 * (size_t)nc, -1);
        std::vector<float> geo(12 * (size_t)nc, 0.0f);
        for (int k = 0; k < 4; ++k) {
            for (int i = 0; i < nc; ++i) {
                const size_t q = (size_t)k * nc + i;
                const int e = h.cf[q];
                if (e < 0) continue;
                const int f = e >> 1;
                nb[q] = (e & 1) ? h.fo[f] : h.fn[f];
                geo[q] = (float)h.nx[f];
                geo[4 * (size_t)nc + q] = (float)h.ny[f];
                geo[8 * (size_t)nc + q] = (float)h.area[f];
            }
        }
        TRYS(dalloc(&s->cfx_nbr, nb.size()));
        TRYS(dalloc(&s->cfx_geo, geo.size()));
        if (cudaMemcpy(s->cfx_nbr, nb.data(), sizeof(int) * nb.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(s->cfx_geo, geo.data(), sizeof(float) * geo.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(CFDG_ERR_CUDA, "mesh upload failed"));
        s->cfx32 = CellFaces<float>{s->cfx_nbr, s->cfx_geo, s->cfx_geo + 4 * (size_t)nc, s->cfx_geo + 8 * (size_t)nc};
    }
    int NW = nv == 6 ? 7 : 5, NG = nv == 6 ? 14 : 10;
    TRYS(dalloc(&s->U, L)); TRYS(dalloc(&s->W, (size_t)NW * nc)); TRYS(dalloc(&s->G, (size_t)NG * nc));
    TRYS(dalloc(&s->phi, nc)); TRYS(dalloc(&s->FA, (size_t)nv * nf)); TRYS(dalloc(&s->R, L));
    TRYS(dalloc(&s->dt, nc)); TRYS(dalloc(&s->D, (size_t)(nv == 6 ? 3 : 1) * nc)); TRYS(dalloc(&s->stage, 14 * (size_t)nc));
    TRYS(dalloc(&s->Ub, L)); TRYS(dalloc(&s->Rb, L)); TRYS(dalloc(&s->Up, L)); TRYS(dalloc(&s->Rp, L));
    TRYS(dalloc(&s->vtmp, L)); TRYS(dalloc(&s->x, L)); TRYS(dalloc(&s->rhs, L));
    TRYS(dalloc(&s->Wj, (size_t)NW * nc)); TRYS(dalloc(&s->Wjd, (size_t)NW * nc));
    TRYS(dalloc(&s->Gj, (size_t)NG * nc)); TRYS(dalloc(&s->Gjd, (size_t)NG * nc));
    TRYS(dalloc(&s->FAjd, (size_t)nv * nf));
    // the FP64 gradient's per-face terms on meshes large enough for the FP64 pipe to bound
    // the gradient; on small meshes the residual is latency-bound and the face kernel would
    // be one launch more
    if (h.n_interior >= GRAD_FACE_TERMS_MIN_FACES) TRYS(dalloc(&s->gft, (size_t)2 * NW * h.n_interior));
    if (nv == 6) {
        TRYS(dalloc(&s->Tt, 4 * (size_t)nc)); TRYS(dalloc(&s->Tj, 4 * (size_t)nc)); TRYS(dalloc(&s->Tjd, 4 * (size_t)nc));
        TRYS(dalloc(&s->dwall, 2 * (size_t)nc)); TRYS(dalloc(&s->dwall32, 2 * (size_t)nc));
        TRYS(dalloc(&s->T32, 4 * (size_t)nc)); TRYS(dalloc(&s->T32d, 4 * (size_t)nc));
        TRYS(s->wall_distance());
    }
    if (c.precision == CFDG_MIXED) {
        TRYS(dalloc(&s->U32, L)); TRYS(dalloc(&s->W32, (size_t)NW * nc)); TRYS(dalloc(&s->W32d, (size_t)NW * nc));
        TRYS(dalloc(&s->G32, (size_t)NG * nc)); TRYS(dalloc(&s->G32d, (size_t)NG * nc));
        TRYS(dalloc(&s->FA32d, (size_t)nv * nf)); TRYS(dalloc(&s->phi32, nc)); TRYS(dalloc(&s->dt32, nc));
    }
    TRYS(dalloc(&s->rs.partial, 4 * (size_t)RED_BLOCKS));
    TRYS(dalloc(&s->rs.counter, 1));
    TRYS(dalloc(&s->scal, 16 + (size_t)(c.gmres_m + 2) * (c.gmres_m + 2) + 8));
    TRYS(dalloc(&s->bad, 1));
    {
        // scal[6] = -1, the constant of rhs = -R; pinned words for the single-sync step
        const double m1 = -1.0;
        if (cudaMemcpy(s->scal + 6, &m1, sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMallocHost((void**)&s->hpin, 8 * sizeof(double)) != cudaSuccess)
            return bail(fail(CFDG_ERR_CUDA, "scalar scratch"));
    }
    if (c.gmres_m <= KRY_MAXM) {  // device-GMRES state, so the driver can be switched at run time
        int m = c.gmres_m;
        TRYS(dalloc(&s->gdi, 8));
        size_t nd = 3 + (size_t)(m + 1) + 2 * (size_t)m + 2 * (size_t)(m + 1) * m + 2 * (size_t)(m + 2) + m +
                    2 * (size_t)(m + 1) + 2 + (size_t)(m + 1) + (2 * (size_t)KRY_MAXM + 3) * RED_BLOCKS + 4;
        TRYS(dalloc(&s->gdd, nd));
        double* q = s->gdd;
        GmresDev& d = s->gd;
        d.gi = s->gdi;
        d.beta = q; q += 3;
        d.g = q; q += m + 1;
        d.cs = q; q += m;
        d.sn = q; q += m;
        d.H = q; q += (size_t)(m + 1) * m;
        d.Hu = q; q += (size_t)(m + 1) * m;
        d.sig = q; q += m + 2;
        d.ilam = q; q += m + 2;
        d.y = q; q += m;
        d.h1 = q; q += m + 1;
        d.h2 = q; q += m + 1;
        d.hsq = q; q += 2;
        d.sc = q; q += m + 1;
        d.partial = q; q += (2 * (size_t)KRY_MAXM + 3) * RED_BLOCKS;
        d.nb1 = 0;  // set by the first kernel's launcher for its basis precision
        d.counter = reinterpret_cast<unsigned*>(q);
        d.in_graph = 1;
        if (c.precision == CFDG_MIXED) TRYS(dalloc(&s->w32, (size_t)L));
        else TRYS(dalloc(&s->w64, (size_t)L));
    }
    // limiter starts at 1 (no limiting) until the first limited evaluation
    std::vector<double> ones(nc, 1.0);
    if (cudaMemcpy(s->phi, ones.data(), sizeof(double) * nc, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail(fail(CFDG_ERR_CUDA, "limiter init failed"));
    s->set_flow();
#undef TRYS
    *out = s;
    return CFDG_OK;
}

void cfdg_solver_destroy(cfdg_solver* s) {
    if (!s) return;
    cudaStreamSynchronize(s->st);
    s->release();
    delete s;
}

cfdg_status cfdg_set_numerical_method(cfdg_solver* s, int flux, int spatial) {
    if (!s || flux < 0 || flux > 3 || spatial < 0 || spatial > 2) return fail(CFDG_ERR_ARG, "bad scheme");
    s->cfg.flux = flux;
    s->cfg.spatial = spatial;
    s->set_flow();
    return CFDG_OK;
}

cfdg_status cfdg_set_flow_conditions(cfdg_solver* s, double M, double P, double T) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    double g = s->cfg.gamma;
    s->M_inf = M;
    double fT = 1.0 + 0.5 * (g - 1.0) * M * M;
    double fP = std::pow(fT, g / (g - 1.0));
    s->T0 = T * fT;
    s->P0 = P * fP;
    s->Pexit = P;
    s->set_flow();
    return CFDG_OK;
}

cfdg_status cfdg_set_freestream_static(cfdg_solver* s, double M, double P, double T) {
    return cfdg_set_flow_conditions(s, M, P, T);
}

cfdg_status cfdg_set_kinematic_viscosity(cfdg_solver* s, double Re, double Lref) {
    if (!s || !(Re > 0)) return fail(CFDG_ERR_ARG, "bad Reynolds number");
    double g = s->cfg.gamma;
    double fT = 1.0 + 0.5 * (g - 1.0) * s->M_inf * s->M_inf;
    double Ts = s->T0 / fT;
    double c = std::sqrt(g * s->cfg.R_gas * Ts);
    double u = s->M_inf * c;
    s->nu = (u * Lref) / Re;
    s->set_flow();
    return CFDG_OK;
}

cfdg_status cfdg_get_params(const cfdg_solver* s, double* o) {
    if (!s || !o) return fail(CFDG_ERR_ARG, "null argument");
    o[0] = s->M_inf; o[1] = s->P0; o[2] = s->T0; o[3] = s->Pexit; o[4] = s->nu; o[5] = s->cfg.R_gas;
    return CFDG_OK;
}

cfdg_status cfdg_initialize(cfdg_solver* s) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    double g = s->cfg.gamma, Rg = s->cfg.R_gas;
    double st4[4];
    if (s->cfg.init == CFDG_INIT_BUMP) {
        // src/Solver.cpp:46-65
        double p = s->Pexit;
        double fT = std::pow(s->P0 / p, (g - 1.0) / g);
        double T = s->T0 / fT;
        double rho = p / (Rg * T);
        double V = std::sqrt(2.0 * (g * Rg / (g - 1.0)) * (s->T0 - T));
        st4[0] = rho; st4[1] = rho * V; st4[2] = rho * 0.0;
        st4[3] = p / (g - 1.0) + 0.5 * rho * (V * V + 0.0 * 0.0);
    } else {
        for (int k = 0; k < 4; ++k) st4[k] = s->F.fs[k];
    }
    std::vector<double> U(6 * (size_t)s->nc, 0.0);
    for (int i = 0; i < s->nc; ++i) {
        for (int k = 0; k < 4; ++k) U[6 * (size_t)i + k] = st4[k];
        if (s->nv == 6) {
            U[6 * (size_t)i + 4] = st4[0] * s->F.k_inf;
            U[6 * (size_t)i + 5] = st4[0] * s->F.w_inf;
        }
    }
    return cfdg_set_state(s, U.data());
}

cfdg_status cfdg_set_state(cfdg_solver* s, const double* U) {
    if (!s || !U) return fail(CFDG_ERR_ARG, "null argument");
    TRY(s->upload_aos(U, s->U));
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_get_state(cfdg_solver* s, double* U) {
    if (!s || !U) return fail(CFDG_ERR_ARG, "null argument");
    return s->download_aos(s->U, U, s->nv, 6);
}

cfdg_status cfdg_residual(cfdg_solver* s, const double* U, double* R, int update_limiters) {
    if (!s || !R) return fail(CFDG_ERR_ARG, "null argument");
    double* hR = s->mapped(R);
    double* hU = U ? s->mapped(U) : nullptr;
    if (hR && (!U || hU)) {
        // pinned state and residual: the primitives are formed as U's rows arrive over the
        // link, and the gather writes R's rows back in place (the transfers overlap the
        // first and the last stage)
        double* Uin = s->U;
        if (U) {
            launch_rows_prim(s->nv, s->nc, s->F, hU, s->iperm, s->f64(s->Ub), s->f64(s->W), s->st);
            ++s->launches;
            Uin = s->Ub;
        }
        TRY(s->residual_dev(Uin, s->R, update_limiters, false, nullptr, nullptr, U != nullptr, hR));
        CK(cudaStreamSynchronize(s->st));
        s->collect();
        return CFDG_OK;
    }
    double* Uin = s->U;
    if (U) {
        TRY(s->upload_aos(U, s->Ub));
        Uin = s->Ub;
    }
    TRY(s->residual_dev(Uin, s->R, update_limiters));
    return s->download_aos(s->R, R, s->nv, 6);
}

cfdg_status cfdg_residual_device(cfdg_solver* s, int update_limiters) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    TRY(s->residual_dev(s->U, s->R, update_limiters));
    if (s->timing) {
        CK(cudaStreamSynchronize(s->st));
        s->collect();
    }
    return CFDG_OK;
}

cfdg_status cfdg_gradients(cfdg_solver* s, const double* U, double* g10) {
    if (!s || !g10) return fail(CFDG_ERR_ARG, "null argument");
    double* Uin = s->U;
    if (U) {
        TRY(s->upload_aos(U, s->Ub));
        Uin = s->Ub;
    }
    // the residual's gradient stage (no limiter update) leaves the gradients in G
    ResArgs<double> a = s->res64(Uin, s->R, 0);
    launch_residual<double>(a);
    s->launches += s->res64_kernels();
    CK(cudaGetLastError());
    return s->download_aos(s->G, g10, 10, 10);
}

cfdg_status cfdg_limiters(cfdg_solver* s, const double* U, double* phi) {
    if (!s || !phi) return fail(CFDG_ERR_ARG, "null argument");
    double* Uin = s->U;
    if (U) {
        TRY(s->upload_aos(U, s->Ub));
        Uin = s->Ub;
    }
    ResArgs<double> a = s->res64(Uin, s->R, 1);
    launch_residual<double>(a);
    s->launches += s->res64_kernels();
    s->limiter_valid = true;
    CK(cudaGetLastError());
    return s->download_aos(s->phi, phi, 1, 1);
}

cfdg_status cfdg_get_limiters(cfdg_solver* s, double* phi) {
    if (!s || !phi) return fail(CFDG_ERR_ARG, "null argument");
    return s->download_aos(s->phi, phi, 1, 1);
}

cfdg_status cfdg_set_limiters(cfdg_solver* s, const double* phi) {
    if (!s || !phi) return fail(CFDG_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(s->stage, phi, sizeof(double) * s->nc, cudaMemcpyHostToDevice, s->st));
    launch_aos_to_soa<double>(s->nc, 1, 1, s->stage, s->perm, s->phi, s->st);
    s->launches += 1;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->st));
    s->limiter_valid = true;
    return CFDG_OK;
}

cfdg_status cfdg_local_timestep(cfdg_solver* s, double cfl, double* dt) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    launch_prim64(s->nv, s->nc, s->F, s->f64(s->U), s->f64(s->W), s->st);
    launch_local_dt(s->nv, s->mv, s->F, s->U, s->W, cfl, s->dt, s->st);
    s->launches += 2;
    CK(cudaGetLastError());
    if (dt) return s->download_aos(s->dt, dt, 1, 1);
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_set_timestep(cfdg_solver* s, const double* dt) {
    if (!s || !dt) return fail(CFDG_ERR_ARG, "null argument");
    CK(cudaMemcpyAsync(s->stage, dt, sizeof(double) * s->nc, cudaMemcpyHostToDevice, s->st));
    launch_aos_to_soa<double>(s->nc, 1, 1, s->stage, s->perm, s->dt, s->st);
    s->launches += 1;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_preconditioner(cfdg_solver* s, double* D) {
    if (!s || !D) return fail(CFDG_ERR_ARG, "null argument");
    launch_prim64(s->nv, s->nc, s->F, s->f64(s->U), s->f64(s->W), s->st);
    launch_precond(s->nv, s->mv, s->F, s->U, s->W, s->dt, s->D, s->Tt, s->st);
    s->launches += 2;
    CK(cudaGetLastError());
    return s->download_aos(s->D, D, 1, 1);
}

cfdg_status cfdg_jv(cfdg_solver* s, const double* Ubase, const double* Rbase, const double* v, double* Jv, int mode) {
    if (!s || !Ubase || !v || !Jv || (mode == CFDG_JV_FD && !Rbase) || mode < 0 || mode > 1)
        return fail(CFDG_ERR_ARG, "cfdg_jv: bad arguments");
    TRY(s->upload_aos(Ubase, s->Ub));
    if (Rbase) TRY(s->upload_aos(Rbase, s->Rb));
    TRY(s->upload_aos(v, s->vtmp));
    TRY(s->jv64(s->Ub, s->Rb, s->vtmp, s->x, mode, false));
    return s->download_aos(s->x, Jv, s->nv, 6);
}

cfdg_status cfdg_time_step_explicit(cfdg_solver* s, double dt, double* res_l2) {
    if (!s || !(dt > 0)) return fail(CFDG_ERR_ARG, "null solver or non-positive dt");
    return s->time_step_explicit(dt, res_l2);
}

cfdg_status cfdg_solve_unsteady(cfdg_solver* s, double dt_phy, int n_steps, int* newton_steps, double* res_vm) {
    if (!s || !(dt_phy > 0) || n_steps < 0) return fail(CFDG_ERR_ARG, "bad arguments");
    return s->solve_unsteady(dt_phy, n_steps, newton_steps, res_vm);
}

cfdg_status cfdg_residual32(cfdg_solver* s, const double* U, double* R) {
    if (!s || !R) return fail(CFDG_ERR_ARG, "null solver or output");
    double* Uin = s->U;
    if (U) {
        TRY(s->upload_aos(U, s->Ub));
        Uin = s->Ub;
    }
    TRY(s->residual32_dev(Uin));
    return s->download_aos32(s->f32out, R);
}

cfdg_status cfdg_jv32(cfdg_solver* s, const double* Ubase, const double* v, double* Jv) {
    if (!s || !Ubase || !v || !Jv) return fail(CFDG_ERR_ARG, "cfdg_jv32: bad arguments");
    TRY(s->upload_aos(Ubase, s->Ub));
    TRY(s->upload_aos(v, s->vtmp));
    TRY(s->jv32_dev(s->Ub, s->vtmp));
    return s->download_aos32(s->f32out, Jv);
}

cfdg_status cfdg_gmres(cfdg_solver* s, const double* Ubase, const double* Rbase, const double* rhs, double* x,
                       int* iters) {
    if (!s || !rhs || !x) return fail(CFDG_ERR_ARG, "cfdg_gmres: bad arguments");
    double* Ud = s->U;
    if (Ubase) {
        TRY(s->upload_aos(Ubase, s->Ub));
        Ud = s->Ub;
    }
    double* Rd = s->R;
    if (Rbase) {
        TRY(s->upload_aos(Rbase, s->Rb));
        Rd = s->Rb;
    }
    TRY(s->upload_aos(rhs, s->rhs));
    int it = 0;
    TRY(s->gmres(Ud, Rd, s->rhs, s->x, &it));
    if (iters) *iters = it;
    return s->download_aos(s->x, x, s->nv, 6);
}

cfdg_status cfdg_norm_vm(cfdg_solver* s, const double* R, double* out) {
    if (!s || !R || !out) return fail(CFDG_ERR_ARG, "null argument");
    TRY(s->upload_aos(R, s->vtmp));
    launch_norm_vm(s->nv, s->nc, s->vtmp, s->g64.vol, s->rs, s->scal + 8, s->st);
    s->launches += 1;
    double v[3];
    TRY(s->read_scalars(8, 3, v));
    *out = v[1] == 0 ? 0.0 : std::sqrt(v[0] / v[1]);
    return CFDG_OK;
}

cfdg_status cfdg_set_krylov(cfdg_solver* s, int mode) {
    if (!s || (mode != CFDG_KRYLOV_HOST && mode != CFDG_KRYLOV_GRAPH && mode != CFDG_KRYLOV_STREAM))
        return fail(CFDG_ERR_ARG, "bad krylov mode");
    if (mode != CFDG_KRYLOV_HOST && !s->gdi) return fail(CFDG_ERR_ARG, "the device drivers need gmres_m <= 128");
    s->cfg.krylov = mode;
    return CFDG_OK;
}

cfdg_status cfdg_reset_newton(cfdg_solver* s) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    s->cfl = s->cfg.cfl0;
    s->step = 0;
    return CFDG_OK;
}

cfdg_status cfdg_get_newton_state(cfdg_solver* s, double* cfl, int* step) {
    if (!s || !cfl || !step) return fail(CFDG_ERR_ARG, "null argument");
    *cfl = s->cfl;
    *step = s->step;
    return CFDG_OK;
}

cfdg_status cfdg_set_newton_state(cfdg_solver* s, double cfl, int step) {
    if (!s || !(cfl > 0.0) || step < 0) return fail(CFDG_ERR_ARG, "bad Newton state");
    s->cfl = cfl;
    s->step = step;
    return CFDG_OK;
}

cfdg_status cfdg_set_cfl_max(cfdg_solver* s, double cfl_max) {
    if (!s || !(cfl_max > 0.0)) return fail(CFDG_ERR_ARG, "bad CFL cap");
    s->cfg.cfl_max = cfl_max;
    if (s->cfl > cfl_max) s->cfl = cfl_max;
    return CFDG_OK;
}

cfdg_status cfdg_newton_step(cfdg_solver* s, double tol, cfdg_step* info, int* converged) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    int cv = 0;
    cfdg_status st = s->newton_step(tol, info, &cv);
    if (converged) *converged = cv;
    return st;
}

cfdg_status cfdg_newton_steps(cfdg_solver* s, double tol, double tol_rho, int k, cfdg_step* trace, int* n_done,
                              int* converged) {
    if (!s || k < 0 || tol_rho < 0) return fail(CFDG_ERR_ARG, "bad arguments");
    int n = 0, cv = 0;
    if (n_done) *n_done = 0;
    if (converged) *converged = 0;
    while (n < k && !cv) {
        int done = 0;
        cfdg_status st;
        if (s->cfg.krylov == CFDG_KRYLOV_GRAPH) {
            st = s->newton_chain(tol, std::min(k - n, (int)cfdg_solver::CHAIN_MAX), trace ? trace + n : nullptr, &done, &cv,
                                 tol_rho);
        } else {
            cfdg_step rec;
            const int step0 = s->step;
            st = s->newton_step(tol, &rec, &cv);
            if (trace) trace[n] = rec;
            done = 1;
            // the density test on the host driver: this step's residual was already low (the
            // update it made is kept)
            if (st == CFDG_OK && !cv && tol_rho > 0.0 && step0 > 5 && rec.res_rho <= tol_rho) cv = 1;
        }
        n += done;
        if (n_done) *n_done = n;
        if (converged) *converged = cv;
        if (st != CFDG_OK) return st;
        if (done == 0) break;
    }
    return CFDG_OK;
}

cfdg_status cfdg_solve_implicit(cfdg_solver* s, double tol, int max_steps, cfdg_step* trace, int* n_steps) {
    if (!s || max_steps < 0) return fail(CFDG_ERR_ARG, "bad arguments");
    TRY(cfdg_reset_newton(s));
    if (s->cfg.krylov == CFDG_KRYLOV_GRAPH && s->cfg.newton_chain > 1) {
        // steps in chains of newton_chain, one host synchronisation per chain
        int n = 0, cv = 0;
        if (n_steps) *n_steps = 0;
        while (n < max_steps) {
            int done = 0;
            const int kk = std::min(max_steps - n, std::min(s->cfg.newton_chain, (int)cfdg_solver::CHAIN_MAX));
            cfdg_status st = s->newton_chain(tol, kk, trace ? trace + n : nullptr, &done, &cv);
            n += done;
            if (n_steps) *n_steps = n;
            if (st != CFDG_OK) return st;
            if (cv) return CFDG_OK;
            if (done == 0) break;
        }
        return fail(CFDG_ERR_NOT_CONVERGED, "solveImplicit reached max_steps above the tolerance");
    }
    int n = 0;
    for (int k = 0; k < max_steps; ++k) {
        cfdg_step rec;
        int cv = 0;
        cfdg_status st = s->newton_step(tol, &rec, &cv);
        if (trace) trace[n] = rec;
        ++n;
        if (n_steps) *n_steps = n;
        if (st != CFDG_OK) return st;
        if (cv) return CFDG_OK;
    }
    if (n_steps) *n_steps = n;
    return fail(CFDG_ERR_NOT_CONVERGED, "solveImplicit reached max_steps above the tolerance");
}

cfdg_status cfdg_vjp(cfdg_solver* s, const double* U, const double* lambda, double* gU) {
    if (!s || !lambda || !gU) return fail(CFDG_ERR_ARG, "cfdg_vjp: null argument");
    double* Uin = s->U;
    if (U) {
        TRY(s->upload_aos(U, s->Ub));
        Uin = s->Ub;
    }
    TRY(s->upload_aos(lambda, s->vtmp));
    TRY(s->vjp_dev(Uin, s->vtmp, s->x));
    return s->download_aos(s->x, gU, s->nv, 6);
}

cfdg_status cfdg_vjp_device(cfdg_solver* s) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    TRY(s->vjp_dev(s->U, s->R, s->x));
    if (s->timing) {
        CK(cudaStreamSynchronize(s->st));
        s->collect();
    }
    return CFDG_OK;
}

cfdg_status cfdg_wall_coefficients(cfdg_solver* s, int tag, double* x_mid, double* cp, double* cf, int* n) {
    if (!s || !n) return fail(CFDG_ERR_ARG, "null solver or count");
    std::vector<int> faces = s->tagged_faces(tag);
    int nw = (int)faces.size();
    *n = nw;
    if (!x_mid && !cp && !cf) return CFDG_OK;
    if (x_mid) {
        const HostMesh& h = s->mesh->h;
        for (int k = 0; k < nw; ++k) x_mid[k] = h.f_xm[h.face_perm[faces[k]]];
    }
    if (!cp && !cf) return CFDG_OK;
    TRY(s->wall_terms(faces));
    if (nw && cp) CK(cudaMemcpyAsync(cp, s->qbuf, sizeof(double) * nw, cudaMemcpyDeviceToHost, s->st));
    if (nw && cf) CK(cudaMemcpyAsync(cf, s->qbuf + s->qcap, sizeof(double) * nw, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_wall_distance(cfdg_solver* s, double* d) {
    if (!s || !d) return fail(CFDG_ERR_ARG, "null solver or output");
    TRY(s->wall_distance());
    std::vector<double> dd(s->nc);
    CK(cudaMemcpy(dd.data(), s->dwall, sizeof(double) * s->nc, cudaMemcpyDeviceToHost));
    const std::vector<int>& perm = s->mesh->h.cell_perm;
    for (int i = 0; i < s->nc; ++i) d[perm[i]] = dd[i];
    return CFDG_OK;
}

cfdg_status cfdg_objective(cfdg_solver* s, int kind, double x0, double x1, double* J, double* dJdU) {
    if (!s || !J) return fail(CFDG_ERR_ARG, "null solver or output");
    if (kind < CFDG_OBJ_PRESSURE_DRAG || kind > CFDG_OBJ_WALL_PRESSURE) return fail(CFDG_ERR_ARG, "unknown objective");
    TRY(s->objective(kind, x0, x1, dJdU ? s->x : nullptr));
    CK(cudaMemcpyAsync(J, s->obuf + 2 * (size_t)s->ocap + (s->nf - s->mesh->h.n_interior), sizeof(double),
                       cudaMemcpyDeviceToHost, s->st));
    if (dJdU) return s->download_aos(s->x, dJdU, s->nv, 6);
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_drag(cfdg_solver* s, double* drag) {
    if (!s || !drag) return fail(CFDG_ERR_ARG, "null solver or output");
    TRY(s->wall_terms(s->tagged_faces(3)));
    CK(cudaMemcpyAsync(drag, s->qbuf + 3 * (size_t)s->qcap, sizeof(double), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_entropy_error(cfdg_solver* s, double* err) {
    if (!s || !err) return fail(CFDG_ERR_ARG, "null solver or output");
    // free-stream entropy (src/Solver.cpp:1621-1625), host IEEE arithmetic
    double g = s->cfg.gamma, M = s->M_inf;
    double T_inf = s->T0 / (1.0 + 0.5 * (g - 1.0) * M * M);
    double P_inf = s->P0 / std::pow(1.0 + 0.5 * (g - 1.0) * M * M, g / (g - 1.0));
    double rho_inf = P_inf / (s->cfg.R_gas * T_inf);
    double S_ref = P_inf / std::pow(rho_inf, g);
    launch_entropy(s->nv, s->nc, s->F, s->U, s->g64.vol, S_ref, s->rs, s->scal + 8, s->st);
    ++s->launches;
    CK(cudaGetLastError());
    double h2[2];
    CK(cudaMemcpyAsync(h2, s->scal + 8, sizeof(h2), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    *err = std::sqrt(h2[0] / h2[1]);
    return CFDG_OK;
}

cfdg_status cfdg_synchronize(cfdg_solver* s) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    CK(cudaStreamSynchronize(s->st));
    return CFDG_OK;
}

cfdg_status cfdg_set_timing(cfdg_solver* s, int on) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    s->timing = on;
    return CFDG_OK;
}

cfdg_status cfdg_kernel_times(cfdg_solver* s, double* a, double* b, double* c, double* d) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    if (a) *a = s->kms[0];
    if (b) *b = s->kms[1];
    if (c) *c = s->kms[2];
    if (d) *d = s->kms[3];
    return CFDG_OK;
}

cfdg_status cfdg_kernel_stats(cfdg_solver* s, double* ms8, long long* n8, int reset) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    for (int k = 0; k < cfdg_solver::NSTAT; ++k) {
        if (ms8) ms8[k] = s->kstat_ms[k];
        if (n8) n8[k] = s->kstat_n[k];
        if (reset) {
            s->kstat_ms[k] = 0;
            s->kstat_n[k] = 0;
        }
    }
    return CFDG_OK;
}

cfdg_status cfdg_flush_l2(cfdg_solver* s, size_t bytes) {
    if (!s) return fail(CFDG_ERR_ARG, "null solver");
    if (bytes > s->l2bytes) {
        cudaFree(s->l2buf);
        s->l2buf = nullptr;
        s->l2bytes = 0;
        CK(cudaMalloc((void**)&s->l2buf, bytes));
        s->l2bytes = bytes;
    }
    CK(cudaMemsetAsync(s->l2buf, ++s->l2fill & 0xff, bytes, s->st));
    return CFDG_OK;
}

cfdg_status cfdg_fp64_pipe_rate(int device, double* fma_per_s) {
    if (!fma_per_s) return fail(CFDG_ERR_ARG, "null argument");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return fail(CFDG_ERR_CUDA, "no such CUDA device");
    CK(cudaSetDevice(device));
    int nsm = 0;
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
    const int blocks = 4 * nsm, threads = 256, iters = 16384;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    double* sink = nullptr;
    cfdg_status rc = CFDG_OK;
    float ms = 0;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess || cudaMalloc((void**)&sink, sizeof(double)) != cudaSuccess) {
        rc = fail(CFDG_ERR_CUDA, "cfdg_fp64_pipe_rate: set-up failed");
    } else {
        launch_fp64_fma_stream(blocks, threads, sink, iters / 8, st);  // warm-up
        cudaEventRecord(e0, st);
        launch_fp64_fma_stream(blocks, threads, sink, iters, st);
        cudaEventRecord(e1, st);
        cudaError_t e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess || ms <= 0) rc = fail(CFDG_ERR_CUDA, std::string("cfdg_fp64_pipe_rate: ") + cudaGetErrorString(e));
    }
    if (rc == CFDG_OK) *fma_per_s = (double)blocks * threads * iters * FP64_STREAM_CHAINS / (ms * 1e-3);
    if (sink) cudaFree(sink);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    return rc;
}

cfdg_status cfdg_launch_count(cfdg_solver* s, long long* n) {
    if (!s || !n) return fail(CFDG_ERR_ARG, "null argument");
    *n = s->launches;
    return CFDG_OK;
}

cfdg_status cfdg_krylov_info(cfdg_solver* s, int* out4) {
    if (!s || !out4) return fail(CFDG_ERR_ARG, "null argument");
    out4[0] = s->cfg.krylov;
    out4[1] = (int)s->graph_body;
    out4[2] = s->cfg.pdl && !s->pdl_failed && !s->use_persistent() ? 1 : 0;
    out4[3] = s->use_persistent() ? 1 : 0;
    return CFDG_OK;
}

}  // extern "C"
