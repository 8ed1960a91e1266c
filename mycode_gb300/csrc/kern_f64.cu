// FP64 kernels, compiled with --fmad=false: the residual, the pseudo-time kernels and
// the FP64 Krylov vector kernels reproduce the reference's CPU arithmetic.
#include "launch.hpp"

namespace cfdg {

template <int NV>
static void residual_nv(const ResArgs<double>& a) {
    long nc = a.m.nc, nf = a.m.nf;
    if (a.ev) cudaEventRecord(a.ev[0], a.stream);
    if (!a.prim_done) k_prim<double, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>((int)nc, a.F, a.U, a.W);
    if (a.ev) cudaEventRecord(a.ev[1], a.stream);
    {
        const unsigned t = tpb_for(nc) < GRAD64_THREADS ? tpb_for(nc) : GRAD64_THREADS;
        if (a.gft && a.m.nfi > 0) {
            k_grad_faces64<NV><<<grid_for(a.m.nfi, 256), 256, 0, a.stream>>>(a.m, a.W, a.gft);
            k_grad64<NV, true><<<grid_for(nc, (int)t), t, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.do_limiter,
                                                                         a.lim_dev, a.gft);
        } else {
            k_grad64<NV, false><<<grid_for(nc, (int)t), t, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.do_limiter,
                                                                          a.lim_dev, nullptr);
        }
    }
    if (NV == 6) k_sst_cell<double, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.W, a.G, a.dwall, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[2], a.stream);
    {
        const unsigned t = tpb_for(nf) < FLUX64_THREADS ? tpb_for(nf) : FLUX64_THREADS;
        k_flux64<NV><<<grid_for(nf, (int)t), t, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.FA, a.T);
    }
    if (a.ev) cudaEventRecord(a.ev[3], a.stream);
    if (a.rows_out)
        k_gather_rows<NV><<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, a.stream>>>(a.m, a.FA.v, a.FA.n,
                                                                               NV == 6 ? a.T.v + 2 * nc : nullptr,
                                                                               a.iperm, a.rows_out);
    else if (a.norms_out)
        k_gather_norms<NV><<<red_grid(nc), RED_THREADS, 0, a.stream>>>(a.m, a.FA.v, a.FA.n, a.out,
                                                                        NV == 6 ? a.T.v + 2 * nc : nullptr, a.rhs_out,
                                                                        a.rs, a.norms_out, a.flag);
    else
        k_gather<double, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.FA.v, a.FA.n, a.out, nc, a.diag_v,
                                                                           a.dt, NV == 6 ? a.T.v + 2 * nc : nullptr);
    if (a.ev) cudaEventRecord(a.ev[4], a.stream);
}

template <>
void launch_residual<double>(const ResArgs<double>& a) {
    if (a.nv == 6) residual_nv<6>(a);
    else residual_nv<4>(a);
}

void launch_prim64(int nv, long nc, const Flow<double>& F, Field<double> U, Field<double> W, cudaStream_t s) {
    if (nv == 6) k_prim<double, 6><<<blocks_for(nc), tpb_for(nc), 0, s>>>((int)nc, F, U, W);
    else k_prim<double, 4><<<blocks_for(nc), tpb_for(nc), 0, s>>>((int)nc, F, U, W);
}

void launch_rows_prim(int nv, long nc, const Flow<double>& F, const double* aos, const int* iperm, Field<double> U,
                      Field<double> W, cudaStream_t s) {
    if (nv == 6) k_rows_prim<6><<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, s>>>((int)nc, F, aos, iperm, U, W);
    else k_rows_prim<4><<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, s>>>((int)nc, F, aos, iperm, U, W);
}

void launch_rows_to_soa(long nc, int np, int stride, const double* aos, const int* iperm, double* soa, cudaStream_t s) {
    k_rows_to_soa<<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, s>>>(nc, np, stride, aos, iperm, soa);
}
template <>
void launch_soa_to_rows<double>(long nc, int np, int stride, const double* soa, const int* iperm, double* aos,
                                cudaStream_t s) {
    k_soa_to_rows<double><<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, s>>>(nc, np, stride, soa, iperm, aos);
}


template <>
void launch_dot<double>(int nv, long nc, const double* a, const double* b, RedScratch rs, double* out, cudaStream_t s) {
    NV_SWITCH(nv, (k_dot<double, double, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, a, b, rs, out)));
}
template <>
void launch_mgs<double>(int nv, long nc, double* w, const double* vprev, const double* hprev, const double* vnext,
                        RedScratch rs, double* out, cudaStream_t s) {
    NV_SWITCH(nv, (k_mgs<double, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, w, vprev, hprev, vnext, rs, out)));
}
template <>
void launch_scale_guard<double>(long n, double* x, const double* h, double thresh, cudaStream_t s) {
    k_scale_guard<double><<<red_grid(n), RED_THREADS, 0, s>>>(n, x, h, thresh);
}
template <>
void launch_scale_from<double>(long n, double* x, const double* a, const double* sc, int invert, cudaStream_t s) {
    k_scale_from<double, double><<<red_grid(n), RED_THREADS, 0, s>>>(n, x, a, sc, invert);
}
template <>
void launch_precond_apply<double>(int nv, long nc, const double* V, const double* D, double* z, RedScratch rs,
                                  double* out_sq, cudaStream_t s) {
    NV_SWITCH(nv, (k_precond_apply<double, double, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, V, D, z, rs, out_sq)));
}
template <>
void launch_gmres_solution<double>(int nv, long nc, const double* V, long vstride, const double* y, int k,
                                   const double* D, double* x, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_solution<double, NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, V, vstride, y, k, D, x)));
}
template <>
void launch_aos_to_soa<double>(long nc, int np, int stride, const double* aos, const int* perm, double* soa,
                                 cudaStream_t s) {
    k_aos_to_soa<double><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, np, stride, aos, perm, soa);
}
template <>
void launch_soa_to_aos<double>(long nc, int np, int stride, const double* soa, const int* perm, double* aos,
                                 cudaStream_t s) {
    k_soa_to_aos<double><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, np, stride, soa, perm, aos);
}

void launch_fd_perturb(long n, const double* U, const double* v, const double* u_sq, const double* v_sq, double* Up,
                       double* eps, cudaStream_t s) {
    k_fd_perturb<<<red_grid(n), RED_THREADS, 0, s>>>(n, U, v, u_sq, v_sq, Up, eps);
}
void launch_fd_combine(int nv, long nc, const double* Rp, const double* Rb, const double* v, const double* eps,
                       const double* vol, const double* dt, double* Jv, cudaStream_t s) {
    NV_SWITCH(nv, (k_fd_combine<NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, Rp, Rb, v, eps, vol, dt, Jv)));
}
void launch_norm_vm(int nv, long nc, const double* R, const double* vol, RedScratch rs, double* out3, cudaStream_t s) {
    NV_SWITCH(nv, (k_norm_vm<NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, R, vol, rs, out3)));
}
void launch_step_norms(int nv, long nc, const double* R, const double* vol, double* rhs, RedScratch rs, double* out4,
                       int* flag, cudaStream_t s) {
    NV_SWITCH(nv, (k_step_norms<NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, R, vol, rhs, rs, out4, flag)));
}
void launch_local_dt(int nv, const MeshView<double>& m, const Flow<double>& F, const double* U, const double* W,
                     double cfl, double* dt, cudaStream_t s, const double* cfl_dev) {
    NV_SWITCH(nv, (k_local_dt<NVC><<<blocks_for(m.nc), tpb_for(m.nc), 0, s>>>(m, F, U, W, cfl, dt, cfl_dev)));
}
void launch_newton_update_chain(int nv, long nc, double* U, const double* dU, const double* norms, double tol,
                                double gam, double wmin, int* bad, const NewtonCtl& c, int k, int step, double ulim,
                                cudaStream_t s) {
    NV_SWITCH(nv, (k_newton_update_chain<NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, U, dU, norms, tol, gam, wmin,
                                                                                     bad, c, k, step, ulim)));
}
void launch_precond(int nv, const MeshView<double>& m, const Flow<double>& F, const double* U, const double* W,
                    const double* dt, double* D, const double* mut, cudaStream_t s) {
    NV_SWITCH(nv, (k_precond<NVC><<<blocks_for(m.nc), tpb_for(m.nc), 0, s>>>(m, F, U, W, dt, D, mut)));
}
void launch_newton_update_dev(int nv, long nc, double* U, const double* dU, const double* norms, double tol, double gam,
                              double wmin, int* bad, cudaStream_t s) {
    NV_SWITCH(nv, (k_newton_update_dev<NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, U, dU, norms, tol, gam, wmin,
                                                                                   bad)));
}
void launch_explicit_update(int nv, long nc, double* U, const double* R, const double* vol, double dt, int* bad,
                            cudaStream_t s) {
    NV_SWITCH(nv, (k_explicit_update<NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, U, R, vol, dt, bad)));
}
void launch_unsteady_rhs(int nv, long nc, const double* U, const double* Uold, const double* R, const double* vol,
                         double dt, double* rhs, RedScratch rs, double* out2, cudaStream_t s) {
    NV_SWITCH(nv, (k_unsteady_rhs<NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, U, Uold, R, vol, dt, rhs, rs, out2)));
}
void launch_relaxed_add(int nv, long nc, double* U, const double* dU, double relax, int* bad, cudaStream_t s) {
    NV_SWITCH(nv, (k_relaxed_add<NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, U, dU, relax, bad)));
}
void launch_fill(long n, double* x, double v, cudaStream_t s) { k_fill<<<red_grid(n), RED_THREADS, 0, s>>>(n, x, v); }

// FP64 pipe probe: FP64_STREAM_CHAINS independent chains x <- fma(x, a, b) per thread, so
// every FP64 pipe issue slot can be filled; the result is stored only under a condition
// no chain meets (x stays finite and positive), which keeps the chains live.
__global__ void __launch_bounds__(256) k_fp64_fma_stream(double* sink, int iters, double a, double b) {
    double x[FP64_STREAM_CHAINS];
#pragma unroll
    for (int k = 0; k < FP64_STREAM_CHAINS; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < FP64_STREAM_CHAINS; ++k) x[k] = fma(x[k], a, b);
    }
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < FP64_STREAM_CHAINS; ++k) acc += x[k];
    if (acc < 0.0) sink[0] = acc;
}

void launch_fp64_fma_stream(int blocks, int threads, double* sink, int iters, cudaStream_t s) {
    k_fp64_fma_stream<<<blocks, threads, 0, s>>>(sink, iters, 0.999999, 1e-6);
}
void launch_newton_update(int nv, long nc, double* U, const double* dU, double relax, double gam, double wmin, int* bad,
                          cudaStream_t s) {
    NV_SWITCH(nv, (k_newton_update<NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, U, dU, relax, gam, wmin, bad)));
}

// ---- device-resident GMRES
void launch_gmres_backsub(const GmresDev& d, cudaStream_t s) { k_gmres_backsub<<<1, 32, 0, s>>>(d); }
template <>
void launch_gmres_start<double>(long n, double* V0, const double* rhs, const GmresDev& d, int m, double tol,
                                cudaGraphConditionalHandle h, const double* bsq, cudaStream_t s) {
    k_gmres_start<double><<<red_grid(n), RED_THREADS, 0, s>>>(n, V0, rhs, d, m, tol, h, bsq);
}
template <>
void launch_gmres_z<double>(int nv, long nc, const double* V, long L, const double* Dinv, double* z, const GmresDev& d,
                        cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_z<double, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, V, L, Dinv, z, d)));
}
template <>
void launch_gmres_dinv<double>(int nv, long nc, const double* D, double* Dinv, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_dinv<double, NVC><<<red_grid((nv == 6 ? 3 : 1) * nc), RED_THREADS, 0, s>>>(nc, D, Dinv)));
}
template <>
void launch_gmres_multidot<double>(long L, const double* w, const double* V, const GmresDev& d, double* h, cudaStream_t s) {
    k_gmres_multidot<double><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d, h);
}
template <>
void launch_gmres_prim_z<double>(int nv, long nc, const Flow<double>& F, const double* U, double* V, long L, const double* Dinv,
                             double* z, Field<double> W, const double* w, const GmresDev& d, cudaGraphConditionalHandle h,
                             cudaStream_t s) {
    // blocks of RED_THREADS (every block sums the gather kernel's partials: wide blocks keep
    // that short, and at most RED_BLOCKS of them and one wave, grid-stride over the cells:
    // prim_z_grid) and one block more for the Givens step; the partials it sums are the
    // gather kernel's (gather_grid blocks with this basis precision)
    GmresDev dd = d;
    dd.nb1 = (int)gather_grid(nc, 8);
    NV_SWITCH(nv, (k_gmres_prim_z<double, NVC><<<prim_z_grid<double, NVC>(nc), RED_THREADS, 0, s>>>((int)nc, F, U, V, L, Dinv, z, W, w, dd,
                                                                                  h)));
}
template <>
void launch_gmres_gather_dot<double>(int nv, const MeshView<double>& m, const double* FA, double* w, const double* z, const double* dt,
                                 const double* src, const double* V, long L, const GmresDev& d, cudaStream_t s, bool pdl, bool split) {
    if (split) {  // the gather, then the dots streamed on their own
        NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_w<double, NVC>, dim3(grid_for(m.nc, 256)), dim3(256), s, m, FA,
                               (long)m.nf, w, z, dt, src, d));
        NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_dot<double, NVC, true>, dim3(gather_grid(m.nc, 8)), dim3(RED_THREADS), s,
                               m, FA, (long)m.nf, w, z, dt, src, V, L, d));
        return;
    }
    NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_dot<double, NVC>, dim3(gather_grid(m.nc, 8)), dim3(RED_THREADS), s, m, FA,
                           (long)m.nf,
                           w, z, dt, src, V, L, d));
}
template <>
void launch_gmres_update_dot<double>(long L, double* w, const double* V, const GmresDev& d, cudaStream_t s) {
    k_gmres_update_dot<double><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d);
}
template <>
void launch_gmres_update_final<double>(long L, const double* w, double* V, const GmresDev& d, cudaGraphConditionalHandle h,
                                   cudaStream_t s) {
    k_gmres_update_final<double><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d, h);
}
template <>
void launch_gmres_solution_dev<double>(int nv, long nc, const double* V, long L, const GmresDev& d, const double* D,
                                   const double* Dinv32, double* x, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_solution_dev<double, NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, V, L, d, D, Dinv32, x)));
}

}  // namespace cfdg
