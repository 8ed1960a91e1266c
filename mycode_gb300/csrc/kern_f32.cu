// FP32 residual and FP32-vector Krylov kernels (mixed precision: FP32 Krylov basis,
// FP64 reductions).  FMA contraction on.
#include "launch.hpp"

namespace cfdg {

template <int NV>
static void residual_nv(const ResArgs<float>& a) {
    long nc = a.m.nc, nf = a.m.nf;
    if (a.ev) cudaEventRecord(a.ev[0], a.stream);
    k_prim<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>((int)nc, a.F, a.U, a.W);
    if (a.ev) cudaEventRecord(a.ev[1], a.stream);
    if (a.cfx.nbr)
        k_grad_cf<float, NV, float, false><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.cfx, a.F, a.U, a.W, a.G,
                                                                                         a.phi, a.do_limiter, nullptr);
    else
        k_grad<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.do_limiter,
                                                                       nullptr, nullptr);
    if (NV == 6) k_sst_cell<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.W, a.G, a.dwall, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[2], a.stream);
    k_flux<float, NV><<<blocks_for(nf), tpb_for(nf), 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.FA, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[3], a.stream);
    k_gather<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.FA.v, a.FA.n, a.out, nc, a.diag_v, a.dt,
                                                           NV == 6 ? a.T.v + 2 * nc : nullptr);
    if (a.ev) cudaEventRecord(a.ev[4], a.stream);
}

template <>
void launch_residual<float>(const ResArgs<float>& a) {
    if (a.nv == 6) residual_nv<6>(a);
    else residual_nv<4>(a);
}

template <int NV>
static void values_nv(const ResArgs<float>& a) {
    long nc = a.m.nc;
    k_prim<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>((int)nc, a.F, a.U, a.W);
    if (a.cfx.nbr)
        k_grad_cf<float, NV, float, false><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.cfx, a.F, a.U, a.W, a.G,
                                                                                         a.phi, 0, nullptr);
    else
        k_grad<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, 0, nullptr,
                                                                       nullptr);
    if (NV == 6) k_sst_cell<float, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.W, a.G, a.dwall, a.T, nullptr);
}

template <>
void launch_values<float>(const ResArgs<float>& a) {
    if (a.nv == 6) values_nv<6>(a);
    else values_nv<4>(a);
}


template <>
void launch_dot<float>(int nv, long nc, const float* a, const float* b, RedScratch rs, double* out, cudaStream_t s) {
    NV_SWITCH(nv, (k_dot<float, float, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, a, b, rs, out)));
}
template <>
void launch_mgs<float>(int nv, long nc, float* w, const float* vprev, const double* hprev, const float* vnext,
                       RedScratch rs, double* out, cudaStream_t s) {
    NV_SWITCH(nv, (k_mgs<float, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, w, vprev, hprev, vnext, rs, out)));
}
template <>
void launch_scale_guard<float>(long n, float* x, const double* h, double thresh, cudaStream_t s) {
    k_scale_guard<float><<<red_grid(n), RED_THREADS, 0, s>>>(n, x, h, thresh);
}
template <>
void launch_scale_from<float>(long n, float* x, const double* a, const double* sc, int invert, cudaStream_t s) {
    k_scale_from<float, double><<<red_grid(n), RED_THREADS, 0, s>>>(n, x, a, sc, invert);
}
template <>
void launch_precond_apply<float>(int nv, long nc, const float* V, const double* D, float* z, RedScratch rs,
                                 double* out_sq, cudaStream_t s) {
    NV_SWITCH(nv, (k_precond_apply<float, float, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, V, D, z, rs, out_sq)));
}
template <>
void launch_gmres_solution<float>(int nv, long nc, const float* V, long vstride, const double* y, int k,
                                  const double* D, double* x, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_solution<float, NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, V, vstride, y, k, D, x)));
}
template <>
void launch_aos_to_soa<float>(long nc, int np, int stride, const double* aos, const int* perm, float* soa,
                                 cudaStream_t s) {
    k_aos_to_soa<float><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, np, stride, aos, perm, soa);
}
template <>
void launch_soa_to_aos<float>(long nc, int np, int stride, const float* soa, const int* perm, double* aos,
                                 cudaStream_t s) {
    k_soa_to_aos<float><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, np, stride, soa, perm, aos);
}
template <>
void launch_soa_to_rows<float>(long nc, int np, int stride, const float* soa, const int* iperm, double* aos,
                               cudaStream_t s) {
    k_soa_to_rows<float><<<grid_for(nc, ROW_BLOCK), ROW_BLOCK, 0, s>>>(nc, np, stride, soa, iperm, aos);
}

__global__ void k_convert_f32(long n, const double* __restrict__ in, float* __restrict__ out) {
    for (long q = (long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x) out[q] = (float)in[q];
}
template <>
void launch_convert<float>(long n, const double* in, float* out, cudaStream_t s) {
    k_convert_f32<<<red_grid(n), RED_THREADS, 0, s>>>(n, in, out);
}

// ---- device-resident GMRES
template <>
void launch_gmres_start<float>(long n, float* V0, const double* rhs, const GmresDev& d, int m, double tol,
                               cudaGraphConditionalHandle h, const double* bsq, cudaStream_t s) {
    k_gmres_start<float><<<red_grid(n), RED_THREADS, 0, s>>>(n, V0, rhs, d, m, tol, h, bsq);
}
void launch_mixed_pre(int nv, const MeshView<float>& m, const Flow<float>& F, const double* U, const double* Ub,
                      const double* W,
                      const double* phi, const double* mut, const double* cfl, const double* dt_in, float* U32,
                      float* phi32, float* dt32, double* D, float* Dinv32, cudaStream_t s) {
    NV_SWITCH(nv, (k_mixed_pre<NVC><<<blocks_for(m.nc), tpb_for(m.nc), 0, s>>>(m, F, U, Ub, W, phi, mut, cfl, dt_in, U32,
                                                                             phi32, dt32, D, Dinv32)));
}
template <>
void launch_gmres_z<float>(int nv, long nc, const float* V, long L, const float* Dinv, float* z, const GmresDev& d,
                        cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_z<float, NVC><<<red_grid(nc), RED_THREADS, 0, s>>>(nc, V, L, Dinv, z, d)));
}
template <>
void launch_gmres_dinv<float>(int nv, long nc, const double* D, float* Dinv, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_dinv<float, NVC><<<red_grid((nv == 6 ? 3 : 1) * nc), RED_THREADS, 0, s>>>(nc, D, Dinv)));
}
template <>
void launch_gmres_multidot<float>(long L, const float* w, const float* V, const GmresDev& d, double* h, cudaStream_t s) {
    k_gmres_multidot<float><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d, h);
}
template <>
void launch_gmres_prim_z<float>(int nv, long nc, const Flow<float>& F, const float* U, float* V, long L, const float* Dinv,
                             float* z, Field<float> W, const float* w, const GmresDev& d, cudaGraphConditionalHandle h,
                             cudaStream_t s) {
    // blocks of RED_THREADS (every block sums the gather kernel's partials: wide blocks keep
    // that short, and at most RED_BLOCKS of them and one wave, grid-stride over the cells:
    // prim_z_grid) and one block more for the Givens step; the partials it sums are the
    // gather kernel's (gather_grid blocks with this basis precision)
    GmresDev dd = d;
    dd.nb1 = (int)gather_grid(nc, 4);
    NV_SWITCH(nv, (k_gmres_prim_z<float, NVC><<<prim_z_grid<float, NVC>(nc), RED_THREADS, 0, s>>>((int)nc, F, U, V, L, Dinv, z, W, w, dd,
                                                                                  h)));
}
template <>
void launch_gmres_gather_dot<float>(int nv, const MeshView<float>& m, const float* FA, float* w, const float* z, const float* dt,
                                 const float* src, const float* V, long L, const GmresDev& d, cudaStream_t s, bool pdl, bool split) {
    if (split) {  // the gather, then the dots streamed on their own
        NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_w<float, NVC>, dim3(grid_for(m.nc, 256)), dim3(256), s, m, FA,
                               (long)m.nf, w, z, dt, src, d));
        NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_dot<float, NVC, true>, dim3(gather_grid(m.nc, 4)), dim3(RED_THREADS), s,
                               m, FA, (long)m.nf, w, z, dt, src, V, L, d));
        return;
    }
    NV_SWITCH(nv, launch_k(pdl, k_gmres_gather_dot<float, NVC>, dim3(gather_grid(m.nc, 4)), dim3(RED_THREADS), s, m, FA,
                           (long)m.nf,
                           w, z, dt, src, V, L, d));
}
template <>
void launch_gmres_update_dot<float>(long L, float* w, const float* V, const GmresDev& d, cudaStream_t s) {
    k_gmres_update_dot<float><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d);
}
template <>
void launch_gmres_update_final<float>(long L, const float* w, float* V, const GmresDev& d, cudaGraphConditionalHandle h,
                                   cudaStream_t s) {
    k_gmres_update_final<float><<<kry_grid(L), RED_THREADS, 0, s>>>(L, w, V, d, h);
}
template <>
void launch_gmres_solution_dev<float>(int nv, long nc, const float* V, long L, const GmresDev& d, const double* D,
                                   const float* Dinv32, double* x, cudaStream_t s) {
    NV_SWITCH(nv, (k_gmres_solution_dev<float, NVC><<<blocks_for(nc), tpb_for(nc), 0, s>>>(nc, V, L, d, D, Dinv32, x)));
}

}  // namespace cfdg
