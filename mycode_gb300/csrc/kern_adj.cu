// Adjoint (VJP) kernels of the FP64 residual: forward recomputation of the primitives,
// gradients and limiter (and the SST cell terms), then the reverse face and cell kernels
// of adjoint_kernels.cuh.
#include "adjoint_kernels.cuh"
#include "launch.hpp"

namespace cfdg {

template <int NV>
static void vjp_nv(const ResArgs<double>& a, const double* lam, const AdjBufs& b, double* gU) {
    long nc = a.m.nc, nf = a.m.nf;
    int limited = a.F.spatial == SP_LIMITED ? 1 : 0;
    if (a.ev) cudaEventRecord(a.ev[0], a.stream);
    k_prim<double, NV><<<grid_for(nc), 256, 0, a.stream>>>((int)nc, a.F, a.U, a.W);
    if (a.gft && a.m.nfi > 0) {  // the residual's split gradient (face terms once per face): the same G and phi
        k_grad_faces64<NV><<<grid_for(a.m.nfi, 256), 256, 0, a.stream>>>(a.m, a.W, a.gft);
        k_grad64<NV, true><<<grid_for(nc, (int)GRAD64_THREADS), GRAD64_THREADS, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G,
                                                                                              a.phi, limited, nullptr,
                                                                                              a.gft);
    } else {
        k_grad64<NV, false><<<grid_for(nc, (int)GRAD64_THREADS), GRAD64_THREADS, 0, a.stream>>>(a.m, a.F, a.U, a.W,
                                                                                               a.G, a.phi, limited,
                                                                                               nullptr, nullptr);
    }
    if (NV == 6) k_sst_cell<double, NV><<<grid_for(nc), 256, 0, a.stream>>>(a.m, a.F, a.W, a.G, a.dwall, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[1], a.stream);
    k_flux_adj<NV><<<grid_for(nf, 128), 128, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, lam, b, a.T);
    if (a.ev) cudaEventRecord(a.ev[2], a.stream);
    k_adj_cell1<NV><<<grid_for(nc, 128), 128, 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, limited, b, lam,
                                                            a.dwall);
    if (a.ev) cudaEventRecord(a.ev[3], a.stream);
    k_adj_cell2<NV><<<grid_for(nc, 128), 128, 0, a.stream>>>(a.m, a.F, a.U, a.W, b, gU);
    if (a.ev) cudaEventRecord(a.ev[4], a.stream);
}

void launch_vjp64(const ResArgs<double>& a, const double* lam, const AdjBufs& b, double* gU) {
    if (a.nv == 6) vjp_nv<6>(a, lam, b, gU);
    else vjp_nv<4>(a, lam, b, gU);
}

}  // namespace cfdg
