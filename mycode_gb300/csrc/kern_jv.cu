// Exact Jacobian-vector products: the residual kernels instantiated on Dual<R>, so the
// derivative follows the primal operation sequence and branch decisions exactly.  The
// limiter is frozen (phi read, zero derivative), as in the reference's applyJacobian
// (src/Solver.cpp:1366).  The gather adds the time term v * vol/(dt + 1e-30).
#include "launch.hpp"
#include "arnoldi.cuh"

namespace cfdg {

template <class R, int NV>
static void jv_nv(const ResArgs<R>& a) {
    typedef Dual<R> S;
    long nc = a.m.nc, nf = a.m.nf;
    if (a.ev) cudaEventRecord(a.ev[0], a.stream);
    k_prim<S, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>((int)nc, a.F, a.U, a.W);
    if (a.ev) cudaEventRecord(a.ev[1], a.stream);
    if (a.cfx.nbr)
        k_grad_cf<S, NV, R, false><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.cfx, a.F, a.U, a.W, a.G, a.phi,
                                                                                 0, nullptr);
    else
        k_grad<S, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, 0, nullptr, nullptr);
    if (NV == 6) k_sst_cell<S, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.F, a.W, a.G, a.dwall, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[2], a.stream);
    k_flux<S, NV><<<blocks_for(nf), tpb_for(nf), 0, a.stream>>>(a.m, a.F, a.U, a.W, a.G, a.phi, a.FA, a.T, nullptr);
    if (a.ev) cudaEventRecord(a.ev[3], a.stream);
    k_gather<R, NV><<<blocks_for(nc), tpb_for(nc), 0, a.stream>>>(a.m, a.FA.d, a.FA.n, a.out, nc, a.diag_v, a.dt,
                                                         NV == 6 ? a.T.d + 2 * nc : nullptr);
    if (a.ev) cudaEventRecord(a.ev[4], a.stream);
}

// a.ev (optional): 3 events around the gradient (+ SST) and flux stages
template <class R, int NV>
static void jv_mid_nv(const ResArgs<R>& a) {
    typedef Dual<R> S;
    long nc = a.m.nc, nf = a.m.nf;
    // write views: derivative planes only when the value planes are current (a.tangent)
    Field<R> Gw = a.G, Tw = a.T;
    if (a.tangent) Gw.v = Tw.v = nullptr;
    if (a.ev) cudaEventRecord(a.ev[0], a.stream);
    if (a.cfx.nbr)
        launch_k(a.pdl, k_grad_cf<S, NV, R, true>, dim3(blocks_for(nc)), dim3(tpb_for(nc)), a.stream, a.m, a.cfx, a.F,
                 a.U, a.W, Gw, a.phi, 0, a.done);
    else
        launch_k(a.pdl, k_grad<S, NV, R>, dim3(blocks_for(nc)), dim3(tpb_for(nc)), a.stream, a.m, a.F, a.U, a.W, Gw,
                 a.phi, 0, a.done, (const int*)nullptr);
    if (NV == 6)
        launch_k(a.pdl, k_sst_cell<S, NV, R>, dim3(blocks_for(nc)), dim3(tpb_for(nc)), a.stream, a.m, a.F, a.W, a.G,
                 a.dwall, Tw, a.done);
    if (a.ev) cudaEventRecord(a.ev[1], a.stream);
    launch_k(a.pdl, k_flux<S, NV, R>, dim3(blocks_for(nf)), dim3(tpb_for(nf)), a.stream, a.m, a.F, a.U, a.W, a.G,
             (const R*)a.phi, a.FA, a.T, a.done);
    if (a.ev) cudaEventRecord(a.ev[2], a.stream);
}

template <>
void launch_jv_mid<double>(const ResArgs<double>& a) {
    if (a.nv == 6) jv_mid_nv<double, 6>(a);
    else jv_mid_nv<double, 4>(a);
}

template <>
void launch_jv_mid<float>(const ResArgs<float>& a) {
    if (a.nv == 6) jv_mid_nv<float, 6>(a);
    else jv_mid_nv<float, 4>(a);
}

template <>
void launch_jv<double>(const ResArgs<double>& a) {
    if (a.nv == 6) jv_nv<double, 6>(a);
    else jv_nv<double, 4>(a);
}

template <>
void launch_jv<float>(const ResArgs<float>& a) {
    if (a.nv == 6) jv_nv<float, 6>(a);
    else jv_nv<float, 4>(a);
}

template <class T>
int arnoldi_blocks(int nv) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (nv == 6) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_arnoldi<T, 6>, RED_THREADS, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_arnoldi<T, 4>, RED_THREADS, 0);
    long b = (long)sms * per;
    return (int)(b < RED_BLOCKS ? b : RED_BLOCKS);
}

template <class T>
cudaError_t launch_arnoldi(int nv, const ArnoldiArgs<T>& a, cudaGraphConditionalHandle h, int blocks, bool coop,
                           cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(RED_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = coop ? attr : nullptr;
    cfg.numAttrs = coop ? 1 : 0;
    if (nv == 6) return cudaLaunchKernelEx(&cfg, k_arnoldi<T, 6>, a, h);
    return cudaLaunchKernelEx(&cfg, k_arnoldi<T, 4>, a, h);
}

template int arnoldi_blocks<float>(int);
template int arnoldi_blocks<double>(int);
template cudaError_t launch_arnoldi<float>(int, const ArnoldiArgs<float>&, cudaGraphConditionalHandle, int, bool,
                                           cudaStream_t);
template cudaError_t launch_arnoldi<double>(int, const ArnoldiArgs<double>&, cudaGraphConditionalHandle, int, bool,
                                            cudaStream_t);

}  // namespace cfdg
