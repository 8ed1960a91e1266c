// tanh_sat (the SST model's tanh, csrc/sst.cuh) against CUDA's tanh and tanhf on the
// given values: writes both results' bits for every value (test-only program).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../mycode_gb300/csrc/sst.cuh"

__global__ void k_check(int n, const double* __restrict__ x, unsigned long long* __restrict__ o) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = x[i];
    const float f = (float)d;
    o[4 * i + 0] = (unsigned long long)__double_as_longlong(cfdg::tanh_sat(d));
    o[4 * i + 1] = (unsigned long long)__double_as_longlong(tanh(d));
    o[4 * i + 2] = (unsigned long long)__float_as_uint(cfdg::tanh_sat(f));
    o[4 * i + 3] = (unsigned long long)__float_as_uint(tanhf(f));
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* fi = std::fopen(argv[1], "rb");
    if (!fi) return 2;
    std::vector<double> h;
    double v;
    while (std::fread(&v, sizeof v, 1, fi) == 1) h.push_back(v);
    std::fclose(fi);
    const int n = (int)h.size();
    double* dx = nullptr;
    unsigned long long* dout = nullptr;
    if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess || cudaMalloc(&dout, 32ull * n) != cudaSuccess) return 3;
    cudaMemcpy(dx, h.data(), sizeof(double) * n, cudaMemcpyHostToDevice);
    k_check<<<(n + 255) / 256, 256>>>(n, dx, dout);
    std::vector<unsigned long long> out(4ull * n);
    if (cudaMemcpy(out.data(), dout, 32ull * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 4;
    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo) return 2;
    std::fwrite(out.data(), sizeof(unsigned long long), out.size(), fo);
    std::fclose(fo);
    cudaFree(dx);
    cudaFree(dout);
    return 0;
}
