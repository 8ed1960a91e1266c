// Evaluates the integer-pipe FP64 operations of exact64.cuh next to the FP64 instructions
// they stand for, on the doubles of a binary file; writes the bit patterns of both.
// Usage: exact64_check in.bin out.bin  (in: n doubles; out: n x 10 uint64)
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>
#include "../../mycode_gb300/csrc/exact64.cuh"

using namespace cfdg;

__global__ void k_check(int n, const double* __restrict__ x, unsigned long long* __restrict__ o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double a = x[i], b = x[(i * 7 + 3) % n];
    volatile double h = 0.5, t = 2.0;  // keeps the FP64 forms FP64 instructions
    unsigned long long* r = o + 10ull * i;
    r[0] = __double_as_longlong(half_exact(a));
    r[1] = __double_as_longlong(a * h);
    r[2] = __double_as_longlong(twice_exact(a));
    r[3] = __double_as_longlong(a * t);
    r[4] = lt_exact(a, b);
    r[5] = a < b;
    r[6] = gt0_exact(a);
    r[7] = a > 0.0;
    r[8] = lt0_exact(a);
    r[9] = a < 0.0;
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<double> h;
    double v;
    while (fread(&v, sizeof v, 1, f) == 1) h.push_back(v);
    fclose(f);
    const int n = (int)h.size();
    if (n == 0) return 4;
    double* dx = nullptr;
    unsigned long long* dout = nullptr;
    if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess) return 5;
    if (cudaMalloc(&dout, 10ull * n * sizeof(unsigned long long)) != cudaSuccess) return 5;
    cudaMemcpy(dx, h.data(), n * sizeof(double), cudaMemcpyHostToDevice);
    k_check<<<(n + 255) / 256, 256>>>(n, dx, dout);
    std::vector<unsigned long long> out(10ull * n);
    if (cudaMemcpy(out.data(), dout, out.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess)
        return 6;
    f = fopen(argv[2], "wb");
    if (!f) return 7;
    fwrite(out.data(), sizeof(unsigned long long), out.size(), f);
    fclose(f);
    cudaFree(dx);
    cudaFree(dout);
    return 0;
}
