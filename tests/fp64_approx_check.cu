// Device check of ex_rcp / ex_rsqrt (phd_physics.cuh: the hardware approximations
// refined by two Newton-Raphson steps) against CUDA's correctly rounded reciprocal and
// square root: the largest difference in units of the last place over n arguments
// spread log-uniformly over [1e-20, 1e20] (positive normal numbers, the iteration's
// domain).  Prints: n, max ulp of ex_rcp, max ulp of ex_rsqrt.  Test-only: compiled
// and run by tests/test_gpu_fp64_approx.py.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>
#include "phd_physics.cuh"

__device__ __forceinline__ long long ulps(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    return ia > ib ? ia - ib : ib - ia;
}

__global__ void k_check(int n, unsigned long long *max_rcp, unsigned long long *max_rsqrt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // log-uniform over 40 decades, with the low bits of the index perturbing the mantissa
    const double t = -20.0 + 40.0 * (double(i) + 0.5) / double(n);
    const double x = exp10(t) * (1.0 + 1e-3 * double(i & 1023) / 1024.0);
    const long long a = ulps(phd::ex_rcp(x), __drcp_rn(x));
    const long long b = ulps(phd::ex_rsqrt(x), __drcp_rn(__dsqrt_rn(x)));
    atomicMax(max_rcp, (unsigned long long)a);
    atomicMax(max_rsqrt, (unsigned long long)b);
}

int main(int argc, char **argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 1 << 22;
    unsigned long long *d = nullptr, h[2] = {0, 0};
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    k_check<<<(n + 255) / 256, 256>>>(n, d, d + 1);
    if (cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    cudaFree(d);
    printf("%d %llu %llu\n", n, h[0], h[1]);
    return 0;
}
