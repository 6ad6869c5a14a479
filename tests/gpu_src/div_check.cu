// Checks div_by() (engine.cuh: division with a rounded reciprocal and one
// correction step) against IEEE division on the GPU: random divisors over a
// wide exponent range, random numerators, and the counts of mismatches.
// Built and run by tests/test_division.py.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#include "engine.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t x) {   // splitmix64 finaliser
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}
// a double with a random 52-bit mantissa, a random sign and an exponent in [lo, hi]
__device__ __forceinline__ double rnd(uint64_t k, int lo, int hi) {
    uint64_t h = mix(k), g = mix(k ^ 0x5555555555555555ULL);
    uint64_t e = (uint64_t)(lo + (int)(g % (uint64_t)(hi - lo + 1)) + 1023);
    uint64_t bits = (h & 0x000fffffffffffffULL) | (e << 52) | ((g >> 63) << 63);
    return __longlong_as_double((long long)bits);
}
__global__ void check(const double *fixed, int nfixed, int ndiv, int nnum, unsigned long long *bad, double *example) {
    int d = blockIdx.x;
    if (d >= ndiv) return;
    double b = d < nfixed ? fixed[d] : fabs(rnd(1000003ULL * d + 7, -30, 30));
    double rb = 1.0 / b;
    for (int k = threadIdx.x; k < nnum; k += blockDim.x) {
        double a = rnd(((uint64_t)d << 32) + k, -200, 200);
        double q0 = a / b, q1 = div_by(a, b, rb);
        if (__double_as_longlong(q0) != __double_as_longlong(q1)) {
            atomicAdd(bad, 1ULL);
            example[0] = a; example[1] = b;
        }
    }
}
int main(int argc, char **argv) {
    int ndiv = argc > 1 ? atoi(argv[1]) : 4096, nnum = argc > 2 ? atoi(argv[2]) : 65536;
    // PRIME20 bead masses (box-independent divisors of the impulse)
    const double fixed_h[] = {1.0, 14.0, 12.0, 28.0, 15.0, 43.0, 57.0, 58.0, 72.0, 73.0, 86.0, 87.0, 100.0, 101.0,
                              114.0, 128.0, 129.0, 131.0, 137.0, 147.0, 156.0, 163.0, 186.0, 0.8675, 1.2345678};
    int nfixed = sizeof fixed_h / sizeof fixed_h[0];
    double *fixed; unsigned long long *bad; double *ex;
    cudaMalloc(&fixed, sizeof fixed_h); cudaMalloc(&bad, 8); cudaMalloc(&ex, 16);
    cudaMemcpy(fixed, fixed_h, sizeof fixed_h, cudaMemcpyHostToDevice);
    cudaMemset(bad, 0, 8);
    check<<<ndiv, 256>>>(fixed, nfixed, ndiv, nnum, bad, ex);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long nb = 0; double exh[2] = {0, 0};
    cudaMemcpy(&nb, bad, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(exh, ex, 16, cudaMemcpyDeviceToHost);
    printf("status %s divisions %llu mismatches %llu example %.17g / %.17g\n", cudaGetErrorString(e),
           (unsigned long long)ndiv * nnum, nb, exh[0], exh[1]);
    return e == cudaSuccess && nb == 0 ? 0 : 1;
}
