// Checks f32_no_event() (engine.cuh: the single-precision screen that
// settles pair predictions with no event) against d_predict_c() on the GPU:
// random pairs and pairs placed at the edges the screen must not cross -
// separating within a hair of bij = 0, grazing a shell within a hair of a
// zero discriminant, sitting on a well's boundary - for every screened pair
// type.  A screened pair whose double-precision prediction is an event is a
// failure.  Built and run by tests/test_screen.py.
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <vector>
#include <cuda_runtime.h>
#include "engine.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t x) {   // splitmix64 finaliser
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}
__device__ __forceinline__ double uni(uint64_t &s) { s = mix(s); return (double)(s >> 11) * 0x1.0p-53; }
__device__ __forceinline__ double gauss(uint64_t &s) {
    double u = fmax(uni(s), 1e-300), v = uni(s);
    return sqrt(-2.0 * log(u)) * cos(6.283185307179586 * v);
}
__device__ __forceinline__ double wrap(double x) { return x - round(x); }

__constant__ int kCodes[] = {1, 2, 3, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 40, 41, 45, 50};
constexpr int kNCodes = sizeof(kCodes) / sizeof(kCodes[0]);

__global__ void check(DSys S, const double *tfs, int M, unsigned long long *cnt, double *example) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= M) return;
    const int i = 2 * k, j = 2 * k + 1;
    const int code = kCodes[k % kNCodes];
    uint64_t s = 0x1234567ULL + (uint64_t)k * 0x9e3779b97f4a7c15ULL;
    const DTab &T = *S.tab;
    const int a = S.ident[i], b = S.ident[j];
    // the shell the pair type meets
    double R = (code <= 3 || (code >= 17 && code <= 26)) ? T.core_sq[core_slot(code)][a][b]
               : code >= 40 ? T.shlddia_sq[a][b] : T.welldia_sq[a][b];
    double vs = pow(10.0, -2.0 + 3.0 * uni(s));
    double v[3] = {gauss(s) * vs, gauss(s) * vs, gauss(s) * vs};
    double u[3] = {gauss(s), gauss(s), gauss(s)};
    double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    for (int c = 0; c < 3; ++c) u[c] /= un;
    double r[3];
    const int mode = (k / kNCodes) % 4;
    double eps = pow(10.0, -12.0 + 10.0 * uni(s)) * (uni(s) < 0.5 ? -1.0 : 1.0);
    double rn = sqrt(R) * (0.5 + 2.5 * uni(s));
    if (mode == 3) rn = sqrt(R * (1.0 + eps));                         // on the shell
    if (mode == 2) rn = sqrt(R) * (1.0 + 2.0 * uni(s));                 // outside, grazing it
    for (int c = 0; c < 3; ++c) r[c] = u[c] * rn;
    if (mode == 1 || mode == 2) {
        // velocity nearly perpendicular to r (bij ~ 0), or grazing (D ~ 0)
        double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        double vr = v[0] * u[0] + v[1] * u[1] + v[2] * u[2];
        for (int c = 0; c < 3; ++c) v[c] -= vr * u[c];                 // perpendicular
        double vn = sqrt(vv);
        double target = mode == 1 ? eps * vn : -vn * sqrt(fmax(0.0, 1.0 - R / (rn * rn))) * (1.0 + eps);
        double vp = sqrt(fmax(0.0, vv - target * target));
        double pn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        for (int c = 0; c < 3; ++c) v[c] = (pn > 0 ? v[c] / pn * vp : 0.0) + target * u[c];
    }
    const double tf = tfs[k];
    // positions so that the relative position at tf is r (up to rounding),
    // anywhere in the box, often across the periodic boundary
    double xi[3] = {uni(s) - 0.5, uni(s) - 0.5, uni(s) - 0.5};
    double vi[3] = {gauss(s) * vs, gauss(s) * vs, gauss(s) * vs};
    double *P[3] = {S.x, S.y, S.z}, *V[3] = {S.vx, S.vy, S.vz};
    for (int c = 0; c < 3; ++c) {
        double vj = vi[c] - v[c];
        P[c][i] = xi[c];
        P[c][j] = wrap(xi[c] - r[c] - v[c] * tf);
        V[c][i] = vi[c];
        V[c][j] = vj;
    }
    __threadfence();
    bool screened = f32_no_event(S, i, j, code, d_hi(&tfs[k]));
    double tij;
    int ty;
    bool ok = d_predict_c(S, i, j, code, tf, tij, ty);
    bool none = ok && tij == DMD_BIG && ty == 0;
    atomicAdd(&cnt[0], 1ULL);
    if (none) atomicAdd(&cnt[1], 1ULL);
    if (screened) atomicAdd(&cnt[2], 1ULL);
    if (screened && !none) {
        atomicAdd(&cnt[3], 1ULL);
        example[0] = code; example[1] = mode; example[2] = tij; example[3] = ty;
    }
}

int main(int argc, char **argv) {
    const int M = argc > 1 ? atoi(argv[1]) : (1 << 20);
    const int rounds = argc > 2 ? atoi(argv[2]) : 4;
    // tables in box units: diameters 0.01-0.06, wells and shoulders 1.2-2x wider
    DTab *T = new DTab();
    srand(7);
    auto u01 = []() { return (double)rand() / RAND_MAX; };
    for (int a = 0; a < DMD_NT; ++a)
        for (int b = 0; b < DMD_NT; ++b) {
            double s = 0.01 + 0.05 * u01();
            T->sigma_sq[a][b] = s * s;
            T->ncfac_sq[a][b] = 1.1025 * s * s;
            double w = s * (1.2 + 0.8 * u01()), h = s * (1.2 + 0.8 * u01());
            T->welldia_sq[a][b] = w * w;
            T->shlddia_sq[a][b] = h * h;
            for (int c = 0; c < 14; ++c) { double q = s * (0.8 + 0.4 * u01()); T->core_sq[c][a][b] = q * q; }
        }
    DTab *dT;
    cudaMalloc(&dT, sizeof(DTab));
    cudaMemcpy(dT, T, sizeof(DTab), cudaMemcpyHostToDevice);
    DSys S{};
    S.tab = dT;
    size_t n = 2 * (size_t)M;
    double *arr[6];
    for (auto &p : arr) cudaMalloc(&p, n * 8);
    S.x = arr[0]; S.y = arr[1]; S.z = arr[2]; S.vx = arr[3]; S.vy = arr[4]; S.vz = arr[5];
    std::vector<int8_t> id(n);
    std::vector<int> bp(n, -1);
    std::vector<double> tfs(M);
    unsigned long long tot[4] = {0, 0, 0, 0};
    double ex[4] = {0, 0, 0, 0};
    int8_t *did; int *dbp; double *dtf, *dex; unsigned long long *dcnt;
    cudaMalloc(&did, n); cudaMalloc(&dbp, n * 4); cudaMalloc(&dtf, M * 8); cudaMalloc(&dex, 32); cudaMalloc(&dcnt, 32);
    S.ident = did; S.bptnr = dbp;
    for (int rd = 0; rd < rounds; ++rd) {
        for (size_t q = 0; q < n; ++q) id[q] = (int8_t)(1 + rand() % 28);
        for (int k = 0; k < M; ++k) {
            bp[2 * k] = (rand() % 4 == 0) ? 2 * k + 1 : -1;
            tfs[k] = (rand() % 8 == 0) ? 0.0 : 0.05 * u01();
        }
        cudaMemcpy(did, id.data(), n, cudaMemcpyHostToDevice);
        cudaMemcpy(dbp, bp.data(), n * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dtf, tfs.data(), M * 8, cudaMemcpyHostToDevice);
        cudaMemset(dcnt, 0, 32);
        check<<<(M + 255) / 256, 256>>>(S, dtf, M, dcnt, dex);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { printf("cuda error %s\n", cudaGetErrorString(e)); return 1; }
        unsigned long long c[4];
        cudaMemcpy(c, dcnt, 32, cudaMemcpyDeviceToHost);
        for (int q = 0; q < 4; ++q) tot[q] += c[q];
        if (c[3]) cudaMemcpy(ex, dex, 32, cudaMemcpyDeviceToHost);
    }
    printf("pairs %llu no-event %llu screened %llu failures %llu\n", tot[0], tot[1], tot[2], tot[3]);
    if (tot[3]) printf("example: code %g mode %g tij %.17g type %g\n", ex[0], ex[1], ex[2], ex[3]);
    return tot[3] ? 2 : 0;
}
