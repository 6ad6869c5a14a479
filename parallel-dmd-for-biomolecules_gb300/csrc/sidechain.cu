/*
 * sidechain.cu -- the side-chain placement search of the reference's
 * initial-configuration generator (genconfig/gen_config_random-SQZ.f90:
 * 250-348) on the GPU: dmd_sidechain_search of include/dmd.h.
 *
 * For residue k the side chain S is moved over a cubic grid of offsets; the
 * winner is the first point in loop order (d1 outermost) with the smallest
 * r3 = |bdln - r(CA)| + |bl_rn - r(NH)| + |bl_rc - r(CO)| below 100 among
 * the points whose squeezed-core distances to CO(k-1), CA(k-1), NH(k+1),
 * CA(k+1) are not below their sqz6to10.data values.  The reference's
 * operation order is kept: a distance component is (S + d) - R, its square
 * a product, a squared distance the sum x + y + z from the left.
 *
 * GB300 mapping.  The squared components depend on one axis each, so the
 * host tabulates, per residue and per reference bead R (7 of them), the
 * exact squares ((S_a + d_i) - R_a)^2 for every grid value d_i of each axis
 * a; a grid point's squared distance is then (X[i1] + Y[i2]) + Z[i3], the
 * same value the per-point expression gives.  One thread takes a line
 * (i1, i2) and walks i3 with the Z tables in shared memory.  Every point is
 * first screened in single precision (tables rounded to float, distance by
 * rsqrtf): a point is dropped when a squeeze distance is certainly below its
 * limit, or when its r3 estimate exceeds the thread's best exact r3 by more
 * than MARGIN; the others are evaluated exactly in double precision (sqrt
 * correctly rounded) and compared as the reference does.  Bounds: the float
 * squared distance is within 4 * 2^-24 relative of the double one (three
 * non-negative terms, each rounded once, two float additions); rsqrtf is
 * within 2 ulp, so the float distance is within 4.2e-7 relative, at most
 * 4.2e-6 A at the <= 10 A distances of the search box; the r3 estimate is
 * then within 2e-5 A of the exact r3 (three distances, float sums of values
 * below 30 A), below MARGIN = 1e-4 A, so no point that could win is dropped.
 * A squeeze limit L is certainly violated when the float squared distance is
 * below L^2 (1 - 1e-5): the exact distance is then below L (1 - 4.8e-6),
 * whose correctly rounded square root stays below L.  Each thread keeps the
 * first minimum of its points (it visits them in increasing grid index);
 * the blocks and then the residues' partial results are reduced by
 * (r3, grid index), which gives the reference's first minimum.
 *
 * Pruning across threads.  The screen's limit is the smallest of the
 * thread's own best r3 and the best any thread of the residue has found so
 * far (a float, atomicMin on its bits), plus MARGIN: a point above it has an
 * exact r3 above that best and can neither win nor tie.  A whole line is
 * skipped when sum over CA, NH, CO of max(0, r_xy - bond) exceeds the limit,
 * r_xy being the distance from the line's (i1, i2) part alone: along the
 * line the squared distance only grows ((X + Y) + Z >= X + Y exactly, and the
 * rounded square root is monotone), so every point's exact r3 is at least
 * that sum, which the float value (distances within 4.2e-6 A) undershoots by
 * less than MARGIN.
 *
 * Seeding.  Before the scan, k_sidechain_seed walks every SC_SEED_STRIDE-th
 * grid value of each axis in single precision, keeps per thread the point
 * of smallest r3 estimate among those whose squeeze distances are certainly
 * clear (float squared distance above L^2 (1 + 1e-5)), evaluates that one
 * point exactly and, when it is admissible, lowers the residue's shared
 * limit to its exact r3 + MARGIN.  The seed is a point of the full grid, so
 * the winner's r3 is at most its r3 and the pruning argument above holds
 * from the first line of the scan on.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dmd.h"

namespace {

constexpr int SC_REFS = 7;          /* CA, NH, CO of k; CO(k-1), CA(k-1); NH(k+1), CA(k+1) */
constexpr int SC_THREADS = 256;
constexpr int SC_MAX_GRID = 4096;   /* grid values per axis (shared memory: 7 x 4 B each) */
constexpr float SC_MARGIN = 1e-4f;
constexpr double SC_SQZ_LO = 1.0 - 1e-5;
constexpr double SC_SQZ_HI = 1.0 + 1e-5;
constexpr int SC_SEED_STRIDE = 8;

struct ScResidue {
    double bd, bn, bc;              /* bdln, bl_rn, bl_rc */
    double lim[4];                  /* squeeze limits of refs 3..6 (sz6, sz8, sz7, sz9) */
    float lo2[4];                   /* certainly-violated bound of each squared distance */
    float hi2[4];                   /* certainly-clear bound of each squared distance */
    float bdf, bnf, bcf;
    int present;                    /* bit j: reference j exists */
};

__device__ __forceinline__ bool sc_less(double a, long long ia, double b, long long ib) {
    return a < b || (a == b && ia < ib);
}

/* tables: [residue][axis][ref][m] doubles (tab64) and floats (tab32) */
__global__ void __launch_bounds__(SC_THREADS) k_sidechain(const ScResidue *res, const double *tab64,
                                                          const float *tab32, int m, double *part_r3,
                                                          long long *part_idx, unsigned int *glim) {
    extern __shared__ float zsh[];  /* [SC_REFS][m] */
    const int r = blockIdx.y;
    const ScResidue R = res[r];
    const size_t per_axis = (size_t)SC_REFS * m;
    const double *X64 = tab64 + (size_t)r * 3 * per_axis, *Y64 = X64 + per_axis, *Z64 = Y64 + per_axis;
    const float *X32 = tab32 + (size_t)r * 3 * per_axis, *Y32 = X32 + per_axis, *Z32 = Y32 + per_axis;
    for (int q = threadIdx.x; q < SC_REFS * m; q += blockDim.x) zsh[q] = Z32[q];
    __syncthreads();
    const bool prev = (R.present >> 3) & 1, next = (R.present >> 5) & 1;
    double best = 100.0;
    long long bidx = -1;
    float lim = 100.0f + SC_MARGIN;
    const long long lines = (long long)m * m;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < lines;
         p += (long long)gridDim.x * blockDim.x) {
        const int i1 = (int)(p / m), i2 = (int)(p % m);
        float xy[SC_REFS];
#pragma unroll
        for (int j = 0; j < SC_REFS; ++j) xy[j] = X32[j * m + i1] + Y32[j * m + i2];
        lim = fminf(lim, __uint_as_float(*(volatile unsigned int *)(glim + r)));
        {
            const float b[3] = {R.bdf, R.bnf, R.bcf};
            float lb = 0.0f;
#pragma unroll
            for (int j = 0; j < 3; ++j)
                if (xy[j] > 0.0f) lb += fmaxf(0.0f, xy[j] * rsqrtf(xy[j]) - b[j]);
            if (lb > lim) continue;
        }
        for (int i3 = 0; i3 < m; ++i3) {
            float q[SC_REFS];
#pragma unroll
            for (int j = 0; j < SC_REFS; ++j) q[j] = xy[j] + zsh[j * m + i3];
            bool drop = false;
            if (prev) drop = q[3] < R.lo2[0] || q[4] < R.lo2[1];
            if (next) drop = drop || q[5] < R.lo2[2] || q[6] < R.lo2[3];
            if (drop) continue;
            const float est = fabsf(R.bdf - q[0] * rsqrtf(q[0])) + fabsf(R.bnf - q[1] * rsqrtf(q[1])) +
                              fabsf(R.bcf - q[2] * rsqrtf(q[2]));
            if (est > lim) continue;   /* a NaN estimate (a zero distance) goes on to the exact test */
            /* exact evaluation, the reference's expressions */
            double d[SC_REFS];
#pragma unroll
            for (int j = 0; j < SC_REFS; ++j)
                d[j] = sqrt(X64[j * m + i1] + Y64[j * m + i2] + Z64[j * m + i3]);
            const double r3 = fabs(R.bd - d[0]) + fabs(R.bn - d[1]) + fabs(R.bc - d[2]);
            bool isz = false;
            if (prev) isz = d[3] < R.lim[0] || d[4] < R.lim[1];
            if (next) isz = isz || d[5] < R.lim[2] || d[6] < R.lim[3];
            if (r3 < best && !isz) {
                best = r3;
                bidx = ((long long)i1 * m + i2) * m + i3;
                lim = (float)(best + (double)SC_MARGIN);
                atomicMin(glim + r, __float_as_uint(lim));
            }
        }
    }
    /* block: (r3, index) minimum */
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double b2 = __shfl_down_sync(0xffffffffu, best, o);
        const long long i2 = __shfl_down_sync(0xffffffffu, bidx, o);
        if (i2 >= 0 && (bidx < 0 || sc_less(b2, i2, best, bidx))) { best = b2; bidx = i2; }
    }
    __shared__ double wb[SC_THREADS / 32];
    __shared__ long long wi[SC_THREADS / 32];
    if (lane == 0) { wb[warp] = best; wi[warp] = bidx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = wb[0];
        long long bi = wi[0];
        for (int w = 1; w < SC_THREADS / 32; ++w)
            if (wi[w] >= 0 && (bi < 0 || sc_less(wb[w], wi[w], b, bi))) { b = wb[w]; bi = wi[w]; }
        part_r3[(size_t)r * gridDim.x + blockIdx.x] = b;
        part_idx[(size_t)r * gridDim.x + blockIdx.x] = bi;
    }
}

/* the residue's exact r3 at grid point (i1, i2, i3), or a negative value
 * when a squeeze limit is violated */
__device__ double sc_exact(const ScResidue &R, const double *X64, const double *Y64, const double *Z64, int m,
                           int i1, int i2, int i3) {
    const bool prev = (R.present >> 3) & 1, next = (R.present >> 5) & 1;
    double d[SC_REFS];
#pragma unroll
    for (int j = 0; j < SC_REFS; ++j) d[j] = sqrt(X64[j * m + i1] + Y64[j * m + i2] + Z64[j * m + i3]);
    bool isz = false;
    if (prev) isz = d[3] < R.lim[0] || d[4] < R.lim[1];
    if (next) isz = isz || d[5] < R.lim[2] || d[6] < R.lim[3];
    return isz ? -1.0 : fabs(R.bd - d[0]) + fabs(R.bn - d[1]) + fabs(R.bc - d[2]);
}

/* the coarse pre-pass: an admissible upper bound of each residue's winner */
__global__ void __launch_bounds__(SC_THREADS) k_sidechain_seed(const ScResidue *res, const double *tab64,
                                                               const float *tab32, int m, unsigned int *glim) {
    const int r = blockIdx.y;
    const ScResidue R = res[r];
    const size_t per_axis = (size_t)SC_REFS * m;
    const double *X64 = tab64 + (size_t)r * 3 * per_axis, *Y64 = X64 + per_axis, *Z64 = Y64 + per_axis;
    const float *X32 = tab32 + (size_t)r * 3 * per_axis, *Y32 = X32 + per_axis, *Z32 = Y32 + per_axis;
    const bool prev = (R.present >> 3) & 1, next = (R.present >> 5) & 1;
    const int mc = (m + SC_SEED_STRIDE - 1) / SC_SEED_STRIDE;
    const long long total = (long long)mc * mc * mc;
    float bestf = 3.0e38f;
    int b1 = -1, b2 = 0, b3 = 0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const int i1 = (int)(p / ((long long)mc * mc)) * SC_SEED_STRIDE;
        const int i2 = (int)((p / mc) % mc) * SC_SEED_STRIDE, i3 = (int)(p % mc) * SC_SEED_STRIDE;
        float q[SC_REFS];
#pragma unroll
        for (int j = 0; j < SC_REFS; ++j) q[j] = X32[j * m + i1] + Y32[j * m + i2] + Z32[j * m + i3];
        bool clear = true;
        if (prev) clear = q[3] > R.hi2[0] && q[4] > R.hi2[1];
        if (next) clear = clear && q[5] > R.hi2[2] && q[6] > R.hi2[3];
        if (!clear || !(q[0] > 0.0f && q[1] > 0.0f && q[2] > 0.0f)) continue;
        const float est = fabsf(R.bdf - q[0] * rsqrtf(q[0])) + fabsf(R.bnf - q[1] * rsqrtf(q[1])) +
                          fabsf(R.bcf - q[2] * rsqrtf(q[2]));
        if (est < bestf) { bestf = est; b1 = i1; b2 = i2; b3 = i3; }
    }
    if (b1 >= 0) {
        const double r3 = sc_exact(R, X64, Y64, Z64, m, b1, b2, b3);
        if (r3 >= 0.0 && r3 < 100.0) atomicMin(glim + r, __float_as_uint((float)(r3 + (double)SC_MARGIN)));
    }
}

/* one block per residue: the minimum over the blocks' partial results */
__global__ void __launch_bounds__(SC_THREADS) k_sidechain_reduce(const double *part_r3, const long long *part_idx,
                                                                 int nparts, double *out_r3, long long *out_idx) {
    const int r = blockIdx.x;
    double best = 100.0;
    long long bidx = -1;
    for (int q = threadIdx.x; q < nparts; q += blockDim.x) {
        const double b = part_r3[(size_t)r * nparts + q];
        const long long i = part_idx[(size_t)r * nparts + q];
        if (i >= 0 && (bidx < 0 || sc_less(b, i, best, bidx))) { best = b; bidx = i; }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double b2 = __shfl_down_sync(0xffffffffu, best, o);
        const long long i2 = __shfl_down_sync(0xffffffffu, bidx, o);
        if (i2 >= 0 && (bidx < 0 || sc_less(b2, i2, best, bidx))) { best = b2; bidx = i2; }
    }
    __shared__ double wb[SC_THREADS / 32];
    __shared__ long long wi[SC_THREADS / 32];
    if (lane == 0) { wb[warp] = best; wi[warp] = bidx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = wb[0];
        long long bi = wi[0];
        for (int w = 1; w < SC_THREADS / 32; ++w)
            if (wi[w] >= 0 && (bi < 0 || sc_less(wb[w], wi[w], b, bi))) { b = wb[w]; bi = wi[w]; }
        out_r3[r] = bi >= 0 ? b : 100.0;
        out_idx[r] = bi;
    }
}

int sc_fail(char *err, int32_t errlen, int code, const std::string &msg) {
    if (err && errlen > 0) {
        std::strncpy(err, msg.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
    }
    return code;
}

}  // namespace

extern "C" int dmd_sidechain_search(int32_t n_res, const double *ca, const double *nh, const double *co,
                                    const double *side, const int32_t *residue, const dmd_tables *T, double move,
                                    double step, double *side_out, double *rmin_out, int64_t *index_out,
                                    char *err, int32_t errlen) {
    if (n_res <= 0 || !ca || !nh || !co || !side || !residue || !T || !side_out || !rmin_out)
        return sc_fail(err, errlen, DMD_E_INPUT, "null or empty argument");
    if (n_res > 65535) return sc_fail(err, errlen, DMD_E_INPUT, "at most 65535 residues per call");
    if (!(step > 0) || !(move >= 0) || !std::isfinite(move) || !std::isfinite(step))
        return sc_fail(err, errlen, DMD_E_INPUT, "move must be >= 0 and step > 0");
    /* the grid of one axis: a Fortran DO loop over a real variable */
    const double trip = (move - (-move) + step) / step;
    if (!(trip < (double)SC_MAX_GRID + 1.0))
        return sc_fail(err, errlen, DMD_E_INPUT, "more than 4096 grid values per axis");
    const int m = trip > 0 ? (int)trip : 0;
    if (m == 0) return sc_fail(err, errlen, DMD_E_INPUT, "empty grid");
    std::vector<double> D(m);
    {
        double d = -move;
        for (int i = 0; i < m; ++i) { D[i] = d; d = d + step; }
    }
    for (int k = 0; k < n_res; ++k) {
        if (residue[k] < 9 || residue[k] > 28) return sc_fail(err, errlen, DMD_E_INPUT, "residue identity out of 9..28");
        for (int a = 0; a < 3; ++a) {
            const double v[4] = {ca[3 * k + a], nh[3 * k + a], co[3 * k + a], side[3 * k + a]};
            for (double x : v)
                if (!std::isfinite(x)) return sc_fail(err, errlen, DMD_E_INPUT, "non-finite position");
        }
    }
    /* per residue: the limits and the squared-component tables */
    const size_t per_axis = (size_t)SC_REFS * m, per_res = 3 * per_axis;
    if ((double)n_res * (double)per_res * 12.0 > (double)(1u << 30))
        return sc_fail(err, errlen, DMD_E_INPUT, "tables above 1 GiB: fewer residues or a coarser grid per call");
    std::vector<ScResidue> hres(n_res);
    std::vector<double> t64((size_t)n_res * per_res);
    std::vector<float> t32((size_t)n_res * per_res);
    for (int k = 0; k < n_res; ++k) {
        const int row = residue[k] - 9;
        ScResidue &R = hres[k];
        R.bd = T->rca[row]; R.bn = T->rnh[row]; R.bc = T->rco[row];
        R.bdf = (float)R.bd; R.bnf = (float)R.bn; R.bcf = (float)R.bc;
        /* sqz6to10.data columns: sz8, sz6, sz7, sz9 (genconfig's SQZ610(1..4)) */
        R.lim[0] = T->sqz[row][1]; R.lim[1] = T->sqz[row][0]; R.lim[2] = T->sqz[row][2]; R.lim[3] = T->sqz[row][3];
        for (int q = 0; q < 4; ++q) {
            R.lo2[q] = (float)(R.lim[q] * R.lim[q] * SC_SQZ_LO);
            R.hi2[q] = (float)(R.lim[q] * R.lim[q] * SC_SQZ_HI);
        }
        const bool prev = k >= 1, next = k + 1 < n_res;
        R.present = 7 | (prev ? (8 | 16) : 0) | (next ? (32 | 64) : 0);
        const double *refs[SC_REFS] = {ca + 3 * k, nh + 3 * k, co + 3 * k, prev ? co + 3 * (k - 1) : ca + 3 * k,
                                       prev ? ca + 3 * (k - 1) : ca + 3 * k, next ? nh + 3 * (k + 1) : ca + 3 * k,
                                       next ? ca + 3 * (k + 1) : ca + 3 * k};
        for (int a = 0; a < 3; ++a)
            for (int j = 0; j < SC_REFS; ++j)
                for (int i = 0; i < m; ++i) {
                    const double c = side[3 * k + a] + D[i] - refs[j][a];
                    const double sq = c * c;
                    const size_t o = (size_t)k * per_res + (size_t)a * per_axis + (size_t)j * m + i;
                    t64[o] = sq;
                    t32[o] = (float)sq;
                }
    }
    /* launch: a few blocks per SM over all residues */
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return sc_fail(err, errlen, DMD_E_CUDA, cudaGetErrorString(e));
    const long long lines = (long long)m * m;
    long long want = (long long)sms * 8 / n_res;
    if (want < 1) want = 1;
    const long long most = (lines + SC_THREADS - 1) / SC_THREADS;
    const int nb = (int)(want < most ? want : most);
    const size_t smem = (size_t)SC_REFS * m * sizeof(float);
    double *d64 = nullptr, *p_r3 = nullptr, *o_r3 = nullptr;
    float *d32 = nullptr;
    long long *p_idx = nullptr, *o_idx = nullptr;
    ScResidue *dres = nullptr;
    unsigned int *dlim = nullptr;
    std::vector<double> h_r3(n_res);
    std::vector<long long> h_idx(n_res);
    auto done = [&](cudaError_t ce) {
        cudaFree(d64); cudaFree(d32); cudaFree(p_r3); cudaFree(p_idx); cudaFree(o_r3); cudaFree(o_idx); cudaFree(dres);
        cudaFree(dlim);
        return ce;
    };
    e = cudaMalloc(&d64, t64.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d32, t32.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p_r3, (size_t)n_res * nb * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&p_idx, (size_t)n_res * nb * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&o_r3, (size_t)n_res * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&o_idx, (size_t)n_res * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&dres, (size_t)n_res * sizeof(ScResidue));
    if (e == cudaSuccess) e = cudaMalloc(&dlim, (size_t)n_res * sizeof(unsigned int));
    {
        /* the residues' shared limits start at 100 + MARGIN, the threads' own */
        const float l0 = 100.0f + SC_MARGIN;
        unsigned int bits = 0;
        std::memcpy(&bits, &l0, sizeof bits);
        const std::vector<unsigned int> init((size_t)n_res, bits);
        if (e == cudaSuccess) e = cudaMemcpy(dlim, init.data(), init.size() * sizeof(unsigned int), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(d64, t64.data(), t64.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d32, t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dres, hres.data(), hres.size() * sizeof(ScResidue), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = cudaFuncSetAttribute(k_sidechain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        long long ws = (long long)sms * 4 / n_res;
        if (ws < 1) ws = 1;
        k_sidechain_seed<<<dim3((unsigned)ws, n_res), SC_THREADS>>>(dres, d64, d32, m, dlim);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_sidechain<<<dim3(nb, n_res), SC_THREADS, smem>>>(dres, d64, d32, m, p_r3, p_idx, dlim);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_sidechain_reduce<<<n_res, SC_THREADS>>>(p_r3, p_idx, nb, o_r3, o_idx);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(h_r3.data(), o_r3, (size_t)n_res * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(h_idx.data(), o_idx, (size_t)n_res * sizeof(long long), cudaMemcpyDeviceToHost);
    done(e);
    if (e != cudaSuccess) return sc_fail(err, errlen, DMD_E_CUDA, cudaGetErrorString(e));
    for (int k = 0; k < n_res; ++k) {
        const long long b = h_idx[k];
        double d[3] = {0.0, 0.0, 0.0};
        if (b >= 0) { d[0] = D[b / ((long long)m * m)]; d[1] = D[(b / m) % m]; d[2] = D[b % m]; }
        for (int a = 0; a < 3; ++a) side_out[3 * k + a] = side[3 * k + a] + d[a];
        rmin_out[k] = h_r3[k];
        if (index_out) index_out[k] = b;
    }
    return DMD_OK;
}

extern "C" int64_t dmd_sidechain_grid(double move, double step) {
    if (!(step > 0) || !(move >= 0)) return -1;
    const double trip = (move - (-move) + step) / step;
    return trip > 0 ? (int64_t)trip : 0;
}
