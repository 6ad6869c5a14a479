// Two-bead known-answer cases on the GPU: the engine's own device predictor
// (d_predict_c, engine.cuh) and collision impulse (warp_eventdyn,
// engine_run.cuh) applied to two beads of a real system, placed by the
// caller, with the tables the library builds from the parameter files.
// Built by tests/test_known_answers.py into a shared library: this file
// includes the library's sources so that it reaches their internal set-up
// (setup_host, upload_system) and device functions without new exports.
#include "engine.cu"
#include "capi.cu"

namespace {

__global__ void k_pair_cases(DSys S_in, int n, const int *ci, const int *cj, const int *cida, const int *cidb,
                             const int *cev, const int *cbond, const double *cst, const int *cct, double *tij_out,
                             int *type_out, int *valid_out, double *st_out, int *ct_out, double *st_light) {
    __shared__ DSys S_sh;
    __shared__ run_compact::WarpArea WA;
    if (threadIdx.x == 0) S_sh = S_in;
    __syncthreads();
    const DSys &S = S_sh;
    const int lane = threadIdx.x & 31;
    for (int q = 0; q < n; ++q) {
        const int i = ci[q], j = cj[q];
        if (lane == 0) {
            if (cida[q] > 0) S.ident[i] = (int8_t)cida[q];
            if (cidb[q] > 0) S.ident[j] = (int8_t)cidb[q];
            S.bptnr[i] = cbond[q] ? j : -1;
            S.bptnr[j] = cbond[q] ? i : -1;
            const double *st = cst + 12 * q;
            S.x[i] = st[0]; S.y[i] = st[1]; S.z[i] = st[2]; S.vx[i] = st[3]; S.vy[i] = st[4]; S.vz[i] = st[5];
            S.x[j] = st[6]; S.y[j] = st[7]; S.z[j] = st[8]; S.vx[j] = st[9]; S.vy[j] = st[10]; S.vz[j] = st[11];
        }
        __syncwarp();
        __threadfence_block();
        double tij = 0.0;
        int ty = 0;
        const bool ok = d_predict_c(S, i, j, cev[q], 0.0, tij, ty);
        int ct = 0;
        if (cct[q] > 0) ct = run_compact::warp_eventdyn(S, i, j, cev[q], cct[q], 0.0);
        __syncwarp();
        __threadfence_block();
        if (lane == 0) {
            tij_out[q] = tij;
            type_out[q] = ty;
            valid_out[q] = ok;
            ct_out[q] = ct;
            double *o = st_out + 12 * q;
            o[0] = S.x[i]; o[1] = S.y[i]; o[2] = S.z[i]; o[3] = S.vx[i]; o[4] = S.vy[i]; o[5] = S.vz[i];
            o[6] = S.x[j]; o[7] = S.y[j]; o[8] = S.z[j]; o[9] = S.vx[j]; o[10] = S.vy[j]; o[11] = S.vz[j];
        }
        __syncwarp();
        /* a core or bond event (coltype 1-3) once more through the light
         * batches' half-warp collision, from the same state, with the
         * case's pair code set as an override (lanes 16..31: no event) */
        if (cct[q] >= 1 && cct[q] <= 3) {
            if (lane == 0) {
                const double *st = cst + 12 * q;
                S.x[i] = st[0]; S.y[i] = st[1]; S.z[i] = st[2]; S.vx[i] = st[3]; S.vy[i] = st[4]; S.vz[i] = st[5];
                S.x[j] = st[6]; S.y[j] = st[7]; S.z[j] = st[8]; S.vx[j] = st[9]; S.vy[j] = st[10]; S.vz[j] = st[11];
                S.colt[i] = (int8_t)cct[q];
                S.ovp[4 * i] = j; S.ovc[4 * i] = (int8_t)cev[q];
            }
            __syncwarp();
            __threadfence_block();
            run_compact::hw_collision_light(S, WA, lane < 16, i, j, 0.0, 1);
            __syncwarp();
            __threadfence_block();
            if (lane == 0) {
                double *o = st_light + 12 * q;
                o[0] = S.x[i]; o[1] = S.y[i]; o[2] = S.z[i]; o[3] = S.vx[i]; o[4] = S.vy[i]; o[5] = S.vz[i];
                o[6] = S.x[j]; o[7] = S.y[j]; o[8] = S.z[j]; o[9] = S.vx[j]; o[10] = S.vy[j]; o[11] = S.vz[j];
                S.ovp[4 * i] = -1;
            }
            __syncwarp();
        }
    }
}

template <class T>
T *dcopy(const T *h, int n) {
    T *d = nullptr;
    if (cudaMalloc(&d, sizeof(T) * (size_t)(n > 0 ? n : 1)) != cudaSuccess) return nullptr;
    if (h && cudaMemcpy(d, h, sizeof(T) * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return d;
}

}  // namespace

/* Runs n cases on the system (cfg, tables, sys): case q places beads i[q],
 * j[q] (0-based) at st[12q..12q+11] (x, y, z, vx, vy, vz of i, then j;
 * positions in box units) with tfalse = 0, identities ida/idb when > 0 and
 * each other's H-bond partner when bond[q]; predicts the pair under ev[q]
 * and applies the impulse of collision type ct[q] when ct[q] > 0.  The
 * cases run one after another on one warp; each starts from the state the
 * previous one left for beads it does not set. */
extern "C" int ka_pair_cases(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys, int n,
                             const int *i, const int *j, const int *ida, const int *idb, const int *ev,
                             const int *bond, const double *st, const int *ct, double *tij, int *type, int *valid,
                             double *st_out, int *ct_out, double *st_light, char *err, int errlen) {
    HostSys H;
    std::string e;
    if (!setup_host(H, cfg, tables, sys, e)) {
        std::snprintf(err, errlen, "%s", e.c_str());
        return DMD_E_INPUT;
    }
    DevSys D;
    if (upload_system(H, D, nullptr, e) != DMD_OK) {
        std::snprintf(err, errlen, "%s", e.c_str());
        return DMD_E_CUDA;
    }
    int *di = dcopy(i, n), *dj = dcopy(j, n), *dida = dcopy(ida, n), *didb = dcopy(idb, n), *dev = dcopy(ev, n);
    int *dbond = dcopy(bond, n), *dct = dcopy(ct, n);
    double *dst = dcopy(st, 12 * n);
    double *dtij = dcopy<double>(nullptr, n), *dso = dcopy<double>(nullptr, 12 * n);
    double *dsl = dcopy<double>(nullptr, 12 * n);
    int *dty = dcopy<int>(nullptr, n), *dval = dcopy<int>(nullptr, n), *dcto = dcopy<int>(nullptr, n);
    int rc = DMD_OK;
    if (!di || !dj || !dida || !didb || !dev || !dbond || !dct || !dst || !dtij || !dso || !dty || !dval || !dcto ||
        !dsl) {
        std::snprintf(err, errlen, "device allocation failed");
        rc = DMD_E_CUDA;
    } else {
        k_pair_cases<<<1, 32>>>(D.d, n, di, dj, dida, didb, dev, dbond, dst, dct, dtij, dty, dval, dso, dcto, dsl);
        cudaError_t ce = cudaDeviceSynchronize();
        if (ce == cudaSuccess) ce = cudaMemcpy(tij, dtij, 8 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess) ce = cudaMemcpy(type, dty, 4 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess) ce = cudaMemcpy(valid, dval, 4 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess) ce = cudaMemcpy(st_out, dso, 96 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess) ce = cudaMemcpy(ct_out, dcto, 4 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce == cudaSuccess) ce = cudaMemcpy(st_light, dsl, 96 * (size_t)n, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess) {
            std::snprintf(err, errlen, "%s", cudaGetErrorString(ce));
            rc = DMD_E_CUDA;
        }
    }
    for (void *p : {(void *)di, (void *)dj, (void *)dida, (void *)didb, (void *)dev, (void *)dbond, (void *)dct,
                    (void *)dst, (void *)dtij, (void *)dso, (void *)dty, (void *)dval, (void *)dcto, (void *)dsl})
        if (p) cudaFree(p);
    cudaFree(D.pool);
    return rc;
}

namespace {
__global__ void k_log_many(const double *x, double *y, long long n) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
        y[k] = dmd_log(x[k]);
}
}  // namespace

/* dmd_log (dmd_rng.h) on the device over n inputs (host arrays) */
extern "C" int ka_log_many(const double *x, double *y, long long n) {
    double *dx = dcopy(x, (int)n), *dy = dcopy<double>(nullptr, (int)n);
    int rc = 0;
    if (!dx || !dy) rc = -1;
    else {
        k_log_many<<<1024, 256>>>(dx, dy, n);
        if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpy(y, dy, 8 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = -1;
    }
    if (dx) cudaFree(dx);
    if (dy) cudaFree(dy);
    return rc;
}
