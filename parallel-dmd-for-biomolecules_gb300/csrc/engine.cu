/*
 * engine.cu -- kernels of the GB300 PRIME20 DMD event engine.
 *
 * One CTA owns one system (a replica or a served request) for the whole
 * launch and runs the reference's main loop (code/main.F90:484-1258) on it.
 * A launch with many CTAs advances many independent systems at once (the
 * batched-replica and serving paths); a launch with one CTA is the plain path.
 *
 * Inside a CTA, pair events are committed in conflict-free batches:
 *   1. candidates: the earliest queued bead events below a time cut (and
 *      below every pseudo event), sorted in (time, index) order;
 *   2. footprints: each candidate claims the beads its commit reads or
 *      writes (its two beads, both neighbour lists, H-bond helpers, and the
 *      lists of beads it may fully re-predict); the batch is the longest
 *      prefix whose footprints are disjoint;
 *   3. one warp per event: collision (written, with a snapshot), then the
 *      re-prediction of code/partial_events.f into a warp-private buffer;
 *   4. validation: event k stands only if no earlier event of the batch
 *      produced a new prediction before it, so the committed events are
 *      exactly the next events of the serial (time, index) order;
 *   5. commit the buffers of the standing events; roll the others back.
 * Because the footprints are disjoint, each event reads exactly what it
 * would read in the serial order and the results are bit-identical to
 * one-at-a-time processing.  Ghost, interval and output events are batch
 * barriers and run alone.
 *
 * GB300 executes an FP64 warp instruction in about 64 cycles per SM
 * sub-partition whatever the number of active lanes (DDIV ~500, DSQRT ~690),
 * so: times are compared as integer keys, the collision's independent
 * components run on separate lanes, and several events share the SM.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <limits.h>

#include <cooperative_groups.h>
#include <algorithm>
#include <mutex>

#include "dmd.h"
#include "engine.cuh"
#include "engine_api.h"

#define NTHREADS 256
#define NWARPS (NTHREADS / 32)
#define NWARPS_MAX 16     /* the most warps any kernel here runs per CTA */
#define CAND_MAX 64
#define META_MAX 16
#define TG_MAX 64         /* full re-predictions per round (i, j, marked beads) */
#define TMAP_MAX 256
#define CASC_MAX 64
#define WSET_MAX 16
/* systems up to this size keep the claim tables in shared memory (full and
 * compact variants of k_run); larger ones use their global array */
#define OWN_SMEM_FULL 2048
#define OWN_SMEM_COMPACT 1024
/* threads of k_run per CTA: one candidate event per warp, so the warps of a
 * CTA bound a batch.  The compact variant's smaller event areas leave room
 * for more warps; 12 keep 168 registers per thread (16 would cap them at 128
 * and spill) and measured fastest on the 32-replica workload (16, 10 and 8
 * warps: 5 %, 3 % and 9 % slower) */
#define RUN_NT_FULL 256
#define RUN_NT_COMPACT 384
#define RUN_CARVEOUT_COMPACT_KB 164
#define DMD_TICKET_SEQ_MAX ((1 << 25) - 2)
#define FULL 0xffffffffu

/* Optional phase timers of k_run (build with -DDMD_PHASE_TIMERS): thread 0
 * of each CTA adds the clock cycles spent in each phase of the event loop;
 * dmd_debug_phase_cycles() reads them back.  Off by default. */
#ifdef DMD_PHASE_TIMERS
#define DMD_PHASE_SLOTS 16
#define DMD_PHASE_CTAS 1024
__device__ long long g_phase_cycles[DMD_PHASE_CTAS][DMD_PHASE_SLOTS];
#define DMD_PHASE_START(row) long long ph_t_ = clock64(); const int ph_row_ = (row)
#define DMD_PHASE(k)                                                                       \
    do {                                                                                   \
        if (threadIdx.x == 0 && ph_row_ >= 0 && ph_row_ < DMD_PHASE_CTAS) {                \
            long long now_ = clock64();                                                    \
            g_phase_cycles[ph_row_][(k)] += now_ - ph_t_;                                  \
            ph_t_ = now_;                                                                  \
        }                                                                                  \
    } while (0)
/* sub-phases of one event's processing, on warp 0 of CTA g_sub_cta only
 * (row DMD_PHASE_CTAS - 1) */
__device__ long long g_sub_last;
__device__ int g_sub_cta;
#define DMD_SUB(k)                                                                         \
    do {                                                                                   \
        if (blockIdx.x == g_sub_cta && threadIdx.x == 0) {                                 \
            long long now_ = clock64();                                                    \
            if ((k) >= 0) g_phase_cycles[DMD_PHASE_CTAS - 1][(k)] += now_ - g_sub_last;    \
            g_sub_last = now_;                                                             \
        }                                                                                  \
    } while (0)
/* sub-phases of the interval event on CTA g_sub_cta (row DMD_PHASE_CTAS - 3) */
__device__ long long g_isub_last;
#define DMD_ISUB(k)                                                                        \
    do {                                                                                   \
        if (blockIdx.x == g_sub_cta && threadIdx.x == 0) {                                 \
            long long now_ = clock64();                                                    \
            if ((k) >= 0) g_phase_cycles[DMD_PHASE_CTAS - 3][(k)] += now_ - g_isub_last;   \
            g_isub_last = now_;                                                            \
        }                                                                                  \
    } while (0)
extern "C" int dmd_debug_set_sub_cta(int cta) { return (int)cudaMemcpyToSymbol(g_sub_cta, &cta, sizeof cta); }
extern "C" int dmd_debug_phase_cycles(long long *out, int nctas) {
    if (nctas > DMD_PHASE_CTAS) nctas = DMD_PHASE_CTAS;
    return (int)cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(long long) * DMD_PHASE_SLOTS * nctas);
}
/* sub-phases of a light batch on warp 0 of CTA g_sub_cta (row DMD_PHASE_CTAS - 5) */
__device__ long long g_lsub_last;
#define DMD_LSUB(k)                                                                        \
    do {                                                                                   \
        if (blockIdx.x == g_sub_cta && threadIdx.x == 0) {                                 \
            long long now_ = clock64();                                                    \
            if ((k) >= 0) g_phase_cycles[DMD_PHASE_CTAS - 5][(k)] += now_ - g_lsub_last;   \
            g_lsub_last = now_;                                                            \
        }                                                                                  \
    } while (0)
/* steps of a light collision on warp 0 of CTA g_sub_cta (row DMD_PHASE_CTAS - 7) */
__device__ long long g_csub_last;
#define DMD_CSUB(k)                                                                        \
    do {                                                                                   \
        if (blockIdx.x == g_sub_cta && threadIdx.x == 0) {                                 \
            long long now_ = clock64();                                                    \
            if ((k) >= 0) g_phase_cycles[DMD_PHASE_CTAS - 7][(k)] += now_ - g_csub_last;   \
            g_csub_last = now_;                                                            \
        }                                                                                  \
    } while (0)
/* sub-phases of the candidate gather, per CTA (rows 512 + block index) */
#define DMD_GSUB_START() long long gs_t_ = clock64()
#define DMD_GSUB(k)                                                                        \
    do {                                                                                   \
        if (threadIdx.x == 0 && blockIdx.x < 500) {                                        \
            long long now_ = clock64();                                                    \
            g_phase_cycles[512 + blockIdx.x][(k)] += now_ - gs_t_;                         \
            gs_t_ = now_;                                                                  \
        }                                                                                  \
    } while (0)
#else
#define DMD_GSUB_START() do { } while (0)
#define DMD_LSUB(k) do { } while (0)
#define DMD_CSUB(k) do { } while (0)
#define DMD_GSUB(k) do { } while (0)
#define DMD_PHASE_START(row) do { (void)(row); } while (0)
#define DMD_PHASE(k) do { (void)(k); } while (0)
#define DMD_SUB(k) do { } while (0)
#define DMD_ISUB(k) do { } while (0)
#endif

/* per-warp scratch of the full re-predictions of up to TG_MAX beads: bead,
 * first task, running minimum (key, partner, time, type), task -> bead map */
struct FullScratch {
    int tg_b[TG_MAX];
    int tg_base[TG_MAX + 1];
    long long tg_k[TG_MAX];
    int tg_p[TG_MAX];
    double tg_raw[TG_MAX];
    int8_t tg_y[TG_MAX];
    int8_t tmap[TMAP_MAX];
};

/* The prediction tasks of all events of a batch on one CTA, executed by all
 * its warps together (a task: bead, partner, static code or -1, flags =
 * down-operation bit | owner warp << 1; result: time, type, valid). */
#define PTASK_MAX 512
struct TaskPool {
    int n, nlive;
    int a[PTASK_MAX], b[PTASK_MAX];
    int8_t st[PTASK_MAX], flag[PTASK_MAX];
    double t[PTASK_MAX];
    int8_t ty[PTASK_MAX], ok[PTASK_MAX];
    int16_t live[PTASK_MAX];      /* the tasks left for double precision */
};

/* the draws of one ghost collision that do not depend on the state
 * (code/main.F90:998-1041): the bead (1-based, before the clamp), the two
 * accepted (v1, v2) pairs, the next ghost time's uniform, and the logarithms
 * of r1, r2 and that uniform; g: the ghost index they belong to (-1: none) */
struct GhostDraws {
    long long g;
    int ok, i;
    double v1a, v2a, v1b, ra, rb, tg;
    double L[3];
};

struct SharedState {
    DScal sc;
    GhostDraws gdraw[2];   /* ghost g's draws at [g & 1], drawn ahead by a free warp */
    int ev;
    long long cand_key[CAND_MAX];
    int cand_idx[CAND_MAX];
    long long sort_key[CAND_MAX];
    int sort_idx[CAND_MAX];
    int ncand, m, nbatch, nvalid, tick_reset;
    long long kcut;
    double delta;        /* time window of the candidate cut */
    int groups[256];
    int ngroups;
    double red_d[NWARPS_MAX];
    int red_i[NWARPS_MAX * 4];
    int rebuild;
    int touched[8];
    int bseq;            /* footprint claims of this launch (ticket base) */
    /* cluster exchange: the leader CTA (rank 0) publishes the batch, every
     * CTA's warps report their candidate's results into the leader's slots,
     * and the other CTAs copy what they need into their own fields */
    int exitf, P, V;
    long long coll0, log0;
    double imax, tnow, tf_iv;
    int c_conflict[CAND_MAX], c_over[CAND_MAX];
    int8_t c_simple[CAND_MAX];    /* the event's collision cannot change H-bond state (coltype 1-3) */
    int8_t c_qbad[CAND_MAX];      /* light batch: the event read a queue entry an earlier one changed */
    long long c_tnew_key[CAND_MAX];
    int c_tnew_idx[CAND_MAX], c_err[CAND_MAX], c_err_info[CAND_MAX], c_ct[CAND_MAX];
    double c_tf[CAND_MAX];
    double red_max[16];
};

namespace cg = cooperative_groups;
/* barrier over the CTAs of one system (the cluster), with release/acquire
 * ordering of global and shared memory at cluster scope */
__device__ __forceinline__ void csync(int C) {
    if (C == 1) __syncthreads();
    else cg::this_cluster().sync();
}

/* where an error goes: the system's status, or the status of one
 * speculative event (raised only if that event is committed) */
struct Err { int *code; int *info; };
__device__ __forceinline__ void set_err(Err e, int code, int info) {
    if (atomicCAS(e.code, 0, code) == 0) *e.info = info;
}
__device__ __forceinline__ Err cta_err(SharedState &sh) { return Err{&sh.sc.err, &sh.sc.err_info}; }
__device__ __forceinline__ void set_err(SharedState &sh, int code, int info) { set_err(cta_err(sh), code, info); }

/* ------------------------------------------------------------------ */
/* keys and minima                                                     */
/* ------------------------------------------------------------------ */
/* lexicographic (key, partner) minimum across the warp, carrying time and type */
__device__ __forceinline__ void warp_keymin(long long &k, int &p, double &t, int &ty) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long k2 = __shfl_xor_sync(FULL, k, o);
        int p2 = __shfl_xor_sync(FULL, p, o);
        double t2 = __shfl_xor_sync(FULL, t, o);
        int y2 = __shfl_xor_sync(FULL, ty, o);
        if (key_less(k2, p2, k, p)) { k = k2; p = p2; t = t2; ty = y2; }
    }
}

__device__ __forceinline__ void set_pred(const DSys &S, int b, double t, int p, int ty, bool q) {
    b = DMD_CHK(b, S.N + 3, 10);
    S.tim[b] = t;
    S.nptnr[b] = p;
    S.colt[b] = (int8_t)ty;
    S.queued[b] = q ? 1 : 0;
    S.key[b] = q ? okey(t) : DMD_KEY_INF;
}

/* ------------------------------------------------------------------ */
/* tournament over the integer keys                                    */
/* ------------------------------------------------------------------ */
/* level-1 group g: argmin over its 32 keys (lowest index on ties); the 32
 * loads are issued before the first comparison */
__device__ void l1_update(const DSys &S, int g, int NE) {
    int lo = g * 32, n = min(32, NE - lo);
    long long k[32];
    int ix[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) { k[q] = q < n ? S.key[lo + q] : DMD_KEY_INF; ix[q] = q; }
    /* pairwise tree, the left entry winning ties: the first minimum, as a
     * left-to-right scan finds it, in five levels instead of 31 steps */
#pragma unroll
    for (int w = 1; w < 32; w <<= 1)
#pragma unroll
        for (int q = 0; q + w < 32; q += 2 * w)
            if (k[q + w] < k[q]) { k[q] = k[q + w]; ix[q] = ix[q + w]; }
    S.l1i[g] = lo + ix[0];
    S.l1k[g] = k[0];
}
__device__ void l2_update(const DSys &S, int h) {
    int lo = h * 32, n = min(32, S.nl1 - lo);
    long long k[32];
    int ix[32];
#pragma unroll
    for (int q = 0; q < 32; ++q) {
        k[q] = q < n ? S.l1k[lo + q] : DMD_KEY_INF;
        ix[q] = q < n ? S.l1i[lo + q] : INT_MAX;
    }
    int best = ix[0];
    long long bk = k[0];
#pragma unroll
    for (int q = 1; q < 32; ++q)
        if (key_less(k[q], ix[q], bk, best)) { bk = k[q]; best = ix[q]; }
    S.l2i[h] = best;
    S.l2k[h] = bk;
}
__device__ void cta_tree_rebuild(const DSys &S) {
    int NE = S.N + 3;
    for (int g = threadIdx.x; g < S.nl1; g += blockDim.x) l1_update(S, g, NE);
    __syncthreads();
    for (int h = threadIdx.x; h < S.nl2; h += blockDim.x) l2_update(S, h);
    __syncthreads();
}
/* warp: refresh the level-1 groups of the given entries */
__device__ void warp_l1_refresh(const DSys &S, const int *entries, int n) {
    int lane = threadIdx.x & 31;
    for (int q = lane; q < n; q += 32) { int e = entries[q]; if (e >= 0) l1_update(S, e >> 5, S.N + 3); }
}

/* ------------------------------------------------------------------ */
/* H-bond bookkeeping (code/repuls_add.f, repuls_del_b.f, main.F90:825-868) */
/* ------------------------------------------------------------------ */
__device__ void ovr_set(const DSys &S, Err E, int a, int b, int code, int hbonds) {
    int *op = S.ovp + 4 * a;
    int8_t *oc = S.ovc + 4 * a;
    int st = static_code(S.info[a], S.info[b], hbonds);
    for (int s = 0; s < 4; ++s)
        if (op[s] == b) {
            if (code == st) op[s] = -1; else oc[s] = (int8_t)code;
            return;
        }
    if (code == st) return;
    for (int s = 0; s < 4; ++s)
        if (op[s] < 0) { op[s] = b; oc[s] = (int8_t)code; return; }
    set_err(E, DMD_E_CAPACITY, a);
}
__device__ __forceinline__ void helpers_of(const DSys &S, int i, int j, int &ncim1, int &ncai, int &ncaj, int &nnjp1) {
    int Li = S.info[i].L, Lj = S.info[j].L;
    ncim1 = i + Li - 1; ncai = i - Li; ncaj = j - 2 * Lj; nnjp1 = j - Lj + 1;
}
/* the two index-derived helpers of an NH or CO bead, else -1 */
__device__ __forceinline__ void own_helpers(const DSys &S, int x, int &h1, int &h2) {
    h1 = h2 = -1;
    if (x < 0) return;
    BeadInfo I = S.info[x];
    if (I.kind == BK_NH) { h1 = x + I.L - 1; h2 = x - I.L; }
    else if (I.kind == BK_CO) { h1 = x - 2 * I.L; h2 = x - I.L + 1; }
}
__device__ void repuls_add(const DSys &S, Err E, int i, int j, int hbonds) {  /* i = NH, j = CO */
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, i, j, ncim1, ncai, ncaj, nnjp1);
    ovr_set(S, E, ncaj, i, 50, hbonds); ovr_set(S, E, i, ncaj, 40, hbonds);
    ovr_set(S, E, i, nnjp1, 40, hbonds); ovr_set(S, E, nnjp1, i, 50, hbonds);
    ovr_set(S, E, ncai, j, 50, hbonds); ovr_set(S, E, j, ncai, 40, hbonds);
    ovr_set(S, E, j, ncim1, 40, hbonds); ovr_set(S, E, ncim1, j, 50, hbonds);
    int *er = S.er;
    er[4 * i + 0] = ncaj; er[4 * i + 1] = nnjp1; er[4 * ncaj + 2] = i; er[4 * nnjp1 + 2] = i;
    er[4 * j + 0] = ncai; er[4 * j + 1] = ncim1; er[4 * ncai + 2] = j; er[4 * ncim1 + 2] = j;
    er[4 * i + 3] = j; er[4 * j + 3] = i;
}
__device__ void shoulders_off(const DSys &S, Err E, int n, int c, int hbonds) {
    int ncaj = S.er[4 * n + 0], nnjp1 = S.er[4 * n + 1], ncai = S.er[4 * c + 0], ncim1 = S.er[4 * c + 1];
    if (ncaj >= 0) { ovr_set(S, E, ncaj, n, 1, hbonds); ovr_set(S, E, n, ncaj, 1, hbonds); }
    if (nnjp1 >= 0) { ovr_set(S, E, n, nnjp1, 1, hbonds); ovr_set(S, E, nnjp1, n, 1, hbonds); }
    if (ncai >= 0) { ovr_set(S, E, ncai, c, 1, hbonds); ovr_set(S, E, c, ncai, 1, hbonds); }
    if (ncim1 >= 0) { ovr_set(S, E, c, ncim1, 1, hbonds); ovr_set(S, E, ncim1, c, 1, hbonds); }
}
__device__ void repuls_del_b(const DSys &S, int i, int j) {
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, i, j, ncim1, ncai, ncaj, nnjp1);
    int *er = S.er;
    er[4 * i + 0] = -1; er[4 * i + 1] = -1; er[4 * ncaj + 2] = -1; er[4 * nnjp1 + 2] = -1;
    er[4 * j + 0] = -1; er[4 * j + 1] = -1; er[4 * ncai + 2] = -1; er[4 * ncim1 + 2] = -1;
    er[4 * i + 3] = -1; er[4 * j + 3] = -1;
}

/* ------------------------------------------------------------------ */
/* CTA-wide reductions                                                 */
/* ------------------------------------------------------------------ */
__device__ double cta_max(SharedState &sh, double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh.red_d[w] = v;
    __syncthreads();
    double r = sh.red_d[0];
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) r = fmax(r, sh.red_d[k]);
    __syncthreads();
    return r;
}
__device__ double cta_sum(SharedState &sh, double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh.red_d[w] = v;
    __syncthreads();
    double r = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r += sh.red_d[k];
    __syncthreads();
    return r;
}
__device__ int cta_sum_i(SharedState &sh, int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    int w = threadIdx.x >> 5;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh.red_i[w] = v;
    __syncthreads();
    int r = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r += sh.red_i[k];
    __syncthreads();
    return r;
}

/* ------------------------------------------------------------------ */
/* CTA-wide: list rebuild and full prediction (code/nbor.f, code/events.f) */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ int cell_coord(double p, int nc) {
    double c = (p + 0.5) * nc;
    if (!(c >= 0.0)) return 0;   /* also catches NaN */
    int k = (int)c;
    return k < nc ? k : nc - 1;
}

/* Working arrays of a rebuild: single-precision positions, each bead's
 * cell, the cell-sorted beads and the cell counts and starts.  Staged in
 * shared memory (scr) when they fit - data the rebuild writes and reads
 * back at once - else the positions and the grid use the system's global
 * arrays. */
struct ListStage {
    const float *xf, *yf, *zf;
    int *cell_of, *cell_count, *cell_start, *cell_beads;
    BeadInfo *info;     /* the bead records, or null: the system's array */
    uint8_t *ovf;       /* 1 where a bead has an override slot in use (null with info) */
};
/* Staging order, each part only if it and the ones before it fit: positions,
 * cells and sorted beads (20 B per bead); bead records and override flags
 * (sizeof(BeadInfo) + 1 B per bead); cell counts and starts. */
__device__ ListStage list_stage(const DSys &S, char *scr, int scr_bytes) {
    const int N = S.N, nc = S.ncell;
    const size_t nc3 = (size_t)nc * nc * nc;
    ListStage L{S.xf, S.yf, S.zf, nullptr, S.cell_count, S.cell_start, S.cell_beads, nullptr, nullptr};
    if (scr == nullptr || (size_t)20 * N > (size_t)scr_bytes) return L;
    float *f = reinterpret_cast<float *>(scr);
    L.xf = f; L.yf = f + N; L.zf = f + 2 * N;
    L.cell_of = reinterpret_cast<int *>(f + 3 * N);
    L.cell_beads = L.cell_of + N;
    size_t used = (size_t)20 * N;
    const size_t info_bytes = ((sizeof(BeadInfo) * (size_t)N + (size_t)N) + 15) & ~(size_t)15;
    if (used + info_bytes <= (size_t)scr_bytes) {
        L.info = reinterpret_cast<BeadInfo *>(scr + used);
        L.ovf = reinterpret_cast<uint8_t *>(scr + used + sizeof(BeadInfo) * (size_t)N);
        used += info_bytes;
    }
    if (used + 4 * (2 * nc3 + 1) <= (size_t)scr_bytes) {
        L.cell_count = reinterpret_cast<int *>(scr + used);
        L.cell_start = L.cell_count + nc3;
    }
    return L;
}

__device__ void cta_build_lists(const DSys &S, SharedState &sh, int hbonds, const ListStage &L) {
    const int N = S.N, nc = S.ncell;
    const int ncell3 = nc * nc * nc;
    const DTab &T = *S.tab;
    int *const cell_count = L.cell_count, *const cell_start = L.cell_start, *const cell_beads = L.cell_beads;
    if (nc >= 3) {
        for (int c = threadIdx.x; c < ncell3; c += blockDim.x) cell_count[c] = 0;
        __syncthreads();
        for (int b = threadIdx.x; b < N; b += blockDim.x) {
            int c;
            if (L.cell_of) c = L.cell_of[b];
            else { int cx = cell_coord(S.x[b], nc), cy = cell_coord(S.y[b], nc), cz = cell_coord(S.z[b], nc); c = (cz * nc + cy) * nc + cx; }
            atomicAdd(&cell_count[c], 1);
        }
        __syncthreads();
        DMD_ISUB(11);
        {
            int per = (ncell3 + blockDim.x - 1) / blockDim.x;
            int lo = threadIdx.x * per, hi = min(lo + per, ncell3);
            int s = 0;
            for (int c = lo; c < hi; ++c) s += cell_count[c];
            int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            int incl = s;
            for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(FULL, incl, o); if (lane >= o) incl += v; }
            __syncthreads();
            if (lane == 31) sh.red_i[w] = incl;
            __syncthreads();
            int woff = 0;
            for (int k = 0; k < w; ++k) woff += sh.red_i[k];
            int run = woff + incl - s;
            for (int c = lo; c < hi; ++c) { int v = cell_count[c]; cell_start[c] = run; run += v; }
            __syncthreads();
            for (int c = lo; c < hi; ++c) cell_count[c] = 0;
            if (threadIdx.x == 0) cell_start[ncell3] = N;
            __syncthreads();
        }
        DMD_ISUB(12);
        for (int b = threadIdx.x; b < N; b += blockDim.x) {
            int c;
            if (L.cell_of) c = L.cell_of[b];
            else { int cx = cell_coord(S.x[b], nc), cy = cell_coord(S.y[b], nc), cz = cell_coord(S.z[b], nc); c = (cz * nc + cy) * nc + cx; }
            int slot = atomicAdd(&cell_count[c], 1);
            cell_beads[cell_start[c] + slot] = b;
        }
        __syncthreads();
        DMD_ISUB(13);
    }
    int mdn = 0;
    const float far_f = T.rlsq_max_f + (4e-7f + 4e-7f * T.rlsq_max_f);   /* above every cut + margin */
#ifdef DMD_PHASE_TIMERS
    const long long walk_t0 = clock64();
    long long walk_n = 0;
#endif
    for (int b = threadIdx.x; b < N; b += blockDim.x) {
        int nu = 0, nd = 0;
        int *up = S.up + (size_t)b * S.cap, *dn = S.dn + (size_t)b * S.cap;
        int8_t *upc = S.upc + (size_t)b * S.cap;
        const BeadInfo ib = L.info ? L.info[b] : S.info[b];
        const float xbf = L.xf[b], ybf = L.yf[b], zbf = L.zf[b];
        auto consider = [&](int c) {
            if (c == b) return;
            /* Single-precision prefilter.  Positions lie in [-0.5, 0.5] at a
             * rebuild, so each wrapped single-precision component is within
             * 1e-7 of the double one and r2 within 4e-7 + 4e-7 * r2; only
             * pairs that close to the cutoff are decided in double
             * precision, as the reference does. */
            float fx = xbf - L.xf[c], fy = ybf - L.yf[c], fz = zbf - L.zf[c];
            fx = fx - rintf(fx); fy = fy - rintf(fy); fz = fz - rintf(fz);
            const float r2f = fx * fx + fy * fy + fz * fz;
            const BeadInfo ic = L.info ? L.info[c] : S.info[c];
            /* a bead without any override: its pair codes are the rule's */
            const bool no_ov = L.ovf && !L.ovf[c];
            /* Beyond every pair type's cutoff: listed only as a bond pair
             * (same chain, residues at most 2 apart) or through an override */
            if (r2f > far_f) {
                const int dres = ic.res - ib.res;
                if (ic.chain != ib.chain || dres < -2 || dres > 2) {
                    if (no_ov) return;
                    const int *op = S.ovp + 4 * c;
                    if (op[0] != b && op[1] != b && op[2] != b && op[3] != b) return;
                }
            }
            int st = static_code(ic, ib, hbonds);
            int code = no_ov ? st : pair_code_st(S, c, b, st);
            bool take;
            if ((code >= 4 && code <= 12) || (code >= 17 && code < 27)) take = true;
            else {
                float cut = T.rlsq_f[code];
                float margin = 4e-7f + 4e-7f * cut;
                if (r2f > cut + margin) take = false;
                else if (r2f < cut - margin) take = true;
                else {
                    double rx = S.x[b] - S.x[c], ry = S.y[b] - S.y[c], rz = S.z[b] - S.z[c];
                    rx = rx - d_nint(rx); ry = ry - d_nint(ry); rz = rz - d_nint(rz);
                    double r2 = rx * rx + ry * ry + rz * rz;
                    take = r2 <= T.rlsq[code];
                }
            }
            if (!take) return;
            if (c > b) {
                if (nu < S.cap) { up[nu] = c; upc[nu] = (int8_t)st; }
                ++nu;
            } else {
                if (nd < S.cap) {
                    dn[nd] = c;
                    if (S.dnc) S.dnc[(size_t)b * S.cap + nd] = (int8_t)st;
                }
                ++nd;
            }
        };
        if (nc >= 3) {
            int cx, cy, cz;
            if (L.cell_of) { const int cb = L.cell_of[b]; cx = cb % nc; cy = (cb / nc) % nc; cz = cb / (nc * nc); }
            else { cx = cell_coord(S.x[b], nc); cy = cell_coord(S.y[b], nc); cz = cell_coord(S.z[b], nc); }
            /* The 27 cells as bead ranges of the cell-sorted array: a row of
             * three cells along x is one range, or two where it wraps around
             * the box.  The ranges are loaded first; then the walk runs over
             * all of them as one sequence, so that the lanes of a warp (one
             * bead each) stay together for as many steps as their longest
             * sequence instead of their longest cell of every one of 27. */
            const int xl = cx == 0 ? nc - 1 : cx - 1, xh = cx == nc - 1 ? 0 : cx + 1;
            const bool wrapx = xl > xh;
            /* range sr (0..17) of the 27 cells: rows of three cells along x,
             * two ranges where a row wraps around the box; its bounds come
             * from the cell starts when the walk reaches it (a dynamically
             * indexed array of them would live in local memory) */
            auto range = [&](int sr, int &lo, int &hi) {
                const int row = sr >> 1;
                int gy = cy + row % 3 - 1, gz = cz + row / 3 - 1;
                gy = gy < 0 ? gy + nc : (gy >= nc ? gy - nc : gy);
                gz = gz < 0 ? gz + nc : (gz >= nc ? gz - nc : gz);
                const int base = (gz * nc + gy) * nc;
                if ((sr & 1) == 0) { lo = cell_start[base + xl]; hi = cell_start[base + (wrapx ? nc : xh + 1)]; }
                else if (wrapx) { lo = cell_start[base]; hi = cell_start[base + xh + 1]; }
                else { lo = 0; hi = 0; }
            };
            int sr = 0, q = 0, e = 0;
            range(0, q, e);
            while (q >= e && ++sr < 18) range(sr, q, e);
            int c = sr < 18 ? cell_beads[q] : -1;
#ifdef DMD_PHASE_TIMERS
            {   /* candidates this bead walks: the total, and the grid size */
                int cnt = 0;
                for (int k = 0; k < 18; ++k) { int lo, hi; range(k, lo, hi); cnt += hi > lo ? hi - lo : 0; }
                walk_n += cnt;
                if (blockIdx.x == g_sub_cta) {
                    atomicAdd((unsigned long long *)&g_phase_cycles[DMD_PHASE_CTAS - 7][13], (unsigned long long)cnt);
                    if (b == 0) g_phase_cycles[DMD_PHASE_CTAS - 7][14] = nc;
                }
            }
#endif
            while (sr < 18) {
                /* the next candidate's index is loaded before this one is tested */
                ++q;
                while (q >= e && ++sr < 18) range(sr, q, e);
                const int cn = sr < 18 ? cell_beads[q] : -1;
                consider(c);
                c = cn;
            }
        } else {
            for (int c = 0; c < N; ++c) consider(c);
        }
        if (nu > S.cap || nd > S.cap) set_err(sh, DMD_E_CAPACITY, b);
        S.upn[b] = min(nu, S.cap);
        S.dnn[b] = min(nd, S.cap);
        mdn = max(mdn, min(nd, S.cap));
    }
#ifdef DMD_PHASE_TIMERS
    if (blockIdx.x == g_sub_cta) {   /* the slowest thread's walk: cycles, and its candidates */
        const unsigned long long wt = (unsigned long long)(clock64() - walk_t0);
        const unsigned long long old = atomicMax((unsigned long long *)&g_phase_cycles[DMD_PHASE_CTAS - 7][12], wt);
        if (wt > old) g_phase_cycles[DMD_PHASE_CTAS - 7][15] = walk_n;
    }
#endif
    /* the longest down list, which selects the k_run variant */
    mdn = __reduce_max_sync(FULL, mdn);
    __syncthreads();
    DMD_ISUB(14);
    if ((threadIdx.x & 31) == 0) sh.red_i[threadIdx.x >> 5] = mdn;
    __syncthreads();
    if (threadIdx.x == 0) {
        int m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = max(m, sh.red_i[w]);
        sh.sc.max_dn = m;
    }
    __syncthreads();
}

/* position of the n-th (0-based) set bit of m; n < popc(m) */
__device__ __forceinline__ int nth_set_bit(unsigned m, int n) {
    int pos = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) {
        const int c = __popc((m >> pos) & ((1u << w) - 1u));
        if (n >= c) { n -= c; pos += w; }
    }
    return pos;
}

/* events() for beads b0 .. b0+nb-1 (nb <= TG_MAX) on one warp: every
 * (bead, partner) pair of the up lists and extras is one task, 32 per pass,
 * and the minimum per bead is a segmented reduction over the lanes
 * (code/events.f:23-123) */
__device__ void warp_predict_beads(const DSys &S, Err E, FullScratch &F, int b0, int nb, double interval_max,
                                   int hbonds) {
    int lane = threadIdx.x & 31;
    const double H = interval_max + DMD_LTSTEP;
    const long long Hkey = okey(H), imax_key = okey(interval_max);
    for (int t = lane; t < nb; t += 32) {
        F.tg_b[t] = b0 + t;
        F.tg_k[t] = Hkey; F.tg_p[t] = -1; F.tg_raw[t] = H; F.tg_y[t] = -1;
    }
    int run = 0;
    for (int base = 0; base < nb; base += 32) {
        int t = base + lane;
        int c = 0;
        if (t < nb) {
            int b = b0 + t;
            c = S.upn[b];
            for (int k = 0; k < 3; ++k) c += S.er[4 * b + k] > b;
        }
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(FULL, incl, o); if (lane >= o) incl += v; }
        if (t < nb) F.tg_base[t] = run + incl - c;
        run += __shfl_sync(FULL, incl, 31);
    }
    if (lane == 0) F.tg_base[nb] = run;
    __syncwarp();
    const bool mapped = run <= TMAP_MAX;
    if (mapped) {
        for (int t = lane; t < nb; t += 32)
            for (int q = F.tg_base[t]; q < F.tg_base[t + 1]; ++q) F.tmap[q] = (int8_t)t;
        __syncwarp();
    }
    /* The tasks are decoded 32 at a time and screened in single precision;
     * the ones that may have an event queue up in two register slots per
     * lane (in task order, so a bead's tasks stay contiguous) and run in
     * double precision 32 at a time. */
    int qa_t = -1, qa_a = -1, qa_b = -1, qa_c = 0;   /* slot A: target, bead, partner, code */
    int qb_t = -1, qb_a = -1, qb_b = -1, qb_c = 0;   /* slot B */
    int pend = 0;
    auto predict32 = [&](int tgt, int pa, int pbb, int code) {
        double tij = 0.0;
        int ty = 0;
        bool ok = false;
        if (pa >= 0) {
            ok = d_predict_c(S, pa, pbb, code, 0.0, tij, ty);
            if (!ok) set_err(E, DMD_E_INPUT, pa);
            else if (okey(tij) < okey(-1.0e-10)) set_err(E, DMD_E_NEG_TIME, pa);
        }
        long long k = (tgt >= 0 && ok) ? okey(tij) : DMD_KEY_INF;
        int p = (tgt >= 0 && ok) ? pbb : INT_MAX;
        double rt = tij;
        int y = ty;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long k2 = __shfl_down_sync(FULL, k, o);
            int p2 = __shfl_down_sync(FULL, p, o);
            double r2 = __shfl_down_sync(FULL, rt, o);
            int y2 = __shfl_down_sync(FULL, y, o);
            int g2 = __shfl_down_sync(FULL, tgt, o);
            if (lane + o < 32 && g2 == tgt && key_less(k2, p2, k, p)) { k = k2; p = p2; rt = r2; y = y2; }
        }
        int gprev = __shfl_up_sync(FULL, tgt, 1);
        bool head = tgt >= 0 && (lane == 0 || gprev != tgt);
        if (head && key_less(k, p, F.tg_k[tgt], F.tg_p[tgt])) {
            F.tg_k[tgt] = k; F.tg_p[tgt] = p; F.tg_raw[tgt] = rt; F.tg_y[tgt] = (int8_t)y;
        }
        __syncwarp();
    };
    for (int base = 0; base < run; base += 32) {
        int q = base + lane;
        int tgt = -1, pa = -1, pbb = -1, st = -1;
        if (q < run) {
            int lo;
            if (mapped) lo = F.tmap[q];
            else {
                int hi = nb - 1;
                lo = 0;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (F.tg_base[mid] <= q) lo = mid; else hi = mid - 1;
                }
            }
            tgt = lo;
            int b = b0 + lo;
            int k = q - F.tg_base[lo];
            int nu = S.upn[b];
            int m;
            if (k < nu) { m = S.up[(size_t)b * S.cap + k]; st = S.upc[(size_t)b * S.cap + k]; }
            else {
                int want = k - nu;
                m = -1;
                for (int k2 = 0; k2 < 3; ++k2) {
                    int e = S.er[4 * b + k2];
                    if (e > b) { if (want == 0) { m = e; break; } --want; }
                }
            }
            if (m > b) { pa = b; pbb = m; }
        }
        int code = 0;
        bool live = false;
        if (pa >= 0) {
            code = st >= 0 ? pair_code_st(S, pbb, pa, st) : pair_code(S, pbb, pa, hbonds);
            /* no event for certain: it cannot win against the horizon */
            live = !f32_no_event(S, pa, pbb, code, 0u);
        }
        const unsigned m = __ballot_sync(FULL, live);
        const int cnt = __popc(m);
        /* lane d of slot A takes the (d - pend)-th live task, of slot B the (d + 32 - pend)-th */
        {
            const int na = lane - pend, nb2 = lane + 32 - pend;
            const int sa = (na >= 0 && na < cnt) ? nth_set_bit(m, na) : 0;
            const int sb = (nb2 < cnt) ? nth_set_bit(m, nb2) : 0;
            const int ta = __shfl_sync(FULL, tgt, sa), aa = __shfl_sync(FULL, pa, sa);
            const int ba = __shfl_sync(FULL, pbb, sa), ca = __shfl_sync(FULL, code, sa);
            const int tb = __shfl_sync(FULL, tgt, sb), ab = __shfl_sync(FULL, pa, sb);
            const int bb = __shfl_sync(FULL, pbb, sb), cb = __shfl_sync(FULL, code, sb);
            if (na >= 0 && na < cnt) { qa_t = ta; qa_a = aa; qa_b = ba; qa_c = ca; }
            if (nb2 < cnt) { qb_t = tb; qb_a = ab; qb_b = bb; qb_c = cb; }
        }
        pend += cnt;
        if (pend >= 32) {
            predict32(qa_t, qa_a, qa_b, qa_c);
            qa_t = qb_t; qa_a = qb_a; qa_b = qb_b; qa_c = qb_c;
            qb_t = -1; qb_a = -1; qb_b = -1; qb_c = 0;
            pend -= 32;
        }
    }
    if (pend > 0) {
        if (lane >= pend) { qa_t = -1; qa_a = -1; }
        predict32(qa_t, qa_a, qa_b, qa_c);
    }
    for (int t = lane; t < nb; t += 32)
        set_pred(S, b0 + t, F.tg_raw[t], F.tg_p[t], F.tg_y[t], F.tg_k[t] < imax_key);
    __syncwarp();
}

/* events(): every bead over its up list and extras, TG_MAX beads per warp
 * at a time */
/* the scratch of warp w is at fs0 + w * stride bytes */
struct ScratchRef { char *fs0; size_t stride; };
__device__ void cta_predict_all(const DSys &S, SharedState &sh, ScratchRef fr, double interval_max, int hbonds) {
    const int N = S.N;
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    FullScratch &F = *(FullScratch *)(fr.fs0 + (size_t)warp * fr.stride);
    for (int b0 = warp * TG_MAX; b0 < N; b0 += nwarps * TG_MAX)
        warp_predict_beads(S, cta_err(sh), F, b0, min(TG_MAX, N - b0), interval_max, hbonds);
    if (threadIdx.x < 3) {
        int e = N + threadIdx.x;
        bool q = S.tim[e] < interval_max;
        S.queued[e] = q;
        S.key[e] = q ? okey(S.tim[e]) : DMD_KEY_INF;
    }
    __syncthreads();
}

/* rebuild: wrap the positions into the box, cell lists, neighbour lists,
 * full prediction, tournament.  scr (scr_bytes, may be null): shared memory
 * free for the list build. */
__device__ void cta_rebuild(const DSys &S, SharedState &sh, ScratchRef fr, int hbonds, char *scr, int scr_bytes) {
    DMD_SUB(-1);
    const ListStage L = list_stage(S, scr, scr_bytes);
    const int nc = S.ncell;
    for (int b = threadIdx.x; b < S.N; b += blockDim.x) {
        double px = S.x[b], py = S.y[b], pz = S.z[b];
        px = px - d_nint(px); py = py - d_nint(py); pz = pz - d_nint(pz);
        S.x[b] = px; S.y[b] = py; S.z[b] = pz;
        S.ox[b] = px; S.oy[b] = py; S.oz[b] = pz;
        const float fx = (float)px, fy = (float)py, fz = (float)pz;
        S.xf[b] = fx; S.yf[b] = fy; S.zf[b] = fz;
        if (L.cell_of) {
            float *sx = const_cast<float *>(L.xf);
            sx[b] = fx; sx[b + S.N] = fy; sx[b + 2 * S.N] = fz;
            if (nc >= 3) L.cell_of[b] = (cell_coord(pz, nc) * nc + cell_coord(py, nc)) * nc + cell_coord(px, nc);
        }
        if (L.info) {
            L.info[b] = S.info[b];
            const int *op = S.ovp + 4 * b;
            L.ovf[b] = (op[0] >= 0) | (op[1] >= 0) | (op[2] >= 0) | (op[3] >= 0);
        }
    }
    __syncthreads();
    DMD_ISUB(7);
    cta_build_lists(S, sh, hbonds, L);
    DMD_ISUB(8);
    cta_predict_all(S, sh, fr, sh.sc.interval_max, hbonds);
    DMD_ISUB(9);
    cta_tree_rebuild(S);
    DMD_ISUB(10);
}

/* interval event N+2 (code/main.F90:1126-1187, code/displ.f), spread over the
 * C CTAs of the system: each shifts the times and advances the positions of
 * its slice of the beads; the leader (L, rank 0) takes the maximum
 * displacement and decides on a rebuild, which it does alone.  sh.tf_iv
 * holds tfalse of the event on every CTA. */
__device__ bool cluster_interval(const DSys &S, SharedState &sh, SharedState *L, int rank, int C, ScratchRef fr,
                                 int hbonds, char *scr, int scr_bytes) {
    const int N = S.N;
    const double tf = sh.tf_iv;
    const DTab &T = *S.tab;
    const int stride = C * blockDim.x, t0 = rank * blockDim.x + threadIdx.x;
    DMD_SUB(-1);
    DMD_ISUB(-1);
    for (int k0 = t0; k0 < N + 3; k0 += 4 * stride) {   /* four entries in flight per thread */
        double tv[4];
        uint8_t qv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int k = k0 + u * stride;
            if (k < N + 3) { tv[u] = S.tim[k]; qv[u] = S.queued[k]; }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int k = k0 + u * stride;
            if (k < N + 3) {
                double tn = tv[u] - tf;
                S.tim[k] = tn;
                S.key[k] = qv[u] ? okey(tn) : DMD_KEY_INF;
            }
        }
    }
    /* displ.f: the largest squared displacement over hdelr; dividing after
     * the maximum gives the same value, division being monotone.  The
     * squared displacements are non-negative: their maximum is taken on the
     * bit patterns. */
    long long dmax_bits = 0;
    for (int k0 = t0; k0 < N; k0 += 2 * stride) {   /* two beads in flight per thread */
        double p[2][9];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            int k = k0 + u * stride;
            if (k < N) {
                p[u][0] = S.x[k]; p[u][1] = S.y[k]; p[u][2] = S.z[k];
                p[u][3] = S.vx[k]; p[u][4] = S.vy[k]; p[u][5] = S.vz[k];
                p[u][6] = S.ox[k]; p[u][7] = S.oy[k]; p[u][8] = S.oz[k];
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            int k = k0 + u * stride;
            if (k < N) {
                double px = p[u][0] + p[u][3] * tf, py = p[u][1] + p[u][4] * tf, pz = p[u][2] + p[u][5] * tf;
                S.x[k] = px; S.y[k] = py; S.z[k] = pz;
                double a = p[u][6] - px, b = p[u][7] - py, c = p[u][8] - pz;
                double dis = a * a + b * b + c * c;
                long long db = dbits(dis);
                if (db > dmax_bits) dmax_bits = db;
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) { long long v = __shfl_xor_sync(FULL, dmax_bits, o); if (v > dmax_bits) dmax_bits = v; }
    DMD_ISUB(0);
    __syncthreads();
    DMD_ISUB(1);
    if ((threadIdx.x & 31) == 0) sh.red_d[threadIdx.x >> 5] = __longlong_as_double(dmax_bits);
    __syncthreads();
    if (threadIdx.x == 0) {
        long long m = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { long long v = dbits(sh.red_d[w]); if (v > m) m = v; }
        L->red_max[rank] = __longlong_as_double(m);
    }
    csync(C);
    if (rank == 0 && threadIdx.x == 0) {
        long long mb = 0;
        for (int q = 0; q < C; ++q) { long long v = dbits(sh.red_max[q]); if (v > mb) mb = v; }
        double dmax = __longlong_as_double(mb);
        double moved_far = 0.0;
        double moved = dmax / T.hdelr;
        if (moved > moved_far) moved_far = moved;
        sh.sc.t = sh.sc.t + tf;
        sh.sc.interval_max = sh.sc.interval_max - tf;
        sh.sc.tfalse = 0.0;
        bool update = false;
        if (moved_far >= 0.1) {
            update = true;
            if (moved_far >= 1.25 * 1.25) {
                sh.sc.t_fact = sh.sc.t_fact / 1.01;
                sh.sc.interval = sh.sc.t_fact / sqrt(T.setemp);
            }
        }
        sh.rebuild = 0;
        if (update || (sh.sc.interval > sh.sc.interval_max)) {
            if (!update) { sh.sc.n_forced_updates += 1; sh.sc.n_forced = sh.sc.n_forced * 1.01; }
            sh.sc.interval_max = sh.sc.interval * sh.sc.n_forced;
            sh.sc.n_updates += 1;
            sh.rebuild = 1;
        }
    }
    if (rank == 0) {
        __syncthreads();
        DMD_ISUB(2);
        if (sh.rebuild) {
            for (int k = threadIdx.x; k < N; k += blockDim.x) set_pred(S, k, sh.sc.interval_max + DMD_LTSTEP, -1, -1, false);
            __syncthreads();
            cta_rebuild(S, sh, fr, hbonds, scr, scr_bytes);
            DMD_ISUB(3);
        }
        if (threadIdx.x == 0) set_pred(S, N + 1, sh.sc.interval * 0.999, -2, -2, true);
    }
    csync(C);
    if (threadIdx.x == 0 && rank != 0) sh.rebuild = L->rebuild;
    __syncthreads();
    bool rb = sh.rebuild != 0;
    /* level 1 of the tournament, spread over the CTAs (level 2 follows at
     * the leader's next selection) */
    DMD_ISUB(4);
    for (int g = t0; g < S.nl1; g += stride) l1_update(S, g, N + 3);
    DMD_ISUB(5);
    return rb;
}

/* diagnostics (code/energy.f:1-105, radgyr.f:1-139, end2end.f:1-48) over the
 * neighbour lists; done by the whole CTA */
__device__ double dist_now(const DSys &S, int a, int b, double tfalse) {
    double vxa = S.vx[a] - S.vx[b], vya = S.vy[a] - S.vy[b], vza = S.vz[a] - S.vz[b];
    double rx = S.x[a] - S.x[b] + vxa * tfalse, ry = S.y[a] - S.y[b] + vya * tfalse, rz = S.z[a] - S.z[b] + vza * tfalse;
    rx = rx - d_nint(rx); ry = ry - d_nint(ry); rz = rz - d_nint(rz);
    double d = rx * rx + ry * ry + rz * rz;
    return sqrt(d);
}
/* code/checkover.f:18-131 over the neighbour lists (each pair once, from
 * the lower bead's up list; every pair the reference can flag is listed:
 * bonded pairs always, the others within their cutoff, which exceeds every
 * contact diameter).  A pair of type 1 or >= 15 whose squared distance
 * times 1.0000000001 is at most its squared core diameter overlaps; a
 * bonded pair (types 4-12) is broken when its squared distance times
 * 0.9999999999 exceeds the squared outer window or times 1.0000000001 falls
 * below the inner one.  The first offence found sets DMD_E_OVERLAP with the
 * pair's beads (0-based) in err_info / err_info2.  Returns the number of
 * offending pairs. */
__device__ int cta_checkover(const DSys &S, SharedState &sh) {
    const int N = S.N;
    const DTab &T = *S.tab;
    const double tf = sh.sc.tfalse;
    int bad_pairs = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const int *up = S.up + (size_t)i * S.cap;
        const int8_t *upc = S.upc + (size_t)i * S.cap;
        for (int k = 0; k < S.upn[i]; ++k) {
            const int j = up[k];
            const int code = pair_code_st(S, i, j, upc[k]);
            const int a = S.ident[i], b = S.ident[j];
            bool bad = false;
            if (code == 1 || code >= 15) {
                /* sigma_sq * ev_param(1,code)**2 (* sqz610**2 for 22-26):
                 * the tables hold these products in that order; the factor
                 * is 1 for 16 and the shoulder codes */
                const double sigsq = code == 15 ? T.core15_sq[a][b]
                                     : (code == 1 || (code >= 17 && code <= 26)) ? T.core_sq[core_slot_d(code)][a][b]
                                                                                 : T.sigma_sq[a][b];
                const Rel r = d_rel(S, i, j, tf);
                bad = r.rijsq * 1.0000000001 <= sigsq;
            } else if (code >= 4 && code <= 12) {
                const bool side = code >= 10;
                const double lo = side ? S.blmin_sq[i] : T.evp2_sq[code];
                const double hi = side ? S.blmax_sq[i] : T.evp3_sq[code];
                const Rel r = d_rel(S, i, j, tf);
                bad = r.rijsq * 0.9999999999 > hi || r.rijsq * 1.0000000001 < lo;
            }
            if (bad) {
                ++bad_pairs;
                if (atomicCAS(&sh.sc.err, 0, DMD_E_OVERLAP) == 0) { sh.sc.err_info = i; sh.sc.err_info2 = j; }
            }
        }
    }
    return cta_sum_i(sh, bad_pairs);
}

/* code/repuls_check.f:1-85 for the H-bond pair (n, c): 10 when the four
 * helper distances all exceed the shoulder distances, else 11 */
__device__ double repuls_rating(const DSys &S, int n, int c, double tf) {
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, n, c, ncim1, ncai, ncaj, nnjp1);
    const int pa[4] = {n, n, c, c}, pb[4] = {ncaj, nnjp1, ncai, ncim1};
    double d[4];
    for (int q = 0; q < 4; ++q) {
        const Rel r = d_rel(S, pa[q], pb[q], tf);
        d[q] = sqrt(r.rijsq);
    }
    const DTab &T = *S.tab;
    return (d[0] > T.shd1 && d[1] > T.shd2 && d[2] > T.shd3 && d[3] > T.shd4) ? 10.0 : 11.0;
}

/* code/check_nc_int.f:9-360 over the up lists: an H-bonded pair whose
 * geometry fails repuls_check (boundbad), and an unbonded NH-CO pair inside
 * its well whose geometry passes it (unboundbad); pairs with an end bead
 * (NH of residue 1, CO of residue L) are not rated. */
__device__ void cta_nc_int(const DSys &S, SharedState &sh, int &boundbad, int &unboundbad) {
    const int N = S.N;
    const DTab &T = *S.tab;
    const double tf = sh.sc.tfalse;
    int bb = 0, ub = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const int *up = S.up + (size_t)i * S.cap;
        const int8_t *upc = S.upc + (size_t)i * S.cap;
        for (int k = 0; k < S.upn[i]; ++k) {
            const int j = up[k];
            if (pair_code_st(S, i, j, upc[k]) != 15) continue;
            const bool ends = S.info[i].is_end || S.info[j].is_end;
            const int a = S.ident[i], b = S.ident[j];
            const int n = a < b ? i : j, c = a < b ? j : i;
            if (S.bptnr[i] == j) {
                const double rating = ends ? 10.0 : repuls_rating(S, n, c, tf);
                if (rating > 10.0) ++bb;
            } else {
                const Rel r = d_rel(S, i, j, tf);
                if (r.rijsq - T.welldia_sq[a][b] < 0.0) {
                    const double rating = ends ? 11.0 : repuls_rating(S, n, c, tf);
                    if (rating <= 10.0) ++ub;
                }
            }
        }
    }
    boundbad = cta_sum_i(sh, bb);
    unboundbad = cta_sum_i(sh, ub);
}

__device__ void cta_diag(const DSys &S, SharedState &sh, const int *chain_start, const int *chain_len,
                         dmd_diag *out) {
    const int N = S.N;
    const DTab &T = *S.tab;
    double tf = sh.sc.tfalse;
    double sumvel = 0.0, ehh_ii = 0.0, ehh_ij = 0.0, nbr = 0.0;
    int hb_ii = 0, hb_ij = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        nbr += (double)(S.upn[i] + S.dnn[i]);
        sumvel += S.bm[i] * (S.vx[i] * S.vx[i] + S.vy[i] * S.vy[i] + S.vz[i] * S.vz[i]);
        int p = S.bptnr[i];
        if (p > i) { if (S.info[p].chain == S.info[i].chain) ++hb_ii; else ++hb_ij; }
        const int *up = S.up + (size_t)i * S.cap;
        const int8_t *upc = S.upc + (size_t)i * S.cap;
        for (int k = 0; k < S.upn[i]; ++k) {
            if (upc[k] != 16) continue;
            int j = up[k];
            if (S.bptnr[i] == j) continue;
            Rel r = d_rel(S, i, j, tf);
            int a = S.ident[i], b = S.ident[j];
            if (r.rijsq <= T.welldia_sq[a][b]) {
                if (S.info[i].chain == S.info[j].chain) ehh_ii += T.ep_sqrt[a][b]; else ehh_ij += T.ep_sqrt[a][b];
            }
        }
    }
    sumvel = cta_sum(sh, sumvel);
    nbr = cta_sum(sh, nbr);
    ehh_ii = cta_sum(sh, ehh_ii);
    ehh_ij = cta_sum(sh, ehh_ij);
    hb_ii = cta_sum_i(sh, hb_ii);
    hb_ij = cta_sum_i(sh, hb_ij);
    int hb_alpha = 0;
    double rgsum = 0.0, e2e = 0.0;
    int nbb = 0;
    for (int c = threadIdx.x; c < S.nchains; c += blockDim.x) {
        int s = chain_start[c], L = chain_len[c];
        for (int a = L + 5; a <= 2 * L; ++a) { int i = s + a - 1, j = i + L - 4; if (S.bptnr[i] == j) ++hb_alpha; }
        /* radius of gyration of the backbone (code/radgyr.f:19-75): C-alpha
         * unwrapped along the chain, NH and CO against their own C-alpha */
        double cx = 0, cy = 0, cz = 0;
        for (int pass = 0; pass < 2; ++pass) {
            double ca[3] = {0, 0, 0};
            for (int k = 1; k <= L; ++k) {
                double p[3][3];
                int bb[3] = {s + k - 1, s + L + k - 1, s + 2 * L + k - 1};
                for (int m = 0; m < 3; ++m) {
                    int q = bb[m];
                    p[m][0] = S.x[q] + S.vx[q] * tf; p[m][1] = S.y[q] + S.vy[q] * tf; p[m][2] = S.z[q] + S.vz[q] * tf;
                }
                for (int d = 0; d < 3; ++d) {
                    if (k > 1) {
                        double d0 = p[0][d] - ca[d];
                        if (d0 > 0.5) p[0][d] -= 1.0; else if (d0 < -0.5) p[0][d] += 1.0;
                    }
                    ca[d] = p[0][d];
                    for (int m = 1; m < 3; ++m) {
                        double d0 = p[m][d] - ca[d];
                        if (d0 > 0.5) p[m][d] -= 1.0; else if (d0 < -0.5) p[m][d] += 1.0;
                    }
                }
                for (int m = 0; m < 3; ++m) {
                    if (pass == 0) { cx += p[m][0]; cy += p[m][1]; cz += p[m][2]; }
                    else {
                        double a0 = p[m][0] - cx, a1 = p[m][1] - cy, a2 = p[m][2] - cz;
                        rgsum += a0 * a0 + a1 * a1 + a2 * a2;
                    }
                }
            }
            if (pass == 0) { cx /= (double)(3 * L); cy /= (double)(3 * L); cz /= (double)(3 * L); }
        }
        nbb += 3 * L;
        int a = s + L, b = s + 3 * L - 1;
        e2e += dist_now(S, a, b, tf);
    }
    hb_alpha = cta_sum_i(sh, hb_alpha);
    e2e = cta_sum(sh, e2e);
    rgsum = cta_sum(sh, rgsum);
    nbb = cta_sum_i(sh, nbb);
    int boundbad = 0, unboundbad = 0;
    cta_nc_int(S, sh, boundbad, unboundbad);
    if (threadIdx.x == 0 && out) {
        double sumeps = -((hb_ii + hb_ij) * T.eps_hb + (ehh_ii + ehh_ij));
        out->e_total = 0.5 * sumvel + sumeps;
        out->e_kin = 0.5 * sumvel;
        out->temperature = sumvel / 3.0 / (double)N;
        out->hb_alpha = hb_alpha; out->hb_ii = hb_ii; out->hb_ij = hb_ij;
        out->ehh_ii = ehh_ii; out->ehh_ij = ehh_ij;
        out->rg = sqrt(rgsum / (double)nbb) * T.boxl_orig;
        out->e2e = e2e / (double)S.nchains * T.boxl_orig;
        for (int k = 0; k < 32; ++k) out->nevents[k] = sh.sc.nevents[k];
        out->coll = sh.sc.coll; out->n_pair = sh.sc.n_pair; out->n_ghost = sh.sc.n_ghost;
        out->n_interval = sh.sc.n_interval; out->n_output = sh.sc.n_output; out->n_updates = sh.sc.n_updates;
        out->n_forced_updates = sh.sc.n_forced_updates; out->t = sh.sc.t; out->tfalse = sh.sc.tfalse;
        out->nbr_mean = nbr / (double)N;
        out->n_batches = sh.sc.n_batches; out->n_rolled_back = sh.sc.n_rolled_back;
        out->n_candidates = sh.sc.n_candidates;
        out->max_down = sh.sc.max_dn;
        out->nc_boundbad = boundbad;
        out->nc_unboundbad = unboundbad;
        out->run_cycles = sh.sc.run_cycles;
    }
    __syncthreads();
}

/* ------------------------------------------------------------------ */
/* batch selection                                                     */
/* ------------------------------------------------------------------ */
/* The bead events below the cut, sorted in (key, index) order into
 * sh.sort_*; returns how many there are (1 when the window could not be
 * made small enough: the root alone). */
/* warp: the earliest queue entry (index, key), or -1 when the queue is
 * empty: the argmin over the level-1 groups, through level 2 for large
 * systems */
__device__ int warp_root(const DSys &S, long long &kroot) {
    const int lane = threadIdx.x & 31;
    long long bk = DMD_KEY_INF;
    int best = INT_MAX;
    if (S.nl1 <= 256) {
        /* eight groups per lane, every load issued before the first compare */
        long long kq[8];
        int eq[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int g = lane + 32 * q;
            kq[q] = g < S.nl1 ? S.l1k[g] : DMD_KEY_INF;
            eq[q] = g < S.nl1 ? S.l1i[g] : INT_MAX;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (key_less(kq[q], eq[q], bk, best)) { bk = kq[q]; best = eq[q]; }
    } else {
        for (int h = lane; h < S.nl2; h += 32) l2_update(S, h);
        __syncwarp();
        for (int h = lane; h < S.nl2; h += 32) {
            const long long k = S.l2k[h];
            const int e = S.l2i[h];
            if (key_less(k, e, bk, best)) { bk = k; best = e; }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long k2 = __shfl_xor_sync(FULL, bk, o);
        int b2 = __shfl_xor_sync(FULL, best, o);
        if (key_less(k2, b2, bk, best)) { bk = k2; best = b2; }
    }
    kroot = bk;
    return bk == DMD_KEY_INF ? -1 : best;
}

/* the double whose okey() is k (k of a finite time) */
__device__ __forceinline__ double key_time(long long k) {
    return __longlong_as_double(k >= 0 ? k : (k ^ 0x7fffffffffffffffLL));
}

#define FEW_GROUPS 256    /* level-1 groups (8 per lane) scanned by every warp from registers */
#define GSEL_MAX 8        /* groups below the cut one warp takes per attempt */

/* The batch candidates: every bead entry whose key lies below a cut (and
 * below every pseudo event), sorted in (key, index) order into
 * sh.sort_key/sort_idx; the first is the root.  The cut is the root's time
 * plus a window sh.delta that adapts to aim at one to two candidates per
 * warp slot.  Every warp scans the level-1 minima against the cut and takes
 * every nw-th group below it; warp 0 sorts.  Each step issues all of its
 * global loads before it uses the first (they take hundreds of cycles
 * each).  sh.ncand must be 0 on entry.  Returns their number (1 if the
 * window cannot be made small enough). */
__device__ int cta_gather_candidates(const DSys &S, SharedState &sh, int root, long long kroot, int slots) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int N = S.N, nl1 = S.nl1;
    DMD_GSUB_START();
    /* the loads that do not depend on the cut, issued together: the pseudo
     * events' keys and, for up to 256 groups, every level-1 minimum (each
     * lane holds eight); the root's time is its key read back */
    const bool few = nl1 <= FEW_GROUPS;
    long long gk[FEW_GROUPS / 32];
#pragma unroll
    for (int q = 0; q < FEW_GROUPS / 32; ++q) {
        const int g = lane + 32 * q;
        gk[q] = few && g < nl1 ? S.l1k[g] : DMD_KEY_INF;
    }
    const long long kp = min(min(S.key[N], S.key[N + 1]), S.key[N + 2]);
    const double t_root = key_time(kroot);
    int nc = 0;
    bool ok = false;
    for (int attempt = 0; attempt < 8; ++attempt) {
        long long kc = okey(t_root + sh.delta);
        if (kc <= kroot) kc = kroot + 1;
        if (kc > kp) kc = kp;
        DMD_GSUB(0);
        bool over = false;
        if (few) {
            /* the groups whose minimum lies below the cut, in order; a group
             * below the cut holds at least one candidate, so more than
             * CAND_MAX of them overflow at once.  This warp takes the
             * ordinals warp, warp + nw, ... and loads their keys together. */
            unsigned gm[FEW_GROUPS / 32];
            int pre[FEW_GROUPS / 32 + 1];
            pre[0] = 0;
#pragma unroll
            for (int q = 0; q < FEW_GROUPS / 32; ++q) {
                gm[q] = __ballot_sync(FULL, gk[q] < kc);
                pre[q + 1] = pre[q] + __popc(gm[q]);
            }
            const int ng = pre[FEW_GROUPS / 32];
            over = ng > CAND_MAX;
            if (!over) {
                int gsel[GSEL_MAX];
                int ns = 0;
#pragma unroll
                for (int u = 0; u < GSEL_MAX; ++u) {
                    const int o = warp + u * nw;
                    gsel[u] = -1;
                    if (o < ng) {
                        /* the register word holding ordinal o, picked with
                         * constant indices (a computed index would put gm
                         * and pre in local memory) */
                        int q = 0, pq = 0;
                        unsigned gq = gm[0];
#pragma unroll
                        for (int qq = 1; qq < FEW_GROUPS / 32; ++qq)
                            if (o >= pre[qq]) { q = qq; pq = pre[qq]; gq = gm[qq]; }
                        gsel[u] = 32 * q + (int)__fns(gq, 0, o - pq + 1);
                        ns = u + 1;
                    }
                }
                long long kv[GSEL_MAX];
#pragma unroll
                for (int u = 0; u < GSEL_MAX; ++u) {
                    const int e = gsel[u] * 32 + lane;
                    kv[u] = (gsel[u] >= 0 && e < N) ? S.key[e] : DMD_KEY_INF;
                }
                unsigned cm[GSEL_MAX];
                int tot = 0;
#pragma unroll
                for (int u = 0; u < GSEL_MAX; ++u) {
                    cm[u] = __ballot_sync(FULL, u < ns && kv[u] < kc);
                    tot += __popc(cm[u]);
                }
                int pos = 0;
                if (lane == 0 && tot) pos = atomicAdd(&sh.ncand, tot);
                pos = __shfl_sync(FULL, pos, 0);
#pragma unroll
                for (int u = 0; u < GSEL_MAX; ++u) {
                    const int p = pos + __popc(cm[u] & lt);
                    if (((cm[u] >> lane) & 1u) && p < CAND_MAX) { sh.cand_key[p] = kv[u]; sh.cand_idx[p] = gsel[u] * 32 + lane; }
                    pos += __popc(cm[u]);
                }
            }
        } else {
            /* many groups: each warp scans blocks of 32 groups in turn */
            for (int gb = 32 * warp; gb < nl1; gb += 32 * nw) {
                const int g = gb + lane;
                unsigned gmk = __ballot_sync(FULL, g < nl1 && S.l1k[g] < kc);
                while (gmk) {
                    const int gg = gb + __ffs(gmk) - 1;
                    gmk &= gmk - 1;
                    const int e = gg * 32 + lane;
                    const long long k = e < N ? S.key[e] : DMD_KEY_INF;
                    const bool c = k < kc;
                    const unsigned cmk = __ballot_sync(FULL, c);
                    int pos = 0;
                    if (lane == 0 && cmk) pos = atomicAdd(&sh.ncand, __popc(cmk));
                    pos = __shfl_sync(FULL, pos, 0) + __popc(cmk & lt);
                    if (c && pos < CAND_MAX) { sh.cand_key[pos] = k; sh.cand_idx[pos] = e; }
                }
            }
        }
        DMD_GSUB(1);
        __syncthreads();
        DMD_GSUB(2);
        nc = sh.ncand;
        ok = !over && nc <= CAND_MAX;
#ifdef DMD_PHASE_TIMERS
        if (threadIdx.x == 0 && blockIdx.x < 500) g_phase_cycles[512 + blockIdx.x][8] += 1;   /* attempts */
#endif
        if (ok) break;
        __syncthreads();                   /* every thread has read ncand */
        if (threadIdx.x == 0) {
            sh.ncand = 0;
            sh.delta = sh.delta * 0.25;
            if (!(sh.delta > sh.sc.interval * 1e-9)) sh.delta = sh.sc.interval * 1e-9;
        }
        __syncthreads();
    }
    if (!ok || nc < 1) {
        if (threadIdx.x == 0) { sh.sort_key[0] = kroot; sh.sort_idx[0] = root; }
        return 1;
    }
#ifdef DMD_PHASE_TIMERS
    if (threadIdx.x == 0 && blockIdx.x < 500) { g_phase_cycles[512 + blockIdx.x][9] += nc; g_phase_cycles[512 + blockIdx.x][10] += 1; }
#endif
    if (warp == 0) {
        /* rank sort: each candidate counts the candidates before it */
        long long kk[2];
        int ee[2], rk[2] = {0, 0};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = lane + 32 * h;
            kk[h] = c < nc ? sh.cand_key[c] : DMD_KEY_INF;
            ee[h] = c < nc ? sh.cand_idx[c] : INT_MAX;
        }
#pragma unroll 8
        for (int u = 0; u < nc; ++u) {
            const long long ku = sh.cand_key[u];
            const int eu = sh.cand_idx[u];
            rk[0] += key_less(ku, eu, kk[0], ee[0]);
            rk[1] += key_less(ku, eu, kk[1], ee[1]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (lane + 32 * h < nc) { sh.sort_key[rk[h]] = kk[h]; sh.sort_idx[rk[h]] = ee[h]; }
    } else if (threadIdx.x == 32) {
        /* the window for the next batch (beside the sort): aim at one to
         * two candidates per slot */
        if (nc < slots) sh.delta = sh.delta * 2.0;
        else if (nc > 2 * slots) sh.delta = sh.delta * 0.5;
        if (!(sh.delta > sh.sc.interval * 1e-9)) sh.delta = sh.sc.interval * 1e-9;
    }
    DMD_GSUB(3);
    return nc;
}

/* ------------------------------------------------------------------ */
/* hot per-bead arrays of a small system in shared memory (k_run)      */
/* ------------------------------------------------------------------ */
struct HotArrays {
    double *x, *y, *z, *vx, *vy, *vz, *tim;
    long long *key, *l1k;
    int *nptnr, *l1i;
    int8_t *colt;
    uint8_t *queued;
};
/* bytes of the hot arrays of a system of N beads and nl1 level-1 groups */
__host__ __device__ constexpr size_t hot_bytes(int N, int nl1) {
    const size_t n = (size_t)N, n3 = n + 3, g = (size_t)nl1;
    return ((48 * n + 16 * n3 + 8 * g + 4 * n3 + 4 * g + 2 * n3) + 15) & ~(size_t)15;
}
/* where they start: after the event areas and task pool (base bytes) and
 * the claim tables of own_cap beads, on a 16-byte boundary */
__host__ __device__ constexpr size_t hot_offset(size_t base, int own_cap) {
    return (base + (size_t)own_cap * 3 * sizeof(unsigned) + 15) & ~(size_t)15;
}
__device__ __forceinline__ HotArrays hot_layout(char *p, int N, int nl1) {
    HotArrays H;
    const size_t n = (size_t)N, n3 = n + 3;
    H.x = (double *)p; H.y = H.x + n; H.z = H.y + n; H.vx = H.z + n; H.vy = H.vx + n; H.vz = H.vy + n;
    H.tim = H.vz + n;
    H.key = (long long *)(H.tim + n3);
    H.l1k = H.key + n3;
    H.nptnr = (int *)(H.l1k + nl1);
    H.l1i = H.nptnr + n3;
    H.colt = (int8_t *)(H.l1i + nl1);
    H.queued = (uint8_t *)(H.colt + n3);
    return H;
}
/* the CTA copies the system's arrays G into H (in) or H back into G */
__device__ void hot_copy(const HotArrays &H, const DSys &G, bool in) {
    const int n = G.N, n3 = n + 3, nl1 = G.nl1;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (in) {
            H.x[k] = G.x[k]; H.y[k] = G.y[k]; H.z[k] = G.z[k]; H.vx[k] = G.vx[k]; H.vy[k] = G.vy[k]; H.vz[k] = G.vz[k];
        } else {
            G.x[k] = H.x[k]; G.y[k] = H.y[k]; G.z[k] = H.z[k]; G.vx[k] = H.vx[k]; G.vy[k] = H.vy[k]; G.vz[k] = H.vz[k];
        }
    }
    for (int k = threadIdx.x; k < n3; k += blockDim.x) {
        if (in) { H.tim[k] = G.tim[k]; H.key[k] = G.key[k]; H.nptnr[k] = G.nptnr[k]; H.colt[k] = G.colt[k]; H.queued[k] = G.queued[k]; }
        else { G.tim[k] = H.tim[k]; G.key[k] = H.key[k]; G.nptnr[k] = H.nptnr[k]; G.colt[k] = H.colt[k]; G.queued[k] = H.queued[k]; }
    }
    for (int k = threadIdx.x; k < nl1; k += blockDim.x) {
        if (in) { H.l1k[k] = G.l1k[k]; H.l1i[k] = G.l1i[k]; }
        else { G.l1k[k] = H.l1k[k]; G.l1i[k] = H.l1i[k]; }
    }
}

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */
__device__ void log_event(const DSys &S, long long slot, long long coll, double t, double tfalse, int i, int j,
                          int type, int evcode) {
    if (!S.log || S.log_cap <= 0) return;
    dmd_event *L = (dmd_event *)S.log + (slot % S.log_cap);
    L->coll = coll; L->t = t; L->tfalse = tfalse;
    L->i = i + 1; L->j = j + 1; L->type = type; L->evcode = evcode;
}

/* shared memory of k_init beyond its static part: the list build's staging */
#define KINIT_DYN_SMEM (96 * 1024)
__global__ void __launch_bounds__(NTHREADS, 1) k_init(DSys *systems, int nsys, int hbonds_mask) {
    extern __shared__ __align__(16) unsigned char kinit_dyn[];
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    int r = blockIdx.x;
    if (r >= nsys) return;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    const DSys &S = S_sh;
    int hbonds = hbonds_mask & 1;
    if (threadIdx.x == 0) { sh.sc = *S.sc; }
    __syncthreads();
    __shared__ FullScratch fs[NWARPS];
    cta_rebuild(S, sh, ScratchRef{(char *)fs, sizeof(FullScratch)}, hbonds, (char *)kinit_dyn, KINIT_DYN_SMEM);
    /* the start-up overlap check of code/main.F90:347 (an error unless the
     * caller accepts overlapping states, as the reference does).  The
     * reference checks before it predicts, so an overlap is reported in
     * place of what the prediction of an overlapping pair raised; with
     * lists over capacity the check cannot run. */
    if (!(S.flags & DMD_FLAG_ALLOW_OVERLAP) && sh.sc.err != DMD_E_CAPACITY) {
        const int saved = sh.sc.err, saved_info = sh.sc.err_info;
        __syncthreads();
        if (threadIdx.x == 0) sh.sc.err = 0;
        __syncthreads();
        if (cta_checkover(S, sh) == 0 && threadIdx.x == 0) { sh.sc.err = saved; sh.sc.err_info = saved_info; }
    }
    __syncthreads();
    if (threadIdx.x == 0) *S.sc = sh.sc;
}

/* k_run and its per-event functions, compiled in two variants that differ
 * only in the size of the per-warp event areas in shared memory.  The full
 * variant takes any list (down lists up to the capacity of 128); the
 * compact one takes systems whose down lists hold at most 32 beads, and
 * its smaller shared-memory footprint leaves about 150 KB of the SM's
 * 256 KB to the L1 cache, which then holds a small system's bead state.
 * A compact launch hands a system whose lists outgrow it back to the host
 * (need_full) at the end of the rebuild that made them, and the host runs
 * the rest of that system's events on the full variant. */
#define DMD_RUN_OPS 264          /* 2 * list capacity (128) + 6 extras + slack */
#define DMD_RUN_RSET 384
#define DMD_RUN_QSET 160
#define DMD_RUN_DN_LIMIT INT_MAX
#define DMD_RUN_NT RUN_NT_FULL
namespace run_full {
#include "engine_run.cuh"
}
#undef DMD_RUN_OPS
#undef DMD_RUN_RSET
#undef DMD_RUN_QSET
#undef DMD_RUN_DN_LIMIT
#undef DMD_RUN_NT
#define DMD_RUN_OPS 72           /* 2 * 32 + 6 extras + slack */
#define DMD_RUN_RSET 192
#define DMD_RUN_QSET 96
#define DMD_RUN_DN_LIMIT DMD_COMPACT_DN
#define DMD_RUN_NT RUN_NT_COMPACT
namespace run_compact {
#include "engine_run.cuh"
}
#undef DMD_RUN_OPS
#undef DMD_RUN_RSET
#undef DMD_RUN_QSET
#undef DMD_RUN_DN_LIMIT
#undef DMD_RUN_NT

/* ------------------------------------------------------------------ */
/* backbone dihedral histogram: code/phipsi.f:25-290 (-Dwrite_phipsi)  */
/* ------------------------------------------------------------------ */
/* The angle of (0, y, z) from the frame's second axis as a whole-degree bin
 * 0..360 (phipsi.f:150-168, 268-285); -1 for a degenerate frame (NaN). */
__device__ int phipsi_bin(double ynew, double znew) {
    const double pi = 3.141592653589793;   /* 4 atan(1) of main.F90:125, rounded to nearest */
    const double d = sqrt(ynew * ynew + znew * znew);
    const double yy = ynew / d, zz = znew / d;
    double c = yy;
    if (c > 1.0) c = 1.0;
    if (c < -1.0) c = -1.0;
    const double angle = acos(c);
    double degs = 180.0 * angle / pi;
    if (zz > 0.0) degs = degs * -1.0;
    if (degs < -180.0) degs = -180.0;
    if (degs > 180.0) degs = 180.0;
    degs = degs + 180.0;
    return degs >= 0.0 && degs <= 360.0 ? (int)trunc(degs) : -1;
}
/* one dihedral in phipsi.f's construction: unit axis a -> b, the
 * perpendicular from the axis to c as the second axis, their cross product
 * as the third, and the fourth point e in that frame (phipsi.f:58-168 for
 * phi with a = N(i), b = Ca(i), c = C(i), e = C(i-1); :170-285 for psi with
 * a = C(i), b = Ca(i), c = N(i), e = N(i+1)) */
__device__ int phipsi_dihedral(const double *a, const double *b, const double *c, const double *e) {
    double x1 = b[0] - a[0], y1 = b[1] - a[1], z1 = b[2] - a[2];
    x1 = x1 - d_nint(x1); y1 = y1 - d_nint(y1); z1 = z1 - d_nint(z1);
    const double d1 = sqrt(x1 * x1 + y1 * y1 + z1 * z1);
    x1 = x1 / d1; y1 = y1 / d1; z1 = z1 / d1;
    double xu = c[0] - b[0], yu = c[1] - b[1], zu = c[2] - b[2];
    xu = xu - d_nint(xu); yu = yu - d_nint(yu); zu = zu - d_nint(zu);
    const double du = sqrt(xu * xu + yu * yu + zu * zu);
    xu = xu / du; yu = yu / du; zu = zu / du;
    double cs = x1 * xu + y1 * yu + z1 * zu;
    if (cs > 1.0) cs = 1.0;
    if (cs < -1.0) cs = -1.0;
    const double dq = cs * du;
    const double dcq = sqrt(du * du - dq * dq);
    const double xr = c[0] - x1 * (d1 + dq), yr = c[1] - y1 * (d1 + dq), zr = c[2] - z1 * (d1 + dq);
    double x2 = xr - a[0], y2 = yr - a[1], z2 = zr - a[2];
    x2 = x2 - d_nint(x2); y2 = y2 - d_nint(y2); z2 = z2 - d_nint(z2);
    x2 = x2 / dcq; y2 = y2 / dcq; z2 = z2 / dcq;
    const double x3 = y1 * z2 - z1 * y2, y3 = z1 * x2 - x1 * z2, z3 = x1 * y2 - y1 * x2;
    double xd = e[0] - a[0], yd = e[1] - a[1], zd = e[2] - a[2];
    xd = xd - d_nint(xd); yd = yd - d_nint(yd); zd = zd - d_nint(zd);
    return phipsi_bin(x2 * xd + y2 * yd + z2 * zd, x3 * xd + y3 * yd + z3 * zd);
}
/* one CTA per system (only: that system alone, or -1): residues 2..L-1 of
 * every chain at the current positions (advanced by tfalse) into the
 * system's 361 x 361 histogram hist + r * 361 * 361 */
__global__ void __launch_bounds__(NTHREADS) k_phipsi(DSys *systems, int nsys, int only, const int *chain_start,
                                                     const int *chain_len, const int *chain_off,
                                                     unsigned long long *hist) {
    const int r = blockIdx.x;
    if (r >= nsys || (only >= 0 && r != only)) return;
    const DSys &S = systems[r];
    const double tf = S.sc->tfalse;
    const int *cs = chain_start + chain_off[r], *cl = chain_len + chain_off[r];
    unsigned long long *h = hist + (size_t)r * 361 * 361;
    for (int c = 0; c < S.nchains; ++c) {
        const int L = cl[c], s0 = cs[c];
        for (int ir = 2 + (int)threadIdx.x; ir <= L - 1; ir += blockDim.x) {
            const int ca = s0 + ir - 1, nh = s0 + L + ir - 1, co = s0 + 2 * L + ir - 1;   /* 0-based */
            double p[5][3];
            const int bead[5] = {nh, ca, co, nh + 1, co - 1};
            for (int k = 0; k < 5; ++k) {
                const int b = bead[k];
                p[k][0] = S.x[b] + S.vx[b] * tf; p[k][1] = S.y[b] + S.vy[b] * tf; p[k][2] = S.z[b] + S.vz[b] * tf;
            }
            const int bphi = phipsi_dihedral(p[0], p[1], p[2], p[4]);
            const int bpsi = phipsi_dihedral(p[2], p[1], p[0], p[3]);
            if (bphi >= 0 && bpsi >= 0) atomicAdd(&h[(size_t)bphi * 361 + bpsi], 1ull);
        }
    }
}

__global__ void __launch_bounds__(NTHREADS) k_diag(DSys *systems, int nsys, const int *chain_start, const int *chain_len,
                                                   const int *chain_off, dmd_diag *out) {
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    int r = blockIdx.x;
    if (r >= nsys) return;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    const DSys &S = S_sh;
    if (threadIdx.x == 0) sh.sc = *S.sc;
    __syncthreads();
    cta_diag(S, sh, chain_start + chain_off[r], chain_len + chain_off[r], out + r);
}

/* ------------------------------------------------------------------ */
/* launch wrappers                                                     */
/* ------------------------------------------------------------------ */
/* dynamic shared memory of k_run: the per-warp event areas, the task pool
 * and, for systems of at most own_cap beads, the claim tables */
template <typename WA> constexpr size_t run_smem_of(int own_cap, int nwarps) {
    return sizeof(WA) * nwarps + sizeof(TaskPool) + (size_t)own_cap * 3 * sizeof(unsigned);
}
static_assert(run_smem_of<run_full::WarpArea>(OWN_SMEM_FULL, RUN_NT_FULL / 32) + sizeof(SharedState) + sizeof(DSys) <=
                  227 * 1024,
              "k_run shared memory above the 227 KB a block may use");
static_assert(run_smem_of<run_compact::WarpArea>(OWN_SMEM_COMPACT, RUN_NT_COMPACT / 32) + sizeof(SharedState) +
                      sizeof(DSys) + 1024 <= RUN_CARVEOUT_COMPACT_KB * 1024,
              "compact k_run (with the 1 KB the system reserves per block) must fit its shared-memory carve-out");
/* the compact variant's shared-memory room for the hot arrays of small
 * single-CTA systems (hot_bytes: 70 B per bead, so up to ~930 beads) */
#define HOT_SMEM_COMPACT (64 * 1024)
constexpr size_t run_compact_base = sizeof(run_compact::WarpArea) * (RUN_NT_COMPACT / 32) + sizeof(TaskPool);
static_assert(hot_offset(run_compact_base, OWN_SMEM_COMPACT) + HOT_SMEM_COMPACT + sizeof(SharedState) +
                      sizeof(DSys) <= 227 * 1024,
              "compact k_run with its hot arrays above the 227 KB a block may use");
static size_t run_smem(int compact, int own_cap, int hot_cap = 0) {
    if (compact && hot_cap > 0) return hot_offset(run_compact_base, own_cap) + (size_t)hot_cap;
    return compact ? run_smem_of<run_compact::WarpArea>(own_cap, RUN_NT_COMPACT / 32)
                   : run_smem_of<run_full::WarpArea>(own_cap, RUN_NT_FULL / 32);
}
static int own_smem_max(int compact) { return compact ? OWN_SMEM_COMPACT : OWN_SMEM_FULL; }

cudaError_t dmd_launch_init(DSys *d_systems, int nsys, int hbonds, cudaStream_t st) {
    static std::mutex mu;
    static bool done[256];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (dev >= 0 && dev < 256 && !done[dev]) {
            e = cudaFuncSetAttribute(k_init, cudaFuncAttributeMaxDynamicSharedMemorySize, KINIT_DYN_SMEM);
            if (e != cudaSuccess) return e;
            done[dev] = true;
        }
    }
    k_init<<<nsys, NTHREADS, KINIT_DYN_SMEM, st>>>(d_systems, nsys, hbonds);
    return cudaGetLastError();
}
static cudaError_t k_run_attributes() {
    static std::mutex mu;
    static bool done[256];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 256 && !done[dev]) {
        /* the shared-memory carve-out is the smallest that holds a launch's
         * blocks; the rest of the SM's 256 KB is L1 cache */
        e = cudaFuncSetAttribute(run_full::k_run, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)run_smem(0, OWN_SMEM_FULL));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(run_compact::k_run, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)run_smem(1, OWN_SMEM_COMPACT, HOT_SMEM_COMPACT));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(run_full::k_run, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxL1);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(run_compact::k_run, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxL1);
        if (e != cudaSuccess) return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

static void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr, int nsys, int C, size_t smem,
                           cudaStream_t st, int nthreads) {
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3((unsigned)(nsys * C), 1, 1);
    cfg.blockDim = dim3((unsigned)nthreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
}

/* k_run with one cluster of C CTAs per system (C = 1, 2, 4 or 8) */
cudaError_t dmd_launch_run(DSys *d_systems, int nsys, int max_beads, int C, int compact, long long target,
                           long long *targets, int hbonds, const int *chain_start, const int *chain_len,
                           const int *chain_off, dmd_diag *outputs, cudaStream_t st, int cycles, int min_beads) {
    if (C != 1 && C != 2 && C != 4 && C != 8) return cudaErrorInvalidValue;
    cudaError_t e = k_run_attributes();
    if (e != cudaSuccess) return e;
    /* claim tables in shared memory for the systems up to own_cap beads */
    int own_cap = C == 1 ? std::min(max_beads, own_smem_max(compact)) : 0;
    /* room for the hot arrays of small systems (compact, one CTA each),
     * when the smallest system fits it: the room comes out of L1 */
    const int hot_cap = (compact && C == 1 && min_beads > 0 &&
                         hot_bytes(min_beads, (min_beads + 3 + 31) / 32) <= (size_t)HOT_SMEM_COMPACT)
                            ? HOT_SMEM_COMPACT : 0;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config(cfg, attr, nsys, C, run_smem(compact, own_cap, hot_cap), st, compact ? RUN_NT_COMPACT : RUN_NT_FULL);
    if (compact)
        return cudaLaunchKernelEx(&cfg, run_compact::k_run, d_systems, nsys, target, targets, hbonds, chain_start,
                                  chain_len, chain_off, outputs, own_cap, C, std::min(compact, (int)DMD_COMPACT_DN), cycles,
                                  hot_cap);
    return cudaLaunchKernelEx(&cfg, run_full::k_run, d_systems, nsys, target, targets, hbonds, chain_start, chain_len,
                              chain_off, outputs, own_cap, C, INT_MAX, cycles, 0);
}

/* how many clusters of C CTAs of k_run can be resident at once */
cudaError_t dmd_max_active_clusters(int C, int *n) {
    cudaError_t e = k_run_attributes();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config(cfg, attr, 1, C, run_smem(0, C == 1 ? OWN_SMEM_FULL : 0), 0, RUN_NT_FULL);
    return cudaOccupancyMaxActiveClusters(n, run_full::k_run, &cfg);
}
cudaError_t dmd_launch_diag(DSys *d_systems, int nsys, const int *chain_start, const int *chain_len,
                            const int *chain_off, dmd_diag *out, cudaStream_t st) {
    k_diag<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, chain_start, chain_len, chain_off, out);
    return cudaGetLastError();
}

cudaError_t dmd_launch_phipsi(DSys *d_systems, int nsys, int only, const int *chain_start, const int *chain_len,
                              const int *chain_off, unsigned long long *hist, cudaStream_t st) {
    k_phipsi<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, only, chain_start, chain_len, chain_off, hist);
    return cudaGetLastError();
}

/* the first out-of-range index of a checked build (-DDMD_BOUNDS), then
 * cleared: 1 and *rec set (site << 40 | extent << 20 | index) if one was
 * recorded, 0 if none, -1 in a build without the checks */
extern "C" int dmd_debug_bounds(long long *rec) {
#ifdef DMD_BOUNDS
    unsigned long long v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_dmd_bounds, sizeof v) != cudaSuccess) return -2;
    if (cudaMemcpyToSymbol(g_dmd_bounds, &zero, sizeof zero) != cudaSuccess) return -2;
    if (rec) *rec = (long long)v;
    return v ? 1 : 0;
#else
    if (rec) *rec = 0;
    return -1;
#endif
}

/* ------------------------------------------------------------------ */
/* allocation-free prediction pass                                     */
/* ------------------------------------------------------------------ */
/* Device memory of dmd_predict_all_noalloc: one file-scope array that every
 * GPU loading this library holds until the process exits.  It carries a
 * whole system (tables, bead state, neighbour lists, cell grid) for at most
 * DMD_NOALLOC_MAX_BEADS beads with lists of DMD_NOALLOC_MAX_CAP entries.
 * Every call reuses it and overwrites what the previous call left; calls
 * whose work overlaps on the GPU (several streams, or several host threads)
 * race on it. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[DMD_NOALLOC_SCRATCH_BYTES];

__global__ void __launch_bounds__(NTHREADS, 1) k_predict_noalloc(DSys S_in, int hbonds, double *tim_out,
                                                              int *nptnr_out, int *colt_out) {
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    __shared__ FullScratch fs[NWARPS];
    if (threadIdx.x == 0) { S_sh = S_in; sh.sc = *S_in.sc; }
    __syncthreads();
    const DSys &S = S_sh;
    cta_rebuild(S, sh, ScratchRef{(char *)fs, sizeof(FullScratch)}, hbonds, nullptr, 0);
    for (int b = threadIdx.x; b < S.N; b += blockDim.x) {
        tim_out[b] = S.tim[b];
        int p = S.nptnr[b];
        nptnr_out[b] = p >= 0 ? p + 1 : p;
        colt_out[b] = S.colt[b];
    }
    __syncthreads();
    if (threadIdx.x == 0) *S.sc = sh.sc;
}

/* Address of the scratch array on the current device, looked up once per
 * device (with that device current) and cached. */
cudaError_t dmd_noalloc_scratch(void **ptr) {
    static void *cached[256];
    static bool have[256];
    static std::mutex mu;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!have[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        cached[dev] = p;
        have[dev] = true;
    }
    *ptr = cached[dev];
    return cudaSuccess;
}

cudaError_t dmd_launch_predict_noalloc(const DSys &S, int hbonds, double *tim_out, int *nptnr_out, int *colt_out,
                                       cudaStream_t st) {
    k_predict_noalloc<<<1, NTHREADS, 0, st>>>(S, hbonds, tim_out, nptnr_out, colt_out);
    return cudaGetLastError();
}
