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
#include <mutex>

#include "dmd.h"
#include "engine.cuh"
#include "engine_api.h"

#define NTHREADS 256
#define NWARPS (NTHREADS / 32)
#define OPS_MAX 264        /* 2 * list capacity (128) + 6 extras + slack */
#define CAND_MAX 64
#define META_MAX 16
#define TG_MAX 64         /* full re-predictions per round (i, j, marked beads) */
#define TMAP_MAX 256
#define CASC_MAX 64
#define RSET_MAX 384
#define WSET_MAX 16
#define QSET_MAX 160
#define OWN_SMEM_MAX 5632    /* systems up to this size keep the claim tables in shared memory */
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
/* sub-phases of one event's processing, on warp 0 of the first CTA only
 * (row DMD_PHASE_CTAS - 1) */
__device__ long long g_sub_last;
#define DMD_SUB(k)                                                                         \
    do {                                                                                   \
        if (blockIdx.x == 0 && threadIdx.x == 0) {                                         \
            long long now_ = clock64();                                                    \
            if ((k) >= 0) g_phase_cycles[DMD_PHASE_CTAS - 1][(k)] += now_ - g_sub_last;    \
            g_sub_last = now_;                                                             \
        }                                                                                  \
    } while (0)
extern "C" int dmd_debug_phase_cycles(long long *out, int nctas) {
    if (nctas > DMD_PHASE_CTAS) nctas = DMD_PHASE_CTAS;
    return (int)cudaMemcpyFromSymbol(out, g_phase_cycles, sizeof(long long) * DMD_PHASE_SLOTS * nctas);
}
#else
#define DMD_PHASE_START(row) do { (void)(row); } while (0)
#define DMD_PHASE(k) do { (void)(k); } while (0)
#define DMD_SUB(k) do { } while (0)
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
    int n;
    int a[PTASK_MAX], b[PTASK_MAX];
    int8_t st[PTASK_MAX], flag[PTASK_MAX];
    double t[PTASK_MAX];
    int8_t ty[PTASK_MAX], ok[PTASK_MAX];
};

/* per-warp working area of one event (dynamic shared memory) */
struct WarpArea {
    int nops, nlead, npred, nmeta, ncasc, ntg, nmarked, ntask;
    int pooled, pool_base;        /* this event's tasks in the CTA's TaskPool, from pool_base */
    /* down-list operations (bead, source) in the reference's order, and
     * the prediction of each operation's pair (time + tfalse, type) */
    int ops_l[OPS_MAX], ops_s[OPS_MAX];
    int8_t ops_c[OPS_MAX];        /* static code of the pair, -1 if not listed */
    double op_t[OPS_MAX];
    int8_t op_y[OPS_MAX];
    /* distinct operation beads: bead, first operation, full-redo mark */
    int lead_l[OPS_MAX];
    int16_t lead_q[OPS_MAX];
    int8_t lead_m[OPS_MAX];
    int16_t mk[OPS_MAX];          /* marked leaders, in leader order */
    FullScratch fs;               /* full re-predictions of one round */
    /* buffered predictions: bead, time, partner, type, queued */
    int pb[OPS_MAX + 2];
    double pt[OPS_MAX + 2];
    int pn[OPS_MAX + 2];
    int8_t pc[OPS_MAX + 2];
    uint8_t pq[OPS_MAX + 2];
    /* snapshot of what the collision may write */
    int mb[META_MAX];
    int8_t mident[META_MAX];
    int mbp[META_MAX];
    int mer[META_MAX][4];
    int movp[META_MAX][4];
    int8_t movc[META_MAX][4];
    double sij[12];
    int8_t colt_i;
    int casc[CASC_MAX];
    int cbase[CASC_MAX + 1];      /* offsets of the cascade beads' claim entries */
    int rset[RSET_MAX];            /* beads of the footprint claim: read, written, queue */
    int wset[WSET_MAX];
    int qset[QSET_MAX];
    int nrset, nwset, nqset;
    /* the event */
    int i, j, ct, evcode, xpulse, conflict, casc_over;
    int err, err_info;
    long long coll;
    double tf;
    long long tnew_key;
    int tnew_idx;
};

struct SharedState {
    DScal sc;
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
    double red_d[NWARPS];
    int red_i[NWARPS * 4];
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
#pragma unroll
    for (int q = 0; q < 32; ++q) k[q] = q < n ? S.key[lo + q] : DMD_KEY_INF;
    int best = 0;
    long long bk = k[0];
#pragma unroll
    for (int q = 1; q < 32; ++q)
        if (k[q] < bk) { bk = k[q]; best = q; }
    S.l1i[g] = lo + best;
    S.l1k[g] = bk;
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
__device__ int warp_tree_root(const DSys &S, long long &kroot) {
    int lane = threadIdx.x & 31;
    long long bk = DMD_KEY_INF;
    int best = INT_MAX;
    for (int h = lane; h < S.nl2; h += 32) {
        int e = S.l2i[h];
        long long k = S.l2k[h];
        if (key_less(k, e, bk, best)) { bk = k; best = e; }
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
/* warp-collective pair geometry: components on lanes 0..2             */
/* ------------------------------------------------------------------ */
struct WRel { double rx, ry, rz, bij, rijsq, vijsq; };

/* relative position at tfalse with the minimum image, and the products of
 * code/core.f:14-26 (sums kept in the reference's left-to-right order) */
__device__ WRel warp_rel(const DSys &S, int i, int j, double tf) {
    int lane = threadIdx.x & 31;
    int d = lane % 3;
    const double *P = d == 0 ? S.x : (d == 1 ? S.y : S.z);
    const double *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
    double v = V[i] - V[j];
    double r = P[i] - P[j] + v * tf;
    r = d_wrap(r);
    double pb = r * v, pr = r * r, pv = v * v;
    WRel w;
    w.rx = __shfl_sync(FULL, r, 0); w.ry = __shfl_sync(FULL, r, 1); w.rz = __shfl_sync(FULL, r, 2);
    double b0 = __shfl_sync(FULL, pb, 0), b1 = __shfl_sync(FULL, pb, 1), b2 = __shfl_sync(FULL, pb, 2);
    double r0 = __shfl_sync(FULL, pr, 0), r1 = __shfl_sync(FULL, pr, 1), r2 = __shfl_sync(FULL, pr, 2);
    double v0 = __shfl_sync(FULL, pv, 0), v1 = __shfl_sync(FULL, pv, 1), v2 = __shfl_sync(FULL, pv, 2);
    /* three independent sums on three lanes, then broadcast */
    double s = lane == 0 ? b0 + b1 + b2 : (lane == 1 ? r0 + r1 + r2 : v0 + v1 + v2);
    w.bij = __shfl_sync(FULL, s, 0);
    w.rijsq = __shfl_sync(FULL, s, 1);
    w.vijsq = __shfl_sync(FULL, s, 2);
    return w;
}

/* four distances at tfalse (code/repuls_check.f), pair q on lanes 3q..3q+2 */
__device__ void warp_dist4(const DSys &S, const int *a, const int *b, double tf, double *dout) {
    int lane = threadIdx.x & 31;
    int q = lane / 3 < 4 ? lane / 3 : 3, d = lane % 3;
    int ia = a[q], ib = b[q];
    const double *P = d == 0 ? S.x : (d == 1 ? S.y : S.z);
    const double *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
    double v = V[ia] - V[ib];
    double r = P[ia] - P[ib] + v * tf;
    r = d_wrap(r);
    double p = r * r;
    double c0 = __shfl_sync(FULL, p, 3 * (lane & 3));
    double c1 = __shfl_sync(FULL, p, 3 * (lane & 3) + 1);
    double c2 = __shfl_sync(FULL, p, 3 * (lane & 3) + 2);
    double dd = c0 + c1 + c2;
    double dist = sqrt(dd);
    for (int k = 0; k < 4; ++k) dout[k] = __shfl_sync(FULL, dist, k);
}

/* the per-component tail of code/eventdyn.f:357-381 after the bumpdist push:
 * lanes 0..5 = (bead i/j) x (x,y,z) */
__device__ void warp_impulse(const DSys &S, int i, int j, const WRel &w, double ratio, double bd, int bump,
                             double tf) {
    int lane = threadIdx.x & 31;
    if (lane < 6) {
        int d = lane % 3;
        bool isj = lane >= 3;
        int b = isj ? j : i;
        double *P = d == 0 ? S.x : (d == 1 ? S.y : S.z);
        double *V = d == 0 ? S.vx : (d == 1 ? S.vy : S.vz);
        double r = d == 0 ? w.rx : (d == 1 ? w.ry : w.rz);
        double p = P[b];
        /* bump = -1: pair pushed together (i - bd*r, j + bd*r); +1: apart; 0: none */
        if (bump != 0) {
            bool minus = (bump < 0) != isj;
            p = minus ? p - bd * r : p + bd * r;
        }
        double bmb = S.bm[b], rbmb = S.tab->rbm[S.ident[b]];   /* bm(b) = mass(identity(b)) */
        double delv = ratio * r;
        double dv = div_by(delv, bmb, rbmb);
        double dp = div_by(delv * tf, bmb, rbmb);
        V[b] = isj ? V[b] + dv : V[b] - dv;
        p = isj ? p - dp : p + dp;
        P[b] = p;
    }
    __syncwarp();
}
__device__ void warp_bump_only(const DSys &S, int i, int j, const WRel &w, double bd, int bump) {
    int lane = threadIdx.x & 31;
    if (lane < 6) {
        int d = lane % 3;
        bool isj = lane >= 3;
        int b = isj ? j : i;
        double *P = d == 0 ? S.x : (d == 1 ? S.y : S.z);
        double r = d == 0 ? w.rx : (d == 1 ? w.ry : w.rz);
        bool minus = (bump < 0) != isj;
        double p = P[b];
        P[b] = minus ? p - bd * r : p + bd * r;
    }
    __syncwarp();
}

/* code/eventdyn.f:4-385: ratio on lane 0, the six component updates on lanes 0..5 */
__device__ int warp_eventdyn(const DSys &S, int i, int j, int evcode, int ct, double tf) {
    int lane = threadIdx.x & 31;
    const DTab &T = *S.tab;
    WRel w = warp_rel(S, i, j, tf);
    DMD_SUB(12);
    double ratio = 0.0, bd = 0.0;
    int bump = 0;
    if (lane == 0) {
        double bij = w.bij;
        int a = S.ident[i], b = S.ident[j];
        /* the masses, squared diameters and bond windows come from tables
         * computed in the same operation order (bm(i) = mass(identity(i))) */
        double rmass = T.rmass[a][b];
        bool side = evcode >= 10 && evcode <= 12;
        if (ct == 2) {
            double lo = side ? S.blmin_sq[i] : T.evp2_sq[evcode];
            double rlo = side ? S.rblmin_sq[i] : T.revp2_sq[evcode];
            ratio = div_by(rmass * bij, lo, rlo);
        } else if (ct == 3) {
            double hi = side ? S.blmax_sq[i] : T.evp3_sq[evcode];
            double rhi = side ? S.rblmax_sq[i] : T.revp3_sq[evcode];
            ratio = div_by(rmass * bij, hi, rhi);
        } else if (ct == 1) {
            double sigsq;
            if (evcode == 15) sigsq = S.bptnr[i] == j ? T.core15_sq[a][b] : T.sigma_sq[a][b];
            else sigsq = T.core_sq[core_slot(evcode)][a][b];
            ratio = rmass * bij / sigsq;
        } else if (ct == 4) {
            double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij + del_pe > 0.0) {
                ratio = rmass * (sqrt((4.0 * wellsq * epsave / rmass) + bij * bij) + bij) / (2.0 * wellsq);
                ct = 20; bump = -1;
            } else {
                ratio = rmass * bij / wellsq;
                ct = 22; bump = 1;
            }
        } else if (ct == 8) {
            double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij > del_pe) {
                ratio = rmass * (-sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
                ct = 21; bump = 1;
            } else {
                ratio = rmass * bij / wellsq;
                ct = 22; bump = -1;
            }
        } else if (ct == 9) {
            double wellsq = T.welldia_sq[a][b];
            ratio = rmass * bij / wellsq;
            ct = 23; bump = 1; bd = DMD_SMDIST * sqrt(wellsq);
        } else if (ct == 5) {
            double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
            double del_pe = 4.0 * wellsq * epsave / rmass;
            bd = DMD_SMDIST * sqrt(wellsq);
            ratio = rmass * (-sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
            ct = 24; bump = 1;
        } else if (ct == 6) {
            double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
            double del_pe = 4.0 * wellsq * epsave / rmass;
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij > -del_pe) {
                ratio = rmass * (sqrt(del_pe + bij * bij) + bij) / (2.0 * wellsq);
                ct = 25; bump = -1;
            } else {
                ratio = rmass * bij / wellsq;
                ct = 26; bump = 1;
            }
        } else if (ct == 13) {
            double wellsq = T.shlddia_sq[a][b];
            ratio = rmass * bij / wellsq;
            ct = 27; bump = 1; bd = DMD_SMDIST * sqrt(wellsq);
        }
    }
    ratio = __shfl_sync(FULL, ratio, 0);
    bd = __shfl_sync(FULL, bd, 0);
    bump = __shfl_sync(FULL, bump, 0);
    ct = __shfl_sync(FULL, ct, 0);
    DMD_SUB(13);
    warp_impulse(S, i, j, w, ratio, bd, bump, tf);
    DMD_SUB(14);
    return ct;
}
/* code/bumped.f:1-47 */
__device__ void warp_bumpoff(const DSys &S, int i, int j, int evcode, double tf) {
    WRel w = warp_rel(S, i, j, tf);
    const DTab &T = *S.tab;
    int a = S.ident[i], b = S.ident[j];
    double bd = (evcode >= 40) ? DMD_SMDIST * sqrt(T.shlddia_sq[a][b]) : DMD_SMDIST * sqrt(T.welldia_sq[a][b]);
    warp_bump_only(S, i, j, w, bd, w.bij < 0.0 ? -1 : 1);
}
__device__ double warp_check_sigma(const DSys &S, int i, int j, double tf) {  /* code/check_sigma.f */
    WRel w = warp_rel(S, i, j, tf);
    double diff = w.rijsq - S.tab->sigma_sq[S.ident[i]][S.ident[j]];
    return diff < 0.0 ? 10.0 : 11.0;
}

/* ------------------------------------------------------------------ */
/* one event on one warp                                               */
/* ------------------------------------------------------------------ */
/* snapshot of everything the collision of (i, j) may write */
/* The positions, velocities and coltype of i and j, taken before every
 * collision; the H-bond bookkeeping state (identity, partner, extra_repuls,
 * overrides) of the beads it may touch is taken by lane_meta_snapshot()
 * only when the collision is about to write it. */
__device__ void warp_snapshot(const DSys &S, WarpArea &W, int i, int j) {
    int lane = threadIdx.x & 31;
    if (lane == 0) { W.nmeta = 0; W.colt_i = S.colt[i]; }
    if (lane < 12) {
        int b = lane < 6 ? i : j, f = lane % 6;
        const double *A = f == 0 ? S.x : f == 1 ? S.y : f == 2 ? S.z : f == 3 ? S.vx : f == 4 ? S.vy : S.vz;
        W.sij[lane] = A[b];
    }
    __syncwarp();
}
__device__ void warp_restore(const DSys &S, WarpArea &W) {
    int lane = threadIdx.x & 31;
    /* entries naming the same bead hold the same values, so order does not matter */
    for (int q = lane; q < W.nmeta; q += 32) {
        int b = W.mb[q];
        S.ident[b] = W.mident[q];
        S.bptnr[b] = W.mbp[q];
        for (int k = 0; k < 4; ++k) { S.er[4 * b + k] = W.mer[q][k]; S.ovp[4 * b + k] = W.movp[q][k]; S.ovc[4 * b + k] = W.movc[q][k]; }
    }
    if (lane < 12) {
        int b = lane < 6 ? W.i : W.j, f = lane % 6;
        double *A = f == 0 ? S.x : f == 1 ? S.y : f == 2 ? S.z : f == 3 ? S.vx : f == 4 ? S.vy : S.vz;
        A[b] = W.sij[lane];
    }
    if (lane == 0) S.colt[W.i] = W.colt_i;
    __syncwarp();
}

__device__ void lane_meta_snapshot(const DSys &S, WarpArea &W, int i, int j) {
    int n = 0;
    auto add = [&](int b) { if (b >= 0 && n < META_MAX) W.mb[n++] = b; };
    add(i); add(j);
    for (int k = 0; k < 4; ++k) { add(S.er[4 * i + k]); add(S.er[4 * j + k]); }
    int h1, h2;
    own_helpers(S, i, h1, h2); add(h1); add(h2);
    own_helpers(S, j, h1, h2); add(h1); add(h2);
    for (int q = 0; q < n; ++q) {
        int b = W.mb[q];
        W.mident[q] = S.ident[b];
        W.mbp[q] = S.bptnr[b];
        for (int k = 0; k < 4; ++k) { W.mer[q][k] = S.er[4 * b + k]; W.movp[q][k] = S.ovp[4 * b + k]; W.movc[q][k] = S.ovc[4 * b + k]; }
    }
    W.nmeta = n;
}

/* worker block (code/main.F90:1432-1956) and master application
 * (code/main.F90:646-943) of the pair event (i, j), warp-wide */
__device__ void warp_collision(const DSys &S, Err E, WarpArea &W, int i, int j, double tf, long long coll,
                               int hbonds) {
    int lane = threadIdx.x & 31;
    int8_t *id = S.ident;
    int *er = S.er;
    int ct = S.colt[i];
    int evcode = pair_code(S, i, j, hbonds);
    bool nonend = !S.info[i].is_end && !S.info[j].is_end;
    int xpulse = 0;
    int nb = id[i] < id[j] ? i : j;
    int cb = id[i] < id[j] ? j : i;
    int err = 0;
    if (ct == 7) {
        if (er[4 * i + 3] < 0 && er[4 * j + 3] < 0) {
            if (nonend) {
                int ncim1, ncai, ncaj, nnjp1;
                helpers_of(S, nb, cb, ncim1, ncai, ncaj, nnjp1);
                int a[4] = {nb, nb, cb, cb}, b[4] = {ncaj, nnjp1, ncai, ncim1};
                double d[4];
                warp_dist4(S, a, b, tf, d);
                const DTab &T = *S.tab;
                double rating = ((d[0] > T.shd1) && (d[1] > T.shd2) && (d[2] > T.shd3) && (d[3] > T.shd4)) ? 10.0 : 11.0;
                ct = rating <= 10.0 ? 4 : 14;
            } else {
                double ran_non = dmd_uniform(S.seed, DMD_STREAM_CAPTURE, (uint64_t)coll, 0);
                ct = ran_non <= 0.2 ? 4 : 9;
            }
        } else {
            ct = 9;
        }
    } else if (ct == 10 || ct == 12) {
        int hb = evcode < 45 ? er[4 * i + 3] : er[4 * j + 3];
        if (hb < 0) err = 1;
        else if (ct == 10) {
            /* code/repuls_check_3.f with (n, c, k) */
            int x = evcode < 45 ? i : j, k = evcode < 45 ? j : i;
            int n = id[x] < id[hb] ? x : hb, c = id[x] < id[hb] ? hb : x;
            int ncim1, ncai, ncaj, nnjp1;
            helpers_of(S, n, c, ncim1, ncai, ncaj, nnjp1);
            int a[4] = {n, n, c, c}, b[4] = {ncaj, nnjp1, ncai, ncim1};
            double d[4];
            warp_dist4(S, a, b, tf, d);
            const DTab &T = *S.tab;
            int m = 0;
            if ((ncaj != k) && (d[0] > T.shd1)) m = m + 1;
            if ((nnjp1 != k) && (d[1] > T.shd2)) m = m + 1;
            if ((ncai != k) && (d[2] > T.shd3)) m = m + 1;
            if ((ncim1 != k) && (d[3] > T.shd4)) m = m + 1;
            ct = (m == 3 ? 10.0 : 11.0) <= 10.0 ? 5 : 15;
        } else {
            int x = evcode < 45 ? i : j;
            if (S.bptnr[x] == hb) ct = warp_check_sigma(S, x, hb, tf) > 10.0 ? 6 : 13;
            else ct = 15;
        }
    }
    if (err) {
        if (lane == 0) { set_err(E, DMD_E_STATE, i); W.ct = ct; W.evcode = evcode; W.xpulse = 0; }
        __syncwarp();
        return;
    }
    DMD_SUB(15);
    if (ct < 14) ct = warp_eventdyn(S, i, j, evcode, ct, tf);
    if ((ct == 24 || ct == 25) && (evcode < 45 ? er[4 * i + 3] : er[4 * j + 3]) < 0) {
        if (lane == 0) { set_err(E, DMD_E_STATE, i); W.ct = ct; W.evcode = evcode; W.xpulse = 0; }
        __syncwarp();
        return;
    }
    if (ct == 14 || ct == 15 || ct == 16) warp_bumpoff(S, i, j, evcode, tf);
    if (lane == 0) {
        if (ct == 20 || ct == 21 || ct == 24 || ct == 25 || ct == 14 || ct == 16) lane_meta_snapshot(S, W, i, j);
        if (ct == 20) {
            if (id[i] + id[j] == 5) {
                S.bptnr[i] = j; S.bptnr[j] = i;
                id[i] = id[i] + 4; id[j] = id[j] + 4;
                if (nonend) { if (id[i] < id[j]) repuls_add(S, E, i, j, hbonds); else repuls_add(S, E, j, i, hbonds); }
            }
        } else if (ct == 21) {
            if (id[i] <= 8) {
                if (nonend) {
                    xpulse = 1;
                    if (id[i] < id[j]) shoulders_off(S, E, i, j, hbonds); else shoulders_off(S, E, j, i, hbonds);
                }
                if (S.bptnr[i] == j) {
                    S.bptnr[i] = -1; S.bptnr[j] = -1;
                    id[i] = id[i] - 4; id[j] = id[j] - 4;
                }
            }
        } else if (ct == 24) {
            int x = evcode < 45 ? i : j, hb = er[4 * x + 3];
            if (id[x] + id[hb] == 5) { S.bptnr[x] = hb; S.bptnr[hb] = x; id[x] += 4; id[hb] += 4; }
        } else if (ct == 25) {
            int x = evcode < 45 ? i : j, hb = er[4 * x + 3];
            if (id[x] >= 5) { S.bptnr[x] = -1; S.bptnr[hb] = -1; id[x] -= 4; id[hb] -= 4; }
        } else if (ct == 14) {
            if (nonend) { if (id[i] < id[j]) repuls_add(S, E, i, j, hbonds); else repuls_add(S, E, j, i, hbonds); }
        } else if (ct == 16) {
            if (nonend) {
                xpulse = 1;
                if (id[i] < id[j]) shoulders_off(S, E, i, j, hbonds); else shoulders_off(S, E, j, i, hbonds);
            }
        }
        S.colt[i] = (int8_t)ct;
        W.ct = ct; W.evcode = evcode; W.xpulse = xpulse;
    }
    __syncwarp();
}

/* Andersen ghost collision (code/main.F90:997-1121) up to the re-prediction;
 * lane 0, returns the bead and the (possibly clamped) event time */
__device__ int lane_ghost(const DSys &S, SharedState &sh, double &tfalse) {
    const DTab &T = *S.tab;
    long long g = sh.sc.ghost_index++;
    uint32_t k = 0;
    int N = S.N;
    int i;
    do { i = (int)(dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) * N) + 1; } while (i == N + 1 && k < 64);
    if (i > N) i = N;
    i -= 1;
    sh.sc.n_ghost += 1;
    S.x[i] = S.x[i] + S.vx[i] * tfalse; S.y[i] = S.y[i] + S.vy[i] * tfalse; S.z[i] = S.z[i] + S.vz[i] * tfalse;
    double v1, v2, r;
    double bmi = S.bm[i];
    do {
        v1 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        v2 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        r = v1 * v1 + v2 * v2;
    } while (((r == 0.0) || (r >= 1.0)) && k < 4096);
    double fact = sqrt(-2.0 * T.setemp * bmi * dmd_log(r) / r);
    S.vx[i] = v1 * fact / bmi;
    S.vy[i] = v2 * fact / bmi;
    do {
        v1 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        v2 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        r = v1 * v1 + v2 * v2;
    } while (((r == 0.0) || (r >= 1.0)) && k < 8192);
    fact = sqrt(-2.0 * T.setemp * bmi * dmd_log(r) / r);
    S.vz[i] = v1 * fact / bmi;
    S.x[i] = S.x[i] - S.vx[i] * tfalse; S.y[i] = S.y[i] - S.vy[i] * tfalse; S.z[i] = S.z[i] - S.vz[i] * tfalse;
    double tgho = 0.0;
    while (((tgho < 1e-18) || (tgho == 1.0)) && k < 12288) tgho = dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++);
    if (r == 0.0 || r >= 1.0 || tgho < 1e-18) set_err(sh, DMD_E_STATE, -1);
    double tn = -1.0 * dmd_log(tgho) * T.avegtime + tfalse;
    set_pred(S, N, tn, -2, -2, tn < sh.sc.interval_max);
    if (tfalse < sh.sc.old_tfalse) tfalse = sh.sc.old_tfalse;
    return i;
}

/* ------------------------------------------------------------------ */
/* re-prediction into the warp's buffer (code/partial_events.f)         */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ bool check_tij(Err E, double tij, int i) {
    /* reference debug check: negative time beyond 1e-10 (code/eventredo_up.f:58-74) */
    if (tij < 0.0 && fabs(tij) > 1.0e-10) { set_err(E, DMD_E_NEG_TIME, i); return false; }
    return true;
}

/* warp: partial_events(i, j) (code/partial_events.f:5-205; j = -1 after a
 * ghost) into W's buffer.
 *
 * The reference updates beads one operation at a time: the full
 * re-prediction of i and of j (eventredo_up over the up list and the
 * extras), then for every bead l of the down lists and the lower extras of
 * i and then j, either a full re-prediction of l (when l's current partner
 * is the source) or a comparison with the pair (l, source)
 * (eventredo_down).  No prediction depends on another: all read the state
 * after the collision.  So the pairs are predicted as one flat task list,
 * 32 per pass with one call site, and the order-dependent part - which
 * candidate wins, when a full re-prediction is due - is replayed per bead
 * on integer keys.  A bead needs its full re-prediction only if its
 * partner before the event is one of its sources or a source repeats;
 * those beads ("marked") are fully re-predicted up front, in rounds of at
 * most TG_MAX - 2. */
/* Steps of partial_events(i, j) (code/partial_events.f:5-205; j = -1
 * after a ghost), run on one warp into W's buffer.
 *
 * The reference updates beads one operation at a time: the full
 * re-prediction of i and of j (eventredo_up over the up list and the
 * extras), then for every bead l of the down lists and the lower extras of
 * i and then j, either a full re-prediction of l (when l's current partner
 * is the source) or a comparison with the pair (l, source)
 * (eventredo_down).  No prediction depends on another: all read the state
 * after the collision.  So the pairs are predicted as one flat task list
 * (32 per pass, one call site; or pooled with the other events of a batch,
 * see k_run) and the order-dependent part - which candidate wins, when a
 * full re-prediction is due - is replayed per bead on integer keys.  A bead
 * needs its full re-prediction only if its partner before the event is one
 * of its sources or a source repeats; those beads ("marked") are fully
 * re-predicted up front, in rounds of at most TG_MAX - 2. */

/* 1-2: the down-list operations in the reference's order, and the distinct
 * beads among them (leaders) with their first operation and mark */
__device__ void warp_rp_lists(const DSys &S, WarpArea &W, int i, int j) {
    int lane = threadIdx.x & 31;
    /* 1. the down-list operations in the reference's order */
    int n = 0;
    {
        int cnt = S.dnn[i];
        const int *dn = S.dn + (size_t)i * S.cap;
        const int8_t *dc = S.dnc ? S.dnc + (size_t)i * S.cap : nullptr;
        for (int q = lane; q < cnt; q += 32) { W.ops_l[q] = dn[q]; W.ops_s[q] = i; W.ops_c[q] = dc ? dc[q] : (int8_t)-1; }
        n = cnt;
        if (lane == 0)
            for (int k = 0; k < 3; ++k) {
                int l = S.er[4 * i + k];
                if (l >= 0 && l < i) { W.ops_l[n] = l; W.ops_s[n] = i; W.ops_c[n] = -1; ++n; }
            }
        n = __shfl_sync(FULL, n, 0);
        if (j >= 0) {
            int cj = S.dnn[j];
            const int *dj = S.dn + (size_t)j * S.cap;
            const int8_t *dcj = S.dnc ? S.dnc + (size_t)j * S.cap : nullptr;
            for (int base = 0; base < cj; base += 32) {
                int q = base + lane;
                int l = q < cj ? dj[q] : -1;
                bool keep = q < cj && l != i;
                unsigned m = __ballot_sync(FULL, keep);
                int pos = n + __popc(m & ((1u << lane) - 1));
                if (keep) { W.ops_l[pos] = l; W.ops_s[pos] = j; W.ops_c[pos] = dcj ? dcj[q] : (int8_t)-1; }
                n += __popc(m);
            }
            if (lane == 0)
                for (int k = 0; k < 3; ++k) {
                    int l = S.er[4 * j + k];
                    if (l >= 0 && l < j) { W.ops_l[n] = l; W.ops_s[n] = j; W.ops_c[n] = -1; ++n; }
                }
            n = __shfl_sync(FULL, n, 0);
        }
    }
    __syncwarp();
    DMD_SUB(2);
    /* 2. distinct beads (leaders), their first operation and mark */
    int nl = 0, nm = 0;
    if (n <= 32) {
        /* one pass: lanes holding the same bead find each other in one step */
        int q = lane;
        bool in = q < n;
        int l = in ? W.ops_l[q] : -1 - lane;
        int src = in ? W.ops_s[q] : -1;
        unsigned peers = __match_any_sync(FULL, l);
        bool lead = in && (__ffs(peers) - 1) == lane;
        int p0 = (in && l != i) ? S.nptnr[l] : -2;
        unsigned hit = __ballot_sync(FULL, in && src == p0);
        unsigned same = __match_any_sync(FULL, in ? ((long long)l << 32) | (unsigned)src : -1LL - lane);
        unsigned dup = __ballot_sync(FULL, in && __popc(same) > 1);
        bool mark = lead && l != i && ((hit | dup) & peers) != 0;
        unsigned m = __ballot_sync(FULL, lead);
        int pos = __popc(m & ((1u << lane) - 1));
        unsigned mm = __ballot_sync(FULL, mark);
        int mpos = __popc(mm & ((1u << lane) - 1));
        if (lead) { W.lead_l[pos] = l; W.lead_q[pos] = (int16_t)q; W.lead_m[pos] = mark; }
        if (mark) W.mk[mpos] = (int16_t)pos;
        nl = __popc(m);
        nm = __popc(mm);
    }
    for (int base = 0; n > 32 && base < n; base += 32) {
        int q = base + lane;
        bool lead = false, mark = false;
        int l = -1;
        if (q < n) {
            l = W.ops_l[q];
            lead = true;
            for (int p = 0; p < q; ++p) if (W.ops_l[p] == l) { lead = false; break; }
            if (lead && l != i) {
                int p0 = S.nptnr[l];
                int s1 = -1, s2 = -1;   /* sources are i or j: two at most */
                for (int pp = q; pp < n; ++pp) {
                    if (W.ops_l[pp] != l) continue;
                    int src = W.ops_s[pp];
                    if (src == p0 || src == s1 || src == s2) mark = true;
                    if (s1 < 0) s1 = src; else s2 = src;
                }
            }
        }
        unsigned m = __ballot_sync(FULL, lead);
        int pos = nl + __popc(m & ((1u << lane) - 1));
        unsigned mm = __ballot_sync(FULL, lead && mark);
        int mpos = nm + __popc(mm & ((1u << lane) - 1));
        if (lead) { W.lead_l[pos] = l; W.lead_q[pos] = (int16_t)q; W.lead_m[pos] = mark; }
        if (lead && mark) W.mk[mpos] = (int16_t)pos;
        nl += __popc(m);
        nm += __popc(mm);
    }
    if (lane == 0) {
        W.nops = n;
        W.nlead = nl; W.nmarked = nm; W.npred = 2 + nl;
        W.pb[0] = i; W.pb[1] = j;
    }
    __syncwarp();
}

/* 3: the full re-predictions of round rd (i, j in round 0, then marked
 * beads), their running minima and task offsets; W.ntg, W.ntask */
__device__ void warp_rp_targets(const DSys &S, WarpArea &W, int i, int j, int rd, double Hraw, long long Hkey) {
    int lane = threadIdx.x & 31;
    const int per_round = TG_MAX - 2;
    const int nm = W.nmarked;
    /* 3. this round's full re-predictions: i, j (round 0), marked beads */
    int m0 = rd * per_round, m1 = min(nm, m0 + per_round);
    int ntg = 2 + (m1 - m0);
    for (int t = lane; t < ntg; t += 32) {
        int b;
        if (t == 0) b = rd == 0 ? i : -1;
        else if (t == 1) b = rd == 0 ? j : -1;
        else b = W.lead_l[W.mk[m0 + t - 2]];
        W.fs.tg_b[t] = b;
        W.fs.tg_k[t] = Hkey; W.fs.tg_p[t] = -1; W.fs.tg_raw[t] = Hraw; W.fs.tg_y[t] = -1;
    }
    /* task offsets: an inclusive scan over the targets of the up-list
     * length plus the extras above the bead */
    int run = 0;
    for (int base = 0; base < ntg; base += 32) {
        int t = base + lane;
        int b = t < ntg ? W.fs.tg_b[t] : -1;
        int c = 0;
        if (b >= 0) {
            c = S.upn[b];
            for (int k = 0; k < 3; ++k) c += S.er[4 * b + k] > b;
        }
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(FULL, incl, o); if (lane >= o) incl += v; }
        if (t < ntg) W.fs.tg_base[t] = run + incl - c;
        run += __shfl_sync(FULL, incl, 31);
    }
    if (lane == 0) W.fs.tg_base[ntg] = run;
    __syncwarp();
    const bool mapped = run <= TMAP_MAX;
    if (mapped) {   /* task -> target map, one target per lane */
        for (int t = lane; t < ntg; t += 32)
            for (int q = W.fs.tg_base[t]; q < W.fs.tg_base[t + 1]; ++q) W.fs.tmap[q] = (int8_t)t;
        __syncwarp();
    }
    if (lane == 0) { W.ntg = ntg; W.ntask = (rd == 0 ? W.nops : 0) + run; }
    __syncwarp();
}

/* the task q of round rd as (bead, partner, static code or -1, target or
 * -1 for a down operation); pa < 0 when the slot holds no pair */
__device__ __forceinline__ void rp_task(const DSys &S, const WarpArea &W, int q, int nop, int &pa, int &pbb, int &st,
                                        int &tgt) {
    pa = -1; pbb = -1; st = -1; tgt = -1;
    if (q < nop) {
        pa = W.ops_l[q]; pbb = W.ops_s[q];
        st = W.ops_c[q];
        return;
    }
    int rel = q - nop;
    int ntg = W.ntg;
    int run = W.fs.tg_base[ntg];
    int lo;
    if (run <= TMAP_MAX) lo = W.fs.tmap[rel];
    else {
        int hi = ntg - 1;                /* last target with tg_base <= rel */
        lo = 0;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (W.fs.tg_base[mid] <= rel) lo = mid; else hi = mid - 1;
        }
    }
    tgt = lo;
    int b = W.fs.tg_b[lo];
    int k = rel - W.fs.tg_base[lo];
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

/* one prediction task: ev_code(l, source) for a down operation, ev_code(m, b)
 * for a full one; the time is tij + tfalse for a down operation and tij for
 * a full one (tfalse is added after its minimum; x + (-0.0) == x) */
__device__ __forceinline__ bool rp_predict(const DSys &S, Err E, int pa, int pbb, int st, bool is_op, double tf,
                                           int hbonds, double &tt, int &ty) {
    double tij = 0.0;
    ty = 0;
    bool ok = false;
    if (pa >= 0) {
        int a1 = is_op ? pa : pbb, a2 = is_op ? pbb : pa;
        int code = st >= 0 ? pair_code_st(S, a1, a2, st) : pair_code(S, a1, a2, hbonds);
        ok = d_predict_c(S, pa, pbb, code, tf, tij, ty);
        if (!ok) set_err(E, DMD_E_INPUT, pa);
        else if (okey(tij) < okey(-1.0e-10)) set_err(E, DMD_E_NEG_TIME, pa);
    }
    tt = tij + (is_op ? tf : -0.0);
    return ok;
}

/* 1-4 into the CTA's task pool for the event of warp `owner` (its tasks
 * must fit one round and the pool), else W.pooled = 0 and the owner warp
 * runs warp_repredict() after the pool */
__device__ void warp_rp_prepare(const DSys &S, WarpArea &W, TaskPool &TP, int owner, int i, int j, double tf,
                                double imax) {
    int lane = threadIdx.x & 31;
    warp_rp_lists(S, W, i, j);
    bool pooled = W.nmarked <= TG_MAX - 2;
    int base = 0;
    if (pooled) {
        const double Hraw = imax + DMD_LTSTEP - tf;
        warp_rp_targets(S, W, i, j, 0, Hraw, okey(Hraw));
        int nt = W.ntask, nop = W.nops;
        if (lane == 0) base = atomicAdd(&TP.n, nt);
        base = __shfl_sync(FULL, base, 0);
        pooled = base + nt <= PTASK_MAX;
        for (int q = lane; q < nt && base + q < PTASK_MAX; q += 32) {
            int pa = -1, pbb = -1, st = -1, tgt = -1;
            if (pooled) rp_task(S, W, q, nop, pa, pbb, st, tgt);
            TP.a[base + q] = pa; TP.b[base + q] = pbb; TP.st[base + q] = (int8_t)st;
            TP.flag[base + q] = (int8_t)((q < nop ? 1 : 0) | (owner << 1));
        }
    }
    if (lane == 0) { W.pooled = pooled; W.pool_base = base; }
    __syncwarp();
}

/* 4: the tasks of the round on this warp, 32 per pass */
__device__ void warp_rp_tasks(const DSys &S, Err E, WarpArea &W, int rd, double tf, int hbonds) {
    int lane = threadIdx.x & 31;
    const int nop = rd == 0 ? W.nops : 0;
    const int ntask = W.ntask;
    for (int base = 0; base < ntask; base += 32) {
        int q = base + lane;
        int pa = -1, pbb = -1, st = -1, tgt = -1;
        if (q < ntask) rp_task(S, W, q, nop, pa, pbb, st, tgt);
        double tt;
        int ty;
        bool ok = rp_predict(S, E, pa, pbb, st, q < nop, tf, hbonds, tt, ty);
        if (q < nop) { W.op_t[q] = tt; W.op_y[q] = ok ? (int8_t)ty : (int8_t)-128; }
        /* segmented minimum of the full tasks, segment = target */
        long long k = (tgt >= 0 && ok) ? okey(tt) : DMD_KEY_INF;
        int p = (tgt >= 0 && ok) ? pbb : INT_MAX;
        double rt = tt;
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
        if (head && key_less(k, p, W.fs.tg_k[tgt], W.fs.tg_p[tgt])) {
            W.fs.tg_k[tgt] = k; W.fs.tg_p[tgt] = p; W.fs.tg_raw[tgt] = rt; W.fs.tg_y[tgt] = (int8_t)y;
        }
        __syncwarp();
    }
}

/* 5-6: the full results (minimum + tfalse) and the replay of the operations
 * per bead: round 0 replays the unmarked beads and i, each round its marked
 * beads */
__device__ void warp_rp_finish(const DSys &S, Err E, WarpArea &W, int i, int j, int rd, double tf, double imax) {
    int lane = threadIdx.x & 31;
    const int per_round = TG_MAX - 2;
    const int n = W.nops, nl = W.nlead, nm = W.nmarked, ntg = W.ntg;
    const int m0 = rd * per_round, m1 = min(nm, m0 + per_round);
    const long long imax_key = okey(imax);
    /* 5. the full results: time = minimum + tfalse */
    for (int t = lane; t < ntg; t += 32) W.fs.tg_raw[t] = W.fs.tg_raw[t] + tf;
    __syncwarp();
    if (rd == 0 && lane < 2 && (lane == 0 || j >= 0)) {
        double tn = W.fs.tg_raw[lane];
        W.pt[lane] = tn; W.pn[lane] = W.fs.tg_p[lane]; W.pc[lane] = W.fs.tg_y[lane];
        W.pq[lane] = okey(tn) < imax_key;
    }
    __syncwarp();
    /* 6. replay of the operations per bead: round 0 replays the
     * unmarked beads and i, each round its marked beads */
    int nrep = rd == 0 ? nl : 0;
    int nrep_m = m1 - m0;
    for (int q = lane; q < nrep + nrep_m; q += 32) {
        int ld, ft;
        if (q < nrep) {
            ld = q;
            if (W.lead_m[ld]) continue;          /* replayed in its round */
            ft = W.lead_l[ld] == i ? 0 : -1;
        } else {
            ld = W.mk[m0 + q - nrep];
            ft = 2 + (q - nrep);
        }
        int l = W.lead_l[ld];
        double t;
        int p, y;
        bool qq;
        if (l == i) { t = W.fs.tg_raw[0]; p = W.fs.tg_p[0]; y = W.fs.tg_y[0]; qq = okey(t) < imax_key; }
        else { t = S.tim[l]; p = S.nptnr[l]; y = S.colt[l]; qq = S.queued[l] != 0; }
        for (int pp = W.lead_q[ld]; pp < n; ++pp) {
            if (W.ops_l[pp] != l) continue;
            int src = W.ops_s[pp];
            if (p == src) {
                if (ft < 0) { set_err(E, DMD_E_STATE, l); break; }
                t = W.fs.tg_raw[ft]; p = W.fs.tg_p[ft]; y = W.fs.tg_y[ft]; qq = okey(t) < imax_key;
            } else if (W.op_y[pp] != -128) {
                double tn = W.op_t[pp];
                long long kn = okey(tn);
                if (key_less(kn, src, okey(t), p)) { t = tn; p = src; y = W.op_y[pp]; qq = kn < imax_key; }
            }
        }
        int slot = 2 + ld;
        if (l == i) {
            W.pb[slot] = -1;
            W.pt[0] = t; W.pn[0] = p; W.pc[0] = (int8_t)y; W.pq[0] = qq;
        } else {
            W.pb[slot] = l;
            W.pt[slot] = t; W.pn[slot] = p; W.pc[slot] = (int8_t)y; W.pq[slot] = qq;
        }
    }
    __syncwarp();
}

/* 7: the earliest new queued entry of this event */
__device__ void warp_rp_tnew(WarpArea &W) {
    int lane = threadIdx.x & 31;
    long long bk = DMD_KEY_INF;
    int bb = INT_MAX;
    for (int q = lane; q < W.npred; q += 32) {
        int b = W.pb[q];
        if (b < 0 || !W.pq[q]) continue;
        long long kk = okey(W.pt[q]);
        if (key_less(kk, b, bk, bb)) { bk = kk; bb = b; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        long long k2 = __shfl_xor_sync(FULL, bk, o);
        int b2 = __shfl_xor_sync(FULL, bb, o);
        if (key_less(k2, b2, bk, bb)) { bk = k2; bb = b2; }
    }
    if (lane == 0) { W.tnew_key = bk; W.tnew_idx = bb; }
    __syncwarp();
}

__device__ void warp_repredict(const DSys &S, Err E, WarpArea &W, int i, int j, double tf, double imax,
                               int hbonds) {
    warp_rp_lists(S, W, i, j);
    DMD_SUB(3);
    const double Hraw = imax + DMD_LTSTEP - tf;   /* eventredo_up's starting time */
    const long long Hkey = okey(Hraw);
    const int nm = W.nmarked;
    const int per_round = TG_MAX - 2;
    int rounds = nm > 0 ? (nm + per_round - 1) / per_round : 1;
    for (int rd = 0; rd < rounds; ++rd) {
        warp_rp_targets(S, W, i, j, rd, Hraw, Hkey);
        DMD_SUB(4);
        warp_rp_tasks(S, E, W, rd, tf, hbonds);
        DMD_SUB(5);
        warp_rp_finish(S, E, W, i, j, rd, tf, imax);
    }
    DMD_SUB(7);
    warp_rp_tnew(W);
}

__device__ void warp_commit_preds(const DSys &S, const WarpArea &W) {
    int lane = threadIdx.x & 31;
    for (int q = lane; q < W.npred; q += 32) {
        int b = W.pb[q];
        if (b < 0) continue;
        set_pred(S, b, W.pt[q], W.pn[q], W.pc[q], W.pq[q] != 0);
    }
    __syncwarp();
}

/* ------------------------------------------------------------------ */
/* footprints of a batch candidate                                     */
/* ------------------------------------------------------------------ */
/* Footprint of one candidate, as three sets of beads:
 *   R: beads whose state (position, velocity, identity, H-bond partner,
 *      extra_repuls, pair-type overrides) the event reads: i, j, their
 *      extra_repuls, the H-bond helpers of i, j and of their H-bond
 *      partners, both neighbour lists of i and j, and for every bead that may
 *      need a full re-prediction its up list and extras;
 *   W: beads whose state the collision may write: i, j, their extra_repuls
 *      and their own helpers (code/repuls_add.f, repuls_del_b.f, the
 *      shoulders of main.F90:825-868) - W is part of R;
 *   Q: beads whose event-queue entry the event reads and rewrites: i, j, the
 *      down lists, the lower extras and the helpers that become extras.
 * Candidate k conflicts with an earlier k' when R(k) meets W(k'), W(k) meets
 * R(k') or Q(k) meets Q(k'): then the two do not commute.  Reading the same
 * neighbour is no conflict.  A claim raises the three tables (own, own + N,
 * own + 2N) to the candidate's ticket, (batch sequence) * 64 + (63 - slot),
 * so that after all claims each entry holds the ticket of the earliest
 * candidate whose set has the bead; tickets grow from batch to batch and
 * the tables need no reset.  The beads are listed in W.rset/wset/qset for
 * warp_footprint_test(). */
__device__ void warp_footprint_claim(const DSys &S, WarpArea &W, unsigned *own, unsigned ticket, int i, int j) {
    int lane = threadIdx.x & 31;
    const int N = S.N;
    unsigned *own_r = own, *own_w = own + N, *own_q = own + 2 * N;
    if (lane == 0) { W.nrset = 0; W.nwset = 0; W.nqset = 0; W.casc_over = 0; }
    __syncwarp();
    auto visit_r = [&](int b) {
        if (b < 0) return;
        atomicMax(&own_r[b], ticket);
        int pos = atomicAdd(&W.nrset, 1);
        if (pos < RSET_MAX) W.rset[pos] = b;
    };
    auto visit_w = [&](int b) {
        if (b < 0) return;
        atomicMax(&own_w[b], ticket);
        int pos = atomicAdd(&W.nwset, 1);
        if (pos < WSET_MAX) W.wset[pos] = b;
        visit_r(b);
    };
    auto visit_q = [&](int b) {
        if (b < 0) return;
        atomicMax(&own_q[b], ticket);
        int pos = atomicAdd(&W.nqset, 1);
        if (pos < QSET_MAX) W.qset[pos] = b;
        visit_r(b);
    };
    /* fixed part on lanes 0..17 */
    if (lane < 18) {
        int b = -1;
        if (lane == 0) b = i;
        else if (lane == 1) b = j;
        else if (lane < 6) b = S.er[4 * i + lane - 2];
        else if (lane < 10) b = S.er[4 * j + lane - 6];
        else {
            int which = (lane - 10) >> 1;
            int x = which == 0 ? i : which == 1 ? j : which == 2 ? S.er[4 * i + 3] : S.er[4 * j + 3];
            int h1, h2;
            own_helpers(S, x, h1, h2);
            b = (lane & 1) ? h2 : h1;
        }
        if (lane < 14) visit_w(b);   /* i, j, extras, own helpers */
        else visit_r(b);             /* the partners' helpers: read only */
        /* queue entries: i, j, the lower extras (0..2) and the helpers */
        bool q = lane < 2 || (lane >= 2 && lane < 5) || (lane >= 6 && lane < 9) || (lane >= 10 && lane < 14);
        if (q) visit_q(b);
    }
    /* neighbour lists of i and j */
    int ui = S.upn[i], di = S.dnn[i], uj = S.upn[j], dj = S.dnn[j];
    const int *UI = S.up + (size_t)i * S.cap, *DI = S.dn + (size_t)i * S.cap;
    const int *UJ = S.up + (size_t)j * S.cap, *DJ = S.dn + (size_t)j * S.cap;
    for (int q = lane; q < ui; q += 32) visit_r(UI[q]);
    for (int q = lane; q < di; q += 32) visit_q(DI[q]);
    for (int q = lane; q < uj; q += 32) visit_r(UJ[q]);
    for (int q = lane; q < dj; q += 32) visit_q(DJ[q]);
    /* beads that may be fully re-predicted */
    int nc = 0;
    for (int base = 0; base < di + dj; base += 32) {
        int q = base + lane;
        int l = -1;
        if (q < di) { l = DI[q]; if (S.nptnr[l] != i) l = -1; }
        else if (q < di + dj) { l = DJ[q - di]; if (S.nptnr[l] != j) l = -1; }
        unsigned m = __ballot_sync(FULL, l >= 0);
        int pos = nc + __popc(m & ((1u << lane) - 1));
        if (l >= 0 && pos < CASC_MAX - 10) W.casc[pos] = l;
        nc += __popc(m);
    }
    bool over = nc > CASC_MAX - 10;
    nc = min(nc, CASC_MAX - 10);
    if (lane < 10) {
        int b;
        if (lane < 3) b = S.er[4 * i + lane];
        else if (lane < 6) b = S.er[4 * j + lane - 3];
        else {
            int x = lane < 8 ? i : j, h1, h2;
            own_helpers(S, x, h1, h2);
            b = (lane & 1) ? h2 : h1;
        }
        W.casc[nc + lane] = b;
    }
    __syncwarp();
    /* their up lists and extras as one flat range over the lanes: entry
     * offsets by a warp scan, then each lane finds its cascade bead */
    nc += 10;
    int run = 0;
    for (int base = 0; base < nc; base += 32) {
        int c = base + lane;
        int l = c < nc ? W.casc[c] : -1;
        int cnt = l >= 0 ? S.upn[l] + 3 : 0;
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(FULL, incl, o); if (lane >= o) incl += v; }
        if (c < nc) W.cbase[c] = run + incl - cnt;
        run += __shfl_sync(FULL, incl, 31);
    }
    if (lane == 0) W.cbase[nc] = run;
    __syncwarp();
    for (int q = lane; q < run; q += 32) {
        int lo = 0, hi = nc - 1;          /* last cascade bead with cbase <= q */
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (W.cbase[mid] <= q) lo = mid; else hi = mid - 1;
        }
        int l = W.casc[lo];
        int k = q - W.cbase[lo];
        int ul = W.cbase[lo + 1] - W.cbase[lo] - 3;
        visit_r(k < ul ? S.up[(size_t)l * S.cap + k] : S.er[4 * l + (k - ul)]);
    }
    __syncwarp();
    /* an incomplete list (cascade or set overflow) ends the batch here */
    if (lane == 0) W.casc_over = over || W.nrset > RSET_MAX || W.nwset > WSET_MAX || W.nqset > QSET_MAX;
    __syncwarp();
}
__device__ bool warp_footprint_test(const WarpArea &W, const volatile unsigned *own, int N, unsigned ticket) {
    int lane = threadIdx.x & 31;
    const volatile unsigned *own_r = own, *own_w = own + N, *own_q = own + 2 * N;
    bool conflict = false;
    int nr = min(W.nrset, RSET_MAX), nw = min(W.nwset, WSET_MAX), nq = min(W.nqset, QSET_MAX);
    for (int q = lane; q < nr; q += 32) conflict |= own_w[W.rset[q]] > ticket;
    for (int q = lane; q < nw; q += 32) conflict |= own_r[W.wset[q]] > ticket;
    for (int q = lane; q < nq; q += 32) conflict |= own_q[W.qset[q]] > ticket;
    return __any_sync(FULL, conflict);
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
    for (int k = 1; k < NWARPS; ++k) r = fmax(r, sh.red_d[k]);
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
    for (int k = 0; k < NWARPS; ++k) r += sh.red_d[k];
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
    for (int k = 0; k < NWARPS; ++k) r += sh.red_i[k];
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

__device__ void cta_build_lists(const DSys &S, SharedState &sh, int hbonds) {
    const int N = S.N, nc = S.ncell;
    const int ncell3 = nc * nc * nc;
    const DTab &T = *S.tab;
    if (nc >= 3) {
        for (int c = threadIdx.x; c < ncell3; c += blockDim.x) S.cell_count[c] = 0;
        __syncthreads();
        for (int b = threadIdx.x; b < N; b += blockDim.x) {
            int cx = cell_coord(S.x[b], nc), cy = cell_coord(S.y[b], nc), cz = cell_coord(S.z[b], nc);
            atomicAdd(&S.cell_count[(cz * nc + cy) * nc + cx], 1);
        }
        __syncthreads();
        {
            int per = (ncell3 + blockDim.x - 1) / blockDim.x;
            int lo = threadIdx.x * per, hi = min(lo + per, ncell3);
            int s = 0;
            for (int c = lo; c < hi; ++c) s += S.cell_count[c];
            int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            int incl = s;
            for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(FULL, incl, o); if (lane >= o) incl += v; }
            __syncthreads();
            if (lane == 31) sh.red_i[w] = incl;
            __syncthreads();
            int woff = 0;
            for (int k = 0; k < w; ++k) woff += sh.red_i[k];
            int run = woff + incl - s;
            for (int c = lo; c < hi; ++c) { int v = S.cell_count[c]; S.cell_start[c] = run; run += v; }
            __syncthreads();
            for (int c = lo; c < hi; ++c) S.cell_count[c] = 0;
            if (threadIdx.x == 0) S.cell_start[ncell3] = N;
            __syncthreads();
        }
        for (int b = threadIdx.x; b < N; b += blockDim.x) {
            int cx = cell_coord(S.x[b], nc), cy = cell_coord(S.y[b], nc), cz = cell_coord(S.z[b], nc);
            int c = (cz * nc + cy) * nc + cx;
            int slot = atomicAdd(&S.cell_count[c], 1);
            S.cell_beads[S.cell_start[c] + slot] = b;
        }
        __syncthreads();
    }
    for (int b = threadIdx.x; b < N; b += blockDim.x) {
        int nu = 0, nd = 0;
        int *up = S.up + (size_t)b * S.cap, *dn = S.dn + (size_t)b * S.cap;
        int8_t *upc = S.upc + (size_t)b * S.cap;
        const BeadInfo ib = S.info[b];
        double xb = S.x[b], yb = S.y[b], zb = S.z[b];
        const float xbf = S.xf[b], ybf = S.yf[b], zbf = S.zf[b];
        auto consider = [&](int c) {
            if (c == b) return;
            int st = static_code(S.info[c], ib, hbonds);
            int code = pair_code_st(S, c, b, st);
            bool take;
            if ((code >= 4 && code <= 12) || (code >= 17 && code < 27)) take = true;
            else {
                /* Single-precision prefilter.  Positions lie in [-0.5, 0.5]
                 * at a rebuild, so each wrapped single-precision component
                 * is within 1e-7 of the double one and r2 within
                 * 4e-7 + 4e-7 * r2; only pairs that close to the cutoff are
                 * decided in double precision, as the reference does. */
                float fx = xbf - S.xf[c], fy = ybf - S.yf[c], fz = zbf - S.zf[c];
                fx = fx - rintf(fx); fy = fy - rintf(fy); fz = fz - rintf(fz);
                float r2f = fx * fx + fy * fy + fz * fz;
                float cut = (float)T.rlsq[code];
                float margin = 4e-7f + 4e-7f * cut;
                if (r2f > cut + margin) take = false;
                else if (r2f < cut - margin) take = true;
                else {
                    double rx = xb - S.x[c], ry = yb - S.y[c], rz = zb - S.z[c];
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
            int cx = cell_coord(xb, nc), cy = cell_coord(yb, nc), cz = cell_coord(zb, nc);
            /* the 27 cell ranges are loaded before the first one is walked */
            int lo[27], hi[27];
#pragma unroll
            for (int s27 = 0; s27 < 27; ++s27) {
                int dx = s27 % 3 - 1, dy = (s27 / 3) % 3 - 1, dz = s27 / 9 - 1;
                int gx = (cx + dx + nc) % nc, gy = (cy + dy + nc) % nc, gz = (cz + dz + nc) % nc;
                int c0 = (gz * nc + gy) * nc + gx;
                lo[s27] = S.cell_start[c0];
                hi[s27] = S.cell_start[c0 + 1];
            }
            for (int s27 = 0; s27 < 27; ++s27)
                for (int q = lo[s27]; q < hi[s27]; ++q) consider(S.cell_beads[q]);
        } else {
            for (int c = 0; c < N; ++c) consider(c);
        }
        if (nu > S.cap || nd > S.cap) set_err(sh, DMD_E_CAPACITY, b);
        S.upn[b] = min(nu, S.cap);
        S.dnn[b] = min(nd, S.cap);
    }
    __syncthreads();
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
        double tij = 0.0;
        int ty = 0;
        bool ok = false;
        if (pa >= 0) {
            int code = st >= 0 ? pair_code_st(S, pbb, pa, st) : pair_code(S, pbb, pa, hbonds);
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

__device__ void cta_rebuild(const DSys &S, SharedState &sh, ScratchRef fr, int hbonds) {
    DMD_SUB(-1);
    for (int b = threadIdx.x; b < S.N; b += blockDim.x) {
        double px = S.x[b], py = S.y[b], pz = S.z[b];
        px = px - d_nint(px); py = py - d_nint(py); pz = pz - d_nint(pz);
        S.x[b] = px; S.y[b] = py; S.z[b] = pz;
        S.ox[b] = px; S.oy[b] = py; S.oz[b] = pz;
        S.xf[b] = (float)px; S.yf[b] = (float)py; S.zf[b] = (float)pz;
    }
    __syncthreads();
    cta_build_lists(S, sh, hbonds);
    cta_predict_all(S, sh, fr, sh.sc.interval_max, hbonds);
    cta_tree_rebuild(S);
}

/* interval event N+2 (code/main.F90:1126-1187, code/displ.f), spread over the
 * C CTAs of the system: each shifts the times and advances the positions of
 * its slice of the beads; the leader (L, rank 0) takes the maximum
 * displacement and decides on a rebuild, which it does alone.  sh.tf_iv
 * holds tfalse of the event on every CTA. */
__device__ bool cluster_interval(const DSys &S, SharedState &sh, SharedState *L, int rank, int C, ScratchRef fr,
                                 int hbonds) {
    const int N = S.N;
    const double tf = sh.tf_iv;
    const DTab &T = *S.tab;
    const int stride = C * blockDim.x, t0 = rank * blockDim.x + threadIdx.x;
    DMD_SUB(-1);
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
    __syncthreads();
    if ((threadIdx.x & 31) == 0) sh.red_d[threadIdx.x >> 5] = __longlong_as_double(dmax_bits);
    __syncthreads();
    if (threadIdx.x == 0) {
        long long m = 0;
        for (int w = 0; w < NWARPS; ++w) { long long v = dbits(sh.red_d[w]); if (v > m) m = v; }
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
        if (sh.rebuild) {
            for (int k = threadIdx.x; k < N; k += blockDim.x) set_pred(S, k, sh.sc.interval_max + DMD_LTSTEP, -1, -1, false);
            __syncthreads();
            cta_rebuild(S, sh, fr, hbonds);
        }
        if (threadIdx.x == 0) set_pred(S, N + 1, sh.sc.interval * 0.999, -2, -2, true);
    }
    csync(C);
    if (threadIdx.x == 0 && rank != 0) sh.rebuild = L->rebuild;
    __syncthreads();
    bool rb = sh.rebuild != 0;
    /* level 1 of the tournament, spread over the CTAs (level 2 follows at
     * the leader's next selection) */
    for (int g = t0; g < S.nl1; g += stride) l1_update(S, g, N + 3);
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
    }
    __syncthreads();
}

/* ------------------------------------------------------------------ */
/* batch selection                                                     */
/* ------------------------------------------------------------------ */
/* The bead events below the cut, sorted in (key, index) order into
 * sh.sort_*; returns how many there are (1 when the window could not be
 * made small enough: the root alone). */
__device__ int cta_candidates(const DSys &S, SharedState &sh, int root, long long kroot, int slots) {
    const int N = S.N;
    long long kp = min(min(S.key[N], S.key[N + 1]), S.key[N + 2]);
    bool ok = false;
    for (int attempt = 0; attempt < 8; ++attempt) {
        if (threadIdx.x == 0) {
            double tr = S.tim[root];
            long long kc = okey(tr + sh.delta);
            if (kc <= kroot) kc = kroot + 1;
            if (kc > kp) kc = kp;
            sh.kcut = kc;
            sh.ncand = 0;
            sh.ngroups = 0;
        }
        __syncthreads();
        long long kc = sh.kcut;
        /* groups whose minimum lies below the cut */
        for (int g = threadIdx.x; g < S.nl1; g += blockDim.x) {
            if (S.l1k[g] < kc) {
                int s = atomicAdd(&sh.ngroups, 1);
                if (s < 256) sh.groups[s] = g;
            }
        }
        __syncthreads();
        int ng = sh.ngroups;
        if (ng <= 256) {
            int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            for (int gi = warp; gi < ng; gi += NWARPS) {
                int e = sh.groups[gi] * 32 + lane;
                long long k = (e < N) ? S.key[e] : DMD_KEY_INF;
                if (k < kc) {
                    int s = atomicAdd(&sh.ncand, 1);
                    if (s < CAND_MAX) { sh.cand_key[s] = k; sh.cand_idx[s] = e; }
                }
            }
        }
        __syncthreads();
        if (ng <= 256 && sh.ncand <= CAND_MAX) { ok = true; break; }
        if (threadIdx.x == 0) {
            sh.delta = sh.delta * 0.25;
            if (!(sh.delta > sh.sc.interval * 1e-9)) sh.delta = sh.sc.interval * 1e-9;
        }
        __syncthreads();
    }
    int nc = sh.ncand;
    if (!ok || nc < 1) {
        if (threadIdx.x == 0) { sh.sort_key[0] = kroot; sh.sort_idx[0] = root; }
        __syncthreads();
        return 1;
    }
    if ((int)threadIdx.x < nc) {
        long long k = sh.cand_key[threadIdx.x];
        int e = sh.cand_idx[threadIdx.x];
        int rank = 0;
        for (int u = 0; u < nc; ++u)
            if (key_less(sh.cand_key[u], sh.cand_idx[u], k, e)) ++rank;
        sh.sort_key[rank] = k;
        sh.sort_idx[rank] = e;
    }
    if (threadIdx.x == 0) {
        /* aim at about one to four candidates per warp */
        if (nc < slots) sh.delta = sh.delta * 2.0;
        else if (nc > 4 * slots) sh.delta = sh.delta * 0.5;
        if (!(sh.delta > sh.sc.interval * 1e-9)) sh.delta = sh.sc.interval * 1e-9;
    }
    __syncthreads();
    return nc;
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

__global__ void __launch_bounds__(NTHREADS, 1) k_init(DSys *systems, int nsys, int hbonds_mask) {
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
    cta_rebuild(S, sh, ScratchRef{(char *)fs, sizeof(FullScratch)}, hbonds);
    if (threadIdx.x == 0) *S.sc = sh.sc;
}

/* The event loop of code/main.F90:484-1258 for nsys systems, each advanced
 * by one cluster of C CTAs (C = 1: one CTA).  The leader CTA (rank 0)
 * selects events and keeps the counters; a batch's candidates go one per
 * warp over all CTAs of the cluster. */
__global__ void __launch_bounds__(NTHREADS, 1) k_run(DSys *systems, int nsys, long long target_all,
                                                     const long long *targets, int hbonds_mask,
                                                     const int *chain_start, const int *chain_len,
                                                     const int *chain_off, dmd_diag *outputs, int own_cap, int C) {
    extern __shared__ WarpArea warea[];
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    const int rank = C > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int r = blockIdx.x / C;
    if (r >= nsys) return;             /* whole clusters only */
    const long long target = targets ? targets[r] : target_all;   /* events for this system */
    const bool leader = rank == 0;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    const DSys &S = S_sh;
    const int N = S.N;
    const int hbonds = hbonds_mask & 1;
    const bool phys = (S.flags & DMD_FLAG_COUNT_PHYSICAL) != 0;
    const bool stop_out = (S.flags & DMD_FLAG_STOP_AT_OUTPUT) != 0;
    const bool serial = (S.flags & DMD_FLAG_SERIAL) != 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gw = rank * NWARPS + warp;          /* candidate slot of this warp */
    const int slots = min(C * NWARPS, CAND_MAX);
    WarpArea &W = warea[warp];
    SharedState *L = C > 1 ? cg::this_cluster().map_shared_rank(&sh, 0) : &sh;
    if (threadIdx.x == 0) {
        sh.sc = *S.sc; sh.sc.done = 0; sh.sc.stop = 0;
        sh.delta = sh.sc.interval * 0.05;
        sh.bseq = 0;
        sh.exitf = 0;
    }
    /* footprint claim table: shared memory when one CTA holds the system and
     * it fits, else the system's global array; cleared at every launch */
    TaskPool &TP = *(TaskPool *)(warea + NWARPS);
    unsigned *own = (C == 1 && N <= own_cap) ? (unsigned *)((char *)(warea + NWARPS) + sizeof(TaskPool)) : S.owner;
    if (threadIdx.x == 0) TP.n = 0;
    for (int b = rank * blockDim.x + threadIdx.x; b < 3 * N; b += C * blockDim.x) own[b] = 0u;
    csync(C);
    DMD_PHASE_START(leader ? r : -1);
    const int *cs = chain_start + chain_off[r], *cl = chain_len + chain_off[r];
    const long long max_iter = 16 * target + 1000000;
    const long long t_start = clock64();
    long long iter = 0;
    while (true) {
        /* ---- the leader selects the next event (and a batch) ---- */
        if (leader) {
            for (int h = threadIdx.x; h < S.nl2; h += blockDim.x) l2_update(S, h);
            __syncthreads();
            if (threadIdx.x == 0) {
                bool ex = sh.sc.done >= target || sh.sc.err || sh.sc.stop;
                if (!ex && ++iter > max_iter) { set_err(sh, DMD_E_DEVICE_TIMEOUT, 0); ex = true; }
                sh.exitf = ex;
            }
            __syncthreads();
            if (!sh.exitf && warp == 0) {
                long long kroot;
                int e = warp_tree_root(S, kroot);
                if (lane == 0) {
                    sh.ev = e;
                    sh.kcut = kroot;
                    if (e < 0) { set_err(sh, DMD_E_STATE, 0); sh.exitf = 1; }
                }
            }
            __syncthreads();
            DMD_PHASE(0);
            if (!sh.exitf && sh.ev < N) {
                int e = sh.ev;
                long long kroot = sh.kcut;
                long long left = target - sh.sc.done;
                int m;
                if (serial || left <= 1) {
                    if (threadIdx.x == 0) { sh.sort_key[0] = kroot; sh.sort_idx[0] = e; }
                    __syncthreads();
                    m = 1;
                } else {
                    m = cta_candidates(S, sh, e, kroot, slots);
                    if (m > slots) m = slots;
                    if (m > left) m = (int)left;
                }
                if (threadIdx.x == 0) {
                    sh.m = m;
                    sh.tick_reset = m > 1 && sh.bseq >= DMD_TICKET_SEQ_MAX;
                    sh.c_simple[0] = 0;    /* set by the footprint test when m > 1 */
                }
                DMD_PHASE(1);
            } else if (!sh.exitf && threadIdx.x == 0) {
                /* a pseudo event: its counter and time */
                sh.sc.coll += 1;
                sh.tf_iv = S.tim[sh.ev];
                if (sh.ev != N) sh.sc.tfalse = sh.tf_iv;
            }
            if (threadIdx.x == 0) {
                sh.coll0 = sh.sc.coll; sh.log0 = sh.sc.log_count; sh.imax = sh.sc.interval_max; sh.tnow = sh.sc.t;
            }
        }
        csync(C);
        /* ---- the other CTAs copy the leader's decision ---- */
        if (!leader) {
            if (threadIdx.x == 0) {
                sh.exitf = L->exitf; sh.ev = L->ev; sh.m = L->m; sh.tick_reset = L->tick_reset; sh.bseq = L->bseq;
                sh.coll0 = L->coll0; sh.log0 = L->log0; sh.imax = L->imax; sh.tnow = L->tnow; sh.tf_iv = L->tf_iv;
            }
            if (threadIdx.x < NWARPS) {
                int k = rank * NWARPS + threadIdx.x;
                if (k < CAND_MAX) { sh.sort_idx[k] = L->sort_idx[k]; sh.sort_key[k] = L->sort_key[k]; }
            }
            __syncthreads();
        }
        if (sh.exitf) break;
        int ph_kind __attribute__((unused)) = 9;
        const int e = sh.ev;
        if (e < N) {
            ph_kind = 5;
            /* ---- a batch of pair events ---- */
            const int m = sh.m;
            int P = 1;
            if (m > 1) {
                if (sh.tick_reset) {   /* tickets exhausted: clear the table */
                    for (int b = rank * blockDim.x + threadIdx.x; b < 3 * N; b += C * blockDim.x) own[b] = 0u;
                    csync(C);
                    if (threadIdx.x == 0) sh.bseq = 0;
                    __syncthreads();
                }
                unsigned ticket = ((unsigned)(sh.bseq + 1) << 6) | (unsigned)(63 - gw);
                if (gw < m) {
                    int i = sh.sort_idx[gw];
                    warp_footprint_claim(S, W, own, ticket, i, S.nptnr[i]);
                }
                csync(C);
                DMD_PHASE(10);
                if (gw < m) {
                    bool c = warp_footprint_test(W, own, N, ticket);
                    if (lane == 0) {
                        int ct0 = S.colt[sh.sort_idx[gw]];
                        L->c_conflict[gw] = c; L->c_over[gw] = W.casc_over;
                        L->c_simple[gw] = ct0 >= 1 && ct0 <= 3;
                    }
                }
                csync(C);
                DMD_PHASE(11);
                if (leader && threadIdx.x == 0) {
                    sh.bseq = sh.tick_reset ? 1 : sh.bseq + 1;
                    /* the longest conflict-free prefix; an incomplete footprint
                     * (cascade list overflow) ends the batch after its event */
                    int p = m;
                    for (int k = 0; k < m; ++k) {
                        if (k > 0 && sh.c_conflict[k]) { p = k; break; }
                        if (sh.c_over[k]) { p = k > 0 ? k : 1; break; }
                    }
                    sh.P = p;
                }
                csync(C);
                if (!leader && threadIdx.x == 0) sh.P = L->P;
                __syncthreads();
                P = sh.P;
                DMD_PHASE(2);
            }
            /* speculative commit of each event on its warp */
            const long long coll0 = sh.coll0;
            const double imax = sh.imax;
            const bool split = C == 1 && P <= NWARPS / 2;
            if (gw < P) {
                int i = sh.sort_idx[gw];
                int j = S.nptnr[i];
                double tf = S.tim[i];
                if (lane == 0) { W.i = i; W.j = j; W.tf = tf; W.coll = coll0 + gw + 1; }
                __syncwarp();
                DMD_SUB(-1);
                warp_snapshot(S, W, i, j);
                DMD_SUB(0);
                if (lane == 0) { W.err = 0; W.err_info = 0; }
                __syncwarp();
                Err E{&W.err, &W.err_info};
                warp_collision(S, E, W, i, j, tf, coll0 + gw + 1, hbonds);
                DMD_SUB(1);
                /* the re-prediction's lists and tasks; the tasks go to the
                 * CTA's pool when they fit (one round of full
                 * re-predictions), else this warp runs them after the pool.
                 * In a batch of at most NWARPS/2 events, a second warp
                 * prepares them while this one computes the collision,
                 * when the collision cannot change the H-bond state they
                 * read (coltype 1-3). */
                if (!(split && sh.c_simple[gw])) warp_rp_prepare(S, W, TP, warp, i, j, tf, imax);
            } else if (split && warp >= NWARPS / 2 && warp - NWARPS / 2 < P && sh.c_simple[warp - NWARPS / 2]) {
                const int k = warp - NWARPS / 2;
                const int i = sh.sort_idx[k];
                warp_rp_prepare(S, warea[k], TP, k, i, S.nptnr[i], S.tim[i], imax);
            }
            __syncthreads();
            /* every pooled prediction task of this CTA's events, all warps */
            {
                const int ntot = min(TP.n, PTASK_MAX);
                for (int q = threadIdx.x; q < ntot; q += blockDim.x) {
                    int pa = TP.a[q];
                    if (pa < 0) { TP.ok[q] = 0; continue; }
                    int owner = TP.flag[q] >> 1;
                    WarpArea &O = warea[owner];
                    Err EO{&O.err, &O.err_info};
                    double tt;
                    int ty;
                    bool ok = rp_predict(S, EO, pa, TP.b[q], TP.st[q], (TP.flag[q] & 1) != 0, O.tf, hbonds, tt, ty);
                    TP.t[q] = tt; TP.ty[q] = (int8_t)ty; TP.ok[q] = ok;
                }
            }
            __syncthreads();
            if (gw < P) {
                const int i = W.i, j = W.j;
                const double tf = W.tf;
                Err E{&W.err, &W.err_info};
                if (W.pooled) {
                    /* down operations' times, and the minimum per full
                     * re-prediction over its contiguous tasks */
                    const int base = W.pool_base, nop = W.nops, ntg = W.ntg;
                    for (int q = lane; q < nop; q += 32) {
                        W.op_t[q] = TP.t[base + q];
                        W.op_y[q] = TP.ok[base + q] ? TP.ty[base + q] : (int8_t)-128;
                    }
                    for (int t = lane; t < ntg; t += 32) {
                        long long bk = W.fs.tg_k[t];
                        int bp = W.fs.tg_p[t];
                        double braw = W.fs.tg_raw[t];
                        int by = W.fs.tg_y[t];
                        for (int x = base + nop + W.fs.tg_base[t]; x < base + nop + W.fs.tg_base[t + 1]; ++x) {
                            if (!TP.ok[x]) continue;
                            long long k = okey(TP.t[x]);
                            if (key_less(k, TP.b[x], bk, bp)) { bk = k; bp = TP.b[x]; braw = TP.t[x]; by = TP.ty[x]; }
                        }
                        W.fs.tg_k[t] = bk; W.fs.tg_p[t] = bp; W.fs.tg_raw[t] = braw; W.fs.tg_y[t] = (int8_t)by;
                    }
                    __syncwarp();
                    warp_rp_finish(S, E, W, i, j, 0, tf, imax);
                    warp_rp_tnew(W);
                } else {
                    warp_repredict(S, E, W, i, j, tf, imax, hbonds);
                }
                DMD_SUB(8);
                if (lane == 0 && W.xpulse) {
                    if (S.ident[i] < S.ident[j]) repuls_del_b(S, i, j); else repuls_del_b(S, j, i);
                }
                __syncwarp();
                if (lane == 0) {
                    L->c_tnew_key[gw] = W.tnew_key; L->c_tnew_idx[gw] = W.tnew_idx;
                    L->c_err[gw] = W.err; L->c_err_info[gw] = W.err_info;
                    L->c_ct[gw] = W.ct; L->c_tf[gw] = W.tf;
                }
            }
            if (threadIdx.x == 0) TP.n = 0;   /* the pool is free until the next batch */
            csync(C);
            DMD_PHASE(3);
            /* validation: event k stands if it precedes every new entry of
             * events 0..k-1; the leader also books the committed events */
            if (leader && threadIdx.x == 0) {
                int v = P;
                long long bk = DMD_KEY_INF;
                int bb = INT_MAX;
                for (int k = 0; k < P; ++k) {
                    if (k > 0 && !key_less(sh.sort_key[k], sh.sort_idx[k], bk, bb)) { v = k; break; }
                    if (sh.c_err[k]) {   /* the run stops after the first event in error */
                        set_err(sh, sh.c_err[k], sh.c_err_info[k]);
                        v = k + 1;
                        break;
                    }
                    if (key_less(sh.c_tnew_key[k], sh.c_tnew_idx[k], bk, bb)) { bk = sh.c_tnew_key[k]; bb = sh.c_tnew_idx[k]; }
                }
                sh.V = v;
                for (int k = 0; k < v; ++k) {
                    int ct = sh.c_ct[k];
                    if (ct >= 1 && ct < 32) sh.sc.nevents[ct] += 1;
                }
                sh.sc.coll = coll0 + v;
                sh.sc.n_pair += v;
                sh.sc.n_batches += 1;
                sh.sc.n_rolled_back += P - v;
                sh.sc.n_candidates += m;
                sh.sc.done += v;
                sh.sc.tfalse = sh.c_tf[v - 1];
                sh.sc.old_tfalse = sh.c_tf[v - 1];
                if (S.log && S.log_cap > 0) sh.sc.log_count += v;
            }
            csync(C);
            if (!leader && threadIdx.x == 0) sh.V = L->V;
            __syncthreads();
            DMD_PHASE(4);
            const int V = sh.V;
            if (gw < P) {
                if (gw < V) {
                    warp_commit_preds(S, W);
                    if (lane == 0) log_event(S, sh.log0 + gw, W.coll, sh.tnow, W.tf, W.i, W.j, W.ct, W.evcode);
                } else {
                    warp_restore(S, W);
                }
            }
            csync(C);   /* every commit lands before any level-1 group is recomputed */
            if (gw < V) warp_l1_refresh(S, W.pb, W.npred);
        } else if (e == N) {
            ph_kind = 6;
            /* ---- ghost collision: leader warp 0 ---- */
            if (leader && warp == 0) {
                double tf = sh.tf_iv;
                if (lane == 0) {
                    int i = lane_ghost(S, sh, tf);
                    W.i = i; W.tf = tf;
                }
                __syncwarp();
                int i = W.i;
                tf = W.tf;
                DMD_SUB(-1);
                warp_repredict(S, cta_err(sh), W, i, -1, tf, sh.sc.interval_max, hbonds);
                warp_commit_preds(S, W);
                if (lane == 0) {
                    W.pb[W.npred] = N;   /* the ghost entry itself */
                    log_event(S, sh.sc.log_count, sh.sc.coll, sh.sc.t, tf, i, -1, DMD_EV_GHOST, 0);
                    if (S.log && S.log_cap > 0) sh.sc.log_count += 1;
                    sh.sc.tfalse = tf;
                    sh.sc.old_tfalse = tf;
                    sh.sc.done += 1;
                }
                __syncwarp();
                warp_l1_refresh(S, W.pb, W.npred + 1);
            }
        } else if (e == N + 1) {
            ph_kind = 7;
            /* ---- interval: all CTAs ---- */
            double t_before = sh.tnow, tf = sh.tf_iv;
            bool rb = cluster_interval(S, sh, L, rank, C, ScratchRef{(char *)&warea[0].fs, sizeof(WarpArea)}, hbonds);
            if (leader && threadIdx.x == 0) {
                sh.sc.n_interval += 1;
                log_event(S, sh.sc.log_count, sh.sc.coll, t_before, tf, N + 1, -1, rb ? DMD_EV_REBUILD : DMD_EV_INTERVAL, 0);
                if (S.log && S.log_cap > 0) sh.sc.log_count += 1;
                sh.sc.old_tfalse = sh.sc.tfalse;
                if (!phys) sh.sc.done += 1;
            }
        } else {
            ph_kind = 8;
            /* ---- output: the leader CTA ---- */
            if (leader) {
                cta_diag(S, sh, cs, cl, outputs ? outputs + r : nullptr);
                if (threadIdx.x == 0) {
                    sh.sc.n_output += 1;
                    double tn = 3.3 / (sqrt(S.tab->setemp)) + 5 + sh.sc.tfalse;
                    set_pred(S, N + 2, tn, -2, -2, tn < sh.sc.interval_max);
                    log_event(S, sh.sc.log_count, sh.sc.coll, sh.sc.t, sh.sc.tfalse, N + 2, -1, DMD_EV_OUTPUT, 0);
                    if (S.log && S.log_cap > 0) sh.sc.log_count += 1;
                    sh.sc.old_tfalse = sh.sc.tfalse;
                    if (!phys) sh.sc.done += 1;
                    if (stop_out) sh.sc.stop = 1;
                    sh.touched[0] = N + 2;
                }
                __syncthreads();
                if (warp == 0) warp_l1_refresh(S, sh.touched, 1);
            }
        }
        csync(C);
        DMD_PHASE(ph_kind);
    }
    if (leader) {
        __syncthreads();
        if (threadIdx.x == 0) {
            sh.sc.run_cycles = clock64() - t_start;
            *S.sc = sh.sc;
        }
    }
    if (C > 1) cg::this_cluster().sync();   /* no CTA leaves while others may read its shared memory */
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
static_assert(sizeof(WarpArea) * NWARPS + sizeof(TaskPool) + OWN_SMEM_MAX * 3 * sizeof(unsigned) + sizeof(SharedState) +
                  sizeof(DSys) <= 227 * 1024,
              "k_run shared memory above the 227 KB a block may use");
static size_t run_smem(int own_cap) {
    return sizeof(WarpArea) * NWARPS + sizeof(TaskPool) + (size_t)own_cap * 3 * sizeof(unsigned);
}

cudaError_t dmd_launch_init(DSys *d_systems, int nsys, int hbonds, cudaStream_t st) {
    k_init<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, hbonds);
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
        e = cudaFuncSetAttribute(k_run, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)run_smem(OWN_SMEM_MAX));
        if (e != cudaSuccess) return e;
        done[dev] = true;
    }
    return cudaSuccess;
}

static void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr, int nsys, int C, size_t smem,
                           cudaStream_t st) {
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = dim3((unsigned)(nsys * C), 1, 1);
    cfg.blockDim = dim3(NTHREADS, 1, 1);
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
cudaError_t dmd_launch_run(DSys *d_systems, int nsys, int max_beads, int C, long long target, const long long *targets,
                           int hbonds, const int *chain_start, const int *chain_len, const int *chain_off,
                           dmd_diag *outputs, cudaStream_t st) {
    if (C != 1 && C != 2 && C != 4 && C != 8) return cudaErrorInvalidValue;
    cudaError_t e = k_run_attributes();
    if (e != cudaSuccess) return e;
    int own_cap = (C == 1 && max_beads <= OWN_SMEM_MAX) ? max_beads : 0;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config(cfg, attr, nsys, C, run_smem(own_cap), st);
    return cudaLaunchKernelEx(&cfg, k_run, d_systems, nsys, target, targets, hbonds, chain_start, chain_len, chain_off,
                              outputs, own_cap, C);
}

/* how many clusters of C CTAs of k_run can be resident at once */
cudaError_t dmd_max_active_clusters(int C, int *n) {
    cudaError_t e = k_run_attributes();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config(cfg, attr, 1, C, run_smem(C == 1 ? OWN_SMEM_MAX : 0), 0);
    return cudaOccupancyMaxActiveClusters(n, k_run, &cfg);
}
cudaError_t dmd_launch_diag(DSys *d_systems, int nsys, const int *chain_start, const int *chain_len,
                            const int *chain_off, dmd_diag *out, cudaStream_t st) {
    k_diag<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, chain_start, chain_len, chain_off, out);
    return cudaGetLastError();
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
    cta_rebuild(S, sh, ScratchRef{(char *)fs, sizeof(FullScratch)}, hbonds);
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
