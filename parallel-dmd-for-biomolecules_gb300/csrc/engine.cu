/*
 * engine.cu -- kernels of the GB300 PRIME20 DMD event engine.
 *
 * One CTA owns one system (a replica or a served request) for the whole
 * launch and runs the reference's main loop (code/main.F90:484-1258) on it:
 * select the earliest queued event, commit it, re-predict what it touched.
 * A launch with many CTAs advances many independent systems at once (the
 * batched-replica path); a launch with one CTA is the plain path.
 *
 * Per-event work inside the CTA:
 *   - event selection: a two-level tournament (argmin of 32 entries, then of
 *     32 groups) over the keys (queued ? tim : inf) in (time, index) order,
 *     which replaces the calendar queue of code/add_tbin.f / del_tbin.f;
 *   - the collision itself on one lane (it is O(1) and branch heavy);
 *   - re-prediction (code/partial_events.f) warp-parallel over neighbour
 *     lists, keeping the reference's per-bead order of down-list operations;
 *   - interval events (code/main.F90:1126-1187) and list rebuilds
 *     (code/nbor.f, code/events.f) spread over all threads of the CTA.
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

#include "dmd.h"
#include "engine.cuh"
#include "engine_api.h"

#define NTHREADS 256
#define NWARPS (NTHREADS / 32)
#define OPS_MAX 1024

struct SharedState {
    DScal sc;            /* this system's scalars while the CTA runs */
    int ev;              /* selected event entry */
    int ops_l[OPS_MAX];  /* down-list operations (bead, source) in reference order */
    int ops_s[OPS_MAX];
    int nops;
    int touched[OPS_MAX + 8];
    int ntouched;
    int redo_flag[32];   /* leaders whose op walk stopped at a full redo */
    double red_d[NWARPS];
    long long red_l[NWARPS * 4];
    int red_i[NWARPS * 4];
    int xpulse, ev_i, ev_j, ev_ct;
    int rebuild;
};

__device__ __forceinline__ void set_err(SharedState &sh, int code, int info) {
    if (sh.sc.err == 0) { sh.sc.err = code; sh.sc.err_info = info; }
}

/* ------------------------------------------------------------------ */
/* warp helpers                                                        */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ void warp_lexmin(double &t, int &p, int &ty) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double t2 = __shfl_xor_sync(0xffffffffu, t, o);
        int p2 = __shfl_xor_sync(0xffffffffu, p, o);
        int y2 = __shfl_xor_sync(0xffffffffu, ty, o);
        if (lex_less(t2, p2, t, p)) { t = t2; p = p2; ty = y2; }
    }
}

__device__ __forceinline__ double entry_key(const DSys &S, int e) {
    return S.queued[e] ? S.tim[e] : HUGE_VAL;
}

/* ------------------------------------------------------------------ */
/* tournament                                                          */
/* ------------------------------------------------------------------ */
__device__ void l1_update(const DSys &S, int g, int NE) {  /* one thread, group g */
    int best = -1;
    double bk = HUGE_VAL;
    int lo = g * 32, hi = min(lo + 32, NE);
    for (int e = lo; e < hi; ++e) {
        double k = entry_key(S, e);
        if (best < 0 || k < bk) { bk = k; best = e; }   /* ascending e: ties keep the lower index */
    }
    S.l1i[g] = best;
}
__device__ void l2_update(const DSys &S, int h) {  /* one thread, group h */
    int best = -1;
    double bk = HUGE_VAL;
    int lo = h * 32, hi = min(lo + 32, S.nl1);
    for (int g = lo; g < hi; ++g) {
        int e = S.l1i[g];
        double k = entry_key(S, e);
        if (best < 0 || lex_less(k, e, bk, best)) { bk = k; best = e; }
    }
    S.l2i[h] = best;
}
__device__ void cta_tree_rebuild(const DSys &S) {
    int NE = S.N + 3;
    for (int g = threadIdx.x; g < S.nl1; g += blockDim.x) l1_update(S, g, NE);
    __syncthreads();
    for (int h = threadIdx.x; h < S.nl2; h += blockDim.x) l2_update(S, h);
    __syncthreads();
}
/* warp: root of the tournament */
__device__ int warp_tree_root(const DSys &S) {
    int lane = threadIdx.x & 31;
    double bk = HUGE_VAL;
    int best = 0x7fffffff, dummy = 0;
    for (int h = lane; h < S.nl2; h += 32) {
        int e = S.l2i[h];
        double k = entry_key(S, e);
        if (lex_less(k, e, bk, best)) { bk = k; best = e; }
    }
    warp_lexmin(bk, best, dummy);
    return bk == HUGE_VAL ? -1 : best;
}
/* warp: refresh the groups holding the touched entries */
__device__ void warp_tree_update(const DSys &S, const int *touched, int nt) {
    int lane = threadIdx.x & 31;
    int NE = S.N + 3;
    for (int q = lane; q < nt; q += 32) l1_update(S, touched[q] >> 5, NE);
    __syncwarp();
    __threadfence_block();
    for (int q = lane; q < nt; q += 32) l2_update(S, touched[q] >> 10);
    __syncwarp();
    __threadfence_block();
}

/* ------------------------------------------------------------------ */
/* re-prediction (code/partial_events.f, eventredo_up.f, eventredo_down.f) */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ bool check_tij(SharedState &sh, double tij, int i, int j) {
    /* reference debug check: negative time beyond 1e-10 (code/eventredo_up.f:58-74) */
    if (tij < 0.0 && fabs(tij) > 1.0e-10) { set_err(sh, DMD_E_NEG_TIME, i); return false; }
    return true;
}

/* warp: full re-prediction of bead l at time tfalse */
__device__ void warp_redo_full(const DSys &S, SharedState &sh, int l, double tfalse, double interval_max, int hbonds) {
    int lane = threadIdx.x & 31;
    double H = interval_max + DMD_LTSTEP - tfalse;
    double bt = H;
    int bp = -1, by = -1;
    int n = S.upn[l];
    const int *up = S.up + (size_t)l * S.cap;
    for (int k = lane; k < n + 3; k += 32) {
        int m;
        int code;
        if (k < n) {
            m = up[k];
            code = pair_code(S, m, l, hbonds);
        } else {
            m = S.er[4 * l + (k - n)];
            if (m <= l) continue;
            code = pair_code(S, m, l, hbonds);
        }
        double tij; int ty;
        if (!d_predict(S, l, m, code, tfalse, tij, ty)) { set_err(sh, DMD_E_INPUT, code); continue; }
        check_tij(sh, tij, l, m);
        if (lex_less(tij, m, bt, bp)) { bt = tij; bp = m; by = ty; }
    }
    warp_lexmin(bt, bp, by);
    if (lane == 0) {
        double tn = bt + tfalse;
        S.tim[l] = tn;
        S.nptnr[l] = bp;
        S.colt[l] = (int8_t)by;
        S.queued[l] = tn < interval_max;
    }
    __syncwarp();
}

/* one lane: eventredo_down(l, src) */
__device__ void lane_redo_down(const DSys &S, SharedState &sh, int l, int src, double tfalse, double interval_max, int hbonds) {
    int code = pair_code(S, l, src, hbonds);
    double tij; int ty;
    if (!d_predict(S, l, src, code, tfalse, tij, ty)) { set_err(sh, DMD_E_INPUT, code); return; }
    check_tij(sh, tij, l, src);
    tij = tij + tfalse;
    if (lex_less(tij, src, S.tim[l], S.nptnr[l])) {
        S.tim[l] = tij;
        S.nptnr[l] = src;
        S.colt[l] = (int8_t)ty;
        S.queued[l] = tij < interval_max;
    }
}

/* warp: partial_events(i, j) after the pair (or ghost, j = -1) event */
__device__ void warp_partial_events(const DSys &S, SharedState &sh, int i, int j, double tfalse, double interval_max, int hbonds) {
    int lane = threadIdx.x & 31;
    warp_redo_full(S, sh, i, tfalse, interval_max, hbonds);
    if (j >= 0) warp_redo_full(S, sh, j, tfalse, interval_max, hbonds);
    /* the down-list operations in reference order */
    if (lane == 0) {
        int n = 0;
        const int *dn = S.dn + (size_t)i * S.cap;
        for (int k = 0; k < S.dnn[i] && n < OPS_MAX; ++k) { sh.ops_l[n] = dn[k]; sh.ops_s[n] = i; ++n; }
        for (int k = 0; k < 3 && n < OPS_MAX; ++k) {
            int l = S.er[4 * i + k];
            if (l >= 0 && l < i) { sh.ops_l[n] = l; sh.ops_s[n] = i; ++n; }
        }
        if (j >= 0) {
            const int *dj = S.dn + (size_t)j * S.cap;
            for (int k = 0; k < S.dnn[j] && n < OPS_MAX; ++k) {
                int l = dj[k];
                if (l != i) { sh.ops_l[n] = l; sh.ops_s[n] = j; ++n; }
            }
            for (int k = 0; k < 3 && n < OPS_MAX; ++k) {
                int l = S.er[4 * j + k];
                if (l >= 0 && l < j) { sh.ops_l[n] = l; sh.ops_s[n] = j; ++n; }
            }
        }
        sh.nops = n;
        sh.ntouched = 0;
    }
    __syncwarp();
    int nops = sh.nops;
    /* lanes walk the operations of distinct beads; a bead whose walk reaches
     * a full redo hands it to the whole warp */
    for (int base = 0; base < nops; base += 32) {
        int q = base + lane;
        bool leader = false;
        int l = -1, stop_at = -1;
        if (q < nops) {
            l = sh.ops_l[q];
            leader = true;
            for (int p = 0; p < q; ++p) if (sh.ops_l[p] == l) { leader = false; break; }
        }
        if (leader) {
            for (int p = q; p < nops; ++p) {
                if (sh.ops_l[p] != l) continue;
                int src = sh.ops_s[p];
                if (S.nptnr[l] != src) lane_redo_down(S, sh, l, src, tfalse, interval_max, hbonds);
                else { stop_at = p; break; }
            }
            int slot = atomicAdd(&sh.ntouched, 1);
            if (slot < OPS_MAX) sh.touched[slot] = l;
        }
        __syncwarp();
        unsigned pend = __ballot_sync(0xffffffffu, stop_at >= 0);
        while (pend) {
            int src_lane = __ffs(pend) - 1;
            pend &= pend - 1;
            int lb = __shfl_sync(0xffffffffu, l, src_lane);
            int p0 = __shfl_sync(0xffffffffu, stop_at, src_lane);
            /* operation p0 needs a full redo; continue this bead's walk */
            for (int p = p0; p < nops; ++p) {
                if (sh.ops_l[p] != lb) continue;
                int src = sh.ops_s[p];
                bool full = S.nptnr[lb] == src;
                __syncwarp();
                if (full) warp_redo_full(S, sh, lb, tfalse, interval_max, hbonds);
                else if (lane == 0) lane_redo_down(S, sh, lb, src, tfalse, interval_max, hbonds);
                __syncwarp();
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        int nt = sh.ntouched < OPS_MAX ? sh.ntouched : OPS_MAX;
        sh.touched[nt++] = i;
        if (j >= 0) sh.touched[nt++] = j;
        sh.ntouched = nt;
    }
    __syncwarp();
}

/* ------------------------------------------------------------------ */
/* H-bond bookkeeping (code/repuls_add.f, repuls_del_b.f, main.F90:825-868) */
/* ------------------------------------------------------------------ */
__device__ void ovr_set(const DSys &S, SharedState &sh, int a, int b, int code, int hbonds) {
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
    set_err(sh, DMD_E_CAPACITY, a);
}
__device__ void helpers_of(const DSys &S, int i, int j, int &ncim1, int &ncai, int &ncaj, int &nnjp1) {
    int Li = S.info[i].L, Lj = S.info[j].L;
    ncim1 = i + Li - 1; ncai = i - Li; ncaj = j - 2 * Lj; nnjp1 = j - Lj + 1;
}
__device__ void repuls_add(const DSys &S, SharedState &sh, int i, int j, int hbonds) {  /* i = NH, j = CO */
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, i, j, ncim1, ncai, ncaj, nnjp1);
    ovr_set(S, sh, ncaj, i, 50, hbonds); ovr_set(S, sh, i, ncaj, 40, hbonds);
    ovr_set(S, sh, i, nnjp1, 40, hbonds); ovr_set(S, sh, nnjp1, i, 50, hbonds);
    ovr_set(S, sh, ncai, j, 50, hbonds); ovr_set(S, sh, j, ncai, 40, hbonds);
    ovr_set(S, sh, j, ncim1, 40, hbonds); ovr_set(S, sh, ncim1, j, 50, hbonds);
    int *er = S.er;
    er[4 * i + 0] = ncaj; er[4 * i + 1] = nnjp1; er[4 * ncaj + 2] = i; er[4 * nnjp1 + 2] = i;
    er[4 * j + 0] = ncai; er[4 * j + 1] = ncim1; er[4 * ncai + 2] = j; er[4 * ncim1 + 2] = j;
    er[4 * i + 3] = j; er[4 * j + 3] = i;
}
__device__ void shoulders_off(const DSys &S, SharedState &sh, int n, int c, int hbonds) {
    int ncaj = S.er[4 * n + 0], nnjp1 = S.er[4 * n + 1], ncai = S.er[4 * c + 0], ncim1 = S.er[4 * c + 1];
    if (ncaj >= 0) { ovr_set(S, sh, ncaj, n, 1, hbonds); ovr_set(S, sh, n, ncaj, 1, hbonds); }
    if (nnjp1 >= 0) { ovr_set(S, sh, n, nnjp1, 1, hbonds); ovr_set(S, sh, nnjp1, n, 1, hbonds); }
    if (ncai >= 0) { ovr_set(S, sh, ncai, c, 1, hbonds); ovr_set(S, sh, c, ncai, 1, hbonds); }
    if (ncim1 >= 0) { ovr_set(S, sh, c, ncim1, 1, hbonds); ovr_set(S, sh, ncim1, c, 1, hbonds); }
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
/* collision dynamics (code/eventdyn.f, bumped.f, repuls_check*.f, check_sigma.f) */
/* ------------------------------------------------------------------ */
__device__ double dist_now(const DSys &S, int a, int b, double tfalse) {
    double vxa = S.vx[a] - S.vx[b], vya = S.vy[a] - S.vy[b], vza = S.vz[a] - S.vz[b];
    double rx = S.x[a] - S.x[b] + vxa * tfalse, ry = S.y[a] - S.y[b] + vya * tfalse, rz = S.z[a] - S.z[b] + vza * tfalse;
    rx = rx - d_nint(rx); ry = ry - d_nint(ry); rz = rz - d_nint(rz);
    double d = rx * rx + ry * ry + rz * rz;
    return sqrt(d);
}
__device__ double repuls_check(const DSys &S, int i, int j, double tfalse) {
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, i, j, ncim1, ncai, ncaj, nnjp1);
    const DTab &T = *S.tab;
    double d1 = dist_now(S, i, ncaj, tfalse), d2 = dist_now(S, i, nnjp1, tfalse);
    double d3 = dist_now(S, j, ncai, tfalse), d4 = dist_now(S, j, ncim1, tfalse);
    if ((d1 > T.shd1) && (d2 > T.shd2) && (d3 > T.shd3) && (d4 > T.shd4)) return 10.0;
    return 11.0;
}
__device__ double repuls_check_3(const DSys &S, int i, int j, int k, double tfalse) {
    int ncim1, ncai, ncaj, nnjp1;
    helpers_of(S, i, j, ncim1, ncai, ncaj, nnjp1);
    const DTab &T = *S.tab;
    int m = 0;
    double d1 = dist_now(S, i, ncaj, tfalse);
    if ((ncaj != k) && (d1 > T.shd1)) m = m + 1;
    double d2 = dist_now(S, i, nnjp1, tfalse);
    if ((nnjp1 != k) && (d2 > T.shd2)) m = m + 1;
    double d3 = dist_now(S, j, ncai, tfalse);
    if ((ncai != k) && (d3 > T.shd3)) m = m + 1;
    double d4 = dist_now(S, j, ncim1, tfalse);
    if ((ncim1 != k) && (d4 > T.shd4)) m = m + 1;
    return m == 3 ? 10.0 : 11.0;
}
__device__ double check_sigma(const DSys &S, int i, int j, double tfalse) {
    double vxa = S.vx[i] - S.vx[j], vya = S.vy[i] - S.vy[j], vza = S.vz[i] - S.vz[j];
    double rx = S.x[i] - S.x[j] + vxa * tfalse, ry = S.y[i] - S.y[j] + vya * tfalse, rz = S.z[i] - S.z[j] + vza * tfalse;
    rx = rx - d_nint(rx); ry = ry - d_nint(ry); rz = rz - d_nint(rz);
    double rijsq = rx * rx + ry * ry + rz * rz;
    double diff = rijsq - S.tab->sigma_sq[S.ident[i]][S.ident[j]];
    return diff < 0.0 ? 10.0 : 11.0;
}
__device__ void bump_in(const DSys &S, int i, int j, const Rel &r, double bd) {
    S.x[i] = S.x[i] - bd * r.rx; S.y[i] = S.y[i] - bd * r.ry; S.z[i] = S.z[i] - bd * r.rz;
    S.x[j] = S.x[j] + bd * r.rx; S.y[j] = S.y[j] + bd * r.ry; S.z[j] = S.z[j] + bd * r.rz;
}
__device__ void bump_out(const DSys &S, int i, int j, const Rel &r, double bd) {
    S.x[i] = S.x[i] + bd * r.rx; S.y[i] = S.y[i] + bd * r.ry; S.z[i] = S.z[i] + bd * r.rz;
    S.x[j] = S.x[j] - bd * r.rx; S.y[j] = S.y[j] - bd * r.ry; S.z[j] = S.z[j] - bd * r.rz;
}
__device__ int eventdyn(const DSys &S, int i, int j, int evcode, int ct, double tfalse) {
    const DTab &T = *S.tab;
    Rel r = d_rel(S, i, j, tfalse);
    double bij = r.bij;
    double bmi = S.bm[i], bmj = S.bm[j];
    double rmass = 2 * bmi * bmj / (bmi + bmj);
    int a = S.ident[i], b = S.ident[j];
    double ratio = 0.0;
    if (ct == 2) {
        double blmin, blmax; bond_limits(S, i, evcode, blmin, blmax);
        ratio = rmass * bij / (blmin * blmin);
    } else if (ct == 3) {
        double blmin, blmax; bond_limits(S, i, evcode, blmin, blmax);
        ratio = rmass * bij / (blmax * blmax);
    } else if (ct == 1) {
        double sigsq;
        if (evcode == 15) {
            if (S.bptnr[i] == j) { double p = T.evp1[evcode]; sigsq = T.sigma_sq[a][b] * (p * p); }
            else sigsq = T.sigma_sq[a][b];
        } else {
            double p = T.evp1[evcode];
            sigsq = T.sigma_sq[a][b] * (p * p);
            if (evcode >= 22 && evcode <= 26) {
                int k = a > b ? a : b;
                double s = T.sqz610[evcode - 21][k];
                sigsq = sigsq * (s * s);
            }
        }
        ratio = rmass * bij / sigsq;
    } else if (ct == 4) {
        double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
        double del_pe = 4.0 * wellsq * epsave / rmass;
        double bd = DMD_SMDIST * sqrt(wellsq);
        if (bij * bij + del_pe > 0.0) {
            ratio = rmass * (sqrt((4.0 * wellsq * epsave / rmass) + bij * bij) + bij) / (2.0 * wellsq);
            ct = 20; bump_in(S, i, j, r, bd);
        } else {
            ratio = rmass * bij / wellsq;
            ct = 22; bump_out(S, i, j, r, bd);
        }
    } else if (ct == 8) {
        double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
        double del_pe = 4.0 * wellsq * epsave / rmass;
        double bd = DMD_SMDIST * sqrt(wellsq);
        if (bij * bij > del_pe) {
            ratio = rmass * (-sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
            ct = 21; bump_out(S, i, j, r, bd);
        } else {
            ratio = rmass * bij / wellsq;
            ct = 22; bump_in(S, i, j, r, bd);
        }
    } else if (ct == 9) {
        double wellsq = T.welldia_sq[a][b];
        ratio = rmass * bij / wellsq;
        ct = 23; bump_out(S, i, j, r, DMD_SMDIST * sqrt(wellsq));
    } else if (ct == 5) {
        double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
        double del_pe = 4.0 * wellsq * epsave / rmass;
        double bd = DMD_SMDIST * sqrt(wellsq);
        ratio = rmass * (-sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
        ct = 24; bump_out(S, i, j, r, bd);
    } else if (ct == 6) {
        double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
        double del_pe = 4.0 * wellsq * epsave / rmass;
        double bd = DMD_SMDIST * sqrt(wellsq);
        if (bij * bij > -del_pe) {
            ratio = rmass * (sqrt(del_pe + bij * bij) + bij) / (2.0 * wellsq);
            ct = 25; bump_in(S, i, j, r, bd);
        } else {
            ratio = rmass * bij / wellsq;
            ct = 26; bump_out(S, i, j, r, bd);
        }
    } else if (ct == 13) {
        double wellsq = T.shlddia_sq[a][b];
        ratio = rmass * bij / wellsq;
        ct = 27; bump_out(S, i, j, r, DMD_SMDIST * sqrt(wellsq));
    }
    double delvx = ratio * r.rx, delvy = ratio * r.ry, delvz = ratio * r.rz;
    S.vx[i] = S.vx[i] - delvx / bmi; S.vx[j] = S.vx[j] + delvx / bmj;
    S.vy[i] = S.vy[i] - delvy / bmi; S.vy[j] = S.vy[j] + delvy / bmj;
    S.vz[i] = S.vz[i] - delvz / bmi; S.vz[j] = S.vz[j] + delvz / bmj;
    S.x[i] = S.x[i] + delvx * tfalse / bmi;
    S.y[i] = S.y[i] + delvy * tfalse / bmi;
    S.z[i] = S.z[i] + delvz * tfalse / bmi;
    S.x[j] = S.x[j] - delvx * tfalse / bmj;
    S.y[j] = S.y[j] - delvy * tfalse / bmj;
    S.z[j] = S.z[j] - delvz * tfalse / bmj;
    return ct;
}
__device__ void bumpoff(const DSys &S, int i, int j, int evcode, double tfalse) {
    Rel r = d_rel(S, i, j, tfalse);
    const DTab &T = *S.tab;
    double bd = (evcode >= 40) ? DMD_SMDIST * sqrt(T.shlddia_sq[S.ident[i]][S.ident[j]])
                               : DMD_SMDIST * sqrt(T.welldia_sq[S.ident[i]][S.ident[j]]);
    if (r.bij < 0.0) bump_in(S, i, j, r, bd); else bump_out(S, i, j, r, bd);
}

/* one lane: worker block (code/main.F90:1432-1956) and master application
 * (code/main.F90:646-943) of the pair event (i, j); returns the final
 * coltype and whether the shoulder links must be cleared afterwards */
__device__ int lane_pair_event(const DSys &S, SharedState &sh, int i, int j, long long coll, double tfalse,
                               int hbonds, int &xpulse_del, int &evcode_out) {
    int8_t *id = S.ident;
    int *er = S.er;
    int ct = S.colt[i];
    int evcode = pair_code(S, i, j, hbonds);
    evcode_out = evcode;
    bool nonend = !S.info[i].is_end && !S.info[j].is_end;
    xpulse_del = 0;
    int nb = id[i] < id[j] ? i : j;
    int cb = id[i] < id[j] ? j : i;
    if (ct == 7) {
        if (er[4 * i + 3] < 0 && er[4 * j + 3] < 0) {
            if (nonend) {
                ct = repuls_check(S, nb, cb, tfalse) <= 10.0 ? 4 : 14;
            } else {
                double ran_non = dmd_uniform(S.seed, DMD_STREAM_CAPTURE, (uint64_t)coll, 0);
                ct = ran_non <= 0.2 ? 4 : 9;
            }
        } else {
            ct = 9;
        }
    } else if (ct == 10) {
        double rating;
        int hbchk = evcode < 45 ? er[4 * i + 3] : er[4 * j + 3];
        if (hbchk < 0) { set_err(sh, DMD_E_STATE, i); return ct; }
        if (evcode < 45) {
            int hb = er[4 * i + 3];
            rating = id[i] < id[hb] ? repuls_check_3(S, i, hb, j, tfalse) : repuls_check_3(S, hb, i, j, tfalse);
        } else {
            int hb = er[4 * j + 3];
            rating = id[j] < id[hb] ? repuls_check_3(S, j, hb, i, tfalse) : repuls_check_3(S, hb, j, i, tfalse);
        }
        ct = rating <= 10.0 ? 5 : 15;
    } else if (ct == 12) {
        int hbchk = evcode < 45 ? er[4 * i + 3] : er[4 * j + 3];
        if (hbchk < 0) { set_err(sh, DMD_E_STATE, i); return ct; }
        if (evcode < 45) {
            int hb = er[4 * i + 3];
            if (S.bptnr[i] == hb) ct = check_sigma(S, i, hb, tfalse) > 10.0 ? 6 : 13; else ct = 15;
        } else {
            int hb = er[4 * j + 3];
            if (S.bptnr[j] == hb) ct = check_sigma(S, j, hb, tfalse) > 10.0 ? 6 : 13; else ct = 15;
        }
    }
    if (ct < 14) ct = eventdyn(S, i, j, evcode, ct, tfalse);
    if (ct == 24 || ct == 25) {
        int hbchk = evcode < 45 ? er[4 * i + 3] : er[4 * j + 3];
        if (hbchk < 0) { set_err(sh, DMD_E_STATE, i); return ct; }
    }
    if (ct == 20) {
        if (id[i] + id[j] == 5) {
            S.bptnr[i] = j; S.bptnr[j] = i;
            id[i] = id[i] + 4; id[j] = id[j] + 4;
            if (nonend) { if (id[i] < id[j]) repuls_add(S, sh, i, j, hbonds); else repuls_add(S, sh, j, i, hbonds); }
        }
    } else if (ct == 21) {
        if (id[i] <= 8) {
            if (nonend) {
                xpulse_del = 1;
                if (id[i] < id[j]) shoulders_off(S, sh, i, j, hbonds); else shoulders_off(S, sh, j, i, hbonds);
            }
            if (S.bptnr[i] == j) {
                S.bptnr[i] = -1; S.bptnr[j] = -1;
                id[i] = id[i] - 4; id[j] = id[j] - 4;
            }
        }
    } else if (ct == 24) {
        if (evcode < 45) {
            int hb = er[4 * i + 3];
            if (id[i] + id[hb] == 5) { S.bptnr[i] = hb; S.bptnr[hb] = i; id[i] += 4; id[hb] += 4; }
        } else {
            int hb = er[4 * j + 3];
            if (id[j] + id[hb] == 5) { S.bptnr[j] = hb; S.bptnr[hb] = j; id[j] += 4; id[hb] += 4; }
        }
    } else if (ct == 25) {
        if (evcode < 45) {
            int hb = er[4 * i + 3];
            if (id[i] >= 5) { S.bptnr[i] = -1; S.bptnr[hb] = -1; id[i] -= 4; id[hb] -= 4; }
        } else {
            int hb = er[4 * j + 3];
            if (id[j] >= 5) { S.bptnr[j] = -1; S.bptnr[hb] = -1; id[j] -= 4; id[hb] -= 4; }
        }
    } else if (ct == 14) {
        bumpoff(S, i, j, evcode, tfalse);
        if (nonend) { if (id[i] < id[j]) repuls_add(S, sh, i, j, hbonds); else repuls_add(S, sh, j, i, hbonds); }
    } else if (ct == 15) {
        bumpoff(S, i, j, evcode, tfalse);
    } else if (ct == 16) {
        bumpoff(S, i, j, evcode, tfalse);
        if (nonend) {
            xpulse_del = 1;
            if (id[i] < id[j]) shoulders_off(S, sh, i, j, hbonds); else shoulders_off(S, sh, j, i, hbonds);
        }
    }
    S.colt[i] = (int8_t)ct;
    return ct;
}

/* one lane: Andersen ghost collision (code/main.F90:997-1121) up to the
 * re-prediction; returns the bead */
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
    if (i > N || r == 0.0 || r >= 1.0 || tgho < 1e-18) set_err(sh, DMD_E_STATE, -1);
    double tn = -1.0 * dmd_log(tgho) * T.avegtime + tfalse;
    S.tim[N] = tn;
    S.queued[N] = tn < sh.sc.interval_max;
    if (tfalse < sh.sc.old_tfalse) tfalse = sh.sc.old_tfalse;
    return i;
}

/* ------------------------------------------------------------------ */
/* CTA-wide: block reductions                                          */
/* ------------------------------------------------------------------ */
__device__ double cta_max(SharedState &sh, double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
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
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
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
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
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
__device__ __forceinline__ int cell_coord(double p, int nc) {
    double c = (p + 0.5) * nc;
    if (!(c >= 0.0)) return 0;   /* also catches NaN */
    int k = (int)c;
    return k < nc ? k : nc - 1;
}
/* ------------------------------------------------------------------ */
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
        /* exclusive scan of the counts: each thread a contiguous chunk */
        {
            int per = (ncell3 + blockDim.x - 1) / blockDim.x;
            int lo = threadIdx.x * per, hi = min(lo + per, ncell3);
            int s = 0;
            for (int c = lo; c < hi; ++c) s += S.cell_count[c];
            int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
            int incl = s;
            for (int o = 1; o < 32; o <<= 1) { int v = __shfl_up_sync(0xffffffffu, incl, o); if (lane >= o) incl += v; }
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
        auto consider = [&](int c) {
            if (c == b) return;
            int code = pair_code(S, c, b, hbonds);
            bool take;
            if ((code >= 4 && code <= 12) || (code >= 17 && code < 27)) take = true;
            else {
                double rx = xb - S.x[c], ry = yb - S.y[c], rz = zb - S.z[c];
                rx = rx - d_nint(rx); ry = ry - d_nint(ry); rz = rz - d_nint(rz);
                double r2 = rx * rx + ry * ry + rz * rz;
                take = r2 <= T.rlsq[code];
            }
            if (!take) return;
            if (c > b) {
                if (nu < S.cap) { up[nu] = c; upc[nu] = (int8_t)static_code(ib, S.info[c], hbonds); }
                ++nu;
            } else {
                if (nd < S.cap) dn[nd] = c;
                ++nd;
            }
        };
        if (nc >= 3) {
            int cx = cell_coord(xb, nc), cy = cell_coord(yb, nc), cz = cell_coord(zb, nc);
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int gx = (cx + dx + nc) % nc, gy = (cy + dy + nc) % nc, gz = (cz + dz + nc) % nc;
                        int c0 = (gz * nc + gy) * nc + gx;
                        for (int q = S.cell_start[c0]; q < S.cell_start[c0 + 1]; ++q) consider(S.cell_beads[q]);
                    }
        } else {
            for (int c = 0; c < N; ++c) consider(c);
        }
        if (nu > S.cap || nd > S.cap) set_err(sh, DMD_E_CAPACITY, b);
        S.upn[b] = min(nu, S.cap);
        S.dnn[b] = min(nd, S.cap);
    }
    __syncthreads();
}

/* events(): every bead over its up list and extras (code/events.f:23-123) */
__device__ void cta_predict_all(const DSys &S, SharedState &sh, double interval_max, int hbonds) {
    const int N = S.N;
    for (int b = threadIdx.x; b < N; b += blockDim.x) {
        double bt = interval_max + DMD_LTSTEP;
        int bp = -1, by = -1;
        const int *up = S.up + (size_t)b * S.cap;
        for (int k = 0; k < S.upn[b]; ++k) {
            int m = up[k];
            double tij; int ty;
            int code = pair_code(S, m, b, hbonds);
            if (!d_predict(S, b, m, code, 0.0, tij, ty)) { set_err(sh, DMD_E_INPUT, code); continue; }
            check_tij(sh, tij, b, m);
            if (lex_less(tij, m, bt, bp)) { bt = tij; bp = m; by = ty; }
        }
        for (int k = 0; k < 3; ++k) {
            int m = S.er[4 * b + k];
            if (m > b) {
                double tij; int ty;
                int code = pair_code(S, m, b, hbonds);
                if (!d_predict(S, b, m, code, 0.0, tij, ty)) { set_err(sh, DMD_E_INPUT, code); continue; }
                check_tij(sh, tij, b, m);
                if (lex_less(tij, m, bt, bp)) { bt = tij; bp = m; by = ty; }
            }
        }
        S.tim[b] = bt; S.nptnr[b] = bp; S.colt[b] = (int8_t)by;
        S.queued[b] = bt < interval_max;
    }
    if (threadIdx.x < 3) S.queued[N + threadIdx.x] = S.tim[N + threadIdx.x] < interval_max;
    __syncthreads();
}

__device__ void cta_rebuild(const DSys &S, SharedState &sh, int hbonds) {
    for (int b = threadIdx.x; b < S.N; b += blockDim.x) {
        double px = S.x[b], py = S.y[b], pz = S.z[b];
        px = px - d_nint(px); py = py - d_nint(py); pz = pz - d_nint(pz);
        S.x[b] = px; S.y[b] = py; S.z[b] = pz;
        S.ox[b] = px; S.oy[b] = py; S.oz[b] = pz;
    }
    __syncthreads();
    cta_build_lists(S, sh, hbonds);
    cta_predict_all(S, sh, sh.sc.interval_max, hbonds);
    cta_tree_rebuild(S);
}

/* interval event N+2 (code/main.F90:1126-1187, code/displ.f) */
__device__ bool cta_interval(const DSys &S, SharedState &sh, int hbonds) {
    const int N = S.N;
    double tf = sh.sc.tfalse;
    const DTab &T = *S.tab;
    __syncthreads();
    for (int k = threadIdx.x; k < N + 3; k += blockDim.x) S.tim[k] = S.tim[k] - tf;
    double moved_far = 0.0;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        double px = S.x[k] + S.vx[k] * tf, py = S.y[k] + S.vy[k] * tf, pz = S.z[k] + S.vz[k] * tf;
        S.x[k] = px; S.y[k] = py; S.z[k] = pz;
        double a = S.ox[k] - px, b = S.oy[k] - py, c = S.oz[k] - pz;
        double dis = a * a + b * b + c * c;
        double moved = dis / T.hdelr;
        if (moved > moved_far) moved_far = moved;
    }
    moved_far = cta_max(sh, moved_far);
    if (threadIdx.x == 0) {
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
    __syncthreads();
    bool rb = sh.rebuild != 0;
    if (rb) {
        for (int k = threadIdx.x; k < N; k += blockDim.x) { S.tim[k] = sh.sc.interval_max + DMD_LTSTEP; S.colt[k] = -1; S.nptnr[k] = -1; }
        __syncthreads();
        cta_rebuild(S, sh, hbonds);
    }
    if (threadIdx.x == 0) {
        S.tim[N + 1] = sh.sc.interval * 0.999;
        S.queued[N + 1] = 1;
    }
    __syncthreads();
    cta_tree_rebuild(S);
    return rb;
}

/* diagnostics (code/energy.f:1-105, radgyr.f:1-139, end2end.f:1-48) over the
 * neighbour lists; done by the whole CTA */
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
    }
    __syncthreads();
}

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */
__device__ void log_event(const DSys &S, SharedState &sh, double t, double tfalse, int i, int j, int type, int evcode) {
    if (!S.log || S.log_cap <= 0) return;
    long long k = sh.sc.log_count++;
    dmd_event *L = (dmd_event *)S.log + (k % S.log_cap);
    L->coll = sh.sc.coll; L->t = t; L->tfalse = tfalse;
    L->i = i + 1; L->j = j + 1; L->type = type; L->evcode = evcode;
}

__global__ void __launch_bounds__(NTHREADS) k_init(DSys *systems, int nsys, int hbonds_mask) {
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    int r = blockIdx.x;
    if (r >= nsys) return;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    const DSys &S = S_sh;
    int hbonds = (hbonds_mask >> 0) & 1;
    if (threadIdx.x == 0) { sh.sc = *S.sc; }
    __syncthreads();
    cta_rebuild(S, sh, hbonds);
    if (threadIdx.x == 0) *S.sc = sh.sc;
}

__global__ void __launch_bounds__(NTHREADS) k_run(DSys *systems, int nsys, long long target, int hbonds_mask,
                                                  const int *chain_start, const int *chain_len,
                                                  const int *chain_off, dmd_diag *outputs) {
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    int r = blockIdx.x;
    if (r >= nsys) return;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    const DSys &S = S_sh;
    const int N = S.N;
    const int hbonds = hbonds_mask & 1;
    const bool phys = (S.flags & DMD_FLAG_COUNT_PHYSICAL) != 0;
    const bool stop_out = (S.flags & DMD_FLAG_STOP_AT_OUTPUT) != 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) { sh.sc = *S.sc; sh.sc.done = 0; sh.sc.stop = 0; }
    __syncthreads();
    const int *cs = chain_start + chain_off[r], *cl = chain_len + chain_off[r];
    /* every committed pair or ghost event advances done; interval and output
     * events are bounded by this cap so that a launch always ends */
    const long long max_iter = 16 * target + 1000000;
    long long iter = 0;
    while (true) {
        if (sh.sc.done >= target || sh.sc.err || sh.sc.stop) break;
        if (++iter > max_iter) {
            if (threadIdx.x == 0) set_err(sh, DMD_E_DEVICE_TIMEOUT, 0);
            __syncthreads();
            break;
        }
        if (warp == 0) {
            int e = warp_tree_root(S);
            if (lane == 0) {
                sh.ev = e;
                if (e < 0) set_err(sh, DMD_E_STATE, 0);
                else {
                    sh.sc.coll += 1;
                    sh.sc.tfalse = S.tim[e];
                }
            }
        }
        __syncthreads();
        int e = sh.ev;
        if (e < 0) break;
        if (e < N) {
            if (warp == 0) {
                double tf = sh.sc.tfalse;
                int j = S.nptnr[e];
                if (lane == 0) {
                    int xp, evc;
                    int ct = lane_pair_event(S, sh, e, j, sh.sc.coll, tf, hbonds, xp, evc);
                    if (ct >= 1 && ct < 32) sh.sc.nevents[ct] += 1;
                    sh.sc.n_pair += 1;
                    sh.xpulse = xp;
                    log_event(S, sh, sh.sc.t, tf, e, j, ct, evc);
                }
                __syncwarp();
                warp_partial_events(S, sh, e, j, tf, sh.sc.interval_max, hbonds);
                if (lane == 0 && sh.xpulse) {
                    if (S.ident[e] < S.ident[j]) repuls_del_b(S, e, j); else repuls_del_b(S, j, e);
                }
                __syncwarp();
                warp_tree_update(S, sh.touched, sh.ntouched);
                if (lane == 0) { sh.sc.old_tfalse = tf; sh.sc.done += 1; }
            }
        } else if (e == N) {
            if (warp == 0) {
                double tf = sh.sc.tfalse;
                int i = 0;
                if (lane == 0) {
                    i = lane_ghost(S, sh, tf);
                    sh.sc.tfalse = tf;
                    sh.ev_i = i;
                }
                __syncwarp();
                i = sh.ev_i;
                tf = sh.sc.tfalse;
                warp_partial_events(S, sh, i, -1, tf, sh.sc.interval_max, hbonds);
                if (lane == 0) {
                    int nt = sh.ntouched;
                    sh.touched[nt++] = N;
                    sh.ntouched = nt;
                }
                __syncwarp();
                warp_tree_update(S, sh.touched, sh.ntouched);
                if (lane == 0) {
                    log_event(S, sh, sh.sc.t, tf, i, -1, DMD_EV_GHOST, 0);
                    sh.sc.old_tfalse = tf;
                    sh.sc.done += 1;
                }
            }
        } else if (e == N + 1) {
            double t_before = sh.sc.t, tf = sh.sc.tfalse;
            bool rb = cta_interval(S, sh, hbonds);
            if (threadIdx.x == 0) {
                sh.sc.n_interval += 1;
                log_event(S, sh, t_before, tf, N + 1, -1, rb ? DMD_EV_REBUILD : DMD_EV_INTERVAL, 0);
                sh.sc.old_tfalse = sh.sc.tfalse;
                if (!phys) sh.sc.done += 1;
            }
        } else {
            cta_diag(S, sh, cs, cl, outputs ? outputs + r : nullptr);
            if (threadIdx.x == 0) {
                sh.sc.n_output += 1;
                double tn = 3.3 / (sqrt(S.tab->setemp)) + 5 + sh.sc.tfalse;
                S.tim[N + 2] = tn;
                S.queued[N + 2] = tn < sh.sc.interval_max;
                log_event(S, sh, sh.sc.t, sh.sc.tfalse, N + 2, -1, DMD_EV_OUTPUT, 0);
                sh.sc.old_tfalse = sh.sc.tfalse;
                if (!phys) sh.sc.done += 1;
                if (stop_out) sh.sc.stop = 1;
                sh.touched[0] = N + 2;
            }
            __syncthreads();
            if (warp == 0) warp_tree_update(S, sh.touched, 1);
        }
        __syncthreads();
    }
    __syncthreads();
    if (threadIdx.x == 0) *S.sc = sh.sc;
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
cudaError_t dmd_launch_init(DSys *d_systems, int nsys, int hbonds, cudaStream_t st) {
    k_init<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, hbonds);
    return cudaGetLastError();
}
cudaError_t dmd_launch_run(DSys *d_systems, int nsys, long long target, int hbonds, const int *chain_start,
                           const int *chain_len, const int *chain_off, dmd_diag *outputs, cudaStream_t st) {
    k_run<<<nsys, NTHREADS, 0, st>>>(d_systems, nsys, target, hbonds, chain_start, chain_len, chain_off, outputs);
    return cudaGetLastError();
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

__global__ void __launch_bounds__(NTHREADS) k_predict_noalloc(DSys S_in, int hbonds, double *tim_out,
                                                              int *nptnr_out, int *colt_out) {
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    if (threadIdx.x == 0) { S_sh = S_in; sh.sc = *S_in.sc; }
    __syncthreads();
    const DSys &S = S_sh;
    cta_rebuild(S, sh, hbonds);
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
