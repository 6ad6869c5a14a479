/*
 * engine_run.cuh -- the event loop kernel k_run and its per-event warp
 * functions (collision, re-prediction, footprint claims).
 *
 * engine.cu includes this file twice, inside namespaces run_full and
 * run_compact, after defining
 *   DMD_RUN_OPS       capacity of the per-warp down-list operation arrays,
 *   DMD_RUN_RSET/QSET capacities of the footprint read and queue sets,
 *   DMD_RUN_DN_LIMIT  the longest down list the variant accepts.
 * Everything else (tables, predictors, lists, intervals, diagnostics) is
 * shared and defined before the inclusion.
 */
constexpr int OPS_MAX = DMD_RUN_OPS;
constexpr int RSET_MAX = DMD_RUN_RSET;
constexpr int QSET_MAX = DMD_RUN_QSET;
constexpr int DN_LIMIT = DMD_RUN_DN_LIMIT;
constexpr int RUN_NT = DMD_RUN_NT;          /* threads per CTA of this variant */
constexpr int RUN_NW = RUN_NT / 32;
static_assert(RUN_NW <= NWARPS_MAX && RUN_NW <= CAND_MAX, "warps per CTA");
static_assert(OPS_MAX >= 2 * (DN_LIMIT < 128 ? DN_LIMIT : 128) + 6, "down-list operations of one event must fit");

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
    double big_tf;                /* DMD_BIG + tf: a down operation's time when it has no event */
    long long tnew_key;
    int tnew_idx;
};

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
    /* three independent sums on three lanes (operands selected first, so
     * that the warp issues two additions, not six), then broadcast */
    const double s0 = lane == 0 ? b0 : (lane == 1 ? r0 : v0);
    const double s1 = lane == 0 ? b1 : (lane == 1 ? r1 : v1);
    const double s2 = lane == 0 ? b2 : (lane == 1 ? r2 : v2);
    double s = s0 + s1 + s2;
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
            if (evcode == 15) {
                const bool hb = S.bptnr[i] == j;
                ratio = div_by(rmass * bij, hb ? T.core15_sq[a][b] : T.sigma_sq[a][b],
                               hb ? T.rcore15_sq[a][b] : T.rsigma_sq[a][b]);
            } else if (evcode <= 3 || (evcode >= 17 && evcode <= 26)) {
                const int sl = core_slot_d(evcode);
                ratio = div_by(rmass * bij, T.core_sq[sl][a][b], T.rcore_sq[sl][a][b]);
            } else {
                /* the other codes with a core (16: inside a hydrophobic well;
                 * 40/50: under a shoulder): eventdyn.f's sigma_sq *
                 * ev_param(1,code)**2 with ev_param(1,code) = 1, which is
                 * sigma_sq */
                ratio = div_by(rmass * bij, T.sigma_sq[a][b], T.rsigma_sq[a][b]);
            }
        } else if (ct == 4) {
            double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
            double del_pe = div_by(4.0 * wellsq * epsave, rmass, T.rrmass[a][b]);
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij + del_pe > 0.0) {
                /* the reference recomputes del_pe here: the same value */
                ratio = div_by(rmass * (sqrt(del_pe + bij * bij) + bij), 2.0 * wellsq, T.r2well_sq[a][b]);
                ct = 20; bump = -1;
            } else {
                ratio = div_by(rmass * bij, wellsq, T.rwell_sq[a][b]);
                ct = 22; bump = 1;
            }
        } else if (ct == 8) {
            double wellsq = T.welldia_sq[a][b], epsave = T.ep_sqrt[a][b];
            double del_pe = div_by(4.0 * wellsq * epsave, rmass, T.rrmass[a][b]);
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij > del_pe) {
                ratio = div_by(rmass * (-sqrt(-del_pe + bij * bij) + bij), 2.0 * wellsq, T.r2well_sq[a][b]);
                ct = 21; bump = 1;
            } else {
                ratio = div_by(rmass * bij, wellsq, T.rwell_sq[a][b]);
                ct = 22; bump = -1;
            }
        } else if (ct == 9) {
            double wellsq = T.welldia_sq[a][b];
            ratio = div_by(rmass * bij, wellsq, T.rwell_sq[a][b]);
            ct = 23; bump = 1; bd = DMD_SMDIST * sqrt(wellsq);
        } else if (ct == 5) {
            double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
            double del_pe = div_by(4.0 * wellsq * epsave, rmass, T.rrmass[a][b]);
            bd = DMD_SMDIST * sqrt(wellsq);
            ratio = div_by(rmass * (-sqrt(-del_pe + bij * bij) + bij), 2.0 * wellsq, T.r2shld_sq[a][b]);
            ct = 24; bump = 1;
        } else if (ct == 6) {
            double wellsq = T.shlddia_sq[a][b], epsave = -T.eps1;
            double del_pe = div_by(4.0 * wellsq * epsave, rmass, T.rrmass[a][b]);
            bd = DMD_SMDIST * sqrt(wellsq);
            if (bij * bij > -del_pe) {
                ratio = div_by(rmass * (sqrt(del_pe + bij * bij) + bij), 2.0 * wellsq, T.r2shld_sq[a][b]);
                ct = 25; bump = -1;
            } else {
                ratio = div_by(rmass * bij, wellsq, T.rshld_sq[a][b]);
                ct = 26; bump = 1;
            }
        } else if (ct == 13) {
            double wellsq = T.shlddia_sq[a][b];
            ratio = div_by(rmass * bij, wellsq, T.rshld_sq[a][b]);
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
    double bmi = S.bm[i], rbmi = T.rbm[S.ident[i]];   /* bm(i) = mass(identity(i)) */
    do {
        v1 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        v2 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        r = v1 * v1 + v2 * v2;
    } while (((r == 0.0) || (r >= 1.0)) && k < 4096);
    double fact = sqrt(-2.0 * T.setemp * bmi * dmd_log(r) / r);
    S.vx[i] = div_by(v1 * fact, bmi, rbmi);
    S.vy[i] = div_by(v2 * fact, bmi, rbmi);
    do {
        v1 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        v2 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, (uint64_t)g, k++) - 1.0;
        r = v1 * v1 + v2 * v2;
    } while (((r == 0.0) || (r >= 1.0)) && k < 8192);
    fact = sqrt(-2.0 * T.setemp * bmi * dmd_log(r) / r);
    S.vz[i] = div_by(v1 * fact, bmi, rbmi);
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
/* The collision of an event of a light batch (coltype 1-3: core bounce,
 * inner or outer bond wall) on one half of a warp, the other half taking
 * another event (or none: has = false, no writes): every FP64 warp
 * instruction serves two events.  The same arithmetic as warp_snapshot,
 * warp_collision, warp_eventdyn, warp_rel and warp_impulse for those
 * coltypes: components on lanes 0..2 (0..5) of the half, the impulse ratio
 * on its lane 0. */
__device__ void hw_collision_light(const DSys &S, WarpArea &W, bool has, int i, int j, double tf, int hbonds) {
    const int lane = threadIdx.x & 31, hl = lane & 15;
    const unsigned hbase = lane & 16;          /* first lane of this half */
    const DTab &T = *S.tab;
    /* Two rounds of loads.  The first holds every load that needs only i
     * and j: lanes 0..11 of the half the positions and velocities of i
     * (0..5) and j (6..11), which are also the snapshot of what the
     * collision writes; lane 0 the coltype, identities, masses, bond
     * windows and everything the pair code is made of (the overrides of i
     * and both bead records, taken whether or not an override applies).
     * The second, on lane 0, the tables indexed by the identities and the
     * pair code. */
    DMD_CSUB(-1);
    const int fb = hl < 6 ? i : j, ff = hl % 6;
    const double *A = ff == 0 ? S.x : ff == 1 ? S.y : ff == 2 ? S.z : ff == 3 ? S.vx : ff == 4 ? S.vy : S.vz;
    const double mine = hl < 12 ? A[fb] : 0.0;
    int ct = 0, evcode = 0;
    double rm = 0.0, R = 1.0, rR = 1.0, bmi = 0.0, bmj = 0.0, rbmi = 0.0, rbmj = 0.0;
    if (hl == 0) {
        ct = S.colt[i];
        const int a = S.ident[i], b = S.ident[j];
        const int o0 = S.ovp[4 * i], o1 = S.ovp[4 * i + 1], o2 = S.ovp[4 * i + 2], o3 = S.ovp[4 * i + 3];
        const int c0 = S.ovc[4 * i], c1 = S.ovc[4 * i + 1], c2 = S.ovc[4 * i + 2], c3 = S.ovc[4 * i + 3];
        const BeadInfo ia = S.info[i], ib = S.info[j];
        bmi = S.bm[i]; bmj = S.bm[j];
        const double lo_s = S.blmin_sq[i], rlo_s = S.rblmin_sq[i], hi_s = S.blmax_sq[i], rhi_s = S.rblmax_sq[i];
        const int bp = S.bptnr[i];
        /* pair_code(): the first override slot holding j, else the rule */
        evcode = o0 == j ? c0 : o1 == j ? c1 : o2 == j ? c2 : o3 == j ? c3 : static_code(ia, ib, hbonds);
        /* second round: the reduced mass, the reciprocal masses and the
         * squared diameter of the wall met (warp_eventdyn, coltypes 1-3) */
        rm = T.rmass[a][b];
        rbmi = T.rbm[a]; rbmj = T.rbm[b];   /* bm(b) = mass(identity(b)) */
        const bool side = evcode >= 10 && evcode <= 12;
        if (ct == 2) {
            R = side ? lo_s : T.evp2_sq[evcode];
            rR = side ? rlo_s : T.revp2_sq[evcode];
        } else if (ct == 3) {
            R = side ? hi_s : T.evp3_sq[evcode];
            rR = side ? rhi_s : T.revp3_sq[evcode];
        } else if (ct == 1) {
            if (evcode == 15) {
                const bool hb = bp == j;
                R = hb ? T.core15_sq[a][b] : T.sigma_sq[a][b];
                rR = hb ? T.rcore15_sq[a][b] : T.rsigma_sq[a][b];
            } else if (evcode <= 3 || (evcode >= 17 && evcode <= 26)) {
                const int sl = core_slot_d(evcode);
                R = T.core_sq[sl][a][b];
                rR = T.rcore_sq[sl][a][b];
            } else {
                /* the other codes with a core (16: inside a hydrophobic well;
                 * 40/50: under a shoulder): eventdyn.f's sigma_sq *
                 * ev_param(1,code)**2 with ev_param(1,code) = 1, which is
                 * sigma_sq */
                R = T.sigma_sq[a][b];
                rR = T.rsigma_sq[a][b];
            }
        }
    }
    if (has && hl < 12) W.sij[hl] = mine;
    if (has && hl == 0) { W.nmeta = 0; W.colt_i = (int8_t)ct; }
    DMD_CSUB(4);
    /* relative position and velocity (warp_rel), lanes 0..2 of the half */
    const int d = hl % 3;
    const double xi = __shfl_sync(FULL, mine, hbase + d), vi = __shfl_sync(FULL, mine, hbase + 3 + d);
    const double xj = __shfl_sync(FULL, mine, hbase + 6 + d), vj = __shfl_sync(FULL, mine, hbase + 9 + d);
    DMD_CSUB(0);
    const double v = vi - vj;
    double r = xi - xj + v * tf;
    r = d_wrap(r);
    const double pb = r * v, pr = r * r, pv = v * v;
    const double rx = __shfl_sync(FULL, r, 0, 16), ry = __shfl_sync(FULL, r, 1, 16), rz = __shfl_sync(FULL, r, 2, 16);
    const double b0 = __shfl_sync(FULL, pb, 0, 16), b1 = __shfl_sync(FULL, pb, 1, 16), b2 = __shfl_sync(FULL, pb, 2, 16);
    const double r0 = __shfl_sync(FULL, pr, 0, 16), r1 = __shfl_sync(FULL, pr, 1, 16), r2 = __shfl_sync(FULL, pr, 2, 16);
    const double v0 = __shfl_sync(FULL, pv, 0, 16), v1 = __shfl_sync(FULL, pv, 1, 16), v2 = __shfl_sync(FULL, pv, 2, 16);
    const double s0 = hl == 0 ? b0 : (hl == 1 ? r0 : v0);
    const double s1 = hl == 0 ? b1 : (hl == 1 ? r1 : v1);
    const double s2 = hl == 0 ? b2 : (hl == 1 ? r2 : v2);
    const double sum = s0 + s1 + s2;
    const double bij = __shfl_sync(FULL, sum, 0, 16);
    DMD_CSUB(1);
    /* the impulse ratio (warp_eventdyn, coltypes 1-3) on lane 0 of the half */
    double ratio = 0.0;
    if (hl == 0 && ct >= 1 && ct <= 3) ratio = div_by(rm * bij, R, rR);
    ratio = __shfl_sync(FULL, ratio, 0, 16);
    const double bm_i = __shfl_sync(FULL, bmi, 0, 16), bm_j = __shfl_sync(FULL, bmj, 0, 16);
    const double rbm_i = __shfl_sync(FULL, rbmi, 0, 16), rbm_j = __shfl_sync(FULL, rbmj, 0, 16);
    ct = __shfl_sync(FULL, ct, 0, 16);
    evcode = __shfl_sync(FULL, evcode, 0, 16);
    DMD_CSUB(2);
    /* the impulse (warp_impulse without a bump), lanes 0..5 of the half;
     * the position and velocity are the values held above (lanes 0..5:
     * position of component dd, lanes 3..5 of i hold velocities, so the
     * component's position of b comes from lane (isj ? 6 : 0) + dd and its
     * velocity from lane (isj ? 9 : 3) + dd) */
    const int dd = hl % 3;
    const bool isj = hl >= 3;
    const double pcur = __shfl_sync(FULL, mine, hbase + (isj ? 6 : 0) + dd);
    const double vcur = __shfl_sync(FULL, mine, hbase + (isj ? 9 : 3) + dd);
    if (has && hl < 6) {
        const int bb = isj ? j : i;
        double *PP = dd == 0 ? S.x : (dd == 1 ? S.y : S.z);
        double *VV = dd == 0 ? S.vx : (dd == 1 ? S.vy : S.vz);
        const double rr = dd == 0 ? rx : (dd == 1 ? ry : rz);
        const double bmb = isj ? bm_j : bm_i, rbmb = isj ? rbm_j : rbm_i;
        const double delv = ratio * rr;
        const double dv = div_by(delv, bmb, rbmb);
        const double dp = div_by(delv * tf, bmb, rbmb);
        VV[bb] = isj ? vcur + dv : vcur - dv;
        PP[bb] = isj ? pcur - dp : pcur + dp;
    }
    if (has && hl == 0) {
        S.colt[i] = (int8_t)ct;
        W.ct = ct; W.evcode = evcode; W.xpulse = 0;
    }
    __syncwarp();
    DMD_CSUB(3);
}

/* The draws of ghost g that do not depend on the state, on a warp: the
 * bead, the two accepted (v1, v2) pairs, the next ghost time's uniform and
 * the logarithms of r1, r2 and that uniform (lanes 0..2).  The lanes draw
 * the counter-based uniforms of each choice in parallel and ballots find the
 * first accepted one, so they equal lane_ghost()'s draws.  D.ok = 0 when 32
 * draws do not settle a choice (never in practice: lane_ghost() then draws
 * one at a time).  D.g is written last. */
__device__ void warp_ghost_draws(const DSys &S, long long gl, GhostDraws &D) {
    const int lane = threadIdx.x & 31;
    const int N = S.N;
    const uint64_t g = (uint64_t)gl;
    /* the bead: the first draw k with (int)(u * N) + 1 != N + 1 */
    const int iv = (int)(dmd_uniform(S.seed, DMD_STREAM_GHOST, g, (uint32_t)lane) * N) + 1;
    const unsigned mi = __ballot_sync(FULL, iv != N + 1);
    bool fallback = mi == 0;
    int i = 0, k = 0;
    if (!fallback) { const int k0 = __ffs(mi) - 1; i = __shfl_sync(FULL, iv, k0); k = k0 + 1; }
    /* two accepted pairs (v1, v2) from draws k, k+1, ... */
    double v1a = 0, v2a = 0, ra = 0, v1b = 0, rb = 0;
    for (int pair = 0; pair < 2 && !fallback; ++pair) {
        const double v1 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, g, (uint32_t)(k + 2 * lane)) - 1.0;
        const double v2 = 2.0 * dmd_uniform(S.seed, DMD_STREAM_GHOST, g, (uint32_t)(k + 2 * lane + 1)) - 1.0;
        const double r = v1 * v1 + v2 * v2;
        const unsigned ma = __ballot_sync(FULL, !((r == 0.0) || (r >= 1.0)));
        if (ma == 0) { fallback = true; break; }
        const int p = __ffs(ma) - 1;
        const double w1 = __shfl_sync(FULL, v1, p), w2 = __shfl_sync(FULL, v2, p), wr = __shfl_sync(FULL, r, p);
        if (pair == 0) { v1a = w1; v2a = w2; ra = wr; } else { v1b = w1; rb = wr; }
        k += 2 * (p + 1);
    }
    /* the next ghost time: the first draw not below 1e-18 and not 1 */
    double tg = 0.0;
    if (!fallback) {
        const double u = dmd_uniform(S.seed, DMD_STREAM_GHOST, g, (uint32_t)(k + lane));
        const unsigned mt = __ballot_sync(FULL, !((u < 1e-18) || (u == 1.0)));
        if (mt == 0) fallback = true;
        else tg = __shfl_sync(FULL, u, __ffs(mt) - 1);
    }
    /* lanes 0, 1: the logarithms of the two factors; lane 2: of the next
     * ghost time's uniform */
    if (!fallback && lane < 3) D.L[lane] = dmd_log(lane == 0 ? ra : (lane == 1 ? rb : tg));
    if (lane == 0) {
        D.ok = !fallback; D.i = i;
        D.v1a = v1a; D.v2a = v2a; D.v1b = v1b; D.ra = ra; D.rb = rb; D.tg = tg;
    }
    __syncwarp();
    if (lane == 0) D.g = gl;
    __syncwarp();
}

/* The ghost collision of lane_ghost() on a warp, with the same draws and
 * arithmetic (code/main.F90:997-1121).  D holds the draws of the current
 * ghost when another warp drew them ahead (D.g == the ghost index), else
 * they are drawn here; the two square roots and the next time run on three
 * lanes, the three velocity components on three lanes.  When the draws did
 * not settle (D.ok == 0), lane 0 runs lane_ghost() itself. */
__device__ int warp_ghost(const DSys &S, SharedState &sh, double &tfalse, GhostDraws &D) {
    const int lane = threadIdx.x & 31;
    const DTab &T = *S.tab;
    const int N = S.N;
    if (D.g != sh.sc.ghost_index) warp_ghost_draws(S, sh.sc.ghost_index, D);
    if (!D.ok) {
        int ii = 0;
        double tf = tfalse;
        if (lane == 0) ii = lane_ghost(S, sh, tf);
        __syncwarp();
        tfalse = __shfl_sync(FULL, tf, 0);
        return __shfl_sync(FULL, ii, 0);
    }
    int i = D.i;
    if (i > N) i = N;
    i -= 1;
    const double bmi = S.bm[i], rbmi = T.rbm[S.ident[i]];   /* bm(i) = mass(identity(i)) */
    /* lanes 0, 1: the two factors; lane 2: the next ghost time */
    const double lx = lane == 0 ? D.ra : (lane == 1 ? D.rb : D.tg);
    const double L = lane < 3 ? D.L[lane] : 0.0;
    double fact = 0.0, tn = 0.0;
    if (lane < 2) fact = sqrt(-2.0 * T.setemp * bmi * L / lx);
    else if (lane == 2) tn = -1.0 * L * T.avegtime + tfalse;
    const double fa = __shfl_sync(FULL, fact, 0), fb = __shfl_sync(FULL, fact, 1);
    tn = __shfl_sync(FULL, tn, 2);
    /* lanes 0..2: one component each, in the reference's order */
    if (lane < 3) {
        double *P = lane == 0 ? S.x : (lane == 1 ? S.y : S.z);
        double *V = lane == 0 ? S.vx : (lane == 1 ? S.vy : S.vz);
        double x = P[i] + V[i] * tfalse;
        const double num = lane == 0 ? D.v1a * fa : (lane == 1 ? D.v2a * fa : D.v1b * fb);
        const double v = div_by(num, bmi, rbmi);
        V[i] = v;
        P[i] = x - v * tfalse;
    }
    if (lane == 0) {
        sh.sc.ghost_index += 1;
        sh.sc.n_ghost += 1;
        set_pred(S, N, tn, -2, -2, tn < sh.sc.interval_max);
    }
    __syncwarp();
    if (tfalse < sh.sc.old_tfalse) tfalse = sh.sc.old_tfalse;
    return i;
}

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
    /* 1. the down-list operations in the reference's order: i's down list,
     * i's lower extras, j's down list without i, j's lower extras.  Every
     * load that needs only i and j is issued first (list lengths, extras),
     * then both lists together, 32 entries of each per pass. */
    int n = 0;
    {
        const int cnt = S.dnn[i];
        const int cj = j >= 0 ? S.dnn[j] : 0;
        const int eri = lane < 3 ? S.er[4 * i + lane] : -1;
        const int erj = (j >= 0 && lane < 3) ? S.er[4 * j + lane] : -1;
        const int *dn = S.dn + (size_t)i * S.cap;
        const int8_t *dc = S.dnc ? S.dnc + (size_t)i * S.cap : nullptr;
        const int *dj = j >= 0 ? S.dn + (size_t)j * S.cap : nullptr;
        const int8_t *dcj = (j >= 0 && S.dnc) ? S.dnc + (size_t)j * S.cap : nullptr;
        const int passes = (max(cnt, cj) + 31) >> 5;
        /* i's list goes to ops[0, cnt); j's kept entries are counted per pass
         * and placed after i's extras once their number is known */
        int nj = 0;
        const bool ei_keep = lane < 3 && eri >= 0 && eri < i;
        const unsigned mei = __ballot_sync(FULL, ei_keep);
        const int base_j = cnt + __popc(mei);
        for (int ps = 0; ps < passes; ++ps) {
            const int q = 32 * ps + lane;
            const int li = q < cnt ? dn[q] : -1;
            const int8_t ci = (q < cnt && dc) ? dc[q] : (int8_t)-1;
            const int lj = q < cj ? dj[q] : -1;
            const int8_t cjv = (q < cj && dcj) ? dcj[q] : (int8_t)-1;
            if (q < cnt) { const int qq = DMD_CHK(q, OPS_MAX, 20); W.ops_l[qq] = li; W.ops_s[qq] = i; W.ops_c[qq] = ci; }
            const bool keep = q < cj && lj != i;
            const unsigned m = __ballot_sync(FULL, keep);
            const int pos = DMD_CHK(base_j + nj + __popc(m & ((1u << lane) - 1)), OPS_MAX, 21);
            if (keep) { W.ops_l[pos] = lj; W.ops_s[pos] = j; W.ops_c[pos] = cjv; }
            nj += __popc(m);
        }
        if (ei_keep) {
            const int pos = DMD_CHK(cnt + __popc(mei & ((1u << lane) - 1)), OPS_MAX, 22);
            W.ops_l[pos] = eri; W.ops_s[pos] = i; W.ops_c[pos] = -1;
        }
        n = base_j + nj;
        if (j >= 0) {
            const bool ej_keep = lane < 3 && erj >= 0 && erj < j;
            const unsigned mej = __ballot_sync(FULL, ej_keep);
            if (ej_keep) {
                const int pos = DMD_CHK(n + __popc(mej & ((1u << lane) - 1)), OPS_MAX, 23);
                W.ops_l[pos] = erj; W.ops_s[pos] = j; W.ops_c[pos] = -1;
            }
            n += __popc(mej);
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
        if (lead) { const int pp = DMD_CHK(pos, OPS_MAX, 24); W.lead_l[pp] = l; W.lead_q[pp] = (int16_t)q; W.lead_m[pp] = mark; }
        if (mark) W.mk[DMD_CHK(mpos, OPS_MAX, 25)] = (int16_t)pos;
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
        if (lead) { const int pp = DMD_CHK(pos, OPS_MAX, 26); W.lead_l[pp] = l; W.lead_q[pp] = (int16_t)q; W.lead_m[pp] = mark; }
        if (lead && mark) W.mk[DMD_CHK(mpos, OPS_MAX, 27)] = (int16_t)pos;
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
        else b = W.lead_l[DMD_CHK(W.mk[DMD_CHK(m0 + t - 2, OPS_MAX, 29)], OPS_MAX, 30)];
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
/* Reads of a light batch.  In a batch whose events are all bond or core
 * events (coltype 1-3), an event writes only the positions and velocities
 * of its own two beads, during its collision, before any re-prediction
 * runs.  A re-prediction of event e that reads a bead written by an earlier
 * event of the batch then sees its new state, as in the serial order; one
 * that reads a bead written by a later event must see its state before the
 * batch - the later event's snapshot.  So those reads are no conflict, and
 * the footprints of light batches hold only the written beads and the
 * queue entries.  The writer of a bead is the earliest claimer of it in
 * the write table (two writers of one bead conflict). */
struct Ver {
    const unsigned *own_w;   /* write table of the batch, or null: current state */
    const WarpArea *wa;      /* the events' areas (C = 1: slot = warp) */
    unsigned tseq;           /* ticket sequence of the batch */
    int e, P;                /* the reading event's slot, the batch size */
};
__device__ __forceinline__ const double *ver_of(const Ver &V, int b) {
    if (!V.own_w || b < 0) return nullptr;
    const unsigned t = V.own_w[b];
    if ((t >> 6) != V.tseq) return nullptr;
    const int g = 63 - (int)(t & 63u);
    if (g <= V.e || g >= V.P) return nullptr;
    const WarpArea &G = V.wa[g];
    return G.sij + (G.i == b ? 0 : 6);
}

__device__ __forceinline__ bool rp_predict_code(const DSys &S, Err E, int pa, int pbb, int code, bool is_op,
                                                double tf, double &tt, int &ty, const double *si = nullptr,
                                                const double *sj = nullptr) {
    double tij = 0.0;
    ty = 0;
    bool ok = d_predict_c(S, pa, pbb, code, tf, tij, ty, si, sj);
#ifdef DMD_PHASE_TIMERS
    {   /* double-precision predictions: all, no event while separating, no event while approaching */
        unsigned long long *cnt = (unsigned long long *)&g_phase_cycles[DMD_PHASE_CTAS - 2][0];
        atomicAdd(cnt, 1ull);
        if (ok && ty == 0) atomicAdd(cnt + (d_lt0(d_rel_c(S, pa, pbb, tf).bij) ? 2 : 1), 1ull);
    }
#endif
    if (!ok) set_err(E, DMD_E_INPUT, pa);
    else if (okey(tij) < okey(-1.0e-10)) set_err(E, DMD_E_NEG_TIME, pa);
    tt = tij + (is_op ? tf : -0.0);
    return ok;
}
__device__ __forceinline__ int rp_code(const DSys &S, int pa, int pbb, int st, bool is_op, int hbonds) {
    int a1 = is_op ? pa : pbb, a2 = is_op ? pbb : pa;
    return st >= 0 ? pair_code_st(S, a1, a2, st) : pair_code(S, a1, a2, hbonds);
}
__device__ __forceinline__ bool rp_predict(const DSys &S, Err E, int pa, int pbb, int st, bool is_op, double tf,
                                           int hbonds, double &tt, int &ty, const Ver &V) {
    if (pa >= 0)
        return rp_predict_code(S, E, pa, pbb, rp_code(S, pa, pbb, st, is_op, hbonds), is_op, tf, tt, ty,
                               ver_of(V, pa), ver_of(V, pbb));
    ty = 0;
    tt = 0.0 + (is_op ? tf : -0.0);
    return false;
}
/* 1-4 into the CTA's task pool for the event of warp `owner` (its tasks
 * must fit one round and the pool), else W.pooled = 0 and the owner warp
 * runs warp_repredict() after the pool */
__device__ void warp_rp_prepare(const DSys &S, WarpArea &W, TaskPool &TP, int owner, int i, int j, double tf,
                                double imax, bool timed = false) {
    int lane = threadIdx.x & 31;
#ifdef DMD_PHASE_TIMERS
    long long pt0 = clock64();
#endif
    warp_rp_lists(S, W, i, j);
#ifdef DMD_PHASE_TIMERS
    if (timed && lane == 0) { long long t = clock64(); g_phase_cycles[DMD_PHASE_CTAS - 6][0] += t - pt0; pt0 = t; }
#endif
    bool pooled = W.nmarked <= TG_MAX - 2;
    int base = 0;
    if (pooled) {
        const double Hraw = imax + DMD_LTSTEP - tf;
        warp_rp_targets(S, W, i, j, 0, Hraw, okey(Hraw));
#ifdef DMD_PHASE_TIMERS
        if (timed && lane == 0) { long long t = clock64(); g_phase_cycles[DMD_PHASE_CTAS - 6][1] += t - pt0; pt0 = t; }
#endif
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
#ifdef DMD_PHASE_TIMERS
        if (timed && lane == 0) {
            long long t = clock64();
            g_phase_cycles[DMD_PHASE_CTAS - 6][2] += t - pt0;
            g_phase_cycles[DMD_PHASE_CTAS - 6][3] += 1;
            g_phase_cycles[DMD_PHASE_CTAS - 6][4] += nt;
            g_phase_cycles[DMD_PHASE_CTAS - 6][5] += W.nops;
            g_phase_cycles[DMD_PHASE_CTAS - 6][6] += W.nmarked;
        }
#endif
    }
    if (lane == 0) { W.pooled = pooled; W.pool_base = base; W.big_tf = DMD_BIG + tf; }
    __syncwarp();
}

/* 4: the tasks of the round on this warp, 32 per pass */
__device__ void warp_rp_tasks(const DSys &S, Err E, WarpArea &W, int rd, double tf, int hbonds, const Ver &V) {
    int lane = threadIdx.x & 31;
    const int nop = rd == 0 ? W.nops : 0;
    const int ntask = W.ntask;
    for (int base = 0; base < ntask; base += 32) {
        int q = base + lane;
        int pa = -1, pbb = -1, st = -1, tgt = -1;
        if (q < ntask) rp_task(S, W, q, nop, pa, pbb, st, tgt);
        double tt;
        int ty;
        bool ok = rp_predict(S, E, pa, pbb, st, q < nop, tf, hbonds, tt, ty, V);
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
        const long long t0 = dbits(t);
        const int p0 = p, y0 = y;
        const bool q0 = qq;
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
        int slot = DMD_CHK(2 + ld, OPS_MAX + 2, 28);
        if (l == i) {
            W.pb[slot] = -1;
            W.pt[0] = t; W.pn[0] = p; W.pc[0] = (int8_t)y; W.pq[0] = qq;
        } else {
            /* bit 1 of pq: the entry is unchanged (not new, not written) */
            const bool same = dbits(t) == t0 && p == p0 && y == y0 && qq == q0;
            W.pb[slot] = l;
            W.pt[slot] = t; W.pn[slot] = p; W.pc[slot] = (int8_t)y; W.pq[slot] = (uint8_t)(qq | (same ? 2 : 0));
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
        if (b < 0 || (W.pq[q] & 3) != 1) continue;   /* queued and changed */
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
                               int hbonds, const Ver &V) {
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
        warp_rp_tasks(S, E, W, rd, tf, hbonds, V);
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
        if (W.pq[q] & 2) continue;   /* unchanged */
        set_pred(S, b, W.pt[q], W.pn[q], W.pc[q], (W.pq[q] & 1) != 0);
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
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1;
    const int N = S.N;
    unsigned *own_r = own, *own_w = own + N, *own_q = own + 2 * N;
    DMD_SUB(-1);
    /* the sets are appended warp-wide: a ballot per chunk of 32 places each
     * lane's bead; the counters stay in registers (warp-uniform) */
    int nr = 0, nw = 0, nq = 0;
    auto put = [&](int *arr, int cap, int &n, bool pred, int b) {
        unsigned m = __ballot_sync(FULL, pred);
        int pos = n + __popc(m & lt);
        if (pred && pos < cap) arr[pos] = b;
        n += __popc(m);
    };
    /* fixed part on lanes 0..17: i, j, their extras (2..9), the own helpers
     * of i, j (10..13) and of their fourth extras (14..17, read only) */
    {
        int b = -1;
        if (lane == 0) b = i;
        else if (lane == 1) b = j;
        else if (lane < 6) b = S.er[4 * i + lane - 2];
        else if (lane < 10) b = S.er[4 * j + lane - 6];
        else if (lane < 18) {
            int which = (lane - 10) >> 1;
            int x = which == 0 ? i : which == 1 ? j : which == 2 ? S.er[4 * i + 3] : S.er[4 * j + 3];
            int h1, h2;
            own_helpers(S, x, h1, h2);
            b = (lane & 1) ? h2 : h1;
        }
        const bool v = b >= 0;
        const bool w = v && lane < 14;
        /* queue entries: i, j, the lower extras (0..2) and the helpers */
        const bool q = v && (lane < 5 || (lane >= 6 && lane < 9) || (lane >= 10 && lane < 14));
        if (v) atomicMax(&own_r[b], ticket);
        if (w) atomicMax(&own_w[b], ticket);
        if (q) atomicMax(&own_q[b], ticket);
        put(W.rset, RSET_MAX, nr, v, b);
        put(W.wset, WSET_MAX, nw, w, b);
        put(W.qset, QSET_MAX, nq, q, b);
    }
    /* the neighbour lists of i and j as one range [up i | down i | up j |
     * down j]: all read, the down lists also queue entries; a down-list
     * bead whose partner is the list's owner may be fully re-predicted
     * (cascade) */
    const int ui = S.upn[i], di = S.dnn[i], uj = S.upn[j], dj = S.dnn[j];
    const int *UI = S.up + (size_t)i * S.cap, *DI = S.dn + (size_t)i * S.cap;
    const int *UJ = S.up + (size_t)j * S.cap, *DJ = S.dn + (size_t)j * S.cap;
    const int e1 = ui, e2 = ui + di, e3 = ui + di + uj, tot = ui + di + uj + dj;
    int nc = 0;
    for (int base = 0; base < tot; base += 32) {
        const int q = base + lane;
        int l = -1, src = -1;
        if (q < e1) l = UI[q];
        else if (q < e2) { l = DI[q - e1]; src = i; }
        else if (q < e3) l = UJ[q - e2];
        else if (q < tot) { l = DJ[q - e3]; src = j; }
        const bool v = l >= 0, down = src >= 0;
        if (v) atomicMax(&own_r[l], ticket);
        if (down) atomicMax(&own_q[l], ticket);
        const bool cas = down && S.nptnr[l] == src;
        put(W.rset, RSET_MAX, nr, v, l);
        put(W.qset, QSET_MAX, nq, down, l);
        put(W.casc, CASC_MAX - 10, nc, cas, l);
    }
    DMD_SUB(9);
    const bool over = nc > CASC_MAX - 10;
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
    DMD_SUB(10);
    for (int base = 0; base < run; base += 32) {
        const int q = base + lane;
        int b = -1;
        if (q < run) {
            int lo = 0, hi = nc - 1;          /* last cascade bead with cbase <= q */
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (W.cbase[mid] <= q) lo = mid; else hi = mid - 1;
            }
            int l = W.casc[lo];
            int k = q - W.cbase[lo];
            int ul = W.cbase[lo + 1] - W.cbase[lo] - 3;
            b = k < ul ? S.up[(size_t)l * S.cap + k] : S.er[4 * l + (k - ul)];
        }
        if (b >= 0) atomicMax(&own_r[b], ticket);
        put(W.rset, RSET_MAX, nr, b >= 0, b);
    }
    /* an incomplete list (cascade or set overflow) ends the batch here */
    if (lane == 0) {
        W.nrset = nr; W.nwset = nw; W.nqset = nq;
        W.casc_over = over || nr > RSET_MAX || nw > WSET_MAX || nq > QSET_MAX;
    }
    __syncwarp();
    DMD_SUB(11);
}
/* The footprint of an event of a light batch (every event of coltype 1-3):
 * R = W = {i, j}, the beads its collision reads and writes; its
 * re-prediction reads other beads through Ver.  Q lists the queue entries
 * it reads (i, j, the lower extras, both down lists): a later event that
 * reads an earlier one's i or j ends the batch before it (those entries
 * always change; k_run compares Q with the earlier candidates' pairs).  Other entries it reads are checked after the fact
 * (warp_mark_queue, warp_check_queue): an event that read an entry an
 * earlier event of the batch changed is rolled back. */
__device__ void warp_footprint_claim_light(const DSys &S, WarpArea &W, unsigned *own, unsigned ticket, int i, int j) {
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int N = S.N;
    int nq = 0;
    auto put = [&](int *arr, int cap, int &n, bool pred, int b) {
        unsigned m = __ballot_sync(FULL, pred);
        int pos = n + __popc(m & lt);
        if (pred && pos < cap) arr[pos] = b;
        n += __popc(m);
    };
    if (lane < 2) {
        const int b = lane == 0 ? i : j;
        atomicMax(&own[b], ticket);
        atomicMax(&own[N + b], ticket);   /* the write table: who writes b (Ver) */
        W.rset[lane] = b;
        W.wset[lane] = b;
    }
    {
        int b = -1;
        if (lane < 2) b = lane == 0 ? i : j;
        else if (lane < 5) { b = S.er[4 * i + lane - 2]; if (b >= i) b = -1; }
        else if (lane >= 6 && lane < 9) { b = S.er[4 * j + lane - 6]; if (b >= j) b = -1; }
        put(W.qset, QSET_MAX, nq, b >= 0, b);
    }
    const int di = S.dnn[i], dj = S.dnn[j];
    const int *DI = S.dn + (size_t)i * S.cap, *DJ = S.dn + (size_t)j * S.cap;
    for (int base = 0; base < di + dj; base += 32) {
        const int q = base + lane;
        const int l = q < di ? DI[q] : (q < di + dj ? DJ[q - di] : -1);
        put(W.qset, QSET_MAX, nq, l >= 0, l);
    }
    if (lane == 0) {
        W.nrset = 2; W.nwset = 2; W.nqset = nq;
        W.casc_over = nq > QSET_MAX;
    }
    __syncwarp();
}
/* light batches, after the re-predictions: the queue entries this event
 * changes (i and j always; the others where the replay's result differs
 * from the entry it started from, W.pq bit 1 clear) are marked with its
 * ticket in own_q */
__device__ void warp_mark_queue(const WarpArea &W, unsigned *own_q, unsigned ticket) {
    const int lane = threadIdx.x & 31;
    for (int q = lane; q < W.npred; q += 32) {
        const int b = W.pb[q];
        if (b >= 0 && !(W.pq[q] & 2)) atomicMax(&own_q[b], ticket);
    }
    __syncwarp();
}
/* ... and, once every event has marked: whether an earlier event of the
 * batch changed an entry this one read */
__device__ bool warp_check_queue(const WarpArea &W, const volatile unsigned *own_q, unsigned ticket) {
    const int lane = threadIdx.x & 31;
    bool bad = false;
    for (int q = lane; q < W.npred; q += 32) {
        const int b = W.pb[q];
        if (b >= 0) bad |= own_q[b] > ticket;
    }
    return __any_sync(FULL, bad);
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

/* The event loop of code/main.F90:484-1258 for nsys systems, each advanced
 * by one cluster of C CTAs (C = 1: one CTA).  The leader CTA (rank 0)
 * selects events and keeps the counters; a batch's candidates go one per
 * warp over all CTAs of the cluster. */
__global__ void __launch_bounds__(RUN_NT, 1) k_run(DSys *systems, int nsys, long long target_all,
                                                     long long *targets, int hbonds_mask,
                                                     const int *chain_start, const int *chain_len,
                                                     const int *chain_off, dmd_diag *outputs, int own_cap, int C,
                                                     int dn_limit, int cycles, int hot_cap) {
    extern __shared__ __align__(16) unsigned char dsmem[];
    WarpArea *warea = reinterpret_cast<WarpArea *>(dsmem);
    __shared__ SharedState sh;
    __shared__ DSys S_sh;
    const int rank = C > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int r = blockIdx.x / C;
    if (r >= nsys) return;             /* whole clusters only */
    const long long target = targets ? targets[r] : target_all;   /* events for this system */
    const bool leader = rank == 0;
    if (threadIdx.x == 0) S_sh = systems[r];
    __syncthreads();
    /* A single-CTA system whose hot per-bead arrays fit hot_cap bytes of
     * shared memory (after the claim tables) keeps them there for the
     * launch: positions, velocities, queue times, keys, partners, coltypes,
     * queue flags and the level-1 tournament.  Every access goes through
     * S_sh's pointers, which now point there; the arrays go back to the
     * system's pool at the end of the launch. */
    char *const hot = (char *)dsmem + hot_offset(sizeof(WarpArea) * RUN_NW + sizeof(TaskPool), own_cap);
    const bool use_hot = C == 1 && hot_cap > 0 && hot_bytes(S_sh.N, S_sh.nl1) <= (size_t)hot_cap;
    if (use_hot) {
        HotArrays H = hot_layout(hot, S_sh.N, S_sh.nl1);
        hot_copy(H, S_sh, true);
        __syncthreads();
        if (threadIdx.x == 0) {
            S_sh.x = H.x; S_sh.y = H.y; S_sh.z = H.z; S_sh.vx = H.vx; S_sh.vy = H.vy; S_sh.vz = H.vz;
            S_sh.tim = H.tim; S_sh.key = H.key; S_sh.l1k = H.l1k; S_sh.nptnr = H.nptnr; S_sh.l1i = H.l1i;
            S_sh.colt = H.colt; S_sh.queued = H.queued;
        }
        __syncthreads();
    }
    const DSys &S = S_sh;
    const int N = S.N;
    const int hbonds = hbonds_mask & 1;
    const bool phys = (S.flags & DMD_FLAG_COUNT_PHYSICAL) != 0;
    const bool stop_out = (S.flags & DMD_FLAG_STOP_AT_OUTPUT) != 0;
    const bool serial = (S.flags & DMD_FLAG_SERIAL) != 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    /* candidate slot of this warp: slots are dealt round robin over the
     * CTAs of a cluster, so that a short batch still spreads its events
     * (and their pooled prediction tasks) over all SMs of the cluster */
    const int gw = warp * C + rank;
    const int slots = min(C * RUN_NW, CAND_MAX);
    WarpArea &W = warea[warp];
    SharedState *L = C > 1 ? cg::this_cluster().map_shared_rank(&sh, 0) : &sh;
    if (threadIdx.x == 0) {
        sh.ncand = 0;
        sh.sc = *S.sc; sh.sc.done = 0; sh.sc.stop = 0; sh.sc.need_full = 0;
        sh.delta = sh.sc.interval * 0.05;
        sh.bseq = 0;
        sh.exitf = 0;
        sh.gdraw[0].g = -1; sh.gdraw[1].g = -1;
    }
    /* footprint claim table: shared memory when one CTA holds the system and
     * it fits, else the system's global array; cleared at every launch */
    TaskPool &TP = *(TaskPool *)(warea + RUN_NW);
    unsigned *own = (C == 1 && N <= own_cap) ? (unsigned *)((char *)(warea + RUN_NW) + sizeof(TaskPool)) : S.owner;
    if (threadIdx.x == 0) { TP.n = 0; TP.nlive = 0; }
    for (int b = rank * blockDim.x + threadIdx.x; b < 3 * N; b += C * blockDim.x) own[b] = 0u;
    csync(C);
    DMD_PHASE_START(leader ? r : -1);
    const int *cs = chain_start + chain_off[r], *cl = chain_len + chain_off[r];
    const long long max_iter = (S.flags & DMD_FLAG_TIGHT_LOOP_BOUND) ? 8 : 16 * target + 1000000;
    const long long t_start = clock64();
    long long iter = 0;
    while (true) {
        /* ---- the leader selects the next event (and a batch) ---- */
        ++iter;   /* on every thread, so that each can take the test below */
        /* the ghost index before this iteration (only a ghost event moves
         * it, after the barrier below) */
        const long long gidx = sh.sc.ghost_index;
        /* One CTA with at most 256 level-1 groups: every warp finds the root
         * itself from the level-1 minima and, when it is a bead's event of a
         * batch, goes straight into the candidate gather without a barrier;
         * otherwise (exit, pseudo event, last event, clusters) warp 0 decides
         * and the others wait for it. */
        bool fast = false;
        int fe = -1;
        long long fk = 0;
        if (C == 1 && !serial && S.nl1 <= 256 && !(sh.sc.done >= target || sh.sc.err || sh.sc.stop) &&
            !(sh.sc.max_dn > dn_limit) && !(iter > max_iter) && target - sh.sc.done > 1) {
            fe = warp_root(S, fk);
            fast = fe >= 0 && fe < N;
        }
        if (fast) {
            if (threadIdx.x == 0) { sh.exitf = 0; sh.ev = fe; sh.kcut = fk; }
            DMD_PHASE(0);
            int m = cta_gather_candidates(S, sh, fe, fk, slots);
            if (m > slots) m = slots;
            const long long left = target - sh.sc.done;
            if (m > left) m = (int)left;
            if (threadIdx.x == 0) {
                sh.m = m;
                sh.tick_reset = m > 1 && sh.bseq >= DMD_TICKET_SEQ_MAX;
                sh.c_simple[0] = 0;
                sh.coll0 = sh.sc.coll; sh.log0 = sh.sc.log_count; sh.imax = sh.sc.interval_max; sh.tnow = sh.sc.t;
            }
            DMD_PHASE(1);
        } else if (leader) {
            if (warp == 0) {
                /* warp 0: the exit test and the root */
                int ex = 0;
                if (lane == 0) {
                    bool x = sh.sc.done >= target || sh.sc.err || sh.sc.stop;
                    /* lists longer than this variant takes: the host goes
                     * on with the full variant from here */
                    if (!x && sh.sc.max_dn > dn_limit) { sh.sc.need_full = 1; x = true; }
                    if (!x && iter > max_iter) { set_err(sh, DMD_E_DEVICE_TIMEOUT, 0); x = true; }
                    ex = x;
                }
                ex = __shfl_sync(FULL, ex, 0);
                long long kroot = 0;
                const int e = ex ? -1 : warp_root(S, kroot);
                if (!ex && e < 0 && lane == 0) set_err(sh, DMD_E_STATE, 0);
                ex = ex || e < 0;
                if (lane == 0) {
                    sh.exitf = ex;
                    sh.ev = e;
                    sh.kcut = kroot;
                    sh.ncand = 0;
                    if (!ex && e >= N) {
                        /* a pseudo event: its counter and time */
                        sh.sc.coll += 1;
                        sh.tf_iv = S.tim[e];
                        if (e != N) sh.sc.tfalse = sh.tf_iv;
                    }
                }
            }
            __syncthreads();
            DMD_PHASE(0);
            if (!sh.exitf && sh.ev < N) {
                const int e = sh.ev;
                const long long kroot = sh.kcut;
                const long long left = target - sh.sc.done;
                int m = 1;
                if (serial || left <= 1) {
                    if (threadIdx.x == 0) { sh.sort_key[0] = kroot; sh.sort_idx[0] = e; }
                } else {
                    m = cta_gather_candidates(S, sh, e, kroot, slots);
                    if (m > slots) m = slots;
                    if (m > left) m = (int)left;
                }
                if (threadIdx.x == 0) {
                    sh.m = m;
                    sh.tick_reset = m > 1 && sh.bseq >= DMD_TICKET_SEQ_MAX;
                    sh.c_simple[0] = 0;    /* set by the footprint test when m > 1 */
                }
                DMD_PHASE(1);
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
            if (threadIdx.x < RUN_NW) {
                int k = threadIdx.x * C + rank;
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
            bool light = false;       /* reads of later events' beads go to their snapshots */
            unsigned tseq = 0, my_ticket = 0;
            if (m > 1) {
                if (sh.tick_reset) {   /* tickets exhausted: clear the table */
                    for (int b = rank * blockDim.x + threadIdx.x; b < 3 * N; b += C * blockDim.x) own[b] = 0u;
                    csync(C);
                    if (threadIdx.x == 0) sh.bseq = 0;
                    __syncthreads();
                }
                unsigned ticket = ((unsigned)(sh.bseq + 1) << 6) | (unsigned)(63 - gw);
                tseq = ticket >> 6;
                my_ticket = ticket;
                /* a light batch: one CTA, every candidate of coltype 1-3 */
                {
                    bool heavy = false;
                    for (int k = lane; k < m; k += 32) {
                        const int ct0 = S.colt[sh.sort_idx[k]];
                        heavy |= ct0 < 1 || ct0 > 3;
                    }
                    light = C == 1 && !__any_sync(FULL, heavy);
                }
                if (light) {
                    /* light batch (one CTA): the earlier events' bead pairs
                     * are known from the candidate list, so each event tests
                     * its queue reads against them directly - one barrier */
                    if (gw < m) {
                        const int i = sh.sort_idx[gw];
                        warp_footprint_claim_light(S, W, own, ticket, i, S.nptnr[i]);
                        int pi = -1, pj = -1;
                        if (lane < gw) { pi = sh.sort_idx[lane]; pj = S.nptnr[pi]; }
                        bool c = false;
                        const int nq = min(W.nqset, QSET_MAX);
                        for (int base = 0; base < nq; base += 32) {
                            const int q = base + lane;
                            const int b = q < nq ? W.qset[q] : -1;
                            for (int k = 0; k < gw; ++k) {
                                const int ik = __shfl_sync(FULL, pi, k), jk = __shfl_sync(FULL, pj, k);
                                c |= b >= 0 && (b == ik || b == jk);
                            }
                        }
                        c = __any_sync(FULL, c);
                        if (lane == 0) { L->c_conflict[gw] = c; L->c_over[gw] = W.casc_over; L->c_simple[gw] = 1; }
                    }
                    __syncthreads();
                    DMD_PHASE(10);
                } else {
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
                }
                DMD_PHASE(11);
                /* every warp: the longest conflict-free prefix (candidate k
                 * >= 1 whose footprint meets an earlier one ends it before
                 * k); an incomplete footprint (cascade list overflow) ends
                 * it after its event */
                if (C == 1) {
                    int p = m;
#pragma unroll
                    for (int h = 0; h < CAND_MAX / 32; ++h) {
                        const int k = lane + 32 * h;
                        const unsigned cf = __ballot_sync(FULL, k > 0 && k < m && sh.c_conflict[k]);
                        const unsigned ov = __ballot_sync(FULL, k < m && sh.c_over[k]);
                        if (cf) p = min(p, 32 * h + __ffs(cf) - 1);
                        if (ov) p = min(p, max(32 * h + __ffs(ov) - 1, 1));
                    }
                    P = p;
                } else {
                    /* clusters: the leader decides, the others copy */
                    if (leader && threadIdx.x == 0) {
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
                }
                if (leader && threadIdx.x == 0) sh.bseq = sh.tick_reset ? 1 : sh.bseq + 1;
                DMD_PHASE(2);
            }
            /* speculative commit of each event on its warp */
            const long long coll0 = sh.coll0;
            const double imax = sh.imax;
            /* this CTA's events are warps 0 .. nloc-1; the free warps
             * nloc .. RUN_NW-1 take over the task preparation of up to two
             * events each when that covers every event */
            const int nloc = P > rank ? (P - rank + C - 1) / C : 0;
            const int nfree = RUN_NW - nloc;
            const bool split = nfree > 0 && 2 * nfree >= nloc;
            if (light) DMD_LSUB(-1);
            if (light) {
                /* light batch (one CTA): two events per collision warp, one
                 * on each half; the other warps prepare the events' tasks
                 * meanwhile (the collisions cannot change what they read) */
                const int ncw = (P + 1) / 2;
                if (warp < ncw) {
                    const int k = 2 * warp + (lane >> 4);
                    const bool has = k < P;
                    const int kk = has ? k : 2 * warp;
                    WarpArea &WE = warea[kk];
                    const int i = sh.sort_idx[kk];
                    const int j = S.nptnr[i];
                    const double tf = S.tim[i];
                    if (has && (lane & 15) == 0) {
                        WE.i = i; WE.j = j; WE.tf = tf; WE.coll = coll0 + k + 1; WE.err = 0; WE.err_info = 0;
                    }
                    hw_collision_light(S, WE, has, i, j, tf, hbonds);
                    DMD_LSUB(1);
                } else {
                    for (int k = warp - ncw; k < P; k += RUN_NW - ncw) {
                        const int i = sh.sort_idx[k];
#ifdef DMD_PHASE_TIMERS
                        const bool timed = blockIdx.x == g_sub_cta && warp == ncw;
#else
                        const bool timed = false;
#endif
                        warp_rp_prepare(S, warea[k], TP, k, i, S.nptnr[i], S.tim[i], imax, timed);
                    }
                }
            } else if (gw < P) {
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
                 * A free warp prepares them while this one computes the
                 * collision, when the collision cannot change the H-bond
                 * state they read (coltype 1-3). */
                if (!(split && L->c_simple[gw])) warp_rp_prepare(S, W, TP, warp, i, j, tf, imax);
            } else if (split) {
                for (int k = warp - nloc; k < nloc; k += nfree) {
                    const int ge = k * C + rank;
                    if (!L->c_simple[ge]) continue;
                    const int i = sh.sort_idx[ge];
                    warp_rp_prepare(S, warea[k], TP, k, i, S.nptnr[i], S.tim[i], imax);
                }
            }
            __syncthreads();
            if (light) DMD_LSUB(2);
            /* every pooled prediction task of this CTA's events, all warps:
             * first the pair codes, settling in single precision the tasks
             * that certainly have no event; then the double-precision
             * predictions of the rest, packed so that their warp
             * instructions (64 cycles each on the FP64 unit whatever the
             * active lanes) have all lanes busy */
            {
                const int ntot = min(TP.n, PTASK_MAX);   /* TP.nlive is 0 (reset with TP.n) */
                DMD_PHASE(12);
                for (int base = 0; base < ntot; base += RUN_NT) {
                    const int q = base + threadIdx.x;
                    bool live = false;
                    if (q < ntot) {
                        const int pa = TP.a[q];
                        if (pa < 0) {
                            TP.ok[q] = 0;
                        } else {
                            const int pbb = TP.b[q];
                            const bool is_op = (TP.flag[q] & 1) != 0;
                            const int owner = TP.flag[q] >> 1;
                            const WarpArea &O = warea[owner];
                            const int code = rp_code(S, pa, pbb, TP.st[q], is_op, hbonds);
                            const Ver V{light ? own + N : nullptr, warea, tseq, owner, P};
                            if (f32_no_event(S, pa, pbb, code, d_hi(&O.tf), ver_of(V, pa), ver_of(V, pbb))) {
                                TP.t[q] = is_op ? O.big_tf : DMD_BIG;
                                TP.ty[q] = 0;
                                TP.ok[q] = 1;
#ifdef DMD_PHASE_TIMERS
                                atomicAdd((unsigned long long *)&g_phase_cycles[DMD_PHASE_CTAS - 2][3], 1ull);
#endif
                            } else {
                                TP.st[q] = (int8_t)code;
                                live = true;
                            }
                        }
                    }
                    const unsigned lm = __ballot_sync(FULL, live);
                    int pos = 0;
                    if (lane == 0 && lm) pos = atomicAdd(&TP.nlive, __popc(lm));
                    pos = __shfl_sync(FULL, pos, 0) + __popc(lm & ((1u << lane) - 1));
                    if (live) TP.live[pos] = (int16_t)q;
                }
                __syncthreads();
                DMD_PHASE(13);
                if (light) DMD_LSUB(3);
                const int nlive = TP.nlive;
                for (int k = threadIdx.x; k < nlive; k += blockDim.x) {
                    const int q = TP.live[k];
                    const int owner = TP.flag[q] >> 1;
                    WarpArea &O = warea[owner];
                    Err EO{&O.err, &O.err_info};
                    double tt;
                    int ty;
                    const Ver V{light ? own + N : nullptr, warea, tseq, owner, P};
                    bool ok = rp_predict_code(S, EO, TP.a[q], TP.b[q], TP.st[q], (TP.flag[q] & 1) != 0, O.tf, tt, ty,
                                              ver_of(V, TP.a[q]), ver_of(V, TP.b[q]));
                    TP.t[q] = tt; TP.ty[q] = (int8_t)ty; TP.ok[q] = ok;
                }
            }
            __syncthreads();
            DMD_PHASE(14);
            if (light) DMD_LSUB(4);
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
                    /* the full tasks, 32 at a time: a segmented (key, partner)
                     * minimum over each target's run of tasks by shuffles, the
                     * run's head lane merging it into the target's minimum */
                    const int f0 = base + nop, nf = W.fs.tg_base[ntg];
                    for (int c = 0; c < nf; c += 32) {
                        const int x = c + lane;
                        int tgt = -1;
                        long long k = DMD_KEY_INF;
                        int p = INT_MAX, y = 0;
                        double rt = 0.0;
                        if (x < nf) {
                            if (nf <= TMAP_MAX) tgt = W.fs.tmap[x];
                            else {
                                int lo = 0, hi = ntg - 1;   /* last target with tg_base <= x */
                                while (lo < hi) {
                                    const int mid = (lo + hi + 1) >> 1;
                                    if (W.fs.tg_base[mid] <= x) lo = mid; else hi = mid - 1;
                                }
                                tgt = lo;
                            }
                            if (TP.ok[f0 + x]) { rt = TP.t[f0 + x]; k = okey(rt); p = TP.b[f0 + x]; y = TP.ty[f0 + x]; }
                        }
#pragma unroll
                        for (int o = 1; o < 32; o <<= 1) {
                            const long long k2 = __shfl_down_sync(FULL, k, o);
                            const int p2 = __shfl_down_sync(FULL, p, o);
                            const double r2 = __shfl_down_sync(FULL, rt, o);
                            const int y2 = __shfl_down_sync(FULL, y, o);
                            const int g2 = __shfl_down_sync(FULL, tgt, o);
                            if (lane + o < 32 && g2 == tgt && key_less(k2, p2, k, p)) { k = k2; p = p2; rt = r2; y = y2; }
                        }
                        const int gprev = __shfl_up_sync(FULL, tgt, 1);
                        const bool head = tgt >= 0 && (lane == 0 || gprev != tgt);
                        if (head && key_less(k, p, W.fs.tg_k[tgt], W.fs.tg_p[tgt])) {
                            W.fs.tg_k[tgt] = k; W.fs.tg_p[tgt] = p; W.fs.tg_raw[tgt] = rt; W.fs.tg_y[tgt] = (int8_t)y;
                        }
                        __syncwarp();
                    }
                    __syncwarp();
                    if (light) DMD_LSUB(5);
                    warp_rp_finish(S, E, W, i, j, 0, tf, imax);
                    if (light) DMD_LSUB(6);
                    if (!light) warp_rp_tnew(W);   /* light: after the marks below */
                } else {
                    warp_repredict(S, E, W, i, j, tf, imax, hbonds, Ver{light ? own + N : nullptr, warea, tseq, warp, P});
                }
#ifdef DMD_PHASE_TIMERS
                if (lane == 0) atomicAdd((unsigned long long *)&g_phase_cycles[DMD_PHASE_CTAS - 2][W.pooled ? 5 : 4], 1ull);
#endif
                DMD_SUB(8);
                if (lane == 0 && W.xpulse) {
                    if (S.ident[i] < S.ident[j]) repuls_del_b(S, i, j); else repuls_del_b(S, j, i);
                }
                __syncwarp();
                if (light) {
                    /* the changed entries only are new: the earliest of them */
                    warp_mark_queue(W, own + 2 * N, my_ticket);
                    warp_rp_tnew(W);
                }
                if (lane == 0) {
                    L->c_tnew_key[gw] = W.tnew_key; L->c_tnew_idx[gw] = W.tnew_idx;
                    L->c_err[gw] = W.err; L->c_err_info[gw] = W.err_info;
                    L->c_ct[gw] = W.ct; L->c_tf[gw] = W.tf;
                }
                if (light) DMD_LSUB(7);
            }
            if (threadIdx.x == 0) { TP.n = 0; TP.nlive = 0; }   /* the pool is free until the next batch */
            csync(C);
            if (light) DMD_LSUB(8);
            if (light) {
                if (gw < P) {
                    const bool bad = warp_check_queue(W, own + 2 * N, my_ticket);
                    if (lane == 0) L->c_qbad[gw] = bad;
                }
                csync(C);
                DMD_LSUB(9);
            }
            DMD_PHASE(3);
            /* validation: event k stands if it precedes every new entry of
             * events 0..k-1; the leader also books the committed events */
            int Vw = P;
            const bool vwarp = C == 1 && P <= 32;
            if (vwarp) {
                /* every warp: a prefix minimum of the events' new entries by
                 * a scan, then the first event that fails */
                const bool in = lane < P;
                long long bk = in ? sh.c_tnew_key[lane] : DMD_KEY_INF;
                int bb = in ? sh.c_tnew_idx[lane] : INT_MAX;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long k2 = __shfl_up_sync(FULL, bk, o);
                    const int b2 = __shfl_up_sync(FULL, bb, o);
                    if (lane >= o && key_less(k2, b2, bk, bb)) { bk = k2; bb = b2; }
                }
                long long ek = __shfl_up_sync(FULL, bk, 1);
                int eb = __shfl_up_sync(FULL, bb, 1);
                int cand = P;
                if (in && lane > 0 &&
                    (!key_less(sh.sort_key[lane], sh.sort_idx[lane], ek, eb) || (light && sh.c_qbad[lane])))
                    cand = lane;
                else if (in && sh.c_err[lane])
                    cand = lane + 1;   /* the run stops after the first event in error */
                Vw = __reduce_min_sync(FULL, cand);
            }
            /* the booking thread: lane 0 of a warp without an event when there
             * is one (so that no event's commit waits for it), else thread 0 */
            const int book_thread = (vwarp && P < RUN_NW) ? 32 * (RUN_NW - 1) : 0;
            if (leader && threadIdx.x == book_thread) {
                int v = P;
                if (vwarp) {
                    v = Vw;
                    if (sh.c_err[v - 1]) set_err(sh, sh.c_err[v - 1], sh.c_err_info[v - 1]);
                } else {
                    long long bk = DMD_KEY_INF;
                    int bb = INT_MAX;
                    for (int k = 0; k < P; ++k) {
                        if (k > 0 && !key_less(sh.sort_key[k], sh.sort_idx[k], bk, bb)) { v = k; break; }
                        /* light batches: it read a queue entry an earlier event changed */
                        if (k > 0 && light && sh.c_qbad[k]) { v = k; break; }
                        if (sh.c_err[k]) {   /* the run stops after the first event in error */
                            set_err(sh, sh.c_err[k], sh.c_err_info[k]);
                            v = k + 1;
                            break;
                        }
                        if (key_less(sh.c_tnew_key[k], sh.c_tnew_idx[k], bk, bb)) { bk = sh.c_tnew_key[k]; bb = sh.c_tnew_idx[k]; }
                    }
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
            if (!vwarp) {
                csync(C);
                if (!leader && threadIdx.x == 0) sh.V = L->V;
                __syncthreads();
            }
            DMD_PHASE(4);
            if (light) DMD_LSUB(10);
            const int V = vwarp ? Vw : sh.V;
            if (light) {
                /* a rolled-back event restores its bead i's coltype, which a
                 * standing earlier event may rewrite: restores land first */
                if (gw < P && gw >= V) warp_restore(S, W);
                if (V < P) csync(C);
                if (gw < V) {
                    warp_commit_preds(S, W);
                    if (lane == 0) log_event(S, sh.log0 + gw, W.coll, sh.tnow, W.tf, W.i, W.j, W.ct, W.evcode);
                }
            } else if (gw < P) {
                if (gw < V) {
                    warp_commit_preds(S, W);
                    if (lane == 0) log_event(S, sh.log0 + gw, W.coll, sh.tnow, W.tf, W.i, W.j, W.ct, W.evcode);
                } else {
                    warp_restore(S, W);
                }
            }
            csync(C);   /* every commit lands before any level-1 group is recomputed */
            if (light) DMD_LSUB(11);
            if (gw < V) warp_l1_refresh(S, W.pb, W.npred);
            if (light) DMD_LSUB(12);
#ifdef DMD_PHASE_TIMERS
            if (light && blockIdx.x == g_sub_cta && threadIdx.x == 0) g_phase_cycles[DMD_PHASE_CTAS - 5][15] += 1;
#endif
        } else if (e == N) {
            ph_kind = 6;
            /* ---- ghost collision: leader warp 0 ---- */
            if (leader && warp == 0) {
                DMD_CSUB(-1);
                double tf = sh.tf_iv;
                const int i = warp_ghost(S, sh, tf, sh.gdraw[gidx & 1]);
                if (lane == 0) { W.i = i; W.tf = tf; }
                __syncwarp();
                DMD_SUB(-1);
                DMD_CSUB(8);
                warp_repredict(S, cta_err(sh), W, i, -1, tf, sh.sc.interval_max, hbonds, Ver{nullptr, warea, 0u, 0, 0});
                DMD_CSUB(9);
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
                DMD_CSUB(10);
                warp_l1_refresh(S, W.pb, W.npred + 1);
                DMD_CSUB(11);
            } else if (leader && warp == 1) {
                /* the next ghost's draws (they depend on the seed and the
                 * ghost index only), while warp 0 handles this one */
                warp_ghost_draws(S, gidx + 1, sh.gdraw[(gidx + 1) & 1]);
            }
        } else if (e == N + 1) {
            ph_kind = 7;
            /* ---- interval: all CTAs ---- */
            double t_before = sh.tnow, tf = sh.tf_iv;
            /* the warp areas are free during an interval: the rebuild's scratch */
            bool rb = cluster_interval(S, sh, L, rank, C, ScratchRef{(char *)&warea[0].fs, sizeof(WarpArea)}, hbonds,
                                       (char *)warea, (int)(RUN_NW * sizeof(WarpArea)));
            if (leader && threadIdx.x == 0) {
                sh.sc.n_interval += 1;
                log_event(S, sh.sc.log_count, sh.sc.coll, t_before, tf, N + 1, -1, rb ? DMD_EV_REBUILD : DMD_EV_INTERVAL, 0);
                /* rebuild-cycle launches end each system at its list rebuild
                 * (the nbor/events call of code/main.F90:1151-1166) */
                if (cycles && rb) sh.sc.stop = 1;
                if (S.log && S.log_cap > 0) sh.sc.log_count += 1;
                sh.sc.old_tfalse = sh.sc.tfalse;
                if (!phys) sh.sc.done += 1;
            }
        } else {
            ph_kind = 8;
            /* ---- output: the leader CTA ---- */
            if (leader) {
                /* the -Ddebugging check of code/main.F90:1193-1205: stop on an
                 * overlap or a broken bond */
                if (S.flags & DMD_FLAG_CHECK_OVERLAP) cta_checkover(S, sh);
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
        if (threadIdx.x == 0) sh.ncand = 0;   /* the next gather may start without a barrier */
        csync(C);
        DMD_PHASE(ph_kind);
    }
    if (use_hot) {   /* the hot arrays back to the system's pool */
        __syncthreads();
        hot_copy(hot_layout(hot, N, S.nl1), systems[r], false);
    }
    if (leader) {
        __syncthreads();
        if (threadIdx.x == 0) {
            sh.sc.run_cycles = clock64() - t_start;
            sh.sc.done_all += sh.sc.done;
            *S.sc = sh.sc;
            /* a rebuild-cycle launch leaves the events still to run */
            if (cycles && targets) targets[r] = target > sh.sc.done ? target - sh.sc.done : 0;
        }
    }
    if (C > 1) cg::this_cluster().sync();   /* no CTA leaves while others may read its shared memory */
}
