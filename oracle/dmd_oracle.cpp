/*
 * dmd_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement, on the CPU and one event at a time, of the serial
 * semantics of the reference PRIME20 DMD program (parallel-dmd-PRIME20/code,
 * Fortran 90 + MPI).  It is the oracle the GB300 engine is tested against and
 * the timed CPU baseline; the engine never calls it.  Each routine cites the reference
 * file:line it restates.  Expressions keep the reference's evaluation order
 * so that, compiled without FMA contraction, they give the same IEEE bits as
 * the CUDA engine.
 *
 * Stated deviations from the reference (each one a deliberate decision):
 *  1. Random numbers come from the Philox streams of dmd_rng.h instead of
 *     the Intel-runtime drandm (unpublished); dmd_log replaces log.
 *  2. The MPI worker block (code/main.F90:1420-1960) runs inline on the
 *     current state; the reference worker reads stale copies of the four
 *     H-bond helper beads (code/repuls_check.f:32-75).
 *  3. Events are committed in strict (time, index) order; the reference's
 *     speculative first-bin batching (code/main.F90:969-993) can reorder.
 *  4. IEEE division (the reference builds with -no-prec-div).
 *  5. Exact time ties between candidate partners are broken by the lower
 *     partner index (the reference takes the first in list order).
 *  6. An ev_code write through a zero helper index (code/main.F90:825-868
 *     when a bond without shoulders dissociates) is skipped; the reference
 *     writes out of bounds there.
 *  7. Chains may have individual sequences and lengths; make_code's per
 *     species blocks are applied per chain, and nbor_setup's cutoffs are
 *     the maximum over every pair type present.
 */
#include "dmd.h"
#include "dmd_oracle.h"
#include "dmd_rng.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

/* code/def.h:1-61 */
const double LTSTEP = 1e-10, SMDIST = 5e-12;
const double DNC = 1.46, DCC = 1.51, DCN = 1.33, DCACA = 3.8, DTIE = 2.41, DTIE2 = 2.45;
const double SQZ1 = 1.1436, SQZ2 = 0.88, SQZ3 = 0.87829, SQZ4 = 0.8, SQZ5 = 0.7713, SQZ11 = 1.0;
const int N_B_HYDRO = 3, N_B_HBOND = 3;
const double DEL = 0.02375;
const int XREPULS1 = 40, XREPULS2 = 50;

inline double dnint(double x) { return std::round(x); }

struct Oracle {
    /* run settings */
    double setemp = 0, t_fact = 0, n_forced = 0, interval = 0, interval_max = 0, avegtime = 0;
    double rl_const = 1.2;
    int n_wrap = 2, numbin = 2000;
    bool canon = true, hbonds = true;
    uint64_t seed = 0;
    int flags = 0;
    int chaptype = 1, species2_chain = 0;   /* -Dchaptype; chains species2_chain.. are species 2 */

    /* system */
    int N = 0, nchains = 0;
    std::vector<int> chain_start, chain_L, chain_nb;  /* 0-based start */
    std::vector<int> chain_of, local_of;              /* per bead (0-based bead), local 1-based */
    std::vector<std::vector<int>> fside;              /* per chain, residue k (1-based) -> local R index or 0 */
    std::vector<std::vector<int>> hp;                 /* per chain, local (1-based) */
    std::vector<std::vector<double>> bdln, bl_rn, bl_rc, del_bdln, del_blrn, del_blrc; /* per chain per residue */

    /* state, 1-based arrays of size N+4 */
    std::vector<double> sx, sy, sz, vx, vy, vz, bm, old_rx, old_ry, old_rz;
    std::vector<int> identity, bptnr;
    std::vector<int> er;  /* extra_repuls(k,1..4) at er[k*4 + (m-1)] */
    std::vector<double> tim;
    std::vector<int> nptnr, coltype;
    std::vector<char> queued;
    std::vector<int8_t> ev;  /* ev_code(a,b) at ev[(a-1)*N + (b-1)] */
    double t = 0, tfalse = 0, old_tfalse = 0, boxl_orig = 0, boxl = 1.0, half = 0.5;
    int64_t coll = 0;

    /* tables */
    double sigma[29] = {}, welldia[29] = {}, epsilon_[29] = {};
    double sigma_sq[29][29] = {}, sigma_2b[29][29] = {}, welldia_sq[29][29] = {};
    double ep_sqrt[29][29] = {}, shlddia_sq[29][29] = {}, bds[29][29] = {}, wel[29][29] = {}, ep[29][29] = {};
    double sqz610[6][29] = {};
    double ev_param[4][51];
    double shder_dist1 = 0, shder_dist2 = 0, shder_dist3 = 0, shder_dist4 = 0;
    double sig_max[51] = {}, sig_max_all = 0, rlsq[51] = {}, hdelr = 0;

    /* neighbour lists (code/nbor.f) */
    int cap = 128;
    std::vector<int> nb, na_npt, dnnab, nnabdn;  /* nb[(i-1)*cap + k] */
    int num_cell = 0;
    double width = 0;
    std::vector<int> cell, clinks, wrap_map, map;

    /* event queue: membership follows code/add_tbin.f / del_tbin.f (an
     * entry is queued when its time is below the horizon interval_max at
     * scheduling); extraction is an exact (time, index) minimum kept in a
     * tournament tree instead of the calendar's first-bin sort. */
    int P = 1;
    std::vector<double> tkey;
    std::vector<int> tidx;
    /* counters */
    int64_t nevents[32] = {};
    int64_t numghosts = 0, nupdates = 0, nforcedupdate = 0, n_pair = 0, n_interval = 0, n_output = 0;
    int64_t ghost_index = 0;

    std::string err;

    int8_t &E(int a, int b) { return ev[(size_t)(a - 1) * N + (b - 1)]; }
    int code(int a, int b) const { return ev[(size_t)(a - 1) * N + (b - 1)]; }
    int &ER(int k, int m) { return er[(size_t)k * 4 + (m - 1)]; }
    int erv(int k, int m) const { return er[(size_t)k * 4 + (m - 1)]; }

    /* ------------------------------------------------------------------ */
    /* input surface: code/inputinfo.f:5-669 and code/scale_down.f:1-87   */
    /* ------------------------------------------------------------------ */
    bool setup(const dmd_run_cfg *cfg, const dmd_tables *T, const dmd_system *S) {
        setemp = cfg->tstar * 12.0;                       /* main.F90:126-127 */
        t_fact = cfg->t_fact > 0 ? cfg->t_fact : 0.00005;  /* main.F90:144 */
        n_forced = cfg->n_forced > 0 ? cfg->n_forced : 150.0;
        rl_const = cfg->rl_const > 0 ? cfg->rl_const : 1.2;
        n_wrap = cfg->n_wrap > 0 ? cfg->n_wrap : 2;
        numbin = cfg->numbin > 0 ? cfg->numbin : 2000;
        canon = cfg->canon != 0;
        hbonds = cfg->hbonds != 0;
        seed = cfg->seed;
        chaptype = cfg->chaptype == 2 ? 2 : 1;
        species2_chain = cfg->species2_chain;
        flags = cfg->flags;
        cap = cfg->list_cap > 0 ? cfg->list_cap : 128;
        if (n_wrap != 2) { err = "oracle supports n_wrap=2 only"; return false; }
        interval = t_fact / std::sqrt(setemp);             /* main.F90:146 */
        interval_max = n_forced * interval;
        avegtime = 0.00005 / std::sqrt(setemp);            /* main.F90:156 */

        N = S->n_beads;
        nchains = S->n_chains;
        chain_start.resize(nchains); chain_L.resize(nchains); chain_nb.resize(nchains);
        fside.assign(nchains, {}); hp.assign(nchains, {});
        bdln.assign(nchains, {}); bl_rn = bdln; bl_rc = bdln; del_bdln = bdln; del_blrn = bdln; del_blrc = bdln;
        chain_of.assign(N + 4, -1); local_of.assign(N + 4, 0);
        identity.assign(N + 4, 0);
        int pos = 0, rpos = 0;
        for (int c = 0; c < nchains; ++c) {
            int L = S->chain_len[c];
            if (L < 3) { err = "chain shorter than 3 residues"; return false; }
            int nr = 0;
            for (int k = 0; k < L; ++k) {
                int r = S->residues[rpos + k];
                if (r < 9 || r > 28) { err = "residue identity out of 9..28"; return false; }
                if (r != 9) ++nr;
            }
            int nbc = 3 * L + nr;
            chain_start[c] = pos; chain_L[c] = L; chain_nb[c] = nbc;
            if (pos + nbc > N) { err = "n_beads smaller than the chains need"; return false; }
            fside[c].assign(L + 1, 0);
            hp[c].assign(nbc + 1, 0);
            /* code/inputinfo.f:103-131: firstside -> local index of R */
            int l = 1;
            for (int k = 1; k <= L; ++k) {
                if (S->residues[rpos + k - 1] != 9) { fside[c][k] = 3 * L + l; ++l; }
            }
            for (int k = 1; k <= L; ++k) {
                identity[pos + k] = 2;            /* C-alpha */
                identity[pos + L + k] = 1;        /* NH */
                identity[pos + 2 * L + k] = 4;    /* CO */
                if (fside[c][k]) identity[pos + fside[c][k]] = S->residues[rpos + k - 1];
            }
            for (int q = 1; q <= nbc; ++q) {
                chain_of[pos + q] = c; local_of[pos + q] = q;
                hp[c][q] = S->hp ? S->hp[pos + q - 1] : (q > 3 * L ? 1 : 0);
            }
            pos += nbc;
            rpos += L;
        }
        if (pos != N) { err = "n_beads larger than the chains need"; return false; }

        /* protein.data (inputinfo.f:152-200) */
        for (int k = 0; k < 29; ++k) { sigma[k] = welldia[k] = epsilon_[k] = 0; }
        for (int k = 1; k <= 4; ++k) {
            sigma[k] = T->sigma[k - 1]; welldia[k] = T->welldia[k - 1]; epsilon_[k] = T->epsilon[k - 1];
            sigma[k + 4] = sigma[k]; welldia[k + 4] = welldia[k]; epsilon_[k + 4] = epsilon_[k];
        }
        for (int a = 9; a <= 28; ++a)
            for (int b = 9; b <= 28; ++b) {
                bds[a][b] = T->bds[a - 9][b - 9];
                wel[a][b] = T->wel[a - 9][b - 9];
                ep[a][b] = -T->ep[a - 9][b - 9];          /* inputinfo.f:280-286 */
            }
        for (int i = 9; i <= 28; ++i) { sigma[i] = 1.00 * bds[i][i]; welldia[i] = 1.5 * sigma[i]; }
        sigma[9] = 1.00 * bds[9][9] - 1.2;                 /* inputinfo.f:402 */
        for (int i = 1; i <= 20; ++i) {                     /* inputinfo.f:403-413 */
            double sz8 = T->sqz[i - 1][0], sz6 = T->sqz[i - 1][1], sz7 = T->sqz[i - 1][2],
                   sz9 = T->sqz[i - 1][3], sz10 = T->sqz[i - 1][4];
            sqz610[1][i + 8] = sz6 * 2 / (sigma[i + 8] + sigma[4]);
            sqz610[2][i + 8] = sz7 * 2 / (sigma[i + 8] + sigma[1]);
            sqz610[3][i + 8] = sz8 * 2 / (sigma[i + 8] + sigma[2]);
            sqz610[4][i + 8] = sz9 * 2 / (sigma[i + 8] + sigma[2]);
            sqz610[5][i + 8] = sz10 * 2 / (sigma[i + 8] + sigma[4]);
        }
        /* masses (inputinfo.f:416-432) */
        double bmass[29] = {};
        for (int k = 1; k <= 28; ++k) bmass[k] = T->mass[k];
        bmass[3] = bmass[20];
        for (int k = 1; k <= 4; ++k) bmass[k + 4] = bmass[k];
        bm.assign(N + 4, 0);
        for (int i = 1; i <= N; ++i) bm[i] = bmass[identity[i]];
        /* per-residue bond tables (inputinfo.f:288-355) */
        double drca[21], drnh[21], drco[21], dra[21], drn[21], drc[21];
        for (int i = 1; i <= 20; ++i) {
            drca[i] = T->rca[i - 1]; drnh[i] = T->rnh[i - 1]; drco[i] = T->rco[i - 1];
            dra[i] = T->del_rca[i - 1] < DEL ? DEL : T->del_rca[i - 1];
            drn[i] = T->del_rnh[i - 1] < DEL ? DEL : T->del_rnh[i - 1];
            drc[i] = T->del_rco[i - 1] < DEL ? DEL : T->del_rco[i - 1];
        }
        boxl_orig = S->boxl;
        rpos = 0;
        for (int c = 0; c < nchains; ++c) {
            int L = chain_L[c];
            bdln[c].assign(L + 1, 0); bl_rn[c] = bdln[c]; bl_rc[c] = bdln[c];
            del_bdln[c] = bdln[c]; del_blrn[c] = bdln[c]; del_blrc[c] = bdln[c];
            for (int k = 1; k <= L; ++k) {
                int r = S->residues[rpos + k - 1];
                int iii = fside[c][k] ? r - 8 : 1;
                bdln[c][k] = drca[iii]; bl_rn[c][k] = drnh[iii]; bl_rc[c][k] = drco[iii];
                del_bdln[c][k] = dra[iii]; del_blrn[c][k] = drn[iii]; del_blrc[c][k] = drc[iii];
            }
            rpos += L;
        }
        /* positions, velocities (main.F90 runr path: positions already in box units) */
        sx.assign(N + 4, 0); sy = sx; sz = sx; vx = sx; vy = sx; vz = sx;
        for (int i = 1; i <= N; ++i) {
            sx[i] = S->x[i - 1]; sy[i] = S->y[i - 1]; sz[i] = S->z[i - 1];
            vx[i] = S->vx[i - 1]; vy[i] = S->vy[i - 1]; vz[i] = S->vz[i - 1];
        }
        scale_down();
        make_code();

        /* main.F90:198-234 */
        t = S->t0; tfalse = 0;
        coll = S->coll0;
        old_rx.assign(N + 4, 0); old_ry = old_rx; old_rz = old_rx;
        tim.assign(N + 4, 0); nptnr.assign(N + 4, 0); coltype.assign(N + 4, 0); queued.assign(N + 4, 0);
        bptnr.assign(N + 4, 0); er.assign((size_t)(N + 4) * 4, 0);
        for (int k = 1; k <= N; ++k) {
            sx[k] = sx[k] - dnint(sx[k]); sy[k] = sy[k] - dnint(sy[k]); sz[k] = sz[k] - dnint(sz[k]);
            old_rx[k] = sx[k]; old_ry[k] = sy[k]; old_rz[k] = sz[k];
            tim[k] = interval_max + LTSTEP; coltype[k] = -1; nptnr[k] = -1;
        }
        for (int k = N + 1; k <= N + 3; ++k) { nptnr[k] = -2; coltype[k] = -2; }
        nbor_setup();   /* main.F90:389; evaluated on the make_code table, before the restore's shoulders */
        if (S->bptnr) runr_restore(S->bptnr);
        if (!(flags & DMD_FLAG_ALLOW_OVERLAP)) {   /* main.F90:347, before the lists and predictions */
            int bi = 0, bj = 0;
            if (checkover(bi, bj) > 0) {
                err = "beads " + std::to_string(bi) + " and " + std::to_string(bj) +
                      " overlap, or their bond is outside its window";
                return false;
            }
        }

        num_cell = (int)(boxl / (sig_max_all * rl_const) * n_wrap) + 2 * n_wrap;
        if (num_cell - 2 * n_wrap < 2 * n_wrap + 1) { err = "box too small for the cell stencil"; return false; }
        width = boxl / (double)(num_cell - 2 * n_wrap);
        half = boxl / 2.0;
        cell_link();
        nbor();
        if (!err.empty()) return false;
        if (canon) {                                       /* main.F90:408-415 */
            double tgho = 0.0;
            uint32_t k = 0;
            while ((tgho < 1e-18) || (tgho == 1.0)) tgho = dmd_uniform(seed, DMD_STREAM_GHOST0, 0, k++);
            tim[N + 1] = -1.0 * dmd_log(tgho) * avegtime * .0000001;
        } else {
            tim[N + 1] = 1000000000.0;
        }
        tim[N + 2] = interval;
        tim[N + 3] = 3.3 / (std::sqrt(setemp)) + 5;
        events();
        old_tfalse = tfalse;
        return err.empty();
    }

    /* code/checkover.f:18-131: every pair i < j; a pair of type 1 or >= 15
     * closer than its core diameter, a bonded pair (4-12) outside its window.
     * Returns the number of offending pairs; (bi, bj) the first (1-based). */
    int checkover(int &bi, int &bj) const {
        int nbad = 0;
        for (int i = 1; i <= N - 1; ++i)
            for (int j = i + 1; j <= N; ++j) {
                int evcode = code(j, i);
                bool bad = false;
                if (evcode == 1 || evcode >= 15) {
                    double p = ev_param[1][evcode];
                    double sigsq = sigma_sq[identity[i]][identity[j]] * (p * p);
                    if (evcode >= 22 && evcode <= 26) {
                        int k = std::max(identity[i], identity[j]);
                        double s = sqz610[evcode - 21][k];
                        sigsq = sigsq * (s * s);
                    }
                    Rel r = rel(i, j);
                    double rijsq = r.rijsq * 1.0000000001;
                    bad = rijsq <= sigsq;
                } else if (evcode >= 4 && evcode <= 12) {
                    double blmin, blmax;
                    bond_limits(i, evcode, blmin, blmax);
                    blmin = blmin * blmin;
                    blmax = blmax * blmax;
                    Rel r = rel(i, j);
                    double rijsq_min = r.rijsq * 1.0000000001, rijsq_max = r.rijsq * 0.9999999999;
                    bad = rijsq_max > blmax || rijsq_min < blmin;
                }
                if (bad && nbad++ == 0) { bi = i; bj = j; }
            }
        return nbad;
    }

    /* code/check_nc_int.f:9-360: over every bead's up list, the H-bonded
     * pairs whose geometry fails repuls_check and the unbonded NH-CO pairs
     * inside their well whose geometry passes it; pairs with an end bead
     * (local index chnln+1 or 3*chnln) are not rated. */
    void check_nc_int(int64_t &boundbad, int64_t &unboundbad) const {
        boundbad = unboundbad = 0;
        for (int i = 1; i <= N; ++i)
            for (int k = 0; k < na_npt[i]; ++k) {
                int j = nb[(size_t)(i - 1) * cap + k];
                if (code(j, i) != 15) continue;
                int ci = chain_of[i], cj = chain_of[j];
                int ii = local_of[i], jj = local_of[j], Li = chain_L[ci], Lj = chain_L[cj];
                bool rated = ii != Li + 1 && jj != Lj + 1 && ii != 3 * Li && jj != 3 * Lj;
                if (bptnr[i] == j) {
                    double rating = 10.0;
                    if (rated) rating = identity[i] < identity[j] ? repuls_check(i, j) : repuls_check(j, i);
                    if (rating > 10.0) boundbad += 1;
                } else {
                    Rel r = rel(i, j);
                    double diff = r.rijsq - welldia_sq[identity[i]][identity[j]];
                    if (diff < 0.0) {
                        double rating = 11.0;
                        if (rated) rating = identity[i] < identity[j] ? repuls_check(i, j) : repuls_check(j, i);
                        if (rating <= 10.0) unboundbad += 1;
                    }
                }
            }
    }

    void scale_down() {  /* code/scale_down.f:1-87 */
        /* positions arrive in box units (the runr path skips their scaling, scale_down.f:18-25) */
        for (int k = 1; k <= 28; ++k) { sigma[k] = sigma[k] / boxl_orig; welldia[k] = welldia[k] / boxl_orig; }
        shder_dist1 = 5.00 / boxl_orig;
        shder_dist2 = 4.74 / boxl_orig;
        shder_dist3 = 4.86 / boxl_orig;
        shder_dist4 = 4.83 / boxl_orig;
        for (int k = 1; k <= 28; ++k)
            for (int kk = 1; kk <= 28; ++kk) {
                double s = sigma[k] + sigma[kk];
                sigma_sq[k][kk] = 0.25 * (s * s);
                sigma_2b[k][kk] = 0.50 * (sigma[k] + sigma[kk]);
                double w = welldia[k] + welldia[kk];
                welldia_sq[k][kk] = 0.25 * (w * w);
                ep_sqrt[k][kk] = std::sqrt(epsilon_[k] * epsilon_[kk]);
                shlddia_sq[k][kk] = shder_dist4 * shder_dist4;
            }
        for (int k = 9; k <= 28; ++k)
            for (int kk = 9; kk <= 28; ++kk) {
                ep_sqrt[k][kk] = epsilon_[1] * ep[k][kk];
                sigma_sq[k][kk] = (bds[k][kk] * bds[k][kk]) / (boxl_orig * boxl_orig);
                sigma_2b[k][kk] = bds[k][kk] / boxl_orig;
                welldia_sq[k][kk] = (wel[k][kk] * wel[k][kk]) / (boxl_orig * boxl_orig);
            }
        double d1 = shder_dist1 * shder_dist1, d2 = shder_dist2 * shder_dist2, d3 = shder_dist3 * shder_dist3;
        shlddia_sq[1][2] = d1; shlddia_sq[2][1] = d1; shlddia_sq[5][2] = d1; shlddia_sq[2][5] = d1;
        shlddia_sq[1][1] = d2; shlddia_sq[5][5] = d2; shlddia_sq[1][5] = d2; shlddia_sq[5][1] = d2;
        shlddia_sq[2][4] = d3; shlddia_sq[4][2] = d3; shlddia_sq[2][8] = d3; shlddia_sq[8][2] = d3;
        for (int c = 0; c < nchains; ++c)
            for (int k = 1; k <= chain_L[c]; ++k) {
                bdln[c][k] = bdln[c][k] / boxl_orig;
                bl_rn[c][k] = bl_rn[c][k] / boxl_orig;
                bl_rc[c][k] = bl_rc[c][k] / boxl_orig;
            }
        boxl = 1.0;
        half = boxl / 2.0;
    }

    /* ------------------------------------------------------------------ */
    /* code/make_code.f:6-573, literal dense table, applied per chain      */
    /* ------------------------------------------------------------------ */
    void make_code() {
        for (int k = 0; k < 4; ++k) for (int l = 0; l < 51; ++l) ev_param[k][l] = 1;
        ev_param[1][15] = 1.05 * ((2.24 / boxl_orig) / ((sigma[1] + sigma[4]) / 2.0));
        ev_param[1][17] = SQZ1; ev_param[1][18] = SQZ2; ev_param[1][19] = SQZ3;
        ev_param[1][20] = SQZ4; ev_param[1][21] = SQZ5; ev_param[1][27] = SQZ11;
        ev_param[2][4] = DNC * (1.0 - DEL) / boxl_orig;
        ev_param[2][5] = DCC * (1.0 - DEL) / boxl_orig;
        ev_param[2][6] = DCN * (1.0 - DEL) / boxl_orig;
        ev_param[2][7] = DTIE * (1.0 - DEL) / boxl_orig;
        ev_param[2][8] = DTIE2 * (1.0 - DEL) / boxl_orig;
        ev_param[2][9] = DCACA * (1.0 - DEL) / boxl_orig;
        ev_param[2][10] = (1.0 - DEL); ev_param[2][11] = (1.0 - DEL); ev_param[2][12] = (1.0 - DEL);
        ev_param[3][4] = DNC * (1.0 + DEL) / boxl_orig;
        ev_param[3][5] = DCC * (1.0 + DEL) / boxl_orig;
        ev_param[3][6] = DCN * (1.0 + DEL) / boxl_orig;
        ev_param[3][7] = (1.0 + DEL) * DTIE / boxl_orig;
        ev_param[3][8] = (1.0 + DEL) * DTIE2 / boxl_orig;
        ev_param[3][9] = (1.0 + DEL) * DCACA / boxl_orig;
        ev_param[3][10] = (1.0 + DEL); ev_param[3][11] = (1.0 + DEL); ev_param[3][12] = (1.0 + DEL);

        ev.assign((size_t)N * N, 1);
        /* inter-chain side chains (make_code.f:80-108) */
        for (int m = 1; m <= N - 1; ++m)
            for (int l = m + 1; l <= N; ++l)
                if (identity[m] > 8 && identity[l] > 8)
                    if (hp[chain_of[m]][local_of[m]] == 1 && hp[chain_of[l]][local_of[l]] == 1)
                        if (chain_of[l] != chain_of[m]) E(m, l) = 16;
        if (hbonds) {
            /* all NH-CO pairs (make_code.f:114-122) */
            for (int m = 1; m <= N - 1; ++m)
                for (int l = m + 1; l <= N; ++l)
                    if ((identity[m] == 1 && identity[l] == 4) || (identity[m] == 4 && identity[l] == 1)) E(m, l) = 15;
            /* same-chain pairs back to core (make_code.f:125-141) */
            for (int c = 0; c < nchains; ++c) {
                int kk = chain_start[c];
                for (int m = kk + 1; m <= kk + chain_nb[c] - 1; ++m)
                    for (int l = m + 1; l <= kk + chain_nb[c]; ++l) E(m, l) = 1;
            }
            /* proline NH (make_code.f:143-169) */
            for (int m = 1; m <= N - 1; ++m)
                for (int l = m + 1; l <= N; ++l) {
                    if (identity[m] == 17 && identity[l] == 4) E(m - 2 * chain_L[chain_of[m]], l) = 1;
                    else if (identity[m] == 4 && identity[l] == 17) E(l - 2 * chain_L[chain_of[l]], m) = 1;
                }
        } else {
            for (int c = 0; c < nchains; ++c) {
                int kk = chain_start[c];
                for (int m = kk + 1; m <= kk + chain_nb[c] - 1; ++m)
                    for (int l = m + 1; l <= kk + chain_nb[c]; ++l) E(m, l) = 1;
            }
        }
        for (int c = 0; c < nchains; ++c) {  /* make_code.f:175-325 */
            int lll = chain_start[c], L = chain_L[c];
            const std::vector<int> &fs = fside[c];
            auto setc = [&](int a, int b, int v) { if (a >= 1 && a <= N && b >= 1 && b <= N) E(a, b) = v; };
            int ncount = 2 + N_B_HYDRO;
            for (int k = 1; k <= L; ++k) {
                if (fs[k] != 0)
                    for (int l = ncount; l <= L; ++l)
                        if (fs[l] != 0)
                            if (hp[c][fs[k]] == 1 && hp[c][fs[l]] == 1) setc(lll + fs[k], lll + fs[l], 16);
                ncount = ncount + 1;
            }
            if (hbonds) {
                for (int k = lll + L + 1; k <= lll + 2 * L; ++k)
                    for (int l = lll + 2 * L + 1; l <= lll + 3 * L; ++l) setc(k, l, 15);
                for (int k = lll + L + 1; k <= lll + 2 * L; ++k)
                    for (int l = k + L - N_B_HBOND; l <= k + L + N_B_HBOND; ++l) setc(k, l, 1);
            }
            for (int k = lll + 1; k <= lll + L; ++k) setc(k, L + k, 4);
            for (int k = lll + 1; k <= lll + L; ++k) setc(k, 2 * L + k, 5);
            for (int k = lll + L + 2; k <= lll + 2 * L; ++k) setc(k, k + L - 1, 6);
            for (int k = lll + 1; k <= lll + L - 1; ++k) setc(k, L + k + 1, 7);
            for (int k = lll + 2; k <= lll + L; ++k) setc(k, 2 * L + k - 1, 8);
            for (int k = lll + L + 1; k <= lll + 2 * L; ++k) setc(k, k + L, 8);
            for (int k = lll + 1; k <= lll + L - 1; ++k) setc(k, k + 1, 9);
            for (int k = lll + 1; k <= lll + L; ++k) if (fs[k - lll] != 0) setc(k, lll + fs[k - lll], 10);
            for (int k = lll + L + 1; k <= lll + 2 * L; ++k) if (fs[k - lll - L] != 0) setc(k, lll + fs[k - lll - L], 11);
            for (int k = lll + 2 * L + 1; k <= lll + 3 * L; ++k) if (fs[k - lll - 2 * L] != 0) setc(k, lll + fs[k - lll - 2 * L], 12);
            for (int k = lll + 1; k <= lll + L - 1; ++k) setc(k, k + 2 * L + 1, 17);
            for (int k = lll + 2; k <= lll + L; ++k) setc(k, k + L - 1, 18);
            for (int k = lll + L + 3; k <= lll + 2 * L; ++k) setc(k, k + L - 2, 19);
            for (int k = lll + L + 1; k <= lll + 2 * L - 1; ++k) setc(k, k + 1, 20);
            for (int k = lll + 2 * L + 1; k <= lll + 3 * L - 1; ++k) setc(k, k + 1, 21);
            for (int k = lll + 2 * L + 1; k <= lll + 3 * L - 1; ++k) if (fs[k - lll - 2 * L + 1] != 0) setc(k, lll + fs[k - lll - 2 * L + 1], 22);
            for (int k = lll + L + 2; k <= lll + 2 * L; ++k) if (fs[k - lll - L - 1] != 0) setc(k, lll + fs[k - lll - L - 1], 23);
            for (int k = lll + 1; k <= lll + L - 1; ++k) if (fs[k - lll + 1] != 0) setc(k, lll + fs[k - lll + 1], 24);
            for (int k = lll + 2; k <= lll + L; ++k) if (fs[k - lll - 1] != 0) setc(k, lll + fs[k - lll - 1], 25);
            for (int k = lll + 2 * L + 1; k <= lll + 3 * L - 2; ++k) if (fs[k - lll - 2 * L + 2] != 0) setc(k, lll + fs[k - lll - 2 * L + 2], 26);
        }
        if (chaptype == 2) {
            /* make_code.f:489-514: hydrophobic side chains of two chains meet
             * in the well; make_code.f:516-541: of two species-2 chains, as
             * hard cores */
            for (int m = 1; m <= N - 1; ++m)
                for (int l = m + 1; l <= N; ++l)
                    if (identity[m] > 8 && identity[l] > 8)
                        if (hp[chain_of[m]][local_of[m]] == 1 && hp[chain_of[l]][local_of[l]] == 1)
                            if (chain_of[l] != chain_of[m]) E(m, l) = 16;
            for (int m = 1; m <= N - 1; ++m) {
                if (chain_of[m] < species2_chain) continue;
                for (int l = m + 1; l <= N; ++l)
                    if (identity[m] > 8 && identity[l] > 8)
                        if (hp[chain_of[m]][local_of[m]] == 1 && hp[chain_of[l]][local_of[l]] == 1)
                            if (chain_of[l] != chain_of[m]) E(m, l) = 1;
            }
        }
        for (int i = 1; i <= N - 1; ++i)       /* make_code.f:560-566 */
            for (int j = i + 1; j <= N; ++j) E(j, i) = E(i, j);
    }

    /* ------------------------------------------------------------------ */
    bool is_end(int b) const {  /* local NH_1 or CO_L (main.F90:1477-1485 ii/jj tests) */
        int c = chain_of[b];
        int L = chain_L[c];
        int q = local_of[b];
        return q == L + 1 || q == 3 * L;
    }

    void repuls_add(int i, int j) {  /* code/repuls_add.f:1-51; i = NH, j = CO */
        int Li = chain_L[chain_of[i]], Lj = chain_L[chain_of[j]];
        int ncim1 = i + Li - 1, ncai = i - Li;
        int ncaj = j - 2 * Lj, nnjp1 = j - Lj + 1;
        E(ncaj, i) = XREPULS2; E(i, ncaj) = XREPULS1;
        E(i, nnjp1) = XREPULS1; E(nnjp1, i) = XREPULS2;
        E(ncai, j) = XREPULS2; E(j, ncai) = XREPULS1;
        E(j, ncim1) = XREPULS1; E(ncim1, j) = XREPULS2;
        ER(i, 1) = ncaj; ER(i, 2) = nnjp1; ER(ncaj, 3) = i; ER(nnjp1, 3) = i;
        ER(j, 1) = ncai; ER(j, 2) = ncim1; ER(ncai, 3) = j; ER(ncim1, 3) = j;
        ER(i, 4) = j; ER(j, 4) = i;
    }
    void shoulders_off(int n, int c) {
        /* master application of a dissociation (code/main.F90:825-868): the
         * helper pairs named by extra_repuls go back to core */
        int ncaj = erv(n, 1), nnjp1 = erv(n, 2), ncai = erv(c, 1), ncim1 = erv(c, 2);
        if (ncaj) { E(ncaj, n) = 1; E(n, ncaj) = 1; }
        if (nnjp1) { E(n, nnjp1) = 1; E(nnjp1, n) = 1; }
        if (ncai) { E(ncai, c) = 1; E(c, ncai) = 1; }
        if (ncim1) { E(c, ncim1) = 1; E(ncim1, c) = 1; }
    }
    void repuls_del_b(int i, int j) {  /* code/repuls_del_b.f:1-43 */
        int Li = chain_L[chain_of[i]], Lj = chain_L[chain_of[j]];
        int ncim1 = i + Li - 1, ncai = i - Li;
        int ncaj = j - 2 * Lj, nnjp1 = j - Lj + 1;
        ER(i, 1) = 0; ER(i, 2) = 0; ER(ncaj, 3) = 0; ER(nnjp1, 3) = 0;
        ER(j, 1) = 0; ER(j, 2) = 0; ER(ncai, 3) = 0; ER(ncim1, 3) = 0;
        ER(i, 4) = 0; ER(j, 4) = 0;
    }

    void runr_restore(const int32_t *bp) {  /* code/main.F90:240-321 */
        for (int k = 1; k <= N; ++k) bptnr[k] = bp[k - 1];
        for (int k = 1; k <= N - 1; ++k)
            for (int kj = k + 1; kj <= N; ++kj) {
                if (identity[k] + identity[kj] == 5 && code(k, kj) == 15) {
                    double rx = sx[k] - sx[kj], ry = sy[k] - sy[kj], rz = sz[k] - sz[kj];
                    rx = rx - dnint(rx); ry = ry - dnint(ry); rz = rz - dnint(rz);
                    double r2 = rx * rx + ry * ry + rz * rz;
                    double diff = r2 - welldia_sq[identity[k]][identity[kj]];
                    if (diff < 0.0 && !is_end(k) && !is_end(kj)) {
                        if (identity[k] == 1) repuls_add(k, kj); else repuls_add(kj, k);
                    }
                }
                if (kj == bptnr[k]) {
                    if (identity[k] == 1) { identity[k] = 5; identity[kj] = 8; }
                    else { identity[k] = 8; identity[kj] = 5; }
                }
            }
    }

    /* ------------------------------------------------------------------ */
    /* neighbour lists: code/nbor_setup.f, cell_link.f, cell_add.f, nbor.f */
    /* ------------------------------------------------------------------ */
    double sig_of(int evcode, int a, int b) const {  /* nbor_setup.f:22-38 */
        if (evcode <= 3) return sigma_2b[identity[a]][identity[b]];
        if (evcode == 15) return 0.5 * (welldia[identity[a]] + welldia[identity[b]]);
        if (evcode == 16) return wel[identity[a]][identity[b]] / boxl_orig;
        return 0.0;
    }
    void nbor_setup() {
        sig_max_all = 0.0;
        for (int i = 0; i <= 50; ++i) sig_max[i] = 0.0;
        auto visit = [&](int a, int b) {
            int e = code(b, a);
            if (e <= 26) {
                double s = sig_of(e, a, b);
                if (s > sig_max[e]) { sig_max[e] = s; if (sig_max[e] > sig_max_all) sig_max_all = sig_max[e]; }
            }
        };
        /* every pair present (generalisation of the per-species loops of
         * nbor_setup.f:16-95 to chains of individual sequences) */
        for (int a = 1; a <= N - 1; ++a)
            for (int b = a + 1; b <= N; ++b) visit(a, b);
        double sigij = 0.0, sg = 0.0;
        for (int i = 1; i <= 4; ++i)
            for (int j = 1; j <= 4; ++j) {
                if ((i != 3) || (j != 3)) sg = sigma[i] + sigma[j];
                if (sg > sigij) sigij = sg;
            }
        for (int i = 40; i <= 50; ++i) {
            sig_max[i] = 0.5 * sigij * 1.0;
            if (sig_max[i] > sig_max_all) sig_max_all = sig_max[i];
        }
        for (int i = 1; i <= 50; ++i) {
            rlsq[i] = 0.0;
            if (sig_max[i] != 0.0) { double r = (rl_const - 1) * sig_max_all + sig_max[i]; rlsq[i] = r * r; }
        }
        double rl = rl_const * sig_max_all;
        double h = 0.4 * (rl - sig_max_all);
        hdelr = h * h;
    }
    void cell_link() {  /* code/cell_link.f:1-96 (n_wrap = 2) */
        int nc = num_cell;
        auto icell = [&](int ix, int iy, int iz) {
            return 1 + (ix - 1 + nc) % nc + ((iy - 1 + nc) % nc) * nc + ((iz - 1 + nc) % nc) * nc * nc;
        };
        const int o[5] = {0, 1, -1, 2, -2};
        const int oy[3] = {0, 1, 2};
        map.clear();
        for (int iz = 1; iz <= 3; ++iz) {
            int dz = o[iz - 1];
            for (int iy = 1; iy <= 2; ++iy) {
                int dy = o[iy - 1];
                for (int ix = 1; ix <= 3; ++ix) {
                    int dx = o[ix - 1];
                    if (dy == 0) {
                        if (dz < 1) { if (dx < 1) continue; }
                        else if (dx < 0) continue;
                    }
                    map.push_back(dx + (dy + dz * nc) * nc);
                }
            }
        }
        for (int iz = 1; iz <= 5; ++iz) {
            int dz = o[iz - 1];
            for (int iy = 1; iy <= 3; ++iy) {
                int dy = oy[iy - 1];
                int min_ix = (iz < 4 && iy != 3) ? 4 : 1;
                for (int ix = min_ix; ix <= 5; ++ix) {
                    int dx = o[ix - 1];
                    if (dy == 0) {
                        if (dz < 1) { if (dx < 1) continue; }
                        else if (dx < 0) continue;
                    }
                    map.push_back(dx + (dy + dz * nc) * nc);
                }
            }
        }
        wrap_map.assign((size_t)nc * nc * nc + 1, 0);
        auto wrapc = [&](int i) {
            if (i <= n_wrap) return i + nc - 2 * n_wrap;
            if (nc - i < n_wrap) return i - nc + 2 * n_wrap;
            return i;
        };
        for (int ix = 1; ix <= nc; ++ix)
            for (int iy = 1; iy <= nc; ++iy)
                for (int iz = 1; iz <= nc; ++iz)
                    wrap_map[icell(ix, iy, iz)] = icell(wrapc(ix), wrapc(iy), wrapc(iz));
        cell.assign((size_t)nc * nc * nc + 2, 0);
        clinks.assign(N + 4, 0);
    }
    void cell_add() {  /* code/cell_add.f:1-48 */
        int nc = num_cell;
        std::fill(clinks.begin(), clinks.end(), 0);
        std::fill(cell.begin(), cell.end(), 0);
        for (int k = 1; k <= N; ++k) {
            int x = (int)((sx[k] + half) / width) + n_wrap;
            int y = (int)((sy[k] + half) / width) + n_wrap;
            int z = (int)((sz[k] + half) / width) + n_wrap;
            int ck = 1 + x + y * nc + z * nc * nc;
            clinks[k] = cell[ck];
            cell[ck] = k;
        }
    }
    void add_pair(int i, int j) {
        if (j < i) std::swap(i, j);
        int l = na_npt[i];
        if (l >= cap) { err = "neighbour list capacity exceeded"; return; }
        nb[(size_t)(i - 1) * cap + l] = j; na_npt[i] = l + 1;
        l = nnabdn[j];
        if (l >= cap) { err = "neighbour list capacity exceeded"; return; }
        dnnab[(size_t)(j - 1) * cap + l] = i; nnabdn[j] = l + 1;
    }
    void nbor() {  /* code/nbor.f:3-141 */
        int nc = num_cell;
        nb.assign((size_t)N * cap, 0); dnnab.assign((size_t)N * cap, 0);
        na_npt.assign(N + 4, 0); nnabdn.assign(N + 4, 0);
        cell_add();
        std::vector<int> ncell;
        ncell.reserve(1024);
        for (int c = n_wrap * nc * nc; c <= nc * nc * (nc - n_wrap); ++c) {
            int bead = cell[c];
            if (bead == 0) continue;
            ncell.clear();
            while (bead != 0) { ncell.push_back(bead); bead = clinks[bead]; }
            int f_bead = (int)ncell.size();
            for (int d : map) {
                int nc2 = wrap_map[c + d];
                bead = cell[nc2];
                while (bead != 0) { ncell.push_back(bead); bead = clinks[bead]; }
            }
            for (int in = 0; in < f_bead; ++in) {
                int i = ncell[in];
                for (size_t jn = in + 1; jn < ncell.size(); ++jn) {
                    int j = ncell[jn];
                    int e = code(j, i);
                    if ((e >= 4 && e <= 12) || (e >= 17 && e < 27)) {
                        add_pair(i, j);
                    } else {
                        double rx = sx[i] - sx[j], ry = sy[i] - sy[j], rz = sz[i] - sz[j];
                        rx = rx - dnint(rx); ry = ry - dnint(ry); rz = rz - dnint(rz);
                        double r2 = rx * rx + ry * ry + rz * rz;
                        if (r2 <= rlsq[e]) add_pair(i, j);
                    }
                }
            }
        }
    }

    /* ------------------------------------------------------------------ */
    /* pair event-time predictors                                          */
    /* ------------------------------------------------------------------ */
    struct Rel { double rx, ry, rz, vx, vy, vz, bij, rijsq, vijsq; };
    Rel rel(int i, int j) const {
        Rel r;
        r.vx = vx[i] - vx[j]; r.vy = vy[i] - vy[j]; r.vz = vz[i] - vz[j];
        r.rx = sx[i] - sx[j] + r.vx * tfalse;
        r.ry = sy[i] - sy[j] + r.vy * tfalse;
        r.rz = sz[i] - sz[j] + r.vz * tfalse;
        r.rx = r.rx - dnint(r.rx); r.ry = r.ry - dnint(r.ry); r.rz = r.rz - dnint(r.rz);
        r.bij = r.rx * r.vx + r.ry * r.vy + r.rz * r.vz;
        r.rijsq = r.rx * r.rx + r.ry * r.ry + r.rz * r.rz;
        r.vijsq = r.vx * r.vx + r.vy * r.vy + r.vz * r.vz;
        return r;
    }
    void core(int i, int j, int evcode, double &tij, int &type) const {  /* code/core.f:3-44 */
        Rel r = rel(i, j);
        if (r.bij < 0.0) {
            double p = ev_param[1][evcode];
            double sigsq = sigma_sq[identity[i]][identity[j]] * (p * p);
            if (evcode >= 22 && evcode <= 26) {
                int k = std::max(identity[i], identity[j]);
                double s = sqz610[evcode - 21][k];
                sigsq = sigsq * (s * s);
            }
            double discr = r.bij * r.bij - r.vijsq * (r.rijsq - sigsq);
            if (discr > 0.0) { tij = (-r.bij - std::sqrt(discr)) / r.vijsq; type = 1; }
        }
    }
    void bond_limits(int i, int evcode, double &blmin, double &blmax) const {  /* code/bond.f:19-33 */
        int c = chain_of[i], ii = local_of[i], L = chain_L[c];
        blmin = ev_param[2][evcode];
        blmax = ev_param[3][evcode];
        if (evcode == 10) {
            blmin = (1.0 - del_bdln[c][ii]) * bdln[c][ii];
            blmax = (1.0 + del_bdln[c][ii]) * bdln[c][ii];
        } else if (evcode == 11) {
            blmin = (1.0 - del_blrn[c][ii - L]) * bl_rn[c][ii - L];
            blmax = (1.0 + del_blrn[c][ii - L]) * bl_rn[c][ii - L];
        } else if (evcode == 12) {
            blmin = (1.0 - del_blrc[c][ii - 2 * L]) * bl_rc[c][ii - 2 * L];
            blmax = (1.0 + del_blrc[c][ii - 2 * L]) * bl_rc[c][ii - 2 * L];
        }
    }
    void bond(int i, int j, int evcode, double &tij, int &type) const {  /* code/bond.f:4-121 */
        double blmin, blmax;
        bond_limits(i, evcode, blmin, blmax);
        Rel r = rel(i, j);
        if (r.bij < 0.0) {
            double discr1 = r.bij * r.bij - r.vijsq * (r.rijsq - blmin * blmin);
            if (discr1 > 0.0) {
                tij = (-r.bij - std::sqrt(discr1)) / r.vijsq; type = 2;
            } else {
                double discr2 = r.bij * r.bij - r.vijsq * (r.rijsq - blmax * blmax);
                if (discr2 > 0.0) { tij = (-r.bij + std::sqrt(discr2)) / r.vijsq; type = 3; }
            }
        } else {
            double discr2 = r.bij * r.bij - r.vijsq * (r.rijsq - blmax * blmax);
            if (discr2 > 0.0) { tij = -(r.rijsq - blmax * blmax) / (std::sqrt(discr2) + r.bij); type = 3; }
        }
    }
    void sqwel(int i, int j, double &tij, int &type) const {  /* code/sqwel.f:5-67 */
        Rel r = rel(i, j);
        int a = identity[i], b = identity[j];
        if (r.bij < 0.0) {
            double diff = r.rijsq - welldia_sq[a][b];
            if (diff < 0.0) {
                double corediscr = r.bij * r.bij - r.vijsq * (r.rijsq - sigma_sq[a][b]);
                if (corediscr > 0.0) {
                    tij = (-r.bij - std::sqrt(corediscr)) / r.vijsq; type = 1;
                } else {
                    double welldiscr = r.bij * r.bij - r.vijsq * diff;
                    tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 8;
                }
            } else {
                double welldiscr = r.bij * r.bij - r.vijsq * diff;
                if (welldiscr > 0.0) { tij = (-r.bij - std::sqrt(welldiscr)) / r.vijsq; type = 4; }
            }
        } else {
            double diff = r.rijsq - welldia_sq[a][b];
            if (diff < 0.0) {
                double welldiscr = r.bij * r.bij - r.vijsq * diff;
                tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 8;
            }
        }
    }
    void nc_sqwel(int i, int j, double &tij, int &type) const {  /* code/nc_sqwel.f:7-126 */
        Rel r = rel(i, j);
        int a = identity[i], b = identity[j];
        double diff = r.rijsq - welldia_sq[a][b];
        if (a + b == 5) {
            if (r.bij < 0.0) {
                if (diff < 0.0) {
                    double corediscr = r.bij * r.bij - r.vijsq * (r.rijsq - sigma_sq[a][b]);
                    if (corediscr > 0.0) {
                        tij = (-r.bij - std::sqrt(corediscr)) / r.vijsq; type = 1;
                    } else {
                        double welldiscr = r.bij * r.bij - r.vijsq * diff;
                        tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 16;
                    }
                } else {
                    double welldiscr = r.bij * r.bij - r.vijsq * diff;
                    if (welldiscr > 0.0) { tij = (-r.bij - std::sqrt(welldiscr)) / r.vijsq; type = 7; }
                }
            } else {
                if (diff < 0.0) {
                    double welldiscr = r.bij * r.bij - r.vijsq * diff;
                    tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 16;
                }
            }
        } else if (bptnr[i] == j) {
            if (r.bij < 0.0) {
                double p = ev_param[1][15];
                double fac_sigsq = sigma_sq[a][b] * p * p;
                double fac_cored = r.bij * r.bij - r.vijsq * (r.rijsq - fac_sigsq);
                if (fac_cored > 0.0) {
                    tij = (-r.bij - std::sqrt(fac_cored)) / r.vijsq; type = 1;
                } else {
                    double welldiscr = r.bij * r.bij - r.vijsq * diff;
                    tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 8;
                }
            } else {
                double welldiscr = r.bij * r.bij - r.vijsq * diff;
                tij = (-r.bij + std::sqrt(welldiscr)) / r.vijsq; type = 8;
            }
        } else {
            if (r.bij < 0.0) {
                double welldiscr = r.bij * r.bij - r.vijsq * diff;
                if (welldiscr > 0.0) { tij = (-r.bij - std::sqrt(welldiscr)) / r.vijsq; type = 9; }
            }
        }
    }
    void sqshlder(int i, int j, double &tij, int &type) const {  /* code/sqshlder.f:5-66 */
        Rel r = rel(i, j);
        int a = identity[i], b = identity[j];
        if (r.bij < 0.0) {
            double diff = r.rijsq - shlddia_sq[a][b];
            if (diff < 0.0) {
                double corediscr = r.bij * r.bij - r.vijsq * (r.rijsq - sigma_sq[a][b]);
                if (corediscr > 0.0) {
                    tij = (-r.bij - std::sqrt(corediscr)) / r.vijsq; type = 1;
                } else {
                    double shlddiscr = r.bij * r.bij - r.vijsq * diff;
                    tij = (-r.bij + std::sqrt(shlddiscr)) / r.vijsq; type = 10;
                }
            } else {
                double shlddiscr = r.bij * r.bij - r.vijsq * diff;
                if (shlddiscr > 0.0) { tij = (-r.bij - std::sqrt(shlddiscr)) / r.vijsq; type = 12; }
            }
        } else {
            double diff = r.rijsq - shlddia_sq[a][b];
            if (diff < 0.0) {
                double shlddiscr = r.bij * r.bij - r.vijsq * diff;
                tij = (-r.bij + std::sqrt(shlddiscr)) / r.vijsq; type = 10;
            }
        }
    }
    /* dispatch of code/eventredo_up.f:28-46 */
    bool predict(int i, int j, int evcode, double &tij, int &type) {
        tij = 1000000000.0; type = 0;
        if (evcode <= 3) core(i, j, evcode, tij, type);
        else if (evcode >= 4 && evcode <= 12) bond(i, j, evcode, tij, type);
        else if (evcode == 15) nc_sqwel(i, j, tij, type);
        else if (evcode == 16) sqwel(i, j, tij, type);
        else if (evcode >= 17 && evcode <= 26) core(i, j, evcode, tij, type);
        else if (evcode >= 40) sqshlder(i, j, tij, type);
        else { err = "error in ev_code matrix"; return false; }
        return true;
    }
    static bool lex_less(double ta, int pa, double tb, int pb) { return ta < tb || (ta == tb && pa < pb); }

    /* ------------------------------------------------------------------ */
    /* scheduler: calendar queue with strict (time, index) extraction      */
    /* ------------------------------------------------------------------ */
    void tree_init() {
        P = 1;
        while (P < N + 3) P <<= 1;
        tkey.assign(2 * P, HUGE_VAL);
        tidx.assign(2 * P, 1 << 30);
        for (int k = 1; k <= N + 3; ++k) tidx[P + k - 1] = k;
        for (int n = P - 1; n >= 1; --n) pull(n);
    }
    void pull(int n) {
        int a = 2 * n, b = 2 * n + 1;
        bool left = tkey[a] < tkey[b] || (tkey[a] == tkey[b] && tidx[a] < tidx[b]);
        tkey[n] = left ? tkey[a] : tkey[b];
        tidx[n] = left ? tidx[a] : tidx[b];
    }
    void tree_set(int i) {
        int n = P + i - 1;
        tkey[n] = queued[i] ? tim[i] : HUGE_VAL;
        for (n >>= 1; n >= 1; n >>= 1) pull(n);
    }
    void tree_rebuild() {
        for (int k = 1; k <= N + 3; ++k) tkey[P + k - 1] = queued[k] ? tim[k] : HUGE_VAL;
        for (int n = P - 1; n >= 1; --n) pull(n);
    }
    void add_tbin(int i) { queued[i] = 1; tree_set(i); }   /* code/add_tbin.f:2-36 */
    void del_tbin(int i) { queued[i] = 0; tree_set(i); }   /* code/del_tbin.f:1-24 */
    bool in_queue(int i) const { return queued[i] != 0; }
    int next_event() const { return tkey[1] == HUGE_VAL ? 0 : tidx[1]; }

    /* code/events.f:11-127 */
    void events() {
        for (int i = 1; i <= N; ++i) {
            for (int k = 0; k < na_npt[i]; ++k) {
                int j = nb[(size_t)(i - 1) * cap + k];
                double tij; int type;
                if (!predict(i, j, code(j, i), tij, type)) return;
                check_tij(tij);
                if (lex_less(tij, j, tim[i], nptnr[i])) { tim[i] = tij; nptnr[i] = j; coltype[i] = type; }
            }
            for (int k = 1; k <= 3; ++k) {
                int j = erv(i, k);
                if (j > i) {
                    double tij = 1000000000.0; int type = 0;
                    int e = code(j, i);
                    if (e == 1) core(i, j, e, tij, type); else sqshlder(i, j, tij, type);
                    check_tij(tij);
                    if (lex_less(tij, j, tim[i], nptnr[i])) { nptnr[i] = j; coltype[i] = type; tim[i] = tij; }
                }
            }
        }
        for (int i = 1; i <= N + 3; ++i) queued[i] = tim[i] < interval_max ? 1 : 0;
        tree_init();
        tree_rebuild();
    }

    /* eventredo_up(i,j) (code/eventredo_up.f:14-78): time relative to tfalse */
    void check_tij(double tij) {  /* code/eventredo_up.f:58-74 (debugging build) */
        if ((tij < 0.0) && (std::fabs(tij) > 1.0e-10) && err.empty()) err = "negative predicted time";
    }
    void redo_up(int i, int j) {
        double tij; int type;
        if (!predict(i, j, code(j, i), tij, type)) return;
        check_tij(tij);
        if (lex_less(tij, j, tim[i], nptnr[i])) { tim[i] = tij; nptnr[i] = j; coltype[i] = type; }
    }
    /* full re-prediction of bead l (code/partial_events.f:16-35 and its copies) */
    void redo_full(int l) {
        if (in_queue(l)) del_tbin(l);
        tim[l] = interval_max + LTSTEP - tfalse;
        coltype[l] = -1; nptnr[l] = -1;
        for (int k = 0; k < na_npt[l]; ++k) redo_up(l, nb[(size_t)(l - 1) * cap + k]);
        for (int k = 1; k <= 3; ++k) if (erv(l, k) > l) redo_up(l, erv(l, k));
        tim[l] = tim[l] + tfalse;
        if (tim[l] < interval_max) add_tbin(l);
    }
    /* eventredo_down(l,i) (code/eventredo_down.f:14-82) */
    void redo_down(int l, int i) {
        double tij; int type;
        if (!predict(l, i, code(l, i), tij, type)) return;
        check_tij(tij);
        tij = tij + tfalse;
        if (lex_less(tij, i, tim[l], nptnr[l])) {
            if (in_queue(l)) del_tbin(l);
            tim[l] = tij; nptnr[l] = i; coltype[l] = type;
            if (tim[l] < interval_max) add_tbin(l);
        }
    }
    void down_op(int l, int src) {
        if (nptnr[l] != src) redo_down(l, src); else redo_full(l);
    }
    /* code/partial_events.f:5-205 */
    void partial_events(int i, int j, bool xpulse_del) {
        redo_full(i);
        if (j != 0) redo_full(j);
        for (int kk = 0; kk < nnabdn[i]; ++kk) down_op(dnnab[(size_t)(i - 1) * cap + kk], i);
        for (int kk = 1; kk <= 3; ++kk) { int l = erv(i, kk); if (l < i && l != 0) down_op(l, i); }
        if (j != 0) {
            for (int kk = 0; kk < nnabdn[j]; ++kk) { int l = dnnab[(size_t)(j - 1) * cap + kk]; if (l != i) down_op(l, j); }
            for (int kk = 1; kk <= 3; ++kk) { int l = erv(j, kk); if (l < j && l != 0) down_op(l, j); }
        }
        if (xpulse_del) {
            if (identity[i] < identity[j]) repuls_del_b(i, j); else repuls_del_b(j, i);
        }
    }

    /* ------------------------------------------------------------------ */
    /* collision dynamics                                                  */
    /* ------------------------------------------------------------------ */
    double dist_now(int a, int b) const {  /* distance at tfalse (repuls_check.f) */
        double vxa = vx[a] - vx[b], vya = vy[a] - vy[b], vza = vz[a] - vz[b];
        double rx = sx[a] - sx[b] + vxa * tfalse, ry = sy[a] - sy[b] + vya * tfalse, rz = sz[a] - sz[b] + vza * tfalse;
        rx = rx - dnint(rx); ry = ry - dnint(ry); rz = rz - dnint(rz);
        double d = rx * rx + ry * ry + rz * rz;
        return std::sqrt(d);
    }
    void helpers(int i, int j, int &ncim1, int &ncai, int &ncaj, int &nnjp1) const {
        int Li = chain_L[chain_of[i]], Lj = chain_L[chain_of[j]];
        ncim1 = i + Li - 1; ncai = i - Li; ncaj = j - 2 * Lj; nnjp1 = j - Lj + 1;
    }
    double repuls_check(int i, int j) const {  /* code/repuls_check.f:1-85 */
        int ncim1, ncai, ncaj, nnjp1;
        helpers(i, j, ncim1, ncai, ncaj, nnjp1);
        double d1 = dist_now(i, ncaj), d2 = dist_now(i, nnjp1), d3 = dist_now(j, ncai), d4 = dist_now(j, ncim1);
        if ((d1 > shder_dist1) && (d2 > shder_dist2) && (d3 > shder_dist3) && (d4 > shder_dist4)) return 10.0;
        return 11.0;
    }
    double repuls_check_3(int i, int j, int k) const {  /* code/repuls_check_3.f:1-106 */
        int ncim1, ncai, ncaj, nnjp1;
        helpers(i, j, ncim1, ncai, ncaj, nnjp1);
        int m = 0;
        double d1 = dist_now(i, ncaj);
        if ((ncaj != k) && (d1 > shder_dist1)) m = m + 1;
        double d2 = dist_now(i, nnjp1);
        if ((nnjp1 != k) && (d2 > shder_dist2)) m = m + 1;
        double d3 = dist_now(j, ncai);
        if ((ncai != k) && (d3 > shder_dist3)) m = m + 1;
        double d4 = dist_now(j, ncim1);
        if ((ncim1 != k) && (d4 > shder_dist4)) m = m + 1;
        return m == 3 ? 10.0 : 11.0;
    }
    double check_sigma(int i, int j) const {  /* code/check_sigma.f:1-32 */
        double vxa = vx[i] - vx[j], vya = vy[i] - vy[j], vza = vz[i] - vz[j];
        double rx = sx[i] - sx[j] + vxa * tfalse, ry = sy[i] - sy[j] + vya * tfalse, rz = sz[i] - sz[j] + vza * tfalse;
        rx = rx - dnint(rx); ry = ry - dnint(ry); rz = rz - dnint(rz);
        double rijsq = rx * rx + ry * ry + rz * rz;
        double diff = rijsq - sigma_sq[identity[i]][identity[j]];
        return diff < 0.0 ? 10.0 : 11.0;
    }
    void bump(int i, int j, const Rel &r, double bumpdist, double sgn) {
        /* sgn = -1: i moves by -bumpdist*r (pair pushed together) */
        sx[i] = sx[i] + sgn * bumpdist * r.rx; sy[i] = sy[i] + sgn * bumpdist * r.ry; sz[i] = sz[i] + sgn * bumpdist * r.rz;
        sx[j] = sx[j] - sgn * bumpdist * r.rx; sy[j] = sy[j] - sgn * bumpdist * r.ry; sz[j] = sz[j] - sgn * bumpdist * r.rz;
    }
    void bump_in(int i, int j, const Rel &r, double bumpdist) {
        sx[i] = sx[i] - bumpdist * r.rx; sy[i] = sy[i] - bumpdist * r.ry; sz[i] = sz[i] - bumpdist * r.rz;
        sx[j] = sx[j] + bumpdist * r.rx; sy[j] = sy[j] + bumpdist * r.ry; sz[j] = sz[j] + bumpdist * r.rz;
    }
    void bump_out(int i, int j, const Rel &r, double bumpdist) {
        sx[i] = sx[i] + bumpdist * r.rx; sy[i] = sy[i] + bumpdist * r.ry; sz[i] = sz[i] + bumpdist * r.rz;
        sx[j] = sx[j] - bumpdist * r.rx; sy[j] = sy[j] - bumpdist * r.ry; sz[j] = sz[j] - bumpdist * r.rz;
    }
    int eventdyn(int i, int j, int evcode, int ct) {  /* code/eventdyn.f:4-385 */
        Rel r = rel(i, j);
        double bij = r.bij;
        double rmass = 2 * bm[i] * bm[j] / (bm[i] + bm[j]);
        int a = identity[i], b = identity[j];
        double ratio = 0.0;
        if (ct == 2) {
            double blmin, blmax;
            bond_limits(i, evcode, blmin, blmax);
            ratio = rmass * bij / (blmin * blmin);
        } else if (ct == 3) {
            double blmin, blmax;
            bond_limits(i, evcode, blmin, blmax);
            ratio = rmass * bij / (blmax * blmax);
        } else if (ct == 1) {
            double sigsq;
            if (evcode == 15) {
                if (bptnr[i] == j) { double p = ev_param[1][evcode]; sigsq = sigma_sq[a][b] * (p * p); }
                else sigsq = sigma_sq[a][b];
            } else {
                double p = ev_param[1][evcode];
                sigsq = sigma_sq[a][b] * (p * p);
                if (evcode >= 22 && evcode <= 26) {
                    int k = std::max(a, b);
                    double s = sqz610[evcode - 21][k];
                    sigsq = sigsq * (s * s);
                }
            }
            ratio = rmass * bij / sigsq;
        } else if (ct == 4) {
            double wellsq = welldia_sq[a][b], epsave = ep_sqrt[a][b];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            double bumpdist = SMDIST * std::sqrt(wellsq);
            if (bij * bij + del_pe > 0.0) {
                ratio = rmass * (std::sqrt((4.0 * wellsq * epsave / rmass) + bij * bij) + bij) / (2.0 * wellsq);
                ct = 20;
                bump_in(i, j, r, bumpdist);
            } else {
                ratio = rmass * bij / wellsq;
                ct = 22;
                bump_out(i, j, r, bumpdist);
            }
        } else if (ct == 8) {
            double wellsq = welldia_sq[a][b], epsave = ep_sqrt[a][b];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            double bumpdist = SMDIST * std::sqrt(wellsq);
            if (bij * bij > del_pe) {
                ratio = rmass * (-std::sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
                ct = 21;
                bump_out(i, j, r, bumpdist);
            } else {
                ratio = rmass * bij / wellsq;
                ct = 22;
                bump_in(i, j, r, bumpdist);
            }
        } else if (ct == 9) {
            double wellsq = welldia_sq[a][b];
            ratio = rmass * bij / wellsq;
            ct = 23;
            bump_out(i, j, r, SMDIST * std::sqrt(wellsq));
        } else if (ct == 5) {
            double wellsq = shlddia_sq[a][b], epsave = -epsilon_[1];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            double bumpdist = SMDIST * std::sqrt(wellsq);
            ratio = rmass * (-std::sqrt(-del_pe + bij * bij) + bij) / (2.0 * wellsq);
            ct = 24;
            bump_out(i, j, r, bumpdist);
        } else if (ct == 6) {
            double wellsq = shlddia_sq[a][b], epsave = -epsilon_[1];
            double del_pe = 4.0 * wellsq * epsave / rmass;
            double bumpdist = SMDIST * std::sqrt(wellsq);
            if (bij * bij > -del_pe) {
                ratio = rmass * (std::sqrt(del_pe + bij * bij) + bij) / (2.0 * wellsq);
                ct = 25;
                bump_in(i, j, r, bumpdist);
            } else {
                ratio = rmass * bij / wellsq;
                ct = 26;
                bump_out(i, j, r, bumpdist);
            }
        } else if (ct == 13) {
            double wellsq = shlddia_sq[a][b];
            ratio = rmass * bij / wellsq;
            ct = 27;
            bump_out(i, j, r, SMDIST * std::sqrt(wellsq));
        }
        double delvx = ratio * r.rx, delvy = ratio * r.ry, delvz = ratio * r.rz;
        vx[i] = vx[i] - delvx / bm[i]; vx[j] = vx[j] + delvx / bm[j];
        vy[i] = vy[i] - delvy / bm[i]; vy[j] = vy[j] + delvy / bm[j];
        vz[i] = vz[i] - delvz / bm[i]; vz[j] = vz[j] + delvz / bm[j];
        sx[i] = sx[i] + delvx * tfalse / bm[i];
        sy[i] = sy[i] + delvy * tfalse / bm[i];
        sz[i] = sz[i] + delvz * tfalse / bm[i];
        sx[j] = sx[j] - delvx * tfalse / bm[j];
        sy[j] = sy[j] - delvy * tfalse / bm[j];
        sz[j] = sz[j] - delvz * tfalse / bm[j];
        return ct;
    }
    void bumpoff(int i, int j, int evcode) {  /* code/bumped.f:1-47 */
        Rel r = rel(i, j);
        double bumpdist = (evcode >= 40) ? SMDIST * std::sqrt(shlddia_sq[identity[i]][identity[j]])
                                         : SMDIST * std::sqrt(welldia_sq[identity[i]][identity[j]]);
        if (r.bij < 0.0) bump_in(i, j, r, bumpdist); else bump_out(i, j, r, bumpdist);
    }

    /* one pair event: worker block (main.F90:1432-1956) then the master
     * application (main.F90:646-943) */
    int pair_event(int i, int j) {
        int ct = coltype[i];
        int evcode = code(i, j);
        bool nonend = !is_end(i) && !is_end(j);
        bool xpulse_del = false;
        int nb_ = identity[i] < identity[j] ? i : j;   /* lower identity: NH */
        int cb_ = identity[i] < identity[j] ? j : i;
        if (ct == 7) {
            if (erv(i, 4) == 0 && erv(j, 4) == 0) {
                if (nonend) {
                    double rating = repuls_check(nb_, cb_);
                    ct = rating <= 10.0 ? 4 : 14;
                } else {
                    double ran_non = dmd_uniform(seed, DMD_STREAM_CAPTURE, (uint64_t)coll, 0);
                    ct = ran_non <= 0.2 ? 4 : 9;
                }
            } else {
                ct = 9;
            }
        } else if (ct == 10) {
            double rating;
            if (evcode < 45) {
                int hb = erv(i, 4);
                rating = identity[i] < identity[hb] ? repuls_check_3(i, hb, j) : repuls_check_3(hb, i, j);
            } else {
                int hb = erv(j, 4);
                rating = identity[j] < identity[hb] ? repuls_check_3(j, hb, i) : repuls_check_3(hb, j, i);
            }
            ct = rating <= 10.0 ? 5 : 15;
        } else if (ct == 12) {
            if (evcode < 45) {
                int hb = erv(i, 4);
                if (bptnr[i] == hb) ct = check_sigma(i, hb) > 10.0 ? 6 : 13; else ct = 15;
            } else {
                int hb = erv(j, 4);
                if (bptnr[j] == hb) ct = check_sigma(j, hb) > 10.0 ? 6 : 13; else ct = 15;
            }
        }
        if (ct < 14) ct = eventdyn(i, j, evcode, ct);
        if (ct == 20) {
            if (identity[i] + identity[j] == 5) {
                bptnr[i] = j; bptnr[j] = i;
                identity[i] = identity[i] + 4; identity[j] = identity[j] + 4;
                if (nonend) { if (identity[i] < identity[j]) repuls_add(i, j); else repuls_add(j, i); }
            }
        } else if (ct == 21) {
            if (identity[i] <= 8) {
                if (nonend) {
                    xpulse_del = true;
                    if (identity[i] < identity[j]) shoulders_off(i, j); else shoulders_off(j, i);
                }
                if (bptnr[i] == j) {
                    bptnr[i] = 0; bptnr[j] = 0;
                    identity[i] = identity[i] - 4; identity[j] = identity[j] - 4;
                }
            }
        } else if (ct == 24) {
            if (evcode < 45) {
                int hb = erv(i, 4);
                if (identity[i] + identity[hb] == 5) {
                    bptnr[i] = hb; bptnr[hb] = i; identity[i] += 4; identity[hb] += 4;
                }
            } else {
                int hb = erv(j, 4);
                if (identity[j] + identity[hb] == 5) {
                    bptnr[j] = hb; bptnr[hb] = j; identity[j] += 4; identity[hb] += 4;
                }
            }
        } else if (ct == 25) {
            if (evcode < 45) {
                int hb = erv(i, 4);
                if (identity[i] >= 5) { bptnr[i] = 0; bptnr[hb] = 0; identity[i] -= 4; identity[hb] -= 4; }
            } else {
                int hb = erv(j, 4);
                if (identity[j] >= 5) { bptnr[j] = 0; bptnr[hb] = 0; identity[j] -= 4; identity[hb] -= 4; }
            }
        } else if (ct == 14) {
            bumpoff(i, j, evcode);
            if (nonend) { if (identity[i] < identity[j]) repuls_add(i, j); else repuls_add(j, i); }
        } else if (ct == 15) {
            bumpoff(i, j, evcode);
        } else if (ct == 16) {
            bumpoff(i, j, evcode);
            if (nonend) {
                xpulse_del = true;
                if (identity[i] < identity[j]) shoulders_off(i, j); else shoulders_off(j, i);
            }
        }
        coltype[i] = ct;
        if (ct >= 1 && ct < 32) nevents[ct] += 1;
        partial_events(i, j, xpulse_del);
        return ct;
    }

    void ghost_event(int64_t g) {  /* code/main.F90:997-1121 */
        uint32_t k = 0;
        auto u = [&]() { return dmd_uniform(seed, DMD_STREAM_GHOST, (uint64_t)g, k++); };
        int i;
        do { i = (int)(u() * N) + 1; } while (i == N + 1);
        numghosts += 1;
        sx[i] = sx[i] + vx[i] * tfalse; sy[i] = sy[i] + vy[i] * tfalse; sz[i] = sz[i] + vz[i] * tfalse;
        double v1, v2, r;
        do { v1 = 2.0 * u() - 1.0; v2 = 2.0 * u() - 1.0; r = v1 * v1 + v2 * v2; } while ((r == 0.0) || (r >= 1.0));
        double fact = std::sqrt(-2.0 * setemp * bm[i] * dmd_log(r) / r);
        vx[i] = v1 * fact / bm[i];
        vy[i] = v2 * fact / bm[i];
        do { v1 = 2.0 * u() - 1.0; v2 = 2.0 * u() - 1.0; r = v1 * v1 + v2 * v2; } while ((r == 0.0) || (r >= 1.0));
        fact = std::sqrt(-2.0 * setemp * bm[i] * dmd_log(r) / r);
        vz[i] = v1 * fact / bm[i];
        sx[i] = sx[i] - vx[i] * tfalse; sy[i] = sy[i] - vy[i] * tfalse; sz[i] = sz[i] - vz[i] * tfalse;
        if (in_queue(N + 1)) del_tbin(N + 1);
        double tgho = 0.0;
        while ((tgho < 1e-18) || (tgho == 1.0)) tgho = u();
        tim[N + 1] = -1.0 * dmd_log(tgho) * avegtime + tfalse;
        if (tim[N + 1] < interval_max) add_tbin(N + 1);
        if (tfalse < old_tfalse) tfalse = old_tfalse;
        last_ghost_bead = i;
        partial_events(i, 0, false);
    }
    int last_ghost_bead = 0;

    bool displ() {  /* code/displ.f:5-50 */
        double moved_far = 0.0;
        for (int i = 1; i <= N; ++i) {
            double a = old_rx[i] - sx[i], b = old_ry[i] - sy[i], c = old_rz[i] - sz[i];
            double dis = a * a + b * b + c * c;
            double moved = dis / hdelr;
            if (moved > moved_far) moved_far = moved;
        }
        if (moved_far >= 0.1) {
            if (moved_far >= 1.25 * 1.25) {
                t_fact = t_fact / 1.01;
                interval = t_fact / std::sqrt(setemp);
            }
            return true;
        }
        return false;
    }
    bool interval_event() {  /* code/main.F90:1126-1187 */
        t = t + tfalse;
        for (int k = 1; k <= N + 3; ++k) tim[k] = tim[k] - tfalse;
        interval_max = interval_max - tfalse;
        tree_rebuild();   /* every key moved */
        for (int k = 1; k <= N; ++k) {
            sx[k] = sx[k] + vx[k] * tfalse; sy[k] = sy[k] + vy[k] * tfalse; sz[k] = sz[k] + vz[k] * tfalse;
        }
        tfalse = 0.0;
        bool update = displ();
        bool rebuilt = false;
        if (update || (interval > interval_max)) {
            if (!update) { nforcedupdate += 1; n_forced = n_forced * 1.01; }
            interval_max = interval * n_forced;
            nupdates += 1;
            for (int k = 1; k <= N; ++k) {
                sx[k] = sx[k] - dnint(sx[k]); sy[k] = sy[k] - dnint(sy[k]); sz[k] = sz[k] - dnint(sz[k]);
                old_rx[k] = sx[k]; old_ry[k] = sy[k]; old_rz[k] = sz[k];
            }
            nbor();
            for (int k = 1; k <= N; ++k) { tim[k] = interval_max + LTSTEP; coltype[k] = -1; nptnr[k] = -1; }
            events();
            rebuilt = true;
        }
        int i = N + 2;
        if (in_queue(i)) del_tbin(i);
        tim[i] = interval * 0.999;
        add_tbin(i);
        return rebuilt;
    }

    void output_event() {  /* code/main.F90:1191-1246 */
        dmd_diag d;
        diagnostics(&d);
        outputs.push_back(d);
        int i = N + 3;
        if (in_queue(i)) del_tbin(i);
        tim[i] = 3.3 / (std::sqrt(setemp)) + 5 + tfalse;
        if (tim[i] < interval_max) add_tbin(i);
    }
    std::vector<dmd_diag> outputs;

    /* one step of the main loop: returns the event kind */
    int step(dmd_event *rec) {
        int i = next_event();
        if (i == 0) { err = "empty event queue"; return -1; }
        coll = coll + 1;
        tfalse = tim[i];
        int type = 0, j = 0, evc = 0;
        if (i <= N) {
            j = nptnr[i];
            evc = code(i, j);
            type = pair_event(i, j);
            n_pair += 1;
            old_tfalse = tfalse;
        } else if (i == N + 1) {
            ghost_event(ghost_index++);
            type = DMD_EV_GHOST;
            old_tfalse = tfalse;
            if (rec) { rec->coll = coll; rec->t = t; rec->tfalse = tfalse; rec->i = last_ghost_bead; rec->j = 0; rec->type = type; rec->evcode = 0; }
            return type;
        } else if (i == N + 2) {
            double tf = tfalse, t_before = t;
            bool rb = interval_event();
            type = rb ? DMD_EV_REBUILD : DMD_EV_INTERVAL;
            n_interval += 1;
            old_tfalse = tfalse;
            if (rec) { rec->coll = coll; rec->t = t_before; rec->tfalse = tf; rec->i = i; rec->j = 0; rec->type = type; rec->evcode = 0; }
            return type;
        } else {
            if (flags & DMD_FLAG_CHECK_OVERLAP) {   /* main.F90:1193-1205 (-Ddebugging) */
                int bi = 0, bj = 0;
                if (checkover(bi, bj) > 0) {
                    err = "overlap at coll " + std::to_string(coll) + ": beads " + std::to_string(bi) + " and " +
                          std::to_string(bj);
                    return -1;
                }
            }
            output_event();
            type = DMD_EV_OUTPUT;
            n_output += 1;
            old_tfalse = tfalse;
        }
        if (rec) { rec->coll = coll; rec->t = t; rec->tfalse = tfalse; rec->i = i; rec->j = j; rec->type = type; rec->evcode = evc; }
        return type;
    }

    /* ------------------------------------------------------------------ */
    /* backbone dihedral histogram: code/phipsi.f:25-290 (-Dwrite_phipsi)  */
    /* ------------------------------------------------------------------ */
    /* Adds the (phi, psi) bin of residues 2..L-1 of every chain to hist
     * (361 x 361, [phi + 180][psi + 180] in whole degrees, res(0:360,0:360)).
     * Each step in phipsi.f's order: positions advanced by tfalse
     * (:30-53), the N->Ca axis and the C-Ca perpendicular (:58-126), C(i-1)
     * in that frame and its angle from the second axis (:128-168); psi the
     * same from the C->Ca axis with N(i+1) (:170-285). */
    void phipsi_sample(int64_t *hist) const {
        const double pi = 4.0 * std::atan(1.0);   /* main.F90:125 */
        auto pos = [&](int k, double &x, double &y, double &z) {   /* k 1-based */
            x = sx[k] + vx[k] * tfalse; y = sy[k] + vy[k] * tfalse; z = sz[k] + vz[k] * tfalse;
        };
        /* the angle of (0, y, z) from the second axis, as a bin 0..360 */
        auto bin_of = [&](double ynew, double znew) {
            const double d = std::sqrt(ynew * ynew + znew * znew);
            const double yy = ynew / d, zz = znew / d;
            double c = yy;
            if (c > 1.0) c = 1.0;
            if (c < -1.0) c = -1.0;
            const double angle = std::acos(c);
            double degs = 180.0 * angle / pi;
            if (zz > 0.0) degs = degs * -1.0;
            if (degs < -180.0) degs = -180.0;
            if (degs > 180.0) degs = 180.0;
            degs = degs + 180.0;
            /* a degenerate frame (collinear beads: a NaN angle) is not counted */
            return degs >= 0.0 && degs <= 360.0 ? (int)std::trunc(degs) : -1;
        };
        /* one dihedral: axis a->b (unit x), third point c (its component
         * perpendicular to the axis gives y), fourth point e in that frame */
        auto dihedral_bin = [&](double xa, double ya, double za, double xb, double yb, double zb, double xc, double yc,
                                double zc, double xe, double ye, double ze) {
            double x1 = xb - xa, y1 = yb - ya, z1 = zb - za;
            x1 = x1 - dnint(x1); y1 = y1 - dnint(y1); z1 = z1 - dnint(z1);
            const double d1 = std::sqrt(x1 * x1 + y1 * y1 + z1 * z1);
            x1 = x1 / d1; y1 = y1 / d1; z1 = z1 / d1;
            double xu = xc - xb, yu = yc - yb, zu = zc - zb;
            xu = xu - dnint(xu); yu = yu - dnint(yu); zu = zu - dnint(zu);
            const double du = std::sqrt(xu * xu + yu * yu + zu * zu);
            xu = xu / du; yu = yu / du; zu = zu / du;
            double c = x1 * xu + y1 * yu + z1 * zu;
            if (c > 1.0) c = 1.0;
            if (c < -1.0) c = -1.0;
            const double dq = c * du;                          /* distance from b to q */
            /* phipsi.f also forms q = b + x1 dq and the unit vector q -> c,
             * of which only the length dcq is used */
            const double dcq = std::sqrt(du * du - dq * dq);
            const double xr = xc - x1 * (d1 + dq), yr = yc - y1 * (d1 + dq), zr = zc - z1 * (d1 + dq);
            double x2 = xr - xa, y2 = yr - ya, z2 = zr - za;
            x2 = x2 - dnint(x2); y2 = y2 - dnint(y2); z2 = z2 - dnint(z2);
            x2 = x2 / dcq; y2 = y2 / dcq; z2 = z2 / dcq;
            const double x3 = y1 * z2 - z1 * y2, y3 = z1 * x2 - x1 * z2, z3 = x1 * y2 - y1 * x2;
            double xd = xe - xa, yd = ye - ya, zd = ze - za;
            xd = xd - dnint(xd); yd = yd - dnint(yd); zd = zd - dnint(zd);
            const double ynew = x2 * xd + y2 * yd + z2 * zd;
            const double znew = x3 * xd + y3 * yd + z3 * zd;
            return bin_of(ynew, znew);
        };
        for (int c = 0; c < nchains; ++c) {
            const int L = chain_L[c], s = chain_start[c];
            for (int r = 2; r <= L - 1; ++r) {
                const int ca = s + r, nh = s + L + r, co = s + 2 * L + r;   /* 1-based beads */
                double xn, yn, zn, xca, yca, zca, xc, yc, zc, xn1, yn1, zn1, xcm, ycm, zcm;
                pos(nh, xn, yn, zn); pos(ca, xca, yca, zca); pos(co, xc, yc, zc);
                pos(nh + 1, xn1, yn1, zn1); pos(co - 1, xcm, ycm, zcm);
                /* phi: axis N(i) -> Ca(i), plane with C(i), point C(i-1) */
                const int bphi = dihedral_bin(xn, yn, zn, xca, yca, zca, xc, yc, zc, xcm, ycm, zcm);
                /* psi: axis C(i) -> Ca(i), plane with N(i), point N(i+1) */
                const int bpsi = dihedral_bin(xc, yc, zc, xca, yca, zca, xn, yn, zn, xn1, yn1, zn1);
                if (bphi >= 0 && bpsi >= 0) hist[(size_t)bphi * 361 + bpsi] += 1;
            }
        }
    }

    /* ------------------------------------------------------------------ */
    /* diagnostics: code/energy.f, code/radgyr.f, code/end2end.f           */
    /* ------------------------------------------------------------------ */
    void diagnostics(dmd_diag *d) {
        std::memset(d, 0, sizeof *d);
        int hb_ii = 0, hb_ij = 0, hb_alpha = 0;
        double ehh_ii = 0, ehh_ij = 0;
        for (int i = 1; i <= N - 1; ++i)
            for (int j = i + 1; j <= N; ++j) {
                if (bptnr[i] == j) {
                    if (chain_of[i] == chain_of[j]) hb_ii++; else hb_ij++;
                } else if (code(j, i) == 16) {
                    Rel r = rel(i, j);
                    double wellsq = welldia_sq[identity[i]][identity[j]];
                    double ep_depth = ep_sqrt[identity[i]][identity[j]];
                    if (r.rijsq <= wellsq) { if (chain_of[i] == chain_of[j]) ehh_ii += ep_depth; else ehh_ij += ep_depth; }
                }
            }
        for (int c = 0; c < nchains; ++c) {
            int s = chain_start[c], L = chain_L[c];
            for (int i = s + L + 5; i <= s + 2 * L; ++i) { int j = i + L - 4; if (bptnr[i] == j) hb_alpha++; }
        }
        double eps_hb = ep_sqrt[5][8];
        double sumeps = -((hb_ii + hb_ij) * eps_hb + (ehh_ii + ehh_ij));
        double sumvel = 0.0;
        for (int i = 1; i <= N; ++i) sumvel = sumvel + bm[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        d->e_total = 0.5 * sumvel + sumeps;
        d->e_kin = 0.5 * sumvel;
        d->temperature = sumvel / 3.0 / (double)N;
        d->hb_alpha = hb_alpha; d->hb_ii = hb_ii; d->hb_ij = hb_ij;
        d->ehh_ii = ehh_ii; d->ehh_ij = ehh_ij;
        /* radgyr.f:19-135 */
        double rg = 0.0; int nbb = 0;
        std::vector<double> tx, ty, tz;
        for (int c = 0; c < nchains; ++c) {
            int s = chain_start[c], L = chain_L[c];
            tx.assign(3 * L + 1, 0); ty = tx; tz = tx;
            for (int q = 1; q <= 3 * L; ++q) {
                int b = s + q;
                tx[q] = sx[b] + vx[b] * tfalse; ty[q] = sy[b] + vy[b] * tfalse; tz[q] = sz[b] + vz[b] * tfalse;
            }
            auto unwrap = [&](std::vector<double> &v, int q, int ref) {
                double d0 = v[q] - v[ref];
                if (d0 > half) v[q] = v[q] - boxl; else if (d0 < -1.0 * half) v[q] = v[q] + boxl;
            };
            for (int q = 2; q <= L; ++q) { unwrap(tx, q, q - 1); unwrap(ty, q, q - 1); unwrap(tz, q, q - 1); }
            for (int q = 1; q <= L; ++q) { unwrap(tx, L + q, q); unwrap(ty, L + q, q); unwrap(tz, L + q, q); }
            for (int q = 1; q <= L; ++q) { unwrap(tx, 2 * L + q, q); unwrap(ty, 2 * L + q, q); unwrap(tz, 2 * L + q, q); }
            double cx = 0, cy = 0, cz = 0, rgsum = 0;
            for (int q = 1; q <= 3 * L; ++q) { cx += tx[q]; cy += ty[q]; cz += tz[q]; }
            cx /= (double)(3 * L); cy /= (double)(3 * L); cz /= (double)(3 * L);
            for (int q = 1; q <= 3 * L; ++q) {
                double a = tx[q] - cx, b = ty[q] - cy, e = tz[q] - cz;
                rgsum = rgsum + a * a + b * b + e * e;
            }
            rg += rgsum; nbb += 3 * L;
        }
        d->rg = std::sqrt(rg / (double)nbb) * boxl_orig;
        double e2e = 0.0;
        for (int c = 0; c < nchains; ++c) {  /* end2end.f:12-46 */
            int s = chain_start[c], L = chain_L[c];
            int a = s + L + 1, b = s + 3 * L;
            e2e += dist_now(a, b);
        }
        d->e2e = e2e / (double)nchains * boxl_orig;
        for (int k = 0; k < 32; ++k) d->nevents[k] = nevents[k];
        d->coll = coll; d->n_pair = n_pair; d->n_ghost = numghosts; d->n_interval = n_interval;
        d->n_output = n_output; d->n_updates = nupdates; d->n_forced_updates = nforcedupdate;
        d->t = t; d->tfalse = tfalse;
        double nbr = 0.0;
        for (int i = 1; i <= N; ++i) nbr += (double)(na_npt[i] + nnabdn[i]);
        d->nbr_mean = nbr / (double)N;
        check_nc_int(d->nc_boundbad, d->nc_unboundbad);
    }
};

}  // namespace

/* ---------------------------------------------------------------------- */
/* C ABI for tests and the CPU baseline                                    */
/* ---------------------------------------------------------------------- */
struct ora_handle { Oracle o; };

extern "C" {

ora_handle *ora_create(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                       char *err, int errlen) {
    ora_handle *h = new ora_handle();
    if (!h->o.setup(cfg, tables, sys)) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", h->o.err.c_str());
        delete h;
        return nullptr;
    }
    return h;
}

int64_t ora_run(ora_handle *h, int64_t n, dmd_event *log, int64_t cap) {
    Oracle &o = h->o;
    int64_t done = 0, written = 0;
    bool phys = (o.flags & DMD_FLAG_COUNT_PHYSICAL) != 0;
    while (done < n) {
        dmd_event rec;
        int ty = o.step(log ? &rec : nullptr);
        if (ty < 0 || !o.err.empty()) return -1;
        if (log) { log[written % cap] = rec; }
        ++written;
        if (!phys || ty <= 27 || ty == DMD_EV_GHOST) ++done;
        if (ty == DMD_EV_OUTPUT && (o.flags & DMD_FLAG_STOP_AT_OUTPUT)) break;
    }
    return written;
}

int ora_predict_all(ora_handle *h, double *tim, int32_t *nptnr, int32_t *coltype) {
    Oracle &o = h->o;
    for (int i = 1; i <= o.N; ++i) { tim[i - 1] = o.tim[i]; nptnr[i - 1] = o.nptnr[i]; coltype[i - 1] = o.coltype[i]; }
    return 0;
}

int ora_get_state(ora_handle *h, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                  int32_t *bptnr, int32_t *identity, int32_t *er, double *t, double *tfalse, int64_t *coll) {
    Oracle &o = h->o;
    for (int i = 1; i <= o.N; ++i) {
        if (x) { x[i - 1] = o.sx[i]; y[i - 1] = o.sy[i]; z[i - 1] = o.sz[i]; }
        if (vx) { vx[i - 1] = o.vx[i]; vy[i - 1] = o.vy[i]; vz[i - 1] = o.vz[i]; }
        if (bptnr) bptnr[i - 1] = o.bptnr[i];
        if (identity) identity[i - 1] = o.identity[i];
        if (er) for (int m = 1; m <= 4; ++m) er[(size_t)(i - 1) * 4 + m - 1] = o.erv(i, m);
    }
    if (t) *t = o.t;
    if (tfalse) *tfalse = o.tfalse;
    if (coll) *coll = o.coll;
    return 0;
}

int ora_diagnostics(ora_handle *h, dmd_diag *d) { h->o.diagnostics(d); return 0; }
int ora_phipsi_sample(ora_handle *h, int64_t *hist) { h->o.phipsi_sample(hist); return 0; }

int ora_get_evcode(ora_handle *h, int8_t *out) {
    std::memcpy(out, h->o.ev.data(), h->o.ev.size());
    return 0;
}

int ora_get_lists(ora_handle *h, int32_t *up_count, int32_t *up, int32_t *dn_count, int32_t *dn, int32_t cap) {
    Oracle &o = h->o;
    for (int i = 1; i <= o.N; ++i) {
        up_count[i - 1] = o.na_npt[i];
        dn_count[i - 1] = o.nnabdn[i];
        for (int k = 0; k < o.na_npt[i] && k < cap; ++k) up[(size_t)(i - 1) * cap + k] = o.nb[(size_t)(i - 1) * o.cap + k];
        for (int k = 0; k < o.nnabdn[i] && k < cap; ++k) dn[(size_t)(i - 1) * cap + k] = o.dnnab[(size_t)(i - 1) * o.cap + k];
    }
    return 0;
}

int ora_get_scalars(ora_handle *h, double *out, int n) {
    Oracle &o = h->o;
    double v[] = {o.interval, o.interval_max, o.sig_max_all, o.hdelr, (double)o.num_cell, o.width,
                  o.rlsq[1], o.rlsq[15], o.rlsq[16], o.rlsq[40], o.n_forced, o.t_fact, o.ev_param[1][15],
                  o.tim[o.N + 1], o.tim[o.N + 2], o.tim[o.N + 3]};
    int m = (int)(sizeof v / sizeof v[0]);
    for (int k = 0; k < n && k < m; ++k) out[k] = v[k];
    return m;
}

int ora_n_outputs(ora_handle *h) { return (int)h->o.outputs.size(); }
int ora_get_output(ora_handle *h, int k, dmd_diag *d) {
    if (k < 0 || k >= (int)h->o.outputs.size()) return -1;
    *d = h->o.outputs[k];
    return 0;
}

void ora_destroy(ora_handle *h) { delete h; }

void ora_log_many(const double *x, double *y, int64_t n) {
    for (int64_t k = 0; k < n; ++k) y[k] = dmd_log(x[k]);
}

int ora_pair_case(ora_handle *h, int32_t i, int32_t j, int32_t ida, int32_t idb, int32_t evcode, int32_t bonded,
                  const double *st, int32_t ct_in, double *tij, int32_t *type, double *st_out, int32_t *ct_out,
                  double *mass) {
    Oracle &o = h->o;
    const int a = i + 1, b = j + 1;
    if (a < 1 || a > o.N || b < 1 || b > o.N || a == b) return -1;
    if (ida > 0) o.identity[a] = ida;
    if (idb > 0) o.identity[b] = idb;
    o.bptnr[a] = bonded ? b : 0;
    o.bptnr[b] = bonded ? a : 0;
    o.tfalse = 0.0;
    o.sx[a] = st[0]; o.sy[a] = st[1]; o.sz[a] = st[2]; o.vx[a] = st[3]; o.vy[a] = st[4]; o.vz[a] = st[5];
    o.sx[b] = st[6]; o.sy[b] = st[7]; o.sz[b] = st[8]; o.vx[b] = st[9]; o.vy[b] = st[10]; o.vz[b] = st[11];
    int ty = 0;
    if (!o.predict(a, b, evcode, *tij, ty)) return -2;
    *type = ty;
    *ct_out = ct_in > 0 ? o.eventdyn(a, b, evcode, ct_in) : 0;
    const double out[12] = {o.sx[a], o.sy[a], o.sz[a], o.vx[a], o.vy[a], o.vz[a],
                            o.sx[b], o.sy[b], o.sz[b], o.vx[b], o.vy[b], o.vz[b]};
    for (int k = 0; k < 12; ++k) st_out[k] = out[k];
    mass[0] = o.bm[a];
    mass[1] = o.bm[b];
    return 0;
}

}  // extern "C"
