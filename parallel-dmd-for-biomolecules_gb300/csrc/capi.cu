/*
 * capi.cu -- host side of the C ABI (include/dmd.h).
 *
 * Turns the reference's input surface (raw parameter tables, chains,
 * positions, velocities, H-bond partners) into the device layout of
 * engine.cuh, then drives the kernels of engine.cu.  The set-up restates
 * code/inputinfo.f:5-669, code/scale_down.f:1-87, code/make_code.f:15-60,
 * code/nbor_setup.f:1-132 and the runr restore of code/main.F90:240-321.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <atomic>
#include <chrono>
#include <cmath>
#include <deque>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <thread>
#include <vector>

#include "dmd.h"
#include "engine.cuh"
#include "engine_api.h"

#include <nvtx3/nvToolsExt.h>

/* NVTX ranges around the host side of each phase (creation: host set-up,
 * upload and the first list build; a run; the state read-back; a serving
 * step's launch, admission and retirement), for timeline tools.  The phases
 * inside the persistent event loop are not host calls; the phase-timer
 * build (-DDMD_PHASE_TIMERS) measures those. */
namespace {
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
}  // namespace

namespace {

const double DEL = 0.02375;
const double DNC = 1.46, DCC = 1.51, DCN = 1.33, DCACA = 3.8, DTIE = 2.41, DTIE2 = 2.45;
const double SQZ[6] = {0, 1.1436, 0.88, 0.87829, 0.8, 0.7713};
const double MAX_BOND_ANGSTROM = 6.5;  /* longest bonded pair (R-CO of arginine with its window) */

struct HostSys {
    dmd_run_cfg cfg;
    int N = 0, nchains = 0, cap = 128, ncell = 0, nl1 = 0, nl2 = 0;
    std::vector<int> chain_start, chain_len;
    std::vector<BeadInfo> info;
    std::vector<double> bm, blmin, blmax, blmin_sq, blmax_sq, rblmin_sq, rblmax_sq;
    std::vector<double> x, y, z, vx, vy, vz;
    std::vector<int8_t> ident;
    std::vector<int> bptnr, er, ovp;
    std::vector<int8_t> ovc;
    DTab tab;
    DScal sc;
    double sigma_raw[29] = {}, welldia_raw[29] = {};
    double sig_max[DMD_NC] = {}, sig_max_all = 0;
};

bool fail(std::string &err, const std::string &m) { err = m; return false; }

/* code/inputinfo.f + scale_down.f + make_code.f:15-60 */
void build_tables(HostSys &H, const dmd_tables *T, double boxl) {
    DTab &D = H.tab;
    std::memset(&D, 0, sizeof D);
    double sigma[29] = {}, welldia[29] = {}, eps[29] = {}, bds[29][29] = {}, wel[29][29] = {}, ep[29][29] = {};
    for (int k = 1; k <= 4; ++k) {
        sigma[k] = T->sigma[k - 1]; welldia[k] = T->welldia[k - 1]; eps[k] = T->epsilon[k - 1];
        sigma[k + 4] = sigma[k]; welldia[k + 4] = welldia[k]; eps[k + 4] = eps[k];
    }
    for (int a = 9; a <= 28; ++a)
        for (int b = 9; b <= 28; ++b) { bds[a][b] = T->bds[a - 9][b - 9]; wel[a][b] = T->wel[a - 9][b - 9]; ep[a][b] = -T->ep[a - 9][b - 9]; }
    for (int i = 9; i <= 28; ++i) { sigma[i] = 1.00 * bds[i][i]; welldia[i] = 1.5 * sigma[i]; }
    sigma[9] = 1.00 * bds[9][9] - 1.2;
    for (int i = 1; i <= 20; ++i) {
        double sz8 = T->sqz[i - 1][0], sz6 = T->sqz[i - 1][1], sz7 = T->sqz[i - 1][2], sz9 = T->sqz[i - 1][3], sz10 = T->sqz[i - 1][4];
        D.sqz610[1][i + 8] = sz6 * 2 / (sigma[i + 8] + sigma[4]);
        D.sqz610[2][i + 8] = sz7 * 2 / (sigma[i + 8] + sigma[1]);
        D.sqz610[3][i + 8] = sz8 * 2 / (sigma[i + 8] + sigma[2]);
        D.sqz610[4][i + 8] = sz9 * 2 / (sigma[i + 8] + sigma[2]);
        D.sqz610[5][i + 8] = sz10 * 2 / (sigma[i + 8] + sigma[4]);
    }
    const double B = boxl;
    for (int k = 1; k <= 28; ++k) { sigma[k] = sigma[k] / B; welldia[k] = welldia[k] / B; }
    D.shd1 = 5.00 / B; D.shd2 = 4.74 / B; D.shd3 = 4.86 / B; D.shd4 = 4.83 / B;
    for (int k = 1; k <= 28; ++k)
        for (int kk = 1; kk <= 28; ++kk) {
            double s = sigma[k] + sigma[kk];
            D.sigma_sq[k][kk] = 0.25 * (s * s);
            double w = welldia[k] + welldia[kk];
            D.welldia_sq[k][kk] = 0.25 * (w * w);
            D.ep_sqrt[k][kk] = std::sqrt(eps[k] * eps[kk]);
            D.shlddia_sq[k][kk] = D.shd4 * D.shd4;
        }
    for (int k = 9; k <= 28; ++k)
        for (int kk = 9; kk <= 28; ++kk) {
            D.ep_sqrt[k][kk] = eps[1] * ep[k][kk];
            D.sigma_sq[k][kk] = (bds[k][kk] * bds[k][kk]) / (B * B);
            D.welldia_sq[k][kk] = (wel[k][kk] * wel[k][kk]) / (B * B);
        }
    double d1 = D.shd1 * D.shd1, d2 = D.shd2 * D.shd2, d3 = D.shd3 * D.shd3;
    D.shlddia_sq[1][2] = d1; D.shlddia_sq[2][1] = d1; D.shlddia_sq[5][2] = d1; D.shlddia_sq[2][5] = d1;
    D.shlddia_sq[1][1] = d2; D.shlddia_sq[5][5] = d2; D.shlddia_sq[1][5] = d2; D.shlddia_sq[5][1] = d2;
    D.shlddia_sq[2][4] = d3; D.shlddia_sq[4][2] = d3; D.shlddia_sq[2][8] = d3; D.shlddia_sq[8][2] = d3;
    for (int l = 0; l < DMD_NC; ++l) { D.evp1[l] = 1; D.evp2[l] = 1; D.evp3[l] = 1; }
    D.evp1[15] = 1.05 * ((2.24 / B) / ((sigma[1] + sigma[4]) / 2.0));
    for (int k = 1; k <= 5; ++k) D.evp1[16 + k] = SQZ[k];
    D.evp1[27] = 1.0;
    const double bl[10] = {0, 0, 0, 0, DNC, DCC, DCN, DTIE, DTIE2, DCACA};
    for (int c = 4; c <= 6; ++c) { D.evp2[c] = bl[c] * (1.0 - DEL) / B; D.evp3[c] = bl[c] * (1.0 + DEL) / B; }
    for (int c = 7; c <= 9; ++c) { D.evp2[c] = bl[c] * (1.0 - DEL) / B; D.evp3[c] = (1.0 + DEL) * bl[c] / B; }
    for (int c = 10; c <= 12; ++c) { D.evp2[c] = (1.0 - DEL); D.evp3[c] = (1.0 + DEL); }
    D.eps1 = eps[1];
    D.eps_hb = D.ep_sqrt[5][8];
    D.boxl_orig = B;
    /* squared diameters in the operation order of code/core.f:27-33 and
     * code/nc_sqwel.f:80-84 (the device looks them up) */
    for (int code = 0; code <= 26; ++code) {
        if (code > 3 && code < 17) continue;
        for (int a = 0; a < DMD_NT; ++a)
            for (int b = 0; b < DMD_NT; ++b) {
                double p = D.evp1[code];
                double sigsq = D.sigma_sq[a][b] * (p * p);
                if (code >= 22 && code <= 26) {
                    int k = a > b ? a : b;
                    double s = D.sqz610[code - 21][k];
                    sigsq = sigsq * (s * s);
                }
                D.core_sq[core_slot(code)][a][b] = sigsq;
            }
    }
    for (int a = 0; a < DMD_NT; ++a)
        for (int b = 0; b < DMD_NT; ++b) {
            double p = D.evp1[15];
            D.ncfac_sq[a][b] = D.sigma_sq[a][b] * p * p;
            D.core15_sq[a][b] = D.sigma_sq[a][b] * (p * p);
        }
    for (int l = 0; l < DMD_NC; ++l) {
        D.evp2_sq[l] = D.evp2[l] * D.evp2[l]; D.evp3_sq[l] = D.evp3[l] * D.evp3[l];
        D.revp2_sq[l] = 1.0 / D.evp2_sq[l]; D.revp3_sq[l] = 1.0 / D.evp3_sq[l];
    }
    /* kept for nbor_setup: scaled bead diameters and the side-chain wells */
    for (int k = 1; k <= 28; ++k) { H.sigma_raw[k] = sigma[k]; H.welldia_raw[k] = welldia[k]; }
    (void)wel;
}

double sig_of(const HostSys &H, const dmd_tables *T, int code, int a, int b) {  /* code/nbor_setup.f:22-38 */
    if (code <= 3) {
        if (a >= 9 && b >= 9) return T->bds[a - 9][b - 9] / H.tab.boxl_orig;
        return 0.50 * (H.sigma_raw[a] + H.sigma_raw[b]);
    }
    if (code == 15) return 0.5 * (H.welldia_raw[a] + H.welldia_raw[b]);
    if (code == 16) return T->wel[a - 9][b - 9] / H.tab.boxl_orig;
    return 0.0;
}

/* code/nbor_setup.f:1-132: cutoffs from the maximum over every pair type
 * present in the system (intra-chain pairs of each distinct chain, and the
 * identity combinations that meet across two different chains) */
void nbor_setup(HostSys &H, const dmd_tables *T, int hbonds) {
    for (int c = 0; c < DMD_NC; ++c) H.sig_max[c] = 0.0;
    H.sig_max_all = 0.0;
    auto visit = [&](int code, int a, int b) {
        if (code > 26) return;
        double s = sig_of(H, T, code, a, b);
        if (s > H.sig_max[code]) { H.sig_max[code] = s; if (s > H.sig_max_all) H.sig_max_all = s; }
    };
    std::set<std::vector<int>> seen;
    for (int c = 0; c < H.nchains; ++c) {
        int s = H.chain_start[c], nb = (c + 1 < H.nchains ? H.chain_start[c + 1] : H.N) - s;
        std::vector<int> key;
        key.push_back(H.chain_len[c]);
        for (int q = 0; q < nb; ++q) { key.push_back(H.ident[s + q]); key.push_back(H.info[s + q].hp); }
        if (!seen.insert(key).second) continue;
        for (int a = s; a < s + nb; ++a)
            for (int b = a + 1; b < s + nb; ++b) visit(static_code(H.info[b], H.info[a], hbonds), H.ident[a], H.ident[b]);
    }
    /* inter-chain: (identity, hp, kind, pro) signatures and the chains holding them */
    std::map<std::vector<int>, std::set<int>> sig_chains;
    for (int b = 0; b < H.N; ++b) {
        const BeadInfo &I = H.info[b];
        std::vector<int> k = {H.ident[b], I.hp, I.kind, I.pro_nh, I.sp2};
        auto &st = sig_chains[k];
        if (st.size() < 2) st.insert(I.chain);
    }
    for (auto &p : sig_chains)
        for (auto &q : sig_chains) {
            bool meet = false;
            for (int c1 : p.second) for (int c2 : q.second) if (c1 != c2) meet = true;
            if (!meet) continue;
            BeadInfo A{}, Bq{};
            A.kind = (int8_t)p.first[2]; A.hp = (int8_t)p.first[1]; A.pro_nh = (int8_t)p.first[3];
            A.sp2 = (int8_t)p.first[4];
            Bq.kind = (int8_t)q.first[2]; Bq.hp = (int8_t)q.first[1]; Bq.pro_nh = (int8_t)q.first[3];
            Bq.sp2 = (int8_t)q.first[4];
            for (int order = 0; order < 2; ++order) {
                A.chain = order; Bq.chain = 1 - order;
                visit(static_code(Bq, A, hbonds), p.first[0], q.first[0]);
            }
        }
    double sigij = 0.0, sg = 0.0;
    for (int i = 1; i <= 4; ++i)
        for (int j = 1; j <= 4; ++j) {
            if ((i != 3) || (j != 3)) sg = H.sigma_raw[i] + H.sigma_raw[j];
            if (sg > sigij) sigij = sg;
        }
    for (int i = 40; i <= 50; ++i) {
        H.sig_max[i] = 0.5 * sigij * 1.0;
        if (H.sig_max[i] > H.sig_max_all) H.sig_max_all = H.sig_max[i];
    }
    const double rl_const = H.cfg.rl_const;
    for (int i = 1; i <= 50; ++i) {
        H.tab.rlsq[i] = 0.0;
        if (H.sig_max[i] != 0.0) { double r = (rl_const - 1) * H.sig_max_all + H.sig_max[i]; H.tab.rlsq[i] = r * r; }
        H.tab.rlsq_f[i] = (float)H.tab.rlsq[i];
    }
    H.tab.rlsq_max_f = 0.0f;
    for (int i = 1; i <= 50; ++i) H.tab.rlsq_max_f = std::max(H.tab.rlsq_max_f, H.tab.rlsq_f[i]);
    double rl = rl_const * H.sig_max_all;
    double h = 0.4 * (rl - H.sig_max_all);
    H.tab.hdelr = h * h;
    H.tab.rl = rl;
    double wmin = std::max(rl, MAX_BOND_ANGSTROM / H.tab.boxl_orig);
    H.ncell = (int)std::floor(1.0 / wmin);
    if (H.ncell < 3) H.ncell = 1;  /* small box: all-pairs list build */
}

void repuls_add_host(HostSys &H, int i, int j, int hbonds, std::string &err) {
    auto set = [&](int a, int b, int code) {
        int st = static_code(H.info[a], H.info[b], hbonds);
        for (int s = 0; s < 4; ++s)
            if (H.ovp[4 * a + s] == b) { if (code == st) H.ovp[4 * a + s] = -1; else H.ovc[4 * a + s] = (int8_t)code; return; }
        if (code == st) return;
        for (int s = 0; s < 4; ++s)
            if (H.ovp[4 * a + s] < 0) { H.ovp[4 * a + s] = b; H.ovc[4 * a + s] = (int8_t)code; return; }
        err = "shoulder override table full";
    };
    int Li = H.info[i].L, Lj = H.info[j].L;
    int ncim1 = i + Li - 1, ncai = i - Li, ncaj = j - 2 * Lj, nnjp1 = j - Lj + 1;
    set(ncaj, i, 50); set(i, ncaj, 40); set(i, nnjp1, 40); set(nnjp1, i, 50);
    set(ncai, j, 50); set(j, ncai, 40); set(j, ncim1, 40); set(ncim1, j, 50);
    int *er = H.er.data();
    er[4 * i + 0] = ncaj; er[4 * i + 1] = nnjp1; er[4 * ncaj + 2] = i; er[4 * nnjp1 + 2] = i;
    er[4 * j + 0] = ncai; er[4 * j + 1] = ncim1; er[4 * ncai + 2] = j; er[4 * ncim1 + 2] = j;
    er[4 * i + 3] = j; er[4 * j + 3] = i;
}

bool setup_host(HostSys &H, const dmd_run_cfg *cfg, const dmd_tables *T, const dmd_system *S, std::string &err) {
    H.cfg = *cfg;
    if (H.cfg.rl_const <= 0) H.cfg.rl_const = 1.2;
    if (H.cfg.t_fact <= 0) H.cfg.t_fact = 0.00005;
    if (H.cfg.n_forced <= 0) H.cfg.n_forced = 150.0;
    if (H.cfg.n_wrap <= 0) H.cfg.n_wrap = 2;
    if (H.cfg.numbin <= 0) H.cfg.numbin = 2000;
    H.cap = cfg->list_cap > 0 ? cfg->list_cap : 128;
    if (H.cap > 128) return fail(err, "list_cap at most 128");
    if (!(cfg->tstar > 0)) return fail(err, "tstar must be positive");
    if (!S || S->n_beads <= 0 || S->n_chains <= 0 || !S->chain_len || !S->residues) return fail(err, "empty system");
    if (!S->x || !S->y || !S->z || !S->vx || !S->vy || !S->vz) return fail(err, "positions and velocities are required");
    if (!(S->boxl > 0)) return fail(err, "boxl must be positive");
    const int hbonds = cfg->hbonds != 0;
    H.N = S->n_beads;
    H.nchains = S->n_chains;
    H.info.assign(H.N, BeadInfo{});
    H.ident.assign(H.N, 0);
    H.chain_start.assign(H.nchains, 0);
    H.chain_len.assign(H.nchains, 0);
    H.blmin.assign(H.N, 0.0);
    H.blmax.assign(H.N, 0.0);
    double bmass[29];
    for (int k = 0; k < 29; ++k) bmass[k] = T->mass[k];
    bmass[3] = bmass[20];
    for (int k = 1; k <= 4; ++k) bmass[k + 4] = bmass[k];
    int pos = 0, rpos = 0;
    for (int c = 0; c < H.nchains; ++c) {
        int L = S->chain_len[c];
        if (L < 3 || L > 30000) return fail(err, "chain length out of range");
        int nr = 0;
        for (int k = 0; k < L; ++k) {
            int r = S->residues[rpos + k];
            if (r < 9 || r > 28) return fail(err, "residue identity out of 9..28");
            nr += r != 9;
        }
        int nb = 3 * L + nr;
        if (pos + nb > H.N) return fail(err, "n_beads smaller than the chains need");
        H.chain_start[c] = pos;
        H.chain_len[c] = L;
        for (int k = 1; k <= L; ++k) {
            int idx[3] = {pos + k - 1, pos + L + k - 1, pos + 2 * L + k - 1};
            int kinds[3] = {BK_CA, BK_NH, BK_CO};
            int ids[3] = {2, 1, 4};
            for (int m = 0; m < 3; ++m) {
                BeadInfo &I = H.info[idx[m]];
                I.chain = c; I.cstart = pos; I.L = (int16_t)L; I.res = (int16_t)k; I.kind = (int8_t)kinds[m];
                I.hp = 0; I.pro_nh = 0; I.is_end = 0;
                H.ident[idx[m]] = (int8_t)ids[m];
            }
            if (k == 1) H.info[pos + L].is_end = 1;           /* NH of residue 1 (local L+1) */
            if (k == L) H.info[pos + 2 * L + L - 1].is_end = 1; /* CO of residue L (local 3L) */
        }
        int q = 0;
        for (int k = 1; k <= L; ++k) {
            int r = S->residues[rpos + k - 1];
            int iii = r != 9 ? r - 8 : 1;  /* code/inputinfo.f:300-318: glycine takes row 1 */
            double dra = std::max(T->del_rca[iii - 1], DEL), drn = std::max(T->del_rnh[iii - 1], DEL),
                   drc = std::max(T->del_rco[iii - 1], DEL);
            double lca = T->rca[iii - 1] / S->boxl, lnh = T->rnh[iii - 1] / S->boxl, lco = T->rco[iii - 1] / S->boxl;
            H.blmin[pos + k - 1] = (1.0 - dra) * lca; H.blmax[pos + k - 1] = (1.0 + dra) * lca;
            H.blmin[pos + L + k - 1] = (1.0 - drn) * lnh; H.blmax[pos + L + k - 1] = (1.0 + drn) * lnh;
            H.blmin[pos + 2 * L + k - 1] = (1.0 - drc) * lco; H.blmax[pos + 2 * L + k - 1] = (1.0 + drc) * lco;
            if (r == 9) continue;
            ++q;
            int b = pos + 3 * L + q - 1;
            BeadInfo &I = H.info[b];
            I.chain = c; I.cstart = pos; I.L = (int16_t)L; I.res = (int16_t)k; I.kind = BK_R;
            I.hp = 1; I.pro_nh = 0; I.is_end = 0;
            H.ident[b] = (int8_t)r;
            if (r == 17) H.info[pos + L + q - 1].pro_nh = 1;  /* code/make_code.f:145-169 */
        }
        if (S->hp)
            for (int m = 0; m < nb; ++m) H.info[pos + m].hp = (int8_t)(S->hp[pos + m] != 0);
        pos += nb;
        rpos += L;
    }
    if (pos != H.N) return fail(err, "n_beads larger than the chains need");
    /* -Dchaptype=2: chains from species2_chain on are species 2 */
    if (cfg->chaptype != 0 && cfg->chaptype != 1 && cfg->chaptype != 2) return fail(err, "chaptype must be 1 or 2");
    if (cfg->chaptype == 2) {
        if (cfg->species2_chain < 0 || cfg->species2_chain > H.nchains)
            return fail(err, "species2_chain outside 0..n_chains");
        for (int b = 0; b < H.N; ++b) H.info[b].sp2 = (int8_t)(H.info[b].chain >= cfg->species2_chain);
    }
    H.bm.assign(H.N, 0.0);
    for (int b = 0; b < H.N; ++b) H.bm[b] = bmass[H.ident[b]];
    H.blmin_sq.assign(H.N, 0.0);
    H.blmax_sq.assign(H.N, 0.0);
    H.rblmin_sq.assign(H.N, 0.0);
    H.rblmax_sq.assign(H.N, 0.0);
    for (int b = 0; b < H.N; ++b) {
        H.blmin_sq[b] = H.blmin[b] * H.blmin[b]; H.blmax_sq[b] = H.blmax[b] * H.blmax[b];
        if (H.blmin_sq[b] != 0.0) H.rblmin_sq[b] = 1.0 / H.blmin_sq[b];
        if (H.blmax_sq[b] != 0.0) H.rblmax_sq[b] = 1.0 / H.blmax_sq[b];
    }

    build_tables(H, T, S->boxl);
    for (int a = 0; a < DMD_NT; ++a)
        for (int b = 0; b < DMD_NT; ++b) {
            double bmi = bmass[a], bmj = bmass[b];
            H.tab.rmass[a][b] = (bmi + bmj) != 0.0 ? 2 * bmi * bmj / (bmi + bmj) : 0.0;
        }
    for (int a = 0; a < DMD_NT; ++a) H.tab.rbm[a] = bmass[a] != 0.0 ? 1.0 / bmass[a] : 0.0;
    {
        DTab &D = H.tab;
        auto rcp = [](double v) { return v != 0.0 ? 1.0 / v : 0.0; };
        for (int c = 0; c < 14; ++c)
            for (int a = 0; a < DMD_NT; ++a)
                for (int b = 0; b < DMD_NT; ++b) D.rcore_sq[c][a][b] = rcp(D.core_sq[c][a][b]);
        for (int a = 0; a < DMD_NT; ++a)
            for (int b = 0; b < DMD_NT; ++b) {
                D.rcore15_sq[a][b] = rcp(D.core15_sq[a][b]);
                D.rsigma_sq[a][b] = rcp(D.sigma_sq[a][b]);
                D.rwell_sq[a][b] = rcp(D.welldia_sq[a][b]);
                D.r2well_sq[a][b] = rcp(2.0 * D.welldia_sq[a][b]);
                D.rshld_sq[a][b] = rcp(D.shlddia_sq[a][b]);
                D.r2shld_sq[a][b] = rcp(2.0 * D.shlddia_sq[a][b]);
                D.rrmass[a][b] = rcp(D.rmass[a][b]);
            }
    }
    H.tab.setemp = cfg->tstar * 12.0;
    H.tab.avegtime = 0.00005 / std::sqrt(H.tab.setemp);

    H.x.assign(S->x, S->x + H.N); H.y.assign(S->y, S->y + H.N); H.z.assign(S->z, S->z + H.N);
    H.vx.assign(S->vx, S->vx + H.N); H.vy.assign(S->vy, S->vy + H.N); H.vz.assign(S->vz, S->vz + H.N);
    for (int k = 0; k < H.N; ++k) {
        if (!std::isfinite(H.x[k]) || !std::isfinite(H.y[k]) || !std::isfinite(H.z[k]) ||
            !std::isfinite(H.vx[k]) || !std::isfinite(H.vy[k]) || !std::isfinite(H.vz[k]))
            return fail(err, "non-finite position or velocity");
        H.x[k] = H.x[k] - std::round(H.x[k]); H.y[k] = H.y[k] - std::round(H.y[k]); H.z[k] = H.z[k] - std::round(H.z[k]);
    }
    H.bptnr.assign(H.N, -1);
    H.er.assign((size_t)4 * H.N, -1);
    H.ovp.assign((size_t)4 * H.N, -1);
    H.ovc.assign((size_t)4 * H.N, 0);
    nbor_setup(H, T, hbonds);
    if (S->bptnr) {  /* code/main.F90:240-321 */
        for (int k = 0; k < H.N; ++k) {
            int p = S->bptnr[k];
            if (p < 0 || p > H.N) return fail(err, "bptnr out of range");
            H.bptnr[k] = p - 1;
        }
        for (int k = 0; k < H.N - 1; ++k)
            for (int kj = k + 1; kj < H.N; ++kj) {
                if (H.ident[k] + H.ident[kj] == 5 && static_code(H.info[k], H.info[kj], hbonds) == 15) {
                    bool over = false;
                    for (int s = 0; s < 4; ++s) if (H.ovp[4 * k + s] == kj) over = true;
                    if (!over) {
                        double rx = H.x[k] - H.x[kj], ry = H.y[k] - H.y[kj], rz = H.z[k] - H.z[kj];
                        rx = rx - std::round(rx); ry = ry - std::round(ry); rz = rz - std::round(rz);
                        double r2 = rx * rx + ry * ry + rz * rz;
                        double diff = r2 - H.tab.welldia_sq[H.ident[k]][H.ident[kj]];
                        if (diff < 0.0 && !H.info[k].is_end && !H.info[kj].is_end) {
                            if (H.ident[k] == 1) repuls_add_host(H, k, kj, hbonds, err); else repuls_add_host(H, kj, k, hbonds, err);
                            if (!err.empty()) return false;
                        }
                    }
                }
                if (kj == H.bptnr[k]) {
                    if (H.ident[k] == 1) { H.ident[k] = 5; H.ident[kj] = 8; } else { H.ident[k] = 8; H.ident[kj] = 5; }
                }
            }
    }
    /* scalars (code/main.F90:144-156, 198-234, 408-423) */
    std::memset(&H.sc, 0, sizeof H.sc);
    H.sc.t = S->t0;
    H.sc.coll = S->coll0;
    H.sc.t_fact = H.cfg.t_fact;
    H.sc.n_forced = H.cfg.n_forced;
    H.sc.interval = H.sc.t_fact / std::sqrt(H.tab.setemp);
    H.sc.interval_max = H.sc.n_forced * H.sc.interval;
    H.nl1 = (H.N + 3 + 31) / 32;
    H.nl2 = (H.nl1 + 31) / 32;
    return true;
}

/* ------------------------------------------------------------------ */
/* device memory of a set of systems                                   */
/* ------------------------------------------------------------------ */
struct DevSys {
    DSys d;          /* device pointers */
    void *pool = nullptr;
    size_t bytes = 0;
};

struct Pool {
    char *base;
    size_t off;
    template <class T> T *take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T *p = (T *)(base + off);
        off += n * sizeof(T);
        return p;
    }
};

/* for_run: the arrays only the event loop uses (down-list codes, claim
 * tables); the allocation-free prediction pass leaves them out.  head:
 * bytes of the pool's head, the arrays filled from host data (those before
 * the neighbour lists). */
size_t layout(const HostSys &H, DSys &d, char *base, bool for_run = true, size_t *head = nullptr) {
    Pool P{base, 0};
    size_t N = H.N, NE = H.N + 3, cap = H.cap;
    size_t nc3 = (size_t)H.ncell * H.ncell * H.ncell;
    d.tab = P.take<DTab>(1);
    d.sc = P.take<DScal>(1);
    d.info = P.take<BeadInfo>(N);
    d.bm = P.take<double>(N); d.blmin = P.take<double>(N); d.blmax = P.take<double>(N);
    d.blmin_sq = P.take<double>(N); d.blmax_sq = P.take<double>(N);
    d.rblmin_sq = P.take<double>(N); d.rblmax_sq = P.take<double>(N);
    d.x = P.take<double>(N); d.y = P.take<double>(N); d.z = P.take<double>(N);
    d.vx = P.take<double>(N); d.vy = P.take<double>(N); d.vz = P.take<double>(N);
    d.ox = P.take<double>(N); d.oy = P.take<double>(N); d.oz = P.take<double>(N);
    d.xf = P.take<float>(N); d.yf = P.take<float>(N); d.zf = P.take<float>(N);
    d.ident = P.take<int8_t>(N);
    d.bptnr = P.take<int>(N);
    d.er = P.take<int>(4 * N);
    d.ovp = P.take<int>(4 * N);
    d.ovc = P.take<int8_t>(4 * N);
    d.tim = P.take<double>(NE); d.nptnr = P.take<int>(NE); d.colt = P.take<int8_t>(NE); d.queued = P.take<uint8_t>(NE);
    if (head) *head = P.off;
    d.up = P.take<int>(N * cap); d.dn = P.take<int>(N * cap); d.upc = P.take<int8_t>(N * cap);
    d.dnc = for_run ? P.take<int8_t>(N * cap) : nullptr;
    d.upn = P.take<int>(N); d.dnn = P.take<int>(N);
    d.cell_count = P.take<int>(nc3 + 1); d.cell_start = P.take<int>(nc3 + 1); d.cell_beads = P.take<int>(N);
    d.l1i = P.take<int>(H.nl1); d.l2i = P.take<int>(H.nl2);
    d.l1k = P.take<long long>(H.nl1); d.l2k = P.take<long long>(H.nl2);
    d.key = P.take<long long>(NE); d.owner = for_run ? P.take<unsigned int>(3 * N) : nullptr;
    return P.off + 256;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) { err = std::string(#call) + ": " + cudaGetErrorString(e_); return DMD_E_CUDA; } \
    } while (0)

}  // namespace

/* ---------------------------------------------------------------------- */
struct dmd_batch {
    std::vector<HostSys> hs;
    std::vector<DevSys> ds;
    DSys *d_sys = nullptr;
    int *d_cstart = nullptr, *d_clen = nullptr, *d_coff = nullptr;
    dmd_diag *d_diag = nullptr;
    dmd_event *d_log = nullptr;
    long long log_cap = 0;
    int hbonds = 1;
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    std::string err;
    int ready = 0;
    void *pool_all = nullptr;           /* the pools of all systems, one allocation */
    std::vector<dmd_diag> diag_cache;   /* diagnostics of all systems, valid until the next run */
    bool diag_valid = false;
    std::vector<char> state_cache;     /* every system's bead state, read back in one copy each */
    std::vector<size_t> state_off;
    bool state_valid = false;          /* until the next run */
    int cluster = 0;        /* CTAs per system: 1, 2, 4, 8, or 0 = chosen at run time */
    int last_cluster = 0;   /* what the last run used */
    int cell_div = 1;       /* rebuild grid: the finest grid's cells per side divided by this */
    cudaGraphExec_t graph = nullptr;   /* captured launches of dmd_batch_run_graph */
    long long graph_events = 0;
    int graph_launches = 0, graph_cluster = 0, graph_compact = -1;
    long long *d_targets = nullptr;    /* per-system event targets of a follow-up launch */
    cudaGraphExec_t cyc_graph = nullptr;   /* captured rebuild-cycle launches of dmd_batch_run_cycles */
    unsigned long long *d_phipsi = nullptr;  /* per system: 361 x 361 (phi, psi) histogram (dmd_*phipsi*) */
    std::vector<long long> phipsi_n;         /* samples in each system's histogram */
    int cyc_launches = 0, cyc_cluster = 0, cyc_compact = -1;
    long long upload_bytes = 0;        /* host-to-device bytes of the creation */
    int compact_dn = DMD_COMPACT_DN;   /* down-list limit of the compact variant, 0: never */
};
/* a single system: its batch of one, and the inputs that define the system
 * apart from its state (kept for dmd_set_state) */
struct dmd_handle {
    dmd_batch b;
    dmd_run_cfg cfg{};
    dmd_tables tables{};
    std::vector<int32_t> chain_len, residues, hp;
    int32_t n_beads = 0;
    double boxl = 0.0;
};

namespace {

/* cells per side of a coarser rebuild grid: cells stay at least as wide
 * as the finest grid's (the cutoff), so the lists are the same */
int coarse_cells(int ncell, int div) {
    if (ncell < 3 || div <= 1) return ncell;
    int c = ncell / div;
    return c >= 3 ? c : 3;
}

/* CTAs per system when the caller has not chosen: one CTA per system for
 * many systems (a system's batches rarely fill more than one CTA's warps),
 * else the largest of 4 and 2 for which every system's cluster can be
 * resident at once */
int auto_cluster(int nsys) {
    static int max_active[9] = {0};
    if (nsys >= 16) return 1;
    for (int C : {4, 2}) {
        if (max_active[C] == 0) {
            int v = 0;
            if (dmd_max_active_clusters(C, &v) != cudaSuccess) v = -1;
            cudaGetLastError();
            max_active[C] = v;
        }
        if (max_active[C] > 0 && nsys <= max_active[C]) return C;
    }
    return 1;
}

/* one system's pool: allocation (stream-ordered when a stream is given),
 * layout and the upload of the host state and the pseudo-event times */
/* The host data of one system's pool: (destination in the pool laid out at
 * d, source, bytes).  `keep` owns the temporary arrays the list points to. */
struct PoolCopy { void *dst; const void *src; size_t n; };
struct PoolTemps { std::vector<double> tim; std::vector<int> np; std::vector<int8_t> ct; std::vector<uint8_t> q; };
void pool_copies(HostSys &H, const DSys &d, PoolTemps &keep, std::vector<PoolCopy> &out) {
    size_t N = H.N;
    /* pseudo events (code/main.F90:408-423) and bead placeholders */
    keep.tim.assign(N + 3, H.sc.interval_max + DMD_LTSTEP);
    keep.np.assign(N + 3, -1);
    keep.ct.assign(N + 3, -1);
    keep.q.assign(N + 3, 0);
    if (H.cfg.canon) {
        double tgho = 0.0;
        uint32_t k = 0;
        while ((tgho < 1e-18) || (tgho == 1.0)) tgho = dmd_uniform(H.cfg.seed, DMD_STREAM_GHOST0, 0, k++);
        keep.tim[N] = -1.0 * dmd_log(tgho) * H.tab.avegtime * .0000001;
    } else {
        keep.tim[N] = 1000000000.0;
    }
    keep.tim[N + 1] = H.sc.interval;
    keep.tim[N + 2] = 3.3 / (std::sqrt(H.tab.setemp)) + 5;
    keep.np[N] = keep.np[N + 1] = keep.np[N + 2] = -2;
    keep.ct[N] = keep.ct[N + 1] = keep.ct[N + 2] = -2;
    out = {
        {(void *)d.tab, &H.tab, sizeof(DTab)}, {d.sc, &H.sc, sizeof(DScal)},
        {(void *)d.info, H.info.data(), N * sizeof(BeadInfo)}, {(void *)d.bm, H.bm.data(), N * 8},
        {(void *)d.blmin, H.blmin.data(), N * 8}, {(void *)d.blmax, H.blmax.data(), N * 8},
        {(void *)d.blmin_sq, H.blmin_sq.data(), N * 8}, {(void *)d.blmax_sq, H.blmax_sq.data(), N * 8},
        {(void *)d.rblmin_sq, H.rblmin_sq.data(), N * 8}, {(void *)d.rblmax_sq, H.rblmax_sq.data(), N * 8},
        {d.x, H.x.data(), N * 8}, {d.y, H.y.data(), N * 8}, {d.z, H.z.data(), N * 8},
        {d.vx, H.vx.data(), N * 8}, {d.vy, H.vy.data(), N * 8}, {d.vz, H.vz.data(), N * 8},
        {d.ident, H.ident.data(), N}, {d.bptnr, H.bptnr.data(), N * 4}, {d.er, H.er.data(), 4 * N * 4},
        {d.ovp, H.ovp.data(), 4 * N * 4}, {d.ovc, H.ovc.data(), 4 * N},
        {d.tim, keep.tim.data(), (N + 3) * 8}, {d.nptnr, keep.np.data(), (N + 3) * 4}, {d.colt, keep.ct.data(), N + 3},
        {d.queued, keep.q.data(), N + 3},
    };
}

void set_scalars(const HostSys &H, DSys &d) {
    d.N = H.N; d.nchains = H.nchains; d.cap = H.cap; d.ncell = H.ncell;
    d.seed = H.cfg.seed; d.canon = H.cfg.canon; d.flags = H.cfg.flags;
    d.nl1 = H.nl1; d.nl2 = H.nl2;
    d.log = nullptr; d.log_cap = 0;
}

/* one system's own pool: allocation (stream-ordered when a stream is
 * given), layout and upload */
int upload_system(HostSys &H, DevSys &D, cudaStream_t st, std::string &err) {
    DSys tmp{};
    size_t bytes = layout(H, tmp, nullptr);
    if (st) CK(cudaMallocAsync(&D.pool, bytes, st));
    else CK(cudaMalloc(&D.pool, bytes));
    D.bytes = bytes;
    DSys &d = D.d;
    layout(H, d, (char *)D.pool);
    set_scalars(H, d);
    PoolTemps keep;
    std::vector<PoolCopy> cps;
    pool_copies(H, d, keep, cps);
    for (const PoolCopy &c : cps) {
        if (st) CK(cudaMemcpyAsync(c.dst, c.src, c.n, cudaMemcpyHostToDevice, st));
        else CK(cudaMemcpy(c.dst, c.src, c.n, cudaMemcpyHostToDevice));
    }
    if (st) CK(cudaStreamSynchronize(st));   /* `keep` goes out of scope */
    return DMD_OK;
}

/* Pinned host staging for batch creation, kept between creations (grown
 * on demand; pinning host memory costs far more than copying into it). */
std::mutex g_stage_mu;
char *g_stage = nullptr;
size_t g_stage_cap = 0;

int upload(dmd_batch &B) {
    std::string &err = B.err;
    int n = (int)B.hs.size();
    B.ds.resize(n);
    CK(cudaStreamCreateWithFlags(&B.st, cudaStreamNonBlocking));
    CK(cudaEventCreate(&B.ev0));
    CK(cudaEventCreate(&B.ev1));
    /* All systems' pools in one allocation.  Each pool's head - tables,
     * scalars and bead arrays that start from host data - is filled from
     * one pinned host image, one copy per system; the neighbour lists,
     * cell grid, tournament and claim tables behind it are written on the
     * device by the list build. */
    std::vector<size_t> off(n + 1, 0), head(n, 0), soff(n + 1, 0);
    for (int r = 0; r < n; ++r) {
        DSys tmp{};
        size_t bytes = (layout(B.hs[r], tmp, nullptr, true, &head[r]) + 255) & ~(size_t)255;
        B.ds[r].bytes = bytes;
        off[r + 1] = off[r] + bytes;
        soff[r + 1] = soff[r] + ((head[r] + 255) & ~(size_t)255);
    }
    size_t total = off[n];
    CK(cudaMalloc(&B.pool_all, total));
    std::lock_guard<std::mutex> stage_lock(g_stage_mu);
    if (g_stage_cap < soff[n]) {
        if (g_stage) cudaFreeHost(g_stage);
        g_stage = nullptr;
        g_stage_cap = 0;
        CK(cudaMallocHost((void **)&g_stage, soff[n]));
        g_stage_cap = soff[n];
    }
    char *stage = g_stage;
    B.upload_bytes = 0;
    std::vector<DSys> hd(n);
    std::vector<int> cstart, clen, coff;
    for (int r = 0; r < n; ++r) {
        HostSys &H = B.hs[r];
        DevSys &D = B.ds[r];
        D.pool = nullptr;                      /* part of pool_all */
        layout(H, D.d, (char *)B.pool_all + off[r]);
        set_scalars(H, D.d);
        PoolTemps keep;
        std::vector<PoolCopy> cps;
        pool_copies(H, D.d, keep, cps);
        char *base = (char *)B.pool_all + off[r];
        for (const PoolCopy &c : cps)
            std::memcpy(stage + soff[r] + ((char *)c.dst - base), c.src, c.n);
        CK(cudaMemcpyAsync(base, stage + soff[r], head[r], cudaMemcpyHostToDevice, B.st));
        B.upload_bytes += (long long)head[r];
        hd[r] = D.d;
        coff.push_back((int)cstart.size());
        for (int c = 0; c < H.nchains; ++c) { cstart.push_back(H.chain_start[c]); clen.push_back(H.chain_len[c]); }
    }
    CK(cudaStreamSynchronize(B.st));   /* the stage is free for the next creation */
    CK(cudaMalloc(&B.d_sys, n * sizeof(DSys)));
    CK(cudaMemcpy(B.d_sys, hd.data(), n * sizeof(DSys), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&B.d_cstart, cstart.size() * 4));
    CK(cudaMalloc(&B.d_clen, clen.size() * 4));
    CK(cudaMalloc(&B.d_coff, coff.size() * 4));
    CK(cudaMemcpy(B.d_cstart, cstart.data(), cstart.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.d_clen, clen.data(), clen.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.d_coff, coff.data(), coff.size() * 4, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&B.d_diag, n * sizeof(dmd_diag)));
    CK(dmd_launch_init(B.d_sys, n, B.hbonds, B.st));
    CK(cudaStreamSynchronize(B.st));
    for (int r = 0; r < n; ++r) {
        DScal sc;
        CK(cudaMemcpy(&sc, B.ds[r].d.sc, sizeof sc, cudaMemcpyDeviceToHost));
        if (sc.err == DMD_E_OVERLAP) {
            err = "system " + std::to_string(r) + ": beads " + std::to_string(sc.err_info + 1) + " and " +
                  std::to_string(sc.err_info2 + 1) +
                  " overlap, or their bond is outside its window (code/checkover.f); DMD_FLAG_ALLOW_OVERLAP "
                  "accepts such a state";
            return sc.err;
        }
        if (sc.err) { err = "device error during list build (code " + std::to_string(sc.err) + ")"; return sc.err; }
    }
    B.ready = 1;
    return DMD_OK;
}

int batch_create(dmd_batch &B, int n, const dmd_run_cfg *cfgs, const dmd_tables *tables, const dmd_system *systems) {
    NvtxRange range("dmd create: set-up, upload, list build");
    if (n <= 0 || !cfgs || !tables || !systems) { B.err = "null or empty argument"; return DMD_E_INPUT; }
    B.hs.resize(n);
    B.hbonds = cfgs[0].hbonds != 0;
    for (int r = 0; r < n; ++r)
        if ((cfgs[r].hbonds != 0) != (B.hbonds != 0)) { B.err = "all replicas of a batch share the hbonds flag"; return DMD_E_INPUT; }
    /* the host set-up of the systems on parallel threads */
    std::vector<std::string> errs(n);
    std::vector<char> ok(n, 0);
    int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), (unsigned)n);
    std::atomic<int> next(0);
    auto work = [&]() {
        for (int r = next++; r < n; r = next++) ok[r] = setup_host(B.hs[r], &cfgs[r], tables, &systems[r], errs[r]);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    for (int r = 0; r < n; ++r)
        if (!ok[r]) { B.err = "system " + std::to_string(r) + ": " + errs[r]; return DMD_E_INPUT; }
    return upload(B);
}

int sync_check(dmd_batch &B) {
    std::string &err = B.err;
    CK(cudaStreamSynchronize(B.st));
    for (size_t r = 0; r < B.ds.size(); ++r) {
        DScal sc;
        CK(cudaMemcpy(&sc, B.ds[r].d.sc, sizeof sc, cudaMemcpyDeviceToHost));
        B.hs[r].sc = sc;
        if (sc.err == DMD_E_OVERLAP) {
            err = "system " + std::to_string(r) + ", coll " + std::to_string(sc.coll) + ": beads " +
                  std::to_string(sc.err_info + 1) + " and " + std::to_string(sc.err_info2 + 1) +
                  " overlap, or their bond is outside its window (output-event check of code/checkover.f)";
            return sc.err;
        }
        if (sc.err == DMD_E_DEVICE_TIMEOUT) {
            err = "system " + std::to_string(r) + ": the event loop reached its iteration bound at coll " +
                  std::to_string(sc.coll) + " and stopped between two batches (DMD_E_DEVICE_TIMEOUT)";
            return sc.err;
        }
        if (sc.err) {
            err = "device error " + std::to_string(sc.err) + " in system " + std::to_string(r) + " (info " + std::to_string(sc.err_info) + ")";
            return sc.err;
        }
    }
    return DMD_OK;
}

/* A follow-up launch of the full variant with per-system targets rem[] (0:
 * the system only enters and leaves). */
int run_full_remainder(dmd_batch &B, const std::vector<long long> &rem, int C, int max_beads) {
    std::string &err = B.err;
    int n = (int)B.hs.size();
    if (!B.d_targets) CK(cudaMalloc(&B.d_targets, (size_t)n * sizeof(long long)));
    CK(cudaMemcpyAsync(B.d_targets, rem.data(), (size_t)n * sizeof(long long), cudaMemcpyHostToDevice, B.st));
    CK(dmd_launch_run(B.d_sys, n, max_beads, C, 0, 0, B.d_targets, B.hbonds, B.d_cstart, B.d_clen, B.d_coff, nullptr,
                      B.st));
    return sync_check(B);
}

int batch_run(dmd_batch &B, int64_t n_events, dmd_event_log *logs) {
    NvtxRange range("dmd run: event loop");
    std::string &err = B.err;
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    B.diag_valid = false;
    B.state_valid = false;
    int n = (int)B.hs.size();
    /* event logs: one device ring per system for this call */
    std::vector<DSys> hd(n);
    long long cap = 0;
    if (logs) for (int r = 0; r < n; ++r) cap = std::max<long long>(cap, logs[r].capacity);
    if (cap > B.log_cap) {
        if (B.d_log) cudaFree(B.d_log);
        B.d_log = nullptr;
        CK(cudaMalloc(&B.d_log, (size_t)cap * n * sizeof(dmd_event)));
        B.log_cap = cap;
    }
    std::vector<long long> count0(n, 0);
    int compact = B.compact_dn;   /* the compact variant when every system's lists fit it */
    for (int r = 0; r < n; ++r) {
        hd[r] = B.ds[r].d;
        hd[r].ncell = coarse_cells(B.hs[r].ncell, B.cell_div);
        if (logs && logs[r].capacity > 0) { hd[r].log = B.d_log + (size_t)r * cap; hd[r].log_cap = logs[r].capacity; }
        else { hd[r].log = nullptr; hd[r].log_cap = 0; }
        DScal sc;
        CK(cudaMemcpy(&sc, B.ds[r].d.sc, sizeof sc, cudaMemcpyDeviceToHost));
        sc.log_count = 0;
        if (sc.max_dn > B.compact_dn) compact = 0;
        CK(cudaMemcpy(B.ds[r].d.sc, &sc, sizeof sc, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(B.d_sys, hd.data(), n * sizeof(DSys), cudaMemcpyHostToDevice));
    CK(cudaEventRecord(B.ev0, B.st));
    int max_beads = 0, min_beads = INT_MAX;
    for (const HostSys &H : B.hs) { max_beads = std::max(max_beads, H.N); min_beads = std::min(min_beads, H.N); }
    int C = B.cluster > 0 ? B.cluster : auto_cluster(n);
    B.last_cluster = C;
    CK(dmd_launch_run(B.d_sys, n, max_beads, C, compact, (long long)n_events, nullptr, B.hbonds, B.d_cstart, B.d_clen,
                      B.d_coff, nullptr, B.st, 0, min_beads));
    CK(cudaEventRecord(B.ev1, B.st));
    int rc = sync_check(B);
    if (rc == DMD_OK && compact) {
        /* systems whose lists outgrew the compact variant at a rebuild go
         * on with the full one for the rest of their events */
        std::vector<long long> rem(n, 0);
        bool any = false;
        for (int r = 0; r < n; ++r)
            if (B.hs[r].sc.need_full) { rem[r] = std::max<long long>(0, (long long)n_events - B.hs[r].sc.done); any = true; }
        if (any) {
            rc = run_full_remainder(B, rem, C, max_beads);
            CK(cudaEventRecord(B.ev1, B.st));
            CK(cudaEventSynchronize(B.ev1));
        }
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, B.ev0, B.ev1) == cudaSuccess) B.last_ms = ms;
    if (logs) {
        for (int r = 0; r < n; ++r) {
            long long cnt = B.hs[r].sc.log_count;
            logs[r].count = cnt;
            long long c = logs[r].capacity;
            if (c <= 0 || !logs[r].events) continue;
            long long m = std::min(cnt, c);
            std::vector<dmd_event> tmp((size_t)m);
            cudaError_t e = cudaMemcpy(tmp.data(), B.d_log + (size_t)r * cap, (size_t)m * sizeof(dmd_event), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { err = cudaGetErrorString(e); return DMD_E_CUDA; }
            /* ring positions are taken modulo the capacity */
            for (long long k = 0; k < m; ++k) logs[r].events[k] = tmp[(size_t)k];
        }
    }
    return rc;
}

/* the bytes of a system's bead state block in its pool: positions and
 * velocities through the extra_repuls array (one contiguous range) */
size_t state_block(const DSys &d) { return (size_t)((const char *)(d.er + 4 * (size_t)d.N) - (const char *)d.x); }

int get_state(dmd_batch &B, int r, double *x, double *y, double *z, double *vx, double *vy, double *vz,
              int32_t *bptnr, int32_t *identity, int32_t *er_out, double *t, double *tfalse, int64_t *coll) {
    NvtxRange range("dmd state read-back");
    std::string &err = B.err;
    if (r < 0 || r >= (int)B.hs.size()) { err = "replica index out of range"; return DMD_E_INPUT; }
    const int n = (int)B.hs.size();
    if (!B.state_valid) {
        /* every system's state block and scalars, one copy each */
        B.state_off.assign(n + 1, 0);
        for (int q = 0; q < n; ++q) B.state_off[q + 1] = B.state_off[q] + state_block(B.ds[q].d);
        B.state_cache.resize(B.state_off[n]);
        CK(cudaStreamSynchronize(B.st));
        for (int q = 0; q < n; ++q)
            CK(cudaMemcpyAsync(B.state_cache.data() + B.state_off[q], B.ds[q].d.x, state_block(B.ds[q].d),
                               cudaMemcpyDeviceToHost, B.st));
        for (int q = 0; q < n; ++q)
            CK(cudaMemcpyAsync(&B.hs[q].sc, B.ds[q].d.sc, sizeof(DScal), cudaMemcpyDeviceToHost, B.st));
        CK(cudaStreamSynchronize(B.st));
        B.state_valid = true;
    }
    const DSys &d = B.ds[r].d;
    const size_t N = d.N;
    const char *blk = B.state_cache.data() + B.state_off[r];
    auto at = [&](const void *p) { return blk + ((const char *)p - (const char *)d.x); };
    if (x) { std::memcpy(x, at(d.x), N * 8); std::memcpy(y, at(d.y), N * 8); std::memcpy(z, at(d.z), N * 8); }
    if (vx) { std::memcpy(vx, at(d.vx), N * 8); std::memcpy(vy, at(d.vy), N * 8); std::memcpy(vz, at(d.vz), N * 8); }
    if (bptnr) {
        const int *b = (const int *)at(d.bptnr);
        for (size_t k = 0; k < N; ++k) bptnr[k] = b[k] + 1;
    }
    if (identity) {
        const int8_t *b = (const int8_t *)at(d.ident);
        for (size_t k = 0; k < N; ++k) identity[k] = b[k];
    }
    if (er_out) {
        const int *b = (const int *)at(d.er);
        for (size_t k = 0; k < 4 * N; ++k) er_out[k] = b[k] + 1;
    }
    const DScal &sc = B.hs[r].sc;
    if (t) *t = sc.t;
    if (tfalse) *tfalse = sc.tfalse;
    if (coll) *coll = sc.coll;
    return DMD_OK;
}

/* The backbone dihedral histogram of code/phipsi.f (-Dwrite_phipsi): each
 * sample adds the current (phi, psi) bins of every residue 2..L-1 of every
 * chain of system r (r < 0: of every system) to the system's histogram on
 * the device.  The reference samples at the output events of a run's second
 * half and at its end (code/main.F90:1227-1231,1315-1317). */
constexpr size_t PHIPSI_BINS = 361 * 361;
int phipsi_sample(dmd_batch &B, int r) {
    std::string &err = B.err;
    const int n = (int)B.hs.size();
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    if (r >= n) { err = "replica index out of range"; return DMD_E_INPUT; }
    if (!B.d_phipsi) {
        CK(cudaMalloc(&B.d_phipsi, (size_t)n * PHIPSI_BINS * sizeof(unsigned long long)));
        CK(cudaMemsetAsync(B.d_phipsi, 0, (size_t)n * PHIPSI_BINS * sizeof(unsigned long long), B.st));
        B.phipsi_n.assign(n, 0);
    }
    CK(dmd_launch_phipsi(B.d_sys, n, r < 0 ? -1 : r, B.d_cstart, B.d_clen, B.d_coff, B.d_phipsi, B.st));
    for (int q = 0; q < n; ++q) if (r < 0 || q == r) B.phipsi_n[q] += 1;
    return DMD_OK;
}
/* system r's histogram ([phi + 180][psi + 180], whole degrees) and its
 * number of samples; reset != 0 then clears both */
int phipsi_histogram(dmd_batch &B, int r, int64_t *hist, int64_t *nsamples, int reset) {
    std::string &err = B.err;
    const int n = (int)B.hs.size();
    if (r < 0 || r >= n) { err = "replica index out of range"; return DMD_E_INPUT; }
    if (!B.d_phipsi) {
        if (hist) std::memset(hist, 0, PHIPSI_BINS * sizeof(int64_t));
        if (nsamples) *nsamples = 0;
        return DMD_OK;
    }
    unsigned long long *blk = B.d_phipsi + (size_t)r * PHIPSI_BINS;
    if (hist) {
        std::vector<unsigned long long> h(PHIPSI_BINS);
        CK(cudaStreamSynchronize(B.st));
        CK(cudaMemcpy(h.data(), blk, PHIPSI_BINS * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < PHIPSI_BINS; ++k) hist[k] = (int64_t)h[k];
    }
    if (nsamples) *nsamples = B.phipsi_n[r];
    if (reset) {
        CK(cudaMemsetAsync(blk, 0, PHIPSI_BINS * sizeof(unsigned long long), B.st));
        B.phipsi_n[r] = 0;
    }
    return DMD_OK;
}

/* diagnostics of every system in one launch, kept until the next run */
int diagnostics(dmd_batch &B, int r, dmd_diag *out) {
    std::string &err = B.err;
    int n = (int)B.hs.size();
    if (r < 0 || r >= n || !out) { err = "bad argument"; return DMD_E_INPUT; }
    if (!B.diag_valid) {
        CK(dmd_launch_diag(B.d_sys, n, B.d_cstart, B.d_clen, B.d_coff, B.d_diag, B.st));
        CK(cudaStreamSynchronize(B.st));
        B.diag_cache.resize(n);
        CK(cudaMemcpy(B.diag_cache.data(), B.d_diag, n * sizeof(dmd_diag), cudaMemcpyDeviceToHost));
        B.diag_valid = true;
    }
    *out = B.diag_cache[r];
    return DMD_OK;
}

/* n_launches consecutive launches of n_events each, captured once into a
 * CUDA graph (captured again when the sizes or the cluster change) and
 * replayed; the result equals one run of n_events * n_launches events */
int batch_run_graph(dmd_batch &B, int64_t n_events, int n_launches) {
    std::string &err = B.err;
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    if (n_launches <= 0 || n_events < 0) { err = "bad launch count"; return DMD_E_INPUT; }
    B.diag_valid = false;
    B.state_valid = false;
    int n = (int)B.hs.size();
    int C = B.cluster > 0 ? B.cluster : auto_cluster(n);
    int probe = 0;
    CK(dmd_max_active_clusters(C, &probe));   /* kernel attributes are set outside the capture */
    std::vector<DSys> hd(n);
    std::vector<long long> done0(n);
    int compact = B.compact_dn;   /* the compact variant when every system's lists fit it */
    for (int r = 0; r < n; ++r) {
        hd[r] = B.ds[r].d;
        hd[r].ncell = coarse_cells(B.hs[r].ncell, B.cell_div);
        hd[r].log = nullptr; hd[r].log_cap = 0;
        DScal sc;
        CK(cudaMemcpy(&sc, B.ds[r].d.sc, sizeof sc, cudaMemcpyDeviceToHost));
        done0[r] = sc.done_all;
        if (sc.max_dn > B.compact_dn) compact = 0;
    }
    int max_beads = 0, min_beads = INT_MAX;
    for (const HostSys &H : B.hs) { max_beads = std::max(max_beads, H.N); min_beads = std::min(min_beads, H.N); }
    CK(cudaMemcpy(B.d_sys, hd.data(), n * sizeof(DSys), cudaMemcpyHostToDevice));
    if (!B.graph || B.graph_events != n_events || B.graph_launches != n_launches || B.graph_cluster != C ||
        B.graph_compact != compact) {
        if (B.graph) cudaGraphExecDestroy(B.graph);
        B.graph = nullptr;
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(B.st, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaSuccess;
        for (int k = 0; k < n_launches && ce == cudaSuccess; ++k)
            ce = dmd_launch_run(B.d_sys, n, max_beads, C, compact, (long long)n_events, nullptr, B.hbonds, B.d_cstart,
                                B.d_clen, B.d_coff, nullptr, B.st, 0, min_beads);
        cudaError_t ce2 = cudaStreamEndCapture(B.st, &g);
        if (ce != cudaSuccess) { err = cudaGetErrorString(ce); if (ce2 == cudaSuccess) cudaGraphDestroy(g); return DMD_E_CUDA; }
        CK(ce2);
        cudaError_t ce3 = cudaGraphInstantiate(&B.graph, g, 0);
        cudaGraphDestroy(g);
        CK(ce3);
        B.graph_events = n_events; B.graph_launches = n_launches; B.graph_cluster = C; B.graph_compact = compact;
    }
    B.last_cluster = C;
    CK(cudaEventRecord(B.ev0, B.st));
    CK(cudaGraphLaunch(B.graph, B.st));
    CK(cudaEventRecord(B.ev1, B.st));
    int rc = sync_check(B);
    if (rc == DMD_OK && compact) {
        /* a system whose lists outgrew the compact variant left its later
         * launches at once: its remaining events run on the full one */
        std::vector<long long> rem(n, 0);
        bool any = false;
        for (int r = 0; r < n; ++r)
            if (B.hs[r].sc.need_full) {
                rem[r] = std::max<long long>(0, (long long)n_events * n_launches - (B.hs[r].sc.done_all - done0[r]));
                any = true;
            }
        if (any) {
            rc = run_full_remainder(B, rem, C, max_beads);
            CK(cudaEventRecord(B.ev1, B.st));
            CK(cudaEventSynchronize(B.ev1));
        }
    }
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, B.ev0, B.ev1) == cudaSuccess) B.last_ms = ms;
    return rc;
}

/* Rebuild cycles from a CUDA graph: per_graph launches captured once, each
 * of which runs every system up to and including its next list rebuild
 * (the nbor/events block of code/main.F90:1144-1166) or to the end of its
 * events.  The events each system still has to run stay on the device
 * (d_targets): a launch reads them and writes them back, so a replay needs
 * nothing from the host.  The graph is replayed until every system has run
 * n_events; between replays the host reads the remaining counts and the
 * systems' scalars (errors, the compact variant's overflow).  The committed
 * events equal those of batch_run with n_events. */
int batch_run_cycles(dmd_batch &B, int64_t n_events, int per_graph, int64_t *launches_out) {
    NvtxRange range("dmd run: rebuild-cycle graph");
    std::string &err = B.err;
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    if (n_events < 0 || per_graph <= 0 || per_graph > 4096) { err = "bad event or launch count"; return DMD_E_INPUT; }
    B.diag_valid = false;
    B.state_valid = false;
    int n = (int)B.hs.size();
    int C = B.cluster > 0 ? B.cluster : auto_cluster(n);
    int probe = 0;
    CK(dmd_max_active_clusters(C, &probe));   /* kernel attributes are set outside the capture */
    std::vector<DSys> hd(n);
    int compact = B.compact_dn;
    for (int r = 0; r < n; ++r) {
        hd[r] = B.ds[r].d;
        hd[r].ncell = coarse_cells(B.hs[r].ncell, B.cell_div);
        hd[r].log = nullptr; hd[r].log_cap = 0;
        DScal sc;
        CK(cudaMemcpy(&sc, B.ds[r].d.sc, sizeof sc, cudaMemcpyDeviceToHost));
        if (sc.max_dn > B.compact_dn) compact = 0;
    }
    int max_beads = 0, min_beads = INT_MAX;
    for (const HostSys &H : B.hs) { max_beads = std::max(max_beads, H.N); min_beads = std::min(min_beads, H.N); }
    CK(cudaMemcpy(B.d_sys, hd.data(), n * sizeof(DSys), cudaMemcpyHostToDevice));
    if (!B.d_targets) CK(cudaMalloc(&B.d_targets, (size_t)n * sizeof(long long)));
    std::vector<long long> rem(n, (long long)n_events);
    CK(cudaMemcpyAsync(B.d_targets, rem.data(), (size_t)n * sizeof(long long), cudaMemcpyHostToDevice, B.st));
    B.last_cluster = C;
    CK(cudaEventRecord(B.ev0, B.st));
    long long launches = 0;
    int rc = DMD_OK;
    while (true) {
        if (!B.cyc_graph || B.cyc_launches != per_graph || B.cyc_cluster != C || B.cyc_compact != compact) {
            if (B.cyc_graph) cudaGraphExecDestroy(B.cyc_graph);
            B.cyc_graph = nullptr;
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(B.st, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = cudaSuccess;
            for (int k = 0; k < per_graph && ce == cudaSuccess; ++k)
                ce = dmd_launch_run(B.d_sys, n, max_beads, C, compact, 0, B.d_targets, B.hbonds, B.d_cstart, B.d_clen,
                                    B.d_coff, nullptr, B.st, 1, min_beads);
            cudaError_t ce2 = cudaStreamEndCapture(B.st, &g);
            if (ce != cudaSuccess) { err = cudaGetErrorString(ce); if (ce2 == cudaSuccess) cudaGraphDestroy(g); return DMD_E_CUDA; }
            CK(ce2);
            cudaError_t ce3 = cudaGraphInstantiate(&B.cyc_graph, g, 0);
            cudaGraphDestroy(g);
            CK(ce3);
            B.cyc_launches = per_graph; B.cyc_cluster = C; B.cyc_compact = compact;
        }
        CK(cudaGraphLaunch(B.cyc_graph, B.st));
        launches += per_graph;
        CK(cudaMemcpyAsync(rem.data(), B.d_targets, (size_t)n * sizeof(long long), cudaMemcpyDeviceToHost, B.st));
        rc = sync_check(B);
        if (rc != DMD_OK) break;
        bool left = false, full = false;
        for (int r = 0; r < n; ++r) {
            left = left || rem[r] > 0;
            full = full || B.hs[r].sc.need_full;
        }
        if (!left) break;
        /* a system whose lists outgrew the compact variant: the rest of the
         * cycles run on the full one */
        if (full) compact = 0;
    }
    CK(cudaEventRecord(B.ev1, B.st));
    CK(cudaEventSynchronize(B.ev1));
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, B.ev0, B.ev1) == cudaSuccess) B.last_ms = ms;
    if (launches_out) *launches_out = launches;
    return rc;
}

void batch_free(dmd_batch &B);

/* Autotuner: times trial runs of a copy of the batch (made from its
 * create-time inputs) for each cluster size that fits and two rebuild
 * grids, and keeps the fastest.  The committed events do not depend on
 * either choice, so only the speed is compared. */
int batch_autotune(dmd_batch &B, int64_t trial_events, int32_t *best_cluster, int32_t *best_cell_div, double *best_ms) {
    std::string &err = B.err;
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    if (trial_events <= 0) { err = "trial_events must be positive"; return DMD_E_INPUT; }
    dmd_batch T;
    T.hs = B.hs;
    T.hbonds = B.hbonds;
    T.compact_dn = B.compact_dn;
    int rc = upload(T);
    if (rc != DMD_OK) { err = T.err; batch_free(T); return rc; }
    int n = (int)B.hs.size();
    double bms = 1e300;
    int bc = 1, bd = 1;
    for (int C : {1, 2, 4}) {
        int act = 0;
        if (dmd_max_active_clusters(C, &act) != cudaSuccess) { cudaGetLastError(); continue; }
        if (C > 1 && act < n) continue;
        for (int div : {1, 2}) {
            T.cluster = C;
            T.cell_div = div;
            rc = batch_run(T, trial_events, nullptr);          /* warm-up */
            if (rc == DMD_OK) rc = batch_run(T, trial_events, nullptr);
            if (rc != DMD_OK) { err = T.err; batch_free(T); return rc; }
            if (T.last_ms < bms) { bms = T.last_ms; bc = C; bd = div; }
        }
    }
    batch_free(T);
    B.cluster = bc;
    B.cell_div = bd;
    if (best_cluster) *best_cluster = bc;
    if (best_cell_div) *best_cell_div = bd;
    if (best_ms) *best_ms = bms;
    return DMD_OK;
}

/* ---- the autotuner's results kept in a JSON file ----
 * {"format": "dmd-autotune-1", "entries": {"<key>": {"cluster": C,
 * "cell_div": D, "trial_ms": T, "trial_events": E, "systems": n,
 * "beads": b}, ...}}.  The key names the device (compute capability and SM
 * count), the library version, the event-loop variant limit, the H-bond
 * flag, the trial length and a 64-bit FNV-1a hash of every system's bead
 * count, chain count, list capacity and finest grid; a batch of the same
 * shapes on the same device takes the stored choice without trial runs. */
struct TuneEntry { int cluster = 1, cell_div = 1; double trial_ms = 0; long long trial_events = 0, systems = 0, beads = 0; };

/* a reader for the file's own subset of JSON: objects, strings without
 * escapes other than \\ and \", and numbers */
struct JsonIn {
    const std::string &s;
    size_t p = 0;
    bool ok = true;
    explicit JsonIn(const std::string &t) : s(t) {}
    void ws() { while (p < s.size() && (s[p] == ' ' || s[p] == '\n' || s[p] == '\r' || s[p] == '\t')) ++p; }
    bool eat(char c) { ws(); if (p < s.size() && s[p] == c) { ++p; return true; } return false; }
    std::string str() {
        std::string o;
        if (!eat('"')) { ok = false; return o; }
        while (p < s.size() && s[p] != '"') {
            if (s[p] == '\\' && p + 1 < s.size()) ++p;
            o += s[p++];
        }
        if (p >= s.size()) { ok = false; return o; }
        ++p;
        return o;
    }
    double num() {
        ws();
        const char *b = s.c_str() + p;
        char *e = nullptr;
        double v = std::strtod(b, &e);
        if (e == b) { ok = false; return 0; }
        p += (size_t)(e - b);
        return v;
    }
};

bool tune_read(const std::string &path, std::map<std::string, TuneEntry> &out, std::string &err) {
    out.clear();
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return true;                      /* no file yet: an empty cache */
    std::string t;
    char buf[4096];
    size_t k;
    while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) t.append(buf, k);
    std::fclose(f);
    JsonIn J(t);
    bool fmt = false;
    if (!J.eat('{')) { err = "autotune cache " + path + ": not a JSON object"; return false; }
    while (J.ok && !J.eat('}')) {
        std::string key = J.str();
        if (!J.ok || !J.eat(':')) break;
        if (key == "format") { fmt = J.str() == "dmd-autotune-1"; }
        else if (key == "entries") {
            if (!J.eat('{')) { J.ok = false; break; }
            while (J.ok && !J.eat('}')) {
                std::string ek = J.str();
                if (!J.ok || !J.eat(':') || !J.eat('{')) { J.ok = false; break; }
                TuneEntry e;
                while (J.ok && !J.eat('}')) {
                    std::string f2 = J.str();
                    if (!J.ok || !J.eat(':')) { J.ok = false; break; }
                    double v = J.num();
                    if (f2 == "cluster") e.cluster = (int)v;
                    else if (f2 == "cell_div") e.cell_div = (int)v;
                    else if (f2 == "trial_ms") e.trial_ms = v;
                    else if (f2 == "trial_events") e.trial_events = (long long)v;
                    else if (f2 == "systems") e.systems = (long long)v;
                    else if (f2 == "beads") e.beads = (long long)v;
                    J.eat(',');
                }
                if (J.ok) out[ek] = e;
                J.eat(',');
            }
        } else { J.ok = false; break; }
        J.eat(',');
    }
    if (!J.ok || !fmt) { err = "autotune cache " + path + ": not a dmd-autotune-1 file"; out.clear(); return false; }
    for (auto &kv : out)
        if ((kv.second.cluster != 1 && kv.second.cluster != 2 && kv.second.cluster != 4 && kv.second.cluster != 8) ||
            kv.second.cell_div < 1 || kv.second.cell_div > 8) {
            err = "autotune cache " + path + ": entry out of range";
            out.clear();
            return false;
        }
    return true;
}

bool tune_write(const std::string &path, const std::map<std::string, TuneEntry> &m, std::string &err) {
    std::string tmp = path + ".tmp" + std::to_string((long long)std::chrono::steady_clock::now().time_since_epoch().count());
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) { err = "autotune cache " + path + ": cannot write"; return false; }
    std::fprintf(f, "{\n  \"format\": \"dmd-autotune-1\",\n  \"entries\": {");
    bool first = true;
    for (auto &kv : m) {
        const TuneEntry &e = kv.second;
        std::fprintf(f, "%s\n    \"%s\": {\"cluster\": %d, \"cell_div\": %d, \"trial_ms\": %.6g, \"trial_events\": %lld, "
                        "\"systems\": %lld, \"beads\": %lld}",
                     first ? "" : ",", kv.first.c_str(), e.cluster, e.cell_div, e.trial_ms, e.trial_events, e.systems, e.beads);
        first = false;
    }
    std::fprintf(f, "\n  }\n}\n");
    bool ok = std::fclose(f) == 0;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
        std::remove(tmp.c_str());
        err = "autotune cache " + path + ": cannot write";
        return false;
    }
    return true;
}

std::string tune_key(const dmd_batch &B, int64_t trial_events, long long *beads) {
    int dev = 0, major = 0, minor = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t h = 1469598103934665603ULL;
    auto mix = [&](long long v) {
        for (int b = 0; b < 8; ++b) { h ^= (uint64_t)((v >> (8 * b)) & 0xff); h *= 1099511628211ULL; }
    };
    *beads = 0;
    for (const HostSys &H : B.hs) { mix(H.N); mix(H.nchains); mix(H.cap); mix(H.ncell); *beads += H.N; }
    char k[256];
    std::snprintf(k, sizeof k, "cc%d.%d/sm%d/%s/compact%d/hb%d/trial%lld/n%zu/%016llx", major, minor, sms,
                  dmd_version(), B.compact_dn, B.hbonds, (long long)trial_events, B.hs.size(), (unsigned long long)h);
    for (char *c = k; *c; ++c) if (*c == '"' || *c == '\\' || *c == ' ') *c = '_';
    return k;
}

/* the autotuner with its results kept in the file at path */
int batch_autotune_cached(dmd_batch &B, int64_t trial_events, const char *path, int32_t *cluster, int32_t *cell_div,
                          double *best_ms, int32_t *from_cache) {
    std::string &err = B.err;
    if (!B.ready) { err = "batch not ready"; return DMD_E_STATE; }
    if (!path || !*path) { err = "no autotune cache path"; return DMD_E_INPUT; }
    if (trial_events <= 0) { err = "trial_events must be positive"; return DMD_E_INPUT; }
    std::map<std::string, TuneEntry> m;
    if (!tune_read(path, m, err)) return DMD_E_INPUT;
    long long beads = 0;
    const std::string key = tune_key(B, trial_events, &beads);
    auto it = m.find(key);
    if (it != m.end()) {
        B.cluster = it->second.cluster;
        B.cell_div = it->second.cell_div;
        if (cluster) *cluster = B.cluster;
        if (cell_div) *cell_div = B.cell_div;
        if (best_ms) *best_ms = it->second.trial_ms;
        if (from_cache) *from_cache = 1;
        return DMD_OK;
    }
    int32_t c = 1, d = 1;
    double ms = 0;
    int rc = batch_autotune(B, trial_events, &c, &d, &ms);
    if (rc != DMD_OK) return rc;
    TuneEntry e;
    e.cluster = c; e.cell_div = d; e.trial_ms = ms; e.trial_events = trial_events;
    e.systems = (long long)B.hs.size(); e.beads = beads;
    m[key] = e;
    if (!tune_read(path, m, err)) return DMD_E_INPUT;   /* entries another process added meanwhile */
    m[key] = e;
    if (!tune_write(path, m, err)) return DMD_E_INPUT;
    if (cluster) *cluster = c;
    if (cell_div) *cell_div = d;
    if (best_ms) *best_ms = ms;
    if (from_cache) *from_cache = 0;
    return DMD_OK;
}

void batch_free(dmd_batch &B) {
    if (B.graph) cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
    if (B.cyc_graph) cudaGraphExecDestroy(B.cyc_graph);
    B.cyc_graph = nullptr;
    if (B.d_phipsi) cudaFree(B.d_phipsi);
    B.d_phipsi = nullptr;
    for (auto &D : B.ds) if (D.pool) cudaFree(D.pool);
    if (B.pool_all) cudaFree(B.pool_all);
    B.pool_all = nullptr;
    if (B.d_sys) cudaFree(B.d_sys);
    if (B.d_cstart) cudaFree(B.d_cstart);
    if (B.d_clen) cudaFree(B.d_clen);
    if (B.d_coff) cudaFree(B.d_coff);
    if (B.d_diag) cudaFree(B.d_diag);
    if (B.d_log) cudaFree(B.d_log);
    if (B.d_targets) cudaFree(B.d_targets);
    if (B.ev0) cudaEventDestroy(B.ev0);
    if (B.ev1) cudaEventDestroy(B.ev1);
    if (B.st) cudaStreamDestroy(B.st);
    B.ds.clear();
}


/* ---------------------------------------------------------------------- */
/* serving: continuous batching of independent requests                   */
/* ---------------------------------------------------------------------- */
struct ServerReq {
    long long id = 0;
    HostSys H;
    DevSys D;
    long long total = 0, done = 0;      /* events requested / committed */
    int state = DMD_REQ_QUEUED;
    int rc = 0;
    std::string err;
    double t_submit = 0, t_admit = 0, t_finish = 0;
    size_t need = 0;                    /* device bytes of its pool */
    double cpe = 0;                     /* measured SM cycles per event (0: not yet) */
    dmd_diag diag{};
    std::vector<double> x, y, z, vx, vy, vz;
    std::vector<int32_t> bptnr, ident;
    double t = 0, tfalse = 0;
    long long coll = 0;
};

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

struct dmd_server {
    int max_slots = 0;
    size_t budget = 0, used = 0;
    long long chunk = 0;
    int hbonds = -1;
    cudaStream_t run_st = nullptr, copy_st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::mutex mu;                              /* submit may come from another host thread */
    std::map<long long, ServerReq *> reqs;
    std::deque<ServerReq *> waiting;
    std::vector<ServerReq *> active;
    long long next_id = 1;
    /* device arrays of the active set, grown as needed */
    DSys *d_sys = nullptr;
    long long *d_targets = nullptr;
    int *d_cstart = nullptr, *d_clen = nullptr, *d_coff = nullptr;
    size_t cap_sys = 0, cap_chains = 0;
    dmd_diag *d_diag = nullptr;
    /* statistics */
    long long steps = 0, events = 0;
    double kernel_ms = 0;
    std::string err;
};

namespace {

int server_grow(dmd_server &V, size_t nsys, size_t nch) {
    std::string &err = V.err;
    if (nsys > V.cap_sys) {
        if (V.d_sys) cudaFree(V.d_sys);
        if (V.d_targets) cudaFree(V.d_targets);
        if (V.d_coff) cudaFree(V.d_coff);
        if (V.d_diag) cudaFree(V.d_diag);
        size_t c = std::max<size_t>(nsys, 2 * V.cap_sys);
        CK(cudaMalloc(&V.d_sys, c * sizeof(DSys)));
        CK(cudaMalloc(&V.d_targets, c * sizeof(long long)));
        CK(cudaMalloc(&V.d_coff, c * sizeof(int)));
        CK(cudaMalloc(&V.d_diag, c * sizeof(dmd_diag)));
        V.cap_sys = c;
    }
    if (nch > V.cap_chains) {
        if (V.d_cstart) cudaFree(V.d_cstart);
        if (V.d_clen) cudaFree(V.d_clen);
        size_t c = std::max<size_t>(nch, 2 * V.cap_chains);
        CK(cudaMalloc(&V.d_cstart, c * sizeof(int)));
        CK(cudaMalloc(&V.d_clen, c * sizeof(int)));
        V.cap_chains = c;
    }
    return DMD_OK;
}

/* Admit queued requests, first in first out, while slots and the
 * device-memory budget allow: allocate, upload and build the lists on the
 * copy stream (concurrently with the running launch). */
void server_admit(dmd_server &V, int n_running, std::vector<ServerReq *> &admitted) {
    while (true) {
        ServerReq *R;
        {
            std::lock_guard<std::mutex> lock(V.mu);
            if (V.waiting.empty()) break;
            if (n_running + (int)admitted.size() >= V.max_slots) break;
            R = V.waiting.front();
            if (V.used + R->need > V.budget) break;
            V.waiting.pop_front();
            V.used += R->need;
        }
        std::string e;
        int rc = upload_system(R->H, R->D, V.copy_st, e);
        if (rc == DMD_OK) {
            DSys *one = nullptr;
            cudaError_t ce = cudaMallocAsync((void **)&one, sizeof(DSys), V.copy_st);
            if (ce == cudaSuccess) ce = cudaMemcpyAsync(one, &R->D.d, sizeof(DSys), cudaMemcpyHostToDevice, V.copy_st);
            if (ce == cudaSuccess) ce = dmd_launch_init(one, 1, R->H.cfg.hbonds != 0, V.copy_st);
            if (ce == cudaSuccess) ce = cudaFreeAsync(one, V.copy_st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(V.copy_st);
            if (ce != cudaSuccess) { rc = DMD_E_CUDA; e = cudaGetErrorString(ce); }
        }
        if (rc == DMD_OK) {
            DScal sc;
            if (cudaMemcpy(&sc, R->D.d.sc, sizeof sc, cudaMemcpyDeviceToHost) != cudaSuccess) { rc = DMD_E_CUDA; e = "read-back"; }
            else if (sc.err == DMD_E_OVERLAP) {
                rc = sc.err;
                e = "beads " + std::to_string(sc.err_info + 1) + " and " + std::to_string(sc.err_info2 + 1) +
                    " overlap, or their bond is outside its window (code/checkover.f)";
            } else if (sc.err) { rc = sc.err; e = "device error during the list build"; }
        }
        std::lock_guard<std::mutex> lock(V.mu);
        if (rc != DMD_OK) {
            R->state = DMD_REQ_FAILED; R->rc = rc; R->err = e; R->t_finish = now_s();
            if (R->D.pool) { cudaFree(R->D.pool); R->D.pool = nullptr; }
            V.used -= R->need;
            continue;
        }
        R->state = DMD_REQ_ACTIVE;
        R->t_admit = now_s();
        admitted.push_back(R);
    }
}

/* a finished request: its state and diagnostics to host memory */
int server_retire(dmd_server &V, ServerReq &R, int slot) {
    std::string &err = V.err;
    size_t N = R.H.N;
    const DSys &d = R.D.d;
    R.x.resize(N); R.y.resize(N); R.z.resize(N); R.vx.resize(N); R.vy.resize(N); R.vz.resize(N);
    CK(cudaMemcpy(R.x.data(), d.x, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.y.data(), d.y, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.z.data(), d.z, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.vx.data(), d.vx, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.vy.data(), d.vy, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(R.vz.data(), d.vz, N * 8, cudaMemcpyDeviceToHost));
    std::vector<int> b(N);
    CK(cudaMemcpy(b.data(), d.bptnr, N * 4, cudaMemcpyDeviceToHost));
    R.bptnr.resize(N);
    for (size_t k = 0; k < N; ++k) R.bptnr[k] = b[k] + 1;
    std::vector<int8_t> id(N);
    CK(cudaMemcpy(id.data(), d.ident, N, cudaMemcpyDeviceToHost));
    R.ident.assign(id.begin(), id.end());
    CK(cudaMemcpy(&R.diag, V.d_diag + slot, sizeof(dmd_diag), cudaMemcpyDeviceToHost));
    R.t = R.H.sc.t; R.tfalse = R.H.sc.tfalse; R.coll = R.H.sc.coll;
    return DMD_OK;
}

/* One round: launch the running requests for up to chunk events each,
 * admit queued requests on the copy stream meanwhile, then retire the
 * finished ones; the admitted requests run from the next round on. */
int server_step(dmd_server &V, int32_t *n_active, int32_t *n_finished) {
    NvtxRange range("dmd server step");
    std::string &err = V.err;
    std::vector<ServerReq *> act;
    {
        std::lock_guard<std::mutex> lock(V.mu);
        act = V.active;
    }
    int n = (int)act.size();
    int finished = 0;
    std::vector<ServerReq *> keep, admitted;
    if (n > 0) {
        std::vector<DSys> hd(n);
        std::vector<long long> tg(n);
        std::vector<int> cstart, clen, coff;
        int max_beads = 0, min_beads = INT_MAX;
        /* Balance the round: every request gets about the SM time that
         * the typical one needs for chunk events (from each request's
         * measured cycles per event), so that no CTA idles while the
         * slowest finishes. */
        std::vector<double> cpes;
        for (ServerReq *R : act) if (R->cpe > 0) cpes.push_back(R->cpe);
        double budget = 0;
        if (!cpes.empty()) {
            std::nth_element(cpes.begin(), cpes.begin() + cpes.size() / 2, cpes.end());
            budget = cpes[cpes.size() / 2] * (double)V.chunk;
        }
        for (int r = 0; r < n; ++r) {
            ServerReq &R = *act[r];
            hd[r] = R.D.d;
            long long want = V.chunk;
            if (budget > 0 && R.cpe > 0)
                want = std::max<long long>(V.chunk / 8, std::min<long long>(4 * V.chunk, (long long)(budget / R.cpe)));
            tg[r] = std::min(want, R.total - R.done);
            coff.push_back((int)cstart.size());
            for (int c = 0; c < R.H.nchains; ++c) { cstart.push_back(R.H.chain_start[c]); clen.push_back(R.H.chain_len[c]); }
            max_beads = std::max(max_beads, R.H.N);
            min_beads = std::min(min_beads, R.H.N);
        }
        int rc = server_grow(V, n, cstart.size());
        if (rc != DMD_OK) return rc;
        CK(cudaMemcpyAsync(V.d_sys, hd.data(), n * sizeof(DSys), cudaMemcpyHostToDevice, V.run_st));
        CK(cudaMemcpyAsync(V.d_targets, tg.data(), n * sizeof(long long), cudaMemcpyHostToDevice, V.run_st));
        CK(cudaMemcpyAsync(V.d_cstart, cstart.data(), cstart.size() * 4, cudaMemcpyHostToDevice, V.run_st));
        CK(cudaMemcpyAsync(V.d_clen, clen.data(), clen.size() * 4, cudaMemcpyHostToDevice, V.run_st));
        CK(cudaMemcpyAsync(V.d_coff, coff.data(), coff.size() * 4, cudaMemcpyHostToDevice, V.run_st));
        CK(cudaEventRecord(V.e0, V.run_st));
        /* the compact variant unless a request's lists are known to need the
         * full one (a request that finds out at a rebuild stops there and
         * goes on in the next round) */
        int compact = DMD_COMPACT_DN;
        for (ServerReq *R : act) if (R->H.sc.max_dn > DMD_COMPACT_DN) compact = 0;
        CK(dmd_launch_run(V.d_sys, n, max_beads, 1, compact, 0, V.d_targets, V.hbonds, V.d_cstart, V.d_clen, V.d_coff,
                          nullptr, V.run_st, 0, min_beads));
        CK(cudaEventRecord(V.e1, V.run_st));
        CK(dmd_launch_diag(V.d_sys, n, V.d_cstart, V.d_clen, V.d_coff, V.d_diag, V.run_st));
        /* From here on requests change state (admitted, retired, failed):
         * every exit goes through the bookkeeping below, so that the active
         * set never names a request whose pool was freed and no admitted
         * request is dropped.  A request whose read-back fails is failed
         * alone; the step reports the first such error after the rest are
         * booked. */
        {
            NvtxRange admit_range("dmd server admit (beside the launch)");
            server_admit(V, n, admitted);      /* overlaps the launch */
        }
        int first_rc = DMD_OK;
        std::string first_err;
        const cudaError_t se = cudaStreamSynchronize(V.run_st);   /* (the host vectors above outlive the copies) */
        if (se != cudaSuccess) {
            first_rc = DMD_E_CUDA;
            first_err = std::string("cudaStreamSynchronize: ") + cudaGetErrorString(se);
        }
        float ms = 0.f;
        if (se == cudaSuccess && cudaEventElapsedTime(&ms, V.e0, V.e1) == cudaSuccess) V.kernel_ms += ms;
        for (int r = 0; r < n; ++r) {
            ServerReq &R = *act[r];
            if (se != cudaSuccess) { keep.push_back(&R); continue; }   /* nothing known about this round */
            DScal sc;
            const cudaError_t ce = cudaMemcpy(&sc, R.D.d.sc, sizeof sc, cudaMemcpyDeviceToHost);
            if (ce != cudaSuccess) {
                R.state = DMD_REQ_FAILED; R.rc = DMD_E_CUDA;
                R.err = std::string("state read-back: ") + cudaGetErrorString(ce);
            } else {
                R.H.sc = sc;
                R.done += sc.done;
                V.events += sc.done;
                if (sc.done > 0 && sc.run_cycles > 0) R.cpe = (double)sc.run_cycles / (double)sc.done;
                if (sc.err) {
                    R.state = DMD_REQ_FAILED; R.rc = sc.err;
                    R.err = "device error " + std::to_string(sc.err) + " (info " + std::to_string(sc.err_info) + ")";
                } else if (R.done >= R.total) {
                    const int rr = server_retire(V, R, r);
                    if (rr == DMD_OK) {
                        R.state = DMD_REQ_DONE;
                    } else {
                        R.state = DMD_REQ_FAILED; R.rc = rr; R.err = "result read-back: " + V.err;
                    }
                }
            }
            if (R.state == DMD_REQ_ACTIVE) { keep.push_back(&R); continue; }
            if (R.state == DMD_REQ_FAILED && first_rc == DMD_OK) {
                first_rc = R.rc;
                first_err = "request " + std::to_string(R.id) + ": " + R.err;
            }
            R.t_finish = now_s();
            cudaFreeAsync(R.D.pool, V.copy_st);   /* an error here leaves the pool to the runtime's teardown */
            R.D.pool = nullptr;
            ++finished;
            std::lock_guard<std::mutex> lock(V.mu);
            V.used -= R.need;
        }
        ++V.steps;
        {
            std::lock_guard<std::mutex> lock(V.mu);
            V.active = keep;
            for (ServerReq *R : admitted) V.active.push_back(R);
            if (n_finished) *n_finished = finished;
            if (n_active) *n_active = (int)V.active.size();
        }
        if (first_rc != DMD_OK) err = first_err;
        return first_rc;
    }
    server_admit(V, 0, admitted);
    std::lock_guard<std::mutex> lock(V.mu);
    V.active = keep;
    for (ServerReq *R : admitted) V.active.push_back(R);
    if (n_finished) *n_finished = finished;
    if (n_active) *n_active = (int)V.active.size();
    return DMD_OK;
}

}  // namespace

/* ---------------------------------------------------------------------- */
/* C ABI                                                                   */
/* ---------------------------------------------------------------------- */
extern "C" {

const char *dmd_version(void) { return "dmd-gb300 0.1 (sm_103a)"; }

int dmd_batch_create(int32_t n, const dmd_run_cfg *cfgs, const dmd_tables *tables, const dmd_system *systems,
                     dmd_batch **out) {
    if (!out) return DMD_E_INPUT;
    dmd_batch *B = new dmd_batch();
    int rc = batch_create(*B, n, cfgs, tables, systems);
    *out = B;  /* returned even on failure so that dmd_batch_last_error works; free with destroy */
    return rc;
}
int dmd_batch_run(dmd_batch *b, int64_t n_events, dmd_event_log *logs) {
    if (!b) return DMD_E_INPUT;
    if (n_events < 0) { b->err = "negative event count"; return DMD_E_INPUT; }
    return batch_run(*b, n_events, logs);
}
int dmd_batch_get_state(dmd_batch *b, int32_t r, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                        int32_t *bptnr, int32_t *identity, int32_t *er, double *t, double *tfalse, int64_t *coll) {
    if (!b) return DMD_E_INPUT;
    return get_state(*b, r, x, y, z, vx, vy, vz, bptnr, identity, er, t, tfalse, coll);
}
int dmd_batch_diagnostics(dmd_batch *b, int32_t r, dmd_diag *out) {
    if (!b) return DMD_E_INPUT;
    return diagnostics(*b, r, out);
}
int dmd_batch_phipsi_sample(dmd_batch *b, int32_t r) {
    if (!b) return DMD_E_INPUT;
    return phipsi_sample(*b, r);
}
int dmd_batch_phipsi_histogram(dmd_batch *b, int32_t r, int64_t *hist, int64_t *nsamples, int32_t reset) {
    if (!b) return DMD_E_INPUT;
    return phipsi_histogram(*b, r, hist, nsamples, reset);
}
void dmd_batch_destroy(dmd_batch *b) {
    if (!b) return;
    batch_free(*b);
    delete b;
}
const char *dmd_batch_last_error(dmd_batch *b) { return b ? b->err.c_str() : "null handle"; }
double dmd_batch_last_run_ms(dmd_batch *b) { return b ? b->last_ms : 0.0; }
int dmd_batch_set_cluster(dmd_batch *b, int32_t ctas) {
    if (!b) return DMD_E_INPUT;
    if (ctas != 0 && ctas != 1 && ctas != 2 && ctas != 4 && ctas != 8) { b->err = "cluster size must be 0, 1, 2, 4 or 8"; return DMD_E_INPUT; }
    b->cluster = ctas;
    return 0;
}
int32_t dmd_batch_cluster(dmd_batch *b) { return b ? b->last_cluster : 0; }
int64_t dmd_batch_device_bytes(dmd_batch *b) {
    if (!b) return 0;
    int64_t s = 0;
    for (const DevSys &D : b->ds) s += (int64_t)D.bytes;
    return s;
}
int64_t dmd_batch_upload_bytes(dmd_batch *b) { return b ? (int64_t)b->upload_bytes : 0; }
int64_t dmd_batch_readback_bytes(dmd_batch *b) {
    if (!b) return 0;
    int64_t s = 0;
    for (const DevSys &D : b->ds) s += (int64_t)(state_block(D.d) + sizeof(DScal));
    return s;
}
int dmd_batch_run_graph(dmd_batch *b, int64_t n_events, int32_t n_launches) {
    if (!b) return DMD_E_INPUT;
    return batch_run_graph(*b, n_events, n_launches);
}
int dmd_batch_run_cycles(dmd_batch *b, int64_t n_events, int32_t launches_per_graph, int64_t *n_launches) {
    if (!b) return DMD_E_INPUT;
    return batch_run_cycles(*b, n_events, launches_per_graph, n_launches);
}
int dmd_batch_autotune(dmd_batch *b, int64_t trial_events, int32_t *cluster, int32_t *cell_div, double *best_ms) {
    if (!b) return DMD_E_INPUT;
    return batch_autotune(*b, trial_events, cluster, cell_div, best_ms);
}
int dmd_batch_autotune_cached(dmd_batch *b, int64_t trial_events, const char *cache_path, int32_t *cluster,
                              int32_t *cell_div, double *best_ms, int32_t *from_cache) {
    if (!b) return DMD_E_INPUT;
    return batch_autotune_cached(*b, trial_events, cache_path, cluster, cell_div, best_ms, from_cache);
}
int dmd_batch_set_cell_div(dmd_batch *b, int32_t div) {
    if (!b) return DMD_E_INPUT;
    if (div < 1 || div > 8) { b->err = "cell_div must be 1..8"; return DMD_E_INPUT; }
    b->cell_div = div;
    return 0;
}
int dmd_set_cluster(dmd_handle *h, int32_t ctas) { return h ? dmd_batch_set_cluster(&h->b, ctas) : DMD_E_INPUT; }
int dmd_batch_set_compact_limit(dmd_batch *b, int32_t max_down) {
    if (!b) return DMD_E_INPUT;
    if (max_down < 0 || max_down > DMD_COMPACT_DN) { b->err = "max_down must be 0..32"; return DMD_E_INPUT; }
    b->compact_dn = max_down;
    return 0;
}
int dmd_set_compact_limit(dmd_handle *h, int32_t max_down) {
    return h ? dmd_batch_set_compact_limit(&h->b, max_down) : DMD_E_INPUT;
}
double dmd_last_run_ms(dmd_handle *h) { return h ? h->b.last_ms : 0.0; }

int dmd_create(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys, dmd_handle **out) {
    if (!out) return DMD_E_INPUT;
    dmd_handle *h = new dmd_handle();
    int rc = batch_create(h->b, 1, cfg, tables, sys);
    if (rc == DMD_OK) {
        h->cfg = *cfg;
        h->tables = *tables;
        h->n_beads = sys->n_beads;
        h->boxl = sys->boxl;
        h->chain_len.assign(sys->chain_len, sys->chain_len + sys->n_chains);
        size_t nres = 0;
        for (int c = 0; c < sys->n_chains; ++c) nres += (size_t)sys->chain_len[c];
        h->residues.assign(sys->residues, sys->residues + nres);
        if (sys->hp) h->hp.assign(sys->hp, sys->hp + sys->n_beads);
    }
    *out = h;
    return rc;
}
int dmd_set_state(dmd_handle *h, const double *x, const double *y, const double *z, const double *vx,
                  const double *vy, const double *vz, const int32_t *bptnr, double t, int64_t coll) {
    if (!h) return DMD_E_INPUT;
    if (!h->b.ready) { h->b.err = "handle not created"; return DMD_E_STATE; }
    if (!x || !y || !z || !vx || !vy || !vz) { h->b.err = "positions and velocities are required"; return DMD_E_INPUT; }
    dmd_system sys{};
    sys.n_beads = h->n_beads;
    sys.n_chains = (int32_t)h->chain_len.size();
    sys.chain_len = h->chain_len.data();
    sys.residues = h->residues.data();
    sys.hp = h->hp.empty() ? nullptr : h->hp.data();
    sys.boxl = h->boxl;
    sys.x = x; sys.y = y; sys.z = z; sys.vx = vx; sys.vy = vy; sys.vz = vz;
    sys.bptnr = bptnr;
    sys.t0 = t;
    sys.coll0 = coll;
    /* the new state is set up beside the old one, which stays in force if
     * that fails */
    dmd_batch nb;
    int rc = batch_create(nb, 1, &h->cfg, &h->tables, &sys);
    if (rc != DMD_OK) {
        h->b.err = nb.err;
        batch_free(nb);
        return rc;
    }
    nb.cluster = h->b.cluster;
    nb.cell_div = h->b.cell_div;
    nb.compact_dn = h->b.compact_dn;
    std::swap(h->b, nb);
    batch_free(nb);
    return DMD_OK;
}
int dmd_run(dmd_handle *h, int64_t n_events, dmd_event_log *log) {
    if (!h) return DMD_E_INPUT;
    if (n_events < 0) { h->b.err = "negative event count"; return DMD_E_INPUT; }
    return batch_run(h->b, n_events, log);
}
int dmd_predict_all(dmd_handle *h, double *tim, int32_t *nptnr, int32_t *coltype) {
    if (!h || !h->b.ready) return DMD_E_STATE;
    dmd_batch &B = h->b;
    std::string &err = B.err;
    const DSys &d = B.ds[0].d;
    size_t N = d.N;
    std::vector<int> np(N);
    std::vector<int8_t> ct(N);
    CK(cudaStreamSynchronize(B.st));
    if (tim) CK(cudaMemcpy(tim, d.tim, N * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(np.data(), d.nptnr, N * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ct.data(), d.colt, N, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < N; ++k) {
        if (nptnr) nptnr[k] = np[k] >= 0 ? np[k] + 1 : np[k];
        if (coltype) coltype[k] = ct[k];
    }
    return DMD_OK;
}
int dmd_get_state(dmd_handle *h, double *x, double *y, double *z, double *vx, double *vy, double *vz, int32_t *bptnr,
                  int32_t *identity, int32_t *er, double *t, double *tfalse, int64_t *coll) {
    if (!h) return DMD_E_INPUT;
    return get_state(h->b, 0, x, y, z, vx, vy, vz, bptnr, identity, er, t, tfalse, coll);
}
int dmd_diagnostics(dmd_handle *h, dmd_diag *out) {
    if (!h) return DMD_E_INPUT;
    return diagnostics(h->b, 0, out);
}
int dmd_phipsi_sample(dmd_handle *h) {
    if (!h) return DMD_E_INPUT;
    return phipsi_sample(h->b, 0);
}
int dmd_phipsi_histogram(dmd_handle *h, int64_t *hist, int64_t *nsamples, int32_t reset) {
    if (!h) return DMD_E_INPUT;
    return phipsi_histogram(h->b, 0, hist, nsamples, reset);
}
int dmd_get_evcode(dmd_handle *h, int8_t *out) {
    if (!h || !out || !h->b.ready) return DMD_E_INPUT;
    dmd_batch &B = h->b;
    std::string &err = B.err;
    const DSys &d = B.ds[0].d;
    const HostSys &H = B.hs[0];
    size_t N = d.N;
    std::vector<int> ovp(4 * N);
    std::vector<int8_t> ovc(4 * N);
    CK(cudaStreamSynchronize(B.st));
    CK(cudaMemcpy(ovp.data(), d.ovp, 4 * N * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ovc.data(), d.ovc, 4 * N, cudaMemcpyDeviceToHost));
    for (size_t a = 0; a < N; ++a)
        for (size_t b = 0; b < N; ++b) out[a * N + b] = a == b ? 1 : (int8_t)static_code(H.info[a], H.info[b], B.hbonds);
    for (size_t a = 0; a < N; ++a)
        for (int s = 0; s < 4; ++s)
            if (ovp[4 * a + s] >= 0) out[a * N + ovp[4 * a + s]] = ovc[4 * a + s];
    return DMD_OK;
}
void dmd_destroy(dmd_handle *h) {
    if (!h) return;
    batch_free(h->b);
    delete h;
}
const char *dmd_last_error(dmd_handle *h) { return h ? h->b.err.c_str() : "null handle"; }

int dmd_static_evcode(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys, int8_t *out,
                      char *err, int32_t errlen) {
    HostSys H;
    std::string e;
    if (!cfg || !tables || !sys || !out) return DMD_E_INPUT;
    if (!setup_host(H, cfg, tables, sys, e)) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.c_str());
        return DMD_E_INPUT;
    }
    size_t N = H.N;
    int hb = cfg->hbonds != 0;
    for (size_t a = 0; a < N; ++a)
        for (size_t b = 0; b < N; ++b) out[a * N + b] = a == b ? 1 : (int8_t)static_code(H.info[a], H.info[b], hb);
    return DMD_OK;
}

/* The prediction pass of dmd_create + dmd_predict_all for callers that cannot
 * allocate device memory: every intermediate array lives in the library's
 * static scratch (engine.cu g_noalloc_scratch), the outputs go to the
 * caller's device buffers, and no device memory is allocated or freed. */
int dmd_predict_all_noalloc(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                            double *d_tim, int32_t *d_nptnr, int32_t *d_coltype, void *stream,
                            char *err, int32_t errlen) {
    auto fail_msg = [&](int rc, const std::string &m) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", m.c_str());
        return rc;
    };
    if (!cfg || !tables || !sys || !d_tim || !d_nptnr || !d_coltype) return fail_msg(DMD_E_INPUT, "null argument");
    if (sys->n_beads > DMD_NOALLOC_MAX_BEADS)
        return fail_msg(DMD_E_CAPACITY, "dmd_predict_all_noalloc: at most " + std::to_string(DMD_NOALLOC_MAX_BEADS) +
                                            " beads (got " + std::to_string(sys->n_beads) + ")");
    if (cfg->list_cap > DMD_NOALLOC_MAX_CAP)
        return fail_msg(DMD_E_CAPACITY, "dmd_predict_all_noalloc: list_cap at most " + std::to_string(DMD_NOALLOC_MAX_CAP));
    dmd_run_cfg c = *cfg;
    if (c.list_cap <= 0) c.list_cap = DMD_NOALLOC_MAX_CAP;
    HostSys H;
    std::string e;
    if (!setup_host(H, &c, tables, sys, e)) return fail_msg(DMD_E_INPUT, e);
    if (H.ncell > DMD_NOALLOC_MAX_CELLS)
        return fail_msg(DMD_E_CAPACITY, "dmd_predict_all_noalloc: the box needs " + std::to_string(H.ncell) +
                                            " cells per side, at most " + std::to_string(DMD_NOALLOC_MAX_CELLS));
    /* the copies below come from pageable host memory and the call waits
     * for the stream: neither is allowed while a stream is captured */
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cap);
    if (ce != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return fail_msg(DMD_E_STATE, std::string("dmd_predict_all_noalloc may not be called while a stream is being "
                                                 "captured (") + (ce != cudaSuccess ? cudaGetErrorString(ce) : "capture active") + ")");
    void *base = nullptr;
    ce = dmd_noalloc_scratch(&base);
    if (ce != cudaSuccess) return fail_msg(DMD_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce));
    DSys d{};
    size_t bytes = layout(H, d, (char *)base, false);
    if (bytes > DMD_NOALLOC_SCRATCH_BYTES)
        return fail_msg(DMD_E_CAPACITY, "dmd_predict_all_noalloc: system needs " + std::to_string(bytes) +
                                            " scratch bytes, the array holds " + std::to_string(DMD_NOALLOC_SCRATCH_BYTES));
    d.N = H.N; d.nchains = H.nchains; d.cap = H.cap; d.ncell = H.ncell;
    d.seed = H.cfg.seed; d.canon = H.cfg.canon; d.flags = H.cfg.flags;
    d.nl1 = H.nl1; d.nl2 = H.nl2; d.log = nullptr; d.log_cap = 0;
    cudaStream_t st = (cudaStream_t)stream;
    size_t N = H.N;
    std::vector<double> tim(N + 3, H.sc.interval_max + DMD_LTSTEP);
    std::vector<int> np(N + 3, -1);
    std::vector<int8_t> ct(N + 3, -1);
    std::vector<uint8_t> q(N + 3, 0);
    if (H.cfg.canon) {
        double tgho = 0.0;
        uint32_t k = 0;
        while ((tgho < 1e-18) || (tgho == 1.0)) tgho = dmd_uniform(H.cfg.seed, DMD_STREAM_GHOST0, 0, k++);
        tim[N] = -1.0 * dmd_log(tgho) * H.tab.avegtime * .0000001;
    } else {
        tim[N] = 1000000000.0;
    }
    tim[N + 1] = H.sc.interval;
    tim[N + 2] = 3.3 / (std::sqrt(H.tab.setemp)) + 5;
    np[N] = np[N + 1] = np[N + 2] = -2;
    ct[N] = ct[N + 1] = ct[N + 2] = -2;
    struct Cp { void *dst; const void *src; size_t n; };
    const Cp cps[] = {
        {(void *)d.tab, &H.tab, sizeof(DTab)}, {d.sc, &H.sc, sizeof(DScal)},
        {(void *)d.info, H.info.data(), N * sizeof(BeadInfo)}, {(void *)d.bm, H.bm.data(), N * 8},
        {(void *)d.blmin, H.blmin.data(), N * 8}, {(void *)d.blmax, H.blmax.data(), N * 8},
        {(void *)d.blmin_sq, H.blmin_sq.data(), N * 8}, {(void *)d.blmax_sq, H.blmax_sq.data(), N * 8},
        {(void *)d.rblmin_sq, H.rblmin_sq.data(), N * 8}, {(void *)d.rblmax_sq, H.rblmax_sq.data(), N * 8},
        {d.x, H.x.data(), N * 8}, {d.y, H.y.data(), N * 8}, {d.z, H.z.data(), N * 8},
        {d.vx, H.vx.data(), N * 8}, {d.vy, H.vy.data(), N * 8}, {d.vz, H.vz.data(), N * 8},
        {d.ident, H.ident.data(), N}, {d.bptnr, H.bptnr.data(), N * 4}, {d.er, H.er.data(), 4 * N * 4},
        {d.ovp, H.ovp.data(), 4 * N * 4}, {d.ovc, H.ovc.data(), 4 * N},
        {d.tim, tim.data(), (N + 3) * 8}, {d.nptnr, np.data(), (N + 3) * 4}, {d.colt, ct.data(), N + 3},
        {d.queued, q.data(), N + 3},
    };
    for (const Cp &cp : cps) {
        ce = cudaMemcpyAsync(cp.dst, cp.src, cp.n, cudaMemcpyHostToDevice, st);
        if (ce != cudaSuccess) return fail_msg(DMD_E_CUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(ce));
    }
    ce = dmd_launch_predict_noalloc(d, H.cfg.hbonds != 0, d_tim, (int *)d_nptnr, (int *)d_coltype, st);
    if (ce != cudaSuccess) return fail_msg(DMD_E_CUDA, std::string("launch: ") + cudaGetErrorString(ce));
    DScal sc;
    ce = cudaMemcpyAsync(&sc, d.sc, sizeof sc, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return fail_msg(DMD_E_CUDA, std::string("sync: ") + cudaGetErrorString(ce));
    if (sc.err) return fail_msg(sc.err, "device error " + std::to_string(sc.err) + " (info " + std::to_string(sc.err_info) + ")");
    return DMD_OK;
}

int dmd_inspect(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys, double *out, int32_t n,
                char *err, int32_t errlen) {
    HostSys H;
    std::string e;
    if (!cfg || !tables || !sys || !out) return DMD_E_INPUT;
    if (!setup_host(H, cfg, tables, sys, e)) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.c_str());
        return DMD_E_INPUT;
    }
    double v[] = {H.sc.interval, H.sc.interval_max, H.sig_max_all, H.tab.hdelr, (double)H.ncell, H.tab.rl,
                  H.tab.rlsq[1], H.tab.rlsq[15], H.tab.rlsq[16], H.tab.rlsq[40], H.sc.n_forced, H.sc.t_fact,
                  H.tab.evp1[15]};
    int m = (int)(sizeof v / sizeof v[0]);
    for (int k = 0; k < n && k < m; ++k) out[k] = v[k];
    return m;
}


/* ---- serving ---- */
int dmd_server_create(int32_t max_slots, int64_t hbm_budget_bytes, int64_t chunk_events, dmd_server **out) {
    if (!out) return DMD_E_INPUT;
    dmd_server *V = new dmd_server();
    *out = V;
    std::string &err = V->err;
    if (max_slots <= 0 || chunk_events <= 0) { err = "max_slots and chunk_events must be positive"; return DMD_E_INPUT; }
    V->max_slots = max_slots;
    V->chunk = chunk_events;
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    size_t cap = (size_t)(0.9 * (double)free_b);
    V->budget = hbm_budget_bytes > 0 ? std::min<size_t>((size_t)hbm_budget_bytes, cap) : cap;
    CK(cudaStreamCreateWithFlags(&V->run_st, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&V->copy_st, cudaStreamNonBlocking));
    CK(cudaEventCreate(&V->e0));
    CK(cudaEventCreate(&V->e1));
    return DMD_OK;
}
int dmd_server_submit(dmd_server *V, const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                      int64_t n_events, int64_t *id) {
    if (!V || !cfg || !tables || !sys || !id) return DMD_E_INPUT;
    if (n_events <= 0) { V->err = "n_events must be positive"; return DMD_E_INPUT; }
    ServerReq *R = new ServerReq();
    std::string e;
    if (!setup_host(R->H, cfg, tables, sys, e)) { delete R; V->err = e; return DMD_E_INPUT; }
    DSys tmp{};
    R->need = layout(R->H, tmp, nullptr);
    R->total = n_events;
    R->t_submit = now_s();
    std::lock_guard<std::mutex> lock(V->mu);
    int hb = cfg->hbonds != 0;
    if (V->hbonds < 0) V->hbonds = hb;
    if (V->hbonds != hb) { delete R; V->err = "all requests of a server share the hbonds flag"; return DMD_E_INPUT; }
    if (R->need > V->budget) { delete R; V->err = "request larger than the device-memory budget"; return DMD_E_CAPACITY; }
    R->id = V->next_id++;
    V->reqs[R->id] = R;
    V->waiting.push_back(R);
    *id = R->id;
    return DMD_OK;
}
int dmd_server_step(dmd_server *V, int32_t *n_active, int32_t *n_finished) {
    if (!V) return DMD_E_INPUT;
    return server_step(*V, n_active, n_finished);
}
int dmd_server_status(dmd_server *V, int64_t id, int32_t *state, int64_t *events_done, double *t_submit,
                      double *t_admit, double *t_finish) {
    if (!V) return DMD_E_INPUT;
    std::lock_guard<std::mutex> lock(V->mu);
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) { V->err = "unknown request"; return DMD_E_INPUT; }
    ServerReq &R = *it->second;
    if (state) *state = R.state;
    if (events_done) *events_done = R.done;
    if (t_submit) *t_submit = R.t_submit;
    if (t_admit) *t_admit = R.t_admit;
    if (t_finish) *t_finish = R.t_finish;
    return R.state == DMD_REQ_FAILED ? R.rc : DMD_OK;
}
int dmd_server_result(dmd_server *V, int64_t id, dmd_diag *diag, double *x, double *y, double *z, double *vx,
                      double *vy, double *vz, int32_t *bptnr, int32_t *identity, double *t, double *tfalse,
                      int64_t *coll) {
    if (!V) return DMD_E_INPUT;
    std::lock_guard<std::mutex> lock(V->mu);
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) { V->err = "unknown request"; return DMD_E_INPUT; }
    ServerReq &R = *it->second;
    if (R.state == DMD_REQ_FAILED) { V->err = R.err; return R.rc; }
    if (R.state != DMD_REQ_DONE) { V->err = "request not finished"; return DMD_E_STATE; }
    size_t N = R.H.N;
    if (diag) *diag = R.diag;
    if (x) { std::memcpy(x, R.x.data(), N * 8); std::memcpy(y, R.y.data(), N * 8); std::memcpy(z, R.z.data(), N * 8); }
    if (vx) { std::memcpy(vx, R.vx.data(), N * 8); std::memcpy(vy, R.vy.data(), N * 8); std::memcpy(vz, R.vz.data(), N * 8); }
    if (bptnr) std::memcpy(bptnr, R.bptnr.data(), N * 4);
    if (identity) std::memcpy(identity, R.ident.data(), N * 4);
    if (t) *t = R.t;
    if (tfalse) *tfalse = R.tfalse;
    if (coll) *coll = R.coll;
    return DMD_OK;
}
int dmd_server_release(dmd_server *V, int64_t id) {
    if (!V) return DMD_E_INPUT;
    std::lock_guard<std::mutex> lock(V->mu);
    auto it = V->reqs.find(id);
    if (it == V->reqs.end()) { V->err = "unknown request"; return DMD_E_INPUT; }
    if (it->second->state == DMD_REQ_QUEUED || it->second->state == DMD_REQ_ACTIVE) {
        V->err = "request still queued or running"; return DMD_E_STATE;
    }
    delete it->second;
    V->reqs.erase(it);
    return DMD_OK;
}
int dmd_server_stats(dmd_server *V, int64_t *steps, int64_t *events, double *kernel_ms, int32_t *n_waiting,
                     int32_t *n_active, int64_t *bytes_used, int64_t *bytes_budget) {
    if (!V) return DMD_E_INPUT;
    std::lock_guard<std::mutex> lock(V->mu);
    if (steps) *steps = V->steps;
    if (events) *events = V->events;
    if (kernel_ms) *kernel_ms = V->kernel_ms;
    if (n_waiting) *n_waiting = (int32_t)V->waiting.size();
    if (n_active) *n_active = (int32_t)V->active.size();
    if (bytes_used) *bytes_used = (int64_t)V->used;
    if (bytes_budget) *bytes_budget = (int64_t)V->budget;
    return DMD_OK;
}
const char *dmd_server_last_error(dmd_server *V) { return V ? V->err.c_str() : "null handle"; }
void dmd_server_destroy(dmd_server *V) {
    if (!V) return;
    if (V->run_st) cudaStreamSynchronize(V->run_st);
    if (V->copy_st) cudaStreamSynchronize(V->copy_st);
    for (auto &kv : V->reqs) {
        if (kv.second->D.pool) cudaFree(kv.second->D.pool);
        delete kv.second;
    }
    if (V->d_sys) cudaFree(V->d_sys);
    if (V->d_targets) cudaFree(V->d_targets);
    if (V->d_cstart) cudaFree(V->d_cstart);
    if (V->d_clen) cudaFree(V->d_clen);
    if (V->d_coff) cudaFree(V->d_coff);
    if (V->d_diag) cudaFree(V->d_diag);
    if (V->e0) cudaEventDestroy(V->e0);
    if (V->e1) cudaEventDestroy(V->e1);
    if (V->run_st) cudaStreamDestroy(V->run_st);
    if (V->copy_st) cudaStreamDestroy(V->copy_st);
    delete V;
}


/* ---- checkpoint: the whole device state of a system ---- */
namespace {
struct CkptHeader {
    char magic[8];                 /* "DMDGBCK1" */
    int64_t n_beads, cap, ncell, bytes;
};
}
int64_t dmd_state_bytes(dmd_handle *h) {
    if (!h || !h->b.ready) return DMD_E_STATE;
    return (int64_t)(sizeof(CkptHeader) + h->b.ds[0].bytes);
}
int dmd_save_state(dmd_handle *h, void *buf, int64_t n) {
    if (!h || !h->b.ready) return DMD_E_STATE;
    dmd_batch &B = h->b;
    std::string &err = B.err;
    const DevSys &D = B.ds[0];
    if (!buf || n < (int64_t)(sizeof(CkptHeader) + D.bytes)) { err = "buffer smaller than dmd_state_bytes()"; return DMD_E_INPUT; }
    CkptHeader hd{};
    std::memcpy(hd.magic, "DMDGBCK1", 8);
    hd.n_beads = B.hs[0].N; hd.cap = B.hs[0].cap; hd.ncell = B.hs[0].ncell; hd.bytes = (int64_t)D.bytes;
    std::memcpy(buf, &hd, sizeof hd);
    CK(cudaStreamSynchronize(B.st));
    CK(cudaMemcpy((char *)buf + sizeof hd, (const void *)D.d.tab, D.bytes, cudaMemcpyDeviceToHost));
    return DMD_OK;
}
int dmd_load_state(dmd_handle *h, const void *buf, int64_t n) {
    if (!h || !h->b.ready) return DMD_E_STATE;
    dmd_batch &B = h->b;
    std::string &err = B.err;
    const DevSys &D = B.ds[0];
    CkptHeader hd{};
    if (!buf || n < (int64_t)sizeof hd) { err = "buffer too small"; return DMD_E_INPUT; }
    std::memcpy(&hd, buf, sizeof hd);
    if (std::memcmp(hd.magic, "DMDGBCK1", 8) != 0) { err = "not a checkpoint of this engine"; return DMD_E_INPUT; }
    if (hd.n_beads != B.hs[0].N || hd.cap != B.hs[0].cap || hd.ncell != B.hs[0].ncell || hd.bytes != (int64_t)D.bytes ||
        n < (int64_t)(sizeof hd + D.bytes)) {
        err = "checkpoint of a different system shape (beads, list capacity or grid)";
        return DMD_E_INPUT;
    }
    CK(cudaStreamSynchronize(B.st));
    CK(cudaMemcpy((void *)D.d.tab, (const char *)buf + sizeof hd, D.bytes, cudaMemcpyHostToDevice));
    DScal sc;
    CK(cudaMemcpy(&sc, D.d.sc, sizeof sc, cudaMemcpyDeviceToHost));
    B.hs[0].sc = sc;
    B.diag_valid = false;
    B.state_valid = false;
    return DMD_OK;
}

}  // extern "C"
