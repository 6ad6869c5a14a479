/*
 * engine.cuh -- device data layout and per-pair physics of the GB300 DMD
 * event engine.
 *
 * Every expression below keeps the operation order of the reference Fortran
 * (cited per function) and the build uses --fmad=false, so a prediction or
 * an impulse computed here is bit-identical to the same arithmetic on the
 * host.  Bead indices are 0-based on the device; -1 means "none".
 */
#ifndef DMD_ENGINE_CUH
#define DMD_ENGINE_CUH

#include <stdint.h>
#include "dmd_rng.h"

#define DMD_NT 29     /* identities 1..28 */
#define DMD_NC 51     /* pair codes 1..50 */
#define DMD_LTSTEP 1e-10
#define DMD_SMDIST 5e-12
#define DMD_BIG 1000000000.0

/* bead kind inside a chain */
#define BK_CA 0
#define BK_NH 1
#define BK_CO 2
#define BK_R 3

/* per-bead static description (make_code inputs, code/make_code.f) */
struct BeadInfo {
    int32_t chain;     /* chain index */
    int32_t cstart;    /* index of the chain's first bead */
    int16_t L;         /* residues in the chain */
    int16_t res;       /* residue number 1..L this bead belongs to */
    int8_t kind;       /* BK_* */
    int8_t hp;         /* hydrophobic flag */
    int8_t pro_nh;     /* NH whose index equals a proline side chain minus 2L */
    int8_t is_end;     /* NH of residue 1 or CO of residue L */
    int8_t sp2;        /* on a species-2 chain of a two-species run (chaptype 2) */
};

/* box-scaled tables (code/scale_down.f, code/make_code.f:15-60, code/nbor_setup.f) */
struct DTab {
    double sigma_sq[DMD_NT][DMD_NT];
    double welldia_sq[DMD_NT][DMD_NT];
    double ep_sqrt[DMD_NT][DMD_NT];
    double shlddia_sq[DMD_NT][DMD_NT];
    double sqz610[6][DMD_NT];
    double evp1[DMD_NC], evp2[DMD_NC], evp3[DMD_NC];
    double rlsq[DMD_NC];
    float rlsq_f[DMD_NC];         /* the same rounded to single precision (list-build prefilter) */
    float rlsq_max_f;             /* their maximum */
    double shd1, shd2, shd3, shd4;
    double eps1;       /* epsilon(1): H-bond depth */
    double setemp, avegtime, hdelr, rl;
    double eps_hb;     /* ep_sqrt(5,8) */
    double boxl_orig;
    /* squared contact diameters, computed once in the predictors' own
     * operation order (so a lookup gives the same bits as the inline
     * product): core codes 1-3 and 17-26 (slot core_slot(code)), the
     * bonded H-bond pair's inner core (code 15), the bond windows */
    double core_sq[14][DMD_NT][DMD_NT];
    double ncfac_sq[DMD_NT][DMD_NT];
    double core15_sq[DMD_NT][DMD_NT];    /* eventdyn.f's bonded H-bond core (code 15) */
    double rmass[DMD_NT][DMD_NT];        /* 2*m_a*m_b/(m_a+m_b), code/eventdyn.f:40 */
    double rbm[DMD_NT];                  /* 1/mass, rounded to nearest (for div_by) */
    double revp2_sq[DMD_NC], revp3_sq[DMD_NC];   /* 1/evp2_sq, 1/evp3_sq */
    double evp2_sq[DMD_NC], evp3_sq[DMD_NC];
    /* reciprocals rounded to nearest of the divisors of eventdyn.f, for
     * div_by(): the core diameters, the wells and shoulders (and twice
     * them), the reduced masses */
    double rcore_sq[14][DMD_NT][DMD_NT];
    double rcore15_sq[DMD_NT][DMD_NT], rsigma_sq[DMD_NT][DMD_NT];
    double rwell_sq[DMD_NT][DMD_NT], r2well_sq[DMD_NT][DMD_NT];
    double rshld_sq[DMD_NT][DMD_NT], r2shld_sq[DMD_NT][DMD_NT];
    double rrmass[DMD_NT][DMD_NT];
};
/* Checked build (-DDMD_BOUNDS): every index DMD_CHK guards is tested
 * against its array's extent; the first one outside it is recorded in
 * g_dmd_bounds (site << 40 | extent << 20 | index, 20 bits each, plus one in
 * bit 62) and replaced by 0, so that the kernel carries on without a fault
 * and the host reports it (dmd_debug_bounds).  Other builds: no check. */
#ifdef DMD_BOUNDS
__device__ unsigned long long g_dmd_bounds;
__device__ __forceinline__ int dmd_chk(int i, int n, int site) {
    if ((unsigned)i < (unsigned)n) return i;
    const unsigned long long rec = (1ull << 62) | ((unsigned long long)(site & 0x3fffff) << 40) |
                                   ((unsigned long long)(n & 0xfffff) << 20) | (unsigned long long)(i & 0xfffff);
    atomicCAS(&g_dmd_bounds, 0ull, rec);
    return 0;
}
#define DMD_CHK(i, n, site) dmd_chk((i), (n), (site))
#else
#define DMD_CHK(i, n, site) (i)
#endif

__host__ __device__ __forceinline__ int core_slot(int code) { return code <= 3 ? code : code - 13; }
/* slot of a squeezed or plain core code (1-3, 17-26) in DTab::core_sq */
__device__ __forceinline__ int core_slot_d(int code) { return DMD_CHK(core_slot(code), 14, 1); }

/* per-system scalars kept between launches */
struct DScal {
    double t, tfalse, old_tfalse, interval, interval_max, t_fact, n_forced;
    long long coll, n_pair, n_ghost, n_interval, n_output, n_updates, n_forced_updates, ghost_index;
    long long nevents[32];
    long long log_count;
    long long done;       /* events counted toward the current run target */
    int err;              /* DMD_E_* of the first device error, 0 if none */
    int err_info;
    int stop;             /* 1: stopped at an output event */
    int max_dn;           /* the longest down list of the last rebuild */
    long long n_batches, n_rolled_back, n_candidates;   /* batch statistics */
    long long bseq;       /* footprint claims made so far (ticket base) */
    long long run_cycles; /* SM clock cycles of this system's last launch (scheduling hint) */
    long long done_all;   /* events over all launches since the host last cleared it */
    int need_full;        /* 1: a compact launch stopped here; lists need the full variant */
    int err_info2;        /* second bead of an overlap error (err_info holds the first) */
};

/* device view of one system; all arrays in global memory */
struct DSys {
    int N, nchains, cap, ncell;   /* ncell: cells per side of the rebuild grid */
    uint64_t seed;
    int canon, flags;
    const DTab *tab;
    DScal *sc;
    const BeadInfo *info;
    const double *bm;
    const double *blmin, *blmax;  /* side-chain bond window of a backbone bead (codes 10/11/12) */
    const double *blmin_sq, *blmax_sq;   /* their squares */
    const double *rblmin_sq, *rblmax_sq; /* and the reciprocals of those, rounded to nearest */
    double *x, *y, *z, *vx, *vy, *vz;
    double *ox, *oy, *oz;          /* positions at the last list rebuild */
    float *xf, *yf, *zf;           /* the same in single precision (list-build prefilter) */
    int8_t *ident;                 /* identity 1..28 (5..8: bonded backbone) */
    int *bptnr;                    /* H-bond partner or -1 */
    int *er;                       /* extra_repuls(b,1..4) at er[4b+0..3], -1 = none */
    int *ovp;                      /* shoulder overrides: partner at ovp[4b+s], -1 free */
    int8_t *ovc;                   /* ev_code(b, partner) of the override */
    double *tim;                   /* N + 3 entries: beads, ghost, interval, output */
    int *nptnr;
    int8_t *colt;
    uint8_t *queued;
    long long *key;                /* ordered integer key of (queued ? tim : +inf), N + 3 entries */
    unsigned int *owner;           /* footprint tickets (read, write, queue: 3N entries), when not in shared memory */
    int *up, *dn;                  /* neighbour lists [N*cap] */
    int8_t *upc;                   /* static pair code of each up entry */
    int8_t *dnc;                   /* ... and of each down entry (event loop only; may be NULL) */
    int *upn, *dnn;
    int *cell_count, *cell_start, *cell_beads;  /* rebuild grid */
    int *l1i;                      /* tournament level 1: argmin of 32 entries */
    int *l2i;                      /* level 2: argmin of 32 level-1 groups */
    long long *l1k, *l2k;          /* the keys of those minima */
    int nl1, nl2;
    void *log;                     /* dmd_event ring or NULL */
    long long log_cap;
};

/* ------------------------------------------------------------------ */
__device__ __forceinline__ double d_nint(double x) { return round(x); }

/* lexicographic (time, partner) order used for every minimum */
__device__ __forceinline__ bool lex_less(double ta, int pa, double tb, int pb) {
    return ta < tb || (ta == tb && pa < pb);
}

/* Integer key with the order of the doubles (finite values; -0 and +0 equal):
 * comparisons of event times run on the integer pipes, not the FP64 unit. */
#define DMD_KEY_INF 0x7fffffffffffffffLL
__host__ __device__ __forceinline__ long long okey(double t) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(t);
#else
    long long b;
    memcpy(&b, &t, sizeof b);
#endif
    if (b == (long long)0x8000000000000000ULL) b = 0;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool key_less(long long ka, int pa, long long kb, int pb) {
    return ka < kb || (ka == kb && pa < pb);
}

/* static pair code: code/make_code.f:6-573 applied per chain, as a rule */
/* codes for residue offsets d = -2..2, 5 bits each */
#define DMD_BOND_ROW(m2, m1, z, p1, p2) \
    ((uint32_t)(m2) | ((uint32_t)(m1) << 5) | ((uint32_t)(z) << 10) | ((uint32_t)(p1) << 15) | ((uint32_t)(p2) << 20))
__host__ __device__ __forceinline__ int bond_code_dir(int ka, int kb, int ra, int rb) {
    /* the bonded and squeezed pair codes of make_code.f by bead kinds and
     * residue offset d = rb - ra: one packed word per pair of kinds, picked
     * by selects rather than a switch (a switch whose lanes take different
     * cases runs them one after another) */
    const int d = rb - ra;
    const int pk = ka * 4 + kb;
    uint32_t w = 0;
    w = pk == BK_CA * 4 + BK_NH ? DMD_BOND_ROW(0, 18, 4, 7, 0) : w;
    w = pk == BK_CA * 4 + BK_CO ? DMD_BOND_ROW(0, 8, 5, 17, 0) : w;
    w = pk == BK_NH * 4 + BK_CO ? DMD_BOND_ROW(19, 6, 8, 0, 0) : w;
    w = pk == BK_CA * 4 + BK_CA ? DMD_BOND_ROW(0, 0, 0, 9, 0) : w;
    w = pk == BK_CA * 4 + BK_R ? DMD_BOND_ROW(0, 25, 10, 24, 0) : w;
    w = pk == BK_NH * 4 + BK_R ? DMD_BOND_ROW(0, 23, 11, 0, 0) : w;
    w = pk == BK_CO * 4 + BK_R ? DMD_BOND_ROW(0, 0, 12, 22, 26) : w;
    w = pk == BK_NH * 4 + BK_NH ? DMD_BOND_ROW(0, 0, 0, 20, 0) : w;
    w = pk == BK_CO * 4 + BK_CO ? DMD_BOND_ROW(0, 0, 0, 21, 0) : w;
    const unsigned sh = (unsigned)(d + 2);
    return sh <= 4u ? (int)((w >> (5u * sh)) & 31u) : 0;
}

__host__ __device__ __forceinline__ int static_code(const BeadInfo &A, const BeadInfo &B, int hbonds) {
    /* every case evaluated and the result picked by selects: the lanes of a
     * warp hold pairs of all kinds, and branches on the kinds would run one
     * after another */
    const bool same = A.chain == B.chain;
    const int c1 = bond_code_dir(A.kind, B.kind, A.res, B.res);
    const int c2 = bond_code_dir(B.kind, A.kind, B.res, A.res);
    const int cb = c1 ? c1 : c2;                       /* bonded or squeezed pair of one chain */
    int dr = A.res - B.res;
    dr = dr < 0 ? -dr : dr;
    const bool rr = A.kind == BK_R && B.kind == BK_R;
    const bool hp = A.hp == 1 && B.hp == 1;
    const bool nc = A.kind == BK_NH && B.kind == BK_CO;
    const bool cn = A.kind == BK_CO && B.kind == BK_NH;
    /* one chain (make_code.f's intra-chain blocks) */
    const int rr_intra = (dr >= 4 && hp) ? 16 : 1;
    const int hb_intra = (hbonds && (nc || cn)) ? (dr >= 4 ? 15 : 1) : 1;
    const int intra = cb ? cb : (rr ? rr_intra : hb_intra);
    /* two chains; two species-2 chains' side chains meet as hard cores
     * (code/make_code.f:515-541) */
    const int rr_inter = (hp && !(A.sp2 && B.sp2)) ? 16 : 1;
    const int nc_inter = (A.pro_nh && B.chain > A.chain) ? 1 : 15;
    const int cn_inter = (B.pro_nh && A.chain > B.chain) ? 1 : 15;
    const int hb_inter = hbonds ? (nc ? nc_inter : (cn ? cn_inter : 1)) : 1;
    const int inter = rr ? rr_inter : hb_inter;
    return same ? intra : inter;
}

/* ev_code(a,b) when the static code of the pair is already known */
__device__ __forceinline__ int pair_code_st(const DSys &S, int a, int b, int st) {
    /* the first override slot holding b, picked by selects (all loads issued
     * together, no early exit) */
    const int *op = S.ovp + 4 * a;
    const int8_t *oc = S.ovc + 4 * a;
    const int o0 = op[0], o1 = op[1], o2 = op[2], o3 = op[3];
    const int c0 = oc[0], c1 = oc[1], c2 = oc[2], c3 = oc[3];
    int r = st;
    r = o3 == b ? c3 : r;
    r = o2 == b ? c2 : r;
    r = o1 == b ? c1 : r;
    r = o0 == b ? c0 : r;
    return r;
}
/* ev_code(a,b): the rule plus the H-bond shoulder overrides of repuls_add */
__device__ __forceinline__ int pair_code(const DSys &S, int a, int b, int hbonds) {
    return pair_code_st(S, a, b, static_code(S.info[a], S.info[b], hbonds));
}

/* ------------------------------------------------------------------ */
struct Rel { double rx, ry, rz, vx, vy, vz, bij, rijsq, vijsq; };

/* relative coordinates advanced to tfalse with the minimum image
 * (code/core.f:14-24 and the copies in every predictor) */
__device__ __forceinline__ Rel d_rel(const DSys &S, int i, int j, double tfalse) {
    Rel r;
    r.vx = S.vx[i] - S.vx[j]; r.vy = S.vy[i] - S.vy[j]; r.vz = S.vz[i] - S.vz[j];
    r.rx = S.x[i] - S.x[j] + r.vx * tfalse;
    r.ry = S.y[i] - S.y[j] + r.vy * tfalse;
    r.rz = S.z[i] - S.z[j] + r.vz * tfalse;
    r.rx = r.rx - d_nint(r.rx); r.ry = r.ry - d_nint(r.ry); r.rz = r.rz - d_nint(r.rz);
    r.bij = r.rx * r.vx + r.ry * r.vy + r.rz * r.vz;
    r.rijsq = r.rx * r.rx + r.ry * r.ry + r.rz * r.rz;
    r.vijsq = r.vx * r.vx + r.vy * r.vy + r.vz * r.vz;
    return r;
}

/* code/bond.f:19-33 */
__device__ __forceinline__ void bond_limits(const DSys &S, int i, int evcode, double &blmin, double &blmax) {
    if (evcode >= 10 && evcode <= 12) { blmin = S.blmin[i]; blmax = S.blmax[i]; }
    else { blmin = S.tab->evp2[evcode]; blmax = S.tab->evp3[evcode]; }
}

/* ------------------------------------------------------------------ */
/* pair prediction with warp-convergent control flow                  */
/* ------------------------------------------------------------------ */
/* Pair prediction: the dispatch of code/eventredo_up.f:28-46 into
 * code/core.f, bond.f, nc_sqwel.f, sqwel.f and sqshlder.f.  Returns false on
 * an invalid code (reference: "error in ev_code matrix").
 *
 * On GB300 an FP64 warp instruction occupies the SM sub-partition's FP64
 * unit for about 64 cycles whatever the number of active lanes, and lanes
 * of one warp that take different branches pay for every branch.  So the
 * predictors are not written branch by branch; they give the reference's
 * (tij, type) bit for bit, because every branch of them is one of
 *   tij = (-bij - sqrt(D)) / vijsq,  (-bij + sqrt(D)) / vijsq,
 *   or  -(rijsq - R) / (sqrt(D) + bij)          (bond.f, outward, bij >= 0)
 * with D = bij*bij - vijsq*(rijsq - R) for one or two squared diameters R
 * chosen by integer tests, so all lanes run one or two discriminants, one
 * square root and one division.  Sign and order tests read the bit
 * patterns on the integer pipes, and the minimum image skips the rounding
 * where |r| < 0.5 (there x - nint(x) == x exactly). */

__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
/* x < 0.0 (false for -0.0) */
__device__ __forceinline__ bool d_lt0(double x) { long long b = dbits(x); return b < 0 && b != (long long)0x8000000000000000ULL; }
/* x > 0.0 */
__device__ __forceinline__ bool d_gt0(double x) { return dbits(x) > 0; }
/* a < b for a, b >= +0.0 (non-negative, not NaN) */
__device__ __forceinline__ bool d_lt_nn(double a, double b) { return dbits(a) < dbits(b); }
/* a / b rounded to nearest, given rb = RN(1/b) (an IEEE division on the
 * host): q = RN(a*rb) is within one ulp of a/b, the remainder a - b*q is
 * exact in one fused multiply-add, and RN(q + remainder*rb) is then the
 * correctly rounded quotient (Markstein's theorem, IBM J. Res. Dev. 34(1),
 * 1990; no overflow or underflow in this engine's ranges).  Three FP64
 * instructions instead of a full division; a zero numerator keeps its
 * sign. */
__device__ __forceinline__ double div_by(double a, double b, double rb) {
    double q = a * rb;
    if ((__double_as_longlong(a) & 0x7fffffffffffffffLL) == 0) return q;
    double r = fma(-q, b, a);
    return fma(r, rb, q);
}
__device__ __forceinline__ double d_negate(double x) { return __longlong_as_double(dbits(x) ^ (long long)0x8000000000000000ULL); }
/* x - nint(x); skips the rounding where |x| < 0.5 and x is not -0.0 */
__device__ __forceinline__ double d_wrap(double x) {
    long long b = dbits(x);
    if ((b & 0x7fffffffffffffffLL) < 0x3fe0000000000000LL && b != (long long)0x8000000000000000ULL) return x;
    return x - round(x);
}
/* x - round(x) (round half away from zero) as one subtraction where
 * |x| < 1.5: round(x) is then +-0 (with the sign of x) or +-1, read from
 * the bits, so a warp of pairs issues one FP64 instruction per component
 * whether or not some lane wraps (neighbours are never a box and a half
 * apart; larger |x| and NaN take the rounding) */
__device__ __forceinline__ double d_wrap1(double x) {
    const long long b = dbits(x), a = b & 0x7fffffffffffffffLL;
    if (a >= 0x3ff8000000000000LL) return x - round(x);
    const long long s = (a >= 0x3fe0000000000000LL ? 0x3ff0000000000000LL : 0LL) | (b & (long long)0x8000000000000000ULL);
    return x - __longlong_as_double(s);
}
/* si, sj: the bead's position and velocity (x, y, z, vx, vy, vz) where they
 * are not the current state (a snapshot), else null */
__device__ __forceinline__ Rel d_rel_cv(const DSys &S, int i, int j, double tfalse, const double *si,
                                        const double *sj) {
    Rel r;
    i = DMD_CHK(i, S.N, 2);
    j = DMD_CHK(j, S.N, 3);
    const double vxi = si ? si[3] : S.vx[i], vyi = si ? si[4] : S.vy[i], vzi = si ? si[5] : S.vz[i];
    const double vxj = sj ? sj[3] : S.vx[j], vyj = sj ? sj[4] : S.vy[j], vzj = sj ? sj[5] : S.vz[j];
    const double xi = si ? si[0] : S.x[i], yi = si ? si[1] : S.y[i], zi = si ? si[2] : S.z[i];
    const double xj = sj ? sj[0] : S.x[j], yj = sj ? sj[1] : S.y[j], zj = sj ? sj[2] : S.z[j];
    r.vx = vxi - vxj; r.vy = vyi - vyj; r.vz = vzi - vzj;
    r.rx = xi - xj + r.vx * tfalse;
    r.ry = yi - yj + r.vy * tfalse;
    r.rz = zi - zj + r.vz * tfalse;
    r.rx = d_wrap1(r.rx); r.ry = d_wrap1(r.ry); r.rz = d_wrap1(r.rz);
    r.bij = r.rx * r.vx + r.ry * r.vy + r.rz * r.vz;
    r.rijsq = r.rx * r.rx + r.ry * r.ry + r.rz * r.rz;
    r.vijsq = r.vx * r.vx + r.vy * r.vy + r.vz * r.vz;
    return r;
}
__device__ __forceinline__ Rel d_rel_c(const DSys &S, int i, int j, double tfalse) {
    return d_rel_cv(S, i, j, tfalse, nullptr, nullptr);
}

/* ------------------------------------------------------------------ */
/* single-precision screen for "no event"                              */
/* ------------------------------------------------------------------ */
/* A double read as a float from its high word: the exponent rebiased and
 * the mantissa truncated to 20 bits (relative error below 2^-20), in three
 * integer operations.  Exact only for exponents that fit a normal float
 * (2^-126 <= |x| < 2^128); `bad` collects the others (zeros among them). */
__device__ __forceinline__ float f32_hi(unsigned hi, unsigned &bad) {
    bad |= ((hi & 0x7ff00000u) - 0x38100000u) > (0x47e00000u - 0x38100000u);
    return __uint_as_float(((hi - 0x38000000u) << 3) | (hi & 0x80000000u));
}
__device__ __forceinline__ unsigned d_hi(const double *p) { return reinterpret_cast<const unsigned *>(p)[1]; }

/* True only when d_predict_c(S, i, j, evcode, tfalse) gives no event
 * (k = PK_NONE, tij = DMD_BIG, type 0): the pair separates (bij > 0), or
 * the discriminant of the shell it would meet is negative, and for the
 * two-stage wells it is outside the well.  bij, rijsq, vijsq and the
 * discriminant are evaluated in single precision from the doubles' high
 * words, each with a bound on every error - the truncation of the inputs,
 * the single-precision arithmetic and the double-precision arithmetic of
 * d_rel_c - and a test is taken only when it holds beyond its bound; the
 * minimum image is taken only away from half a box, and inputs outside the
 * normal float range (zeros) decide nothing.  Bond pairs (always an
 * event), bonded H-bond pairs and invalid codes are not screened.  tf_hi
 * is the high word of tfalse. */
__device__ __forceinline__ bool f32_no_event(const DSys &S, int i, int j, int evcode, unsigned tf_hi,
                                             const double *si = nullptr, const double *sj = nullptr) {
    /* every load first: positions and velocities (or the snapshots si, sj,
     * as in d_rel_cv), identities, H-bond partner */
    unsigned h[12];
    const double *P[6] = {S.x, S.y, S.z, S.vx, S.vy, S.vz};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        h[2 * k] = si ? d_hi(si + k) : d_hi(P[k] + i);
        h[2 * k + 1] = sj ? d_hi(sj + k) : d_hi(P[k] + j);
    }
    const int a = S.ident[i], b = S.ident[j];
    const bool core = evcode <= 3 || (evcode >= 17 && evcode <= 26);
    const bool well = evcode == 15 || evcode == 16 || evcode >= 40;
    if (!core && !well) return false;
    if (evcode == 15 && a + b != 5 && S.bptnr[i] == j) return false;
    const DTab &T = *S.tab;
    const double *Rp = core ? &T.core_sq[core_slot_d(evcode)][a][b]
                            : evcode >= 40 ? &T.shlddia_sq[a][b] : &T.welldia_sq[a][b];
    const bool need_out = well && (evcode != 15 || a + b == 5);
    const unsigned Rh = d_hi(Rp);
    const float C1 = 3.814697265625e-06f;   /* 2^-18 */
    const float C2 = 1.9073486328125e-06f;  /* 2^-19 */
    const float C3 = 4.76837158203125e-07f; /* 2^-21 */
    const float TINY = 1e-30f;
    unsigned bad = 0;
    const float tf = tf_hi == 0u ? 0.0f : f32_hi(tf_hi, bad);   /* tfalse is often exactly 0 */
    const float atf = fabsf(tf);
    float r[3], dv[3], Er[3], Edv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float xi = f32_hi(h[2 * k], bad), xj = f32_hi(h[2 * k + 1], bad);
        const float vi = f32_hi(h[6 + 2 * k], bad), vj = f32_hi(h[6 + 2 * k + 1], bad);
        const float d = vi - vj;
        const float av = fabsf(vi) + fabsf(vj);
        const float x = (xi - xj) + d * tf;
        const float xr = x - rintf(x);
        r[k] = xr;
        dv[k] = d;
        Er[k] = C1 * (fabsf(xi) + fabsf(xj) + av * atf + fabsf(x));
        Edv[k] = C2 * av;
        bad |= !(fabsf(xr) <= 0.45f);   /* near half a box, or NaN */
    }
    const float Rf = f32_hi(Rh, bad), ER = C2 * Rf;
    if (bad) return false;
    float bf = 0.f, r2 = 0.f, v2 = 0.f, Eb = TINY, Er2 = TINY, Ev2 = TINY, sb = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float ar = fabsf(r[k]), ad = fabsf(dv[k]);
        bf = bf + r[k] * dv[k];
        r2 = r2 + r[k] * r[k];
        v2 = v2 + dv[k] * dv[k];
        sb = sb + ar * ad;
        Eb = Eb + Er[k] * (ad + Edv[k]) + (ar + Er[k]) * Edv[k];
        Er2 = Er2 + (2.f * ar + Er[k]) * Er[k];
        Ev2 = Ev2 + (2.f * ad + Edv[k]) * Edv[k];
    }
    Eb = Eb + C3 * sb;
    Er2 = Er2 + C3 * r2;
    Ev2 = Ev2 + C3 * v2;
    if (need_out && !(r2 - Er2 > Rf + ER)) return false;
    if (bf > Eb) return true;
    const float c = r2 - Rf;
    const float Ec = Er2 + ER + C3 * fabsf(c);
    const float D = bf * bf - v2 * c;
    const float ED = (2.f * fabsf(bf) + Eb) * Eb + Ev2 * fabsf(c) + (v2 + Ev2) * Ec +
                     C3 * (bf * bf + fabsf(v2 * c)) + TINY;
    return D + ED < 0.f;
}

#define PK_NONE 0
#define PK_MINUS 1
#define PK_PLUS 2
#define PK_BOND 3   /* -(rijsq - R) / (sqrt(D) + bij) */
#define PK_STAGE2 4

__device__ __forceinline__ bool d_predict_c(const DSys &S, int i, int j, int evcode, double tfalse,
                                            double &tij, int &type, const double *si = nullptr,
                                            const double *sj = nullptr) {
    const DTab &T = *S.tab;
    Rel r = d_rel_cv(S, i, j, tfalse, si, sj);
    int a = DMD_CHK(S.ident[DMD_CHK(i, S.N, 2)], DMD_NT, 4), b = DMD_CHK(S.ident[DMD_CHK(j, S.N, 3)], DMD_NT, 4);
    evcode = DMD_CHK(evcode, DMD_NC, 5);
    bool neg = d_lt0(r.bij);
    bool valid = true;
    /* stage 1: diameter R1; outcome if D1 > 0 (k1p, y1p) or not (k1n, y1n);
     * stage 2 (k1n == PK_STAGE2): diameter R2, outcome (k2p, y2p) / (k2n, y2n) */
    double R1 = 0.0, R2 = 0.0;
    int k1p = PK_NONE, y1p = 0, k1n = PK_NONE, y1n = 0, k2p = PK_NONE, y2p = 0, k2n = PK_NONE, y2n = 0;
    if (evcode <= 3 || (evcode >= 17 && evcode <= 26)) {                 /* core.f:3-44 */
        if (neg) { R1 = T.core_sq[core_slot_d(evcode)][a][b]; k1p = PK_MINUS; y1p = 1; }
    } else if (evcode >= 4 && evcode <= 12) {                           /* bond.f:4-121 */
        bool side = evcode >= 10;
        double lo = side ? S.blmin_sq[i] : T.evp2_sq[evcode];
        double hi = side ? S.blmax_sq[i] : T.evp3_sq[evcode];
        if (neg) {
            R1 = lo; k1p = PK_MINUS; y1p = 2; k1n = PK_STAGE2;
            R2 = hi; k2p = PK_PLUS; y2p = 3;
        } else {
            R1 = hi; k1p = PK_BOND; y1p = 3;
        }
    } else if (evcode == 15 || evcode == 16 || evcode >= 40) {
        /* nc_sqwel.f:7-126, sqwel.f:5-67, sqshlder.f:5-66 */
        double well = evcode >= 40 ? T.shlddia_sq[a][b] : T.welldia_sq[a][b];
        bool inside = d_lt_nn(r.rijsq, well);          /* diff < 0 */
        int y_in, y_out;                                /* exit / entry types */
        bool two_stage = true;                          /* core inside the well */
        double core = T.sigma_sq[a][b];
        if (evcode == 16) { y_in = 8; y_out = 4; }
        else if (evcode >= 40) { y_in = 10; y_out = 12; }
        else if (a + b == 5) { y_in = 16; y_out = 7; }
        else if (S.bptnr[i] == j) {
            /* bonded H-bond pair: always inside, core with the 1.05 factor */
            y_in = 8; y_out = 8; inside = true; core = T.ncfac_sq[a][b];
        } else { y_in = 0; y_out = 9; two_stage = false; inside = false; }
        if (neg) {
            if (inside && two_stage) {
                R1 = core; k1p = PK_MINUS; y1p = 1; k1n = PK_STAGE2;
                R2 = well; k2p = PK_PLUS; y2p = y_in; k2n = PK_PLUS; y2n = y_in;
            } else {
                R1 = well; k1p = PK_MINUS; y1p = y_out;
            }
        } else if (inside) {
            R1 = well; k1p = PK_PLUS; y1p = y_in; k1n = PK_PLUS; y1n = y_in;
        }
    } else {
        valid = false;
    }
    double b2 = r.bij * r.bij;
    double c = r.rijsq - R1;
    double D = b2 - r.vijsq * c;
    int k, y;
    if (d_gt0(D)) { k = k1p; y = y1p; } else { k = k1n; y = y1n; }
    if (k == PK_STAGE2) {
        c = r.rijsq - R2;
        D = b2 - r.vijsq * c;
        if (d_gt0(D)) { k = k2p; y = y2p; } else { k = k2n; y = y2n; }
    }
    tij = DMD_BIG; type = 0;
    if (k != PK_NONE) {
        double sq = sqrt(D);
        bool bond = k == PK_BOND;
        double X = bond ? sq : d_negate(r.bij);
        double Y = bond ? r.bij : (k == PK_MINUS ? d_negate(sq) : sq);
        double s1 = X + Y;
        double num = bond ? d_negate(c) : s1;
        double den = bond ? s1 : r.vijsq;
        tij = num / den;
        type = y;
        /* A bonded H-bond pair that rounding left just outside its well
         * takes the square root of a negative discriminant (the reference's
         * nc_sqwel.f:69-93 does not test it): a NaN time, which no
         * comparison of the reference ever selects and its negative-time
         * check never flags.  Its integer key would depend on the NaN's sign
         * bit, so it becomes "no event", which is selected just as rarely. */
        if ((dbits(tij) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) { tij = DMD_BIG; type = 0; }
    }
    return valid;
}

#endif /* DMD_ENGINE_CUH */
