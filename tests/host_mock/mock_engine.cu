/*
 * mock_engine.cu -- TEST INFRASTRUCTURE ONLY: stand-ins for the kernel
 * launches of engine.cu (engine_api.h), for checking the host code of
 * capi.cu on a machine without a GPU (with mock_rt.cpp).  A launch runs no
 * kernel; it checks what the kernel would be given: every array of every
 * system's DSys lies inside one device allocation, with the extent the
 * kernels index (N, N + 3, N x cap, cells^3 + 1, tournament levels),
 * without overlapping another array or another system's pool; the chain
 * tables start each system at bead 0 and increase; an event log fits its
 * ring.  The failures are collected as text (mock_report).
 */
#include <algorithm>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "engine_api.h"

bool mock_alloc_of(const void *p, const char **base, size_t *n);
bool mock_capture_push(std::function<void()> f);

namespace {
std::string g_report;
int g_init = 0, g_run = 0, g_diag = 0;
long long g_last_target = -2;
int g_last_C = 0, g_last_compact = -1;
int g_handoff = -1;                  /* system that outgrows the compact variant at its next compact launch */
int g_outgrown = -1;                 /* the system that has outgrown it */
std::vector<long long> g_last_targets;

struct Span { const char *name; const void *p; size_t n; };

void fail(const char *what, int r, const std::string &msg) {
    if (g_report.size() < 4000) g_report += std::string(what) + " system " + std::to_string(r) + ": " + msg + "\n";
}

void check(const char *what, const DSys *d, int nsys, const int *cs, const int *cl, const int *co) {
    std::vector<std::pair<const char *, const char *>> pools;
    for (int r = 0; r < nsys; ++r) {
        const DSys &S = d[r];
        const size_t N = (size_t)S.N, NE = N + 3, cap = (size_t)S.cap, nc3 = (size_t)S.ncell * S.ncell * S.ncell;
        if (S.N <= 0 || S.cap <= 0 || S.nchains <= 0) { fail(what, r, "bad sizes"); continue; }
        if (S.nl1 != (S.N + 3 + 31) / 32 || S.nl2 != (S.nl1 + 31) / 32) fail(what, r, "tournament sizes");
        std::vector<Span> sp = {
            {"tab", S.tab, sizeof(DTab)}, {"sc", S.sc, sizeof(DScal)}, {"info", S.info, N * sizeof(BeadInfo)},
            {"bm", S.bm, N * 8}, {"blmin", S.blmin, N * 8}, {"blmax", S.blmax, N * 8},
            {"blmin_sq", S.blmin_sq, N * 8}, {"blmax_sq", S.blmax_sq, N * 8}, {"rblmin_sq", S.rblmin_sq, N * 8},
            {"rblmax_sq", S.rblmax_sq, N * 8}, {"x", S.x, N * 8}, {"y", S.y, N * 8}, {"z", S.z, N * 8},
            {"vx", S.vx, N * 8}, {"vy", S.vy, N * 8}, {"vz", S.vz, N * 8}, {"ox", S.ox, N * 8}, {"oy", S.oy, N * 8},
            {"oz", S.oz, N * 8}, {"xf", S.xf, N * 4}, {"yf", S.yf, N * 4}, {"zf", S.zf, N * 4},
            {"ident", S.ident, N}, {"bptnr", S.bptnr, N * 4}, {"er", S.er, 16 * N}, {"ovp", S.ovp, 16 * N},
            {"ovc", S.ovc, 4 * N}, {"tim", S.tim, NE * 8}, {"nptnr", S.nptnr, NE * 4}, {"colt", S.colt, NE},
            {"queued", S.queued, NE}, {"key", S.key, NE * 8}, {"up", S.up, N * cap * 4}, {"dn", S.dn, N * cap * 4},
            {"upc", S.upc, N * cap}, {"upn", S.upn, N * 4}, {"dnn", S.dnn, N * 4},
            {"cell_count", S.cell_count, (nc3 + 1) * 4}, {"cell_start", S.cell_start, (nc3 + 1) * 4},
            {"cell_beads", S.cell_beads, N * 4}, {"l1i", S.l1i, (size_t)S.nl1 * 4}, {"l2i", S.l2i, (size_t)S.nl2 * 4},
            {"l1k", S.l1k, (size_t)S.nl1 * 8}, {"l2k", S.l2k, (size_t)S.nl2 * 8}};
        if (S.dnc) sp.push_back({"dnc", S.dnc, N * cap});
        if (S.owner) sp.push_back({"owner", S.owner, 3 * N * 4});
        const char *pool = nullptr;
        size_t pool_n = 0;
        for (const Span &s : sp) {
            const char *base = nullptr;
            size_t n = 0;
            if (!s.p || !mock_alloc_of(s.p, &base, &n)) { fail(what, r, std::string(s.name) + " outside any allocation"); continue; }
            if (!pool) { pool = base; pool_n = n; }
            if (base != pool) fail(what, r, std::string(s.name) + " in another allocation than the pool");
            if ((const char *)s.p + s.n > base + n) fail(what, r, std::string(s.name) + " runs past its allocation");
        }
        std::sort(sp.begin(), sp.end(), [](const Span &a, const Span &b) { return a.p < b.p; });
        for (size_t q = 1; q < sp.size(); ++q)
            if ((const char *)sp[q - 1].p + sp[q - 1].n > (const char *)sp[q].p)
                fail(what, r, std::string(sp[q - 1].name) + " overlaps " + sp[q].name);
        if (!sp.empty()) pools.push_back({(const char *)sp.front().p, (const char *)sp.back().p + sp.back().n});
        (void)pool_n;
        if (S.log) {
            const char *base = nullptr;
            size_t n = 0;
            if (!mock_alloc_of(S.log, &base, &n) || (const char *)S.log + S.log_cap * sizeof(dmd_event) > base + n)
                fail(what, r, "event log ring outside its allocation");
        }
        if (cs) {
            const int *c0 = cs + co[r], *l0 = cl + co[r];
            if (c0[0] != 0) fail(what, r, "first chain does not start at bead 0");
            for (int c = 0; c < S.nchains; ++c) {
                if (l0[c] < 3 || c0[c] < 0 || c0[c] >= S.N) fail(what, r, "chain table entry out of range");
                if (c > 0 && c0[c] <= c0[c - 1] + 3 * l0[c - 1] - 1) fail(what, r, "chain starts do not increase");
            }
            if (r + 1 < nsys && co[r + 1] != co[r] + S.nchains) fail(what, r, "chain offsets");
        }
    }
    std::sort(pools.begin(), pools.end());
    for (size_t q = 1; q < pools.size(); ++q)
        if (pools[q - 1].second > pools[q].first) fail(what, (int)q, "pool overlaps the previous system's");
}
}  // namespace

extern "C" {
const char *mock_report(void) { return g_report.c_str(); }
void mock_reset(void) { g_report.clear(); g_init = g_run = g_diag = 0; g_handoff = -1; g_outgrown = -1; g_last_targets.clear(); }
void mock_set_handoff(int system) { g_handoff = system; }
long long mock_last_target_of(int system) {
    return system >= 0 && system < (int)g_last_targets.size() ? g_last_targets[system] : -2;
}
void mock_counts(int *init, int *run, int *diag, long long *target, int *C, int *compact) {
    *init = g_init; *run = g_run; *diag = g_diag; *target = g_last_target; *C = g_last_C; *compact = g_last_compact;
}
}

cudaError_t dmd_launch_init(DSys *d, int nsys, int, cudaStream_t) {
    ++g_init;
    check("init", d, nsys, nullptr, nullptr, nullptr);
    return cudaSuccess;
}
/* the run launch also stands in for the kernel's bookkeeping: every system
 * counts its target (the per-system one when given) as done, 1,000 cycles
 * per event, and its collision count advances by as much; positions do not
 * move.  The system set by mock_set_handoff stops halfway at its next compact
 * launch with need_full set, as a system whose lists outgrew the compact
 * variant at a rebuild does, and leaves every later compact launch at once
 * with need_full set again.  A rebuild-cycle launch (cycles != 0) runs
 * system r for at most 1000 + 500 r events (its mock rebuild interval) and
 * writes the rest of its target back.  A launch made during a capture is
 * recorded and runs when the graph is launched. */
cudaError_t dmd_launch_run(DSys *d, int nsys, int mb, int C, int compact, long long target, long long *targets,
                           int hb, const int *cs, const int *cl, const int *co, dmd_diag *out, cudaStream_t st,
                           int cycles, int min_beads) {
    if (mock_capture_push([=]() { dmd_launch_run(d, nsys, mb, C, compact, target, targets, hb, cs, cl, co, out, st, cycles, min_beads); }))
        return cudaSuccess;
    ++g_run;
    g_last_target = target; g_last_C = C; g_last_compact = compact;
    check("run", d, nsys, cs, cl, co);
    g_last_targets.assign(nsys, 0);
    for (int r = 0; r < nsys; ++r) {
        DScal &sc = *d[r].sc;
        long long t = targets ? targets[r] : target;
        const long long want = t;
        g_last_targets[r] = t;
        sc.need_full = 0;
        if (cycles) t = std::min(t, 1000LL + 500LL * r);
        if (compact > 0 && r == g_handoff) {
            t = t / 2;
            sc.need_full = 1;
            g_handoff = -1;
            g_outgrown = r;
            sc.max_dn = DMD_COMPACT_DN + 1;
        } else if (compact > 0 && r == g_outgrown) {   /* its lists stay too long: it leaves at once */
            t = 0;
            sc.need_full = 1;
        }
        if (cycles && targets) targets[r] = want - t;
        sc.done = t;
        sc.done_all += t;
        sc.coll += t;
        sc.run_cycles = 1000 * t;
        sc.stop = 0;
    }
    return cudaSuccess;
}
cudaError_t dmd_max_active_clusters(int, int *n) { *n = 1000; return cudaSuccess; }
cudaError_t dmd_launch_diag(DSys *d, int nsys, const int *cs, const int *cl, const int *co, dmd_diag *, cudaStream_t) {
    ++g_diag;
    check("diag", d, nsys, cs, cl, co);
    return cudaSuccess;
}
cudaError_t dmd_launch_phipsi(DSys *d, int nsys, int, const int *cs, const int *cl, const int *co,
                              unsigned long long *, cudaStream_t) {
    check("phipsi", d, nsys, cs, cl, co);
    return cudaSuccess;
}
cudaError_t dmd_noalloc_scratch(void **) { return cudaErrorNotSupported; }
cudaError_t dmd_launch_predict_noalloc(const DSys &, int, double *, int *, int *, cudaStream_t) {
    return cudaErrorNotSupported;
}

/* the layout check flags a pool whose arrays overlap (its own test) */
extern "C" int mock_selftest(void) {
    const std::string saved = g_report;
    g_report.clear();
    const int N = 40, cap = 8;
    char *pool = nullptr;
    cudaMalloc((void **)&pool, 1 << 20);
    DSys S{};
    S.N = N; S.nchains = 1; S.cap = cap; S.ncell = 3; S.nl1 = (N + 3 + 31) / 32; S.nl2 = 1;
    char *p = pool;
    auto take = [&](size_t n) { char *q = p; p += (n + 255) & ~(size_t)255; return q; };
    S.tab = (const DTab *)take(sizeof(DTab)); S.sc = (DScal *)take(sizeof(DScal));
    S.info = (const BeadInfo *)take(N * sizeof(BeadInfo));
    double **dbl[] = {&S.x, &S.y, &S.z, &S.vx, &S.vy, &S.vz, &S.ox, &S.oy, &S.oz, &S.tim};
    for (double **q : dbl) *q = (double *)take((N + 3) * 8);
    S.bm = S.blmin = S.blmax = S.blmin_sq = S.blmax_sq = S.rblmin_sq = S.rblmax_sq = (const double *)take(N * 8);
    S.y = S.x + 1;   /* the planted overlap */
    S.xf = S.yf = S.zf = (float *)take(N * 4);
    S.ident = (int8_t *)take(N); S.bptnr = (int *)take(N * 4); S.er = (int *)take(16 * N); S.ovp = (int *)take(16 * N);
    S.ovc = (int8_t *)take(4 * N); S.nptnr = (int *)take((N + 3) * 4); S.colt = (int8_t *)take(N + 3);
    S.queued = (uint8_t *)take(N + 3); S.key = (long long *)take((N + 3) * 8); S.up = (int *)take(N * cap * 4);
    S.dn = (int *)take(N * cap * 4); S.upc = (int8_t *)take(N * cap); S.upn = (int *)take(N * 4);
    S.dnn = (int *)take(N * 4); S.cell_count = (int *)take(28 * 4); S.cell_start = (int *)take(28 * 4);
    S.cell_beads = (int *)take(N * 4); S.l1i = (int *)take(8); S.l2i = (int *)take(4); S.l1k = (long long *)take(16);
    S.l2k = (long long *)take(8);
    check("selftest", &S, 1, nullptr, nullptr, nullptr);
    const bool flagged = g_report.find("overlaps") != std::string::npos;
    cudaFree(pool);
    g_report = saved;
    return flagged ? 1 : 0;
}
