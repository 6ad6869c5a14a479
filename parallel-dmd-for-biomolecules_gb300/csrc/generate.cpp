/*
 * generate.cpp -- seeded synthetic PRIME20 systems.
 *
 * Restates the insertion and velocity steps of the reference's initial
 * configuration generator (genconfig/gen_config_random-SQZ.f90:665-694 for
 * random non-overlapping chain insertion by translation, :806-891 for the
 * Maxwell-Boltzmann velocities) on a template chain of this project's own:
 * the reference builds its template from a stored 31-residue backbone and a
 * brute-force side-chain search (:250-348); here the backbone is built from
 * the PRIME20 bond and pseudo-bond lengths (code/def.h:4-10) with the trans
 * peptide (omega = 180) and phi = -95, psi = 125 degrees, and each side chain
 * sits at a per-residue-type offset in the local (N, C-alpha, C) frame.  The
 * offsets were chosen to maximise the smallest relative margin to every
 * intra-chain bond window (1 +- 0.02375) and squeezed / full core diameter;
 * over random sequences every constraint holds with a margin of at least
 * 0.25 %.  Random numbers come from the Philox streams of dmd_rng.h.
 */
#include "dmd.h"
#include "dmd_rng.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

struct V3 { double x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a) { return (1.0 / std::sqrt(dot(a, a))) * a; }

const double DNC = 1.46, DCC = 1.51, DCN = 1.33, DTIE = 2.41, DTIE2 = 2.45;
const double PHI = -95.0, PSI = 125.0, OMEGA = 180.0;
const double DEG = 3.14159265358979323846 / 180.0;

/* side-chain offset of residue identity 10..28 in the frame
 * e1 = unit(N - CA), e2 = unit((C - CA) orthogonalised to e1), e3 = e1 x e2 */
const double R_OFFSET[19][3] = {
    {-0.6109523375, -3.9378231330, -2.4870407350},  /* 10 R */
    {-0.2970603502, -1.0510648929, 2.2583204878},   /* 11 N */
    {-0.7230165795, -2.2142235310, 0.9041097026},   /* 12 D */
    {-0.6528599106, -2.5248463280, 2.1785050179},   /* 13 Q */
    {-0.6985252868, -1.3518077492, 2.7902820682},   /* 14 E */
    {-0.1880537260, -3.0715288004, 0.6749151309},   /* 15 H */
    {-0.5698999324, -1.3472634253, 3.2323958635},   /* 16 K */
    {0.8374254354, -0.5271365657, 1.6926822666},    /* 17 P */
    {-0.3487166120, -0.7336136490, 1.7902330509},   /* 18 S */
    {-0.8456186677, -1.3190227616, 1.2087542389},   /* 19 T */
    {-0.5322737488, -0.8126683414, 1.2701841726},   /* 20 A */
    {-0.2577539312, -2.0563666173, 1.1050752557},   /* 21 C */
    {-0.4818178911, -1.1961615649, 2.0225111686},   /* 22 I */
    {-0.6155626094, -1.3292434677, 2.1764753292},   /* 23 L */
    {-0.2551874956, -1.0065323305, 3.2355423357},   /* 24 M */
    {0.1854520626, -0.7755586956, 3.3288907719},    /* 25 F */
    {-0.4741200839, -3.8458773619, 1.6138587658},   /* 26 W */
    {-0.0909925189, -3.7437708693, 0.8841272679},   /* 27 Y */
    {-0.5331700999, -1.0804396402, 1.5974550300},   /* 28 V */
};

double angle_from_sides(double a, double b, double c) { return std::acos((a * a + b * b - c * c) / (2 * a * b)) / DEG; }

/* place d with |cd| = bond, angle(b,c,d) = ang, torsion(a,b,c,d) = tor */
V3 place(V3 a, V3 b, V3 c, double bond, double ang, double tor) {
    V3 bc = unit(c - b);
    V3 n = unit(cross(b - a, bc));
    V3 m = cross(n, bc);
    double A = ang * DEG, T = tor * DEG;
    return c + (-bond * std::cos(A)) * bc + (bond * std::sin(A) * std::cos(T)) * m + (bond * std::sin(A) * std::sin(T)) * n;
}

/* template chain in engine bead order, angstrom, first bead at the origin */
void build_chain(int L, const int32_t *res, std::vector<V3> &out) {
    double tau = angle_from_sides(DNC, DCC, DTIE2);
    double a2 = angle_from_sides(DCC, DCN, DTIE);
    double a3 = angle_from_sides(DCN, DNC, DTIE2);
    std::vector<V3> N(L), CA(L), C(L);
    N[0] = {0, 0, 0};
    CA[0] = {DNC, 0, 0};
    C[0] = CA[0] + DCC * V3{std::cos((180 - tau) * DEG), std::sin((180 - tau) * DEG), 0};
    for (int k = 1; k < L; ++k) {
        N[k] = place(N[k - 1], CA[k - 1], C[k - 1], DCN, a2, PSI);
        CA[k] = place(CA[k - 1], C[k - 1], N[k], DNC, a3, OMEGA);
        C[k] = place(C[k - 1], N[k], CA[k], DCC, tau, PHI);
    }
    out.clear();
    for (int k = 0; k < L; ++k) out.push_back(CA[k]);
    for (int k = 0; k < L; ++k) out.push_back(N[k]);
    for (int k = 0; k < L; ++k) out.push_back(C[k]);
    for (int k = 0; k < L; ++k) {
        int r = res[k];
        if (r == 9) continue;
        V3 e1 = unit(N[k] - CA[k]);
        V3 v = C[k] - CA[k];
        V3 e2 = unit(v - dot(v, e1) * e1);
        V3 e3 = cross(e1, e2);
        const double *o = R_OFFSET[r - 10];
        out.push_back(CA[k] + o[0] * e1 + o[1] * e2 + o[2] * e3);
    }
    V3 b0 = out[0];
    for (auto &p : out) p = p - b0;
}

inline double wrap(double x, double box) { return x - box * std::nearbyint(x / box); }

}  // namespace

extern "C" int dmd_generate(const dmd_gen_spec *spec, const dmd_tables *tables, int32_t n_beads,
                            double *x, double *y, double *z, double *vx, double *vy, double *vz,
                            char *err, int32_t errlen) {
    auto fail = [&](const char *m) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", m);
        return DMD_E_INPUT;
    };
    if (!spec || !tables || !x || !vx) return fail("null argument");
    const double box = spec->boxl;
    const double sep = spec->min_sep > 0 ? spec->min_sep : 5.0;
    int total = 0, rpos = 0;
    for (int c = 0; c < spec->n_chains; ++c) {
        int L = spec->chain_len[c];
        if (L < 3) return fail("chain shorter than 3 residues");
        int nr = 0;
        for (int k = 0; k < L; ++k) {
            int r = spec->residues[rpos + k];
            if (r < 9 || r > 28) return fail("residue identity out of 9..28");
            nr += r != 9;
        }
        total += 3 * L + nr;
        rpos += L;
    }
    if (total != n_beads) return fail("n_beads does not match the chains");

    /* cell grid of placed beads for the rejection test */
    int nc = (int)(box / sep);
    if (nc < 3) nc = 3;
    double cw = box / nc;
    std::vector<std::vector<int>> grid((size_t)nc * nc * nc);
    auto cell_of = [&](double px, double py, double pz, int &cx, int &cy, int &cz) {
        cx = (int)std::floor((px + 0.5 * box) / cw); cy = (int)std::floor((py + 0.5 * box) / cw); cz = (int)std::floor((pz + 0.5 * box) / cw);
        cx = ((cx % nc) + nc) % nc; cy = ((cy % nc) + nc) % nc; cz = ((cz % nc) + nc) % nc;
    };
    std::vector<double> px(n_beads), py(n_beads), pz(n_beads);
    std::vector<V3> tmpl;
    uint64_t draw = 0;
    const double sep2 = sep * sep * 1.0000000001;
    int pos = 0;
    rpos = 0;
    for (int c = 0; c < spec->n_chains; ++c) {
        int L = spec->chain_len[c];
        build_chain(L, spec->residues + rpos, tmpl);
        int nb = (int)tmpl.size();
        {   /* the extended chain must not meet its own periodic image */
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (const V3 &p : tmpl) {
                double v[3] = {p.x, p.y, p.z};
                for (int d = 0; d < 3; ++d) { lo[d] = v[d] < lo[d] ? v[d] : lo[d]; hi[d] = v[d] > hi[d] ? v[d] : hi[d]; }
            }
            for (int d = 0; d < 3; ++d)
                if (hi[d] - lo[d] > box - sep) return fail("box too small for an extended chain");
        }
        int attempts = 0;
        for (;;) {
            if (++attempts > 200000) return fail("random insertion failed: box too crowded");
            double s0 = dmd_uniform(spec->seed, 10u, draw, 0) * box;
            double s1 = dmd_uniform(spec->seed, 10u, draw, 1) * box;
            double s2 = dmd_uniform(spec->seed, 10u, draw, 2) * box;
            ++draw;
            bool ok = true;
            for (int q = 0; q < nb && ok; ++q) {
                double qx = wrap(s0 + tmpl[q].x, box), qy = wrap(s1 + tmpl[q].y, box), qz = wrap(s2 + tmpl[q].z, box);
                px[pos + q] = qx; py[pos + q] = qy; pz[pos + q] = qz;
                int cx, cy, cz;
                cell_of(qx, qy, qz, cx, cy, cz);
                for (int dx = -1; dx <= 1 && ok; ++dx)
                    for (int dy = -1; dy <= 1 && ok; ++dy)
                        for (int dz = -1; dz <= 1 && ok; ++dz) {
                            int gx = (cx + dx + nc) % nc, gy = (cy + dy + nc) % nc, gz = (cz + dz + nc) % nc;
                            for (int b : grid[((size_t)gz * nc + gy) * nc + gx]) {
                                double rx = wrap(qx - px[b], box), ry = wrap(qy - py[b], box), rz = wrap(qz - pz[b], box);
                                if (rx * rx + ry * ry + rz * rz <= sep2) { ok = false; break; }
                            }
                        }
            }
            if (ok) break;
        }
        for (int q = 0; q < nb; ++q) {
            int cx, cy, cz;
            cell_of(px[pos + q], py[pos + q], pz[pos + q], cx, cy, cz);
            grid[((size_t)cz * nc + cy) * nc + cx].push_back(pos + q);
        }
        pos += nb;
        rpos += L;
    }
    for (int i = 0; i < n_beads; ++i) { x[i] = px[i] / box; y[i] = py[i] / box; z[i] = pz[i] / box; }

    /* velocities (gen_config_random-SQZ.f90:806-891) */
    std::vector<double> bm(n_beads);
    double bmass[29];
    for (int k = 0; k < 29; ++k) bmass[k] = tables->mass[k];
    bmass[3] = bmass[20];
    pos = 0;
    rpos = 0;
    for (int c = 0; c < spec->n_chains; ++c) {
        int L = spec->chain_len[c];
        for (int k = 0; k < L; ++k) bm[pos + k] = bmass[2];
        for (int k = 0; k < L; ++k) bm[pos + L + k] = bmass[1];
        for (int k = 0; k < L; ++k) bm[pos + 2 * L + k] = bmass[4];
        int q = 3 * L;
        for (int k = 0; k < L; ++k) if (spec->residues[rpos + k] != 9) bm[pos + q++] = bmass[spec->residues[rpos + k]];
        pos += q;
        rpos += L;
    }
    const double pi = 4.0 * std::atan(1.0);
    double sumx = 0, sumy = 0, sumz = 0;
    for (int k = 0; k < n_beads; ++k) {
        double x1 = dmd_uniform(spec->seed, 11u, (uint64_t)k, 0) * 0.75 + 0.2;
        double x2 = dmd_uniform(spec->seed, 11u, (uint64_t)k, 1) * 0.75 + 0.2;
        double y1 = dmd_uniform(spec->seed, 11u, (uint64_t)k, 2) * 0.75 + 0.2;
        double y2 = dmd_uniform(spec->seed, 11u, (uint64_t)k, 3) * 0.75 + 0.2;
        vx[k] = std::sqrt(-2.0 * std::log(x1)) * std::cos(2.0 * pi * y1);
        vy[k] = std::sqrt(-2.0 * std::log(x1)) * std::sin(2.0 * pi * y1);
        vz[k] = std::sqrt(-2.0 * std::log(x2)) * std::cos(2.0 * pi * y2);
        sumx += vx[k]; sumy += vy[k]; sumz += vz[k];
    }
    for (int k = 0; k < n_beads; ++k) { vx[k] -= sumx / n_beads; vy[k] -= sumy / n_beads; vz[k] -= sumz / n_beads; }
    double sumvel = 0;
    for (int k = 0; k < n_beads; ++k) sumvel += (vx[k] * vx[k] + vy[k] * vy[k] + vz[k] * vz[k]) / bm[k];
    double setemp = spec->tstar * 12.0;
    double tred = sumvel / 3.0 / n_beads;
    double cst = std::sqrt(setemp / tred);
    for (int k = 0; k < n_beads; ++k) { vx[k] = cst * vx[k] / bm[k]; vy[k] = cst * vy[k] / bm[k]; vz[k] = cst * vz[k] / bm[k]; }
    return DMD_OK;
}
