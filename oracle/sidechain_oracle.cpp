/*
 * sidechain_oracle.cpp -- TEST INFRASTRUCTURE ONLY: CPU restatement of the
 * side-chain placement search of the reference's initial-configuration
 * generator (genconfig/gen_config_random-SQZ.f90:250-348), the oracle of
 * dmd_sidechain_search.
 *
 * For every residue k the side-chain bead is moved over a cubic grid of
 * offsets (d1, d2, d3), each running from -move to +move in steps of
 * `step` as a Fortran DO loop over a real variable does (trip count
 * INT((move - (-move) + step) / step), the variable advanced by repeated
 * addition: :252, :260, :268).  A grid point is admissible when no
 * squeezed-core distance to the neighbouring residues' backbone beads is
 * below its sqz6to10.data value (:294-306: CO(k-1) and CA(k-1) for k >= 2,
 * NH(k+1) and CA(k+1) for k < n); among the admissible points the first in
 * loop order (d1 outermost) with the smallest
 * r3 = |bdln - r(CA)| + |bl_rn - r(NH)| + |bl_rc - r(CO)| below 100 wins
 * (:291, :307-312), and the bead moves by its offset (:317-319).  Every
 * expression keeps the reference's operation order: the offset is added to
 * the bead's coordinate before the reference bead's is subtracted, squares
 * are summed x, y, z from the left, and r3 is summed CA, NH, CO from the
 * left.
 */
#include <cmath>
#include <cstdint>
#include <vector>

#include "dmd.h"

extern "C" {

/* the grid of one axis: DO-loop trip count and values */
int64_t ora_sidechain_grid(double move, double step, double *values, int64_t cap) {
    if (!(step > 0) || !(move >= 0)) return -1;
    const double trip = (move - (-move) + step) / step;
    const int64_t m = trip > 0 ? (int64_t)trip : 0;
    double d = -move;
    for (int64_t i = 0; i < m; ++i) {
        if (values && i < cap) values[i] = d;
        d = d + step;
    }
    return m;
}

/* positions [n][3] in angstrom; residue identities 9..28; residues r0 <=
 * k < r1 are searched, the others copied.  side_out gets the moved side
 * chains, rmin_out the smallest r3 (100 and no move when no
 * grid point is admissible), index_out (may be NULL) the winning point
 * (i1 * m + i2) * m + i3, or -1.  Returns the grid size m per axis, or -1
 * on bad input. */
int64_t ora_sidechain_search(int32_t n, const double *ca, const double *nh, const double *co, const double *side,
                             const int32_t *residue, const dmd_tables *T, double move, double step, int32_t r0,
                             int32_t r1, double *side_out, double *rmin_out, int64_t *index_out) {
    const int64_t m = ora_sidechain_grid(move, step, nullptr, 0);
    if (m < 0 || n <= 0 || r0 < 0 || r1 > n || r0 > r1) return -1;
    std::vector<double> D((size_t)m);
    ora_sidechain_grid(move, step, D.data(), m);
    for (int k = 0; k < n; ++k)
        if (residue[k] < 9 || residue[k] > 28) return -1;
    for (int k = 0; k < n; ++k) {
        if (k < r0 || k >= r1) {
            for (int a = 0; a < 3; ++a) side_out[3 * k + a] = side[3 * k + a];
            rmin_out[k] = 100.0;
            if (index_out) index_out[k] = -1;
            continue;
        }
        const int id = residue[k];
        const int row = id - 9;
        const double bdln = T->rca[row], bl_rn = T->rnh[row], bl_rc = T->rco[row];
        const double s8 = T->sqz[row][0], s6 = T->sqz[row][1], s7 = T->sqz[row][2], s9 = T->sqz[row][3];
        const double *S = side + 3 * k;
        const bool prev = k >= 1, next = k + 1 < n;
        double rmin = 100.0;
        int64_t best = -1;
        for (int64_t i1 = 0; i1 < m; ++i1) {
            const double d1 = D[i1];
            const double rcax = S[0] + d1 - ca[3 * k], rnhx = S[0] + d1 - nh[3 * k], rcox = S[0] + d1 - co[3 * k];
            const double sz6x = prev ? S[0] + d1 - co[3 * (k - 1)] : 0.0, sz8x = prev ? S[0] + d1 - ca[3 * (k - 1)] : 0.0;
            const double sz7x = next ? S[0] + d1 - nh[3 * (k + 1)] : 0.0, sz9x = next ? S[0] + d1 - ca[3 * (k + 1)] : 0.0;
            for (int64_t i2 = 0; i2 < m; ++i2) {
                const double d2 = D[i2];
                const double rcay = S[1] + d2 - ca[3 * k + 1], rnhy = S[1] + d2 - nh[3 * k + 1], rcoy = S[1] + d2 - co[3 * k + 1];
                const double sz6y = prev ? S[1] + d2 - co[3 * (k - 1) + 1] : 0.0;
                const double sz8y = prev ? S[1] + d2 - ca[3 * (k - 1) + 1] : 0.0;
                const double sz7y = next ? S[1] + d2 - nh[3 * (k + 1) + 1] : 0.0;
                const double sz9y = next ? S[1] + d2 - ca[3 * (k + 1) + 1] : 0.0;
                for (int64_t i3 = 0; i3 < m; ++i3) {
                    const double d3 = D[i3];
                    const double rcaz = S[2] + d3 - ca[3 * k + 2], rnhz = S[2] + d3 - nh[3 * k + 2];
                    const double rcoz = S[2] + d3 - co[3 * k + 2];
                    const double rca = std::sqrt(rcax * rcax + rcay * rcay + rcaz * rcaz);
                    const double rnh = std::sqrt(rnhx * rnhx + rnhy * rnhy + rnhz * rnhz);
                    const double rco = std::sqrt(rcox * rcox + rcoy * rcoy + rcoz * rcoz);
                    const double r3 = std::fabs(bdln - rca) + std::fabs(bl_rn - rnh) + std::fabs(bl_rc - rco);
                    bool isz = false;
                    if (prev) {
                        const double sz6z = S[2] + d3 - co[3 * (k - 1) + 2], sz8z = S[2] + d3 - ca[3 * (k - 1) + 2];
                        const double sz6 = std::sqrt(sz6x * sz6x + sz6y * sz6y + sz6z * sz6z);
                        const double sz8 = std::sqrt(sz8x * sz8x + sz8y * sz8y + sz8z * sz8z);
                        if (sz6 < s6) isz = true;
                        if (sz8 < s8) isz = true;
                    }
                    if (next) {
                        const double sz7z = S[2] + d3 - nh[3 * (k + 1) + 2], sz9z = S[2] + d3 - ca[3 * (k + 1) + 2];
                        const double sz7 = std::sqrt(sz7x * sz7x + sz7y * sz7y + sz7z * sz7z);
                        const double sz9 = std::sqrt(sz9x * sz9x + sz9y * sz9y + sz9z * sz9z);
                        if (sz7 < s7) isz = true;
                        if (sz9 < s9) isz = true;
                    }
                    if (r3 < rmin && !isz) {
                        rmin = r3;
                        best = (i1 * m + i2) * m + i3;
                    }
                }
            }
        }
        double d[3] = {0.0, 0.0, 0.0};
        if (best >= 0) { d[0] = D[best / (m * m)]; d[1] = D[(best / m) % m]; d[2] = D[best % m]; }
        for (int a = 0; a < 3; ++a) side_out[3 * k + a] = S[a] + d[a];
        rmin_out[k] = rmin;
        if (index_out) index_out[k] = best;
    }
    return m;
}

}  // extern "C"
