/*
 * dmd_oracle.h -- TEST INFRASTRUCTURE ONLY: C ABI of the CPU restatement of
 * the reference PRIME20 DMD engine (see dmd_oracle.cpp).  Used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the
 * oracle; the GB300 engine never links it.
 */
#ifndef DMD_ORACLE_H
#define DMD_ORACLE_H
#include "dmd.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct ora_handle ora_handle;
ora_handle *ora_create(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys, char *err, int errlen);
int64_t ora_run(ora_handle *h, int64_t n, dmd_event *log, int64_t cap);
int ora_predict_all(ora_handle *h, double *tim, int32_t *nptnr, int32_t *coltype);
int ora_get_state(ora_handle *h, double *x, double *y, double *z, double *vx, double *vy, double *vz,
                  int32_t *bptnr, int32_t *identity, int32_t *er, double *t, double *tfalse, int64_t *coll);
int ora_diagnostics(ora_handle *h, dmd_diag *d);
/* adds the current state's backbone (phi, psi) bins (code/phipsi.f) to
 * hist[361 * 361] */
int ora_phipsi_sample(ora_handle *h, int64_t *hist);
int ora_get_evcode(ora_handle *h, int8_t *out);
int ora_get_lists(ora_handle *h, int32_t *up_count, int32_t *up, int32_t *dn_count, int32_t *dn, int32_t cap);
int ora_get_scalars(ora_handle *h, double *out, int n);
int ora_n_outputs(ora_handle *h);
int ora_get_output(ora_handle *h, int k, dmd_diag *d);
void ora_destroy(ora_handle *h);
/* dmd_log (dmd_rng.h, the logarithm of the ghost draws) over n inputs */
void ora_log_many(const double *x, double *y, int64_t n);
/* Known-answer hook: beads i and j (0-based; identities ida/idb when > 0,
 * H-bond partners of each other when bonded) placed at st[0..5] = x, y, z,
 * vx, vy, vz of i (positions in box units) and st[6..11] for j at tfalse = 0;
 * returns the pair prediction under evcode (code/eventredo_up.f:28-46:
 * time, type) and, when ct_in > 0, the impulse of code/eventdyn.f for
 * collision type ct_in (final type, state after it); mass[0..1] = bm(i),
 * bm(j).  Overwrites the handle's state of i and j. */
int ora_pair_case(ora_handle *h, int32_t i, int32_t j, int32_t ida, int32_t idb, int32_t evcode, int32_t bonded,
                  const double *st, int32_t ct_in, double *tij, int32_t *type, double *st_out, int32_t *ct_out,
                  double *mass);
/* genconfig's side-chain placement search (sidechain_oracle.cpp) */
int64_t ora_sidechain_grid(double move, double step, double *values, int64_t cap);
int64_t ora_sidechain_search(int32_t n, const double *ca, const double *nh, const double *co, const double *side,
                             const int32_t *residue, const dmd_tables *T, double move, double step, int32_t r0,
                             int32_t r1, double *side_out, double *rmin_out, int64_t *index_out);
#ifdef __cplusplus
}
#endif
#endif
