/*
 * dmd_oracle.h -- TEST INFRASTRUCTURE ONLY: C ABI of the CPU restatement of
 * the reference PRIME20 DMD engine (see dmd_oracle.cpp).  Used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the
 * checker; the GB300 engine never links it.
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
int ora_get_evcode(ora_handle *h, int8_t *out);
int ora_get_lists(ora_handle *h, int32_t *up_count, int32_t *up, int32_t *dn_count, int32_t *dn, int32_t cap);
int ora_get_scalars(ora_handle *h, double *out, int n);
int ora_n_outputs(ora_handle *h);
int ora_get_output(ora_handle *h, int k, dmd_diag *d);
void ora_destroy(ora_handle *h);
/* genconfig's side-chain placement search (sidechain_oracle.cpp) */
int64_t ora_sidechain_grid(double move, double step, double *values, int64_t cap);
int64_t ora_sidechain_search(int32_t n, const double *ca, const double *nh, const double *co, const double *side,
                             const int32_t *residue, const dmd_tables *T, double move, double step, int32_t r0,
                             int32_t r1, double *side_out, double *rmin_out, int64_t *index_out);
#ifdef __cplusplus
}
#endif
#endif
