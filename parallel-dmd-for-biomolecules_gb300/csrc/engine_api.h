/*
 * engine_api.h -- launch entry points of engine.cu used by the host code
 * in capi.cu (internal to the library).
 */
#ifndef DMD_ENGINE_API_H
#define DMD_ENGINE_API_H
#include <cuda_runtime.h>
#include "dmd.h"
#include "engine.cuh"

cudaError_t dmd_launch_init(DSys *d_systems, int nsys, int hbonds, cudaStream_t st);
/* The compact variant of the event loop takes systems whose down lists
 * hold at most DMD_COMPACT_DN beads (DScal::max_dn); a system whose lists
 * outgrow it stops with DScal::need_full set and continues on the full
 * variant, which takes any list.  compact: 0 = the full variant, k > 0 =
 * the compact one with the down-list limit min(k, DMD_COMPACT_DN). */
#define DMD_COMPACT_DN 32
/* targets: per-system event counts (device array), or NULL for target.
 * cycles != 0: each system also stops after its next list rebuild and
 * writes the events it still has to run back into targets[r].
 * min_beads: the smallest system of the launch (0: unknown); when it is
 * small enough, a compact one-CTA launch gets shared memory for the hot
 * per-bead arrays of the systems that fit. */
cudaError_t dmd_launch_run(DSys *d_systems, int nsys, int max_beads, int C, int compact, long long target,
                           long long *targets, int hbonds, const int *chain_start, const int *chain_len,
                           const int *chain_off, dmd_diag *outputs, cudaStream_t st, int cycles = 0,
                           int min_beads = 0);
cudaError_t dmd_max_active_clusters(int C, int *n);
/* backbone (phi, psi) bins of every system (only < 0) or system only, added
 * to its 361 x 361 histogram at hist + r * 361 * 361 (code/phipsi.f) */
cudaError_t dmd_launch_phipsi(DSys *d_systems, int nsys, int only, const int *chain_start, const int *chain_len,
                              const int *chain_off, unsigned long long *hist, cudaStream_t st);
cudaError_t dmd_launch_diag(DSys *d_systems, int nsys, const int *chain_start, const int *chain_len,
                            const int *chain_off, dmd_diag *out, cudaStream_t st);

/* allocation-free prediction pass (engine.cu): the scratch array's size and
 * limits, its per-device address, and the launch */
#define DMD_NOALLOC_SCRATCH_BYTES (8u << 20)
#define DMD_NOALLOC_MAX_BEADS 8192
#define DMD_NOALLOC_MAX_CAP 64
#define DMD_NOALLOC_MAX_CELLS 48
cudaError_t dmd_noalloc_scratch(void **ptr);
cudaError_t dmd_launch_predict_noalloc(const DSys &S, int hbonds, double *tim_out, int *nptnr_out, int *colt_out,
                                       cudaStream_t st);
#endif
