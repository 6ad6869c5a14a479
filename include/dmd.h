/*
 * dmd.h -- C ABI of the GB300 PRIME20 discontinuous-MD event engine.
 *
 * The engine replaces the event engine of the reference Fortran program
 * (parallel-dmd-PRIME20/code): the subroutines events(), partial_events(),
 * eventredo_up/down(), core(), bond(), sqwel(), nc_sqwel(), sqshlder(),
 * eventdyn(), bumpoff(), repuls_*(), check_sigma(), nbor_setup(),
 * cell_link(), cell_add(), nbor(), displ(), add_tbin()/del_tbin() and the
 * master loop of program dmd (code/main.F90:484-1258) with the worker block
 * (code/main.F90:1420-1960) folded in.  Those subroutines share the module
 * GLOBAL (code/header.f:2-65) and have no API of their own; the functions
 * below are the calls a host (a Fortran program through ISO_C_BINDING, C++,
 * or Python ctypes) makes instead of running that loop.
 *
 * Conventions
 *   - Plain C types only.  All floating point is IEEE double.
 *   - Bead indices crossing the ABI are 1-based, as in the reference
 *     (0 means "none").  Bead order inside every chain is
 *     C-alpha(1..L), NH(1..L), CO(1..L), side chains R of the non-glycine
 *     residues in sequence order (code/inputinfo.f:218-228).
 *   - Every function returns 0 on success or a negative DMD_E_* status and
 *     never calls exit(); dmd_last_error() gives the text.
 *   - The library copies host inputs; the caller keeps ownership.
 *   - A handle is single threaded.  Different handles may be used from
 *     different threads.
 */
#ifndef DMD_H
#define DMD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DMD_OK                 0
#define DMD_E_INPUT          (-1)  /* malformed or inconsistent input */
#define DMD_E_OVERLAP        (-2)  /* overlapping / broken-bond initial state */
#define DMD_E_NEG_TIME       (-3)  /* negative predicted time beyond 1e-10 (reference debug check) */
#define DMD_E_DEVICE_TIMEOUT (-4)  /* a bounded device wait gave up */
#define DMD_E_OOM            (-5)  /* device or host memory exhausted / does not fit */
#define DMD_E_CUDA           (-6)  /* a CUDA runtime call failed */
#define DMD_E_CAPACITY       (-7)  /* a fixed-capacity structure (neighbour list, override table) overflowed */
#define DMD_E_STATE          (-8)  /* call not valid in the handle's current state */

/* Raw PRIME20 parameter tables in angstrom, exactly as the reference reads
 * them from parameters/ and parametersep/ (code/inputinfo.f:152-420).
 * Residue identities 9..28 map to row/column index 0..19 (order g r n d q e
 * h k p s t a c i l m f w y v).  The engine scales by the box inside
 * (code/scale_down.f:1-87). */
typedef struct dmd_tables {
    double sigma[4];      /* protein.data lines 1-4: NH, CA, generic side chain, CO bead diameters */
    double welldia[4];    /* protein.data lines 5-8 */
    double epsilon[4];    /* protein.data lines 9-12 (epsilon[0] is the H-bond depth) */
    double mass[29];      /* mass.data, indexed by identity 1..28 ([0], [3] unused: mass(3)=mass(20)) */
    double bds[20][20];   /* beadwell_*.data column 5: side-chain pair diameters */
    double wel[20][20];   /* beadwell_*.data column 6: side-chain pair well diameters */
    double ep[20][20];    /* parametersep table raw value; the well depth is -value */
    double rca[20], rnh[20], rco[20];              /* rcarnrco.data columns 1-3 */
    double del_rca[20], del_rnh[20], del_rco[20];  /* rcarnrco.data columns 4-6 (raised to del) */
    double sqz[20][5];    /* sqz6to10.data in file column order: sz8, sz6, sz7, sz9, sz10 */
} dmd_tables;

/* Run settings: the temp_* file (T*, ncoll), the hard-coded constants of
 * code/main.F90:144-174 and code/def.h, and the -D flags of qfile/script.sh. */
typedef struct dmd_run_cfg {
    double   tstar;       /* reduced temperature; setemp = 12 T* (code/main.F90:126-127) */
    uint64_t seed;        /* key of the counter-based random streams */
    int32_t  canon;       /* 1: Andersen ghost collisions (-Dcanon) */
    int32_t  hbonds;      /* 1: backbone H-bonds on (0 = -Dno_hbs) */
    int32_t  numbin;      /* calendar bins (reference: 2000); kept for reporting */
    int32_t  n_wrap;      /* cells per neighbour-list radius (reference: 2) */
    double   rl_const;    /* neighbour-list radius / largest interaction (1.2) */
    double   t_fact;      /* interval = t_fact / sqrt(setemp) (5e-5) */
    double   n_forced;    /* list horizon in intervals (150) */
    int32_t  list_cap;    /* per-bead capacity of each neighbour list (0: default 128) */
    int32_t  flags;       /* DMD_FLAG_* */
    /* -Dchaptype (code/make_code.f:489-548): 1 (or 0) one peptide type; 2
     * two, chains species2_chain.. being species 2, and the side chains of
     * two different species-2 chains then meet as hard cores (type 1)
     * instead of in the hydrophobic well (type 16) */
    int32_t  chaptype;
    int32_t  species2_chain;
} dmd_run_cfg;

#define DMD_FLAG_STOP_AT_OUTPUT 1  /* dmd_run returns after every output (N+3) event */
#define DMD_FLAG_COUNT_PHYSICAL 2  /* dmd_run counts pair + ghost events only (else the reference's coll) */
#define DMD_FLAG_SERIAL         4  /* one event per step (no conflict-free batching) */
/* The overlap check of code/checkover.f:18-131 (a non-bonded pair inside
 * its core, a bonded pair outside its window) runs on every initial state
 * (dmd_create, dmd_set_state, batch and server creation) and fails it with
 * DMD_E_OVERLAP naming the pair; the reference only reports it at start-up
 * (code/main.F90:347-354).  ALLOW_OVERLAP skips that check. */
#define DMD_FLAG_ALLOW_OVERLAP  8
/* The -Ddebugging checks at every output event (code/main.F90:1193-1205):
 * an overlap or a broken bond stops the run with DMD_E_OVERLAP. */
#define DMD_FLAG_CHECK_OVERLAP 16
/* Test of the failure path: the event loop's iteration bound (normally
 * 16 * events + 10^6 batches) becomes 8 batches, so a longer run stops with
 * DMD_E_DEVICE_TIMEOUT between two batches, its state intact. */
#define DMD_FLAG_TIGHT_LOOP_BOUND 32

/* One system: chains, sequences, initial state (code/inputinfo.f:5-101,
 * code/main.F90:240-321). */
typedef struct dmd_system {
    int32_t n_beads;
    int32_t n_chains;
    const int32_t *chain_len;  /* residues per chain, [n_chains] */
    const int32_t *residues;   /* residue identity 9..28 per residue, chains concatenated */
    const int32_t *hp;         /* per-bead hydrophobic flag (hp*.inp), or NULL: 1 for side chains */
    double boxl;               /* box side in angstrom */
    const double *x, *y, *z;   /* positions in box units */
    const double *vx, *vy, *vz;/* velocities */
    const int32_t *bptnr;      /* H-bond partners, 1-based, or NULL; restored as with -Drunr */
    double  t0;                /* starting time */
    int64_t coll0;             /* starting collision count */
} dmd_system;

/* One committed event of the log (dmd_run's optional ring buffer). */
typedef struct dmd_event {
    int64_t coll;      /* reference collision counter after this event */
    double  t;         /* time of the last interval commit */
    double  tfalse;    /* event time relative to t */
    int32_t i, j;      /* beads (1-based); j = 0 for pseudo events */
    int32_t type;      /* final coltype 1..27, or DMD_EV_* for pseudo events */
    int32_t evcode;    /* pair type ev_code(i,j) at the event */
} dmd_event;

#define DMD_EV_GHOST    100
#define DMD_EV_INTERVAL 101
#define DMD_EV_REBUILD  102   /* interval event that rebuilt the lists */
#define DMD_EV_OUTPUT   103

typedef struct dmd_event_log {
    dmd_event *events;   /* caller-owned ring of capacity entries */
    int64_t    capacity;
    int64_t    count;    /* out: events written (may exceed capacity: ring wrapped) */
} dmd_event_log;

/* Diagnostics of code/energy.f, code/radgyr.f, code/end2end.f plus counters. */
typedef struct dmd_diag {
    double  e_total, temperature, rg, e2e, ehh_ii, ehh_ij, e_kin;
    int32_t hb_alpha, hb_ii, hb_ij;
    int32_t max_down;         /* engine: the longest down neighbour list at the last rebuild */
    int64_t nevents[32];      /* per final coltype */
    int64_t coll, n_pair, n_ghost, n_interval, n_output, n_updates, n_forced_updates;
    double  t, tfalse;
    double  nbr_mean;         /* mean neighbour-list entries per bead (up + down) */
    int64_t n_batches;        /* engine: pair-event batches committed (0 in a serial run) */
    int64_t n_rolled_back;    /* engine: speculative pair events undone and redone later */
    int64_t n_candidates;     /* engine: pair events that entered a batch (before validation) */
    /* code/check_nc_int.f:9-360: H-bonded pairs whose geometry fails
     * repuls_check, and unbonded NH-CO pairs inside their well whose
     * geometry passes it (0 and 0 in a consistent state) */
    int64_t nc_boundbad, nc_unboundbad;
    /* SM clock cycles the system's (leader) CTA spent in its last event-loop
     * launch (0 before any, and in the CPU restatement) */
    int64_t run_cycles;
} dmd_diag;

typedef struct dmd_handle dmd_handle;

/* Replaces the set-up of program dmd (code/main.F90:117-424: inputinfo,
 * scale_down, make_code, runr restore, nbor_setup, cell_link, nbor, events). */
int dmd_create(const dmd_run_cfg *cfg, const dmd_tables *tables,
               const dmd_system *sys, dmd_handle **out);

/* Replaces the main event loop (code/main.F90:484-1258): commits n_events
 * events (the reference's coll counting unless DMD_FLAG_COUNT_PHYSICAL).
 * log may be NULL. */
int dmd_run(dmd_handle *h, int64_t n_events, dmd_event_log *log);

/* The per-bead event predictions: after dmd_create the full pass of
 * code/events.f:11-127; after a run the queue's current entries (those the
 * partial re-predictions of code/partial_events.f left).  tim/nptnr/coltype
 * per bead (1-based partners, times relative to t). */
int dmd_predict_all(dmd_handle *h, double *tim, int32_t *nptnr, int32_t *coltype);

/* State read-back: the stored positions (box units; the position at the
 * current time is x + vx * tfalse, as in code/config.f:15-24),
 * velocities, H-bond partners, identities, extra_repuls (4 per bead). */
int dmd_get_state(dmd_handle *h, double *x, double *y, double *z,
                  double *vx, double *vy, double *vz, int32_t *bptnr,
                  int32_t *identity, int32_t *extra_repuls,
                  double *t, double *tfalse, int64_t *coll);

/* State write: replaces the system's state by the given positions (box
 * units, at time t: read back as x + vx * tfalse), velocities, 1-based
 * H-bond partners (or NULL) and collision count, as the reference's
 * restart from .config/.bptnr/.lastvel records does (code/main.F90:240-321:
 * identities and shoulders restored from bptnr, lists, cell grid and event
 * queue rebuilt, intervals restarted; the ghost random stream starts again
 * from the seed).  The result is that of dmd_create from the same system
 * with that state; the cluster, rebuild-grid and compact-variant settings
 * are kept.  On an error the previous state stays in force. */
int dmd_set_state(dmd_handle *h, const double *x, const double *y, const double *z,
                  const double *vx, const double *vy, const double *vz, const int32_t *bptnr,
                  double t, int64_t coll);

/* Replaces code/energy.f, code/radgyr.f, code/end2end.f at the current time. */
int dmd_diagnostics(dmd_handle *h, dmd_diag *out);
/* The backbone dihedral histogram of code/phipsi.f (-Dwrite_phipsi, the
 * reference's in-run analysis): dmd_phipsi_sample adds the current (phi,
 * psi) of every residue 2..L-1 of every chain, each as its whole-degree bin
 * res(phi + 180, psi + 180) of a 361 x 361 histogram kept on the device
 * (code/phipsi.f:25-290; the reference samples at the output events of a
 * run's second half and at its end, code/main.F90:1227-1231,1315-1317).
 * dmd_phipsi_histogram copies it out (hist: 361 * 361 counts, index
 * (phi + 180) * 361 + (psi + 180); may be NULL) with the number of samples
 * (may be NULL) and clears both when reset != 0.  A residue whose frame is
 * degenerate (collinear beads) is not counted. */
int dmd_phipsi_sample(dmd_handle *h);
int dmd_phipsi_histogram(dmd_handle *h, int64_t *hist, int64_t *nsamples, int32_t reset);

/* Dense pair-type table ev_code (n_beads x n_beads, row-major, 1-based
 * rows/cols mapped to 0-based), reconstructed from the rule function and
 * the shoulder overrides (code/make_code.f:6-573, code/repuls_add.f). */
int dmd_get_evcode(dmd_handle *h, int8_t *out);

/* Device time in ms of the kernel of the last dmd_run, measured with CUDA
 * events on the stream it was launched on (no reference counterpart). */
double dmd_last_run_ms(dmd_handle *h);

/* Checkpoint of the whole engine state of a system (positions, velocities,
 * H-bond state, lists, event queue, counters, random-stream position), so
 * that a run resumes bit-identically (the reference's restart from
 * .config/.bptnr/.lastvel records, code/main.F90:240-321, rebuilds the
 * queue and restarts the intervals instead).  Load into a handle created
 * from the same system. */
int64_t dmd_state_bytes(dmd_handle *h);
int dmd_save_state(dmd_handle *h, void *buf, int64_t n);
int dmd_load_state(dmd_handle *h, const void *buf, int64_t n);

void dmd_destroy(dmd_handle *h);

/* Checked build only (compiled with -DDMD_BOUNDS; no reference
 * counterpart): the first out-of-range index any device array access met
 * since the last call, recorded instead of faulting (the access used index
 * 0), then cleared.  Returns 1 with *rec = site << 40 | extent << 20 |
 * index, 0 if none, -1 in a build without the checks. */
int dmd_debug_bounds(long long *rec);

const char *dmd_last_error(dmd_handle *h);
const char *dmd_version(void);

/* Host-only (no GPU): the static pair-type table ev_code of code/make_code.f
 * as the engine's rule computes it, before any H-bond shoulder (dense,
 * row-major n_beads x n_beads). */
int dmd_static_evcode(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                      int8_t *out, char *err, int32_t errlen);
/* Allocation-free variant of dmd_create + dmd_predict_all (no counterpart in
 * the reference, which has no device code).  For callers that cannot allocate
 * device memory themselves: a host whose device memory is owned by another
 * runtime or pool (a Fortran program under OpenACC/CUDA Fortran data regions,
 * a serving process that reserves a fixed budget up front), where a
 * cudaMalloc would synchronise the device, fail, or break that accounting.
 * The caller passes the same host inputs as dmd_create and three device
 * buffers of n_beads entries that receive the full prediction pass: times,
 * 1-based partners, event types, equal to what dmd_predict_all returns right
 * after dmd_create from the same inputs.  All intermediate
 * data lives in one static device array of 8 MiB inside the library, which
 * every GPU that loads the library holds until the process exits; systems of
 * at most 8192 beads, neighbour lists of at most 64 entries (list_cap) and a
 * rebuild grid of at most 48 cells per side fit, and larger inputs are
 * rejected with DMD_E_CAPACITY and a message.  The first call on a device
 * looks up the array's address there (with that device current) and keeps
 * it for later calls.  The call copies its inputs from
 * pageable host memory and waits for the stream, so it may not be called
 * while any stream is being captured into a CUDA graph; such a call returns
 * DMD_E_STATE with a message and leaves the capture alone.  Every call
 * reuses the array: calls whose work overlaps on the GPU (different streams
 * or host threads) race on it.
 * stream: a cudaStream_t, or NULL for the default stream; the call returns
 * after the stream has finished the pass. */
int dmd_predict_all_noalloc(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                            double *d_tim, int32_t *d_nptnr, int32_t *d_coltype, void *stream,
                            char *err, int32_t errlen);

/* Host-only: set-up values of code/main.F90:144-156 and code/nbor_setup.f:
 * interval, interval_max, sig_max_all, hdelr, cells per side, rl, rlsq(1),
 * rlsq(15), rlsq(16), rlsq(40), n_forced, t_fact, ev_param(1,15).
 * Returns the number of values available. */
int dmd_inspect(const dmd_run_cfg *cfg, const dmd_tables *tables, const dmd_system *sys,
                double *out, int32_t n, char *err, int32_t errlen);

/* ---- batched replicas: many independent systems in one persistent launch
 * (no reference counterpart: the reference runs one system per MPI job). */
typedef struct dmd_batch dmd_batch;
int dmd_batch_create(int32_t n, const dmd_run_cfg *cfgs, const dmd_tables *tables,
                     const dmd_system *systems, dmd_batch **out);
/* Advances every replica by n_events (per replica); per-replica logs optional. */
int dmd_batch_run(dmd_batch *b, int64_t n_events, dmd_event_log *logs);
int dmd_batch_get_state(dmd_batch *b, int32_t r, double *x, double *y, double *z,
                        double *vx, double *vy, double *vz, int32_t *bptnr,
                        int32_t *identity, int32_t *extra_repuls,
                        double *t, double *tfalse, int64_t *coll);
int dmd_batch_diagnostics(dmd_batch *b, int32_t r, dmd_diag *out);
/* dmd_phipsi_* for system r of a batch (sample: r < 0 samples every system) */
int dmd_batch_phipsi_sample(dmd_batch *b, int32_t r);
int dmd_batch_phipsi_histogram(dmd_batch *b, int32_t r, int64_t *hist, int64_t *nsamples, int32_t reset);
double dmd_batch_last_run_ms(dmd_batch *b);
/* CTAs (one thread-block cluster) that advance each system: 1, 2, 4 or 8,
 * or 0 (default) to let the library choose from the number of systems and
 * what the GPU can hold at once.  Results do not depend on it: the
 * committed event sequence is the serial one for every value. */
int dmd_batch_set_cluster(dmd_batch *b, int32_t ctas);
int dmd_set_cluster(dmd_handle *h, int32_t ctas);
/* the cluster size the last run used */
int32_t dmd_batch_cluster(dmd_batch *b);
/* device bytes of the batch's system pools */
int64_t dmd_batch_device_bytes(dmd_batch *b);
/* host-to-device bytes dmd_batch_create copied: each pool's head (tables,
 * scalars, bead state), one copy per system from a pinned host image; the
 * rest of a pool (lists, grid, tournament) is written on the device */
int64_t dmd_batch_upload_bytes(dmd_batch *b);
/* device-to-host bytes of reading every system's state after a run
 * (dmd_batch_get_state): one block per system - positions, velocities,
 * identities, H-bond partners, extra_repuls - plus its scalars */
int64_t dmd_batch_readback_bytes(dmd_batch *b);
/* Rebuild grid: cells per side of the finest grid (cells as wide as the
 * list cutoff) divided by div (1..8, at least 3 cells per side).  Lists
 * and results do not depend on it. */
int dmd_batch_set_cell_div(dmd_batch *b, int32_t div);
/* Event-loop variant: the compact one (per-warp event areas sized for down
 * neighbour lists of at most 32 beads, which leaves most of the SM's
 * shared memory to the L1 cache) runs while every system's longest down
 * list is at most max_down; a system whose lists outgrow it at a rebuild
 * finishes the run on the full variant.  max_down 0..32 (default 32; 0:
 * always the full variant).  Results do not depend on it. */
int dmd_batch_set_compact_limit(dmd_batch *b, int32_t max_down);
int dmd_set_compact_limit(dmd_handle *h, int32_t max_down);
/* n_launches launches of n_events each, captured into a CUDA graph on the
 * first call (and again when the sizes or the cluster size change) and
 * replayed; the same result as dmd_batch_run with n_events * n_launches. */
int dmd_batch_run_graph(dmd_batch *b, int64_t n_events, int32_t n_launches);
/* Rebuild cycles from a CUDA graph (the loop of code/main.F90:1126-1187,
 * one list rebuild per launch): launches_per_graph launches are captured
 * into a graph on the first call (and again when the cluster size or the
 * event-loop variant changes); each launch runs every system up to and
 * including its next neighbour-list rebuild, or to the end of its events,
 * and keeps the events it still has to run on the device.  The graph is
 * replayed until every system has run n_events; n_launches (may be NULL)
 * receives the launches replayed.  The same result as dmd_batch_run with
 * n_events.  The host regains control at each replay, every
 * launches_per_graph rebuild cycles. */
int dmd_batch_run_cycles(dmd_batch *b, int64_t n_events, int32_t launches_per_graph, int64_t *n_launches);
/* Autotuner: trial runs of a copy of the batch (from its create-time inputs)
 * for each cluster size that fits and rebuild grids with div 1 and 2; keeps
 * the fastest for this batch and reports it (best_ms: device time of its
 * trial).  The batch's own state is not advanced. */
int dmd_batch_autotune(dmd_batch *b, int64_t trial_events, int32_t *cluster, int32_t *cell_div,
                       double *best_ms);
/* The autotuner with its choices kept in a JSON file (created if absent):
 * a batch whose systems have the same bead counts, chain counts, list
 * capacities and grids, on a device of the same compute capability and SM
 * count, with the same library version, compact limit, H-bond flag and
 * trial_events, takes the stored cluster size and rebuild grid without
 * trial runs (*from_cache = 1); otherwise the trials run and their result
 * is added to the file (*from_cache = 0).  A file that is not such a cache
 * is left untouched and DMD_E_INPUT returned.  Output pointers may be NULL. */
int dmd_batch_autotune_cached(dmd_batch *b, int64_t trial_events, const char *cache_path, int32_t *cluster,
                              int32_t *cell_div, double *best_ms, int32_t *from_cache);
void dmd_batch_destroy(dmd_batch *b);
const char *dmd_batch_last_error(dmd_batch *b);

/* ---- serving: continuous batching of independent simulation requests (no
 * reference counterpart: the reference runs one system per MPI job).
 * Requests are admitted first in, first out while slots and the
 * device-memory budget allow; every dmd_server_step() advances all running
 * requests by up to chunk_events in one launch while the next requests are
 * uploaded on a second stream, then hands back the finished ones.  A
 * request's result does not depend on what runs beside it. */
#define DMD_REQ_QUEUED 0
#define DMD_REQ_ACTIVE 1
#define DMD_REQ_DONE   2
#define DMD_REQ_FAILED 3
typedef struct dmd_server dmd_server;
/* hbm_budget_bytes <= 0: 90 % of the free device memory at creation */
int dmd_server_create(int32_t max_slots, int64_t hbm_budget_bytes, int64_t chunk_events, dmd_server **out);
/* thread-safe with respect to dmd_server_step; the set-up work runs on the
 * calling thread */
int dmd_server_submit(dmd_server *s, const dmd_run_cfg *cfg, const dmd_tables *tables,
                      const dmd_system *sys, int64_t n_events, int64_t *id);
int dmd_server_step(dmd_server *s, int32_t *n_active, int32_t *n_finished);
/* times are seconds of a monotonic host clock */
int dmd_server_status(dmd_server *s, int64_t id, int32_t *state, int64_t *events_done,
                      double *t_submit, double *t_admit, double *t_finish);
int dmd_server_result(dmd_server *s, int64_t id, dmd_diag *diag, double *x, double *y, double *z,
                      double *vx, double *vy, double *vz, int32_t *bptnr, int32_t *identity,
                      double *t, double *tfalse, int64_t *coll);
int dmd_server_release(dmd_server *s, int64_t id);
int dmd_server_stats(dmd_server *s, int64_t *steps, int64_t *events, double *kernel_ms,
                     int32_t *n_waiting, int32_t *n_active, int64_t *bytes_used, int64_t *bytes_budget);
const char *dmd_server_last_error(dmd_server *s);
void dmd_server_destroy(dmd_server *s);

/* ---- synthetic systems (restates the insertion and velocity steps of
 * genconfig/gen_config_random-SQZ.f90:665-891 on an extended template). */
typedef struct dmd_gen_spec {
    int32_t n_chains;
    const int32_t *chain_len;  /* residues per chain */
    const int32_t *residues;   /* residue identities 9..28, concatenated */
    double  boxl;              /* angstrom */
    double  tstar;
    uint64_t seed;
    double  min_sep;           /* inter-chain rejection distance, angstrom (5) */
} dmd_gen_spec;
/* Fills positions (box units) and velocities of n_beads beads. */
int dmd_generate(const dmd_gen_spec *spec, const dmd_tables *tables, int32_t n_beads,
                 double *x, double *y, double *z, double *vx, double *vy, double *vz,
                 char *err, int32_t errlen);

/* The side-chain placement search of the reference's initial-configuration
 * generator (genconfig/gen_config_random-SQZ.f90:250-348), on the GPU.  For
 * each of n_res consecutive residues of one chain (positions [n_res][3] in
 * angstrom: C-alpha, NH, CO, and the side chain's start), the side chain is
 * moved over the grid of offsets -move .. move in steps of step on each axis
 * (the generator's Fortran DO loops over real variables: trip count
 * INT((2 move + step) / step), values by repeated addition; the reference
 * uses move 3.5, step 0.005, i.e. 1,401^3 points); the winner is the first
 * point in the generator's loop order (x outermost) with the smallest
 * r3 = |rca - r(CA)| + |rnh - r(NH)| + |rco - r(CO)| (tables->rca/rnh/rco of
 * the residue's identity 9..28) below 100 among the points whose distances
 * to CO and CA of the previous residue and NH and CA of the next one are
 * not below tables->sqz (sz6, sz8, sz7, sz9).  side_out gets the moved side
 * chains, rmin_out each residue's r3, index_out (may be NULL) the winning
 * point (i1 * m + i2) * m + i3 with m = dmd_sidechain_grid(move, step).  A
 * residue without an admissible point keeps its start (rmin 100, index -1;
 * the generator would apply the previous residue's offset).  Results are
 * exactly those of the generator's expressions in double precision.  Up to
 * 4,096 grid values per axis and 65,535 residues per call. */
int dmd_sidechain_search(int32_t n_res, const double *ca, const double *nh, const double *co,
                         const double *side, const int32_t *residue, const dmd_tables *tables,
                         double move, double step, double *side_out, double *rmin_out,
                         int64_t *index_out, char *err, int32_t errlen);
/* grid values per axis of dmd_sidechain_search, -1 for a bad move or step */
int64_t dmd_sidechain_grid(double move, double step);

#ifdef __cplusplus
}
#endif
#endif /* DMD_H */
