/*
 * mcsgpu.h -- C ABI of the GB300 Monte Carlo spin-lattice engine (libmcsgpu.so).
 *
 * Plain C: pointers, sizes and int status codes; no exceptions and no
 * framework types cross this boundary.  The CPython modules isinglib, xylib and
 * heisenberglib (drop-in for mcsolver's compiled libraries) are thin wrappers
 * over mcs_solve(); ctypes, a serving loop or a C program can call it directly.
 *
 * Reference interfaces replaced (golddoushi/mcsolver):
 *   mcs_solve() with model MCS_ISING      <- MCMainFunction, mcsolver/isingLib.c:259-451
 *                                            (arguments isingLib.c:277-284, result :436-447)
 *   mcs_solve() with model MCS_XY         <- MCMainFunction, mcsolver/xyLib.c:413-809
 *                                            (arguments xyLib.c:439-447, result :778-807)
 *   mcs_solve() with model MCS_HEISENBERG <- MCMainFunction, mcsolver/heisenbergLib.c:478-885
 *                                            (arguments heisenbergLib.c:504-512, result :853-884)
 *   mcs_batch_*()                         <- the process-pool fan-out over the (T,H) grid,
 *                                            mcsolver/win.py:399-428 and :440-469
 *   mcs_pt_*()                            <- (no counterpart: the reference runs each
 *                                            temperature independently, win.py:440-444)
 *   mcs_server_*()                        <- (no counterpart: continuous-batching request loop)
 */
#ifndef MCSGPU_H
#define MCSGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MCS_OK 0
#define MCS_EINVAL 1       /* malformed input (sizes, indices, ranges)        */
#define MCS_ECUDA 2        /* CUDA runtime error                              */
#define MCS_ETIMEOUT 3     /* a bounded device wait ran out                   */
#define MCS_ENOMEM 4       /* device memory / HBM budget exhausted            */
#define MCS_EUNSUPPORTED 5 /* model outside what the engine implements        */
#define MCS_EBUSY 6        /* server: no free slot (try again)                */
#define MCS_ENOTFOUND 7    /* server: unknown ticket                          */
#define MCS_ECANCELLED 8   /* server: the request was cancelled               */
#define MCS_EFAILED 9      /* server: the request failed while it ran         */

#define MCS_ISING 1
#define MCS_XY 2
#define MCS_HEISENBERG 3

#define MCS_METROPOLIS 0
#define MCS_WOLFF 1

/* One solve, in the reference's flattened layout (units: energies already
 * multiplied by beta = 1/T, exactly as mcMain.py passes them: mcMain.py:26,
 * :30-31, :121, :244).  Arrays are borrowed for the duration of the call. */
typedef struct mcs_problem {
    int32_t model;              /* MCS_ISING / MCS_XY / MCS_HEISENBERG        */
    int32_t algorithm;          /* MCS_METROPOLIS / MCS_WOLFF                 */
    int32_t n_sites;            /* totOrbs = len(initSpin)                    */
    int32_t max_links;          /* maxNLinking                                */
    int64_t nthermal, nsweep, ninterval;
    const double *init_spin;    /* [n_sites] signed spin length S            */
    const double *init_d;       /* [3*n_sites] D/T, O(n) only (may be NULL)  */
    const int32_t *nlink;       /* [n_sites]                                  */
    const double *link_strength;/* Ising [n_sites*max_links]; O(n) [9*n_sites*max_links],
                                   components xx,yy,zz,xy,xz,yz,yx,zx,zy     */
    const int32_t *linked_orb;  /* [n_sites*max_links], -1 padded            */
    const int32_t *circuits;    /* [3*n_circuits] (Heisenberg)               */
    const int32_t *corr_pair;   /* [2*n_lat]                                  */
    const int32_t *group_list;  /* [n_group*max_group], -1 padded            */
    const int32_t *r_orb;       /* [n_rorb]                                   */
    const int32_t *r_cluster;   /* [n_rorb*n_in_cluster]                      */
    const int32_t *r_link;      /* [n_rorb*max_links], -1 padded             */
    double flunc, h;            /* initial tilt; field h/T                    */
    int32_t n_circuits, n_lat, n_group, max_group;
    int32_t n_rorb, n_in_cluster, ignore_offdiag, spin_frames;
} mcs_problem;

/* Engine knobs that the reference signature does not carry. */
typedef struct mcs_options {
    uint64_t seed;              /* Philox key of this solve                   */
    int32_t schedule;           /* 0 auto, 1 plain (host-driven, one launch per
                                   colour and per measurement), 2 resident
                                   (whole lattice in one CTA's shared memory),
                                   3 tiled (lattice in global memory)        */
    int32_t absolute_energy;    /* Ising Metropolis: report absolute <e>
                                   instead of the reference's offset one      */
    int32_t recheck_every;      /* O(n): full FP64 energy re-check every k
                                   measurements (0 = default 32)             */
    int32_t record_series;      /* keep per-measurement e, M, e_r, <si.sj>    */
    int32_t random_init;        /* 1: ignore init_spin directions, draw them
                                   from the seed (Ising sign, XY angle,
                                   Heisenberg sphere); lengths stay |S|       */
    int32_t fp64_update;        /* must be 0: FP32 spin updates only (1 is    */
                                /* rejected with MCS_EUNSUPPORTED)            */
    int32_t device;             /* CUDA device ordinal                        */
    int32_t reserved_;
} mcs_options;

#define MCS_RESULT_VALUES 29
typedef struct mcs_result {
    /* the reference's result tuple; Ising uses values[0..9] (isingLib.c:437-446),
       O(n) uses values[0..26] (heisenbergLib.c:855-881) */
    double values[MCS_RESULT_VALUES];
    double *group_values;       /* caller buffer, (G+1)^2+(G+1) doubles (or NULL) */
    int32_t group_capacity;
    int32_t frames_written;
    float *frames;              /* caller buffer, spin_frames*n_sites*3 floats (or NULL) */
    double *series;             /* caller buffer, nsweep*4 doubles (or NULL)   */
    int64_t site_updates;       /* Metropolis site visits + Wolff flipped sites */
    int64_t clusters;           /* Wolff clusters built                       */
    int64_t flipped;            /* Wolff sites flipped                        */
    int64_t accepted;           /* accepted moves / clusters                  */
    int64_t exact_mismatches;   /* Ising: measurements where incremental E != full recompute */
    double energy_drift;        /* O(n): max |E_incr - E_full| seen at re-checks (beta units) */
    double device_ms;           /* device time of the solve                   */
    int32_t schedule_used;
    int32_t n_colours;
} mcs_result;

/* Solve one (T,H) point.  Returns MCS_OK or an error code; the message is in
 * mcs_last_error().  Never aborts the process. */
int mcs_solve(const mcs_problem *problem, const mcs_options *options, mcs_result *result);

/* Last error message of this thread. */
const char *mcs_last_error(void);

/* Version and build information. */
int mcs_abi_version(void);
const char *mcs_build_info(void);

/* ---- batched engine: many replicas of uneven sizes in one launch sequence -- */
typedef struct mcs_batch mcs_batch;
int mcs_batch_create(int32_t device, mcs_batch **out);
/* Compile and upload one replica; returns its index in *replica. */
int mcs_batch_add(mcs_batch *b, const mcs_problem *problem, const mcs_options *options, int32_t *replica);
/* Run every replica to completion (persistent launches, CUDA graphs). */
int mcs_batch_run(mcs_batch *b);
/* Upload and initialise without running (optional; mcs_batch_advance does it). */
int mcs_batch_prepare(mcs_batch *b);
/* Advance every unfinished replica by up to `units` units (Metropolis sweeps
 * or Wolff clusters, each followed by its measurements); *device_ms receives
 * the device time of this call. */
int mcs_batch_advance(mcs_batch *b, int64_t units, double *device_ms);
int mcs_batch_result(mcs_batch *b, int32_t replica, mcs_result *result);
/* Device time of the last mcs_batch_run and its total site updates. */
int mcs_batch_stats(mcs_batch *b, double *device_ms, int64_t *site_updates, int32_t *launches);
/* Device bytes the batch holds (uploaded from the host) and bytes read back
 * per result collection. */
int mcs_batch_memory(mcs_batch *b, uint64_t *device_bytes, uint64_t *readback_bytes);
/* Schedule of launch group `group` (0-based) after preparation: *kind 1 plain,
 * 2 resident (one CTA per replica), 3 tiled (global memory, graphs),
 * 4 Wolff in shared memory, 5 Wolff in global memory, 6 thread-block cluster;
 * *cluster = CTAs per replica of the cluster kernel (0 = the one-CTA resident
 * kernel; -k = the resident kernel with k copies of each replica, one per CTA
 * of a cluster), *threads per CTA, *replicas in the group.
 * Returns MCS_EINVAL when `group` is out of range (no counterpart in the
 * reference, which has one schedule). */
int mcs_batch_schedule(mcs_batch *b, int32_t group, int32_t *kind, int32_t *cluster, int32_t *threads,
                       int32_t *replicas);
void mcs_batch_destroy(mcs_batch *b);

/* ---- parallel tempering over a temperature ladder (one model) ------------- */
/* The problem's couplings, anisotropy and field are PHYSICAL (not divided by T);
 * betas[k] = 1/T_k.  One replica per temperature; after every sweep neighbouring
 * temperatures try to swap with probability min(1, exp((b_i-b_j)(E_i-E_j))).
 * Results are per temperature (index k). */
typedef struct mcs_pt mcs_pt;
int mcs_pt_create(const mcs_problem *problem, const mcs_options *options, const double *betas,
                  int32_t n_temps, mcs_pt **out);
int mcs_pt_run(mcs_pt *pt);
int mcs_pt_result(mcs_pt *pt, int32_t temp_index, mcs_result *result);
/* swap acceptance per neighbouring pair [n_temps-1] and round trips */
int mcs_pt_stats(mcs_pt *pt, double *swap_acceptance, double *device_ms, int64_t *site_updates);
void mcs_pt_destroy(mcs_pt *pt);

/* ---- continuous-batching server --------------------------------------- */
typedef struct mcs_server mcs_server;
/* hbm_budget_bytes: device memory the server may hold for request state. */
int mcs_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots, mcs_server **out);
/* Queue one solve; *ticket identifies it.  The problem is compiled on the
 * calling thread before this returns (its arrays may be freed afterwards).
 * Admission happens in mcs_server_step when slots and memory allow.
 * submit, poll and stats may run on any threads concurrently with step. */
int mcs_server_submit(mcs_server *s, const mcs_problem *problem, const mcs_options *options, uint64_t *ticket);
/* Advance the device by one tick: retire cancelled requests, admit queued
 * ones, advance every active request by its own quota of units (about the
 * same device time per request and step, MCSGPU_SERVER_STEP_US, default
 * 2000 us: small lattices run many sweeps per step, large ones few), retire
 * finished ones.  *completed receives the number of requests completed.  One
 * step at a time.  A request that fails is retired with its own status (see
 * mcs_server_poll) and the others go on; the step itself returns an error only
 * when the device context is lost, and then every active request has failed. */
int mcs_server_step(mcs_server *s, int32_t *completed);
/* 0 = done (result filled, ticket released), 1 = pending; a request that
 * failed or was cancelled returns its own status (MCS_ENOMEM, MCS_ECUDA,
 * MCS_ECANCELLED, MCS_EFAILED ...; never 1), releases the ticket and leaves its
 * message in mcs_last_error(); MCS_ENOTFOUND for an unknown ticket. */
int mcs_server_poll(mcs_server *s, uint64_t ticket, mcs_result *result);
/* Cancel a queued or active request (no counterpart in the reference, whose
 * solves cannot be stopped): a queued one is released at once, an active one
 * at the start of the next step; its poll then returns MCS_ECANCELLED.  A
 * request that already finished keeps its result (MCS_OK). */
int mcs_server_cancel(mcs_server *s, uint64_t ticket);
int mcs_server_stats(mcs_server *s, int32_t *active, int32_t *queued, uint64_t *bytes_in_use, int64_t *site_updates);
void mcs_server_destroy(mcs_server *s);

/* ---- allocation-free sweeps ------------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc --
 * a framework that owns all device memory through its own allocator, a process
 * that reserved the GPU's memory up front, code inside another library's
 * allocation scope -- this entry point allocates nothing (no device, no pinned
 * host memory).  The caller passes device pointers:
 *   d_sigma  [Lx*Ly] int8 spins +-1 of a periodic square lattice, site order
 *            x*Ly + y, updated in place;
 *   d_sums   [nsweeps][2] int64, written after each sweep: the sum of the
 *            spins and the sum of s_i*s_j over the 2*Lx*Ly bonds.
 * K = J/T and h = H/T follow the reference's sign convention (K < 0 is a
 * ferromagnet; the acceptance rule is isingLib.c:242-252).  The sweeps are the
 * Ising Metropolis sweeps of mcs_solve(): same colour order, same Philox words
 * (sweep index sweep0 + k), same integer thresholds, so the spins equal those
 * mcs_solve() produces for the same lattice, couplings and seed.
 * Scratch: a fixed 64 KiB array in device memory owned by the library (held by
 * every GPU that loads it until exit), which limits the lattice to 8,388,608
 * sites (larger lattices are rejected with MCS_EINVAL).  Every call looks up
 * that array's address on the current device; the first call on a device
 * (and the first after a device reset) also loads the library's kernels,
 * which takes some device memory for the module: make that call before
 * reserving the device's memory or beginning a stream capture.  `stream`
 * must belong to the current device (MCS_EINVAL otherwise).  Calls that
 * overlap on the GPU share the array and race: issue them on one stream, one
 * after the other.  Lx, Ly even and >= 4. */
int mcs_ising_square_noalloc(int8_t *d_sigma, int32_t Lx, int32_t Ly, double K, double h, uint64_t seed,
                             int64_t sweep0, int32_t nsweeps, int64_t *d_sums, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MCSGPU_H */
