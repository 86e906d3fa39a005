// mcs_internal.h -- data layout shared by the host engine and the sm_103a kernels.
//
// One "replica" is one Monte Carlo solve (one (T,H) point of one model).  Its
// lattice is stored on the device in colour-major order: the sites of colour 0
// first, then colour 1, ..., ascending original site id inside a colour.  The
// position of a site in that order is its "sweep index"; every device array
// (spins, neighbour table, measurement lists) is indexed by sweep index, and
// every Philox counter names sites by sweep index.
#pragma once
#include <stdint.h>

#define MCS_MAXC 4        // Ising coupling classes handled exactly
#define MCS_MAXT 4        // Ising site types
#define MCS_MAXG 8        // orbital groups (per-site bitmask)
#define MCS_NSER 4        // per-measurement series: e, M, e_r, <si.sj>
#define MCS_MAXZ 32       // links per site

#define MCS_GEOM_ELL 0    // general neighbour table
#define MCS_GEOM_SQUARE 1 // 2D square lattice, 4 neighbours, parity colouring

// ---- FP64 accumulators of an O(n) replica (indices into Rep::acc)
enum {
    A_SI = 0, A_SJ = 3, A_SIJ = 6, A_E = 7, A_E2 = 8, A_M2 = 9, A_M4 = 10, A_MTOT = 11,
    A_MDM = 12, A_MPREV = 13, A_SIR = 14, A_SJR = 17, A_SIJR = 20, A_ER = 21, A_ER2 = 22,
    A_SIZ = 23, A_SJZ = 24, A_STZ = 25, A_SIH = 26, A_SJH = 27, A_STH = 28, A_Q = 29,
    A_ECUR = 30,   // running energy (table units)
    A_DRIFT = 31,  // max |E_incr - E_full| at re-checks
    A_GRP = 32     // (G+1)^2 spin.spin between groups, then (G+1) 4th moments
};
// ---- FP64 accumulators of an Ising replica
enum {
    B_SI = 0, B_SJ = 1, B_SIJ = 2, B_E = 3, B_E2 = 4, B_ER = 5, B_ER2 = 6, B_M2 = 7, B_M4 = 8,
    B_MTOT = 9, B_MDM = 10, B_MPREV = 11, B_STOT = 12, B_EMEAS0 = 13, B_NACC = 16
};
// ---- Ising integer counters (int64, Rep::icnt)
enum {
    C_DN = 0,      // [MAXC] running change of the directed bond sums N_c (incremental)
    C_DM = 4,      // [MAXT] running change of the per-type sign sums M_t (incremental)
    C_N0 = 8,      // [MAXC] N_c at run start (full recompute)
    C_M0 = 12,     // [MAXT] M_t at run start
    C_MISM = 16,   // measurements where incremental != full recompute
    C_ACC_MEAS = 17, // Wolff: an accepted cluster happened since the measurement phase began
    C_NINT = 24
};
// ---- generic counters (int64, Rep::stats)
enum { S_VISITS = 0, S_ACCEPT = 1, S_CLUSTERS = 2, S_FLIPPED = 3, S_NSTAT = 4 };

// ---- O(n) measurement frame (sums over the lattice of one measurement)
enum {
    F_SI = 0, F_SJ = 3, F_SIJ = 6, F_TOT = 7, F_Q = 10, F_SIR = 11, F_SJR = 14, F_SIJR = 17,
    F_ERB = 18, F_ERO = 19, F_EFB = 20, F_EFO = 21, F_G = 22,
    F_NON = 22 + 3 * MCS_MAXG
};
// ---- Ising measurement frame
enum {
    G_SI = 0, G_SJ = 1, G_SIJ = 2, G_ER = 3, G_M = 4 /*[MAXT]*/, G_N = 8 /*[MAXC]*/, G_LAST = 12,
    G_NIS = 13
};
#define MCS_NFMAX F_NON

// One Ising acceptance-table entry: for a site type and a neighbour-sign
// pattern, the Philox-word thresholds for sigma_i = -1 / +1 (accept iff
// w < thr; 2^32 = always) and the per-class neighbour sums n_c (int8 x 4).
struct IsEntry {
    unsigned long long thr[2];
    int nc;
    int pad;
};

struct Rep {
    // ---- geometry
    int model, dim, geom, alg;
    int N, zmax, ncol, Ly;          // Ly: square lattice side along y (N = Lx*Ly)
    int Lx, hy, half;               // square: Lx, Ly/2, N/2
    int sq_code[4];                 // square: link code for +x, -x, +y, -y
    int sq_cls[4];                  // square Ising: class of +x, -x, +y, -y
    int col_start[65];              // colour ranges in sweep-index space
    const int *nbr;                 // ELL [zmax][N]
    const unsigned short *lcode;    // ELL [zmax][N]: O(n) J class; Ising table stride
    const unsigned char *lcls;      // ELL Ising [zmax][N]: coupling class
    const unsigned char *deg;       // ELL [N]
    const unsigned char *stype;     // per site: Ising type / O(n) D class (NULL = 0)
    // ---- parameters
    const float *jtab; int njc; int fullJ;       // O(n) [njc][9] xx,yy,zz,xy,xz,yz,yx,zx,zy
    const double *jtab64;                        // same in FP64 (fp64 updates)
    const float *dtab; int ndc; int has_d;       // O(n) [ndc][4]: Dx, Dy, Dz, |S|
    const IsEntry *itab; int nite; int ntype;    // Ising
    int ibase[MCS_MAXT];
    double Q[MCS_MAXC]; int nclass; int exact_ok;
    double Stype[MCS_MAXT];
    double Qw[MCS_MAXC];                         // Wolff: add thresholds per class (as double)
    unsigned long long wthr[MCS_MAXC][2];        // Ising Wolff add threshold, [class][sigma_i*sigma_j>0]
    float beta; float h; double hd;
    int fp64;
    unsigned long long seed;
    // ---- measurement lists (sweep indices)
    int nlat; const int *cpair;                  // [2*nlat]
    int n_rorb, ncl;
    const int *rorb;                             // [n_rorb]
    const int *rcl;                              // [n_rorb*ncl]
    const int *rlink;                            // [n_rorb*zmax] (-1 = none)
    const unsigned short *rjc;                   // O(n) [n_rorb*zmax]: J class of the link
    const double *rK;                            // Ising [n_rorb*zmax]: link strength
    const unsigned char *rkc;                    // Ising [n_rorb*zmax]: class of rK (fast path)
    double rKv[4];                               // Ising: the <= 4 distinct rK values
    int is_fast;                                 // Ising: one spin length and <= 4 rK values
    const unsigned char *rdeg;                   // [n_rorb]: nlink of the chosen site
    const int *rindex;                           // [N]: index in rorb or -1
    int ncirc; const int *circ;                  // [3*ncirc]
    const float *slen;                           // [N] |S| (circuit normalisation)
    const float *sval;                           // [N] signed S (majority scaling)
    int ngroup; const unsigned char *gmask;      // [N]
    int gall;                                    // bitmask of groups that hold every site
    int ci, cj, cij;                             // chosen counts of the pair lists
    double inv_nl, inv_N, inv_ci, inv_cj, inv_cij, inv_nr;  // reciprocals of the divisors above
    float finv_nl, finv_N, finv_ci, finv_cj, finv_cij, finv_nr;  // the same in FP32 (per-measurement observables)
    int nacc;                                    // FP64 accumulators in acc[]
    int uniform_len;                             // every |S| equal (circuit fast path)
    float inv_len3;                              // 1/|S|^3 when uniform_len
    int pair_identity;                           // every pair is (v, v), each site at most once
    const unsigned char *sflag;                  // [N] bit0: site is a pair member, bit1: chosen
    const int *rtgt;                             // [n_rorb*zmax] index in rorb of the l-th renormalised target (-1)
    // regular square measurement (cluster schedule): every site is a (v, v)
    // pair, one signed spin value sval0, every group holds every site, and each
    // chosen block links to the blocks two sites away along +x, -x, +y, -y with
    // exchange classes rdir_cls[0..3]; the frame then needs no index lists
    int meas_regular;
    float sval0;
    int rdir_cls[4];
    unsigned char rdir_slot[16];                 // Ising cluster frame: list slot of the +x, -x, +y, -y renormalised link,
                                                 // [4 * kind + direction], kind = (first row) | 2 (first column)
    // ---- program
    long long units_thermal, units_total, nsweep;
    int upm;                                     // units per measurement
    int frames; long long frame_every;
    int recheck;                                 // O(n): full energy every k measurements
    double ts_const;                             // Ising: reference totSpin offset
    int ts_wolff_last;                           // Ising Wolff: totSpin excludes the last site
    int last_site;                               // sweep index of original site N-1
    int offset_energy;                           // Ising Metropolis offset semantics
    int rinit;                                   // draw the initial state from Philox (a, 0, 0, 0x5000)
    // ---- state
    void *spins;                                 // Ising int8[N]; O(n) float[dim][spad] (or double)
    int spad;
    double *acc;
    double *series;                              // [nsweep][MCS_NSER]
    void *frame_buf;                             // spin frames in page-locked host memory mapped into the
                                                 // device: Ising [frames][N] int8 signs, O(n) [frames][N][dim] FP32
    long long *icnt;                             // Ising counters
    long long *stats;                            // generic counters
    unsigned int *wbits;                         // Wolff in-cluster bits (global schedule)
    int *wqueue;                                 // Wolff queue (global schedule)
    float *wmaj;                                 // O(n) Wolff: the block spins of a measurement ([n_rorb][3])
    long long u0;                                // RNG unit offset
    long long u;                                 // next unit
    long long u_stop;                            // a launch stops the replica here (units_total, or the
                                                 // server's per-step bound u + quota)
    long long quota;                             // server: units per step (0 = none)
    long long m;                                 // next measurement
    int frames_written;
    int err;
    // ---- parallel tempering (temperature-dependent fields swap between replicas)
    int tslot;
};

// Work item of the tiled (global-memory) schedule.
struct Item {
    int rep;
    int begin, end;   // colour-local index range (sweep) or virtual index range (measure)
    int slot;         // sweep: partial-sum slot of this tile (per replica contiguous)
};

// ---- launchers (mcs_kernels.cu)
#include <cuda_runtime.h>
namespace mcs {
// shared memory a resident replica needs (bytes), or -1 if it cannot be resident
long long resident_smem_bytes(const Rep &r);
int resident_max_smem();
long long wolff_smem_bytes(const Rep &r, int *gstate);
cudaError_t launch_wolff(int dim, int geom, Rep *reps, const int *ids, int nrep, int threads, size_t smem,
                         long long max_units, int gstate, cudaStream_t st);
long long cluster_smem_bytes(const Rep &r, int C);
int cluster_active(int dim, int C, int threads, size_t smem);  // 0: this cluster shape cannot launch
cudaError_t launch_pt_exchange(Rep *reps, int nt, int *perm, unsigned long long seed, long long *acc_cnt,
                               long long *att_cnt, cudaStream_t st);
cudaError_t launch_cluster_metro(int dim, Rep *reps, const int *ids, int nrep, int C, int threads, size_t smem,
                                 long long max_units, cudaStream_t st);
cudaError_t launch_resident_metro(int dim, int geom, Rep *reps, const int *ids, int nrep, int threads,
                                  size_t smem, long long max_units, cudaStream_t st, int copies = 1);
int resident_copies_active(int dim, int geom, int copies, int threads, size_t smem);  // 0: cannot launch
cudaError_t launch_tiled_sweep(int dim, int geom, Rep *reps, const Item *items, int nitems, int colour,
                               double *dEpart, long long *ipart, int threads, cudaStream_t st);
cudaError_t launch_tiled_measure(int dim, int geom, Rep *reps, const Item *items, int nitems,
                                 double *fpart, int threads, cudaStream_t st);
cudaError_t launch_tiled_finalize_dim(int dim, Rep *reps, const int *ids, int nrep, const int *item_off,
                                      double *dEpart, long long *ipart, const int *mitem_off, double *fpart,
                                      cudaStream_t st);
cudaError_t launch_init_state_dg(int dim, int geom, Rep *reps, const int *ids, int nrep, cudaStream_t st);
// reps[items[i].id]: quota = items[i].quota, u_stop = min(units_total, u + quota)
struct StopItem {
    int id;
    int pad;
    long long quota;
};
cudaError_t launch_set_stop(Rep *reps, const StopItem *items, int n, cudaStream_t st);
// load the engine's kernels on the current device ahead of their first launch
cudaError_t preload_kernels_main();
cudaError_t preload_kernels_cluster();
}  // namespace mcs
