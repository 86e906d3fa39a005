/*
 * mcs_oracle.c -- CPU restatement of mcsolver's compiled Monte Carlo solve
 * (isingLib.c / xyLib.c / heisenbergLib.c, function MCMainFunction).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA engine is
 * checked against; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg load it.  The product never links or calls it.
 *
 * It takes the same flattened arrays that MCMainFunction receives
 * (isingLib.c:277-335, heisenbergLib.c:504-583, xyLib.c:439-513) and returns the
 * same result values (isingLib.c:436-447, heisenbergLib.c:853-884,
 * xyLib.c:778-807).  The update and measurement arithmetic is restated in the
 * reference's own evaluation order, in double precision.
 *
 * Two random streams:
 *   mode 0 "reference": glibc rand() after srand(seed), random-site order, exactly
 *          as the reference consumes it (XY with the 15-bit rand() contract of
 *          the reference, see oracle/xy_shim.c).  In this mode the output is
 *          bit-identical to the reference library built in oracle/_ref; that is
 *          how the restatement is pinned.
 *   mode 2 "reference algorithm, SplitMix64": mode 0's algorithm and order of
 *          draws (random-site order, the reference's direction, acceptance and
 *          tie-break draws, RAND_MAX = 2^31 - 1) with a SplitMix64 generator
 *          (Steele, Lea and Flood, OOPSLA 2014; 31-bit outputs, state seeded
 *          from the seed) in place of glibc rand().  It separates the
 *          reference's algorithm from its random source: glibc rand() (an
 *          additive lagged-Fibonacci generator) and the 15-bit rand() of the XY
 *          library both shift low-temperature XY energies measurably.
 *   mode 1 "engine": the GPU engine's stream.  A Metropolis sweep visits the
 *          sites colour by colour (greedy colouring of the bond graph in site
 *          order; ascending site id within a colour) and draws its random words
 *          from Philox4x32-10 with the counter layout below.  The Wolff cluster,
 *          its direction and every bond coin are drawn from Philox too.  The
 *          arithmetic is the reference's; only site order and random source
 *          change.
 *
 * The "sweep index" of a site is its position in the concatenation of the
 * colour lists (colour 0 first, ascending site id inside a colour).  Every
 * counter below names sites by sweep index, so that a device that stores the
 * lattice in that order draws the same words.
 * Philox counter layout of the engine stream (key = seed lo/hi 32 bits):
 *   Metropolis, sweep t, colour c, k-th site of the colour:
 *       Ising       ctr = (k>>2, t_lo, t_hi, c), word k&3
 *       XY          ctr = (k>>1, t_lo, t_hi, c), words 2(k&1) (direction) and
 *                   2(k&1)+1 (accept)
 *       Heisenberg  ctr = (k,    t_lo, t_hi, c), words 0, 1 (direction), 2 (accept)
 *   Wolff cluster q: ctr = (0, q_lo, q_hi, 0x1000): seed = sites[(w0*N)>>32],
 *       w1/w2 direction, w3 cluster acceptance
 *   Wolff bond coin, cluster q, directed bond from sweep index a to b:
 *       ctr = (a, b, q_lo, 0x2000 ^ (q_hi << 16)), word 0
 *   Ising majority tie-break, measurement m, chosen site of sweep index a, slot s
 *       (0 = the site itself, 1+l = its l-th renormalised neighbour):
 *       ctr = (a, m_lo, m_hi, 0x3000 + (s>>2)), word s&3
 *   O(n) initial tilt (flunc) of the site of sweep index a: ctr = (a, 0, 0, 0x4000)
 *   random initial state (engine API option) of sweep index a: ctr = (a, 0, 0, 0x5000)
 *   uniform in [0,1): Ising/coins of Ising  U = w * 2^-32,
 *                     O(n)                  U = (w>>8) * 2^-24
 *   directions: XY  phi = 2*pi*U(w);  Heisenberg z = 2U(w0)-1, phi = 2*pi*U(w1)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "philox.h"

#define OR_PI 3.1415926535 /* the constant of heisenbergLib.c:6 */
#define OR_NSER 4
#define OR_TWO_PI 6.28318530717958647692528676655900577

typedef struct OrProblem {
    int32_t model;      /* 1 Ising, 2 XY, 3 Heisenberg */
    int32_t algorithm;  /* 0 Metropolis, 1 Wolff */
    int32_t N;          /* totOrbs */
    int32_t z;          /* maxNLinking */
    int64_t nthermal, nsweep, ninterval;
    const double *init_spin;     /* N */
    const double *init_D;        /* 3N, O(n) only */
    const int32_t *nlink;        /* N */
    const double *link_strength; /* N*z (Ising) or 9*N*z (O(n)) */
    const int32_t *linked_orb;   /* N*z, -1 padded */
    const int32_t *circuits;     /* 3*ncirc */
    const int32_t *corr_pair;    /* 2*nlat */
    const int32_t *group_list;   /* n_group*max_group, -1 padded */
    const int32_t *r_orb;        /* n_rorb */
    const int32_t *r_cluster;    /* n_rorb*n_in_cluster */
    const int32_t *r_link;       /* n_rorb*z */
    double flunc, h;
    int32_t ncirc, nlat, n_group, max_group;
    int32_t n_rorb, n_in_cluster, ignore_offdiag, pad_;
} OrProblem;

typedef struct OrRun {
    int32_t mode;          /* 0 reference stream, 1 engine stream */
    int32_t use_spins_in;  /* start from spins_io (engine mode) */
    uint64_t seed;
    int64_t sweep_offset;  /* engine: index of the first sweep / cluster */
    int64_t meas_offset;   /* engine: index of the first measurement */
    double *spins_io;      /* 3N: optional initial state in, final state out */
    double *series;        /* nsweep*OR_NSER, optional */
    double *result;        /* >= 29 + (G+1)^2 + (G+1) */
    int64_t *stats;        /* [0] accepted single-site moves or clusters,
                              [1] flipped sites (Wolff), [2] clusters built,
                              [3] Metropolis site visits */
    int32_t result_cap;
    int32_t pad_;
} OrRun;

/* ------------------------------------------------------------------ RNG */
typedef struct Rng {
    int mode;
    int rand15;      /* XY reference contract: 15-bit rand() */
    uint32_t key[2];
    uint64_t sm;     /* mode 2: SplitMix64 state */
} Rng;

static int splitmix31(Rng *g)
{
    uint64_t z = (g->sm += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (int)(z >> 33);
}
static double rmax(const Rng *g) { return g->rand15 ? 32767.0 : 2147483647.0; }
static int rnd(const Rng *g)
{
    if (g->mode == 2) return splitmix31((Rng *)g);
    return g->rand15 ? (rand() & 0x7fff) : rand();
}
static void ref_seed(Rng *g, uint64_t seed)
{
    if (g->mode == 2) {
        g->rand15 = 0;
        g->sm = 0x6A09E667F3BCC909ULL ^ (seed * 0x9E3779B97F4A7C15ULL);
    } else if (g->mode == 0) {
        srand((unsigned)seed);
    }
}
/* rand()/(double)RAND_MAX as written throughout the reference */
static double ref_u(const Rng *g) { return (double)rnd(g) / rmax(g); }

static void phil(const Rng *g, uint32_t c0, uint64_t t, uint32_t c3, uint32_t out[4])
{
    uint32_t c[4] = {c0, (uint32_t)t, (uint32_t)(t >> 32), c3};
    or_philox4x32_10(c, g->key, out);
}
static uint32_t coin(const Rng *g, uint32_t a, uint32_t b, uint64_t q)
{
    uint32_t c[4] = {a, b, (uint32_t)q, 0x2000u ^ ((uint32_t)(q >> 32) << 16)}, out[4];
    or_philox4x32_10(c, g->key, out);
    return out[0];
}
static double u32d(uint32_t w) { return (double)w * (1.0 / 4294967296.0); }
static double u24d(uint32_t w) { return (double)(w >> 8) * (1.0 / 16777216.0); }

/* reference seed selection: isingLib.c:239-241, heisenbergLib.c:444-446 */
static long ref_seed_site(const Rng *g, int N)
{
    if (g->rand15) { /* xyLib.c:384, int arithmetic, 15-bit rand */
        int r1 = rnd(g);
        int r2 = rnd(g);
        return (r1 * 32767 + r2) % N;
    }
    unsigned long long r1 = (unsigned long long)rnd(g);
    unsigned long long r2 = (unsigned long long)rnd(g);
    return (long)((r1 * 2147483647ULL + r2) % (unsigned long long)N);
}

/* ------------------------------------------------------------ colouring */
/* Greedy colouring in site order over the undirected bond graph (self links
 * and -1 padding ignored).  Returns the number of colours. */
static int greedy_colour(const OrProblem *p, int *colour)
{
    int N = p->N, z = p->z;
    /* build undirected adjacency via CSR */
    int *deg = calloc((size_t)N + 1, sizeof(int));
    for (int i = 0; i < N; i++)
        for (int l = 0; l < p->nlink[i]; l++) {
            int j = p->linked_orb[(size_t)i * z + l];
            if (j < 0 || j == i) continue;
            deg[i]++; deg[j]++;
        }
    int *off = malloc(((size_t)N + 1) * sizeof(int));
    off[0] = 0;
    for (int i = 0; i < N; i++) off[i + 1] = off[i] + deg[i];
    int *adj = malloc((size_t)off[N] * sizeof(int) + 1);
    int *fill = calloc((size_t)N, sizeof(int));
    for (int i = 0; i < N; i++)
        for (int l = 0; l < p->nlink[i]; l++) {
            int j = p->linked_orb[(size_t)i * z + l];
            if (j < 0 || j == i) continue;
            adj[off[i] + fill[i]++] = j;
            adj[off[j] + fill[j]++] = i;
        }
    int ncol = 0;
    int maxdeg = 0;
    for (int i = 0; i < N; i++) if (deg[i] > maxdeg) maxdeg = deg[i];
    char *used = calloc((size_t)maxdeg + 2, 1);
    for (int i = 0; i < N; i++) {
        memset(used, 0, (size_t)maxdeg + 2);
        for (int k = off[i]; k < off[i + 1]; k++) {
            int j = adj[k];
            if (j < i && colour[j] <= maxdeg) used[colour[j]] = 1;
        }
        int c = 0;
        while (used[c]) c++;
        colour[i] = c;
        if (c + 1 > ncol) ncol = c + 1;
    }
    free(used); free(fill); free(adj); free(off); free(deg);
    return ncol;
}

typedef struct Sweep {
    int ncol;
    int *start;  /* ncol+1 */
    int *sites;  /* N: sweep index -> site */
    int *pos;    /* N: site -> sweep index */
} Sweep;

static void sweep_build(const OrProblem *p, Sweep *s)
{
    int N = p->N;
    int *colour = malloc((size_t)N * sizeof(int));
    s->ncol = greedy_colour(p, colour);
    s->start = calloc((size_t)s->ncol + 1, sizeof(int));
    for (int i = 0; i < N; i++) s->start[colour[i] + 1]++;
    for (int c = 0; c < s->ncol; c++) s->start[c + 1] += s->start[c];
    int *pos = malloc((size_t)s->ncol * sizeof(int));
    for (int c = 0; c < s->ncol; c++) pos[c] = s->start[c];
    s->sites = malloc((size_t)N * sizeof(int));
    for (int i = 0; i < N; i++) s->sites[pos[colour[i]]++] = i;
    s->pos = malloc((size_t)N * sizeof(int));
    for (int k = 0; k < N; k++) s->pos[s->sites[k]] = k;
    free(pos); free(colour);
}
static void sweep_free(Sweep *s) { free(s->start); free(s->sites); free(s->pos); }

static int64_t sweeps_per(int64_t tau, int N) { return (tau + N - 1) / N; }

/* ================================================================ ISING */
typedef struct IsingState {
    const OrProblem *p;
    Rng g;
    double *s;      /* spins, +-S */
    char *inblock;
    int *block, *buffer;
    int *chosen;    /* chosen[i] = index in r_orb + 1, or 0 */
    double energy, totspin;
    int64_t *stats;
    int64_t meas_index; /* engine: measurement counter for tie-breaks */
    const Sweep *sw;    /* engine: colour lists and sweep indices */
} IsingState;

/* getCorrEnergy, isingLib.c:121-127 */
static double is_corr(const IsingState *S, int i)
{
    const OrProblem *p = S->p;
    double corr = 0;
    for (int l = 0; l < p->nlink[i]; l++) {
        int j = p->linked_orb[(size_t)i * p->z + l];
        corr += (p->link_strength[(size_t)i * p->z + l]) * (S->s[i]) * (S->s[j]);
    }
    return corr;
}

/* localUpdate body for a given site and uniform source; isingLib.c:242-252 */
static void is_metropolis_site(IsingState *S, int i, int engine, uint32_t w)
{
    const OrProblem *p = S->p;
    double corr = 2 * (is_corr(S, i) - p->h * S->s[i]);
    int acc;
    if (corr >= 0) acc = 1;
    else acc = engine ? (exp(corr) > u32d(w)) : (exp(corr) > ref_u(&S->g));
    if (acc) {
        S->s[i] *= -1;
        S->totspin += (S->s[i] * 2);
        S->energy -= corr;
        S->stats[0]++;
    }
}

/* expandBlock + blockUpdate, isingLib.c:165-236 */
static void is_wolff(IsingState *S, uint64_t q)
{
    const OrProblem *p = S->p;
    int N = p->N, z = p->z;
    int engine = S->g.mode == 1;
    uint32_t w[4] = {0, 0, 0, 0};
    for (int i = 0; i < N; i++) S->inblock[i] = 0;
    long seed;
    if (engine) {
        phil(&S->g, 0, q, 0x1000, w);
        seed = S->sw->sites[(((uint64_t)w[0] * (uint64_t)N) >> 32)];
    } else {
        seed = ref_seed_site(&S->g, N);
    }
    S->block[0] = (int)seed;
    S->buffer[0] = (int)seed;
    S->inblock[seed] = 1;
    int begin = 0, end = 0, blen = 1;
    while (begin <= end) {
        int out = S->buffer[begin++];
        for (int l = 0; l < p->nlink[out]; l++) {
            int j = p->linked_orb[(size_t)out * z + l];
            if (S->inblock[j] == 0) {
                double corr = (p->link_strength[(size_t)out * z + l]) * (S->s[out]) * (S->s[j]);
                if (corr < 0) {
                    double u = engine ? u32d(coin(&S->g, (uint32_t)S->sw->pos[out], (uint32_t)S->sw->pos[j], q))
                                      : ref_u(&S->g);
                    if ((1 - exp(2 * corr)) > u) {
                        S->block[blen++] = j;
                        S->inblock[j] = 1;
                        S->buffer[++end] = j;
                    }
                }
            }
        }
    }
    S->stats[2]++;
    double tot = 0;
    for (int i = 0; i < blen; i++) tot += 2 * p->h * S->s[S->block[i]];
    int acc;
    if (tot <= 0) acc = 1;
    else acc = engine ? (exp(-tot) > u32d(w[3])) : (exp(-tot) > ref_u(&S->g));
    if (acc) {
        for (int i = 0; i < blen; i++) {
            int b = S->block[i];
            S->s[b] *= -1;
            if (b < N - 1) S->totspin += (S->s[b] * 2);
        }
        S->energy = 0.;
        for (int i = 0; i < N; i++) S->energy += is_corr(S, i) / 2 - p->h * S->s[i];
        S->stats[0]++;
        S->stats[1] += blen;
    }
}

/* getMajoritySpin, isingLib.c:133-150 (tie -> random sign) */
static double is_majority(IsingState *S, int x, int engine, const uint32_t *tw, int slot)
{
    const OrProblem *p = S->p;
    double avg = 0.0;
    int r = S->chosen[x] - 1;
    if (r >= 0)
        for (int k = 0; k < p->n_in_cluster; k++) avg += S->s[p->r_cluster[(size_t)r * p->n_in_cluster + k]];
    if (avg > 0) return fabs(S->s[x]);
    if (avg < 0) return -fabs(S->s[x]);
    double u = engine ? u32d(tw[slot & 3]) : ref_u(&S->g);
    return (u > 0.5) ? fabs(S->s[x]) : -fabs(S->s[x]);
}

/* getCorrEnergy_rnorm, isingLib.c:152-163 */
static double is_corr_rnorm(IsingState *S, int j)
{
    const OrProblem *p = S->p;
    int engine = S->g.mode == 1;
    int r = S->chosen[j] - 1;
    uint32_t tw[4] = {0, 0, 0, 0};
    uint32_t sj = engine ? (uint32_t)S->sw->pos[j] : 0;
    if (engine) phil(&S->g, sj, (uint64_t)S->meas_index, 0x3000, tw);
    double corr = 0;
    double a = is_majority(S, j, engine, tw, 0);
    for (int l = 0; l < p->nlink[j]; l++) {
        int slot = 1 + l;
        if (engine && (slot & 3) == 0) phil(&S->g, sj, (uint64_t)S->meas_index, 0x3000u + (uint32_t)(slot >> 2), tw);
        int t = p->r_link[(size_t)r * p->z + l];
        if (t < 0) continue; /* the reference reads lattice[-1] here (undefined); skipped */
        double b = is_majority(S, t, engine, tw, slot);
        corr += (p->link_strength[(size_t)j * p->z + l]) * a * b;
    }
    return corr;
}

static int ising_run(const OrProblem *p, OrRun *run)
{
    int N = p->N;
    IsingState S;
    memset(&S, 0, sizeof S);
    S.p = p;
    S.g.mode = run->mode;
    S.g.rand15 = 0;
    S.g.key[0] = (uint32_t)run->seed;
    S.g.key[1] = (uint32_t)(run->seed >> 32);
    S.stats = run->stats;
    ref_seed(&S.g, run->seed);
    S.s = malloc((size_t)N * sizeof(double));
    S.inblock = calloc((size_t)N, 1);
    S.block = malloc((size_t)N * sizeof(int));
    S.buffer = malloc((size_t)N * sizeof(int));
    S.chosen = calloc((size_t)N, sizeof(int));
    for (int i = 0; i < p->n_rorb; i++) S.chosen[p->r_orb[i]] = i + 1;
    for (int i = 0; i < N; i++) S.s[i] = p->init_spin[i];
    if (run->use_spins_in && run->spins_io)
        for (int i = 0; i < N; i++) S.s[i] = run->spins_io[3 * i];

    /* isingLib.c:348-350: totSpin starts as the sum of the first ninterval spins */
    S.energy = 0;
    S.totspin = 0;
    int64_t nfirst = p->ninterval < N ? p->ninterval : N;
    for (int64_t i = 0; i < nfirst; i++) S.totspin += p->init_spin[i];

    Sweep sw = {0, NULL, NULL, NULL};
    int engine = run->mode == 1;
    if (engine) sweep_build(p, &sw);
    S.sw = &sw;
    int64_t t = run->sweep_offset; /* engine sweep / cluster counter */

    /* one reference "update" or one engine unit of ninterval updates */
#define IS_UNIT_REF() do { if (p->algorithm == 1) is_wolff(&S, 0); else { long i_ = ref_seed_site(&S.g, N); is_metropolis_site(&S, (int)i_, 0, 0); run->stats[3]++; } } while (0)
    if (!engine) {
        for (int64_t i = 0; i < p->nthermal * p->ninterval; i++) IS_UNIT_REF();
    } else {
        int64_t units = p->algorithm == 1 ? p->nthermal * p->ninterval : p->nthermal * sweeps_per(p->ninterval, N);
        for (int64_t u = 0; u < units; u++) {
            if (p->algorithm == 1) is_wolff(&S, (uint64_t)t++);
            else {
                for (int c = 0; c < sw.ncol; c++) {
                    uint32_t w[4];
                    for (int k = sw.start[c]; k < sw.start[c + 1]; k++) {
                        int kk = k - sw.start[c];
                        if ((kk & 3) == 0) phil(&S.g, (uint32_t)(kk >> 2), (uint64_t)t, (uint32_t)c, w);
                        is_metropolis_site(&S, sw.sites[k], 1, w[kk & 3]);
                        run->stats[3]++;
                    }
                }
                t++;
            }
        }
    }

    double spin_i = 0, spin_j = 0, spin_ij = 0;
    double totEnergy = 0, totEnergy_r = 0, E2 = 0, E2_r = 0;
    S.energy = 0; /* isingLib.c:359 */
    double M = 0, M2 = 0, M4 = 0, M_tmp = 0, MdotM = 0, M_tot = 0;
    double spin_tot = 0;
    int nlat = p->nlat;
    for (int64_t m = 0; m < p->nsweep; m++) {
        if (!engine) {
            for (int64_t j = 0; j < p->ninterval; j++) IS_UNIT_REF();
        } else {
            int64_t units = p->algorithm == 1 ? p->ninterval : sweeps_per(p->ninterval, N);
            for (int64_t u = 0; u < units; u++) {
                if (p->algorithm == 1) is_wolff(&S, (uint64_t)t++);
                else {
                    for (int c = 0; c < sw.ncol; c++) {
                        uint32_t w[4];
                        for (int k = sw.start[c]; k < sw.start[c + 1]; k++) {
                            int kk = k - sw.start[c];
                            if ((kk & 3) == 0) phil(&S.g, (uint32_t)(kk >> 2), (uint64_t)t, (uint32_t)c, w);
                            is_metropolis_site(&S, sw.sites[k], 1, w[kk & 3]);
                            run->stats[3]++;
                        }
                    }
                    t++;
                }
            }
        }
        S.meas_index = run->meas_offset + m;
        double energy_rnorm = 0;
        for (int j = 0; j < N; j++)
            if (S.chosen[j] > 0) energy_rnorm += is_corr_rnorm(&S, j) / 2 - p->h * S.s[j];
        double si_avg = 0, sj_avg = 0, corrAvg = 0.0;
        for (int j = 0; j < nlat; j++) {
            double a = S.s[p->corr_pair[2 * j]];
            double b = S.s[p->corr_pair[2 * j + 1]];
            si_avg += a;
            sj_avg += b;
            corrAvg += a * b;
        }
        spin_tot += S.totspin;
        M = si_avg / nlat;
        M2 += M * M;
        M4 += M * M * M * M;
        M_tot += M;
        MdotM += M_tmp * M;
        M_tmp = M;
        spin_i += fabs(si_avg) / nlat;
        spin_j += fabs(sj_avg) / nlat;
        spin_ij += corrAvg / nlat;
        double e_avg = S.energy / N, e_avg_r = energy_rnorm / p->n_rorb;
        totEnergy += e_avg;
        totEnergy_r += e_avg_r;
        E2 += e_avg * e_avg;
        E2_r += e_avg_r * e_avg_r;
        if (run->series) {
            double *q = run->series + (size_t)m * OR_NSER;
            q[0] = e_avg; q[1] = M; q[2] = e_avg_r; q[3] = corrAvg / nlat;
        }
    }
    double ns = (double)p->nsweep;
    double U4 = (M2 / ns) * (M2 / ns) / (M4 / ns);
    double autoCorr = (MdotM / ns - (M_tot / ns) * (M_tot / ns));
    double *r = run->result;
    r[0] = spin_i / ns; r[1] = spin_j / ns; r[2] = spin_ij / ns; r[3] = autoCorr;
    r[4] = totEnergy / ns; r[5] = E2 / ns; r[6] = totEnergy_r / ns; r[7] = E2_r / ns;
    r[8] = U4; r[9] = spin_tot / ns / nlat; r[10] = 0.0;
    if (run->spins_io)
        for (int i = 0; i < N; i++) { run->spins_io[3 * i] = S.s[i]; run->spins_io[3 * i + 1] = 0; run->spins_io[3 * i + 2] = 0; }
    if (engine) sweep_free(&sw);
    free(S.s); free(S.inblock); free(S.block); free(S.buffer); free(S.chosen);
#undef IS_UNIT_REF
    return 0;
}

/* ================================================================= O(n) */
typedef struct V3 { double x, y, z; } V3;

typedef struct OnState {
    const OrProblem *p;
    int dim;       /* 2 XY, 3 Heisenberg */
    Rng g;
    V3 *s, *trans, *perp;
    double *sdotn;
    double *len;   /* Vec.len = |initSpin| (heisenbergLib.c:160) */
    char *inblock, *projected;
    int *block, *buffer;
    int *chosen;
    double *J;     /* per link 9 comps, XY uses xx,yy,xy,yx */
    double energy;
    V3 totspin;
    int64_t *stats;
    const Sweep *sw;
} OnState;

static double v_dot(int dim, V3 a, V3 b)
{
    if (dim == 3) return a.x * b.x + a.y * b.y + a.z * b.z;
    return a.x * b.x + a.y * b.y;
}
static void v_normalize(int dim, V3 *v)
{
    double len = dim == 3 ? sqrt(v->x * v->x + v->y * v->y + v->z * v->z) : sqrt(v->x * v->x + v->y * v->y);
    if (len < 1e-5) return;
    v->x /= len; v->y /= len;
    if (dim == 3) v->z /= len;
}

/* diagonalDot / diagonalDot_simple: heisenbergLib.c:77-93, xyLib.c:59-68.
 * J layout per link: xx,yy,zz,xy,xz,yz,yx,zx,zy (Lattice.py:136). */
static double v_jdot(const OnState *S, V3 a, V3 b, const double *J)
{
    if (S->dim == 3) {
        if (S->p->ignore_offdiag > 0)
            return a.x * b.x * J[0] + a.y * b.y * J[1] + a.z * b.z * J[2];
        return a.x * b.x * J[0] + a.y * b.y * J[1] + a.z * b.z * J[2] +
               a.x * b.y * J[3] + a.x * b.z * J[4] + a.y * b.z * J[5] +
               a.y * b.x * J[6] + a.z * b.x * J[7] + a.z * b.y * J[8];
    }
    if (S->p->ignore_offdiag > 0)
        return a.x * b.x * J[0] + a.y * b.y * J[1];
    return a.x * b.x * J[0] + a.y * b.y * J[1] + a.x * b.y * J[3] + a.y * b.x * J[6];
}

static const double *on_J(const OnState *S, int i, int l) { return S->p->link_strength + ((size_t)i * S->p->z + l) * 9; }

/* generateRandomVec: heisenbergLib.c:95-112, xyLib.c:73-88 (cube rejection) */
static V3 on_ref_randvec(OnState *S)
{
    for (;;) {
        double x = ref_u(&S->g) - 0.5;
        double y = ref_u(&S->g) - 0.5;
        double z = 0, len2;
        if (S->dim == 3) { z = ref_u(&S->g) - 0.5; len2 = (x * x + y * y + z * z); }
        else len2 = (x * x + y * y);
        if (len2 > 0.25) continue;
        double len = sqrt(len2);
        V3 d = {x / len, y / len, S->dim == 3 ? z / len : 0};
        return d;
    }
}
/* engine direction from two words */
static V3 on_eng_dir(int dim, uint32_t w0, uint32_t w1)
{
    V3 d;
    if (dim == 2) {
        double phi = OR_TWO_PI * u24d(w0);
        d.x = cos(phi); d.y = sin(phi); d.z = 0;
    } else {
        double zz = 2.0 * u24d(w0) - 1.0;
        double phi = OR_TWO_PI * u24d(w1);
        double rho = sqrt(fmax(0.0, 1.0 - zz * zz));
        d.x = rho * cos(phi); d.y = rho * sin(phi); d.z = zz;
    }
    return d;
}

/* getCorrEnergy */
static double on_corr(const OnState *S, int i)
{
    double corr = 0;
    for (int l = 0; l < S->p->nlink[i]; l++) {
        int j = S->p->linked_orb[(size_t)i * S->p->z + l];
        corr += v_jdot(S, S->s[i], S->s[j], on_J(S, i, l));
    }
    return corr;
}
/* getOnsiteEnergy: heisenbergLib.c:243-248, xyLib.c:207-211 */
static double on_onsite(const OnState *S, int i, V3 v)
{
    const double *D = S->p->init_D + 3 * (size_t)i;
    if (S->dim == 3)
        return D[0] * v.x * v.x + D[1] * v.y * v.y + D[2] * v.z * v.z - S->p->h * v.z;
    return D[0] * v.x * v.x + D[1] * v.y * v.y - S->p->h * v.x;
}
/* getDeltaOnsiteEnergy: heisenbergLib.c:299-308, xyLib.c:247-254 */
static double on_donsite(const OnState *S, int i)
{
    const double *D = S->p->init_D + 3 * (size_t)i;
    V3 s = S->s[i], t = S->trans[i];
    double s1x = s.x + t.x, s1y = s.y + t.y, s1z = s.z + t.z;
    if (S->dim == 3)
        return D[0] * (s1x * s1x - s.x * s.x) + D[1] * (s1y * s1y - s.y * s.y) +
               D[2] * (s1z * s1z - s.z * s.z) - S->p->h * t.z;
    return D[0] * (s1x * s1x - s.x * s.x) + D[1] * (s1y * s1y - s.y * s.y) - S->p->h * t.x;
}
static double on_full_energy(const OnState *S)
{
    double e = 0.;
    for (int i = 0; i < S->p->N; i++) e += on_corr(S, i);
    e /= 2;
    for (int i = 0; i < S->p->N; i++) e += on_onsite(S, i, S->s[i]);
    return e;
}
static void v_add(int dim, V3 *a, V3 b) { a->x += b.x; a->y += b.y; if (dim == 3) a->z += b.z; }

/* localUpdate: heisenbergLib.c:441-473, xyLib.c:382-409 */
static void on_metropolis_site(OnState *S, int i, V3 r, int engine, uint32_t wacc)
{
    double s1n = -2 * v_dot(S->dim, S->s[i], r);
    V3 t = r;
    t.x *= s1n; t.y *= s1n; if (S->dim == 3) t.z *= s1n;
    S->trans[i] = t;
    double corr = 0;
    for (int l = 0; l < S->p->nlink[i]; l++) {
        int j = S->p->linked_orb[(size_t)i * S->p->z + l];
        corr += v_jdot(S, t, S->s[j], on_J(S, i, l));
    }
    corr += on_donsite(S, i);
    int acc;
    if (corr <= 0) acc = 1;
    else acc = engine ? (exp(-corr) > u24d(wacc)) : (exp(-corr) > ref_u(&S->g));
    if (acc) {
        v_add(S->dim, &S->totspin, t);
        v_add(S->dim, &S->s[i], t);
        S->energy += corr;
        S->stats[0]++;
    }
}

static void on_project(OnState *S, int i, V3 r)
{
    if (S->projected[i]) return;
    S->sdotn[i] = -v_dot(S->dim, S->s[i], r);
    V3 t = r;
    t.x *= S->sdotn[i]; t.y *= S->sdotn[i]; if (S->dim == 3) t.z *= S->sdotn[i];
    S->trans[i] = t;
    V3 pp = S->s[i];
    v_add(S->dim, &pp, t);
    S->perp[i] = pp;
    S->projected[i] = 1;
}

/* expandBlock + blockUpdate: heisenbergLib.c:310-439, xyLib.c:256-380 */
static void on_wolff(OnState *S, uint64_t q)
{
    const OrProblem *p = S->p;
    int N = p->N, z = p->z, dim = S->dim;
    int engine = S->g.mode == 1;
    for (int i = 0; i < N; i++) { S->projected[i] = 0; S->inblock[i] = 0; }
    uint32_t w[4] = {0, 0, 0, 0};
    long seed;
    V3 r;
    if (engine) {
        phil(&S->g, 0, q, 0x1000, w);
        seed = S->sw->sites[(((uint64_t)w[0] * (uint64_t)N) >> 32)];
        r = on_eng_dir(dim, w[1], w[2]);
    } else {
        seed = ref_seed_site(&S->g, N);
        r = on_ref_randvec(S);
    }
    S->block[0] = (int)seed;
    S->buffer[0] = (int)seed;
    S->inblock[seed] = 1;
    int begin = 0, end = 0, blen = 1;
    while (begin <= end) {
        int out = S->buffer[begin++];
        on_project(S, out, r);
        for (int l = 0; l < p->nlink[out]; l++) {
            int j = p->linked_orb[(size_t)out * z + l];
            if (S->inblock[j] == 0) {
                on_project(S, j, r);
                double corr = 2 * S->sdotn[out] * S->sdotn[j] * v_jdot(S, r, r, on_J(S, out, l));
                if (corr < 0) {
                    double u = engine ? u24d(coin(&S->g, (uint32_t)S->sw->pos[out], (uint32_t)S->sw->pos[j], q))
                                      : ref_u(&S->g);
                    if ((1 - exp(corr)) > u) {
                        S->block[blen++] = j;
                        S->inblock[j] = 1;
                        S->buffer[++end] = j;
                    }
                }
            }
        }
    }
    S->stats[2]++;
    double tot = 0;
    for (int b = 0; b < blen; b++) {
        int i = S->block[b];
        for (int l = 0; l < p->nlink[i]; l++) {
            int j = p->linked_orb[(size_t)i * z + l];
            const double *J = on_J(S, i, l);
            double src = S->sdotn[i] * v_jdot(S, r, S->perp[j], J);
            tot += src;
            if (S->inblock[j] > 0) tot += S->sdotn[j] * v_jdot(S, S->perp[i], r, J);
            else tot += src;
        }
    }
    for (int b = 0; b < blen; b++) tot += on_donsite(S, S->block[b]);
    int acc;
    if (tot <= 0) acc = 1;
    else acc = engine ? (exp(-tot) > u24d(w[3])) : (exp(-tot) > ref_u(&S->g));
    if (acc) {
        for (int b = 0; b < blen; b++) {
            int i = S->block[b];
            V3 t = S->trans[i];
            t.x *= 2; t.y *= 2; if (dim == 3) t.z *= 2;
            v_add(dim, &S->s[i], t);
            v_add(dim, &S->totspin, t);
        }
        S->energy = on_full_energy(S);
        S->stats[0]++;
        S->stats[1] += blen;
    }
}

/* getMajoritySpin: heisenbergLib.c:250-262, xyLib.c:213-225 */
static V3 on_majority(const OnState *S, int x)
{
    V3 a = {0, 0, 0};
    int r = S->chosen[x] - 1;
    if (r >= 0)
        for (int k = 0; k < S->p->n_in_cluster; k++) v_add(S->dim, &a, S->s[S->p->r_cluster[(size_t)r * S->p->n_in_cluster + k]]);
    v_normalize(S->dim, &a);
    double Sx = S->p->init_spin[x];
    a.x *= Sx; a.y *= Sx; if (S->dim == 3) a.z *= Sx;
    return a;
}
/* getCorrEnergy_rnorm */
static double on_corr_rnorm(const OnState *S, int j)
{
    double corr = 0;
    V3 a = on_majority(S, j);
    int r = S->chosen[j] - 1;
    for (int l = 0; l < S->p->nlink[j]; l++) {
        int t = S->p->r_link[(size_t)r * S->p->z + l];
        if (t < 0) continue; /* reference reads lattice[-1] (undefined); skipped */
        V3 b = on_majority(S, t);
        corr += v_jdot(S, a, b, on_J(S, j, l));
    }
    return corr;
}

/* calcSignedArea: heisenbergLib.c:114-127 (atan, not atan2; +-pi near 0) */
static double on_signed_area(const OnState *S, int i1, int i2, int i3)
{
    V3 s1 = S->s[i1], s2 = S->s[i2], s3 = S->s[i3];
    double l1 = S->len[i1], l2 = S->len[i2], l3 = S->len[i3];
    double s1s2 = v_dot(3, s1, s2) / l1 / l2;
    double s2s3 = v_dot(3, s2, s3) / l2 / l3;
    double s3s1 = v_dot(3, s3, s1) / l3 / l1;
    V3 c;
    c.x = s2.y * s3.z - s2.z * s3.y;
    c.y = s2.z * s3.x - s2.x * s3.z;
    c.z = s2.x * s3.y - s2.y * s3.x;
    double re = 1 + s1s2 + s2s3 + s3s1;
    double im = v_dot(3, s1, c) / l1 / l2 / l3;
    if (fabs(re) < 1e-6) {
        if (im > 0) return OR_PI;
        return -OR_PI;
    }
    return 2 * atan(im / re);
}

static void on_unit(OnState *S, Sweep *sw, int64_t *t)
{
    const OrProblem *p = S->p;
    int N = p->N;
    if (S->g.mode != 1) {
        if (p->algorithm == 1) on_wolff(S, 0);
        else {
            long i = ref_seed_site(&S->g, N);
            V3 r = on_ref_randvec(S);
            on_metropolis_site(S, (int)i, r, 0, 0);
            S->stats[3]++;
        }
        return;
    }
    if (p->algorithm == 1) { on_wolff(S, (uint64_t)(*t)++); return; }
    for (int c = 0; c < sw->ncol; c++) {
        for (int k = sw->start[c]; k < sw->start[c + 1]; k++) {
            uint32_t w[4];
            const uint32_t kk = (uint32_t)(k - sw->start[c]);
            if (S->dim == 2) {
                /* XY: sites kk and kk^1 share one block, even kk words 0-1, odd kk words 2-3 */
                phil(&S->g, kk >> 1, (uint64_t)*t, (uint32_t)c, w);
                if (kk & 1u) { w[0] = w[2]; w[1] = w[3]; }
            } else {
                phil(&S->g, kk, (uint64_t)*t, (uint32_t)c, w);
            }
            V3 r = on_eng_dir(S->dim, w[0], w[1]);
            on_metropolis_site(S, sw->sites[k], r, 1, S->dim == 3 ? w[2] : w[1]);
            S->stats[3]++;
        }
    }
    (*t)++;
}

static int on_run(const OrProblem *p, OrRun *run)
{
    int N = p->N, dim = p->model == 3 ? 3 : 2;
    OnState S;
    memset(&S, 0, sizeof S);
    S.p = p;
    S.dim = dim;
    S.g.mode = run->mode;
    S.g.rand15 = (dim == 2);
    S.g.key[0] = (uint32_t)run->seed;
    S.g.key[1] = (uint32_t)(run->seed >> 32);
    S.stats = run->stats;
    ref_seed(&S.g, run->seed);
    S.s = calloc((size_t)N, sizeof(V3));
    S.trans = calloc((size_t)N, sizeof(V3));
    S.perp = calloc((size_t)N, sizeof(V3));
    S.sdotn = calloc((size_t)N, sizeof(double));
    S.len = calloc((size_t)N, sizeof(double));
    S.inblock = calloc((size_t)N, 1);
    S.projected = calloc((size_t)N, 1);
    S.block = malloc((size_t)N * sizeof(int));
    S.buffer = malloc((size_t)N * sizeof(int));
    S.chosen = calloc((size_t)N, sizeof(int));
    for (int i = 0; i < p->n_rorb; i++) S.chosen[p->r_orb[i]] = i + 1;
    Sweep sw = {0, NULL, NULL, NULL};
    if (run->mode == 1) sweep_build(p, &sw);
    S.sw = &sw;

    /* establishLattice: heisenbergLib.c:153-220, xyLib.c:116-165 */
    for (int i = 0; i < N; i++) {
        double S0 = p->init_spin[i];
        V3 v = {S0, 0, 0};
        S.len[i] = fabs(S0);
        V3 fl;
        if (run->mode != 1) fl = on_ref_randvec(&S);
        else {
            uint32_t w[4];
            phil(&S.g, (uint32_t)sw.pos[i], 0, 0x4000, w);
            fl = on_eng_dir(dim, w[0], w[1]);
        }
        fl.x *= p->flunc; fl.y *= p->flunc; if (dim == 3) fl.z *= p->flunc;
        v_add(dim, &v, fl);
        v_normalize(dim, &v);
        double a = fabs(S0);
        v.x *= a; v.y *= a; if (dim == 3) v.z *= a;
        S.s[i] = v;
    }
    if (run->use_spins_in && run->spins_io)
        for (int i = 0; i < N; i++) {
            S.s[i].x = run->spins_io[3 * i];
            S.s[i].y = run->spins_io[3 * i + 1];
            S.s[i].z = dim == 3 ? run->spins_io[3 * i + 2] : 0;
        }

    S.energy = on_full_energy(&S);
    S.totspin.x = S.totspin.y = S.totspin.z = 0;
    for (int i = 0; i < N; i++) v_add(dim, &S.totspin, S.s[i]);

    int64_t t = run->sweep_offset;

    if (run->mode != 1) {
        for (int64_t i = 0; i < p->nthermal * p->ninterval; i++) on_unit(&S, &sw, &t);
    } else {
        int64_t units = p->algorithm == 1 ? p->nthermal * p->ninterval : p->nthermal * sweeps_per(p->ninterval, N);
        for (int64_t u = 0; u < units; u++) on_unit(&S, &sw, &t);
    }

    V3 spin_i = {0, 0, 0}, spin_j = {0, 0, 0}, spin_i_r = {0, 0, 0}, spin_j_r = {0, 0, 0};
    double spin_ij = 0, spin_ij_r = 0;
    double totEnergy = 0, totEnergy_r = 0, E2 = 0, E2_r = 0;
    double M = 0, M2 = 0, M4 = 0, M_tmp = 0, MdotM = 0, M_tot = 0;
    double topo = 0;
    double spin_i_z = 0, spin_j_z = 0, spin_tot_z = 0, spin_i_h = 0, spin_j_h = 0, spin_tot_h = 0;
    int G = p->n_group;
    double *sds = calloc((size_t)(G + 1) * (G + 1), sizeof(double));
    double *s4 = calloc((size_t)G + 1, sizeof(double));
    V3 *gsum = calloc((size_t)G + 1, sizeof(V3));
    double nlat = (double)p->nlat;
    for (int64_t m = 0; m < p->nsweep; m++) {
        if (run->mode != 1) {
            for (int64_t j = 0; j < p->ninterval; j++) on_unit(&S, &sw, &t);
        } else {
            int64_t units = p->algorithm == 1 ? p->ninterval : sweeps_per(p->ninterval, N);
            for (int64_t u = 0; u < units; u++) on_unit(&S, &sw, &t);
        }
        V3 dir = S.totspin;
        v_normalize(dim, &dir);
        V3 si = {0, 0, 0}, sj = {0, 0, 0};
        double sij = 0.0, siz = 0, sjz = 0, sih = 0, sjh = 0;
        for (int j = 0; j < p->nlat; j++) {
            V3 a = S.s[p->corr_pair[2 * j]], b = S.s[p->corr_pair[2 * j + 1]];
            v_add(dim, &si, a);
            v_add(dim, &sj, b);
            sij += v_dot(dim, a, b);
            siz += v_dot(dim, dir, a);
            sjz += v_dot(dim, dir, b);
            if (dim == 3) { sih += a.z; sjh += b.z; }
            else { sih += a.x; sjh += b.x; }
        }
        if (dim == 3) {
            double ql = 0;
            for (int c = 0; c < p->ncirc; c++)
                ql += on_signed_area(&S, p->circuits[3 * c], p->circuits[3 * c + 1], p->circuits[3 * c + 2]);
            topo += ql / OR_PI / 4;
        }
        spin_i_z += siz / nlat;
        spin_j_z += sjz / nlat;
        spin_tot_z += (v_dot(dim, dir, S.totspin) / nlat);
        spin_i_h += sih / nlat;
        spin_j_h += sjh / nlat;
        spin_tot_h += (dim == 3 ? S.totspin.z : S.totspin.x) / nlat;
        if (dim == 3) M = sqrt(v_dot(3, S.totspin, S.totspin)) / nlat; /* heisenbergLib.c:726 */
        else M = sqrt(v_dot(2, si, si)) / nlat;                       /* xyLib.c:654 */
        M2 += M * M;
        M4 += M * M * M * M;
        M_tot += M;
        MdotM += M_tmp * M;
        M_tmp = M;
        si.x /= nlat; si.y /= nlat; if (dim == 3) si.z /= nlat;
        sj.x /= nlat; sj.y /= nlat; if (dim == 3) sj.z /= nlat;
        si.x = fabs(si.x); si.y = fabs(si.y); si.z = fabs(si.z);
        sj.x = fabs(sj.x); sj.y = fabs(sj.y); sj.z = fabs(sj.z);
        v_add(dim, &spin_i, si);
        v_add(dim, &spin_j, sj);
        spin_ij += sij / nlat;
        double e_avg = S.energy / N;
        totEnergy += e_avg;
        E2 += e_avg * e_avg;

        V3 sir = {0, 0, 0}, sjr = {0, 0, 0};
        int ci = 0, cj = 0, cij = 0;
        double sijr = 0.0;
        for (int j = 0; j < p->nlat; j++) {
            int oi = p->corr_pair[2 * j], oj = p->corr_pair[2 * j + 1];
            if (S.chosen[oi] > 0) { ci++; v_add(dim, &sir, on_majority(&S, oi)); }
            if (S.chosen[oj] > 0) { cj++; v_add(dim, &sjr, on_majority(&S, oj)); }
            if ((S.chosen[oi] > 0) && (S.chosen[oj] > 0)) {
                cij++;
                sijr += v_dot(dim, on_majority(&S, oi), on_majority(&S, oj));
            }
        }
        sir.x /= ci; sir.y /= ci; if (dim == 3) sir.z /= ci;
        sjr.x /= cj; sjr.y /= cj; if (dim == 3) sjr.z /= cj;
        sir.x = fabs(sir.x); sir.y = fabs(sir.y); sir.z = fabs(sir.z);
        sjr.x = fabs(sjr.x); sjr.y = fabs(sjr.y); sjr.z = fabs(sjr.z);
        v_add(dim, &spin_i_r, sir);
        v_add(dim, &spin_j_r, sjr);
        spin_ij_r += sijr / cij;
        double er = 0;
        for (int j = 0; j < N; j++)
            if (S.chosen[j] > 0) er += on_corr_rnorm(&S, j);
        er /= 2;
        for (int j = 0; j < N; j++)
            if (S.chosen[j] > 0) er += on_onsite(&S, j, S.s[j]);
        er /= p->n_rorb;
        totEnergy_r += er;
        E2_r += er * er;

        int g;
        for (g = 0; g < G; g++) {
            V3 acc = {0, 0, 0};
            for (int k = 0; k < p->max_group; k++) {
                int id = p->group_list[(size_t)g * p->max_group + k];
                if (id < 0) break;
                v_add(dim, &acc, S.s[id]);
            }
            gsum[g] = acc;
        }
        gsum[g].x = S.totspin.x / nlat;
        gsum[g].y = S.totspin.y / nlat;
        gsum[g].z = dim == 3 ? S.totspin.z / nlat : 0;
        for (int a = 0; a < G + 1; a++)
            for (int b = 0; b < G + 1; b++) {
                double d = v_dot(dim, gsum[a], gsum[b]);
                sds[a * (G + 1) + b] += d;
                if (a == b) s4[a] += d * d;
            }
        if (run->series) {
            double *q = run->series + (size_t)m * OR_NSER;
            q[0] = e_avg; q[1] = M; q[2] = er; q[3] = sij / nlat;
        }
    }
    double ns = (double)p->nsweep;
    double U4 = (M2 / ns) * (M2 / ns) / (M4 / ns);
    double autoCorr = dim == 3 ? (MdotM / ns - M_tot / ns * M_tot / ns)      /* heisenbergLib.c:834 */
                               : (MdotM / ns - (M_tot / ns) * (M_tot / ns)); /* xyLib.c:761 */
    double *r = run->result;
    int xy = dim == 2;
    r[0] = spin_i.x / ns; r[1] = spin_i.y / ns; r[2] = xy ? 0 : spin_i.z / ns;
    r[3] = spin_j.x / ns; r[4] = spin_j.y / ns; r[5] = xy ? 0 : spin_j.z / ns;
    r[6] = spin_ij / ns; r[7] = autoCorr; r[8] = totEnergy / ns; r[9] = E2 / ns; r[10] = U4;
    r[11] = spin_i_r.x / ns; r[12] = spin_i_r.y / ns; r[13] = xy ? 0 : spin_i_r.z / ns;
    r[14] = spin_j_r.x / ns; r[15] = spin_j_r.y / ns; r[16] = xy ? 0 : spin_j_r.z / ns;
    r[17] = spin_ij_r / ns; r[18] = totEnergy_r / ns; r[19] = E2_r / ns;
    r[20] = spin_i_z / ns; r[21] = spin_j_z / ns; r[22] = spin_tot_z / ns;
    r[23] = spin_i_h / ns; r[24] = spin_j_h / ns; r[25] = spin_tot_h / ns;
    r[26] = xy ? 0 : topo / ns;
    r[27] = 0.0;
    int need = 29 + (G + 1) * (G + 1) + (G + 1);
    r[28] = G;
    if (run->result_cap >= need) {
        for (int a = 0; a < (G + 1) * (G + 1); a++) r[29 + a] = sds[a] / ns;
        for (int a = 0; a < G + 1; a++) r[29 + (G + 1) * (G + 1) + a] = s4[a] / ns;
    }
    if (run->spins_io)
        for (int i = 0; i < N; i++) {
            run->spins_io[3 * i] = S.s[i].x;
            run->spins_io[3 * i + 1] = S.s[i].y;
            run->spins_io[3 * i + 2] = dim == 3 ? S.s[i].z : 0;
        }
    if (run->mode == 1) sweep_free(&sw);
    free(sds); free(s4); free(gsum);
    free(S.s); free(S.trans); free(S.perp); free(S.sdotn); free(S.len);
    free(S.inblock); free(S.projected); free(S.block); free(S.buffer); free(S.chosen);
    return 0;
}

/* ------------------------------------------------------------ entry points */
int mcs_oracle_solve(const OrProblem *p, OrRun *run)
{
    if (!p || !run || !run->result || !run->stats) return -1;
    if (p->N <= 0 || p->z < 0 || p->nsweep < 0) return -2;
    if (p->model == 1) return ising_run(p, run);
    if (p->model == 2 || p->model == 3) return on_run(p, run);
    return -3;
}

/* Greedy colouring exported for cross-checks of the engine's model compiler. */
int mcs_oracle_colour(const OrProblem *p, int32_t *colour_out)
{
    int *c = malloc((size_t)p->N * sizeof(int));
    int n = greedy_colour(p, c);
    for (int i = 0; i < p->N; i++) colour_out[i] = c[i];
    free(c);
    return n;
}

void mcs_oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    or_philox4x32_10(ctr, key, out);
}

int mcs_oracle_abi_version(void) { return 1; }
