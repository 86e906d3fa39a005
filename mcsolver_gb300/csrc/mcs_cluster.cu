// mcs_cluster.cu -- cluster schedule of the Metropolis sweep (square lattice: XY / Heisenberg
// in k_cluster_metro, Ising in k_cluster_ising further down).
//
// One replica is split by rows over a thread-block cluster of C CTAs (any C
// from 1 to 16; the autotuner offers the powers of two and one wave-filling
// size).  The Lx/2 row pairs are dealt out as evenly as possible:
// CTA r owns RP_r = 2*(P/C + (r < P%C)) rows starting at x0_r (P = Lx/2; every
// slab starts on an even row, so the parity colouring of a local row is that
// of the global row) and keeps one ghost row on each side:
//
//   local index (c, xl, yh) = c*rows*hy + (xl+1)*hy + yh,   xl in [-1, RP_r]
//
// (rows = the largest RP_r + 2, the same stride in every CTA).  A colour phase
// updates the CTA's own sites of that colour from local data; a CTA that
// accepts a move on its first or last row also stores the new spin into the
// neighbouring CTA's ghost row (DSMEM), and one cluster barrier per colour
// publishes those stores.  Measurements reduce per-CTA partial sums through
// DSMEM into rank 0, which owns the replica's FP64 accumulators for the
// launch.  The per-site update, the Philox counters and the measurement sums
// are the ones of the other schedules, so the spin trajectory is the same.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "mcs_device.cuh"
#include "mcs_internal.h"

namespace cg = cooperative_groups;

namespace mcs {

static __host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }

#define CL_NV 28
// per-CTA partial slot of one measurement: CL_NV frame sums, then the energy
// change and the accepted count since the previous measurement, the full-energy
// flag and the measurement index; two slots (measurement parity) and a third
// for the energy change after the last measurement of a launch
#define CL_SLOT 32
#define CL_PART (3 * CL_SLOT)
#define CL_RED (32 * CL_SLOT + 32)

struct ClusterLayout {
    size_t spins, tables, majc, part, red, acc, total;
    int rows, hy, nloc, nchosen;
};

// Row slab of CTA r: first row x0 and row count rp (both even).
__host__ __device__ inline void cl_split(int Lx, int C, int r, int *x0, int *rp)
{
    const int P = Lx >> 1, b = P / C, e = P % C;
    *x0 = 2 * (r * b + (r < e ? r : e));
    *rp = 2 * (b + (r < e ? 1 : 0));
}
// CTA that owns row pair `pr` (rows 2pr, 2pr+1).
__host__ __device__ inline int cl_owner(int Lx, int C, int pr)
{
    const int P = Lx >> 1, b = P / C, e = P % C, big = e * (b + 1);
    return pr < big ? pr / (b + 1) : e + (pr - big) / b;
}

__host__ __device__ inline ClusterLayout cluster_layout(const Rep &R, int C)
{
    ClusterLayout L;
    const int P = R.Lx >> 1;
    const int RP = 2 * (P / C + (P % C ? 1 : 0));  // the largest slab
    L.rows = RP + 2;
    L.hy = R.hy;
    L.nloc = 2 * L.rows * L.hy;
    L.nchosen = (RP / 2) * (R.Ly / 2);  // chosen sites of the largest slab
    size_t off = 0;
    L.spins = off; off += a16((size_t)R.dim * L.nloc * sizeof(float));
    L.tables = off; off += a16((size_t)R.njc * 9 * sizeof(float) + (size_t)R.ndc * 4 * sizeof(float));
    L.majc = off; off += a16((size_t)L.nchosen * 3 * sizeof(float));
    L.part = off; off += CL_PART * sizeof(double);
    L.red = off; off += CL_RED * sizeof(double);
    L.acc = off; off += a16((size_t)R.nacc * sizeof(double) + C_NINT * sizeof(long long));
    L.total = off;
    return L;
}

// Square-lattice neighbours of an owned site in local coordinates.
template <class F>
__device__ __forceinline__ void cl_links(const Rep &R, int rows, int c, int xl, int yh, F &&f)
{
    const int Ly = R.Ly, hy = R.hy;
    const int x = xl;  // parity of the global row equals the parity of xl (RP even)
    const int y = 2 * yh + ((x + c) & 1);
    const int base = (1 - c) * rows * hy;
    const int yp = (y + 1 == Ly) ? 0 : y + 1;
    const int ym = (y == 0) ? Ly - 1 : y - 1;
    f(0, base + (xl + 2) * hy + yh, R.sq_code[0]);
    f(1, base + xl * hy + yh, R.sq_code[1]);
    f(2, base + (xl + 1) * hy + (yp >> 1), R.sq_code[2]);
    f(3, base + (xl + 1) * hy + (ym >> 1), R.sq_code[3]);
}

// The same with the lattice side and the four link codes in registers (the
// sweep loop's copy; the descriptor lives in shared memory).
struct SqLinks {
    int Ly, hy, rows, q0, q1, q2, q3;
};
template <class F>
__device__ __forceinline__ void cl_links_r(const SqLinks &K, int c, int xl, int yh, F &&f)
{
    const int hy = K.hy;
    const int y = 2 * yh + ((xl + c) & 1);
    const int base = (1 - c) * K.rows * hy;
    const int yp = (y + 1 == K.Ly) ? 0 : y + 1;
    const int ym = (y == 0) ? K.Ly - 1 : y - 1;
    f(0, base + (xl + 2) * hy + yh, K.q0);
    f(1, base + xl * hy + yh, K.q1);
    f(2, base + (xl + 1) * hy + (yp >> 1), K.q2);
    f(3, base + (xl + 1) * hy + (ym >> 1), K.q3);
}
// Register copies of the descriptor flags the trial reads.
struct TrialFlags {
    bool fullJ, has_d;
};

// The XY trial of on_trial with the couplings of the four link directions in
// registers (cj[d] = M[0], M[1], M[3], M[6] of direction d's class: a
// regular lattice has one class per direction), the local field formed in
// on_field's order so that the result is the same to the bit; the site's spin
// after the trial in (fx, fy), for the sums the sweep forms on the way.
template <class LINKS>
__device__ __forceinline__ bool on_trial_xy_r(const TrialFlags &F, const float (&cj)[4][4], const float *__restrict__ dt,
                                              const Spins &S, int v, const uint4 &w, float beta, float h,
                                              LINKS &&links, float *dEout, float &fx, float &fy)
{
    float h0 = 0.f, h1 = 0.f;
    links([&](int d, int j, int) {
        const float a = S.x[j], b = S.y[j];
        h0 = fmaf(cj[d][0], a, h0);
        h1 = fmaf(cj[d][1], b, h1);
        if (F.fullJ) {
            h0 = fmaf(cj[d][2], b, h0);
            h1 = fmaf(cj[d][3], a, h1);
        }
    });
    float r0, r1, r2;
    on_direction<2>(w, r0, r1, r2);
    const float s0 = S.x[v], s1 = S.y[v];
    const float sr = s0 * r0 + s1 * r1;
    const float f = -2.f * sr;
    const float d0 = f * r0, d1 = f * r1;
    float dE = d0 * h0 + d1 * h1;
    if (F.has_d) dE += dt[0] * (d0 * (2.f * s0 + d0)) + dt[1] * (d1 * (2.f * s1 + d1));
    dE -= h * d0;
    const float x = beta * dE;
    const bool acc = (x <= 0.f) || (__expf(-x) > u24(w.y));
    fx = s0;
    fy = s1;
    if (acc) {
        const float n0 = s0 + d0, n1 = s1 + d1;
        const float len2 = n0 * n0 + n1 * n1;
        const float k = len2 > 0.f ? dt[3] * rsqrtf(len2) : 1.f;
        fx = n0 * k;
        fy = n1 * k;
        S.x[v] = fx;
        S.y[v] = fy;
        *dEout = dE;
    }
    return acc;
}

// Index of the slot sum that feeds frame entry f (frame layout F_*), -1 for 0.
__device__ __forceinline__ int cl_frame_src(int f, int ngroup, int gall)
{
    if (f >= F_G) {
        const int g = (f - F_G) / 3, k = (f - F_G) - 3 * g;
        if (g >= ngroup) return -1;
        return ((gall >> g) & 1) ? k : 16 + 3 * g + k;
    }
    if (f < F_SJ) return 3 + (f - F_SI);
    if (f < F_SIJ) return 3 + (f - F_SJ);
    if (f == F_SIJ) return 6;
    if (f < F_Q) return f - F_TOT;
    if (f == F_Q) return 9;
    if (f < F_SJR) return 10 + (f - F_SIR);
    if (f < F_SIJR) return 10 + (f - F_SJR);
    if (f == F_SIJR) return 13;
    if (f == F_ERB) return 14;
    if (f == F_ERO) return 15;
    if (f == F_EFB) return 7;
    return 8;  // F_EFO
}

// Measurement slots folded per batch by rank 0 (consecutive measurements).
#define CL_RING 16

// Rank 0, warp 0 (lane = slot entry): sum slot `slot` of every CTA of the
// cluster in fixed rank order into one ring entry (FP64), and write the
// measurement's frame in FP32: frame entry f takes slot entry fsrc[f] (a table
// of cl_frame_src made once per launch), passed between lanes by a shuffle.
// The last two entries (re-check flag, measurement index) are the same in
// every CTA and are taken from rank 0's slot, not summed.
// The remote loads are issued eight at a time before any is added, so a
// gather waits about one DSMEM round trip per eight CTAs instead of one per
// CTA; the sum is still taken in rank order (adding the 0.0 of an absent
// rank changes nothing).
__device__ __forceinline__ void cluster_gather(double *part, double *entry, float *frame, const signed char *fsrc,
                                               int C, int slot, int lane)
{
    cg::cluster_group cl = cg::this_cluster();
    double o = 0.0;
    const int idx = slot * CL_SLOT + lane;
    if (lane >= CL_NV + 2) o = part[idx];
    else
        for (int q0 = 0; q0 < C; q0 += 8) {
            double v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = (q0 + j < C) ? cl.map_shared_rank(part, q0 + j)[idx] : 0.0;
#pragma unroll
            for (int j = 0; j < 8; ++j) o += v[j];
        }
    entry[lane] = o;
    const float of = (float)o;
    for (int f = lane; f - lane < F_NON; f += 32) {  // the bound is the same for every lane
        const int k = f < F_NON ? (int)fsrc[f] : -1;
        const float v = __shfl_sync(0xffffffffu, of, k < 0 ? 0 : k);
        if (f < F_NON) frame[f] = k < 0 ? 0.f : v;
    }
}

// Rank 0, warp 0: fold the n ring entries (consecutive measurements; their
// FP32 frames in fs) into the FP64 accumulators: running energy in order
// (lane 0), then the frames together.  Kept out of line so that its registers do not add to the sweep
// loop's.
template <int DIM>
__device__ __noinline__ void cluster_fold_ring(Rep &R, const double *ring, int n, float *fs, double *Eb, int lane)
{
    __syncwarp();
    if (lane == 0) {
        for (int j = 0; j < n; ++j) {
            const double *o = ring + j * CL_SLOT;
            R.acc[A_ECUR] += o[CL_NV];
            R.stats[S_ACCEPT] += (long long)o[CL_NV + 1];
            if (o[CL_NV + 2] != 0.0) {  // full-energy re-check
                const double Ef = o[7] / 2 + o[8];
                const double d = fabs(R.acc[A_ECUR] - Ef);
                if (d > R.acc[A_DRIFT]) R.acc[A_DRIFT] = d;
                R.acc[A_ECUR] = Ef;
            }
            Eb[j] = R.acc[A_ECUR];
        }
    }
    __syncwarp();
    on_accumulate_frames<DIM>(R, fs, Eb, (long long)ring[CL_NV + 3], n, lane);
}

// NT: block size the kernel is compiled for (256, 512 or 1024 threads; the
// register budget per thread follows from it)
template <int DIM, int NT>
__global__ void __launch_bounds__(NT) k_cluster_metro(Rep *reps, const int *ids, long long max_units, int C)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Rep R;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    Rep *Rg = reps + ids[blockIdx.x / C];
    {
        const int *s = (const int *)Rg;
        int *d = (int *)&R;
        for (int i = threadIdx.x; i < (int)(sizeof(Rep) / 4); i += blockDim.x) d[i] = s[i];
    }
    __syncthreads();
    // every CTA of the cluster reads the same descriptor: the early exit is uniform over the cluster
    if (R.u >= R.u_stop) return;
    const ClusterLayout L = cluster_layout(R, C);
    const int tid = threadIdx.x, bd = blockDim.x;
    const int hy = L.hy, rows = L.rows, nloc = L.nloc;
    int x0, RP;
    cl_split(R.Lx, C, rank, &x0, &RP);
    const int nch = (RP / 2) * (R.Ly / 2);  // chosen sites (even rows x even columns) of this slab
    const int hb = R.Ly >> 1;
    const int half = R.half;
    float *sp = (float *)(smem + L.spins);
    Spins S;
    S.x = sp; S.y = sp + nloc; S.z = sp + 2 * nloc;
    float *jt = (float *)(smem + L.tables);
    float *dt = jt + R.njc * 9;
    float *majc = (float *)(smem + L.majc);
    double *part = (double *)(smem + L.part);
    double *red = (double *)(smem + L.red);
    Spins G = spins_global(R);
    // own rows and ghost rows from global memory
    for (int i = tid; i < nloc; i += bd) {
        const int c = i / (rows * hy);
        const int rem = i - c * rows * hy;
        const int xl = rem / hy - 1, yh = rem - (xl + 1) * hy;
        if (xl > RP) continue;  // beyond this slab's bottom ghost row
        int x = x0 + xl;
        if (x < 0) x += R.Lx;
        if (x >= R.Lx) x -= R.Lx;
        const int v = c * half + x * hy + yh;
        S.x[i] = G.x[v]; S.y[i] = G.y[v];
        if (DIM == 3) S.z[i] = G.z[v];
    }
    for (int k = tid; k < R.njc * 9; k += bd) jt[k] = R.jtab[k];
    for (int k = tid; k < R.ndc * 4; k += bd) dt[k] = R.dtab[k];
    if (rank == 0) {
        double *a = (double *)(smem + L.acc);
        for (int k = tid; k < R.nacc; k += bd) a[k] = R.acc[k];
        __syncthreads();
        if (tid == 0) R.acc = a;
    }
    __syncthreads();
    cl.sync();

    // Regular lattices whose -x and -y block links carry the transposes of the
    // +x and +y couplings: summed over the blocks, the -x term of block b is the
    // +x term of block b - x, so the renormalised bond sum is twice the sum of
    // the +x and +y terms (pass B then reads no -x neighbour across a slab)
    bool bpair = false;
    if (R.meas_regular) {
        auto transposed = [&](int ca, int cb) {
            const float *A = jt + 9 * ca, *B = jt + 9 * cb;
            bool t = A[0] == B[0] && A[1] == B[1] && (!R.fullJ || (A[3] == B[6] && A[6] == B[3]));
            if (DIM == 3) t = t && A[2] == B[2] && (!R.fullJ || (A[4] == B[7] && A[7] == B[4] && A[5] == B[8] && A[8] == B[5]));
            return t;
        };
        bpair = transposed(R.rdir_cls[0], R.rdir_cls[1]) && transposed(R.rdir_cls[2], R.rdir_cls[3]);
    }

    const float beta = R.beta, h = R.h;
    double dEd = 0.0;
    long long nacc = 0;
    const int nown = RP * hy;  // own sites per colour
    const int rprev = (rank + C - 1) % C, rnext = (rank + 1) % C;
    float *prev_sp = cl.map_shared_rank(sp, rprev);
    float *next_sp = cl.map_shared_rank(sp, rnext);
    int x0p, RPp, x0n, RPn;  // the neighbouring slabs (the previous one's bottom ghost row is its local row RPp + 1)
    cl_split(R.Lx, C, rprev, &x0p, &RPp);
    cl_split(R.Lx, C, rnext, &x0n, &RPn);
    (void)RPn;
    // chosen index t (block row t / hb) -> owning CTA and index in its majc
    auto chosen_owner = [&](int t, int &lq) {
        const int o = cl_owner(R.Lx, C, t / hb);
        int xo, rpo;
        cl_split(R.Lx, C, o, &xo, &rpo);
        lq = t - (xo >> 1) * hb;
        return o;
    };

    // Measurements.  Every CTA reduces its own sites into its partial slot
    // part[m & 1]; rank 0 folds measurement m into the FP64 accumulators while
    // measurement m + 1 runs (after that measurement's first cluster barrier,
    // when every slot of m is complete), so a measurement costs one cluster
    // barrier.  The fold of the launch's last measurement runs at launch end.
    long long mloc = R.m;
    int fw = R.frames_written;
    int pending = -1;  // slot of a measurement not yet folded
    // rank 0, warp 0: fold slot `slot` (fixed rank order)
    __shared__ double ring[CL_RING * CL_SLOT];
    __shared__ float fsx[CL_RING * MCS_FS_STRIDE];
    __shared__ double Eb[CL_RING];
    __shared__ signed char fsrc[F_NON];
    for (int f = tid; f < F_NON; f += bd) fsrc[f] = (signed char)cl_frame_src(f, R.ngroup, R.gall);
    __syncthreads();
    int nring = 0;  // ring entries gathered and not yet folded (rank 0)
    // rank 0, warp 0: gather the pending slot; fold when the ring is full
    auto gather = [&](bool flush) {
        if (pending >= 0) {
            if (tid < 32)
                cluster_gather(part, ring + nring * CL_SLOT, fsx + nring * MCS_FS_STRIDE, fsrc, C, pending, tid);
            ++nring;
        }
        if (nring > 0 && (flush || nring == CL_RING)) {
            if (tid < 32) cluster_fold_ring<DIM>(R, ring, nring, fsx, Eb, tid);
            nring = 0;
        }
    };
    // sums of pass A gathered by the sweep itself (regular lattices, no
    // full-energy pass): each site's value right after its colour phase, in
    // the order pass A would read them
    float fa[4] = {0.f, 0.f, 0.f, 0.f};
    // Block spins of the own chosen sites (own rows only) into majc.  The
    // sweep computes them after its last colour phase and before that
    // phase's cluster barrier, which then also publishes them to the other
    // CTAs' pass B: the measurement needs no barrier of its own.
    auto block_spins = [&]() {
        const int r0 = (x0 >> 1) * hb;  // first chosen index of this slab
        for (int q = tid; q < nch; q += bd) {
            const int pr = q / (R.Ly / 2);           // even-row index inside the CTA
            const int yc = q - pr * (R.Ly / 2);
            const int xl = 2 * pr, y = 2 * yc;     // chosen: even x, even y
            const int yh = y >> 1;
            // cluster (x,y), (x,y+1), (x+1,y), (x+1,y+1) for Lz = 1
            const int y1 = (y + 1 == R.Ly) ? 0 : y + 1;
            const int c00 = (xl + y) & 1, c01 = (xl + y1) & 1, c10 = (xl + 1 + y) & 1, c11 = (xl + 1 + y1) & 1;
            const int i00 = c00 * rows * hy + (xl + 1) * hy + yh;
            const int i01 = c01 * rows * hy + (xl + 1) * hy + (y1 >> 1);
            const int i10 = c10 * rows * hy + (xl + 2) * hy + yh;
            const int i11 = c11 * rows * hy + (xl + 2) * hy + (y1 >> 1);
            float mx = S.x[i00] + S.x[i01] + S.x[i10] + S.x[i11];
            float my = S.y[i00] + S.y[i01] + S.y[i10] + S.y[i11];
            float mz = DIM == 3 ? S.z[i00] + S.z[i01] + S.z[i10] + S.z[i11] : 0.f;
            v_norm_ref(mx, my, mz);
            const float sv = R.meas_regular ? R.sval0 : R.sval[R.rorb[r0 + q]];
            majc[3 * q] = mx * sv; majc[3 * q + 1] = my * sv; majc[3 * q + 2] = mz * sv;
        }
    };
    auto measure = [&](long long m, bool efull, bool fused) {
        const int r0 = (x0 >> 1) * hb;  // first chosen index of this slab
        if (rank == 0) gather(false);
        const bool full = R.fullJ;
        // partial layout: 0-2 total spin, 3-5 pair sum, 6 pair s.s, 7/8 full
        // energy bond/onsite, 9 solid angles, 10-12 block-spin pair sum,
        // 13 block s.s, 14/15 renormalised bond/onsite, 16-27 four groups
        float a[32];  // CL_NV values and the energy change, padded to the warp width for the halving sum
#pragma unroll
        for (int k = 0; k < 32; ++k) a[k] = 0.f;
        a[CL_NV] = (float)dEd;  // this thread's energy change since the last measurement
        if (fused) {
            a[0] = fa[0]; a[1] = fa[1]; a[2] = fa[2];
            a[3] = fa[0]; a[4] = fa[1]; a[5] = fa[2]; a[6] = fa[3];
        }
        // pass A over own sites: total spin, pair sums, groups, full energy
        for (int c = 0; c < (fused ? 0 : 2); ++c)
            for (int kk = tid; kk < nown; kk += bd) {
                const int xl = kk / hy, yh = kk - xl * hy;
                const int li = c * rows * hy + (xl + 1) * hy + yh;
                const int v = c * half + (x0 + xl) * hy + yh;
                const float sx = S.x[li], sy = S.y[li], sz = DIM == 3 ? S.z[li] : 0.f;
                a[0] += sx; a[1] += sy; a[2] += sz;
                if (R.meas_regular || (R.sflag[v] & 1)) { a[3] += sx; a[4] += sy; a[5] += sz; a[6] += sx * sx + sy * sy + sz * sz; }
                if (efull) {
                    float h0, h1, h2;
                    on_field<DIM>(R, jt, S, [&](auto &&f) { cl_links(R, rows, c, xl, yh, f); }, h0, h1, h2);
                    a[7] += sx * h0 + sy * h1 + sz * h2;
                    float e = 0.f;
                    if (R.has_d) {
                        e = dt[0] * sx * sx + dt[1] * sy * sy;
                        if (DIM == 3) e += dt[2] * sz * sz;
                    }
                    a[8] += e - h * ((DIM == 3) ? sz : sx);
                }
                const int gm = (R.ngroup && !R.meas_regular) ? (R.gmask[v] & ~R.gall) : 0;
                if (gm) {
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        if (gm & (1 << g)) { a[16 + 3 * g] += sx; a[17 + 3 * g] += sy; a[18 + 3 * g] += sz; }
                }
            }
        // circuits of the cells this CTA owns (Heisenberg): circuit (cell, q)
        // has index cell*per + q and its sites lie in rows x and x+1
        if (DIM == 3 && R.ncirc > 0) {
            const int per = R.ncirc / R.N;
            for (int c = 0; c < 2; ++c)
                for (int kk = tid; kk < nown; kk += bd) {
                    const int xl = kk / hy, yh = kk - xl * hy;
                    const int xg = x0 + xl, yg = 2 * yh + ((xg + c) & 1);
                    for (int q = 0; q < per; ++q) {
                        const int ci = (xg * R.Ly + yg) * per + q;
                        const int tv[3] = {__ldg(&R.circ[3 * ci]), __ldg(&R.circ[3 * ci + 1]), __ldg(&R.circ[3 * ci + 2])};
                        int li3[3];
#pragma unroll
                        for (int e3 = 0; e3 < 3; ++e3) {
                            const int w = tv[e3];
                            const int cc = w >= half;
                            const int k2 = w - cc * half;
                            const int xw = k2 / hy, yy = k2 - xw * hy;
                            int xl2 = xw - x0;
                            if (xl2 < -1) xl2 += R.Lx;
                            if (xl2 > RP) xl2 -= R.Lx;
                            li3[e3] = cc * rows * hy + (xl2 + 1) * hy + yy;
                        }
                        const int ia = li3[0], ib = li3[1], ic = li3[2];
                        const float ax = S.x[ia], ay = S.y[ia], az = S.z[ia];
                        const float bx = S.x[ib], by = S.y[ib], bz = S.z[ib];
                        const float cx = S.x[ic], cy = S.y[ic], cz = S.z[ic];
                        const float l = R.slen[0], il2 = 1.f / (l * l);
                        const float s1s2 = (ax * bx + ay * by + az * bz) * il2;
                        const float s2s3 = (bx * cx + by * cy + bz * cz) * il2;
                        const float s3s1 = (cx * ax + cy * ay + cz * az) * il2;
                        const float kx = by * cz - bz * cy, ky = bz * cx - bx * cz, kz = bx * cy - by * cx;
                        const float re = 1.f + s1s2 + s2s3 + s3s1;
                        const float im = (ax * kx + ay * ky + az * kz) * R.inv_len3;
                        a[9] += (fabsf(re) < 1e-6f) ? (im > 0.f ? (float)MCS_PI_REF : -(float)MCS_PI_REF)
                                                    : 2.f * atanf(__fdividef(im, re));
                    }
                }
        }
        // pass B over own chosen sites; regular lattices by arithmetic (block
        // (xr, yb) links to its four neighbour blocks), others from the lists
        if (R.meas_regular) {
            const int nbx = R.Lx >> 1;
            for (int q = tid; q < nch; q += bd) {
                const int r = r0 + q;
                const int xr = r / hb, yb = r - xr * hb;
                const float mx = majc[3 * q], my = majc[3 * q + 1], mz = majc[3 * q + 2];
                a[10] += mx; a[11] += my; a[12] += mz; a[13] += mx * mx + my * my + mz * mz;
                const int tg[4] = {(xr + 1 == nbx ? 0 : xr + 1) * hb + yb, (xr == 0 ? nbx - 1 : xr - 1) * hb + yb,
                                   xr * hb + (yb + 1 == hb ? 0 : yb + 1), xr * hb + (yb == 0 ? hb - 1 : yb - 1)};
                // +-y neighbours are in the same block row; +x leaves the slab
                // after its last block row, -x before its first
                const int brl = (x0 >> 1) + (RP >> 1) - 1;
                float corr = 0.f;
#pragma unroll
                for (int d = 0; d < 4; ++d) {
                    if (bpair && (d & 1)) continue;
                    int owner = rank, lq = tg[d] - r0;
                    if (d == 0 && xr == brl) { owner = rnext; lq = tg[d] - (x0n >> 1) * hb; }
                    if (d == 1 && xr == (x0 >> 1)) { owner = rprev; lq = tg[d] - (x0p >> 1) * hb; }
                    const float *mc = owner == rank ? majc : cl.map_shared_rank(majc, owner);
                    corr += on_jdot<DIM>(jt + 9 * R.rdir_cls[d], full, mx, my, mz, mc[3 * lq], mc[3 * lq + 1], mc[3 * lq + 2]);
                }
                a[14] += bpair ? 2.f * corr : corr;
                // onsite energy of the actual spin at (2 xr, 2 yb): colour 0
                const int li = (2 * xr - x0 + 1) * hy + yb;
                const float sx = S.x[li], sy = S.y[li], sz = DIM == 3 ? S.z[li] : 0.f;
                float e = 0.f;
                if (R.has_d) {
                    e = dt[0] * sx * sx + dt[1] * sy * sy;
                    if (DIM == 3) e += dt[2] * sz * sz;
                }
                a[15] += e - h * ((DIM == 3) ? sz : sx);
            }
        } else
        for (int q = tid; q < nch; q += bd) {
            const int r = r0 + q;
            const int v = R.rorb[r];
            const float mx = majc[3 * q], my = majc[3 * q + 1], mz = majc[3 * q + 2];
            if (R.sflag[v] & 1) { a[10] += mx; a[11] += my; a[12] += mz; a[13] += mx * mx + my * my + mz * mz; }
            float corr = 0.f;
            const int d = R.rdeg[r];
            for (int l = 0; l < d; ++l) {
                const int tr = __ldg(&R.rtgt[(size_t)r * R.zmax + l]);
                if (tr < 0) continue;
                int lq;
                const int owner = chosen_owner(tr, lq);
                const float *mc = owner == rank ? majc : cl.map_shared_rank(majc, owner);
                corr += on_jdot<DIM>(jt + 9 * R.rjc[(size_t)r * R.zmax + l], full, mx, my, mz, mc[3 * lq], mc[3 * lq + 1], mc[3 * lq + 2]);
            }
            a[14] += corr;
            // onsite energy of the actual spin
            const int cc = v >= half;
            const int k2 = v - cc * half;
            const int xg = k2 / hy, yy = k2 - xg * hy;
            const int li = cc * rows * hy + (xg - x0 + 1) * hy + yy;
            const float sx = S.x[li], sy = S.y[li], sz = DIM == 3 ? S.z[li] : 0.f;
            float e = 0.f;
            if (R.has_d) {
                e = dt[0] * sx * sx + dt[1] * sy * sy;
                if (DIM == 3) e += dt[2] * sz * sz;
            }
            a[15] += e - h * ((DIM == 3) ? sz : sx);
        }
        // warp sums (FP32 frame values by recursive halving, FP64 energy
        // change and count), then the CTA's slot in FP64 across the warps
        {
            const int lane = tid & 31, wid = tid >> 5, nw = (bd + 31) >> 5;
            float *redf = (float *)red;                       // [32 warps][CL_SLOT]
            long long *redl = (long long *)(red + 16 * CL_SLOT);  // [32 warps]
            if (R.meas_regular) {
                // regular lattices: entries 3-5 equal 0-2 (every site is a
                // correlated-pair site) and the group entries 16-27 are 0, so
                // 14 distinct values are halved over 16 lanes (lane l holds
                // value l of b, then the xor-16 step adds the two half-warps)
                float b[16] = {a[0], a[1], a[2], a[6], a[7], a[8], a[9], a[10], a[11], a[12], a[13], a[14], a[15],
                               a[CL_NV], 0.f, 0.f};
#pragma unroll
                for (int w = 8; w >= 1; w >>= 1) {
                    const bool up = (lane & w) != 0;
#pragma unroll
                    for (int j = 0; j < w; ++j) {
                        const float send = up ? b[j] : b[j + w];
                        const float keep = up ? b[j + w] : b[j];
                        b[j] = keep + __shfl_xor_sync(0xffffffffu, send, w);
                    }
                }
                const float y = b[0] + __shfl_xor_sync(0xffffffffu, b[0], 16);
                if (lane < 14) redf[wid * CL_SLOT + lane] = y;
            } else {
#pragma unroll
                for (int w = 16; w >= 1; w >>= 1) {
                    const bool up = (lane & w) != 0;
#pragma unroll
                    for (int j = 0; j < w; ++j) {
                        const float send = up ? a[j] : a[j + w];
                        const float keep = up ? a[j + w] : a[j];
                        a[j] = keep + __shfl_xor_sync(0xffffffffu, send, w);
                    }
                }
                if (lane <= CL_NV) redf[wid * CL_SLOT + lane] = a[0];
            }
            // the energy change went through the FP32 halving with the frame
            // values (lane CL_NV); the count stays integer
            long long na = nacc;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) na += __shfl_xor_sync(0xffffffffu, na, o);
            // warp values in FP32 (redf) and the counts as integers (redl),
            // both inside the red area; across the warps the FP32 values are
            // summed with Neumaier compensation and enter the FP64 slot as the
            // sum plus its rounding error (FP64 instructions issue slowly and
            // this sum is on the measurement's critical path)
            if (lane == 0) redl[wid] = na;
            __syncthreads();
            const int slot = (int)(m & 1);
            if (tid <= CL_NV) {
                // slot entry tid from warp entry src (regular lattices: the compact order above)
                const int src = !R.meas_regular ? tid
                                                : (tid < 3 ? tid : tid < 16 ? tid - 3 : tid == CL_NV ? 13 : -1);
                float sh = 0.f, sl = 0.f;
                if (src >= 0)
                    for (int w = 0; w < nw; ++w) ksum_add(sh, sl, redf[w * CL_SLOT + src]);
                part[slot * CL_SLOT + tid] = (double)sh + (double)sl;
            } else if (tid == CL_NV + 1) {
                long long n = 0;
                for (int w = 0; w < nw; ++w) n += redl[w];
                part[slot * CL_SLOT + tid] = (double)n;
            } else if (tid == CL_NV + 2) {
                part[slot * CL_SLOT + tid] = efull ? 1.0 : 0.0;
            } else if (tid == CL_NV + 3) {
                part[slot * CL_SLOT + tid] = (double)m;
            }
            pending = slot;
        }
        dEd = 0.0;
        nacc = 0;
        // spin frame: every CTA writes its own rows
        if (R.frames > 0 && (m % R.frame_every) == 0 && fw < R.frames) {
            for (int c = 0; c < 2; ++c)
                for (int kk = tid; kk < nown; kk += bd) {
                    const int xl = kk / hy, yh = kk - xl * hy;
                    const int li = c * rows * hy + (xl + 1) * hy + yh;
                    const int v = c * half + (x0 + xl) * hy + yh;
                    frame_store<DIM>(R, fw, v, S, li);
                }
            ++fw;
        }
        // a full-energy pass and the solid angles read ghost rows, which the
        // neighbours' next colour phase overwrites: hold them back until every
        // CTA is done reading
        if (efull || (DIM == 3 && R.ncirc > 0)) cl.sync();
    };

    // Sweeps.  A CTA that accepts a move on its first or last own row writes
    // the new spin straight into the neighbouring CTA's ghost row as well
    // (DSMEM store); sites that reject keep the value the ghost already holds.
    // Colour phase c reads only colour 1-c ghosts and writes only colour-c
    // ghosts, so one cluster barrier per colour both publishes the pushes and
    // orders them before the next phase's reads.
    long long u = R.u;
    const long long uend = min(R.u_stop, u + max_units);
    const SqLinks sql = {R.Ly, hy, rows, R.sq_code[0], R.sq_code[1], R.sq_code[2], R.sq_code[3]};
    const TrialFlags tflags = {R.fullJ != 0, R.has_d != 0};
    float cj[4][4];  // XY: the four directions' couplings (see on_trial_xy_r)
#pragma unroll
    for (int d = 0; d < 4; ++d) {
        const float *M = jt + 9 * R.sq_code[d];
        cj[d][0] = M[0]; cj[d][1] = M[1]; cj[d][2] = M[3]; cj[d][3] = M[6];
    }
    for (; u < uend; ++u) {
        const long long t = R.u0 + u;
        const bool fuse = R.meas_regular && measures_after(R, u) && (mloc % R.recheck) != 0;
        fa[0] = fa[1] = fa[2] = fa[3] = 0.f;
        float dEf = 0.f;  // this thread's energy change over the sweep (FP32; summed in FP64 per sweep)
        for (int c = 0; c < 2; ++c) {
            SqWalk wk;
            wk.init(tid, bd, hy);
            const int cb = c * rows * hy;
            // four sites per thread at a time: their Philox words are drawn
            // first, as independent instruction streams, then the trials run.
            // The loop bound is the warp's first lane's index, the same for
            // every lane, so the whole warp reaches the pair exchange below;
            // sites past the end are skipped one by one.
            const int lane = tid & 31;
            for (int kb = tid; kb - lane < nown; kb += 4 * bd) {
                uint4 ws[4];
                int xs[4], ys[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    xs[e] = wk.x; ys[e] = wk.yh;
                    wk.next();
                }
                // colour-local index of the whole lattice of site e: x0*hy + kb + e*bd
                const uint32_t kg = (uint32_t)(x0 * hy + kb);
                if (DIM == 2) {
                    // XY: sites k and k^1 share one Philox block (on_words).
                    // x0 and bd are even, so lanes 2i and 2i+1 hold the two
                    // sites of one block for every e.  The even lane draws the
                    // blocks of e = 0, 1 and the odd lane those of e = 2, 3;
                    // each passes its partner the partner's half.
                    const bool odd = (lane & 1) != 0;
                    const uint32_t ka = kg + (uint32_t)((odd ? 2 : 0) * bd);
                    const uint4 A = philox_t(ka >> 1, t, (uint32_t)c, R.seed);
                    const uint4 B = philox_t((ka + (uint32_t)bd) >> 1, t, (uint32_t)c, R.seed);
                    const uint32_t r0 = __shfl_xor_sync(0xffffffffu, odd ? A.x : A.z, 1);
                    const uint32_t r1 = __shfl_xor_sync(0xffffffffu, odd ? A.y : A.w, 1);
                    const uint32_t r2 = __shfl_xor_sync(0xffffffffu, odd ? B.x : B.z, 1);
                    const uint32_t r3 = __shfl_xor_sync(0xffffffffu, odd ? B.y : B.w, 1);
                    const uint32_t o0 = odd ? A.z : A.x, o1 = odd ? A.w : A.y;
                    const uint32_t p0 = odd ? B.z : B.x, p1 = odd ? B.w : B.y;
                    ws[0] = make_uint4(odd ? r0 : o0, odd ? r1 : o1, 0u, 0u);
                    ws[1] = make_uint4(odd ? r2 : p0, odd ? r3 : p1, 0u, 0u);
                    ws[2] = make_uint4(odd ? o0 : r0, odd ? o1 : r1, 0u, 0u);
                    ws[3] = make_uint4(odd ? p0 : r2, odd ? p1 : r3, 0u, 0u);
                } else {
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (kb + e * bd < nown) ws[e] = on_words<DIM>(kg + (uint32_t)(e * bd), t, (uint32_t)c, R.seed);
                }
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                if (kb + e * bd >= nown) break;
                const int xl = xs[e], yh = ys[e];
                const int li = cb + (xl + 1) * hy + yh;
                const uint4 w = ws[e];
                float dE;
                bool acc;
                float fx = 0.f, fy = 0.f;
                if (DIM == 2)  // XY: register copies (the Heisenberg loop has no registers to spare)
                    acc = on_trial_xy_r(tflags, cj, dt, S, li, w, beta, h, [&](auto &&f) { cl_links_r(sql, c, xl, yh, f); },
                                        &dE, fx, fy);
                else
                    acc = on_trial<DIM>(R, jt, dt, S, li, 0, w, beta, h, [&](auto &&f) { cl_links(R, rows, c, xl, yh, f); }, &dE);
                if (acc) {
                    dEf += dE;
                    ++nacc;
                    // own row 0 is the previous CTA's bottom ghost (its local row
                    // RPp+1), own row RP-1 the next CTA's top ghost (local row 0)
                    if (xl == 0) {
                        const int g = cb + (RPp + 1) * hy + yh;
                        prev_sp[g] = S.x[li];
                        prev_sp[nloc + g] = S.y[li];
                        if (DIM == 3) prev_sp[2 * nloc + g] = S.z[li];
                    }
                    if (xl == RP - 1) {
                        const int g = cb + yh;
                        next_sp[g] = S.x[li];
                        next_sp[nloc + g] = S.y[li];
                        if (DIM == 3) next_sp[2 * nloc + g] = S.z[li];
                    }
                }
                if (fuse) {
                    const float sx = DIM == 2 ? fx : S.x[li], sy = DIM == 2 ? fy : S.y[li], sz = DIM == 3 ? S.z[li] : 0.f;
                    fa[0] += sx; fa[1] += sy; fa[2] += sz;
                    fa[3] += sx * sx + sy * sy + sz * sz;
                }
              }
            }
            if (c == 1 && measures_after(R, u)) {
                __syncthreads();  // every own site of both colours is final
                block_spins();
            }
            cl.sync();
        }
        dEd += (double)dEf;
        if (measures_after(R, u)) {
            measure(mloc, (mloc % R.recheck) == 0, fuse);
            ++mloc;
        }
    }
    // the energy change after the last measurement -> slot 2
    {
        double de[2] = {dEd, (double)nacc};
        block_sum<2>(de, red, red + 64);
        if (tid == 0) { part[2 * CL_SLOT + CL_NV] = red[64]; part[2 * CL_SLOT + CL_NV + 1] = red[65]; }
    }
    __syncthreads();
    cl.sync();
    if (rank == 0) {
        gather(true);
        if (tid == 0) {
            double s = 0.0, na = 0.0;
            for (int q = 0; q < C; ++q) {
                const double *pq = cl.map_shared_rank(part, q) + 2 * CL_SLOT;
                s += pq[CL_NV];
                na += pq[CL_NV + 1];
            }
            R.acc[A_ECUR] += s;
            R.stats[S_ACCEPT] += (long long)na;
        }
    }
    cl.sync();
    // own rows back to global memory
    for (int c = 0; c < 2; ++c)
        for (int kk = tid; kk < nown; kk += bd) {
            const int xl = kk / hy, yh = kk - xl * hy;
            const int li = c * rows * hy + (xl + 1) * hy + yh;
            const int v = c * half + (x0 + xl) * hy + yh;
            G.x[v] = S.x[li]; G.y[v] = S.y[li];
            if (DIM == 3) G.z[v] = S.z[li];
        }
    if (rank == 0) {
        __syncthreads();
        for (int k = tid; k < R.nacc; k += bd) Rg->acc[k] = R.acc[k];
        if (tid == 0) {
            R.stats[S_VISITS] += (uend - R.u) * (long long)R.N;
            Rg->u = uend;
            Rg->m = mloc;
            Rg->frames_written = fw;
        }
    }
}


// ======================================================================= Ising
// Ising on the row-split cluster schedule: a square lattice with one site
// type and the regular renormalisation (2x2 blocks on even rows and columns,
// each linked to its four neighbour blocks in the same list order at every
// chosen site).  The slabs, ghost rows and pushes are those of the O(n)
// kernel above, on int8 spins; a trial is ising_trial on the local layout
// with the Philox words of the other schedules (block k >> 2 of colour-local
// index k = x*hy + yh, word k & 3).  A measurement is is_frame's integer fast
// path split by slabs: every CTA sums its own sites and its own chosen blocks
// (a block's neighbour across a slab boundary is read from the neighbouring
// CTA's block sums over DSMEM), and rank 0 adds the CTAs' sums in rank order
// and folds them with is_accumulate.  The sums are integers, so the result
// equals the other schedules' to the bit.

// per-CTA sums of one measurement: frame c[0..15] of is_frame, dn[4], dm[4],
// accepted moves; two slots by measurement parity and a third for the counts
// of the sweeps after the last measurement (or before the thermal boundary)
#define CI_NV 25
#define CI_SLOT 32

struct ClusterLayoutI {
    size_t spins, itab, msum, part, acc, total;
    int rows, hy, nloc;
};

__host__ __device__ inline ClusterLayoutI cluster_layout_ising(const Rep &R, int C)
{
    ClusterLayoutI L;
    const int P = R.Lx >> 1;
    const int RP = 2 * (P / C + (P % C ? 1 : 0));  // the largest slab
    L.rows = RP + 2;
    L.hy = R.hy;
    L.nloc = 2 * L.rows * L.hy;
    size_t off = 0;
    L.spins = off; off += a16((size_t)L.nloc);
    L.itab = off; off += a16((size_t)R.nite * sizeof(IsEntry));
    L.msum = off; off += a16((size_t)(RP / 2) * (R.Ly / 2));
    L.part = off; off += 3 * CI_SLOT * sizeof(long long);
    L.acc = off; off += a16((size_t)R.nacc * sizeof(double) + C_NINT * sizeof(long long));
    L.total = off;
    return L;
}

// Rank 0, warp 0: add slot `slot` of every CTA in rank order (lane k sums
// value k, its remote loads issued eight at a time); then lane 0 applies the
// counts to the replica's integer bookkeeping and, for a measurement slot,
// folds the frame (is_frame's fast-path arithmetic) with is_accumulate.
// sum: shared scratch of CI_NV values.
__device__ __noinline__ void cluster_ising_fold(Rep &R, long long *part, int C, int slot, bool frame, long long m,
                                                long long *sum, int lane)
{
    cg::cluster_group cl = cg::this_cluster();
    if (lane < CI_NV) {
        long long a = 0;
        for (int q0 = 0; q0 < C; q0 += 8) {
            long long v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) v[j] = (q0 + j < C) ? cl.map_shared_rank(part, q0 + j)[slot * CI_SLOT + lane] : 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) a += v[j];
        }
        sum[lane] = a;
    }
    __syncwarp();
    if (lane != 0) return;
    const long long *o = sum;
    for (int k = 0; k < MCS_MAXC; ++k) R.icnt[C_DN + k] += -4 * o[16 + k];
    for (int k = 0; k < MCS_MAXT; ++k) R.icnt[C_DM + k] += -2 * o[20 + k];
    R.stats[S_ACCEPT] += o[24];
    if (!frame) return;
    const double S0 = R.Stype[0];
    double Fd[4];
    Fd[0] = S0 * (double)o[0];
    Fd[1] = S0 * (double)o[1];
    Fd[2] = S0 * S0 * (double)o[2];
    double er = 0;
    for (int k = 0; k < 4; ++k) er += R.rKv[k] * (double)o[3 + k];
    Fd[3] = S0 * S0 * er / 2 - R.hd * S0 * (double)o[7];
    long long Fi[MCS_MAXT + MCS_MAXC];
    for (int k = 0; k < MCS_MAXT + MCS_MAXC; ++k) Fi[k] = o[8 + k];
    is_accumulate(R, Fd, Fi, 0, m);
}

template <int NT>
__global__ void __launch_bounds__(NT) k_cluster_ising(Rep *reps, const int *ids, long long max_units, int C)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Rep R;
    __shared__ int wsum[NT / 32][CI_NV];
    __shared__ long long fsum[CI_NV];  // rank 0's gathered sums of one slot
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    Rep *Rg = reps + ids[blockIdx.x / C];
    {
        const int *src = (const int *)Rg;
        int *d = (int *)&R;
        for (int i = threadIdx.x; i < (int)(sizeof(Rep) / 4); i += blockDim.x) d[i] = src[i];
    }
    __syncthreads();
    // every CTA of the cluster reads the same descriptor: the early exit is uniform over the cluster
    if (R.u >= R.u_stop) return;
    const ClusterLayoutI L = cluster_layout_ising(R, C);
    const int tid = threadIdx.x, bd = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = bd >> 5;
    const int hy = L.hy, rows = L.rows, nloc = L.nloc;
    int x0, RP;
    cl_split(R.Lx, C, rank, &x0, &RP);
    const int hb = R.Ly >> 1, half = R.half;
    const int nch = (RP / 2) * hb;  // own chosen blocks
    signed char *s = (signed char *)(smem + L.spins);
    IsEntry *itab = (IsEntry *)(smem + L.itab);
    signed char *msum = (signed char *)(smem + L.msum);
    long long *part = (long long *)(smem + L.part);
    const signed char *G = (const signed char *)R.spins;
    for (int i = tid; i < nloc; i += bd) {
        const int c = i / (rows * hy);
        const int rem = i - c * rows * hy;
        const int xl = rem / hy - 1, yh = rem - (xl + 1) * hy;
        if (xl > RP) continue;  // beyond this slab's bottom ghost row
        int x = x0 + xl;
        if (x < 0) x += R.Lx;
        if (x >= R.Lx) x -= R.Lx;
        s[i] = G[c * half + x * hy + yh];
    }
    for (int k = tid; k < R.nite; k += bd) itab[k] = R.itab[k];
    if (rank == 0) {
        double *a = (double *)(smem + L.acc);
        long long *ic = (long long *)(a + R.nacc);
        for (int k = tid; k < R.nacc; k += bd) a[k] = R.acc[k];
        for (int k = tid; k < C_NINT; k += bd) ic[k] = R.icnt[k];
        __syncthreads();
        if (tid == 0) { R.acc = a; R.icnt = ic; }
    }
    __syncthreads();
    cl.sync();

    const int rprev = (rank + C - 1) % C, rnext = (rank + 1) % C;
    signed char *prev_s = cl.map_shared_rank(s, rprev);
    signed char *next_s = cl.map_shared_rank(s, rnext);
    const signed char *prev_m = cl.map_shared_rank(msum, rprev);
    const signed char *next_m = cl.map_shared_rank(msum, rnext);
    int x0p, RPp, x0n, RPn;  // the previous slab's bottom ghost row is its local row RPp + 1
    cl_split(R.Lx, C, rprev, &x0p, &RPp);
    cl_split(R.Lx, C, rnext, &x0n, &RPn);
    (void)x0n; (void)RPn;
    const SqLinks sql = {R.Ly, hy, rows, R.sq_code[0], R.sq_code[1], R.sq_code[2], R.sq_code[3]};
    const int k_lo = x0 * hy, k_hi = (x0 + RP) * hy;  // own colour-local indices
    const int q_lo = k_lo >> 2, q_hi = (k_hi + 3) >> 2;

    int dn[MCS_MAXC] = {0, 0, 0, 0}, dm[MCS_MAXT] = {0, 0, 0, 0}, nacc = 0;
    int frame[16];
    // this CTA's per-thread counts and frame sums -> slot (fixed order of warps).
    // The leading barrier keeps warp 0's reads of wsum in the previous call
    // (a launch's last measurement is followed at once by the closing call)
    // ahead of this call's writes.
    // the frame sums over the own sites of colour c: the pair sums (every site
    // is its own pair), the sign sum and the per-class bond sums of the full
    // recompute; a colour-c site's neighbours have colour 1 - c
    auto site_sums = [&](int c) {
        SqWalk wk;
        wk.init(tid, bd, hy);
        for (int k = tid; k < RP * hy; k += bd, wk.next()) {
            const int xl = wk.x, yh = wk.yh;
            const int li = c * rows * hy + (xl + 1) * hy + yh;
            const int si = s[li];
            int idx = R.ibase[0];
            cl_links_r(sql, c, xl, yh, [&](int, int j, int code) { if (s[j] > 0) idx += code; });
            const int nc = itab[idx].nc;
            frame[0] += si; frame[1] += si; frame[2] += si * si;
            frame[8] += si;
            frame[12] += si * (int)(signed char)(nc & 0xff);
            frame[13] += si * (int)(signed char)((nc >> 8) & 0xff);
            frame[14] += si * (int)(signed char)((nc >> 16) & 0xff);
            frame[15] += si * (int)(signed char)((nc >> 24) & 0xff);
        }
    };
    auto to_slot = [&](int slot, bool with_frame) {
        __syncthreads();
        int v[CI_NV];
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] = with_frame ? frame[k] : 0;
#pragma unroll
        for (int k = 0; k < MCS_MAXC; ++k) v[16 + k] = dn[k];
#pragma unroll
        for (int k = 0; k < MCS_MAXT; ++k) v[20 + k] = dm[k];
        v[24] = nacc;
#pragma unroll
        for (int k = 0; k < CI_NV; ++k) {
            const int w = __reduce_add_sync(0xffffffffu, v[k]);
            if (lane == 0) wsum[wid][k] = w;
        }
        __syncthreads();
        if (tid < CI_NV) {
            long long a = 0;
            for (int w = 0; w < nw; ++w) a += wsum[w][tid];
            part[slot * CI_SLOT + tid] = a;
        }
#pragma unroll
        for (int k = 0; k < MCS_MAXC; ++k) dn[k] = 0;
#pragma unroll
        for (int k = 0; k < MCS_MAXT; ++k) dm[k] = 0;
        nacc = 0;
    };

    long long mloc = R.m;
    int fw = R.frames_written;
    int pending = -1;  // measurement slot not yet folded (rank 0 folds it at the next measurement)
    long long pending_m = 0;
    long long u = R.u;
    const long long uend = min(R.u_stop, u + max_units);
    for (; u < uend; ++u) {
        if (R.alg == 0 && u == R.units_thermal) {
            // the thermal boundary: the counts so far give the reference's energy offset
            to_slot(2, false);
            cl.sync();
            if (rank == 0 && tid < 32) {
                if (pending >= 0) cluster_ising_fold(R, part, C, pending, true, pending_m, fsum, tid);
                __syncwarp();
                cluster_ising_fold(R, part, C, 2, false, 0, fsum, tid);
            }
            pending = -1;
            if (rank == 0 && tid == 0) {
                double Einc = 0;
                for (int c = 0; c < R.nclass; ++c) Einc += 0.5 * R.Q[c] * (double)R.icnt[C_DN + c];
                for (int t = 0; t < R.ntype; ++t) Einc -= R.hd * R.Stype[t] * (double)R.icnt[C_DM + t];
                R.acc[B_EMEAS0] = Einc;
            }
            cl.sync();
        }
        const long long t = R.u0 + u;
        const bool meas = measures_after(R, u);
        for (int c = 0; c < 2; ++c) {
            const int cb = c * rows * hy;
            SqWalk wq;  // (row, half-column) of each block's first site, without divisions
            wq.init(4 * (q_lo + tid), 4 * bd, hy);
            for (int q = q_lo + tid; q < q_hi; q += bd, wq.next()) {
                const uint4 w = philox_t((uint32_t)q, t, (uint32_t)c, R.seed);
                const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
                int x = wq.x, yh = wq.yh;  // walked along the block's four sites
#pragma unroll
                for (int e = 0; e < 4; ++e, ++yh) {
                    if (yh == hy) { yh = 0; ++x; }
                    const int k = 4 * q + e;
                    if (k < k_lo || k >= k_hi) continue;
                    const int xl = x - x0;
                    const int li = cb + (xl + 1) * hy + yh;
                    const bool a = ising_trial(R, itab, s, li, 0, ws[e], [&](auto &&f) { cl_links_r(sql, c, xl, yh, f); },
                                               dn, dm);
                    if (a) {
                        ++nacc;
                        // own row 0 is the previous CTA's bottom ghost (its local row
                        // RPp+1), own row RP-1 the next CTA's top ghost (local row 0)
                        if (xl == 0) prev_s[cb + (RPp + 1) * hy + yh] = s[li];
                        if (xl == RP - 1) next_s[cb + yh] = s[li];
                    }
                }
            }
            if (c == 1 && meas) {
                // own sites are final: the sums of the own chosen blocks
                // (2x2 blocks on even rows and columns lie inside the slab),
                // published by the colour's cluster barrier, and the colour-1
                // site sums, whose colour-0 neighbours (ghost rows included)
                // no CTA changes before this barrier
                __syncthreads();
                SqWalk wb;
                wb.init(tid, bd, hb);
                for (int lq = tid; lq < nch; lq += bd, wb.next()) {
                    const int br = wb.x, bc = wb.yh, xl = 2 * br;
                    msum[lq] = (signed char)(s[(xl + 1) * hy + bc] + s[rows * hy + (xl + 1) * hy + bc] +
                                             s[rows * hy + (xl + 2) * hy + bc] + s[(xl + 2) * hy + bc]);
                }
#pragma unroll
                for (int k = 0; k < 16; ++k) frame[k] = 0;
                site_sums(1);
            }
            cl.sync();
        }
        if (!meas) continue;
        // rank 0 folds the previous measurement (every CTA wrote its slot
        // before this sweep's barriers)
        if (rank == 0 && tid < 32 && pending >= 0) cluster_ising_fold(R, part, C, pending, true, pending_m, fsum, tid);
        // the colour-0 site sums read own colour-0 sites and colour-1
        // neighbours, which the next sweep's colour-0 phase leaves alone in
        // every CTA (its pushes go to colour-0 ghost rows)
        site_sums(0);
        // own chosen blocks: majority with the engine's tie-breaks, its
        // renormalised links to the four neighbour blocks (list slot and
        // coupling class per direction)
        SqWalk wb;
        wb.init(tid, bd, hb);
        for (int lq = tid; lq < nch; lq += bd, wb.next()) {
            const int br = wb.x, bc = wb.yh, xl = 2 * br;
            const uint32_t j = (uint32_t)((x0 + xl) * hy + bc);  // sweep index of the chosen site (colour 0)
            const int mj = is_majority_lazy(msum[lq], j, mloc, 0, R.seed);
            const int bcp = bc + 1 == hb ? 0 : bc + 1, bcm = bc == 0 ? hb - 1 : bc - 1;
            int tsum[4];
            tsum[0] = (br + 1 < RP / 2) ? msum[lq + hb] : next_m[bc];
            tsum[1] = (br > 0) ? msum[lq - hb] : prev_m[(RPp / 2 - 1) * hb + bc];
            tsum[2] = msum[br * hb + bcp];
            tsum[3] = msum[br * hb + bcm];
            const int kind = (x0 + xl == 0 ? 1 : 0) | (bc == 0 ? 2 : 0);
#pragma unroll
            for (int d = 0; d < 4; ++d) {
                const int mt = is_majority_lazy(tsum[d], j, mloc, 1 + R.rdir_slot[4 * kind + d], R.seed);
                const int kc = R.rdir_cls[d];
#pragma unroll
                for (int q = 0; q < 4; ++q) frame[3 + q] += (q == kc) ? mj * mt : 0;
            }
            frame[7] += s[(xl + 1) * hy + bc];
        }
        to_slot((int)(mloc & 1), true);
        if (R.frames > 0 && (mloc % R.frame_every) == 0 && fw < R.frames) {
            Spins S;
            S.s = s;
            for (int i = tid; i < 2 * RP * hy; i += bd) {
                const int c = i / (RP * hy), k = i - c * RP * hy;
                const int xl = k / hy, yh = k - xl * hy;
                frame_store<1>(R, fw, c * half + (x0 + xl) * hy + yh, S, c * rows * hy + (xl + 1) * hy + yh);
            }
            ++fw;
            __syncthreads();  // every own site stored before the next colour-0 phase changes them
        }
        pending = (int)(mloc & 1);
        pending_m = mloc;
        ++mloc;
        // no cluster barrier here: the measurement read colour-0 ghost rows only
        // before the colour-1 barrier, and the neighbour block sums it reads are
        // rewritten only after the next sweep's colour-0 barrier
    }
    // the counts after the last measurement -> slot 2
    to_slot(2, false);
    cl.sync();
    if (rank == 0 && tid < 32) {
        if (pending >= 0) cluster_ising_fold(R, part, C, pending, true, pending_m, fsum, tid);
        __syncwarp();
        cluster_ising_fold(R, part, C, 2, false, 0, fsum, tid);
    }
    // rank 0 has read every CTA's slots before any CTA exits
    cl.sync();
    signed char *Gw = (signed char *)R.spins;
    for (int i = tid; i < 2 * RP * hy; i += bd) {
        const int c = i / (RP * hy), k = i - c * RP * hy;
        const int xl = k / hy, yh = k - xl * hy;
        Gw[c * half + (x0 + xl) * hy + yh] = s[c * rows * hy + (xl + 1) * hy + yh];
    }
    if (rank == 0) {
        __syncthreads();
        for (int k = tid; k < R.nacc; k += bd) Rg->acc[k] = R.acc[k];
        for (int k = tid; k < C_NINT; k += bd) Rg->icnt[k] = R.icnt[k];
        if (tid == 0) {
            R.stats[S_VISITS] += (uend - R.u) * (long long)R.N;
            Rg->u = uend;
            Rg->m = mloc;
            Rg->frames_written = fw;
        }
    }
}

long long cluster_smem_bytes(const Rep &r, int C)
{
    return r.dim == 1 ? (long long)cluster_layout_ising(r, C).total : (long long)cluster_layout(r, C).total;
}

// Load the cluster kernels on the current device (see preload_kernels_main).
cudaError_t preload_kernels_cluster()
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<2, 256>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_ising<256>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_ising<512>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_ising<1024>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<2, 512>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<2, 1024>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<3, 256>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<3, 512>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, (const void *)k_cluster_metro<3, 1024>);
    return e;
}

// The cluster kernel of a spin dimension (1: Ising).
template <int DIM, int NT>
static auto cluster_kernel()
{
    if constexpr (DIM == 1) return &k_cluster_ising<NT>;
    else return &k_cluster_metro<DIM, NT>;
}

// Shared-memory and cluster-size attributes of one instantiation (set once,
// raised when a larger request comes).
template <int DIM, int NT>
static cudaError_t prep_cluster_kernel(size_t smem, int C)
{
    static size_t done = 0;
    static bool nonportable = false;
    if (smem > done) {
        cudaError_t e = cudaFuncSetAttribute(cluster_kernel<DIM, NT>(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        done = smem;
    }
    if (C > 8 && !nonportable) {  // clusters above 8 CTAs are an opt-in
        cudaError_t e = cudaFuncSetAttribute(cluster_kernel<DIM, NT>(), cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        nonportable = true;
    }
    return cudaSuccess;
}

template <int DIM, int NT>
static void cluster_config(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr, int nrep, int C, size_t smem,
                           cudaStream_t st)
{
    cfg = {};
    cfg.gridDim = dim3(nrep * C, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
}

template <int DIM, int NT>
static cudaError_t launch_cluster_t(Rep *reps, const int *ids, int nrep, int C, size_t smem, long long max_units,
                                    cudaStream_t st)
{
    cudaError_t e = prep_cluster_kernel<DIM, NT>(smem, C);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config<DIM, NT>(cfg, attr, nrep, C, smem, st);
    return cudaLaunchKernelEx(&cfg, cluster_kernel<DIM, NT>(), reps, ids, max_units, C);
}

// Clusters of this shape the device can hold at once (0: it cannot launch one).
template <int DIM, int NT>
static int cluster_active_t(int C, size_t smem)
{
    if (prep_cluster_kernel<DIM, NT>(smem, C) != cudaSuccess) { cudaGetLastError(); return 0; }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    cluster_config<DIM, NT>(cfg, attr, 1, C, smem, 0);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, cluster_kernel<DIM, NT>(), &cfg) != cudaSuccess) { cudaGetLastError(); return 0; }
    return n;
}

int cluster_active(int dim, int C, int threads, size_t smem)
{
    if (dim == 1) {
        if (threads == 256) return cluster_active_t<1, 256>(C, smem);
        if (threads == 512) return cluster_active_t<1, 512>(C, smem);
        if (threads == 1024) return cluster_active_t<1, 1024>(C, smem);
    } else if (dim == 2) {
        if (threads == 256) return cluster_active_t<2, 256>(C, smem);
        if (threads == 512) return cluster_active_t<2, 512>(C, smem);
        if (threads == 1024) return cluster_active_t<2, 1024>(C, smem);
    } else if (dim == 3) {
        if (threads == 256) return cluster_active_t<3, 256>(C, smem);
        if (threads == 512) return cluster_active_t<3, 512>(C, smem);
        if (threads == 1024) return cluster_active_t<3, 1024>(C, smem);
    }
    return 0;
}

template <int DIM>
static cudaError_t launch_cluster_d(Rep *reps, const int *ids, int nrep, int C, int threads, size_t smem,
                                    long long max_units, cudaStream_t st)
{
    if (threads == 256) return launch_cluster_t<DIM, 256>(reps, ids, nrep, C, smem, max_units, st);
    if (threads == 512) return launch_cluster_t<DIM, 512>(reps, ids, nrep, C, smem, max_units, st);
    if (threads == 1024) return launch_cluster_t<DIM, 1024>(reps, ids, nrep, C, smem, max_units, st);
    return cudaErrorInvalidValue;
}

cudaError_t launch_cluster_metro(int dim, Rep *reps, const int *ids, int nrep, int C, int threads, size_t smem,
                                 long long max_units, cudaStream_t st)
{
    if (nrep <= 0) return cudaSuccess;
    if (dim == 1) return launch_cluster_d<1>(reps, ids, nrep, C, threads, smem, max_units, st);
    if (dim == 2) return launch_cluster_d<2>(reps, ids, nrep, C, threads, smem, max_units, st);
    return launch_cluster_d<3>(reps, ids, nrep, C, threads, smem, max_units, st);
}

}  // namespace mcs
