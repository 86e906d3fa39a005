// mcs_kernels.cu -- sm_103a kernels of the Monte Carlo engine.
//
// Schedules
//   resident : one CTA owns one replica; its whole lattice, coupling tables and
//              reduction scratch live in shared memory; the CTA runs many sweeps
//              (and the measurements between them) per launch.  Lattices up to
//              ~220 KB of spin state (Heisenberg L=128, XY L~165, Ising L~470).
//   tiled    : the lattice lives in global memory (L2-resident for the sizes of
//              interest); one launch per colour updates that colour of every
//              replica of the group, tile by tile; a measurement launch writes
//              per-tile partial sums and a finalize launch (one CTA per replica)
//              folds them in a fixed order.
//   resident with copies: a thread-block cluster of C CTAs (C = 2 or 4) per
//              replica, each holding a full copy of the lattice; a colour phase
//              is shared out among the CTAs, every accepted move is stored into
//              every copy (DSMEM), and one cluster barrier ends the phase.
//              Measurements split the index range among the CTAs; rank 0 sums
//              the partial frames and owns the accumulators.  For lattices that
//              fit one CTA but would leave SMs idle (few replicas, any geometry).
// Both schedules call the same per-site update, so a replica's spin trajectory
// does not depend on the schedule or on the other replicas of the batch.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mcs_device.cuh"
#include "mcs_internal.h"
#include "mcs_wolff.cuh"

namespace cg = cooperative_groups;

namespace mcs {

static __host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

#define MCS_RED_DOUBLES MCS_RED

struct SmemLayout {
    size_t spins, tables, stype, majc, red, F, redl, Fi, acc, total;
    size_t il_rorb, il_rdeg, il_tgt, il_kc;  // staged Ising chosen-site lists (0: not staged)
    size_t il_cp, il_rcl;                    // staged Ising pair and block lists (0: not staged)
};
// Shared-memory plan of a resident replica.  The block-spin cache of the
// renormalised lattice is included only when it fits (flag returned in majc
// != 0).
__host__ __device__ inline SmemLayout smem_layout(const Rep &R, size_t limit = 232448)
{
    SmemLayout L;
    size_t off = 0;
    L.spins = off;
    if (R.dim == 1) off += align16((size_t)R.N);
    else off += align16((size_t)R.dim * R.N * sizeof(float));
    L.tables = off;
    if (R.dim == 1) off += align16((size_t)R.nite * sizeof(IsEntry));
    else off += align16((size_t)R.njc * 9 * sizeof(float) + (size_t)R.ndc * 4 * sizeof(float));
    L.stype = off;
    bool need_st = R.dim == 1 ? R.ntype > 1 : R.ndc > 1;
    if (need_st) off += align16((size_t)R.N);
    L.red = off; off += MCS_RED_DOUBLES * sizeof(double);
    L.F = off; off += F_NON * sizeof(double);
    L.redl = off; off += (32 * 16 + 16) * sizeof(long long);
    L.Fi = off; off += 16 * sizeof(long long);
    L.acc = off; off += align16((size_t)R.nacc * sizeof(double) + C_NINT * sizeof(long long));
    L.majc = 0;  // O(n): block spins of the chosen sites; Ising: their sign sums
    size_t mbytes = R.dim > 1 ? align16((size_t)R.n_rorb * 3 * sizeof(float)) : align16((size_t)R.n_rorb);
    if (off + mbytes <= limit) { L.majc = off; off += mbytes; }
    // Ising with one spin length: the chosen-site lists of the frame, when they fit
    L.il_rorb = L.il_rdeg = L.il_tgt = L.il_kc = 0;
    if (R.dim == 1 && R.is_fast && L.majc) {
        const size_t nz = (size_t)R.n_rorb * (R.zmax > 0 ? R.zmax : 1);
        const size_t need = align16((size_t)R.n_rorb * 4) + align16((size_t)R.n_rorb) + align16(nz * 4) + align16(nz);
        if (off + need <= limit) {
            L.il_rorb = off; off += align16((size_t)R.n_rorb * 4);
            L.il_rdeg = off; off += align16((size_t)R.n_rorb);
            L.il_tgt = off; off += align16(nz * 4);
            L.il_kc = off; off += align16(nz);
        }
    }
    // and the correlated pairs and the block members, when they fit as well
    L.il_cp = L.il_rcl = 0;
    if (L.il_rorb) {
        const size_t need = align16((size_t)R.nlat * 2 * 4) + align16((size_t)R.n_rorb * R.ncl * 4);
        if (off + need <= limit) {
            L.il_cp = off; off += align16((size_t)R.nlat * 2 * 4);
            L.il_rcl = off; off += align16((size_t)R.n_rorb * R.ncl * 4);
        }
    }
    L.total = off;
    return L;
}

long long resident_smem_bytes(const Rep &r) { return (long long)smem_layout(r).total; }

int resident_max_smem()
{
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v;
}

// The FP64 accumulators and the Ising integer counters of a replica are kept
// in shared memory for the life of a launch (thread 0 updates them at every
// measurement) and written back at its end.
__device__ __forceinline__ void acc_to_smem(Rep &R, unsigned char *buf)
{
    double *a = (double *)buf;
    long long *ic = (long long *)(a + R.nacc);
    for (int k = threadIdx.x; k < R.nacc; k += blockDim.x) a[k] = R.acc[k];
    for (int k = threadIdx.x; k < C_NINT; k += blockDim.x) ic[k] = R.icnt[k];
    __syncthreads();
    if (threadIdx.x == 0) { R.acc = a; R.icnt = ic; }
    __syncthreads();
}
__device__ __forceinline__ void acc_to_global(const Rep &R, const Rep *Rg)
{
    for (int k = threadIdx.x; k < R.nacc; k += blockDim.x) Rg->acc[k] = R.acc[k];
    for (int k = threadIdx.x; k < C_NINT; k += blockDim.x) Rg->icnt[k] = R.icnt[k];
}

// copy the replica descriptor into shared memory with all threads
__device__ __forceinline__ void load_rep(Rep &dst, const Rep *src)
{
    const int *s = (const int *)src;
    int *d = (int *)&dst;
    for (int i = threadIdx.x; i < (int)(sizeof(Rep) / 4); i += blockDim.x) d[i] = s[i];
    __syncthreads();
}

// ======================================================================= resident Metropolis
template <int DIM, int GEOM>
__global__ void __launch_bounds__(1024) k_resident_metro(Rep *reps, const int *ids, long long max_units, int C)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Rep R;
    __shared__ float fsx[MCS_FS_STRIDE];  // FP32 frame for the warp fold
    cg::cluster_group cl = cg::this_cluster();
    const int rank = C > 1 ? (int)cl.block_rank() : 0;
    Rep *Rg = reps + ids[blockIdx.x / C];
    load_rep(R, Rg);
    if (R.u >= R.u_stop) return;
    const SmemLayout L = smem_layout(R);
    const int tid = threadIdx.x, bd = blockDim.x, N = R.N;
    double *red = (double *)(smem + L.red);
    double *F = (double *)(smem + L.F);
    long long *redl = (long long *)(smem + L.redl);
    long long *Fi = (long long *)(smem + L.Fi);
    float *majc = L.majc ? (float *)(smem + L.majc) : nullptr;
    Spins S;
    Spins G = spins_global(R);
    IsEntry *itab = (IsEntry *)(smem + L.tables);
    float *jt = (float *)(smem + L.tables);
    float *dt = jt + R.njc * 9;
    const bool multi = DIM == 1 ? R.ntype > 1 : R.ndc > 1;
    unsigned char *st = multi ? (unsigned char *)(smem + L.stype) : nullptr;
    if (multi)
        for (int v = tid; v < N; v += bd) st[v] = R.stype[v];
    if (DIM == 1) {
        S.s = (signed char *)(smem + L.spins);
        for (int v = tid; v < N; v += bd) S.s[v] = G.s[v];
        for (int k = tid; k < R.nite; k += bd) itab[k] = R.itab[k];
    } else {
        S.x = (float *)(smem + L.spins);
        S.y = S.x + N;
        S.z = S.y + N;
        for (int v = tid; v < N; v += bd) {
            S.x[v] = G.x[v]; S.y[v] = G.y[v];
            if (DIM == 3) S.z[v] = G.z[v];
        }
        for (int k = tid; k < R.njc * 9; k += bd) jt[k] = R.jtab[k];
        for (int k = tid; k < R.ndc * 4; k += bd) dt[k] = R.dtab[k];
    }
    IsLists il;
    il.rorb = nullptr;
    if (DIM == 1 && L.il_rorb) {
        int *rorb = (int *)(smem + L.il_rorb);
        unsigned char *rdeg = smem + L.il_rdeg;
        int *tgt = (int *)(smem + L.il_tgt);
        unsigned char *kc = smem + L.il_kc;
        const int z = R.zmax > 0 ? R.zmax : 1;
        for (int r = tid; r < R.n_rorb; r += bd) { rorb[r] = R.rorb[r]; rdeg[r] = R.rdeg[r]; }
        for (int i = tid; i < R.n_rorb * z; i += bd) {
            tgt[i] = R.rlink[i] < 0 ? -2 : R.rtgt[i];
            kc[i] = R.rkc[i];
        }
        il.rorb = rorb; il.rdeg = rdeg; il.tgt = tgt; il.kc = kc;
        il.cp = nullptr; il.rcl = nullptr;
        if (L.il_cp) {
            int *cp = (int *)(smem + L.il_cp);
            int *rcl = (int *)(smem + L.il_rcl);
            for (int i = tid; i < 2 * R.nlat; i += bd) cp[i] = R.cpair[i];
            for (int i = tid; i < R.n_rorb * R.ncl; i += bd) rcl[i] = R.rcl[i];
            il.cp = cp; il.rcl = rcl;
        }
    }
    __syncthreads();
    acc_to_smem(R, smem + L.acc);

    // the other copies of this replica (C > 1): an accepted move is stored
    // into each of them as well
    float *rx[3] = {nullptr, nullptr, nullptr}, *ry[3] = {nullptr, nullptr, nullptr}, *rz[3] = {nullptr, nullptr, nullptr};
    signed char *rs[3] = {nullptr, nullptr, nullptr};
    int nrem = 0;
    for (int q = 0; q < C && C > 1; ++q) {
        if (q == rank) continue;
        if (DIM == 1) rs[nrem] = cl.map_shared_rank(S.s, q);
        else {
            rx[nrem] = cl.map_shared_rank(S.x, q);
            ry[nrem] = cl.map_shared_rank(S.y, q);
            if (DIM == 3) rz[nrem] = cl.map_shared_rank(S.z, q);
        }
        ++nrem;
    }
    // rank 0 adds the other CTAs' values of buf[0..n) to its own (fixed rank order)
    auto cl_sum = [&](auto *buf, int n) {
        if (C <= 1) return;
        cl.sync();
        if (rank == 0)
            for (int k = tid; k < n; k += bd) {
                auto a = buf[k];
                for (int q = 1; q < C; ++q) a += cl.map_shared_rank(buf, q)[k];
                buf[k] = a;
            }
        cl.sync();
    };

    int dn[MCS_MAXC] = {0, 0, 0, 0}, dm[MCS_MAXT] = {0, 0, 0, 0};
    long long nacc = 0;
    double dEd = 0.0;
    const float beta = R.beta, h = R.h;

    auto fold = [&]() {
        if (DIM == 1) {
            long long c[MCS_MAXC + MCS_MAXT + 1];
#pragma unroll
            for (int k = 0; k < MCS_MAXC; ++k) c[k] = dn[k];
#pragma unroll
            for (int k = 0; k < MCS_MAXT; ++k) c[MCS_MAXC + k] = dm[k];
            c[MCS_MAXC + MCS_MAXT] = nacc;
            block_sum_ll<MCS_MAXC + MCS_MAXT + 1>(c, redl, Fi);
            cl_sum(Fi, MCS_MAXC + MCS_MAXT + 1);
            if (rank == 0 && tid == 0) {
                for (int k = 0; k < MCS_MAXC; ++k) R.icnt[C_DN + k] += -4 * Fi[k];
                for (int k = 0; k < MCS_MAXT; ++k) R.icnt[C_DM + k] += -2 * Fi[MCS_MAXC + k];
                R.stats[S_ACCEPT] += Fi[MCS_MAXC + MCS_MAXT];
            }
#pragma unroll
            for (int k = 0; k < MCS_MAXC; ++k) dn[k] = 0;
#pragma unroll
            for (int k = 0; k < MCS_MAXT; ++k) dm[k] = 0;
        } else {
            double c[2] = {dEd, (double)nacc};
            block_sum<2>(c, red, F);
            cl_sum(F, 2);
            if (rank == 0 && tid == 0) {
                R.acc[A_ECUR] += F[0];
                R.stats[S_ACCEPT] += (long long)F[1];
            }
            dEd = 0.0;
        }
        nacc = 0;
        __syncthreads();
    };

    long long u = R.u;
    const long long uend = min(R.u_stop, u + max_units);
    for (; u < uend; ++u) {
        if (DIM == 1 && u == R.units_thermal) {
            fold();
            if (rank == 0 && tid == 0) {
                double Einc = 0;
                for (int c = 0; c < R.nclass; ++c) Einc += 0.5 * R.Q[c] * (double)R.icnt[C_DN + c];
                for (int t = 0; t < R.ntype; ++t) Einc -= R.hd * R.Stype[t] * (double)R.icnt[C_DM + t];
                R.acc[B_EMEAS0] = Einc;
            }
        }
        const long long t = R.u0 + u;
        for (int c = 0; c < R.ncol; ++c) {
            const int c0 = R.col_start[c], nc = R.col_start[c + 1] - c0;
            if (DIM == 1) {
                const int nq = (nc + 3) >> 2;
                SqWalk wk;
                // with copies the colour is dealt out among the C CTAs
                const int q0 = rank * bd + tid, qs = C * bd;
                if (GEOM == MCS_GEOM_SQUARE) wk.init(4 * q0, 4 * qs, R.hy);
                for (int q = q0; q < nq; q += qs) {
                    uint4 w = philox_t((uint32_t)q, t, (uint32_t)c, R.seed);
                    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
                    int x = 0, yh = 0;
                    if (GEOM == MCS_GEOM_SQUARE) { x = wk.x; yh = wk.yh; }
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int k = 4 * q + e;
                        if (k < nc) {
                            const int v = c0 + k;
                            const int ty = multi ? st[v] : 0;
                            bool a;
                            if (GEOM == MCS_GEOM_SQUARE)
                                a = ising_trial(R, itab, S.s, v, ty, ws[e], [&](auto &&f) { sq_links(R, c, x, yh, f); }, dn, dm);
                            else
                                a = ising_trial(R, itab, S.s, v, ty, ws[e], [&](auto &&f) { for_links<GEOM>(R, v, f); }, dn, dm);
                            nacc += a;
                            if (a)
                                for (int i = 0; i < nrem; ++i) rs[i][v] = S.s[v];
                        }
                        if (GEOM == MCS_GEOM_SQUARE) { if (++yh == R.hy) { yh = 0; ++x; } }
                    }
                    if (GEOM == MCS_GEOM_SQUARE) wk.next();
                }
            } else {
                float dEf = 0.f;
                SqWalk wk;
                const int k0 = rank * bd + tid, ks = C * bd;  // shared out among the copies
                if (GEOM == MCS_GEOM_SQUARE) wk.init(k0, ks, R.hy);
                for (int k = k0; k < nc; k += ks) {
                    const int v = c0 + k;
                    uint4 w = on_words<DIM>((uint32_t)k, t, (uint32_t)c, R.seed);
                    const int dc = multi ? st[v] : 0;
                    float dE;
                    bool a;
                    if (GEOM == MCS_GEOM_SQUARE)
                        a = on_trial<DIM>(R, jt, dt, S, v, dc, w, beta, h, [&](auto &&f) { sq_links(R, c, wk.x, wk.yh, f); }, &dE);
                    else
                        a = on_trial<DIM>(R, jt, dt, S, v, dc, w, beta, h, [&](auto &&f) { for_links<GEOM>(R, v, f); }, &dE);
                    if (a) {
                        dEf += dE;
                        ++nacc;
                        for (int i = 0; i < nrem; ++i) {
                            rx[i][v] = S.x[v];
                            ry[i][v] = S.y[v];
                            if (DIM == 3) rz[i][v] = S.z[v];
                        }
                    }
                    if (GEOM == MCS_GEOM_SQUARE) wk.next();
                }
                dEd += (double)dEf;
            }
            // every copy holds this colour's new spins before the next phase reads them
            if (C > 1) cl.sync();
            else __syncthreads();
        }
        if (measures_after(R, u)) {
            fold();
            const long long m = R.m;
            if (DIM == 1) {
                const int V = max(N, max(R.nlat, R.n_rorb)), share = (V + C - 1) / C;
                const int vb = min(V, rank * share), ve = min(V, vb + share);
                is_frame<GEOM>(R, itab, S.s, vb, ve, m, red, F, redl, Fi,
                               L.majc ? (signed char *)(smem + L.majc) : nullptr, il.rorb ? &il : nullptr);
                cl_sum(F, 4);
                cl_sum(Fi, MCS_MAXT + MCS_MAXC);
                if (rank == 0 && tid == 0) {
                    if (R.alg == 1 && u >= R.units_thermal) R.icnt[C_ACC_MEAS] = 1;
                    is_accumulate(R, F, Fi, S.s[R.last_site], m);
                }
            } else {
                const bool efull = (m % R.recheck) == 0;
                const int V = max(max(N, R.nlat), max(R.n_rorb, R.ncirc)), share = (V + C - 1) / C;
                const int vb = min(V, rank * share), ve = min(V, vb + share);
                on_frame<DIM, GEOM>(R, jt, dt, S, vb, ve, efull, red, F, majc);
                cl_sum(F, F_NON);
                if (rank == 0 && tid == 0 && efull) {
                    double Ef = F[F_EFB] / 2 + F[F_EFO];
                    double d = fabs(R.acc[A_ECUR] - Ef);
                    if (d > R.acc[A_DRIFT]) R.acc[A_DRIFT] = d;
                    R.acc[A_ECUR] = Ef;
                }
                if (rank == 0 && tid < 32) {
                    __syncwarp();
                    for (int f = tid; f < F_NON; f += 32) fsx[f] = (float)F[f];
                    __syncwarp();
                    on_accumulate_frames<DIM>(R, fsx, &R.acc[A_ECUR], m, 1, tid);
                }
            }
            if (rank == 0 && R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames)
                for (int v = tid; v < N; v += bd) frame_store<DIM>(R, R.frames_written, v, S, v);
            __syncthreads();
            if (tid == 0) {
                if (R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames) R.frames_written++;
                R.m = m + 1;
            }
            // rank 0 has read its copy (frames, the last site): only now may
            // the next colour phase store into it
            if (C > 1) cl.sync();
            else __syncthreads();
        }
    }
    fold();
    if (rank != 0) return;  // the copies are identical; rank 0 writes the replica back
    acc_to_global(R, Rg);
    for (int v = tid; v < N; v += bd) {
        if (DIM == 1) G.s[v] = S.s[v];
        else {
            G.x[v] = S.x[v]; G.y[v] = S.y[v];
            if (DIM == 3) G.z[v] = S.z[v];
        }
    }
    if (tid == 0) {
        R.stats[S_VISITS] += (uend - R.u) * (long long)N;
        Rg->u = uend;
        Rg->m = R.m;
        Rg->frames_written = R.frames_written;
    }
}

// ======================================================================= tiled Metropolis
template <int DIM, int GEOM>
__global__ void __launch_bounds__(256) k_tiled_sweep(Rep *reps, const Item *items, int colour, double *dEpart,
                                                     long long *ipart)
{
    __shared__ double red[32 * 2 + 4];
    __shared__ long long redl[32 * 9 + 9];
    // the descriptor in shared memory: its fields are read in every trial,
    // and from global memory every spin store (which might alias them)
    // would make the compiler read them again
    __shared__ Rep R;
    const Item it = items[blockIdx.x];
    load_rep(R, reps + it.rep);
    if (R.u >= R.u_stop) return;
    const long long t = R.u0 + R.u;
    const int c = colour, c0 = R.col_start[c];
    Spins S = spins_global(R);
    const int tid = threadIdx.x;
    const bool multi = DIM == 1 ? R.ntype > 1 : R.ndc > 1;
    if (DIM == 1) {
        int dn[MCS_MAXC] = {0, 0, 0, 0}, dm[MCS_MAXT] = {0, 0, 0, 0};
        long long nacc = 0;
        const int k0 = it.begin + 4 * tid;
        if (k0 < it.end) {
            uint4 w = philox_t((uint32_t)(k0 >> 2), t, (uint32_t)c, R.seed);
            const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
            int x = 0, yh = 0;
            if (GEOM == MCS_GEOM_SQUARE) { x = k0 / R.hy; yh = k0 - x * R.hy; }
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int k = k0 + e;
                if (k < it.end) {
                    const int v = c0 + k;
                    const int ty = multi ? R.stype[v] : 0;
                    bool a;
                    if (GEOM == MCS_GEOM_SQUARE)
                        a = ising_trial(R, R.itab, S.s, v, ty, ws[e], [&](auto &&f) { sq_links(R, c, x, yh, f); }, dn, dm);
                    else
                        a = ising_trial(R, R.itab, S.s, v, ty, ws[e], [&](auto &&f) { for_links<GEOM>(R, v, f); }, dn, dm);
                    nacc += a;
                }
                if (GEOM == MCS_GEOM_SQUARE) { if (++yh == R.hy) { yh = 0; ++x; } }
            }
        }
        long long v[9] = {dn[0], dn[1], dn[2], dn[3], dm[0], dm[1], dm[2], dm[3], nacc};
        block_sum_ll<9>(v, redl, redl + 32 * 9);
        if (tid < 9) ipart[(size_t)it.slot * 9 + tid] = redl[32 * 9 + tid];
    } else {
        float dEf = 0.f;
        unsigned nacc = 0;
        const int k = it.begin + tid;
        if (k < it.end) {
            const int v = c0 + k;
            uint4 w = on_words<DIM>((uint32_t)k, t, (uint32_t)c, R.seed);
            const int dc = multi ? R.stype[v] : 0;
            float dE;
            bool a;
            if (GEOM == MCS_GEOM_SQUARE) {
                const int x = k / R.hy, yh = k - x * R.hy;
                a = on_trial<DIM>(R, R.jtab, R.dtab, S, v, dc, w, R.beta, R.h, [&](auto &&f) { sq_links(R, c, x, yh, f); }, &dE);
            } else {
                a = on_trial<DIM>(R, R.jtab, R.dtab, S, v, dc, w, R.beta, R.h, [&](auto &&f) { for_links<GEOM>(R, v, f); }, &dE);
            }
            if (a) { dEf = dE; nacc = 1; }
        }
        // energy change: FP32 inside each warp, FP64 across the warps; the
        // accepted count as an integer (one warp reduction instruction)
        const unsigned cnt = __reduce_add_sync(0xffffffffu, nacc);
        if ((tid & 31) == 0) redl[tid >> 5] = (long long)cnt;
        float v[1] = {dEf};
        block_sum_f<1>(v, red, red + 64);  // its barriers also publish redl
        if (tid == 0) {
            long long n = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) n += redl[w];
            dEpart[it.slot] = red[64];
            ipart[(size_t)it.slot * 9 + 8] = n;
        }
    }
}

#define MCS_FPART 24  // doubles per measurement tile (Ising: 4 + 8 ints; O(n): compact F)

// O(n) tile partial: the F frame restricted to the tile's virtual index range.
template <int DIM, int GEOM>
__global__ void __launch_bounds__(256) k_tiled_measure(Rep *reps, const Item *items, double *fpart)
{
    __shared__ double red[MCS_RED_DOUBLES];
    __shared__ double F[F_NON];
    __shared__ long long redl[32 * 16 + 16];
    __shared__ long long Fi[16];
    __shared__ Rep R;
    const Item it = items[blockIdx.x];
    load_rep(R, reps + it.rep);
    if (R.u >= R.u_stop || !measures_after(R, R.u)) return;
    Spins S = spins_global(R);
    double *out = fpart + (size_t)blockIdx.x * F_NON;
    if (DIM == 1) {
        is_frame<GEOM>(R, R.itab, S.s, it.begin, it.end, R.m, red, F, redl, Fi);
        if (threadIdx.x < 4) out[threadIdx.x] = F[threadIdx.x];
        if (threadIdx.x < MCS_MAXT + MCS_MAXC) out[4 + threadIdx.x] = (double)Fi[threadIdx.x];
    } else {
        const bool efull = (R.m % R.recheck) == 0;
        for (int k = threadIdx.x; k < F_NON; k += blockDim.x) F[k] = 0.0;
        __syncthreads();
        on_frame<DIM, GEOM>(R, R.jtab, R.dtab, S, it.begin, it.end, efull, red, F, nullptr);
        for (int k = threadIdx.x; k < F_NON; k += blockDim.x) out[k] = F[k];
    }
}

// One CTA per replica: fold sweep partials, measurement partials, advance.
template <int DIM>
__global__ void __launch_bounds__(256) k_tiled_finalize(Rep *reps, const int *ids, const int *item_off, double *dEpart,
                                                        long long *ipart, const int *mitem_off, double *fpart)
{
    __shared__ double red[MCS_RED_DOUBLES];
    __shared__ double F[F_NON];
    __shared__ float fsx[MCS_FS_STRIDE];  // FP32 frame for the warp fold
    __shared__ long long redl[32 * 9 + 9];
    __shared__ long long Fi[16];
    __shared__ int meas;
    __shared__ Rep R;  // written back below: u, m, frames_written
    const int r = ids[blockIdx.x];
    Rep *Rg = reps + r;
    load_rep(R, Rg);
    if (R.u >= R.u_stop) return;
    const int tid = threadIdx.x;
    const int i0 = item_off[blockIdx.x], i1 = item_off[blockIdx.x + 1];
    const long long u = R.u;
    if (DIM == 1) {
        long long v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = i0 + tid; i < i1; i += blockDim.x)
            for (int k = 0; k < 9; ++k) v[k] += ipart[(size_t)i * 9 + k];
        block_sum_ll<9>(v, redl, redl + 32 * 9);
        if (tid == 0) {
            for (int k = 0; k < MCS_MAXC; ++k) R.icnt[C_DN + k] += -4 * redl[32 * 9 + k];
            for (int k = 0; k < MCS_MAXT; ++k) R.icnt[C_DM + k] += -2 * redl[32 * 9 + MCS_MAXC + k];
            R.stats[S_ACCEPT] += redl[32 * 9 + 8];
            if (R.alg == 0 && u + 1 == R.units_thermal) {
                double Einc = 0;
                for (int c = 0; c < R.nclass; ++c) Einc += 0.5 * R.Q[c] * (double)R.icnt[C_DN + c];
                for (int t = 0; t < R.ntype; ++t) Einc -= R.hd * R.Stype[t] * (double)R.icnt[C_DM + t];
                R.acc[B_EMEAS0] = Einc;
            }
        }
    } else {
        double v[2] = {0.0, 0.0};
        for (int i = i0 + tid; i < i1; i += blockDim.x) { v[0] += dEpart[i]; v[1] += (double)ipart[(size_t)i * 9 + 8]; }
        block_sum<2>(v, red, F);
        if (tid == 0) { R.acc[A_ECUR] += F[0]; R.stats[S_ACCEPT] += (long long)F[1]; }
    }
    if (tid == 0) meas = measures_after(R, u);
    __syncthreads();
    if (meas) {
        const int m0 = mitem_off[blockIdx.x], m1 = mitem_off[blockIdx.x + 1];
        const int nf = DIM == 1 ? 4 + MCS_MAXT + MCS_MAXC : F_NON;
        // the measurement tiles' partials: one warp per frame value, lanes
        // over the tiles, then an FP64 shuffle tree (a replica of a large
        // lattice has a hundred tiles or more)
        {
            const int lane = tid & 31, wid = tid >> 5, nwb = blockDim.x >> 5;
            for (int k = wid; k < nf; k += nwb) {
                // four loads in flight per lane
                double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
                int i = m0 + lane;
                for (; i + 96 < m1; i += 128) {
                    a0 += fpart[(size_t)i * F_NON + k];
                    a1 += fpart[(size_t)(i + 32) * F_NON + k];
                    a2 += fpart[(size_t)(i + 64) * F_NON + k];
                    a3 += fpart[(size_t)(i + 96) * F_NON + k];
                }
                for (; i < m1; i += 32) a0 += fpart[(size_t)i * F_NON + k];
                double a = (a0 + a1) + (a2 + a3);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                if (lane == 0) F[k] = a;
            }
        }
        __syncthreads();
        const long long m = R.m;
        if (tid == 0) {
            if (DIM == 1) {
                for (int k = 0; k < MCS_MAXT + MCS_MAXC; ++k) Fi[k] = (long long)F[4 + k];
                signed char *s = (signed char *)R.spins;
                is_accumulate(R, F, Fi, s[R.last_site], m);
            } else if ((m % R.recheck) == 0) {
                double Ef = F[F_EFB] / 2 + F[F_EFO];
                double d = fabs(R.acc[A_ECUR] - Ef);
                if (d > R.acc[A_DRIFT]) R.acc[A_DRIFT] = d;
                R.acc[A_ECUR] = Ef;
            }
        }
        if (DIM > 1 && tid < 32) {
            __syncwarp();
            for (int f = tid; f < F_NON; f += 32) fsx[f] = (float)F[f];
            __syncwarp();
            if (DIM == 2) on_accumulate_frames<2>(R, fsx, &R.acc[A_ECUR], m, 1, tid);
            else on_accumulate_frames<3>(R, fsx, &R.acc[A_ECUR], m, 1, tid);
        }
        if (R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames) {
            Spins S = spins_global(R);
            for (int v = tid; v < R.N; v += blockDim.x) frame_store<DIM>(R, R.frames_written, v, S, v);
        }
        __syncthreads();
        if (tid == 0) {
            if (R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames) R.frames_written++;
            R.m = m + 1;
        }
    }
    if (tid == 0) {
        R.stats[S_VISITS] += R.N;
        Rg->u = u + 1;
        Rg->m = R.m;
        Rg->frames_written = R.frames_written;
    }
}

// ======================================================================= initial state
// One CTA per replica: full energy (O(n)) or the exact integer sums (Ising)
// of the initial lattice.
template <int DIM, int GEOM>
__global__ void __launch_bounds__(1024) k_init(Rep *reps, const int *ids)
{
    __shared__ double red[MCS_RED_DOUBLES];
    __shared__ double F[F_NON];
    __shared__ long long redl[32 * 16 + 16];
    __shared__ long long Fi[16];
    Rep &R = reps[ids[blockIdx.x]];
    if (R.dim != (DIM == 1 ? 1 : DIM) || R.geom != GEOM) return;
    Spins S = spins_global(R);
    const int vmax = max(max(R.N, R.nlat), max(R.n_rorb, R.ncirc));
    if (R.rinit) {
        // random initial state keyed by the sweep index: Ising sign, XY angle, Heisenberg sphere
        for (int v = threadIdx.x; v < R.N; v += blockDim.x) {
            const uint4 w = philox((uint32_t)v, 0u, 0u, 0x5000u, R.seed);
            if (DIM == 1) {
                S.s[v] = (w.x & 1) ? 1 : -1;
            } else {
                float r0, r1, r2;
                on_direction_exact<DIM>(w, r0, r1, r2);
                const float a = R.slen[v];
                S.x[v] = r0 * a; S.y[v] = r1 * a;
                if (DIM == 3) S.z[v] = r2 * a;
            }
        }
        __syncthreads();
    }
    if (DIM == 1) {
        is_frame<GEOM>(R, R.itab, S.s, 0, vmax, 0, red, F, redl, Fi);
        if (threadIdx.x == 0) {
            for (int k = 0; k < MCS_MAXT; ++k) { R.icnt[C_M0 + k] = Fi[k]; R.icnt[C_DM + k] = 0; }
            for (int k = 0; k < MCS_MAXC; ++k) { R.icnt[C_N0 + k] = Fi[MCS_MAXT + k]; R.icnt[C_DN + k] = 0; }
        }
    } else {
        for (int k = threadIdx.x; k < F_NON; k += blockDim.x) F[k] = 0.0;
        __syncthreads();
        on_frame<DIM, GEOM>(R, R.jtab, R.dtab, S, 0, vmax, true, red, F, nullptr);
        if (threadIdx.x == 0) R.acc[A_ECUR] = F[F_EFB] / 2 + F[F_EFO];
    }
}

// ======================================================================= Wolff
struct WolffLayout {
    size_t spins, tables, stype, bits, queue, red, F, redl, Fi, sh, acc, total;
    int gstate;     // 1: spins, bits and queue live in global memory
    int q16;
};
__host__ __device__ inline WolffLayout wolff_layout(const Rep &R, size_t limit = 232448)
{
    WolffLayout L;
    for (int g = 0; g < 2; ++g) {
        size_t off = 0;
        L.gstate = g;
        L.spins = off;
        if (!g) {
            if (R.dim == 1) off += align16((size_t)R.N);
            else off += align16((size_t)R.dim * R.N * sizeof(float));
        }
        L.tables = off;
        if (R.dim == 1) off += align16((size_t)R.nite * sizeof(IsEntry));
        else off += align16((size_t)R.njc * 9 * sizeof(float) + (size_t)R.ndc * 4 * sizeof(float));
        L.stype = off;
        if (!g) off += align16((size_t)R.N);
        L.bits = off;
        if (!g) off += align16(((size_t)R.N + 31) / 32 * 4);
        L.queue = off;
        L.q16 = !g && R.N <= 65536;
        if (!g) off += align16((size_t)R.N * (L.q16 ? 2 : 4));
        L.red = off; off += MCS_RED_DOUBLES * sizeof(double);
        L.F = off; off += F_NON * sizeof(double);
        L.redl = off; off += (32 * 16 + 16) * sizeof(long long);
        L.Fi = off; off += 16 * sizeof(long long);
        L.sh = off; off += 64;
        L.acc = off; off += align16((size_t)R.nacc * sizeof(double) + C_NINT * sizeof(long long));
        L.total = off;
        if (L.total <= limit) return L;
    }
    return L;
}
long long resident_wolff_smem_bytes(const Rep &r) { return (long long)wolff_layout(r).total; }

// GS: the host keeps this group's state (spins, bitmask, queue) in global
// memory; otherwise it lives in shared memory, which the compiler then knows.
template <int DIM, int GEOM, bool GS>
__global__ void __launch_bounds__(512) k_wolff(Rep *reps, const int *ids, long long max_units)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ Rep R;
    Rep *Rg = reps + ids[blockIdx.x];
    load_rep(R, Rg);
    if (R.u >= R.u_stop) return;
    const WolffLayout L = GS ? wolff_layout(R, 0) : wolff_layout(R);
    const int tid = threadIdx.x, bd = blockDim.x, N = R.N;
    double *red = (double *)(smem + L.red);
    double *F = (double *)(smem + L.F);
    long long *redl = (long long *)(smem + L.redl);
    long long *Fi = (long long *)(smem + L.Fi);
    int *sh = (int *)(smem + L.sh);
    float *shf = (float *)(sh + 8);
    __shared__ float wfs[MCS_FS_STRIDE];  // one measurement frame in FP32
    const unsigned char *st = R.stype;
    if (!GS) {
        unsigned char *sts = (unsigned char *)(smem + L.stype);
        for (int v = tid; v < N; v += bd) sts[v] = R.stype[v];
        st = sts;
    }
    IsEntry *itab = (IsEntry *)(smem + L.tables);
    float *jt = (float *)(smem + L.tables);
    float *dt = jt + R.njc * 9;
    Spins G = spins_global(R);
    Spins S = G;
    WolffMem W;
    if (GS) {
        W.bits = R.wbits; W.queue = R.wqueue; W.q16 = nullptr;
    } else {
        W.bits = (unsigned int *)(smem + L.bits);
        W.queue = (int *)(smem + L.queue);
        W.q16 = L.q16 ? (unsigned short *)(smem + L.queue) : nullptr;
        for (int k = tid; k < (N + 31) / 32; k += bd) W.bits[k] = 0u;
        if (DIM == 1) {
            S.s = (signed char *)(smem + L.spins);
            for (int v = tid; v < N; v += bd) S.s[v] = G.s[v];
        } else {
            S.x = (float *)(smem + L.spins);
            S.y = S.x + N;
            S.z = S.y + N;
            for (int v = tid; v < N; v += bd) {
                S.x[v] = G.x[v]; S.y[v] = G.y[v];
                if (DIM == 3) S.z[v] = G.z[v];
            }
        }
    }
    if (DIM == 1) for (int k = tid; k < R.nite; k += bd) itab[k] = R.itab[k];
    else {
        for (int k = tid; k < R.njc * 9; k += bd) jt[k] = R.jtab[k];
        for (int k = tid; k < R.ndc * 4; k += bd) dt[k] = R.dtab[k];
    }
    __syncthreads();
    acc_to_smem(R, smem + L.acc);
    double dEd = 0.0;
    long long dnacc = 0;
    int dn[MCS_MAXC] = {0, 0, 0, 0}, dm[MCS_MAXT] = {0, 0, 0, 0};
    long long u = R.u;
    const long long uend = min(R.u_stop, u + max_units);
    for (; u < uend; ++u) {
        if (tid == 0) R.u = u;
        __syncthreads();
        wolff_cluster<DIM, GEOM>(R, jt, dt, itab, st, S, W, R.u0 + u, sh, shf, red, F, redl, Fi, dEd, dnacc, dn, dm);
        if (measures_after(R, u)) {
            const long long m = R.m;
            if (DIM == 1) {
                is_frame<GEOM>(R, itab, S.s, 0, max(N, max(R.nlat, R.n_rorb)), m, red, F, redl, Fi);
                if (tid == 0) is_accumulate(R, F, Fi, S.s[R.last_site], m);
            } else {
                if (tid == 0) { R.acc[A_ECUR] += dEd; dEd = 0.0; }
                const bool efull = (m % R.recheck) == 0;
                // the block spins once per measurement, in the replica's global
                // scratch (L2): each is read by its own chosen site and by the
                // renormalised links of its neighbours instead of formed again
                on_frame_inline<DIM, GEOM>(R, jt, dt, S, 0, max(max(N, R.nlat), max(R.n_rorb, R.ncirc)), efull, red, F, R.wmaj);
                if (tid == 0 && efull) {
                    double Ef = F[F_EFB] / 2 + F[F_EFO];
                    double d = fabs(R.acc[A_ECUR] - Ef);
                    if (d > R.acc[A_DRIFT]) R.acc[A_DRIFT] = d;
                    R.acc[A_ECUR] = Ef;
                }
                // the frame folds into the accumulators with one warp (as in the resident kernel)
                if (tid < 32) {
                    __syncwarp();
                    for (int f = tid; f < F_NON; f += 32) wfs[f] = (float)F[f];
                    __syncwarp();
                    on_accumulate_frames<DIM>(R, wfs, &R.acc[A_ECUR], m, 1, tid);
                }
            }
            if (R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames)
                for (int v = tid; v < N; v += bd) frame_store<DIM>(R, R.frames_written, v, S, v);
            __syncthreads();
            if (tid == 0) {
                if (R.frames > 0 && (m % R.frame_every) == 0 && R.frames_written < R.frames) R.frames_written++;
                R.m = m + 1;
            }
            __syncthreads();
        }
    }
    if (DIM > 1 && tid == 0) R.acc[A_ECUR] += dEd;
    __syncthreads();
    acc_to_global(R, Rg);
    if (!GS)
        for (int v = tid; v < N; v += bd) {
            if (DIM == 1) G.s[v] = S.s[v];
            else {
                G.x[v] = S.x[v]; G.y[v] = S.y[v];
                if (DIM == 3) G.z[v] = S.z[v];
            }
        }
    if (tid == 0) {
        Rg->u = uend;
        Rg->m = R.m;
        Rg->frames_written = R.frames_written;
    }
}

// ======================================================================= launchers
template <int DIM, int GEOM>
static cudaError_t set_smem_attr(size_t smem)
{
    static size_t done = 0;
    if (smem > 48 * 1024 && smem > done) {
        cudaError_t e = cudaFuncSetAttribute(k_resident_metro<DIM, GEOM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        done = smem;
    }
    return cudaSuccess;
}

#define MCS_DISPATCH(dim, geom, CALL)                                                   \
    do {                                                                                 \
        if (geom == MCS_GEOM_SQUARE) {                                                   \
            if (dim == 1) { CALL(1, MCS_GEOM_SQUARE); }                                  \
            else if (dim == 2) { CALL(2, MCS_GEOM_SQUARE); }                             \
            else { CALL(3, MCS_GEOM_SQUARE); }                                           \
        } else {                                                                         \
            if (dim == 1) { CALL(1, MCS_GEOM_ELL); }                                     \
            else if (dim == 2) { CALL(2, MCS_GEOM_ELL); }                                \
            else { CALL(3, MCS_GEOM_ELL); }                                              \
        }                                                                                \
    } while (0)

template <int DIM, int GEOM>
static cudaError_t launch_resident_t(Rep *reps, const int *ids, int nrep, int copies, int threads, size_t smem,
                                     long long max_units, cudaStream_t st)
{
    cudaError_t e = set_smem_attr<DIM, GEOM>(smem);
    if (e != cudaSuccess) return e;
    if (copies <= 1) {
        k_resident_metro<DIM, GEOM><<<nrep, threads, smem, st>>>(reps, ids, max_units, 1);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nrep * copies, 1, 1);
    cfg.blockDim = dim3(threads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = copies;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_resident_metro<DIM, GEOM>, reps, ids, max_units, copies);
}

// copies: CTAs per replica, each with a full copy of the lattice (1 = one CTA)
cudaError_t launch_resident_metro(int dim, int geom, Rep *reps, const int *ids, int nrep, int threads, size_t smem,
                                  long long max_units, cudaStream_t st, int copies)
{
    if (nrep <= 0) return cudaSuccess;
#define CALL_RES(D, G) return launch_resident_t<D, G>(reps, ids, nrep, copies, threads, smem, max_units, st);
    MCS_DISPATCH(dim, geom, CALL_RES);
#undef CALL_RES
    return cudaErrorInvalidValue;
}

// Resident clusters of `copies` CTAs the device can hold at once (0: cannot launch).
int resident_copies_active(int dim, int geom, int copies, int threads, size_t smem)
{
    int n = 0;
#define CALL_OCC(D, G)                                                                                   \
    {                                                                                                    \
        if (set_smem_attr<D, G>(smem) != cudaSuccess) { cudaGetLastError(); return 0; }                  \
        cudaLaunchConfig_t cfg = {};                                                                     \
        cfg.gridDim = dim3(copies, 1, 1);                                                                \
        cfg.blockDim = dim3(threads, 1, 1);                                                              \
        cfg.dynamicSmemBytes = smem;                                                                     \
        cudaLaunchAttribute attr[1];                                                                     \
        attr[0].id = cudaLaunchAttributeClusterDimension;                                                \
        attr[0].val.clusterDim.x = copies;                                                               \
        attr[0].val.clusterDim.y = 1;                                                                    \
        attr[0].val.clusterDim.z = 1;                                                                    \
        cfg.attrs = attr;                                                                                \
        cfg.numAttrs = 1;                                                                                \
        if (cudaOccupancyMaxActiveClusters(&n, k_resident_metro<D, G>, &cfg) != cudaSuccess) {          \
            cudaGetLastError();                                                                          \
            return 0;                                                                                    \
        }                                                                                                \
        return n;                                                                                        \
    }
    MCS_DISPATCH(dim, geom, CALL_OCC);
#undef CALL_OCC
    return 0;
}

cudaError_t launch_tiled_sweep(int dim, int geom, Rep *reps, const Item *items, int nitems, int colour,
                               double *dEpart, long long *ipart, int threads, cudaStream_t st)
{
    if (nitems <= 0) return cudaSuccess;
#define CALL_TS(D, G) k_tiled_sweep<D, G><<<nitems, threads, 0, st>>>(reps, items, colour, dEpart, ipart);
    MCS_DISPATCH(dim, geom, CALL_TS);
#undef CALL_TS
    return cudaGetLastError();
}

cudaError_t launch_tiled_measure(int dim, int geom, Rep *reps, const Item *items, int nitems, double *fpart,
                                 int threads, cudaStream_t st)
{
    if (nitems <= 0) return cudaSuccess;
#define CALL_TM(D, G) k_tiled_measure<D, G><<<nitems, threads, 0, st>>>(reps, items, fpart);
    MCS_DISPATCH(dim, geom, CALL_TM);
#undef CALL_TM
    return cudaGetLastError();
}

cudaError_t launch_tiled_finalize_dim(int dim, Rep *reps, const int *ids, int nrep, const int *item_off,
                                      double *dEpart, long long *ipart, const int *mitem_off, double *fpart,
                                      cudaStream_t st)
{
    if (nrep <= 0) return cudaSuccess;
    if (dim == 1) k_tiled_finalize<1><<<nrep, 256, 0, st>>>(reps, ids, item_off, dEpart, ipart, mitem_off, fpart);
    else if (dim == 2) k_tiled_finalize<2><<<nrep, 256, 0, st>>>(reps, ids, item_off, dEpart, ipart, mitem_off, fpart);
    else k_tiled_finalize<3><<<nrep, 256, 0, st>>>(reps, ids, item_off, dEpart, ipart, mitem_off, fpart);
    return cudaGetLastError();
}

// Server step bound: each listed replica takes its quota for this step and
// stops after that many units.
__global__ void k_set_stop(Rep *reps, const StopItem *items, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rep &R = reps[items[i].id];
    R.quota = items[i].quota;
    const long long s = R.u + R.quota;
    R.u_stop = s < R.units_total ? s : R.units_total;
}

// Load every kernel of this file on the current device (CUDA loads a kernel
// at its first launch otherwise, which stalls that launch by milliseconds).
cudaError_t preload_kernels_main()
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaSuccess;
    auto touch = [&](const void *f) {
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, f);
    };
#define MCS_TOUCH(D, G)                                                                  \
    touch((const void *)k_resident_metro<D, G>); touch((const void *)k_tiled_sweep<D, G>); \
    touch((const void *)k_tiled_measure<D, G>); touch((const void *)k_init<D, G>);        \
    touch((const void *)k_wolff<D, G, false>); touch((const void *)k_wolff<D, G, true>);
    MCS_TOUCH(1, MCS_GEOM_SQUARE) MCS_TOUCH(2, MCS_GEOM_SQUARE) MCS_TOUCH(3, MCS_GEOM_SQUARE)
    MCS_TOUCH(1, MCS_GEOM_ELL) MCS_TOUCH(2, MCS_GEOM_ELL) MCS_TOUCH(3, MCS_GEOM_ELL)
#undef MCS_TOUCH
    touch((const void *)k_tiled_finalize<1>);
    touch((const void *)k_tiled_finalize<2>);
    touch((const void *)k_tiled_finalize<3>);
    touch((const void *)k_set_stop);
    return e;
}

cudaError_t launch_set_stop(Rep *reps, const StopItem *items, int n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    k_set_stop<<<(n + 127) / 128, 128, 0, st>>>(reps, items, n);
    return cudaGetLastError();
}

cudaError_t launch_init_state_dg(int dim, int geom, Rep *reps, const int *ids, int nrep, cudaStream_t st)
{
    if (nrep <= 0) return cudaSuccess;
#define CALL_IN(D, G) k_init<D, G><<<nrep, 1024, 0, st>>>(reps, ids);
    MCS_DISPATCH(dim, geom, CALL_IN);
#undef CALL_IN
    return cudaGetLastError();
}


template <int DIM, int GEOM, bool GS>
static cudaError_t set_wolff_attr(size_t smem)
{
    static size_t done = 0;
    if (smem > 48 * 1024 && smem > done) {
        cudaError_t e = cudaFuncSetAttribute(k_wolff<DIM, GEOM, GS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        done = smem;
    }
    return cudaSuccess;
}

template <int DIM, int GEOM>
static cudaError_t launch_wolff_t(Rep *reps, const int *ids, int nrep, int threads, size_t smem, long long max_units,
                                  int gstate, cudaStream_t st)
{
    cudaError_t e;
    if (gstate) {
        if ((e = set_wolff_attr<DIM, GEOM, true>(smem)) != cudaSuccess) return e;
        k_wolff<DIM, GEOM, true><<<nrep, threads, smem, st>>>(reps, ids, max_units);
    } else {
        if ((e = set_wolff_attr<DIM, GEOM, false>(smem)) != cudaSuccess) return e;
        k_wolff<DIM, GEOM, false><<<nrep, threads, smem, st>>>(reps, ids, max_units);
    }
    return cudaGetLastError();
}

cudaError_t launch_wolff(int dim, int geom, Rep *reps, const int *ids, int nrep, int threads, size_t smem,
                         long long max_units, int gstate, cudaStream_t st)
{
    if (nrep <= 0) return cudaSuccess;
#define CALL_W(D, G) return launch_wolff_t<D, G>(reps, ids, nrep, threads, smem, max_units, gstate, st);
    MCS_DISPATCH(dim, geom, CALL_W);
#undef CALL_W
    return cudaGetLastError();
}

long long wolff_smem_bytes(const Rep &r, int *gstate)
{
    WolffLayout L = wolff_layout(r);
    if (gstate) *gstate = L.gstate;
    return (long long)L.total;
}
}  // namespace mcs
