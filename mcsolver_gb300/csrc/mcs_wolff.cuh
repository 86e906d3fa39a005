// mcs_wolff.cuh -- Wolff single-cluster updates on the device.
//
// Restated algorithm (reference file:line):
//   Ising:  expandBlock/blockUpdate isingLib.c:165-236 -- FIFO growth, bond from
//           i to j added with probability 1-exp(2 K s_i s_j) when K s_i s_j < 0;
//           cluster flip accepted with exp(-sum 2 h s_i).
//   O(n):   expandBlock/blockUpdate heisenbergLib.c:310-439, xyLib.c:256-380 --
//           embedding along a random direction r, sDotN = -s.r; bond added with
//           probability 1-exp(2 sDotN_i sDotN_j (r.J.r)) when that is < 1; the
//           cluster reflection is accepted with exp(-dE') where dE' holds the
//           exchange terms the embedding leaves out and the single-ion / field
//           change of s + sDotN r (the reference's own rule, kept as is).
// The cluster is the set of sites reachable from the seed along bonds whose
// coin came up, each directed bond (a -> b) drawing its own Philox word
// (a, b, q); growth order does not change that set, so the level-synchronous
// parallel growth here builds exactly the cluster of the sequential FIFO.
// The reference recomputes the whole energy after every accepted cluster; the
// engine adds the exact energy change of the flip instead (Ising: integer bond
// sums; O(n): FP32 per site, FP64 sum, with periodic full re-checks).
#pragma once
#include "mcs_device.cuh"

namespace mcs {

struct WolffMem {
    unsigned int *bits;     // in-cluster bitmask, N/32 words
    int *queue;             // cluster sites in discovery order
    unsigned short *q16;    // same, 16-bit (shared memory, N <= 65536)
};

__device__ __forceinline__ int wq_get(const WolffMem &W, int i) { return W.q16 ? (int)W.q16[i] : W.queue[i]; }
__device__ __forceinline__ void wq_put(const WolffMem &W, int i, int v)
{
    if (W.q16) W.q16[i] = (unsigned short)v;
    else W.queue[i] = v;
}

__device__ __forceinline__ uint32_t wolff_coin(int a, int b, long long q, unsigned long long seed)
{
    uint4 w = philox((uint32_t)a, (uint32_t)b, (uint32_t)q, 0x2000u ^ ((uint32_t)((unsigned long long)q >> 32) << 16), seed);
    return w.x;
}

// The links of site v as for_links, with the square lattice's row taken by a
// multiply-high instead of an integer division when mdiv != 0: mdiv =
// ceil(2^32 / hy) gives floor(k / hy) exactly for k < 2^16 and 1 < hy < 2^16
// (the error term k (mdiv hy - 2^32) / (hy 2^32) stays below 1/hy).
__device__ __forceinline__ uint32_t wolff_mdiv(const Rep &R, int geom)
{
    return (geom == MCS_GEOM_SQUARE && R.N <= 65536 && R.hy > 1) ? (uint32_t)((0x100000000ull + R.hy - 1) / R.hy) : 0u;
}
template <int GEOM, class F>
__device__ __forceinline__ void wolff_links(const Rep &R, int v, uint32_t mdiv, F &&f)
{
    if (GEOM == MCS_GEOM_SQUARE && mdiv != 0u) {
        const int c = v >= R.half;
        const int k = v - c * R.half;
        const int x = (int)__umulhi((uint32_t)k, mdiv);
        sq_links(R, c, x, k - x * R.hy, f);
    } else {
        for_links<GEOM>(R, v, f);
    }
}

// O(n) models whose exchange classes are all isotropic (J s_i.s_j), with no
// single-ion term and no field.
template <int DIM>
__device__ __forceinline__ bool wolff_isotropic(const Rep &R, const float *jt)
{
    if (R.fullJ || R.has_d || R.h != 0.f) return false;
    for (int c = 0; c < R.njc; ++c) {
        const float *M = jt + 9 * c;
        if (M[0] != M[1] || (DIM == 3 && M[1] != M[2])) return false;
    }
    return true;
}

// One cluster (index q) on a replica.  All threads of the block call it.
// sh: shared scratch {int head, tail, accept; float r[3]} ; red/F/redl/Fi as in the frame code.
// Returns nothing; updates spins, bookkeeping and statistics.
template <int DIM, int GEOM>
__device__ __forceinline__ void wolff_cluster(Rep &R, const float *jt, const float *dt, const IsEntry *itab, const unsigned char *st,
                              const Spins &S, const WolffMem &W, long long q, int *sh, float *shf, double *red,
                              double *F, long long *redl, long long *Fi, double &dEd, long long &dnacc,
                              int (&dn)[MCS_MAXC], int (&dm)[MCS_MAXT])
{
    const int tid = threadIdx.x, bd = blockDim.x, N = R.N;
    if (tid == 0) {
        uint4 w = philox_t(0u, q, 0x1000u, R.seed);
        int seed = (int)(((unsigned long long)w.x * (unsigned long long)N) >> 32);
        wq_put(W, 0, seed);
        W.bits[seed >> 5] |= 1u << (seed & 31);
        sh[0] = 0; sh[1] = 1;
        sh[4] = 0; sh[5] = 0; sh[6] = 0;  // discoveries per level, three in rotation
        float r0 = 0, r1 = 0, r2 = 0;
        if (DIM > 1) on_direction<DIM>(make_uint4(w.y, w.z, 0, 0), r0, r1, r2);
        shf[0] = r0; shf[1] = r1; shf[2] = r2;
        sh[3] = (int)w.w;
    }
    __syncthreads();
    const float r0 = shf[0], r1 = shf[1], r2 = shf[2];
    const bool full = R.fullJ;
    const uint32_t mdiv = wolff_mdiv(R, GEOM);
    // square lattice: r.J.r of the four link directions (the same for every site)
    float rj[4] = {0.f, 0.f, 0.f, 0.f};
    if (DIM > 1 && GEOM == MCS_GEOM_SQUARE) {
#pragma unroll
        for (int l = 0; l < 4; ++l) rj[l] = on_jdot<DIM>(jt + 9 * R.sq_code[l], full, r0, r1, r2, r0, r1, r2);
    }
    // ---- growth, one frontier level at a time.  Level k appends the sites
    // it discovers after the queue's current end, counting them in
    // sh[4 + k % 3]; after the level's barrier every thread reads that count.
    // The counter of level k + 3 (= k's) is cleared by thread 0 during level
    // k + 2: after the barrier that ends level k + 1 (every read of it is done)
    // and before the barrier that starts level k + 3.  One barrier per level.
    int lb = 0, le = 1, k = 0;
    while (lb < le) {
        int *cnt = sh + 4 + k % 3;
        if (tid == 0) sh[4 + (k + 1) % 3] = 0;
        if (GEOM == MCS_GEOM_SQUARE) {
            // square lattice: one lane per bond.  A level is a chain of
            // dependent latencies, so it is spread as wide as it goes: bond b
            // of the level is link b & 3 of frontier entry b >> 2, and its lane
            // draws that bond's coin, tests it and claims the site on the
            // bitmask (a site reached along two bonds is claimed once: the
            // first atomicOr wins).  One ballot places the warp's discoveries
            // in lane order, i.e. by (frontier entry, link).  The loop bound is
            // the warp's first lane's, the same for every lane, so the whole
            // warp reaches the ballot.
            const int lane = tid & 31;
            const int nb = 4 * le;
            for (int b0 = 4 * lb + tid - lane; b0 < nb; b0 += bd) {
                const int b = b0 + lane;
                bool take = false;
                int j = 0;
                if (b < nb) {
                    const int i = wq_get(W, b >> 2);
                    const int l = b & 3;
                    wolff_links<GEOM>(R, i, mdiv, [&](int ll, int jj, int) { if (ll == l) j = jj; });
                    const uint32_t cw = wolff_coin(i, j, q, R.seed);
                    const bool in = (W.bits[j >> 5] >> (j & 31)) & 1u;
                    bool bond;
                    if (DIM == 1) {
                        const unsigned long long thr = R.wthr[R.sq_cls[l]][S.s[i] * S.s[j] > 0];
                        bond = (unsigned long long)cw < thr;
                    } else {
                        const float sdi = -(S.x[i] * r0 + S.y[i] * r1 + (DIM == 3 ? S.z[i] * r2 : 0.f));
                        const float sdj = -(S.x[j] * r0 + S.y[j] * r1 + (DIM == 3 ? S.z[j] * r2 : 0.f));
                        const float rjl = l == 0 ? rj[0] : l == 1 ? rj[1] : l == 2 ? rj[2] : rj[3];
                        const float corr = 2.f * sdi * sdj * rjl;
                        bond = corr < 0.f && (1.f - __expf(corr)) > u24(cw);
                    }
                    if (!in && bond) {
                        const unsigned int old = atomicOr(&W.bits[j >> 5], 1u << (j & 31));
                        take = !((old >> (j & 31)) & 1u);
                    }
                }
                const unsigned int bal = __ballot_sync(0xffffffffu, take);
                int base = 0;
                if (lane == 0 && bal) base = atomicAdd(cnt, __popc(bal));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (take) wq_put(W, le + base + __popc(bal & ((1u << lane) - 1u)), j);
            }
        } else
        for (int f = lb + tid; f < le; f += bd) {
            const int i = wq_get(W, f);
            if (DIM == 1) {
                const int si = S.s[i];
                for_links<GEOM>(R, i, [&](int l, int j, int) {
                    if ((W.bits[j >> 5] >> (j & 31)) & 1u) return;
                    const int cls = link_class<GEOM>(R, i, l);
                    const unsigned long long thr = R.wthr[cls][si * S.s[j] > 0];
                    if (thr == 0) return;
                    if ((unsigned long long)wolff_coin(i, j, q, R.seed) < thr) {
                        unsigned int old = atomicOr(&W.bits[j >> 5], 1u << (j & 31));
                        if (!((old >> (j & 31)) & 1u)) wq_put(W, le + atomicAdd(cnt, 1), j);
                    }
                });
            } else {
                const float sdi = -(S.x[i] * r0 + S.y[i] * r1 + (DIM == 3 ? S.z[i] * r2 : 0.f));
                for_links<GEOM>(R, i, [&](int, int j, int code) {
                    if ((W.bits[j >> 5] >> (j & 31)) & 1u) return;
                    const float sdj = -(S.x[j] * r0 + S.y[j] * r1 + (DIM == 3 ? S.z[j] * r2 : 0.f));
                    const float rjr = on_jdot<DIM>(jt + 9 * code, full, r0, r1, r2, r0, r1, r2);
                    const float corr = 2.f * sdi * sdj * rjr;
                    if (!(corr < 0.f)) return;
                    if ((1.f - __expf(corr)) > u24(wolff_coin(i, j, q, R.seed))) {
                        unsigned int old = atomicOr(&W.bits[j >> 5], 1u << (j & 31));
                        if (!((old >> (j & 31)) & 1u)) wq_put(W, le + atomicAdd(cnt, 1), j);
                    }
                });
            }
        }
        __syncthreads();
        lb = le;
        le += *cnt;
        ++k;
    }
    const int n = le;
    // ---- acceptance step and the energy change of the flip
    if (DIM == 1) {
        long long c[MCS_MAXT + MCS_MAXC];
#pragma unroll
        for (int k = 0; k < MCS_MAXT + MCS_MAXC; ++k) c[k] = 0;
        for (int f = tid; f < n; f += bd) {
            const int i = wq_get(W, f);
            const int si = S.s[i];
            const int t = st ? st[i] : 0;
#pragma unroll
            for (int k = 0; k < MCS_MAXT; ++k) c[k] += (k == t) ? si : 0;
            for_links<GEOM>(R, i, [&](int l, int j, int) {
                if ((W.bits[j >> 5] >> (j & 31)) & 1u) return;
                const int cls = link_class<GEOM>(R, i, l);
                const int p = si * S.s[j];
#pragma unroll
                for (int k = 0; k < MCS_MAXC; ++k) c[MCS_MAXT + k] += (k == cls) ? p : 0;
            });
        }
        block_sum_ll<MCS_MAXT + MCS_MAXC>(c, redl, Fi);
        if (tid == 0) {
            double tot = 0;
            for (int t = 0; t < R.ntype; ++t) tot += 2 * R.hd * R.Stype[t] * (double)Fi[t];
            bool acc = tot <= 0 || exp(-tot) > (double)(uint32_t)sh[3] * (1.0 / 4294967296.0);
            sh[2] = acc;
            R.stats[S_CLUSTERS] += 1;
            if (acc) {
                for (int k = 0; k < MCS_MAXC; ++k) R.icnt[C_DN + k] += -4 * Fi[MCS_MAXT + k];
                for (int t = 0; t < MCS_MAXT; ++t) R.icnt[C_DM + t] += -2 * Fi[t];
                R.stats[S_ACCEPT] += 1;
                R.stats[S_FLIPPED] += n;
                if (R.u >= R.units_thermal) R.icnt[C_ACC_MEAS] = 1;
            }
        }
        __syncthreads();
        const bool acc = sh[2];
        for (int f = tid; f < n; f += bd) {
            const int i = wq_get(W, f);
            if (acc) S.s[i] = (signed char)(-S.s[i]);
        }
    } else if (wolff_isotropic<DIM>(R, jt)) {
        // Isotropic exchange, no single-ion term, no field: the embedding is
        // exact.  The exchange terms the acceptance holds are r.J.p_j with p_j
        // perpendicular to r, which vanish, so the reflection is always
        // accepted; a bond inside the cluster keeps its energy (both ends are
        // reflected), and a boundary bond changes by J d_i.s_j with d_i =
        // 2 sdi r, i.e. -2 J sdi sdj.  A boundary site is never reflected, so
        // each cluster site is reflected in the same pass that reads its
        // boundary neighbours.
        float a_dE = 0.f;
        for (int f = tid; f < n; f += bd) {
            const int i = wq_get(W, f);
            const float si0 = S.x[i], si1 = S.y[i], si2 = DIM == 3 ? S.z[i] : 0.f;
            const float sdi = -(si0 * r0 + si1 * r1 + si2 * r2);
            wolff_links<GEOM>(R, i, mdiv, [&](int, int j, int code) {
                if ((W.bits[j >> 5] >> (j & 31)) & 1u) return;
                const float sdj = -(S.x[j] * r0 + S.y[j] * r1 + (DIM == 3 ? S.z[j] * r2 : 0.f));
                a_dE += -2.f * jt[9 * code] * sdi * sdj;
            });
            float n0 = si0 + 2.f * sdi * r0, n1 = si1 + 2.f * sdi * r1, n2 = si2 + 2.f * sdi * r2;
            const int dc = st ? st[i] : 0;
            const float len2 = n0 * n0 + n1 * n1 + n2 * n2;
            const float k = len2 > 0.f ? dt[4 * dc + 3] * rsqrtf(len2) : 1.f;
            S.x[i] = n0 * k; S.y[i] = n1 * k;
            if (DIM == 3) S.z[i] = n2 * k;
        }
        float c2[2] = {0.f, a_dE};
        block_sum_f<2>(c2, red, F);  // its barriers also end every read of the bitmask above
        if (tid == 0) {
            R.stats[S_CLUSTERS] += 1;
            dEd += F[1];
            R.stats[S_ACCEPT] += 1;
            R.stats[S_FLIPPED] += n;
        }
    } else {
        float a_tot = 0.f, a_dE = 0.f;
        for (int f = tid; f < n; f += bd) {
            const int i = wq_get(W, f);
            const float si0 = S.x[i], si1 = S.y[i], si2 = DIM == 3 ? S.z[i] : 0.f;
            const float sdi = -(si0 * r0 + si1 * r1 + si2 * r2);
            const float pi0 = si0 + sdi * r0, pi1 = si1 + sdi * r1, pi2 = si2 + sdi * r2;  // perpenSpin
            const float di0 = 2.f * sdi * r0, di1 = 2.f * sdi * r1, di2 = 2.f * sdi * r2;  // flip change
            for_links<GEOM>(R, i, [&](int, int j, int code) {
                const float *M = jt + 9 * code;
                const float sj0 = S.x[j], sj1 = S.y[j], sj2 = DIM == 3 ? S.z[j] : 0.f;
                const float sdj = -(sj0 * r0 + sj1 * r1 + sj2 * r2);
                const float pj0 = sj0 + sdj * r0, pj1 = sj1 + sdj * r1, pj2 = sj2 + sdj * r2;
                const float src = sdi * on_jdot<DIM>(M, full, r0, r1, r2, pj0, pj1, pj2);
                a_tot += src;
                const bool in = (W.bits[j >> 5] >> (j & 31)) & 1u;
                if (in) {
                    a_tot += sdj * on_jdot<DIM>(M, full, pi0, pi1, pi2, r0, r1, r2);
                    // both ends flip: half of the bond change, the other half comes from j
                    const float dj0 = 2.f * sdj * r0, dj1 = 2.f * sdj * r1, dj2 = 2.f * sdj * r2;
                    const float after = on_jdot<DIM>(M, full, si0 + di0, si1 + di1, si2 + di2, sj0 + dj0, sj1 + dj1, sj2 + dj2);
                    const float before = on_jdot<DIM>(M, full, si0, si1, si2, sj0, sj1, sj2);
                    a_dE += 0.5f * (after - before);
                } else {
                    a_tot += src;
                    a_dE += on_jdot<DIM>(M, full, di0, di1, di2, sj0, sj1, sj2);
                }
            });
            // single-ion and field: the reference evaluates them at s + sDotN r
            const int dc = st ? st[i] : 0;
            const float *D = dt + 4 * dc;
            const float ti0 = sdi * r0, ti1 = sdi * r1, ti2 = sdi * r2;
            if (R.has_d) {
                a_tot += D[0] * (ti0 * (2.f * si0 + ti0)) + D[1] * (ti1 * (2.f * si1 + ti1));
                if (DIM == 3) a_tot += D[2] * (ti2 * (2.f * si2 + ti2));
                a_dE += D[0] * (di0 * (2.f * si0 + di0)) + D[1] * (di1 * (2.f * si1 + di1));
                if (DIM == 3) a_dE += D[2] * (di2 * (2.f * si2 + di2));
            }
            a_tot -= R.h * (DIM == 3 ? ti2 : ti0);
            a_dE -= R.h * (DIM == 3 ? di2 : di0);
        }
        float c2[2] = {a_tot, a_dE};
        block_sum_f<2>(c2, red, F);  // FP32 inside a warp, FP64 across the warps
        if (tid == 0) {
            const double tot = F[0];
            bool acc = tot <= 0 || exp(-tot) > (double)u24((uint32_t)sh[3]);
            sh[2] = acc;
            R.stats[S_CLUSTERS] += 1;
            if (acc) {
                dEd += F[1];
                R.stats[S_ACCEPT] += 1;
                R.stats[S_FLIPPED] += n;
            }
        }
        __syncthreads();
        if (sh[2]) {
            for (int f = tid; f < n; f += bd) {
                const int i = wq_get(W, f);
                const float si0 = S.x[i], si1 = S.y[i], si2 = DIM == 3 ? S.z[i] : 0.f;
                const float sdi = -(si0 * r0 + si1 * r1 + si2 * r2);
                float n0 = si0 + 2.f * sdi * r0, n1 = si1 + 2.f * sdi * r1, n2 = si2 + 2.f * sdi * r2;
                const int dc = st ? st[i] : 0;
                const float len2 = n0 * n0 + n1 * n1 + n2 * n2;
                const float k = len2 > 0.f ? dt[4 * dc + 3] * rsqrtf(len2) : 1.f;
                S.x[i] = n0 * k; S.y[i] = n1 * k;
                if (DIM == 3) S.z[i] = n2 * k;
            }
        }
    }
    // ---- clear the cluster's bits: the whole bitmask word by word when that
    // is fewer stores than the cluster has sites, else site by site
    const int nw = (N + 31) >> 5;
    if (n >= nw)
        for (int k = tid; k < nw; k += bd) W.bits[k] = 0u;
    else
        for (int f = tid; f < n; f += bd) {
            const int i = wq_get(W, f);
            atomicAnd(&W.bits[i >> 5], ~(1u << (i & 31)));
        }
    __syncthreads();
    (void)itab; (void)dnacc; (void)dn; (void)dm;
}

}  // namespace mcs
